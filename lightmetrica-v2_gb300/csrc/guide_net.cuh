// The path-guiding network: a small MLP mapping a surface point, its normal
// and the outgoing direction to a mixture of 8 von Mises-Fisher lobes over
// incident directions, trained online on the path tracer's own radiance
// samples.
//
//   input   128 features: position normalised to the scene box and encoded
//           by 16 frequencies half an octave apart (sin, cos of 2^(f/2) pi x,
//           f = 0..15, per axis: 96), normal (3), outgoing direction (3), zero
//           padding (26)
//   hidden  4 x 64 ReLU
//   output  8 lobes x (mean 3, kappa 1, weight 1) = 40 (padded to 48)
//   lobe    mean = m / |m|, kappa = 0.01 + softplus(b) (b clamped to
//           [-20, 4000]), weights = softmax over the 8 logits
//   pdf     q(w) = sum_j pi_j kappa_j / (2 pi (1 - e^{-2 kappa_j}))
//                  exp(kappa_j (mu_j . w - 1))
//   loss    -E[w_s log q(w_s)], w_s = target / sampling pdf (KL divergence
//           of q to the target, as in neural importance sampling)
//
// Parameters, one FP32 array (the master copy Adam updates):
//   W1 [64][128], b1 [64], W2 [64][64], b2, W3 [64][64], b3, W4 [64][64], b4,
//   W5 [48][64], b5 [48]   (rows / entries 40..47 of layer 5 stay zero)
// W_l[o][i] multiplies input i into output o: z = W h + b.
#pragma once

#include <math.h>
#include <stdint.h>

namespace lmgpu {
namespace guide {

constexpr int kIn = 128;
constexpr int kHid = 64;
constexpr int kOut = 48;
constexpr int kOutUsed = 40;
constexpr int kLobes = 8;
constexpr int kFreqs = 16;

constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid * kHid;
constexpr int kOffW4 = kOffB3 + kHid;
constexpr int kOffB4 = kOffW4 + kHid * kHid;
constexpr int kOffW5 = kOffB4 + kHid;
constexpr int kOffB5 = kOffW5 + kOut * kHid;
constexpr int kNumParams = kOffB5 + kOut;

constexpr float kKappaMin = 0.01f;
constexpr float kTwoPi = 6.28318530717958647692f;

__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int layer_out(int l) { return l == 4 ? kOut : kHid; }
__host__ __device__ constexpr int w_off(int l)
{
    return l == 0 ? kOffW1 : l == 1 ? kOffW2 : l == 2 ? kOffW3 : l == 3 ? kOffW4 : kOffW5;
}
__host__ __device__ constexpr int b_off(int l)
{
    return l == 0 ? kOffB1 : l == 1 ? kOffB2 : l == 2 ? kOffB3 : l == 3 ? kOffB4 : kOffB5;
}

// Position features of one axis, u the box-normalised coordinate: the 32
// values sin, cos of 2^(k/2) pi u, k = 0..15, in pairs (sin, cos) by k.
// Two sincospif calls give k = 0 and k = 1; every further octave follows by
// the double-angle identities sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a.
// Seven doublings amplify an error of the first values by at most 2^7: a few
// 1e-5 at most, below the rounding of the argument 2^7.5 pi u itself and far
// below the BF16 rounding of the features.
__device__ __forceinline__ void axis_features(float u, float f[32])
{
    sincospif(u, &f[0], &f[1]);
    sincospif(u * 1.41421356237309505f, &f[2], &f[3]);
#pragma unroll
    for (int k = 2; k < 16; k++) {
        const float s = f[2 * (k - 2)], c = f[2 * (k - 2) + 1];
        f[2 * k] = 2.0f * s * c;
        f[2 * k + 1] = fmaf(-2.0f * s, s, 1.0f);
    }
}

struct Lobes {
    float mu[kLobes][3];
    float kappa[kLobes];
    float logw[kLobes];   // log softmax weights
    float mnorm[kLobes];  // |m|
    float sig[kLobes];    // d kappa / d b
};

__device__ __forceinline__ float softplus(float b) { return b > 20.0f ? b : log1pf(expf(b)); }

__device__ __forceinline__ void lobes_from_raw(const float raw[kOutUsed], Lobes& L)
{
    float amax = -1e30f;
    for (int j = 0; j < kLobes; j++) amax = fmaxf(amax, raw[5 * j + 4]);
    float se = 0.0f;
    for (int j = 0; j < kLobes; j++) se += expf(raw[5 * j + 4] - amax);
    const float lse = amax + logf(se);
    for (int j = 0; j < kLobes; j++) {
        const float mx = raw[5 * j], my = raw[5 * j + 1], mz = raw[5 * j + 2];
        const float nm = fmaxf(sqrtf(mx * mx + my * my + mz * mz), 1e-6f);
        L.mnorm[j] = nm;
        L.mu[j][0] = mx / nm;
        L.mu[j][1] = my / nm;
        L.mu[j][2] = mz / nm;
        const float b = fminf(fmaxf(raw[5 * j + 3], -20.0f), 4000.0f);
        L.kappa[j] = kKappaMin + softplus(b);
        L.sig[j] = (raw[5 * j + 3] > -20.0f && raw[5 * j + 3] < 4000.0f) ? 1.0f / (1.0f + expf(-b)) : 0.0f;
        L.logw[j] = raw[5 * j + 4] - lse;
    }
}

// log of kappa / (2 pi (1 - e^{-2 kappa}))
__device__ __forceinline__ float vmf_log_norm(float k) { return logf(k / (kTwoPi * -expm1f(-2.0f * k))); }

// log q(w) and the responsibilities r_j = pi_j vmf_j(w) / q(w).
__device__ __forceinline__ float mixture_logpdf(const Lobes& L, const float w[3], float r[kLobes])
{
    float l[kLobes], lmax = -1e30f;
    for (int j = 0; j < kLobes; j++) {
        const float c = L.mu[j][0] * w[0] + L.mu[j][1] * w[1] + L.mu[j][2] * w[2];
        l[j] = L.logw[j] + vmf_log_norm(L.kappa[j]) + L.kappa[j] * (c - 1.0f);
        lmax = fmaxf(lmax, l[j]);
    }
    float s = 0.0f;
    for (int j = 0; j < kLobes; j++) s += expf(l[j] - lmax);
    const float lq = lmax + logf(s);
    for (int j = 0; j < kLobes; j++) r[j] = expf(l[j] - lq);
    return lq;
}

// Gradient of -weight * log q(w) with respect to the 40 raw outputs.
__device__ __forceinline__ float loss_grad(const Lobes& L, const float w[3], float weight, float g[kOutUsed])
{
    float r[kLobes];
    const float lq = mixture_logpdf(L, w, r);
    for (int j = 0; j < kLobes; j++) {
        const float k = L.kappa[j];
        const float c = L.mu[j][0] * w[0] + L.mu[j][1] * w[1] + L.mu[j][2] * w[2];
        // d log q / d m: r kappa (w - (mu.w) mu) / |m|
        const float s = -weight * r[j] * k / L.mnorm[j];
        for (int d = 0; d < 3; d++) g[5 * j + d] = s * (w[d] - c * L.mu[j][d]);
        // d log vmf / d kappa = 1/kappa - 2 / (e^{2 kappa} - 1) + (mu.w - 1)
        const float dlogc = 1.0f / k - (k > 40.0f ? 0.0f : 2.0f / expm1f(2.0f * k));
        g[5 * j + 3] = -weight * r[j] * (dlogc + c - 1.0f) * L.sig[j];
        // d log q / d a_j = r_j - pi_j
        g[5 * j + 4] = -weight * (r[j] - expf(L.logw[j]));
    }
    return -weight * lq;
}

// Samples a direction from the mixture with (u0 lobe, u1, u2 direction).
__device__ __forceinline__ void mixture_sample(const Lobes& L, float u0, float u1, float u2, float w[3])
{
    int j = kLobes - 1;
    float acc = 0.0f;
    for (int q = 0; q < kLobes; q++) {
        acc += expf(L.logw[q]);
        if (u0 < acc) { j = q; break; }
    }
    const float k = L.kappa[j];
    // cos(theta) of a vMF sample: 1 + log(u + (1 - u) e^{-2 kappa}) / kappa,
    // written as -1 + log1p(u (e^{2 kappa} - 1)) / kappa while e^{2 kappa}
    // is finite, and as 1 + log(u) / kappa beyond
    const float ct0 = k < 40.0f ? -1.0f + log1pf(u1 * expm1f(2.0f * k)) / k : 1.0f + logf(fmaxf(u1, 1e-30f)) / k;
    const float ct = fminf(1.0f, fmaxf(-1.0f, ct0));
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float sp, cp;
    sincospif(2.0f * u2, &sp, &cp);
    const float* m = L.mu[j];
    // orthonormal frame around m
    const float sgn = m[2] >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sgn + m[2]), b = m[0] * m[1] * a;
    const float t1[3] = {1.0f + sgn * m[0] * m[0] * a, sgn * b, -sgn * m[0]};
    const float t2[3] = {b, sgn + m[1] * m[1] * a, -m[1]};
    for (int d = 0; d < 3; d++) w[d] = st * cp * t1[d] + st * sp * t2[d] + ct * m[d];
}

}  // namespace guide
}  // namespace lmgpu
