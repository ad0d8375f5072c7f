// Command-line driver around the reference's own Accel3 implementations
// (accel::naive, accel::bvh_sahbin, accel::qbvh, ...), compiled from the
// reference sources as a CPU oracle.  It follows the pattern of the
// reference's accel test (src/lightmetrica-test/test_accel3.cpp:241-345):
// a stub Scene3 whose primitives hold stub triangle meshes, then
// Create<Accel3>(key) -> Initialize(nullptr) -> Build(&scene) -> Intersect.
//
// Usage: ref_accel <accel-key> <scene.bin> <rays.bin> <out.bin> [threads]
//        ref_accel --normalize <in.bin> <out.bin>
//   (applies the reference's Math::Normalize to u32 n, f32 v[n*3]; the
//   reference's accel test builds its ray directions with it)
//   scene.bin : u32 nprims, u32 nfaces[nprims], then per primitive
//               f32 positions[nfaces*9] (three unshared vertices per face)
//   rays.bin  : u32 nrays, f32 rays[nrays*8] = (ox,oy,oz,tmin, dx,dy,dz,tmax)
//   out.bin   : per ray i32 global triangle id (-1 miss), f32 p[3], f32 b[2]
// Global triangle id = faces of primitive 0, then primitive 1, ... (the
// enumeration order of accel_naive.cpp:62-87).  Each face carries texcoords
// (0,0),(1,0),(0,1), so Intersection::geom.uv equals the barycentrics that
// weight vertices 2 and 3 (intersectionutils.h:115-124).
#include <pch.h>
#include <lightmetrica/component.h>
#include <lightmetrica/accel3.h>
#include <lightmetrica/scene3.h>
#include <lightmetrica/trianglemesh.h>
#include <lightmetrica/primitive.h>
#include <lightmetrica/intersection.h>
#include <lightmetrica/ray.h>

#include <cstdint>
#include <chrono>
#include <thread>

LM_NAMESPACE_BEGIN

class HarnessMesh : public TriangleMesh
{
public:
    LM_IMPL_CLASS(HarnessMesh, TriangleMesh);
public:
    LM_IMPL_F(NumVertices) = [this]() -> int { return (int)(ps.size() / 3); };
    LM_IMPL_F(NumFaces)    = [this]() -> int { return (int)(fs.size() / 3); };
    LM_IMPL_F(Positions)   = [this]() -> const Float* { return ps.data(); };
    LM_IMPL_F(Normals)     = [this]() -> const Float* { return nullptr; };
    LM_IMPL_F(Texcoords)   = [this]() -> const Float* { return ts.data(); };
    LM_IMPL_F(Faces)       = [this]() -> const unsigned int* { return fs.data(); };
public:
    std::vector<Float> ps;
    std::vector<Float> ts;
    std::vector<unsigned int> fs;
};

class HarnessScene : public Scene3
{
public:
    LM_IMPL_CLASS(HarnessScene, Scene3);
public:
    LM_IMPL_F(NumPrimitives) = [this]() -> int { return (int)prims.size(); };
    LM_IMPL_F(PrimitiveAt) = [this](int index) -> const Primitive* { return prims[index].get(); };
public:
    std::vector<std::unique_ptr<HarnessMesh>> meshes;
    std::vector<std::unique_ptr<Primitive>> prims;
};

LM_NAMESPACE_END

using namespace lightmetrica_v2;

static bool ReadAll(const char* path, std::vector<char>& buf)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize((size_t)n);
    bool ok = std::fread(buf.data(), 1, (size_t)n, f) == (size_t)n;
    std::fclose(f);
    return ok;
}

static int NormalizeMode(const char* in, const char* out)
{
    std::vector<char> b;
    if (!ReadAll(in, b)) return 2;
    uint32_t n; std::memcpy(&n, b.data(), 4);
    const float* v = reinterpret_cast<const float*>(b.data() + 4);
    std::vector<float> r(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++)
    {
        const Vec3 d = Math::Normalize(Vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
        r[3 * i] = d.x; r[3 * i + 1] = d.y; r[3 * i + 2] = d.z;
    }
    FILE* f = std::fopen(out, "wb");
    if (!f) return 6;
    std::fwrite(r.data(), sizeof(float), r.size(), f);
    std::fclose(f);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc == 4 && std::string(argv[1]) == "--normalize") return NormalizeMode(argv[2], argv[3]);
    if (argc < 5)
    {
        std::fprintf(stderr, "usage: %s key scene.bin rays.bin out.bin [threads]\n", argv[0]);
        return 2;
    }
    const std::string key = argv[1];
    int threads = argc > 5 ? std::atoi(argv[5]) : 1;
    if (threads < 1) threads = 1;

    std::vector<char> sb, rb;
    if (!ReadAll(argv[2], sb) || !ReadAll(argv[3], rb)) { std::fprintf(stderr, "read failed\n"); return 2; }

    HarnessScene scene;
    std::vector<uint32_t> faceOffset;
    {
        const char* p = sb.data();
        uint32_t np; std::memcpy(&np, p, 4); p += 4;
        std::vector<uint32_t> nf(np);
        std::memcpy(nf.data(), p, 4 * np); p += 4 * np;
        uint32_t acc = 0;
        for (uint32_t i = 0; i < np; i++)
        {
            faceOffset.push_back(acc);
            acc += nf[i];
            std::unique_ptr<HarnessMesh> m(new HarnessMesh);
            m->ps.resize((size_t)nf[i] * 9);
            std::memcpy(m->ps.data(), p, sizeof(float) * 9 * nf[i]); p += sizeof(float) * 9 * nf[i];
            m->fs.resize((size_t)nf[i] * 3);
            m->ts.resize((size_t)nf[i] * 6);
            for (uint32_t j = 0; j < nf[i]; j++)
            {
                m->fs[3 * j + 0] = 3 * j + 0;
                m->fs[3 * j + 1] = 3 * j + 1;
                m->fs[3 * j + 2] = 3 * j + 2;
                const Float tc[6] = { 0, 0, 1, 0, 0, 1 };
                for (int k = 0; k < 6; k++) m->ts[6 * j + k] = tc[k];
            }
            std::unique_ptr<Primitive> prim(new Primitive);
            prim->index = (int)i;
            prim->transform = Mat4::Identity();
            prim->normalTransform = Mat3::Identity();
            prim->mesh = m.get();
            scene.meshes.push_back(std::move(m));
            scene.prims.push_back(std::move(prim));
        }
    }

    uint32_t nr; std::memcpy(&nr, rb.data(), 4);
    const float* rays = reinterpret_cast<const float*>(rb.data() + 4);

    auto accel = ComponentFactory::Create<Accel3>(key);
    if (!accel) { std::fprintf(stderr, "unknown accel %s\n", key.c_str()); return 3; }
    if (!accel->Initialize(nullptr)) return 4;
    auto tb0 = std::chrono::high_resolution_clock::now();
    if (!accel->Build(&scene)) return 5;
    auto tb1 = std::chrono::high_resolution_clock::now();

    struct Rec { int32_t id; float p[3]; float b[2]; };
    std::vector<Rec> out(nr);
    auto work = [&](uint32_t begin, uint32_t end)
    {
        for (uint32_t i = begin; i < end; i++)
        {
            const float* r = rays + 8 * (size_t)i;
            Ray ray;
            ray.o = Vec3(r[0], r[1], r[2]);
            ray.d = Vec3(r[4], r[5], r[6]);
            Intersection isect;
            Rec rec{ -1, {0, 0, 0}, {0, 0} };
            if (accel->Intersect(&scene, ray, isect, r[3], r[7]))
            {
                rec.id = (int32_t)(faceOffset[isect.primitive->index] + (uint32_t)isect.geom.faceindex);
                rec.p[0] = isect.geom.p.x; rec.p[1] = isect.geom.p.y; rec.p[2] = isect.geom.p.z;
                rec.b[0] = isect.geom.uv.x; rec.b[1] = isect.geom.uv.y;
            }
            out[i] = rec;
        }
    };
    auto t0 = std::chrono::high_resolution_clock::now();
    {
        std::vector<std::thread> ts;
        for (int k = 0; k < threads; k++)
        {
            uint32_t b = (uint32_t)((uint64_t)nr * k / threads), e = (uint32_t)((uint64_t)nr * (k + 1) / threads);
            ts.emplace_back(work, b, e);
        }
        for (auto& t : ts) t.join();
    }
    auto t1 = std::chrono::high_resolution_clock::now();

    FILE* f = std::fopen(argv[4], "wb");
    if (!f) return 6;
    std::fwrite(out.data(), sizeof(Rec), out.size(), f);
    std::fclose(f);
    const double build_s = std::chrono::duration<double>(tb1 - tb0).count();
    const double trace_s = std::chrono::duration<double>(t1 - t0).count();
    std::printf("{\"accel\": \"%s\", \"rays\": %u, \"threads\": %d, \"build_s\": %.6f, \"trace_s\": %.6f}\n",
                key.c_str(), nr, threads, build_s, trace_s);
    return 0;
}
