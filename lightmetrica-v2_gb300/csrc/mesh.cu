// Mesh ingestion on the GPU: a scene's primitives, each an indexed triangle
// mesh (TriangleMesh::Positions / Faces, trianglemesh.h:60-90) with its
// transform (Primitive::transform, primitive.h:56-80), flattened into the
// accel's triangle buffer in global order -- primitives in order, faces in
// mesh order -- as the reference's accels enumerate them
// (accel_naive.cpp:59-90, accel_bvh_sahbin.cpp:70-100).  Each vertex goes
// through the transform with the reference's single-precision arithmetic:
// Mat4 x Vec4 on SSE (math.h:1268-1279) computes, per row r,
//     (m[0][r] x + m[1][r] y) + (m[2][r] z + m[3][r] w)
// with every product and sum rounded to float, here with round-to-nearest
// intrinsics (no fused multiply-add), so the triangles equal the reference's
// bit for bit.
//
// One thread per global face: the face's mesh by binary search over the
// meshes' first global face, its three indices checked against the mesh's
// vertex count (an index out of range raises the status word and writes a
// zero triangle), nine floats out.  Uploading positions and faces as they
// are moves 12 bytes per vertex and 12 per face over the host link instead
// of the 36 per face of a host-flattened buffer.
#include <vector>

#include "accel.cuh"

namespace lmgpu {
namespace {

// A mesh as the kernel sees it (device pointers).
struct DevMesh {
    const float* positions;
    const uint32_t* faces;
    uint32_t num_vertices;
    uint32_t num_faces;
    uint64_t first_face;  // global id of the mesh's face 0
    float m[16];          // column-major m[c][r] = m[4 c + r]
};

__device__ __forceinline__ float3 transform_point(const float* m, float x, float y, float z)
{
    float r[3];
    for (int k = 0; k < 3; k++)
        r[k] = __fadd_rn(__fadd_rn(__fmul_rn(m[k], x), __fmul_rn(m[4 + k], y)),
                         __fadd_rn(__fmul_rn(m[8 + k], z), m[12 + k]));  // m[3][r] * 1 is exact
    return make_float3(r[0], r[1], r[2]);
}

__global__ void k_flatten(const DevMesh* __restrict__ meshes, uint32_t nmeshes, uint64_t total,
                          float* __restrict__ tris, int32_t* __restrict__ tri_prim, uint32_t* __restrict__ status)
{
    const uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (g >= total) return;
    // the last mesh whose first face is <= g
    uint32_t lo = 0, hi = nmeshes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (meshes[mid].first_face <= g) lo = mid;
        else hi = mid;
    }
    const DevMesh& M = meshes[lo];
    const uint64_t f = g - M.first_face;
    float* out = tris + 9 * g;
    if (tri_prim) tri_prim[g] = (int32_t)lo;
    bool ok = true;
    uint32_t idx[3];
    for (int k = 0; k < 3; k++) {
        idx[k] = M.faces[3 * f + k];
        ok = ok && idx[k] < M.num_vertices;
    }
    if (!ok) {
        atomicOr(status, 1u);
        for (int k = 0; k < 9; k++) out[k] = 0.0f;
        return;
    }
    for (int k = 0; k < 3; k++) {
        const float* p = M.positions + 3 * (size_t)idx[k];
        const float3 q = transform_point(M.m, p[0], p[1], p[2]);
        out[3 * k] = q.x;
        out[3 * k + 1] = q.y;
        out[3 * k + 2] = q.z;
    }
}

// Flattens meshes whose positions / faces are device pointers; returns the
// total face count through *total.
int flatten(const lmgpu_mesh* meshes, uint32_t n, float* d_tris, int32_t* d_tri_prim, cudaStream_t stream,
            const char* name)
{
    std::vector<DevMesh> table(n);
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; i++) {
        const lmgpu_mesh& m = meshes[i];
        if (m.num_faces > 0 && (!m.positions || !m.faces)) {
            set_error(std::string(name) + ": mesh " + std::to_string(i) + " has faces but no buffers");
            return LMGPU_ERR_INVALID;
        }
        table[i].positions = m.positions;
        table[i].faces = m.faces;
        table[i].num_vertices = m.num_vertices;
        table[i].num_faces = m.num_faces;
        table[i].first_face = total;
        for (int k = 0; k < 16; k++) table[i].m[k] = m.transform[k];
        total += m.num_faces;
    }
    if (total == 0) return LMGPU_OK;
    if (!d_tris) {
        set_error(std::string(name) + ": NULL triangle buffer");
        return LMGPU_ERR_INVALID;
    }
    DevMesh* d_table = nullptr;
    uint32_t* d_status = nullptr;
    LMGPU_CUDA_TRY(cudaMalloc((void**)&d_table, sizeof(DevMesh) * n));
    if (cudaMalloc((void**)&d_status, sizeof(uint32_t)) != cudaSuccess) {
        cudaFree(d_table);
        set_error(std::string(name) + ": cudaMalloc failed");
        return LMGPU_ERR_CUDA;
    }
    cudaError_t e = cudaMemcpyAsync(d_table, table.data(), sizeof(DevMesh) * n, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(uint32_t), stream);
    if (e == cudaSuccess) {
        k_flatten<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(d_table, n, total, d_tris, d_tri_prim,
                                                                      d_status);
        e = cudaGetLastError();
    }
    uint32_t st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    cudaFree(d_table);
    cudaFree(d_status);
    if (e != cudaSuccess) {
        set_error(std::string(name) + ": " + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    if (st) {
        set_error(std::string(name) + ": a face index is out of its mesh's vertex range");
        return LMGPU_ERR_INVALID;
    }
    return LMGPU_OK;
}

}  // namespace
}  // namespace lmgpu

extern "C" {

int lmgpu_flatten_meshes_device(const lmgpu_mesh* meshes, uint32_t n, float* d_triangles, int32_t* d_tri_prim,
                                void* stream)
{
    lmgpu::clear_error();
    if (n > 0 && !meshes) {
        lmgpu::set_error("lmgpu_flatten_meshes_device: NULL meshes");
        return LMGPU_ERR_INVALID;
    }
    return lmgpu::flatten(meshes, n, d_triangles, d_tri_prim, (cudaStream_t)stream, "lmgpu_flatten_meshes_device");
}

int lmgpu_accel_build_meshes(lmgpu_accel* a, const lmgpu_mesh* meshes, uint32_t n)
{
    lmgpu::clear_error();
    const char* name = "lmgpu_accel_build_meshes";
    if (!a || (n > 0 && !meshes)) {
        lmgpu::set_error(std::string(name) + ": NULL argument");
        return LMGPU_ERR_INVALID;
    }
    // host checks, then one upload of all positions and faces
    uint64_t nv = 0, nf = 0;
    for (uint32_t i = 0; i < n; i++) {
        const lmgpu_mesh& m = meshes[i];
        if (m.num_faces > 0 && (!m.positions || !m.faces)) {
            lmgpu::set_error(std::string(name) + ": mesh " + std::to_string(i) + " has faces but no buffers");
            return LMGPU_ERR_INVALID;
        }
        for (uint64_t k = 0; k < 3ull * m.num_faces; k++)
            if (m.faces[k] >= m.num_vertices) {
                lmgpu::set_error(std::string(name) + ": mesh " + std::to_string(i) + " face index " +
                                 std::to_string(m.faces[k]) + " >= " + std::to_string(m.num_vertices) + " vertices");
                return LMGPU_ERR_INVALID;
            }
        nv += m.num_vertices;
        nf += m.num_faces;
    }
    if (nf == 0) return lmgpu_accel_build_device(a, nullptr, 0, nullptr);
    float *d_pos = nullptr, *d_tris = nullptr;
    uint32_t* d_faces = nullptr;
    auto release = [&]() {
        if (d_pos) cudaFree(d_pos);
        if (d_faces) cudaFree(d_faces);
        if (d_tris) cudaFree(d_tris);
    };
    if (cudaMalloc((void**)&d_pos, sizeof(float) * 3 * (nv ? nv : 1)) != cudaSuccess ||
        cudaMalloc((void**)&d_faces, sizeof(uint32_t) * 3 * nf) != cudaSuccess ||
        cudaMalloc((void**)&d_tris, sizeof(float) * 9 * nf) != cudaSuccess) {
        release();
        lmgpu::set_error(std::string(name) + ": cudaMalloc failed");
        return LMGPU_ERR_CUDA;
    }
    std::vector<lmgpu_mesh> dev(meshes, meshes + n);
    uint64_t ov = 0, of = 0;
    for (uint32_t i = 0; i < n; i++) {
        const lmgpu_mesh& m = meshes[i];
        if (m.num_vertices > 0 && m.positions &&
            cudaMemcpy(d_pos + 3 * ov, m.positions, sizeof(float) * 3 * m.num_vertices, cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            release();
            lmgpu::set_error(std::string(name) + ": position upload failed");
            return LMGPU_ERR_CUDA;
        }
        if (m.num_faces > 0 &&
            cudaMemcpy(d_faces + 3 * of, m.faces, sizeof(uint32_t) * 3 * m.num_faces, cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            release();
            lmgpu::set_error(std::string(name) + ": face upload failed");
            return LMGPU_ERR_CUDA;
        }
        dev[i].positions = d_pos + 3 * ov;
        dev[i].faces = d_faces + 3 * of;
        ov += m.num_vertices;
        of += m.num_faces;
    }
    int rc = lmgpu::flatten(dev.data(), n, d_tris, nullptr, nullptr, name);
    if (rc == LMGPU_OK) rc = lmgpu_accel_build_device(a, d_tris, nf, nullptr);
    if (rc == LMGPU_OK) {
        const cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            lmgpu::set_error(std::string(name) + ": " + cudaGetErrorString(e));
            rc = LMGPU_ERR_CUDA;
        }
    }
    release();
    return rc;
}

}  // extern "C"
