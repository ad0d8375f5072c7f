// Command-line driver around the reference's own
// IntersectionUtils::CreateTriangleIntersection (intersectionutils.h:59-135),
// compiled from the reference headers as a CPU oracle: the surface geometry
// (p, gn, sn, dpdu, dpdv, dndu, dndv, uv) an Accel3 returns for a hit.
//
// Usage: ref_isect <in.bin> <out.bin>
//   in.bin : u32 nprims; per primitive
//              f64 transform[16] (column-major, m[c][r]), u32 nverts, u32 nfaces,
//              u32 flags (1: per-vertex normals, 2: per-vertex texcoords),
//              f64 positions[nverts*3], [f64 normals[nverts*3]], [f64 texcoords[nverts*2]],
//              u32 faces[nfaces*3]
//            u32 nq; per query i32 prim, i32 face, f64 o[3], f64 d[3], f64 t, f64 b[2]
//   out.bin: u32 ntri; per triangle of the scene in global order (faces of
//            primitive 0, then 1, ...): f64 p[9] (vertices through the primitive
//            transform), f64 n[9] (normals through the normal transform, zero
//            without normals), f64 uv[6], u32 flags;
//            u32 nq; per query f64 p[3] gn[3] sn[3] dpdu[3] dpdv[3] dndu[3]
//            dndv[3] uv[2], i32 faceindex
// The hit point is p = o + d * t in the reference's arithmetic, as an accel's
// Intersect computes it before calling CreateTriangleIntersection.  The
// primitive's normal transform is Transpose(Inverse(transform)) as
// Scene3::Initialize sets it (scene3.cpp:293).
#include <pch.h>
#include <lightmetrica/component.h>
#include <lightmetrica/trianglemesh.h>
#include <lightmetrica/primitive.h>
#include <lightmetrica/intersection.h>
#include <lightmetrica/intersectionutils.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

LM_NAMESPACE_BEGIN

class IsectMesh : public TriangleMesh
{
public:
    LM_IMPL_CLASS(IsectMesh, TriangleMesh);
public:
    LM_IMPL_F(NumVertices) = [this]() -> int { return (int)(ps.size() / 3); };
    LM_IMPL_F(NumFaces)    = [this]() -> int { return (int)(fs.size() / 3); };
    LM_IMPL_F(Positions)   = [this]() -> const Float* { return ps.data(); };
    LM_IMPL_F(Normals)     = [this]() -> const Float* { return ns.empty() ? nullptr : ns.data(); };
    LM_IMPL_F(Texcoords)   = [this]() -> const Float* { return ts.empty() ? nullptr : ts.data(); };
    LM_IMPL_F(Faces)       = [this]() -> const unsigned int* { return fs.data(); };
public:
    std::vector<Float> ps, ns, ts;
    std::vector<unsigned int> fs;
};

LM_NAMESPACE_END

using namespace lightmetrica_v2;

namespace {

struct Reader {
    const char* p;
    const char* end;
    template <typename T>
    T get()
    {
        T v;
        if (p + sizeof(T) > end) throw std::runtime_error("truncated input");
        std::memcpy(&v, p, sizeof(T));
        p += sizeof(T);
        return v;
    }
};

void put3(std::vector<double>& o, const Vec3& v)
{
    o.push_back((double)v.x);
    o.push_back((double)v.y);
    o.push_back((double)v.z);
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    std::vector<char> buf;
    {
        FILE* f = std::fopen(argv[1], "rb");
        if (!f) return 3;
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        buf.resize((size_t)n);
        if (std::fread(buf.data(), 1, (size_t)n, f) != (size_t)n) return 4;
        std::fclose(f);
    }
    Reader r{buf.data(), buf.data() + buf.size()};
    std::vector<std::unique_ptr<IsectMesh>> meshes;
    std::vector<std::unique_ptr<Primitive>> prims;
    std::vector<double> tri_out;
    std::vector<uint32_t> tri_flags;
    const uint32_t nprims = r.get<uint32_t>();
    for (uint32_t pi = 0; pi < nprims; pi++)
    {
        double m[16];
        for (int k = 0; k < 16; k++) m[k] = r.get<double>();
        const uint32_t nv = r.get<uint32_t>(), nf = r.get<uint32_t>(), flags = r.get<uint32_t>();
        std::unique_ptr<IsectMesh> mesh(new IsectMesh);
        for (uint32_t k = 0; k < 3 * nv; k++) mesh->ps.push_back((Float)r.get<double>());
        if (flags & 1u) for (uint32_t k = 0; k < 3 * nv; k++) mesh->ns.push_back((Float)r.get<double>());
        if (flags & 2u) for (uint32_t k = 0; k < 2 * nv; k++) mesh->ts.push_back((Float)r.get<double>());
        for (uint32_t k = 0; k < 3 * nf; k++) mesh->fs.push_back(r.get<uint32_t>());
        std::unique_ptr<Primitive> prim(new Primitive);
        prim->transform = Mat4(Vec4((Float)m[0], (Float)m[1], (Float)m[2], (Float)m[3]),
                               Vec4((Float)m[4], (Float)m[5], (Float)m[6], (Float)m[7]),
                               Vec4((Float)m[8], (Float)m[9], (Float)m[10], (Float)m[11]),
                               Vec4((Float)m[12], (Float)m[13], (Float)m[14], (Float)m[15]));
        prim->normalTransform = Mat3(Math::Transpose(Math::Inverse(prim->transform)));
        prim->mesh = mesh.get();
        for (uint32_t fi = 0; fi < nf; fi++)
        {
            for (int k = 0; k < 3; k++)
            {
                const unsigned v = mesh->fs[3 * fi + k];
                put3(tri_out, Vec3(prim->transform * Vec4(mesh->ps[3 * v], mesh->ps[3 * v + 1], mesh->ps[3 * v + 2], 1_f)));
            }
            for (int k = 0; k < 3; k++)
            {
                const unsigned v = mesh->fs[3 * fi + k];
                if (flags & 1u) put3(tri_out, prim->normalTransform * Vec3(mesh->ns[3 * v], mesh->ns[3 * v + 1], mesh->ns[3 * v + 2]));
                else put3(tri_out, Vec3(0_f, 0_f, 0_f));
            }
            for (int k = 0; k < 3; k++)
            {
                const unsigned v = mesh->fs[3 * fi + k];
                tri_out.push_back((flags & 2u) ? (double)mesh->ts[2 * v] : 0.0);
                tri_out.push_back((flags & 2u) ? (double)mesh->ts[2 * v + 1] : 0.0);
            }
            tri_flags.push_back(flags & 3u);
        }
        meshes.push_back(std::move(mesh));
        prims.push_back(std::move(prim));
    }
    const uint32_t nq = r.get<uint32_t>();
    std::vector<double> q_out;
    std::vector<int32_t> q_face;
    for (uint32_t qi = 0; qi < nq; qi++)
    {
        const int32_t pi = r.get<int32_t>(), fi = r.get<int32_t>();
        double v[9];
        for (int k = 0; k < 9; k++) v[k] = r.get<double>();
        if (pi < 0 || (uint32_t)pi >= nprims) return 5;
        const Vec3 o((Float)v[0], (Float)v[1], (Float)v[2]), d((Float)v[3], (Float)v[4], (Float)v[5]);
        const Float t = (Float)v[6];
        const Intersection isect = IntersectionUtils::CreateTriangleIntersection(
            prims[pi].get(), o + d * t, Vec2((Float)v[7], (Float)v[8]), fi);
        const SurfaceGeometry& g = isect.geom;
        put3(q_out, g.p);
        put3(q_out, g.gn);
        put3(q_out, g.sn);
        put3(q_out, g.dpdu);
        put3(q_out, g.dpdv);
        put3(q_out, g.dndu);
        put3(q_out, g.dndv);
        q_out.push_back((double)g.uv.x);
        q_out.push_back((double)g.uv.y);
        q_face.push_back(g.faceindex);
    }
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 6;
    const uint32_t ntri = (uint32_t)tri_flags.size();
    std::fwrite(&ntri, 4, 1, f);
    for (uint32_t i = 0; i < ntri; i++)
    {
        std::fwrite(&tri_out[24 * (size_t)i], sizeof(double), 24, f);
        std::fwrite(&tri_flags[i], 4, 1, f);
    }
    std::fwrite(&nq, 4, 1, f);
    for (uint32_t i = 0; i < nq; i++)
    {
        std::fwrite(&q_out[23 * (size_t)i], sizeof(double), 23, f);
        std::fwrite(&q_face[i], 4, 1, f);
    }
    std::fclose(f);
    return 0;
}
