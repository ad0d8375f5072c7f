// Runs the reference-side accel plugin (plugin/accel_cuda.cpp, registered as
// "accel::cuda" by its LM_COMPONENT_REGISTER_IMPL static initialiser through
// ComponentFactory_Register) the way the reference's own code calls an accel:
// ComponentFactory::Create<Accel3>("accel::cuda") -> Initialize(nullptr) ->
// Build(&scene) -> Intersect through the portable vtable (slot 2), and the
// batch slots of plugin/accel3_batch.h (IntersectBatch = 3,
// IntersectBatchGeometry = 4).  Test infrastructure: linked with the
// reference's sources and a C-ABI implementation (on this machine the CPU
// stand-in oracle/refharness/lmgpu_cpu_fake.cpp).
//
// Usage:
//   ref_plugin accel3test simple|simple2 <mesh.bin>
//       The checks of Accel3Test.Simple / Simple2
//       (src/lightmetrica-test/test_accel3.cpp:272-345) on the test's own
//       stub mesh: 9 x 9 rays, p, gn, sn and uv within Math::EpsLarge(); the
//       same rays through IntersectBatch and IntersectBatchGeometry must give
//       the same hits.  Prints one JSON line; exit status 0 iff all pass.
//   ref_plugin trace <scene.bin> <rays.bin> <out.bin>
//       Several primitives with transforms; per ray (slot 2, then slot 4):
//       i32 hit, i32 primitive index, i32 face index, f32 p[3], gn[3], sn[3], uv[2].
//   mesh.bin  : f32 transform[16] (columns of Mat4), u32 nv, u32 nf, u32 has_n, u32 has_t,
//               f32 ps[3 nv], [f32 ns[3 nv]], [f32 ts[2 nv]], u32 fs[3 nf]
//   scene.bin : u32 nprims, then nprims records as mesh.bin
//   rays.bin  : u32 n, f32 rays[8 n] = (ox, oy, oz, tmin, dx, dy, dz, tmax)
#include <pch.h>
#include <lightmetrica/component.h>
#include <lightmetrica/accel3.h>
#include <lightmetrica/scene3.h>
#include <lightmetrica/trianglemesh.h>
#include <lightmetrica/primitive.h>
#include <lightmetrica/intersection.h>
#include <lightmetrica/ray.h>
#include "../../lightmetrica-v2_gb300/plugin/accel3_batch.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

LM_NAMESPACE_BEGIN

class PluginMesh : public TriangleMesh
{
public:
    LM_IMPL_CLASS(PluginMesh, TriangleMesh);
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

class PluginScene : public Scene3
{
public:
    LM_IMPL_CLASS(PluginScene, Scene3);
public:
    LM_IMPL_F(NumPrimitives) = [this]() -> int { return (int)prims.size(); };
    LM_IMPL_F(PrimitiveAt) = [this](int index) -> const Primitive* { return prims[index].get(); };
public:
    std::vector<std::unique_ptr<PluginMesh>> meshes;
    std::vector<std::unique_ptr<Primitive>> prims;
};

LM_NAMESPACE_END

using namespace lightmetrica_v2;

namespace {

bool ReadAll(const char* path, std::vector<char>& buf)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize((size_t)n);
    const bool ok = std::fread(buf.data(), 1, (size_t)n, f) == (size_t)n;
    std::fclose(f);
    return ok;
}

template <typename T> T Rd(const char*& p) { T v; std::memcpy(&v, p, sizeof(T)); p += sizeof(T); return v; }

// One primitive record (mesh.bin layout) into the scene.
void ReadPrimitive(const char*& p, PluginScene& scene)
{
    float m[16];
    for (int k = 0; k < 16; k++) m[k] = Rd<float>(p);
    const uint32_t nv = Rd<uint32_t>(p), nf = Rd<uint32_t>(p), hasN = Rd<uint32_t>(p), hasT = Rd<uint32_t>(p);
    std::unique_ptr<PluginMesh> mesh(new PluginMesh);
    mesh->ps.resize(3 * (size_t)nv);
    for (auto& v : mesh->ps) v = (Float)Rd<float>(p);
    if (hasN) { mesh->ns.resize(3 * (size_t)nv); for (auto& v : mesh->ns) v = (Float)Rd<float>(p); }
    if (hasT) { mesh->ts.resize(2 * (size_t)nv); for (auto& v : mesh->ts) v = (Float)Rd<float>(p); }
    mesh->fs.resize(3 * (size_t)nf);
    for (auto& v : mesh->fs) v = Rd<uint32_t>(p);
    std::unique_ptr<Primitive> prim(new Primitive);
    prim->index = (int)scene.prims.size();
    prim->transform = Mat4(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12], m[13],
                           m[14], m[15]);
    // scene3.cpp:293
    prim->normalTransform = Mat3(Math::Transpose(Math::Inverse(prim->transform)));
    prim->mesh = mesh.get();
    scene.meshes.push_back(std::move(mesh));
    scene.prims.push_back(std::move(prim));
}

// ExpectVecNear of the reference's tests (include/lightmetrica-test/mathutils.h:76-104):
// every component within eps.
template <typename V> bool Near(const V& a, const V& b, int n, Float eps)
{
    for (int k = 0; k < n; k++)
        if (std::abs(a[k] - b[k]) > eps) return false;
    return true;
}

std::unique_ptr<Accel3Batch, ReleaseFuncPointerType> CreateAccel()
{
    return ComponentFactory::Create<Accel3Batch>("accel::cuda");
}

int Accel3TestMode(const std::string& which, const char* meshPath)
{
    std::vector<char> b;
    if (!ReadAll(meshPath, b)) return 2;
    const char* p = b.data();
    PluginScene scene;
    ReadPrimitive(p, scene);
    auto accel = CreateAccel();
    if (!accel) { std::fprintf(stderr, "accel::cuda is not registered\n"); return 3; }
    if (!accel->Initialize(nullptr) || !accel->Build(&scene)) { std::fprintf(stderr, "Initialize/Build failed\n"); return 4; }

    // test_accel3.cpp:283-307 (Simple) and :322-344 (Simple2)
    const bool simple2 = which == "simple2";
    const int Steps = 10;
    const Float Delta = 1_f / Float(Steps);
    std::vector<Ray> rays;
    std::vector<Vec3> expP;
    std::vector<Vec2> expUV;
    for (int i = 1; i < Steps; i++)
    {
        const Float y = Delta * Float(i);
        for (int j = 1; j < Steps; j++)
        {
            const Float x = Delta * Float(j);
            Ray ray;
            if (simple2) { ray.o = Vec3(x, y, 1); ray.d = Vec3(0, 0, -1); expP.push_back(Vec3(x, y, -x)); }
            else { ray.o = Vec3(0, 0, 1); ray.d = Math::Normalize(Vec3(x, y, 0) - ray.o); expP.push_back(Vec3(x, y, 0)); }
            expUV.push_back(Vec2(x, y));
            rays.push_back(ray);
        }
    }
    const Vec3 expN = simple2 ? Math::Normalize(Vec3(1, 0, 1)) : Vec3(0, 0, 1);
    const Float eps = Math::EpsLarge();
    const long long n = (long long)rays.size();

    int failed = 0, missed = 0, batchMismatch = 0, geomMismatch = 0;
    std::vector<Intersection> single((size_t)n);
    for (long long i = 0; i < n; i++)
    {
        Intersection& isect = single[(size_t)i];
        if (!accel->Intersect(&scene, rays[(size_t)i], isect, 0_f, Math::Inf())) { missed++; failed++; continue; }
        const bool ok = Near(expP[(size_t)i], isect.geom.p, 3, eps) && Near(expN, isect.geom.gn, 3, eps) &&
                        Near(expN, isect.geom.sn, 3, eps) && Near(expUV[(size_t)i], isect.geom.uv, 2, eps);
        if (!ok) failed++;
    }
    // slot 3: raw hits of the same rays
    std::vector<float> r(8 * (size_t)n);
    for (long long i = 0; i < n; i++)
    {
        const Ray& ray = rays[(size_t)i];
        const float v[8] = { (float)ray.o.x, (float)ray.o.y, (float)ray.o.z, 0.f,
                             (float)ray.d.x, (float)ray.d.y, (float)ray.d.z, (float)Math::Inf() };
        std::memcpy(&r[8 * (size_t)i], v, sizeof(v));
    }
    struct Hit { float t; int32_t prim; float b1, b2; };
    std::vector<Hit> hits((size_t)n);
    if (!accel->IntersectBatch(r.data(), hits.data(), n, false)) return 5;
    for (long long i = 0; i < n; i++)
        if (hits[(size_t)i].prim != single[(size_t)i].geom.faceindex) batchMismatch++;
    // slot 4: Intersection records of the whole batch
    std::vector<Intersection> geo((size_t)n);
    std::unique_ptr<bool[]> hit(new bool[(size_t)n]);
    if (!accel->IntersectBatchGeometry(&scene, rays.data(), geo.data(), hit.get(), n, 0_f, Math::Inf())) return 5;
    for (long long i = 0; i < n; i++)
    {
        const auto& a = single[(size_t)i].geom;
        const auto& g = geo[(size_t)i].geom;
        const bool ok = hit[(size_t)i] && g.faceindex == a.faceindex && geo[(size_t)i].primitive == single[(size_t)i].primitive &&
                        Near(a.p, g.p, 3, eps) && Near(a.gn, g.gn, 3, eps) && Near(a.sn, g.sn, 3, eps) &&
                        Near(a.uv, g.uv, 2, eps) && Near(expP[(size_t)i], g.p, 3, eps);
        if (!ok) geomMismatch++;
    }
    std::printf("{\"case\": \"%s\", \"rays\": %lld, \"failed\": %d, \"missed\": %d, \"batch_mismatch\": %d, "
                "\"geometry_mismatch\": %d}\n", which.c_str(), n, failed, missed, batchMismatch, geomMismatch);
    return failed || batchMismatch || geomMismatch ? 1 : 0;
}

int TraceMode(const char* scenePath, const char* raysPath, const char* outPath)
{
    std::vector<char> sb, rb;
    if (!ReadAll(scenePath, sb) || !ReadAll(raysPath, rb)) return 2;
    const char* p = sb.data();
    PluginScene scene;
    const uint32_t np = Rd<uint32_t>(p);
    for (uint32_t i = 0; i < np; i++) ReadPrimitive(p, scene);
    const char* q = rb.data();
    const uint32_t n = Rd<uint32_t>(q);
    const float* r = reinterpret_cast<const float*>(q);
    auto accel = CreateAccel();
    if (!accel || !accel->Initialize(nullptr) || !accel->Build(&scene)) return 4;
    std::vector<Ray> rays(n);
    for (uint32_t i = 0; i < n; i++)
    {
        rays[i].o = Vec3(r[8 * i], r[8 * i + 1], r[8 * i + 2]);
        rays[i].d = Vec3(r[8 * i + 4], r[8 * i + 5], r[8 * i + 6]);
    }
    struct Rec { int32_t hit, prim, face; float p[3], gn[3], sn[3], uv[2]; };
    auto pack = [](bool h, const Intersection& is) {
        Rec rec;
        std::memset(&rec, 0, sizeof(rec));
        rec.hit = h ? 1 : 0;
        rec.prim = h ? is.primitive->index : -1;
        rec.face = h ? is.geom.faceindex : -1;
        if (h)
            for (int k = 0; k < 3; k++)
            {
                rec.p[k] = (float)is.geom.p[k];
                rec.gn[k] = (float)is.geom.gn[k];
                rec.sn[k] = (float)is.geom.sn[k];
                if (k < 2) rec.uv[k] = (float)is.geom.uv[k];
            }
        return rec;
    };
    std::vector<Rec> out(2 * (size_t)n);
    // every ray carries its own range; the batch slot takes one range, so the
    // rays file uses one (tmin, tmax) for all
    const Float minT = n ? (Float)r[3] : 0_f, maxT = n ? (Float)r[7] : Math::Inf();
    for (uint32_t i = 0; i < n; i++)
    {
        Intersection isect;
        const bool h = accel->Intersect(&scene, rays[i], isect, minT, maxT);
        out[i] = pack(h, isect);
    }
    std::vector<Intersection> geo(n);
    std::unique_ptr<bool[]> hit(new bool[n]);
    if (!accel->IntersectBatchGeometry(&scene, rays.data(), geo.data(), hit.get(), (long long)n, minT, maxT)) return 5;
    for (uint32_t i = 0; i < n; i++) out[n + i] = pack(hit[i], geo[i]);
    FILE* f = std::fopen(outPath, "wb");
    if (!f) return 6;
    std::fwrite(out.data(), sizeof(Rec), out.size(), f);
    std::fclose(f);
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc == 4 && std::string(argv[1]) == "accel3test") return Accel3TestMode(argv[2], argv[3]);
    if (argc == 5 && std::string(argv[1]) == "trace") return TraceMode(argv[2], argv[3], argv[4]);
    std::fprintf(stderr, "usage: %s accel3test simple|simple2 mesh.bin | trace scene.bin rays.bin out.bin\n", argv[0]);
    return 2;
}
