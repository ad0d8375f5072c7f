// Command-line driver around the reference's own renderer::pt, renderer::bdpt,
// renderer::ptmis, renderer::ptdirect, renderer::ltdirect and renderer::vcm
// (src/liblightmetrica/renderer/renderer_{pt,bdpt,ptmis,ptdirect,ltdirect,vcm}.cpp,
// the last with SubpathSampler, subpathsampler.cpp)
// with the reference's own
// bsdf::diffuse, bsdf::null, light::area, sensor::pinhole, Random (dSFMT)
// and accel components, compiled from the reference sources as a CPU oracle.
//
// The parts of liblightmetrica that cannot be built here (boost/TBB/
// yaml-cpp/FreeImage) are replaced by small stand-ins written for this
// harness, each restating the reference behaviour it replaces:
//   HarnessProp       PropertyNode over an in-memory map (property.h:47-215)
//   HarnessAssets     Assets::AssetByIDAndType for the film only (assets.h:88)
//   HarnessFilm       Film_HDR::Splat/Accumulate/Rescale/Clear
//                     (film_hdr.cpp:218-305); additionally sums, per pixel,
//                     the square of each sample's total contribution there
//                     (a sample's splats are merged by pixel when the
//                     scheduler finishes it), which the oracle needs for
//                     per-pixel variance
//   HarnessScheduler  Scheduler_::Process (scheduler.cpp:78-295) with
//                     std::thread: each worker seeds its Random from
//                     initRng->NextUInt() in worker order, renders into its
//                     own film, then films are accumulated and rescaled by
//                     W*H / processed samples
//   Parallel          Parallel::GetNumThreads / For (parallel.h:44-71,
//                     parallel.cpp) with std::thread over contiguous index
//                     ranges; after each index the calling thread's cloned
//                     film (Film clones are made by renderer::vcm, one per
//                     thread, right before its sample loop) closes its sample
//                     for the per-pixel squares
//   HarnessFilm::Clone  Film_HDR::Clone (copies size and contents)
//   HarnessScene      Scene3 queries (scene3.cpp:458-539): Intersect with
//                     [EpsIsect, Inf] then the emitter shapes (environment),
//                     uniform light-primitive selection, the sensor, lookat
//                     camera basis (scene3.cpp:213-221), scene bound and
//                     bounding sphere (scene3.cpp:52-78).  One deliberate
//                     difference: EmitterShape_EnvLight::Intersect leaves
//                     isect.primitive unset (light_env.cpp:52-75), which makes
//                     renderer::pt dereference a null primitive on an
//                     environment hit; the harness sets it to the environment
//                     light's primitive, as a fixed scene would.
//
// Usage: ref_render <scene.bin> <out.bin> [pt|bdpt|ptmis|ptdirect|ltdirect|vcm] [key=value ...]
//        (renderer::pt by default; key=value: further renderer parameters,
//        e.g. mis=simple, min_num_vertices=3)
//   scene.bin: u32 magic 'LMRS', u32 version 2, u32 W, H,
//              f32 eye[3], center[3], up[3], fov_deg,
//              u32 nprims, per primitive: i32 bsdf (0 null, 1 diffuse,
//              2 flesnel, 3 cook_torrance), i32 is_light, f32 R[3], Le[3],
//              eta1, eta2, ct_eta[3], ct_k[3], roughness, u32 nfaces,
//              f32 pos[nfaces*9],
//              i32 has_env, f32 env_Le[3],
//              u64 num_samples, i32 max_num_vertices, u32 seed, u32 threads
//   out.bin:   f32 image[W*H*3] (the reference film after Rescale),
//              f64 sumsq[W*H*3] (sum of squared splats per pixel),
//              u64 processed samples
#include <pch.h>
#include <lightmetrica/component.h>
#include <lightmetrica/property.h>
#include <lightmetrica/assets.h>
#include <lightmetrica/film.h>
#include <lightmetrica/scheduler.h>
#include <lightmetrica/scene3.h>
#include <lightmetrica/accel3.h>
#include <lightmetrica/renderer.h>
#include <lightmetrica/random.h>
#include <lightmetrica/primitive.h>
#include <lightmetrica/trianglemesh.h>
#include <lightmetrica/intersection.h>
#include <lightmetrica/bsdf.h>
#include <lightmetrica/light.h>
#include <lightmetrica/sensor.h>
#include <lightmetrica/spectrum.h>
#include <lightmetrica/ray.h>
#include <lightmetrica/emitter.h>
#include <lightmetrica/detail/parallel.h>

#include <cstdint>
#include <map>
#include <thread>

LM_NAMESPACE_BEGIN

namespace { int g_threads = 1; }

class HarnessFilm;
namespace { std::vector<HarnessFilm*> g_clones; }  // films cloned for the current Parallel::For, by thread

class HarnessProp : public PropertyNode
{
public:
    LM_IMPL_CLASS(HarnessProp, PropertyNode);
public:
    LM_IMPL_F(Tree) = [this]() -> const PropertyTree* { return nullptr; };
    LM_IMPL_F(Type) = [this]() -> PropertyNodeType { return children.empty() ? PropertyNodeType::Scalar : PropertyNodeType::Map; };
    LM_IMPL_F(Line) = [this]() -> int { return 0; };
    LM_IMPL_F(Key) = [this]() -> std::string { return key; };
    LM_IMPL_F(RawScalar) = [this]() -> const char* { return value.c_str(); };
    LM_IMPL_F(Size) = [this]() -> int { return (int)children.size(); };
    LM_IMPL_F(Child) = [this](const std::string& name) -> const PropertyNode*
    {
        auto it = children.find(name);
        return it == children.end() ? nullptr : it->second.get();
    };
    LM_IMPL_F(At) = [this](int) -> const PropertyNode* { return nullptr; };
    LM_IMPL_F(Parent) = [this]() -> const PropertyNode* { return nullptr; };
public:
    auto Set(const std::string& name, const std::string& v) -> HarnessProp&
    {
        std::unique_ptr<HarnessProp> c(new HarnessProp);
        c->key = name;
        c->value = v;
        children[name] = std::move(c);
        return *this;
    }
    std::string key, value;
    std::map<std::string, std::unique_ptr<HarnessProp>> children;
};

class HarnessFilm : public Film
{
public:
    LM_IMPL_CLASS(HarnessFilm, Film);
public:
    LM_IMPL_F(Width) = [this]() -> int { return width; };
    LM_IMPL_F(Height) = [this]() -> int { return height; };
    LM_IMPL_F(Splat) = [this](const Vec2& rasterPos, const SPD& v) -> void
    {
        // film_hdr.cpp:218-223
        const int pX = Math::Clamp((int)(rasterPos.x * Float(width)), 0, width - 1);
        const int pY = Math::Clamp((int)(rasterPos.y * Float(height)), 0, height - 1);
        const Vec3 c = v.ToRGB();
        data[pY * width + pX] += c;
        pending.push_back({ pY * width + pX, { (double)c[0], (double)c[1], (double)c[2] } });
    };
    LM_IMPL_F(Save) = [this](const std::string&) -> bool { return true; };
    // film_hdr.cpp's SetPixel: the pixel's value replaced (the GPU renderer
    // plugins write their finished image this way)
    LM_IMPL_F(SetPixel) = [this](int x, int y, const SPD& v) -> void { data[(size_t)y * width + x] = v.ToRGB(); };
    LM_IMPL_F(Accumulate) = [this](const Film* f_) -> void
    {
        const auto* f = static_cast<const HarnessFilm*>(f_);
        for (size_t i = 0; i < data.size(); i++) data[i] += f->data[i];
        for (size_t i = 0; i < sumsq.size(); i++) sumsq[i] += f->sumsq[i];
    };
    LM_IMPL_F(Rescale) = [this](Float w) -> void { for (auto& v : data) v *= w; };
    LM_IMPL_F(Clear) = [this]() -> void
    {
        data.assign((size_t)width * height, Vec3());
        sumsq.assign((size_t)width * height * 3, 0.0);
    };
    LM_IMPL_F(Clone) = [this](BasicComponent* o) -> void
    {
        auto* f = static_cast<HarnessFilm*>(o);
        f->width = width;
        f->height = height;
        f->data = data;
        f->sumsq = sumsq;
        g_clones.push_back(f);
    };
public:
    void Resize(int w, int h) { width = w; height = h; data.assign((size_t)w * h, Vec3()); sumsq.assign((size_t)w * h * 3, 0.0); }
    // Called after every sample: squares of the sample's per-pixel totals.
    void EndSample()
    {
        for (size_t i = 0; i < pending.size(); i++)
        {
            if (pending[i].pixel < 0) continue;
            double c[3] = { pending[i].c[0], pending[i].c[1], pending[i].c[2] };
            for (size_t j = i + 1; j < pending.size(); j++)
            {
                if (pending[j].pixel != pending[i].pixel) continue;
                for (int k = 0; k < 3; k++) c[k] += pending[j].c[k];
                pending[j].pixel = -1;
            }
            for (int k = 0; k < 3; k++) sumsq[3 * (size_t)pending[i].pixel + k] += c[k] * c[k];
        }
        pending.clear();
    }
    struct Pending { int pixel; double c[3]; };
    int width = 0, height = 0;
    std::vector<Vec3> data;
    std::vector<double> sumsq;
    std::vector<Pending> pending;
};

// Parallel (parallel.h:44-71): contiguous index ranges over g_threads
// std::threads; `init` is true on a thread's first index.
auto Parallel::SetNumThreads(int numThreads) -> void { g_threads = numThreads > 0 ? numThreads : 1; }
auto Parallel::GetNumThreads() -> int { return g_threads; }
auto Parallel::For(long long numSamples, const std::function<void(long long index, int threadid, bool init)>& processFunc) -> void
{
    const int T = g_threads;
    std::vector<std::thread> ts;
    for (int t = 0; t < T; t++)
    {
        const long long b = numSamples * t / T, e = numSamples * (t + 1) / T;
        ts.emplace_back([&, t, b, e]()
        {
            for (long long i = b; i < e; i++)
            {
                processFunc(i, t, i == b);
                if (t < (int)g_clones.size()) g_clones[t]->EndSample();
            }
        });
    }
    for (auto& th : ts) th.join();
    g_clones.clear();
}

class HarnessAssets : public Assets
{
public:
    LM_IMPL_CLASS(HarnessAssets, Assets);
public:
    LM_IMPL_F(AssetByIDAndType) = [this](const std::string& id, const std::string& type, const Primitive*) -> Asset*
    {
        return (id == "film" && type == "film") ? film : nullptr;
    };
    HarnessFilm* film = nullptr;
};

class HarnessScheduler : public Scheduler
{
public:
    LM_IMPL_CLASS(HarnessScheduler, Scheduler);
public:
    LM_IMPL_F(Load) = [this](const PropertyNode* prop) -> void
    {
        numSamples = prop->ChildAs<long long>("num_samples", 10000000L);
    };
    LM_IMPL_F(GetNumSamples) = [this]() -> long long { return numSamples; };
    LM_IMPL_F(Process) = [this](const Scene*, Film* film_, Random* initRng, const std::function<void(Film*, Random*)>& func) -> long long
    {
        auto* film = static_cast<HarnessFilm*>(film_);
        const int T = g_threads;
        std::vector<std::unique_ptr<Random>> rngs;
        std::vector<std::unique_ptr<HarnessFilm>> films;
        for (int t = 0; t < T; t++)
        {
            rngs.emplace_back(new Random);
            rngs.back()->SetSeed(initRng->NextUInt());
            films.emplace_back(new HarnessFilm);
            films.back()->Resize(film->width, film->height);
        }
        std::vector<std::thread> ts;
        for (int t = 0; t < T; t++)
        {
            const long long b = numSamples * t / T, e = numSamples * (t + 1) / T;
            ts.emplace_back([&, t, b, e]() { for (long long s = b; s < e; s++) { func(films[t].get(), rngs[t].get()); films[t]->EndSample(); } });
        }
        for (auto& th : ts) th.join();
        film->Clear();
        for (auto& f : films) film->Accumulate(f.get());
        film->Rescale((Float)(film->Width() * film->Height()) / (Float)numSamples);
        return numSamples;
    };
    long long numSamples = 0;
};

class HarnessMesh : public TriangleMesh
{
public:
    LM_IMPL_CLASS(HarnessMesh, TriangleMesh);
public:
    LM_IMPL_F(NumVertices) = [this]() -> int { return (int)(ps.size() / 3); };
    LM_IMPL_F(NumFaces) = [this]() -> int { return (int)(fs.size() / 3); };
    LM_IMPL_F(Positions) = [this]() -> const Float* { return ps.data(); };
    LM_IMPL_F(Normals) = [this]() -> const Float* { return nullptr; };
    LM_IMPL_F(Texcoords) = [this]() -> const Float* { return nullptr; };
    LM_IMPL_F(Faces) = [this]() -> const unsigned int* { return fs.data(); };
public:
    std::vector<Float> ps;
    std::vector<unsigned int> fs;
};

class HarnessScene : public Scene3
{
public:
    LM_IMPL_CLASS(HarnessScene, Scene3);
public:
    LM_IMPL_F(GetAccel) = [this]() -> const Accel* { return accel; };
    LM_IMPL_F(Intersect) = [this](const Ray& ray, Intersection& isect) -> bool
    {
        bool hit = accel->Intersect(this, ray, isect, Math::EpsIsect(), Math::Inf());
        if (!hit)
        {
            Float maxT = Math::Inf();
            for (size_t i = 0; i < emitterShapes.size(); i++)
            {
                if (emitterShapes[i]->Intersect(ray, Math::EpsIsect(), maxT, isect))
                {
                    maxT = Math::Length(isect.geom.p - ray.o);
                    isect.primitive = emitterShapePrims[i];
                    hit = true;
                }
            }
        }
        return hit;
    };
    LM_IMPL_F(IntersectWithRange) = [this](const Ray& ray, Intersection& isect, Float minT, Float maxT) -> bool
    {
        return accel->Intersect(this, ray, isect, minT, maxT);
    };
    LM_IMPL_F(PrimitiveByID) = [this](const std::string&) -> const Primitive* { return nullptr; };
    LM_IMPL_F(NumPrimitives) = [this]() -> int { return (int)prims.size(); };
    LM_IMPL_F(PrimitiveAt) = [this](int i) -> const Primitive* { return prims.at(i).get(); };
    LM_IMPL_F(GetSensor) = [this]() -> const Primitive* { return prims.at(sensorIndex).get(); };
    LM_IMPL_F(SampleEmitter) = [this](int type, Float u) -> const Primitive*
    {
        // scene3.cpp:506-523
        if ((type & SurfaceInteractionType::L) > 0)
        {
            const int n = (int)lightIndices.size();
            const int i = Math::Clamp((int)(u * n), 0, n - 1);
            return prims.at(lightIndices[i]).get();
        }
        if ((type & SurfaceInteractionType::E) > 0) return prims.at(sensorIndex).get();
        return nullptr;
    };
    LM_IMPL_F(EvaluateEmitterPDF) = [this](const Primitive* p) -> PDFVal
    {
        // scene3.cpp:525-539
        if ((p->emitter->Type() & SurfaceInteractionType::L) > 0) return PDFVal(PDFMeasure::Discrete, 1_f / Float(lightIndices.size()));
        if ((p->emitter->Type() & SurfaceInteractionType::E) > 0) return PDFVal(PDFMeasure::Discrete, 1_f);
        return PDFVal(PDFMeasure::Discrete, 0_f);
    };
    LM_IMPL_F(GetBound) = [this]() -> Bound { return bound; };
    LM_IMPL_F(GetSphereBound) = [this]() -> SphereBound { return sphereBound; };
    LM_IMPL_F(NumLightPrimitives) = [this]() -> int { return (int)lightIndices.size(); };
public:
    std::vector<std::unique_ptr<Primitive>> prims;
    std::vector<int> lightIndices;
    int sensorIndex = -1;
    const Accel3* accel = nullptr;
    Bound bound;
    SphereBound sphereBound;
    std::vector<const EmitterShape*> emitterShapes;
    std::vector<const Primitive*> emitterShapePrims;
};

LM_COMPONENT_REGISTER_IMPL(HarnessScheduler, "Scheduler_");

LM_NAMESPACE_END

using namespace lightmetrica_v2;

template <typename T>
static T Rd(const char*& p) { T v; std::memcpy(&v, p, sizeof(T)); p += sizeof(T); return v; }

static std::string Vec3Str(const float* v)
{
    char buf[128];
    std::snprintf(buf, sizeof(buf), "%.9g %.9g %.9g", v[0], v[1], v[2]);
    return buf;
}

int main(int argc, char** argv)
{
    if (argc < 3) { std::fprintf(stderr, "usage: %s scene.bin out.bin [pt|bdpt|ptmis|ptdirect|ltdirect|vcm]\n", argv[0]); return 2; }
    const std::string rendererKey = std::string("renderer::") + (argc > 3 ? argv[3] : "pt");
    std::vector<char> buf;
    {
        FILE* f = std::fopen(argv[1], "rb");
        if (!f) return 2;
        std::fseek(f, 0, SEEK_END); long n = std::ftell(f); std::fseek(f, 0, SEEK_SET);
        buf.resize((size_t)n);
        if (std::fread(buf.data(), 1, (size_t)n, f) != (size_t)n) return 2;
        std::fclose(f);
    }
    const char* p = buf.data();
    if (Rd<uint32_t>(p) != 0x53524D4Cu || Rd<uint32_t>(p) != 2u) { std::fprintf(stderr, "bad scene file\n"); return 2; }
    const int W = (int)Rd<uint32_t>(p), H = (int)Rd<uint32_t>(p);
    float eye[3], center[3], up[3];
    for (auto* v : { eye, center, up }) for (int k = 0; k < 3; k++) v[k] = Rd<float>(p);
    const float fov = Rd<float>(p);
    const uint32_t nprims = Rd<uint32_t>(p);

    HarnessFilm film;
    film.Resize(W, H);
    // ComponentFactory::Clone (component.h:552-572) creates through these
    film.createFunc = []() -> Component* { return new HarnessFilm; };
    film.releaseFunc = [](Component* c) { delete static_cast<HarnessFilm*>(c); };
    HarnessAssets assets;
    assets.film = &film;
    HarnessScene scene;
    std::vector<std::unique_ptr<HarnessMesh>> meshes;
    std::vector<std::unique_ptr<Component, ReleaseFuncPointerType>> keep;
    std::vector<std::unique_ptr<HarnessProp>> props;
    auto nullBSDF = ComponentFactory::Create<BSDF>("bsdf::null");

    for (uint32_t i = 0; i < nprims; i++)
    {
        const int bsdfKind = Rd<int32_t>(p);
        const int isLight = Rd<int32_t>(p);
        float R[3], Le[3], ctEta[3], ctK[3];
        for (int k = 0; k < 3; k++) R[k] = Rd<float>(p);
        for (int k = 0; k < 3; k++) Le[k] = Rd<float>(p);
        const float eta1 = Rd<float>(p), eta2 = Rd<float>(p);
        for (int k = 0; k < 3; k++) ctEta[k] = Rd<float>(p);
        for (int k = 0; k < 3; k++) ctK[k] = Rd<float>(p);
        const float roughness = Rd<float>(p);
        const uint32_t nf = Rd<uint32_t>(p);
        std::unique_ptr<HarnessMesh> m(new HarnessMesh);
        m->ps.resize((size_t)nf * 9);
        for (size_t k = 0; k < (size_t)nf * 9; k++) m->ps[k] = (Float)Rd<float>(p);
        m->fs.resize((size_t)nf * 3);
        for (uint32_t k = 0; k < nf * 3; k++) m->fs[k] = k;
        std::unique_ptr<Primitive> prim(new Primitive);
        prim->index = (int)scene.prims.size();
        prim->transform = Mat4::Identity();
        prim->normalTransform = Mat3::Identity();
        prim->mesh = m.get();
        char fb[64];
        if (bsdfKind == 0)
        {
            prim->bsdf = nullBSDF.get();
        }
        else
        {
            static const char* keys[] = { "", "bsdf::diffuse", "bsdf::flesnel", "bsdf::cook_torrance" };
            if (bsdfKind < 1 || bsdfKind > 3) return 3;
            auto b = ComponentFactory::Create<BSDF>(keys[bsdfKind]);
            props.emplace_back(new HarnessProp);
            props.back()->Set("R", Vec3Str(R));
            if (bsdfKind == 2)
            {
                std::snprintf(fb, sizeof(fb), "%.9g", eta1); props.back()->Set("eta1", fb);
                std::snprintf(fb, sizeof(fb), "%.9g", eta2); props.back()->Set("eta2", fb);
            }
            if (bsdfKind == 3)
            {
                props.back()->Set("eta", Vec3Str(ctEta)).Set("k", Vec3Str(ctK));
                std::snprintf(fb, sizeof(fb), "%.9g", roughness); props.back()->Set("roughness", fb);
            }
            if (!b->Load(props.back().get(), &assets, prim.get())) return 3;
            prim->bsdf = b.get();
            keep.emplace_back(b.release(), b.get_deleter());
        }
        if (isLight)
        {
            auto l = ComponentFactory::Create<Light>("light::area");
            props.emplace_back(new HarnessProp);
            props.back()->Set("Le", Vec3Str(Le));
            if (!l->Load(props.back().get(), &assets, prim.get())) return 3;
            prim->light = l.get();
            prim->emitter = l.get();
            prim->lightIndex = scene.lightIndices.size();
            scene.lightIndices.push_back((int)scene.prims.size());
            keep.emplace_back(l.release(), l.get_deleter());
        }
        meshes.push_back(std::move(m));
        scene.prims.push_back(std::move(prim));
    }
    const int hasEnv = Rd<int32_t>(p);
    float envLe[3];
    for (int k = 0; k < 3; k++) envLe[k] = Rd<float>(p);
    const uint64_t numSamples = Rd<uint64_t>(p);
    const int maxNumVertices = Rd<int32_t>(p);
    const uint32_t seed = Rd<uint32_t>(p);
    g_threads = (int)Rd<uint32_t>(p);
    if (g_threads < 1) g_threads = 1;

    // Sensor primitive: lookat transform as scene3.cpp:213-221 builds it.
    {
        const Vec3 e(eye[0], eye[1], eye[2]), c(center[0], center[1], center[2]), u(up[0], up[1], up[2]);
        const auto vz = Math::Normalize(e - c);
        const auto vx = Math::Normalize(Math::Cross(u, vz));
        const auto vy = Math::Cross(vz, vx);
        std::unique_ptr<Primitive> prim(new Primitive);
        prim->index = (int)scene.prims.size();
        prim->transform = Mat4(vx.x, vx.y, vx.z, 0_f, vy.x, vy.y, vy.z, 0_f, vz.x, vz.y, vz.z, 0_f, e.x, e.y, e.z, 1_f);
        prim->normalTransform = Mat3::Identity();
        prim->bsdf = nullBSDF.get();
        auto s = ComponentFactory::Create<Sensor>("sensor::pinhole");
        props.emplace_back(new HarnessProp);
        char fb[64];
        std::snprintf(fb, sizeof(fb), "%.9g", fov);
        props.back()->Set("fov", fb).Set("film", "film");
        if (!s->Load(props.back().get(), &assets, prim.get())) return 3;
        prim->sensor = s.get();
        prim->emitter = s.get();
        keep.emplace_back(s.release(), s.get_deleter());
        scene.sensorIndex = (int)scene.prims.size();
        scene.prims.push_back(std::move(prim));
    }

    // scene bound and bounding sphere (scene3.cpp:52-78): mesh vertices and
    // the sensor position
    for (const auto& prim : scene.prims)
    {
        if (prim->mesh)
        {
            const auto* ps = prim->mesh->Positions();
            for (int i = 0; i < prim->mesh->NumVertices(); i++)
                scene.bound = Math::Union(scene.bound, Vec3(prim->transform * Vec4(ps[3 * i], ps[3 * i + 1], ps[3 * i + 2], 1_f)));
        }
        if (prim->emitter && prim->emitter->GetBound.Implemented()) scene.bound = Math::Union(scene.bound, prim->emitter->GetBound());
    }
    scene.sphereBound.center = (scene.bound.max + scene.bound.min) * .5_f;
    scene.sphereBound.radius = Math::Length(scene.sphereBound.center - scene.bound.max) * 1.01_f;
    if (hasEnv)
    {
        std::unique_ptr<Primitive> prim(new Primitive);
        prim->index = (int)scene.prims.size();
        prim->transform = Mat4::Identity();
        prim->normalTransform = Mat3::Identity();
        prim->bsdf = nullBSDF.get();
        auto l = ComponentFactory::Create<Light>("light::env");
        props.emplace_back(new HarnessProp);
        props.back()->Set("Le", Vec3Str(envLe));
        if (!l->Load(props.back().get(), &assets, prim.get())) return 3;
        if (!l->PostLoad(&scene)) return 3;
        prim->light = l.get();
        prim->emitter = l.get();
        prim->lightIndex = scene.lightIndices.size();
        scene.lightIndices.push_back((int)scene.prims.size());
        scene.emitterShapes.push_back(l->GetEmitterShape());
        scene.emitterShapePrims.push_back(prim.get());
        keep.emplace_back(l.release(), l.get_deleter());
        scene.prims.push_back(std::move(prim));
    }

#if LM_SINGLE_PRECISION && LM_SSE
    const char* accelKey = "accel::qbvh";
#else
    const char* accelKey = "accel::bvh_sahbin";
#endif
    if (const char* k = std::getenv("LM_REF_ACCEL")) accelKey = k;  // e.g. accel::bvh_sahbin
    auto accel = ComponentFactory::Create<Accel3>(accelKey);
    if (!accel || !accel->Initialize(nullptr) || !accel->Build(&scene)) return 4;
    scene.accel = accel.get();

    auto renderer = ComponentFactory::Create<Renderer>(rendererKey);
    if (!renderer) { std::fprintf(stderr, "unknown renderer %s\n", rendererKey.c_str()); return 5; }
    HarnessProp rprop;
    rprop.Set("num_samples", std::to_string(numSamples)).Set("max_num_vertices", std::to_string(maxNumVertices));
    // further renderer parameters as key=value (mis, min_num_vertices, ...)
    for (int a = 4; a < argc; a++)
    {
        const std::string kv = argv[a];
        const auto eq = kv.find('=');
        if (eq == std::string::npos) { std::fprintf(stderr, "bad parameter %s\n", argv[a]); return 2; }
        rprop.Set(kv.substr(0, eq), kv.substr(eq + 1));
    }
    if (!renderer->Initialize(&rprop)) return 5;
    Random initRng;
    initRng.SetSeed(seed);
    const auto t0 = std::chrono::high_resolution_clock::now();
    renderer->Render(&scene, &initRng, "");
    const auto t1 = std::chrono::high_resolution_clock::now();

    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 6;
    std::vector<float> img((size_t)W * H * 3);
    for (size_t i = 0; i < (size_t)W * H; i++) for (int k = 0; k < 3; k++) img[3 * i + k] = (float)film.data[i][k];
    std::fwrite(img.data(), sizeof(float), img.size(), f);
    std::fwrite(film.sumsq.data(), sizeof(double), film.sumsq.size(), f);
    std::fwrite(&numSamples, sizeof(uint64_t), 1, f);
    std::fclose(f);
    std::printf("{\"renderer\": \"%s\", \"accel\": \"%s\", \"samples\": %llu, \"threads\": %d, \"render_s\": %.6f, \"float_bytes\": %d}\n",
                rendererKey.c_str(), accelKey, (unsigned long long)numSamples, g_threads,
                std::chrono::duration<double>(t1 - t0).count(), (int)sizeof(Float));
    return 0;
}
