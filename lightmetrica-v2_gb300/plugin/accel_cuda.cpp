/*
    accel::cuda -- Lightmetrica v2 plugin that answers Accel3 queries with the
    lmgpu library (GPU-built binned-SAH BVH8, watertight traversal on sm_103a).

    This file is compiled inside the reference tree as a plugin
    (plugin/accel_cuda/, cmake/AddPlugin.cmake:26-61) and linked against
    liblmgpu.so; a scene file then selects it with

        accel:
          type: cuda

    in place of accel::embree / accel::nanort (src/lightmetrica/main.cpp:617).

    Interface followed:
      Accel::Initialize      include/lightmetrica/accel.h:67
      Accel::Build           include/lightmetrica/accel.h:79
      Accel3::Intersect      include/lightmetrica/accel3.h:68
      Accel3Batch::IntersectBatch, IntersectBatchGeometry
                             accel3_batch.h (this plugin's batch extension)
    Geometry is read the way accel_naive.cpp:59-90 reads it (primitive
    transform applied to every vertex, global triangle id = faces of
    primitive 0, then primitive 1, ...), and hits are turned into an
    Intersection with IntersectionUtils::CreateTriangleIntersection
    (intersectionutils.h:59), exactly as the in-tree accels do.
*/
#include <pch.h>
#include "accel3_batch.h"
#include <lightmetrica/scene3.h>
#include <lightmetrica/primitive.h>
#include <lightmetrica/trianglemesh.h>
#include <lightmetrica/intersection.h>
#include <lightmetrica/intersectionutils.h>
#include <lightmetrica/ray.h>
#include <lightmetrica/logger.h>
#include <lmgpu.h>

#include <vector>

LM_NAMESPACE_BEGIN

class Accel_CUDA final : public Accel3Batch
{
public:

    LM_IMPL_CLASS(Accel_CUDA, Accel3Batch);

public:

    ~Accel_CUDA()
    {
        lmgpu_accel_destroy(accel_);
    }

public:

    LM_IMPL_F(Initialize) = [this](const PropertyNode* prop) -> bool
    {
        if (lmgpu_accel_create(&accel_) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("accel::cuda: ") + lmgpu_last_error());
            return false;
        }
        return true;
    };

    LM_IMPL_F(Build) = [this](const Scene* scene_) -> bool
    {
        const auto* scene = static_cast<const Scene3*>(scene_);
        // the meshes as the primitives hold them, flattened and transformed
        // on the GPU (lmgpu_accel_build_meshes) in the global order the
        // reference's accels use (accel_naive.cpp:59-90)
        primOf_.clear();
        faceOf_.clear();
        std::vector<lmgpu_mesh> meshes;
        std::vector<std::vector<float>> pos32;       // Float -> float where Float is double
        std::vector<std::vector<uint32_t>> faces32;  // unsigned int -> uint32_t where they differ
        const int np = scene->NumPrimitives();
        for (int i = 0; i < np; i++)
        {
            const auto* prim = scene->PrimitiveAt(i);
            const auto* mesh = prim->mesh;
            if (!mesh) continue;
            lmgpu_mesh m = {};
            m.num_vertices = (uint32_t)mesh->NumVertices();
            m.num_faces = (uint32_t)mesh->NumFaces();
            pos32.emplace_back(mesh->Positions(), mesh->Positions() + 3 * (size_t)m.num_vertices);
            faces32.emplace_back(mesh->Faces(), mesh->Faces() + 3 * (size_t)m.num_faces);
            for (int c = 0; c < 4; c++)
                for (int r = 0; r < 4; r++) m.transform[4 * c + r] = (float)prim->transform[c][r];
            meshes.push_back(m);
            for (int j = 0; j < mesh->NumFaces(); j++)
            {
                primOf_.push_back(i);
                faceOf_.push_back(j);
            }
        }
        for (size_t k = 0; k < meshes.size(); k++)
        {
            meshes[k].positions = pos32[k].data();
            meshes[k].faces = faces32[k].data();
        }
        if (lmgpu_accel_build_meshes(accel_, meshes.data(), (uint32_t)meshes.size()) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("accel::cuda: ") + lmgpu_last_error());
            return false;
        }
        // shading attributes for the batched surface geometry, per triangle
        // as CreateTriangleIntersection reads them (intersectionutils.h:84-115)
        std::vector<float> normals(9 * primOf_.size(), 0.0f), texcoords(6 * primOf_.size(), 0.0f);
        std::vector<uint8_t> flags(primOf_.size(), 0);
        for (size_t t = 0; t < primOf_.size(); t++)
        {
            const auto* prim = scene->PrimitiveAt(primOf_[t]);
            const auto* mesh = prim->mesh;
            const auto* fs = mesh->Faces();
            const auto* ns = mesh->Normals();
            const auto* tc = mesh->Texcoords();
            for (int k = 0; k < 3; k++)
            {
                const unsigned int v = fs[3 * faceOf_[t] + k];
                if (ns)
                {
                    const Vec3 n = prim->normalTransform * Vec3(ns[3 * v], ns[3 * v + 1], ns[3 * v + 2]);
                    normals[9 * t + 3 * k] = (float)n.x;
                    normals[9 * t + 3 * k + 1] = (float)n.y;
                    normals[9 * t + 3 * k + 2] = (float)n.z;
                }
                if (tc)
                {
                    texcoords[6 * t + 2 * k] = (float)tc[2 * v];
                    texcoords[6 * t + 2 * k + 1] = (float)tc[2 * v + 1];
                }
            }
            flags[t] = (uint8_t)((ns ? 1 : 0) | (tc ? 2 : 0));
        }
        if (lmgpu_accel_set_attributes(accel_, normals.data(), texcoords.data(), flags.data(),
                                       (uint64_t)primOf_.size()) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("accel::cuda: ") + lmgpu_last_error());
            return false;
        }
        return true;
    };

    LM_IMPL_F(Intersect) = [this](const Scene* scene_, const Ray& ray, Intersection& isect, Float minT, Float maxT) -> bool
    {
        const float r[8] = { (float)ray.o.x, (float)ray.o.y, (float)ray.o.z, (float)minT,
                             (float)ray.d.x, (float)ray.d.y, (float)ray.d.z, (float)maxT };
        lmgpu_hit h;
        if (lmgpu_trace(accel_, r, &h, 1, 0) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("accel::cuda: ") + lmgpu_last_error());
            return false;
        }
        if (h.prim < 0) return false;
        const auto* scene = static_cast<const Scene3*>(scene_);
        isect = IntersectionUtils::CreateTriangleIntersection(
            scene->PrimitiveAt(primOf_[h.prim]), ray.o + ray.d * (Float)h.t, Vec2((Float)h.b1, (Float)h.b2), faceOf_[h.prim]);
        return true;
    };

    // Accel3Batch::IntersectBatch (slot 3): n rays in host memory, one
    // lmgpu_hit per ray.
    LM_IMPL_F(IntersectBatch) = [this](const float* rays, void* hits, long long n, bool anyHit) -> bool
    {
        if (lmgpu_trace(accel_, rays, static_cast<lmgpu_hit*>(hits), (uint64_t)n, anyHit ? 1 : 0) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("accel::cuda: ") + lmgpu_last_error());
            return false;
        }
        return true;
    };

    // Accel3Batch::IntersectBatchGeometry (slot 4): closest hits and their
    // surface geometry for a whole batch, composed into Intersection records.
    LM_IMPL_F(IntersectBatchGeometry) = [this](const Scene* scene_, const Ray* rays, Intersection* isects, bool* hit,
                                               long long n, Float minT, Float maxT) -> bool
    {
        if (n <= 0) return true;
        const auto* scene = static_cast<const Scene3*>(scene_);
        std::vector<float> r(8 * (size_t)n);
        for (long long i = 0; i < n; i++)
        {
            const float v[8] = { (float)rays[i].o.x, (float)rays[i].o.y, (float)rays[i].o.z, (float)minT,
                                 (float)rays[i].d.x, (float)rays[i].d.y, (float)rays[i].d.z, (float)maxT };
            std::copy(v, v + 8, &r[8 * (size_t)i]);
        }
        std::vector<lmgpu_hit> h((size_t)n);
        std::vector<float> g((size_t)LMGPU_SURFACE_PLANES * (size_t)n);
        if (lmgpu_trace(accel_, r.data(), h.data(), (uint64_t)n, 0) != LMGPU_OK ||
            lmgpu_surface(accel_, r.data(), h.data(), (uint64_t)n, g.data()) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("accel::cuda: ") + lmgpu_last_error());
            return false;
        }
        const size_t N = (size_t)n;
        auto plane3 = [&](int k, size_t i) { return Vec3((Float)g[k * N + i], (Float)g[(k + 1) * N + i], (Float)g[(k + 2) * N + i]); };
        for (size_t i = 0; i < N; i++)
        {
            hit[i] = h[i].prim >= 0;
            if (!hit[i]) continue;
            Intersection& isect = isects[i];
            isect = Intersection();
            isect.primitive = scene->PrimitiveAt(primOf_[h[i].prim]);
            SurfaceGeometry& geom = isect.geom;
            geom.faceindex = faceOf_[h[i].prim];
            geom.degenerated = false;
            geom.p = plane3(0, i);
            geom.gn = plane3(3, i);
            geom.sn = plane3(6, i);
            geom.dpdu = plane3(9, i);
            geom.dpdv = plane3(12, i);
            geom.dndu = plane3(15, i);
            geom.dndv = plane3(18, i);
            geom.uv = Vec2((Float)g[21 * N + i], (Float)g[22 * N + i]);
            geom.ToWorld = Mat3(geom.dpdu, geom.dpdv, geom.sn);
            geom.ToLocal = Math::Transpose(geom.ToWorld);
        }
        return true;
    };

private:

    lmgpu_accel* accel_ = nullptr;
    std::vector<int> primOf_;
    std::vector<int> faceOf_;

};

LM_COMPONENT_REGISTER_IMPL(Accel_CUDA, "accel::cuda");

LM_NAMESPACE_END
