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
      Accel3Batch::IntersectBatch  accel3_batch.h (this plugin's batch extension)
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
        std::vector<float> tris;
        primOf_.clear();
        faceOf_.clear();
        const int np = scene->NumPrimitives();
        for (int i = 0; i < np; i++)
        {
            const auto* prim = scene->PrimitiveAt(i);
            const auto* mesh = prim->mesh;
            if (!mesh) continue;
            const auto* ps = mesh->Positions();
            const auto* fs = mesh->Faces();
            for (int j = 0; j < mesh->NumFaces(); j++)
            {
                for (int k = 0; k < 3; k++)
                {
                    const unsigned int v = fs[3 * j + k];
                    const Vec3 p(prim->transform * Vec4(ps[3 * v], ps[3 * v + 1], ps[3 * v + 2], 1_f));
                    tris.push_back((float)p.x);
                    tris.push_back((float)p.y);
                    tris.push_back((float)p.z);
                }
                primOf_.push_back(i);
                faceOf_.push_back(j);
            }
        }
        if (lmgpu_accel_build(accel_, tris.data(), (uint64_t)primOf_.size()) != LMGPU_OK)
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

private:

    lmgpu_accel* accel_ = nullptr;
    std::vector<int> primOf_;
    std::vector<int> faceOf_;

};

LM_COMPONENT_REGISTER_IMPL(Accel_CUDA, "accel::cuda");

LM_NAMESPACE_END
