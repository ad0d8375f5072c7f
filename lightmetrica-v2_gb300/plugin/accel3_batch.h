/*
    Accel3Batch -- the batch query interface a GPU accel adds to the
    reference's Accel3 (include/lightmetrica/accel3.h:39-71).  Not part of
    the reference: its renderers call Accel3::Intersect once per ray; callers
    aware of this interface hand the accel whole ray batches instead.

    Slot numbering follows the reference's cumulative interface IDs
    (Accel: Initialize = 0, Build = 1; Accel3: Intersect = 2), so
    IntersectBatch occupies slot 3 and IntersectBatchGeometry slot 4.
*/
#pragma once

#include <lightmetrica/accel3.h>
#include <lightmetrica/intersection.h>
#include <lightmetrica/ray.h>

LM_NAMESPACE_BEGIN

class Accel3Batch : public Accel3
{
public:

    LM_INTERFACE_CLASS(Accel3Batch, Accel3, 2);

public:

    Accel3Batch() = default;
    LM_DISABLE_COPY_AND_MOVE(Accel3Batch);

public:

    /*!
        Closest (anyHit = false) or any (anyHit = true) hit of n rays.
        rays: n x (ox, oy, oz, tmin, dx, dy, dz, tmax) floats, host memory;
        hits: n x (float t, int32 prim, float b1, float b2), prim = -1 for a
        miss, with (b1, b2) the barycentrics of vertices 2 and 3 of global
        triangle prim (the order of accel_naive.cpp:62-87).
    */
    LM_INTERFACE_F(0, IntersectBatch, bool(const float* rays, void* hits, long long n, bool anyHit));

    /*!
        Closest hits of n rays with their full Intersection records: for
        every ray, what Accel3::Intersect(scene, rays[i], isects[i], minT,
        maxT) gives (hit[i] its return value), with the surface geometry of
        IntersectionUtils::CreateTriangleIntersection computed for the
        whole batch on the GPU.  The batched form of Scene3::Intersect for
        CPU renderers.
    */
    LM_INTERFACE_F(1, IntersectBatchGeometry, bool(const Scene* scene, const Ray* rays, Intersection* isects,
                                                   bool* hit, long long n, Float minT, Float maxT));

};

LM_NAMESPACE_END
