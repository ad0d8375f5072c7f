/*
    Scene export for the lmgpu renderer plugins: turns the reference's Scene3
    into the flat arrays of lmgpu_scene_create (include/lmgpu.h).

    Read through the public interfaces only:
      geometry   Scene3::NumPrimitives / PrimitiveAt (scene3.h:82-88),
                 Primitive::{transform, mesh} (primitive.h:56-80),
                 TriangleMesh::{Positions, Faces, NumFaces}; global triangle
                 order as accel_naive.cpp:59-90 enumerates it;
      BSDFs      the component key (Component::createKey, component.h:178)
                 names the kind; bsdf::diffuse and bsdf::cook_torrance give R
                 through BSDF::Reflectance and the roughness through
                 BSDF::Glossiness (bsdf.h:55-58); bsdf::flesnel gives
                 eta1 / eta2 through BSDF::Eta (bsdf.h:64) and R through one
                 EvaluateDirection of normal-incidence transmission divided by
                 its known Fresnel factor; the conductor eta / k of
                 bsdf::cook_torrance are not exposed by the BSDF interface,
                 so the reference's defaults (bsdf_cooktorrance.cpp:61-62)
                 are used;
      lights     light::area: Light::Emittance (light.h:57); light::env
                 without an envmap: its constant Le from
                 EvaluateDirection (light_env.cpp:199-216);
      sensor     the sensor primitive's transform (lookat basis,
                 scene3.cpp:213-221) and Sensor::GetProjectionMatrix
                 (sensor_pinhole.cpp:192-202) for the vertical fov; the film
                 for the resolution.
*/
#pragma once

#include <lightmetrica/scene3.h>
#include <lightmetrica/primitive.h>
#include <lightmetrica/trianglemesh.h>
#include <lightmetrica/bsdf.h>
#include <lightmetrica/light.h>
#include <lightmetrica/sensor.h>
#include <lightmetrica/film.h>
#include <lightmetrica/surfacegeometry.h>
#include <lightmetrica/surfaceinteraction.h>
#include <lightmetrica/logger.h>
#include <lmgpu.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

LM_NAMESPACE_BEGIN

struct LmgpuSceneArrays
{
    std::vector<float> tris;        // 9 floats per triangle, global order
    std::vector<int32_t> triPrim;   // primitive of each triangle
    std::vector<lmgpu_prim> prims;  // one per scene primitive
    lmgpu_camera camera;
    bool hasEnv = false;
    float envLe[3] = { 0.f, 0.f, 0.f };
    Film* film = nullptr;
};

namespace lmgpu_export
{
    inline auto Key(const Component* c) -> std::string
    {
        return c && c->createKey ? std::string(c->createKey) : std::string();
    }

    // A shading frame at the origin with normal +z.
    inline auto Frame() -> SurfaceGeometry
    {
        SurfaceGeometry g;
        g.degenerated = false;
        g.p = Vec3();
        g.gn = g.sn = Vec3(0_f, 0_f, 1_f);
        g.ComputeTangentSpace();
        return g;
    }

    inline auto Bsdf(const BSDF* bsdf, lmgpu_prim& p) -> bool
    {
        const auto key = Key(bsdf);
        if (!bsdf || key == "bsdf::null")
        {
            p.bsdf = LMGPU_BSDF_NULL;
            return true;
        }
        if (key == "bsdf::diffuse")
        {
            p.bsdf = LMGPU_BSDF_DIFFUSE;
            const auto R = bsdf->Reflectance().ToRGB();
            p.R[0] = (float)R.x; p.R[1] = (float)R.y; p.R[2] = (float)R.z;
            return true;
        }
        if (key == "bsdf::cook_torrance")
        {
            p.bsdf = LMGPU_BSDF_COOK_TORRANCE;
            const auto R = bsdf->Reflectance().ToRGB();
            p.R[0] = (float)R.x; p.R[1] = (float)R.y; p.R[2] = (float)R.z;
            p.roughness = (float)bsdf->Glossiness();
            return true;
        }
        if (key == "bsdf::flesnel")
        {
            p.bsdf = LMGPU_BSDF_DIELECTRIC;
            const auto g = Frame();
            const Vec3 up(0_f, 0_f, 1_f), down(0_f, 0_f, -1_f);
            // Eta(wi outside) = eta1 / eta2; only the ratio enters the BSDF
            const double eta = (double)bsdf->Eta(g, up);
            p.eta1 = 1.f;
            p.eta2 = (float)(1.0 / eta);
            // normal-incidence transmission (EL): R (1 - Fr) eta^2, Fr = ((1 - eta) / (1 + eta))^2
            const double fr = ((1.0 - eta) / (1.0 + eta)) * ((1.0 - eta) / (1.0 + eta));
            const auto fT = bsdf->EvaluateDirection(g, SurfaceInteractionType::BSDF, up, down,
                                                    TransportDirection::EL, false).ToRGB();
            const double scale = (1.0 - fr) * eta * eta;
            p.R[0] = (float)(fT.x / scale); p.R[1] = (float)(fT.y / scale); p.R[2] = (float)(fT.z / scale);
            return true;
        }
        LM_LOG_ERROR("lmgpu: unsupported BSDF '" + key + "'");
        return false;
    }

    // Fills `out` from the scene; false (with a logged reason) if the scene
    // holds something the GPU renderers do not implement.
    inline auto Export(const Scene3* scene, LmgpuSceneArrays& out) -> bool
    {
        const int np = scene->NumPrimitives();
        out.prims.assign((size_t)np, lmgpu_prim());
        for (int i = 0; i < np; i++)
        {
            const auto* prim = scene->PrimitiveAt(i);
            auto& p = out.prims[(size_t)i];
            std::memset(&p, 0, sizeof(p));
            p.eta1 = 1.f; p.eta2 = 2.f;
            p.ct_eta[0] = 0.14f;    p.ct_eta[1] = 0.129f;   p.ct_eta[2] = 0.1585f;
            p.ct_k[0]   = 4.58625f; p.ct_k[1]   = 3.348125f; p.ct_k[2]  = 2.329375f;
            p.roughness = 0.1f;
            if (!Bsdf(prim->bsdf, p)) return false;
            if (prim->light)
            {
                const auto key = Key(prim->light);
                if (key == "light::area")
                {
                    const auto Le = prim->light->Emittance().ToRGB();
                    p.is_light = 1;
                    p.Le[0] = (float)Le.x; p.Le[1] = (float)Le.y; p.Le[2] = (float)Le.z;
                }
                else if (key == "light::env")
                {
                    const auto g = Frame();
                    const Vec3 up(0_f, 0_f, 1_f);
                    const auto Le = prim->light->EvaluateDirection(g, SurfaceInteractionType::L, Vec3(), up,
                                                                   TransportDirection::LE, false).ToRGB();
                    out.hasEnv = true;
                    out.envLe[0] = (float)Le.x; out.envLe[1] = (float)Le.y; out.envLe[2] = (float)Le.z;
                }
                else
                {
                    LM_LOG_ERROR("lmgpu: unsupported light '" + key + "'");
                    return false;
                }
            }
            const auto* mesh = prim->mesh;
            if (!mesh) continue;
            const auto* ps = mesh->Positions();
            const auto* fs = mesh->Faces();
            for (int j = 0; j < mesh->NumFaces(); j++)
            {
                for (int k = 0; k < 3; k++)
                {
                    const unsigned int v = fs[3 * j + k];
                    const Vec3 q(prim->transform * Vec4(ps[3 * v], ps[3 * v + 1], ps[3 * v + 2], 1_f));
                    out.tris.push_back((float)q.x);
                    out.tris.push_back((float)q.y);
                    out.tris.push_back((float)q.z);
                }
                out.triPrim.push_back(i);
            }
        }

        // sensor: lookat basis from the transform, vertical fov from the projection
        const auto* sp = scene->GetSensor();
        const auto* sensor = static_cast<const Sensor*>(sp->emitter);
        out.film = sensor->GetFilm();
        const Vec3 eye(sp->transform * Vec4(0_f, 0_f, 0_f, 1_f));
        const Vec3 vz(sp->transform * Vec4(0_f, 0_f, 1_f, 0_f));
        const Vec3 vy(sp->transform * Vec4(0_f, 1_f, 0_f, 0_f));
        const auto P = sensor->GetProjectionMatrix(0.1_f, 100_f);
        const double tanFov = 1.0 / (double)P[1][1];
        auto& c = out.camera;
        for (int k = 0; k < 3; k++)
        {
            c.eye[k] = (float)eye[k];
            c.center[k] = (float)(eye[k] - vz[k]);
            c.up[k] = (float)vy[k];
        }
        c.fov_deg = (float)(2.0 * std::atan(tanFov) * 180.0 / 3.14159265358979323846);
        c.width = out.film->Width();
        c.height = out.film->Height();
        return true;
    }

    // Creates the lmgpu scene (BVH built on the GPU); nullptr on failure.
    inline auto Create(const LmgpuSceneArrays& a) -> lmgpu_scene*
    {
        lmgpu_scene* sc = nullptr;
        if (lmgpu_scene_create(a.tris.data(), a.triPrim.data(), (uint64_t)a.triPrim.size(), a.prims.data(),
                               (uint32_t)a.prims.size(), &a.camera, &sc) != LMGPU_OK ||
            (a.hasEnv && lmgpu_scene_set_environment(sc, a.envLe) != LMGPU_OK))
        {
            LM_LOG_ERROR(std::string("lmgpu: ") + lmgpu_last_error());
            lmgpu_scene_destroy(sc);
            return nullptr;
        }
        return sc;
    }

    // Writes an (H x W x 3) image, row 0 = raster y 0 (bottom), into the film.
    inline auto WriteFilm(Film* film, const std::vector<float>& img) -> void
    {
        const int W = film->Width(), H = film->Height();
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
            {
                const float* v = &img[3 * ((size_t)y * W + x)];
                film->SetPixel(x, y, SPD::FromRGB(Vec3((Float)v[0], (Float)v[1], (Float)v[2])));
            }
    }
}

LM_NAMESPACE_END
