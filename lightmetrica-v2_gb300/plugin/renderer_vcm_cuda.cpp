/*
    renderer::vcm_cuda -- Lightmetrica v2 plugin that renders renderer::vcm's
    estimator (src/liblightmetrica/renderer/renderer_vcm.cpp: vertex
    connection and merging over num_iteration_pass passes) with the lmgpu
    VCM renderer on the GPU.

    Built inside the reference tree as a plugin (plugin/renderer_vcm_cuda/,
    cmake/AddPlugin.cmake:26-61) linked against liblmgpu.so; a scene file
    selects it with

        renderer:
          type: vcm_cuda
          params:
            max_num_vertices: 10
            num_iteration_pass: 100
            num_photon_trace_samples: 1000000
            num_eye_trace_samples: 1000000
            initial_radius: 0.05
            alpha: 0.7
            mode: vcm

    Interface followed:
      Renderer::Initialize   include/lightmetrica/renderer.h:68 (the
                             parameters and defaults of renderer::vcm,
                             renderer_vcm.cpp:573-593; mode vcm, bdpt or bdpm)
      Renderer::Render       include/lightmetrica/renderer.h:81
    max_num_vertices must be in [1, 16]: the reference's subpaths have no
    roulette, so an unbounded length (-1) has no GPU form and is rejected.
*/
#include <pch.h>
#include <lightmetrica/renderer.h>
#include <lightmetrica/property.h>
#include <lightmetrica/random.h>
#include "lmgpu_scene_export.h"

LM_NAMESPACE_BEGIN

class Renderer_VCM_CUDA final : public Renderer
{
public:

    LM_IMPL_CLASS(Renderer_VCM_CUDA, Renderer);

public:

    LM_IMPL_F(Initialize) = [this](const PropertyNode* p) -> bool
    {
        prm_ = {};
        prm_.max_num_vertices = p->ChildAs<int>("max_num_vertices", 10);
        prm_.min_num_vertices = p->ChildAs<int>("min_num_vertices", 0);
        prm_.num_iteration_pass = (uint64_t)p->ChildAs<long long>("num_iteration_pass", 100L);
        prm_.num_photon_trace_samples = (uint64_t)p->ChildAs<long long>("num_photon_trace_samples", 10000L);
        prm_.num_eye_trace_samples = (uint64_t)p->ChildAs<long long>("num_eye_trace_samples", 10000L);
        prm_.initial_radius = (float)p->ChildAs<Float>("initial_radius", 0.1_f);
        prm_.alpha = (float)p->ChildAs<Float>("alpha", 0.7_f);
        const auto mode = p->ChildAs<std::string>("mode", "vcm");
        if (mode == "vcm") prm_.mode = LMGPU_VCM_MODE_VCM;
        else if (mode == "bdpt") prm_.mode = LMGPU_VCM_MODE_BDPT;
        else if (mode == "bdpm") prm_.mode = LMGPU_VCM_MODE_BDPM;
        else
        {
            LM_LOG_ERROR("renderer::vcm_cuda: unknown mode '" + mode + "'");
            return false;
        }
        if (prm_.max_num_vertices < 1 || prm_.max_num_vertices > 16)
        {
            LM_LOG_ERROR("renderer::vcm_cuda: max_num_vertices must be in [1, 16]");
            return false;
        }
        return true;
    };

    LM_IMPL_F(Render) = [this](const Scene* scene_, Random* initRng, const std::string& outputPath) -> void
    {
        const auto* scene = static_cast<const Scene3*>(scene_);
        LmgpuSceneArrays a;
        if (!lmgpu_export::Export(scene, a)) return;
        lmgpu_scene* sc = lmgpu_export::Create(a);
        if (!sc) return;
        const long long npix = (long long)a.camera.width * a.camera.height;
        lmgpu_vcm_params prm = prm_;
        prm.seed = initRng->NextUInt();
        std::vector<float> img((size_t)npix * 3);
        if (lmgpu_render_vcm(sc, &prm, img.data(), nullptr) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("renderer::vcm_cuda: ") + lmgpu_last_error());
            lmgpu_scene_destroy(sc);
            return;
        }
        lmgpu_scene_destroy(sc);
        lmgpu_export::WriteFilm(a.film, img);
        a.film->Save(outputPath);
    };

private:

    lmgpu_vcm_params prm_ = {};

};

LM_COMPONENT_REGISTER_IMPL(Renderer_VCM_CUDA, "renderer::vcm_cuda");

LM_NAMESPACE_END
