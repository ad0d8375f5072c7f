/*
    renderer::bdpt_cuda -- Lightmetrica v2 plugin that renders renderer::bdpt's
    estimator (src/liblightmetrica/renderer/renderer_bdpt.cpp, power
    heuristic) with the lmgpu wavefront BDPT on the GPU.

    Built inside the reference tree as a plugin (plugin/renderer_bdpt_cuda/,
    cmake/AddPlugin.cmake:26-61) linked against liblmgpu.so; a scene file
    selects it with

        renderer:
          type: bdpt_cuda
          params:
            num_samples: 29491200
            max_num_vertices: 11

    Interface followed:
      Renderer::Initialize   include/lightmetrica/renderer.h:68 (parameters of
                             renderer::bdpt, renderer_bdpt.cpp:832-839: mis =
                             powerheuristics (the default) or simple)
      Renderer::Render       include/lightmetrica/renderer.h:81
    num_samples becomes ceil(num_samples / (W H)) samples per pixel.  Subpaths
    are capped at 16 vertices each (max_num_vertices = -1 included).
*/
#include <pch.h>
#include <lightmetrica/renderer.h>
#include <lightmetrica/property.h>
#include <lightmetrica/random.h>
#include "lmgpu_scene_export.h"

LM_NAMESPACE_BEGIN

class Renderer_BDPT_CUDA final : public Renderer
{
public:

    LM_IMPL_CLASS(Renderer_BDPT_CUDA, Renderer);

public:

    LM_IMPL_F(Initialize) = [this](const PropertyNode* prop) -> bool
    {
        numSamples_ = prop->ChildAs<long long>("num_samples", 10000000L);
        maxNumVertices_ = prop->ChildAs("max_num_vertices", -1);
        minNumVertices_ = prop->ChildAs("min_num_vertices", 0);
        // the MIS weight component, misweight::<mis> (renderer_bdpt.cpp:837)
        const auto mis = prop->ChildAs<std::string>("mis", "powerheuristics");
        if (mis == "powerheuristics") mis_ = LMGPU_MIS_POWER;
        else if (mis == "simple") mis_ = LMGPU_MIS_SIMPLE;
        else
        {
            LM_LOG_ERROR("renderer::bdpt_cuda: unknown mis '" + mis + "'");
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
        lmgpu_pt_params prm = {};
        prm.spp = (uint64_t)((numSamples_ + npix - 1) / npix);
        prm.spp = prm.spp > 0 ? prm.spp : 1;
        prm.max_num_vertices = maxNumVertices_;
        prm.min_num_vertices = minNumVertices_;
        prm.seed = initRng->NextUInt();
        std::vector<float> img((size_t)npix * 3);
        if (lmgpu_render_bdpt_mis(sc, &prm, mis_, img.data(), nullptr) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("renderer::bdpt_cuda: ") + lmgpu_last_error());
            lmgpu_scene_destroy(sc);
            return;
        }
        lmgpu_scene_destroy(sc);
        lmgpu_export::WriteFilm(a.film, img);
        a.film->Save(outputPath);
    };

private:

    long long numSamples_ = 0;
    int maxNumVertices_ = -1;
    int minNumVertices_ = 0;
    int mis_ = LMGPU_MIS_POWER;

};

LM_COMPONENT_REGISTER_IMPL(Renderer_BDPT_CUDA, "renderer::bdpt_cuda");

LM_NAMESPACE_END
