/*
    renderer::ltdirect_cuda -- Lightmetrica v2 plugin that renders
    renderer::ltdirect's estimator (src/liblightmetrica/renderer/
    renderer_ltdirect.cpp: light paths connected to the sensor at every
    vertex with weight 1) with the lmgpu wavefront light tracer on the GPU.
    Scenes with light::env are rejected (area lights start the paths).

    Built inside the reference tree as a plugin (plugin/renderer_ltdirect_cuda/,
    cmake/AddPlugin.cmake:26-61) linked against liblmgpu.so; a scene file
    selects it with

        renderer:
          type: ltdirect_cuda
          params:
            num_samples: 4194304
            max_num_vertices: 9

    Interface followed:
      Renderer::Initialize   include/lightmetrica/renderer.h:68 (the same
                             parameters as renderer::ltdirect,
                             renderer_ltdirect.cpp:63-68,
                             and the scheduler's num_samples, scheduler.cpp:56)
      Renderer::Render       include/lightmetrica/renderer.h:81 (writes the
                             sensor's film and saves it, renderer_ltdirect.cpp:266-271)
    num_samples light paths are rounded up to a multiple of W H.  The seed of
    the GPU's counter-based random numbers is drawn from initRng.
*/
#include <pch.h>
#include <lightmetrica/renderer.h>
#include <lightmetrica/property.h>
#include <lightmetrica/random.h>
#include "lmgpu_scene_export.h"

LM_NAMESPACE_BEGIN

class Renderer_LTDirect_CUDA final : public Renderer
{
public:

    LM_IMPL_CLASS(Renderer_LTDirect_CUDA, Renderer);

public:

    LM_IMPL_F(Initialize) = [this](const PropertyNode* prop) -> bool
    {
        numSamples_ = prop->ChildAs<long long>("num_samples", 10000000L);
        maxNumVertices_ = prop->ChildAs("max_num_vertices", -1);
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
        prm.seed = initRng->NextUInt();
        std::vector<float> img((size_t)npix * 3);
        if (lmgpu_render_ltdirect(sc, &prm, img.data(), nullptr) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("renderer::ltdirect_cuda: ") + lmgpu_last_error());
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

};

LM_COMPONENT_REGISTER_IMPL(Renderer_LTDirect_CUDA, "renderer::ltdirect_cuda");

LM_NAMESPACE_END
