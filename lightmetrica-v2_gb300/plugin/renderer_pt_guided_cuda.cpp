/*
    renderer::pt_guided_cuda -- Lightmetrica v2 plugin that renders
    renderer::pt's image (src/liblightmetrica/renderer/renderer_pt.cpp) with
    the lmgpu guided path tracer: at diffuse vertices the direction comes from
    a one-sample MIS mixture of BSDF sampling and a learned von Mises-Fisher
    mixture (an MLP on the tensor cores, trained online on the tracer's own
    radiance samples).  Unbiased for every state of the network; no
    counterpart in the reference.

    Built inside the reference tree as a plugin (plugin/renderer_pt_guided_cuda/,
    cmake/AddPlugin.cmake:26-61) linked against liblmgpu.so; a scene file
    selects it with

        renderer:
          type: pt_guided_cuda
          params:
            num_samples: 4194304
            max_num_vertices: -1
            alpha: 0.5            # probability of BSDF sampling
            learning_rate: 0.001
            throughput_roulette: 1

    Interface followed:
      Renderer::Initialize   include/lightmetrica/renderer.h:68
      Renderer::Render       include/lightmetrica/renderer.h:81
    The network's position box is the scene's bounding box (Scene3::GetBound,
    scene3.h:99).
*/
#include <pch.h>
#include <lightmetrica/renderer.h>
#include <lightmetrica/property.h>
#include <lightmetrica/random.h>
#include <lightmetrica/bound.h>
#include "lmgpu_scene_export.h"

LM_NAMESPACE_BEGIN

class Renderer_PT_Guided_CUDA final : public Renderer
{
public:

    LM_IMPL_CLASS(Renderer_PT_Guided_CUDA, Renderer);

public:

    LM_IMPL_F(Initialize) = [this](const PropertyNode* prop) -> bool
    {
        numSamples_ = prop->ChildAs<long long>("num_samples", 10000000L);
        maxNumVertices_ = prop->ChildAs("max_num_vertices", -1);
        minNumVertices_ = prop->ChildAs("min_num_vertices", 0);
        alpha_ = prop->ChildAs<Float>("alpha", 0.5_f);
        learningRate_ = prop->ChildAs<Float>("learning_rate", 0.001_f);
        // an int flag: PropertyNode::As has no bool form (property.h:151-156)
        throughputRoulette_ = prop->ChildAs<int>("throughput_roulette", 1) != 0;
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
        const Bound bound = scene->GetBound();
        const float box[6] = { (float)bound.min.x, (float)bound.min.y, (float)bound.min.z,
                               (float)bound.max.x, (float)bound.max.y, (float)bound.max.z };
        lmgpu_guide* guide = nullptr;
        if (lmgpu_guide_create(box, prm.seed, &guide) != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("renderer::pt_guided_cuda: ") + lmgpu_last_error());
            lmgpu_scene_destroy(sc);
            return;
        }
        lmgpu_guiding_params gp;
        gp.alpha = (float)alpha_;
        gp.learning_rate = (float)learningRate_;
        gp.train = 1;
        gp.batch = 1u << 18;
        gp.max_steps_per_pass = 4;
        gp.rr_mode = throughputRoulette_ ? 1u : 0u;
        std::vector<float> img((size_t)npix * 3);
        const int rc = lmgpu_render_pt_guided(sc, guide, &prm, &gp, img.data(), nullptr, nullptr);
        lmgpu_guide_destroy(guide);
        lmgpu_scene_destroy(sc);
        if (rc != LMGPU_OK)
        {
            LM_LOG_ERROR(std::string("renderer::pt_guided_cuda: ") + lmgpu_last_error());
            return;
        }
        lmgpu_export::WriteFilm(a.film, img);
        a.film->Save(outputPath);
    };

private:

    long long numSamples_ = 0;
    int maxNumVertices_ = -1;
    int minNumVertices_ = 0;
    Float alpha_ = 0.5_f;
    Float learningRate_ = 0.001_f;
    bool throughputRoulette_ = true;

};

LM_COMPONENT_REGISTER_IMPL(Renderer_PT_Guided_CUDA, "renderer::pt_guided_cuda");

LM_NAMESPACE_END
