// C++ drop-in for the reference's Renderer and SceneDesc (include/renderer.h:
// 19-206 and include/scene_desc.h:9-42 of markcmagro/optix_pt), implemented
// over the C ABI in optpt.h. Method names, call order and per-frame flow are
// the reference's: construct from a SceneDesc, run the init sequence, then per
// frame updateLaunchParams() + launch() + getFrameBuffer(). OptiX set-up
// steps that have no counterpart are kept as no-ops so an existing init
// sequence compiles and runs unchanged. Errors throw std::runtime_error, as
// the reference's CUDA()/OPTIX() macros do in debug builds
// (include/cuda_helpers.h:8-38).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include "../optpt.h"

namespace optix_pt {

inline void check(int rc, const char *what)
{
    if (rc != OPTPT_OK)
        throw std::runtime_error(std::string(what) + ": " + optpt_last_error());
}

// Camera (include/camera.h:5-27): eye/target/up and vertical field of view;
// U, V, W are derived by the renderer (src/camera.cpp:19-40).
struct Camera {
    float eye[3] = {0.0f, 0.0f, 3.0f};
    float target[3] = {0.0f, 0.0f, 0.0f};
    float upHint[3] = {0.0f, 1.0f, 0.0f};
    float vertFovDeg = 40.0f;
};

// SceneDesc (src/scene_desc.cpp:35-116): resolves a scene-selection list and
// parses the selected scene file. The reference throws int -1 on an
// unreadable file; this throws std::runtime_error.
class SceneDesc {
  public:
    optpt_scene scene{};
    int resX = 0, resY = 0;

    explicit SceneDesc(const char *sceneListFile)
    {
        check(optpt_scene_from_config(sceneListFile, &scene), "SceneDesc");
        resX = (int)scene.resX;
        resY = (int)scene.resY;
    }
    static SceneDesc procedural(const char *name, uint32_t seed = 1) { return SceneDesc(name, seed); }
    SceneDesc(const SceneDesc &) = delete;
    SceneDesc &operator=(const SceneDesc &) = delete;
    SceneDesc(SceneDesc &&o) noexcept : scene(o.scene), resX(o.resX), resY(o.resY) { o.scene = optpt_scene{}; }
    ~SceneDesc() { optpt_scene_release(&scene); }
    bool parse() { return true; }  // parsing happens in the constructor

  private:
    SceneDesc(const char *name, uint32_t seed)
    {
        check(optpt_scene_procedural(name, seed, &scene), "SceneDesc");
        resX = (int)scene.resX;
        resY = (int)scene.resY;
    }
};

class Renderer {
    optpt_renderer *h_ = nullptr;
    SceneDesc &sceneDesc_;

  public:
    Camera cam;

    explicit Renderer(SceneDesc &sceneDesc, const optpt_options *options = nullptr) : sceneDesc_(sceneDesc)
    {
        check(optpt_create(&sceneDesc.scene, options, &h_), "Renderer");
        for (int k = 0; k < 3; ++k) {
            cam.eye[k] = sceneDesc.scene.camEye[k];
            cam.target[k] = sceneDesc.scene.camTarget[k];
            cam.upHint[k] = sceneDesc.scene.camUp[k];
        }
        if (sceneDesc.scene.camFovYDeg > 0.0f)
            cam.vertFovDeg = sceneDesc.scene.camFovYDeg;
    }
    Renderer(const Renderer &) = delete;
    Renderer &operator=(const Renderer &) = delete;
    ~Renderer() { optpt_destroy(h_); }

    // Init sequence (src/main_window.cpp:36-49). Scene upload and the BVH
    // build happen in the constructor; the OptiX steps have no counterpart.
    void initOptix() {}
    void createContext() {}
    void loadScene() {}
    void buildAccel(bool = true) {}
    void setupCompilationOptions() {}
    void createModules() {}
    void createProgramGroups() {}
    void createPipeline() {}
    void setupSbt() {}
    void createDenoiser() {}
    void createRandomState() {}

    void setupOutputBuffer(uint32_t width, uint32_t height)
    {
        check(optpt_setup_output_buffer(h_, width, height), "setupOutputBuffer");
    }
    void setupCamera(uint32_t, uint32_t)
    {
        check(optpt_setup_camera(h_, cam.eye, cam.target, cam.upHint, cam.vertFovDeg), "setupCamera");
    }
    void setupLaunchParams(SceneDesc &) {}

    // Per frame (src/main_window.cpp:128-130).
    void updateScene() {}
    void updateLaunchParams()
    {
        check(optpt_setup_camera(h_, cam.eye, cam.target, cam.upHint, cam.vertFovDeg), "updateLaunchParams");
    }
    void launch() { check(optpt_launch(h_), "launch"); }
    // Frame loop without a stall per frame: renders a frame and returns the
    // previous one (its download overlapped this frame's render); nullptr
    // on the first call. launchFlush() returns the last frame.
    const float *launchPipelined()
    {
        const float *f = nullptr;
        check(optpt_launch_pipelined(h_, &f), "launchPipelined");
        return f;
    }
    const float *launchFlush()
    {
        const float *f = nullptr;
        check(optpt_launch_flush(h_, &f), "launchFlush");
        return f;
    }

    void *getFrameBuffer() { return (void *)optpt_get_frame_buffer(h_); }
    uint32_t getSampleCount() { return optpt_get_sample_count(h_); }
    void resetSampleCount() { check(optpt_reset_sample_count(h_), "resetSampleCount"); }

    bool getDenoiserState() { return false; }
    void setDenoiserState(bool on)
    {
        if (on)
            throw std::runtime_error("the OptiX AI denoiser is not part of this renderer");
    }

    void setVis(int vis) { edit([&](LaunchParams &lp) { lp.vis = vis; }); }
    int getVis() { return params().vis; }
    void setToneMappingState(bool enable) { edit([&](LaunchParams &lp) { lp.toneMapping = enable; }); }
    bool getToneMappingState() { return params().toneMapping != 0; }
    void setToneMappingImpl(int impl) { edit([&](LaunchParams &lp) { lp.toneMappingImpl = impl; }); }
    int getToneMappingImpl() { return params().toneMappingImpl; }
    void setGammaCorrectionState(bool enable) { edit([&](LaunchParams &lp) { lp.gammaCorrection = enable; }); }
    int getGammaCorrectionState() { return params().gammaCorrection; }
    void setGammaCorrectionTerm(float value) { edit([&](LaunchParams &lp) { lp.gammaTerm = value; }); }
    float getGammaCorrectionTerm() { return params().gammaTerm; }

    // Beyond the reference: asynchronous multi-sample rendering on a stream.
    void render(uint32_t spp, void *stream = nullptr) { check(optpt_render(h_, spp, stream), "render"); }
    optpt_renderer *handle() { return h_; }

  private:
    LaunchParams params()
    {
        LaunchParams lp;
        check(optpt_get_launch_params(h_, &lp), "launch params");
        return lp;
    }
    template <class F> void edit(F f)
    {
        LaunchParams lp = params();
        f(lp);
        check(optpt_set_launch_params(h_, &lp), "launch params");
    }
};

}  // namespace optix_pt
