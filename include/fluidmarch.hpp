// fluidmarch.hpp -- C++ host interface of the GB300 marcher, shaped like the
// reference's CPU classes so that the renderer's call sites stay as they are:
//
//   class RayMarcher   src/app/AdvancedRenderer/RayMarcher.h:28-77
//     RayMarcher()     RayMarcher.cpp:66-69   -> fm_create
//     Prepare(...)     RayMarcher.cpp:76-100  -> stores the arguments
//     Start()          RayMarcher.cpp:102-112 -> fm_march (returns when the outputs are written)
//     IsDone()         RayMarcher.h:44        -> true once Start() returned (no race on the last pixel)
//     Exit()           RayMarcher.cpp:71-74   -> fm_sync
//   struct VisualizationSettings  RayMarcher.h:12-26
//   class Frame        src/app/Dataset.h:37-65 -> fm_scene_create / fm_scene_destroy
//
// Header only, on top of the C ABI in fluidmarch.h (no CUDA headers needed).
// Errors throw fluidmarch::Error with the library's message.
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>

#include "fluidmarch.h"

namespace fluidmarch {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(fm_ctx* ctx, int rc, const char* what) {
    if (rc != FM_OK) throw Error(rc, std::string(what) + ": " + fm_last_error(ctx));
}

// The reference's settings (RayMarcher.h:12-26), plus bisection, skip mode and
// the Dataset's extended-radius multiplier (Dataset.cpp:175).
struct VisualizationSettings {
    int Frame = 0;
    int MaxSteps = 128;
    float StepSize = 0.009f;
    float IsoDensity = 1.0f;
    bool EnableAnisotropy = false;  // RayMarcher::PerPixel_Anisotropic (RayMarcher.cpp:346-423)
    float k_n = 0.5f, k_r = 2.0f, k_s = 2000.0f;
    int N_eps = 1;
    float ParticleRadiusMultiplier = 2.0f;
    int BisectIters = 0;               // 0: the reference's first-sample hit
    int SkipMode = FM_SKIP_REFERENCE;  // the reference's empty-space skip
};

// Particles of one frame and their uniform grid (Frame::Frame, Dataset.cpp:9-24).
class Frame {
public:
    Frame(fm_ctx* ctx, const float* xyz, std::size_t n, float particle_radius, unsigned stride = 3)
        : ctx_(ctx), radius_(particle_radius) {
        check(ctx_, fm_scene_create(ctx_, xyz, n, stride, particle_radius, FM_MEM_HOST, &scene_), "fm_scene_create");
    }
    ~Frame() { fm_scene_destroy(scene_); }
    Frame(const Frame&) = delete;
    Frame& operator=(const Frame&) = delete;
    fm_scene* handle() const { return scene_; }
    float ParticleRadius() const { return radius_; }

private:
    fm_ctx* ctx_;
    fm_scene* scene_ = nullptr;
    float radius_;
};

class RayMarcher {
public:
    explicit RayMarcher(int device = 0) { check(nullptr, fm_create(&ctx_, device), "fm_create"); }
    ~RayMarcher() { fm_destroy(ctx_); }
    RayMarcher(const RayMarcher&) = delete;
    RayMarcher& operator=(const RayMarcher&) = delete;

    fm_ctx* context() const { return ctx_; }

    // positions / normals: W*H vec4 (float[4]) outputs; depth: the W*H ray-start
    // (splat) depth buffer the reference consumes, 1.0 = no particle.
    void Prepare(const VisualizationSettings& settings, const fm_camera& camera, Frame& frame, float* positions,
                 float* normals, float* depth) {
        settings_ = settings;
        camera_ = camera;
        frame_ = &frame;
        out_ = fm_frame_out{};
        out_.position = positions;
        out_.normal = normals;
        out_.start_depth = depth;
        done_ = false;
    }

    void Start() {
        if (!frame_) throw Error(FM_ERR_INVALID, "Prepare() first");
        fm_march_params p{};
        p.iso_density = settings_.IsoDensity;
        p.step_size = settings_.StepSize;
        p.max_steps = settings_.MaxSteps;
        p.bisect_iters = settings_.BisectIters;
        p.skip_mode = settings_.SkipMode;
        p.flags = FM_MARCH_EXTERNAL_DEPTH;
        if (settings_.EnableAnisotropy) {
            fm_aniso_params a{settings_.ParticleRadiusMultiplier, settings_.k_n, settings_.k_r, settings_.k_s,
                              settings_.N_eps, 0};
            check(ctx_, fm_set_anisotropy(ctx_, &a), "fm_set_anisotropy");
            p.flags |= FM_MARCH_ANISOTROPIC;
            if (p.skip_mode == FM_SKIP_EXACT) p.skip_mode = FM_SKIP_REFERENCE;  // the reference always skips here
        }
        check(ctx_, fm_march(ctx_, frame_->handle(), &camera_, &p, &out_, FM_MEM_HOST, nullptr), "fm_march");
        done_ = true;
    }

    bool IsDone() const { return done_; }

    void Exit() { check(ctx_, fm_sync(ctx_, -1), "fm_sync"); }

private:
    fm_ctx* ctx_ = nullptr;
    VisualizationSettings settings_{};
    fm_camera camera_{};
    Frame* frame_ = nullptr;
    fm_frame_out out_{};
    bool done_ = false;
};

}  // namespace fluidmarch
