// fluidmarch.hpp -- C++ host interface of the GB300 marcher, shaped like the
// reference's CPU classes so that the renderer's call sites stay as they are:
//
//   class RayMarcher   src/app/AdvancedRenderer/RayMarcher.h:28-77
//     RayMarcher()     RayMarcher.cpp:66-69   -> fm_create
//     Prepare(...)     RayMarcher.cpp:76-100  -> stores the arguments
//     Start()          RayMarcher.cpp:102-112 -> fm_march into library-pinned blocks (asynchronous)
//     IsDone()         RayMarcher.h:44        -> fm_query; on completion the outputs are copied to the
//                                                caller's buffers (no race on the last pixel)
//     Exit()           RayMarcher.cpp:71-74   -> fm_sync
//   struct VisualizationSettings  RayMarcher.h:12-26
//   class Frame        src/app/Dataset.h:37-65 -> fm_scene_create / fm_scene_destroy
//   class Dataset      src/app/Dataset.h:67-105, Dataset.cpp:169-227 -> fm_dataset_* (every frame a
//                      scene resident on the device, as the reference keeps every Frame in memory)
//
// Header only, on top of the C ABI in fluidmarch.h (no CUDA headers needed).
// Errors throw fluidmarch::Error with the library's message.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

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
    // RayMarcher::PerPixel_Anisotropic (RayMarcher.cpp:346-423), on by default as
    // g_VisualizationSettings has it (AdvancedRenderer.cpp:23)
    bool EnableAnisotropy = true;
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
    // adopts a scene the library created (particle files)
    Frame(fm_ctx* ctx, fm_scene* scene, float particle_radius) : ctx_(ctx), scene_(scene), radius_(particle_radius) {}
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

// The reference's Dataset: the particle files pathPrefix + i + pathSuffix,
// i = 1, 2, ... until one is missing or i > count, each read into a Frame at
// construction.  As in the reference, a file that fails to load stops the
// loading and leaves Loaded false (LastError() has the message).
class Dataset {
public:
    Dataset() = default;
    Dataset(fm_ctx* ctx, const std::string& pathPrefix, const std::string& pathSuffix, float particleRadius,
            float particleRadiusMultiplier, int count = -1, int threads = 2)
        : ParticleRadius(particleRadius),
          ParticleRadiusExt(particleRadiusMultiplier * particleRadius),
          ParticleRadiusInv(1.0f / particleRadius),
          ParticleRadiusExtInv(1.0f / (particleRadiusMultiplier * particleRadius)) {
        char err[512] = {0};
        fm_dataset* ds = nullptr;
        if (fm_dataset_open(pathPrefix.c_str(), pathSuffix.c_str(), count, threads, &ds, err, sizeof err) != FM_OK) {
            error_ = err;
            return;
        }
        const int32_t n = fm_dataset_frames(ds);
        Frames.reserve((std::size_t)n);
        for (int32_t i = 0; i < n; ++i) {
            fm_scene* s = nullptr;
            if (fm_dataset_scene(ds, ctx, i, ParticleRadius, &s) != FM_OK) {
                error_ = fm_last_error(ctx);
                fm_dataset_close(ds);
                return;
            }
            fm_grid_info g{};
            fm_scene_grid(s, &g);
            MaxParticles = g.n_particles > MaxParticles ? (std::size_t)g.n_particles : MaxParticles;
            Frames.push_back(std::unique_ptr<Frame>(new Frame(ctx, s, ParticleRadius)));
        }
        fm_dataset_close(ds);
        Loaded = true;
    }

    // Dataset::makeCube (Dataset.cpp:228-262): a frame of numParticles uniform
    // in [-extent, extent]^3 plus one particle at (0, 2 extent, 0), appended to
    // Frames.  The positions come from a seeded std::mt19937_64, not from the
    // reference's RandomFloat.
    static void makeCube(fm_ctx* ctx, Dataset& r, float extent, std::size_t numParticles, float particleRadius,
                         float particleRadiusMultiplier, uint64_t seed = 0) {
        r.ParticleRadius = particleRadius;
        r.ParticleRadiusExt = particleRadiusMultiplier * particleRadius;
        r.ParticleRadiusInv = 1.0f / particleRadius;
        r.ParticleRadiusExtInv = 1.0f / r.ParticleRadiusExt;
        std::mt19937_64 rng(seed);
        std::uniform_real_distribution<float> u(-extent, extent);
        std::vector<float> xyz;
        xyz.reserve(3 * (numParticles + 1));
        for (std::size_t i = 0; i < numParticles; ++i) {
            const float x = u(rng), y = u(rng), z = u(rng);
            xyz.push_back(x);
            xyz.push_back(y);
            xyz.push_back(z);
        }
        xyz.push_back(0.0f);
        xyz.push_back(2.0f * extent);
        xyz.push_back(0.0f);
        r.Frames.push_back(std::unique_ptr<Frame>(new Frame(ctx, xyz.data(), numParticles + 1, particleRadius)));
        r.MaxParticles = r.MaxParticles > numParticles + 1 ? r.MaxParticles : numParticles + 1;
        r.Loaded = true;
    }

    const std::string& LastError() const { return error_; }

    float ParticleRadius = 0.0f;
    float ParticleRadiusExt = 0.0f;
    float ParticleRadiusInv = 0.0f;
    float ParticleRadiusExtInv = 0.0f;
    std::vector<std::unique_ptr<Frame>> Frames;
    std::size_t MaxParticles = 0;
    bool Loaded = false;

private:
    std::string error_;
};

class RayMarcher {
public:
    explicit RayMarcher(int device = 0) { check(nullptr, fm_create(&ctx_, device), "fm_create"); }
    ~RayMarcher() {
        if (started_) fm_sync(ctx_, -1);
        release();
        fm_destroy(ctx_);
    }
    RayMarcher(const RayMarcher&) = delete;
    RayMarcher& operator=(const RayMarcher&) = delete;

    fm_ctx* context() const { return ctx_; }

    // positions / normals: W*H vec4 (float[4]) outputs; depth: the W*H ray-start
    // (splat) depth buffer the reference consumes, 1.0 = no particle.
    void Prepare(const VisualizationSettings& settings, const fm_camera& camera, Frame& frame, float* positions,
                 float* normals, float* depth) {
        if (started_) Exit();
        settings_ = settings;
        camera_ = camera;
        frame_ = &frame;
        positions_ = positions;
        normals_ = normals;
        depth_ = depth;
        done_ = false;
    }

    // Asynchronous, like the reference's thread pool: the march runs into
    // pinned blocks of the library (written by the kernels directly) and
    // returns at once; IsDone() polls the context's stream.
    void Start() {
        if (!frame_) throw Error(FM_ERR_INVALID, "Prepare() first");
        if (started_) Exit();
        const std::size_t npx = (std::size_t)camera_.width * (std::size_t)camera_.height;
        reserve(npx);
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
        }
        std::memcpy(pin_depth_, depth_, npx * sizeof(float));
        fm_frame_out out{};
        out.position = positions_ ? pin_pos_ : nullptr;
        out.normal = normals_ ? pin_nrm_ : nullptr;
        out.start_depth = pin_depth_;
        check(ctx_, fm_march(ctx_, frame_->handle(), &camera_, &p, &out, FM_MEM_HOST, nullptr), "fm_march");
        started_ = true;
        done_ = false;
    }

    // True once every pixel is written (the reference's IsDone could report done
    // while a worker still wrote its last pixel; this one cannot).
    bool IsDone() {
        if (!started_) return done_;
        const int q = fm_query(ctx_);
        if (q < 0) throw Error(-q, std::string("fm_query: ") + fm_last_error(ctx_));
        if (q == 0) return false;
        finish();
        return true;
    }

    // Waits for the march and delivers its outputs (RayMarcher::Exit joins the workers).
    void Exit() {
        if (started_) finish();
        check(ctx_, fm_sync(ctx_, -1), "fm_sync");
    }

private:
    void finish() {
        check(ctx_, fm_sync(ctx_, -1), "fm_sync");  // also reports kernel status
        const std::size_t npx = (std::size_t)camera_.width * (std::size_t)camera_.height;
        if (positions_) std::memcpy(positions_, pin_pos_, npx * 16);
        if (normals_) std::memcpy(normals_, pin_nrm_, npx * 16);
        started_ = false;
        done_ = true;
    }
    void reserve(std::size_t npx) {
        if (npx <= cap_) return;
        release();
        void* p = nullptr;
        check(ctx_, fm_host_alloc(ctx_, npx * 16, &p), "fm_host_alloc");
        pin_pos_ = (float*)p;
        check(ctx_, fm_host_alloc(ctx_, npx * 16, &p), "fm_host_alloc");
        pin_nrm_ = (float*)p;
        check(ctx_, fm_host_alloc(ctx_, npx * 4, &p), "fm_host_alloc");
        pin_depth_ = (float*)p;
        cap_ = npx;
    }
    void release() {
        fm_host_free(ctx_, pin_pos_);
        fm_host_free(ctx_, pin_nrm_);
        fm_host_free(ctx_, pin_depth_);
        pin_pos_ = pin_nrm_ = pin_depth_ = nullptr;
        cap_ = 0;
    }

    fm_ctx* ctx_ = nullptr;
    VisualizationSettings settings_{};
    fm_camera camera_{};
    Frame* frame_ = nullptr;
    float *positions_ = nullptr, *normals_ = nullptr, *depth_ = nullptr;
    float *pin_pos_ = nullptr, *pin_nrm_ = nullptr, *pin_depth_ = nullptr;
    std::size_t cap_ = 0;
    bool started_ = false, done_ = false;
};

}  // namespace fluidmarch
