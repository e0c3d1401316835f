// ref_harness.cpp -- drives the reference's own RayMarcher (Oracle A).
//
// TEST INFRASTRUCTURE ONLY.  Linked with the reference translation units
// src/app/AdvancedRenderer/RayMarcher.cpp, src/app/Kernel.cpp,
// src/app/ThreadPool.cpp and src/app/Dataset.cpp, compiled unmodified from the
// reference tree against the stand-in headers in oracle/shim.  The result is
// oracle/_ref/libfmref.so, which the tests load with ctypes to pin the CPU
// restatement (fm_oracle.cpp) and to write golden vectors.
//
// The march is driven the way AdvancedRenderer::Render does it
// (AdvancedRenderer.cpp:257-275): Prepare -> Start, then wait until the pool
// reports done and join the workers with Exit() (ThreadPool.cpp:33-36 reports
// done while a worker may still be writing its last pixel; Exit waits for it).
// Pixel W*H-1 is never marched by the reference (ThreadPool.cpp:50); the
// output buffers are zeroed first so that pixel reads as a miss.
//
// The reference's vendored Partio (vendor/partio/src, compiled unmodified
// against the system zlib) is linked in, so the Dataset constructor reads
// particle files as the application does; ref_bgeo_* below pin the library's
// own BGEO reader against it.

#include <engine/hzpch.h>

#include "app/AdvancedRenderer/RayMarcher.h"
#include "app/Dataset.h"

#include <engine/renderer/Renderer.h>

#include <chrono>
#include <cstring>

FmShimVulkan Vulkan;
int fm_shim_box_mode = 0;

float RandomFloat(float min, float max) { return min + (max - min) * 0.5f; }

CameraController3D::CameraController3D(Camera3D& camera) : Camera(camera) {}


namespace
{
glm::mat4 MatFrom(const float* m)
{
    glm::mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) r[c][k] = m[c * 4 + k];
    return r;
}
}  // namespace

extern "C" {

// Build the reference Frame (search, AABB, density grid) for the particles.
// Writes the sorted particle order (xyz, stride 3) when sorted_out is given
// and the grid origin/dims when grid_out (min[3], cellwidth, dims[3] as float).
// Then marches the whole W x H image with the reference's isotropic marcher
// (aniso == 0) or its anisotropic marcher (RayMarcher.cpp:346-423) with the
// extended radius radius_mult * radius and the k_n / k_r / k_s / N_eps clamp.
// box_mode: 0 = every skip flag true (skip off), 1 = own-cell counts.
// Returns the wall time of Prepare -> Start -> Exit in seconds, or < 0 on error.
double ref_march_any(const float* xyz, int64_t n, float radius, const float* inv_proj_view, const float* cam_pos,
                     int32_t width, int32_t height, const float* depth_in, int32_t max_steps, float step_size,
                     float iso, int32_t box_mode, float* out_pos, float* out_nrm, float* sorted_out, float* grid_out,
                     double* build_seconds, int32_t aniso, float radius_mult, float k_n, float k_r, float k_s,
                     int32_t n_eps)
{
    if (n <= 0 || width <= 0 || height <= 0) return -1.0;
    fm_shim_box_mode = box_mode;
    Vulkan.SwapchainExtent.width = uint32_t(width);
    Vulkan.SwapchainExtent.height = uint32_t(height);

    auto t0 = std::chrono::steady_clock::now();
    Dataset* ds = new Dataset();
    ds->ParticleRadius = radius;
    ds->ParticleRadiusExt = radius_mult * radius;  // Dataset.cpp:175
    ds->ParticleRadiusInv = 1.0f / radius;
    ds->ParticleRadiusExtInv = 1.0f / ds->ParticleRadiusExt;
    ds->m_IsotropicKernel = CubicSplineKernel(radius);
    ds->m_AnisotropicKernel = AnisotropicKernel(radius);
    std::vector<Particle> particles(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) particles[i] = Particle(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    ds->Frames.reserve(1);
    ds->Frames.emplace_back(ds, particles, ds->ParticleRadius, ds->ParticleRadiusExt);
    ds->MaxParticles = size_t(n);
    ds->Loaded = true;
    auto t1 = std::chrono::steady_clock::now();
    if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();

    Frame& fr = ds->Frames[0];
    if (sorted_out)
        for (int64_t i = 0; i < n; ++i)
        {
            sorted_out[3 * i] = fr.m_Particles[i].x;
            sorted_out[3 * i + 1] = fr.m_Particles[i].y;
            sorted_out[3 * i + 2] = fr.m_Particles[i].z;
        }
    if (grid_out)
    {
        grid_out[0] = fr.m_Min.x; grid_out[1] = fr.m_Min.y; grid_out[2] = fr.m_Min.z;
        grid_out[3] = fr.m_DensityGrid.m_CellWidth;
        grid_out[4] = float(fr.m_DensityGrid.m_Width);
        grid_out[5] = float(fr.m_DensityGrid.m_Height);
        grid_out[6] = float(fr.m_DensityGrid.m_Depth);
    }

    Camera3D cam;
    cam.InvProjectionView = MatFrom(inv_proj_view);
    CameraController3D ctl(cam);
    ctl.Position = glm::vec3(cam_pos[0], cam_pos[1], cam_pos[2]);

    VisualizationSettings s{};
    s.Frame = 0;
    s.MaxSteps = max_steps;
    s.StepSize = step_size;
    s.IsoDensity = iso;
    s.EnableAnisotropy = aniso != 0;
    s.k_n = k_n; s.k_r = k_r; s.k_s = k_s; s.N_eps = n_eps;

    const size_t npx = size_t(width) * size_t(height);
    std::vector<glm::vec4> pos(npx, glm::vec4(0)), nrm(npx, glm::vec4(0));
    std::vector<float> depth(depth_in, depth_in + npx);

    auto t2 = std::chrono::steady_clock::now();
    RayMarcher* rm = new RayMarcher();
    rm->Prepare(s, ctl, ds, pos.data(), nrm.data(), depth.data());
    rm->Start();
    while (!rm->IsDone()) std::this_thread::sleep_for(std::chrono::microseconds(200));
    auto t3 = std::chrono::steady_clock::now();
    // The reference's pool can deadlock in Exit() when the work is short: a worker
    // released from the start barrier late reads m_Exit only after Exit() set it
    // and returns without arriving at the barrier Exit() waits on
    // (ThreadPool.cpp:17-18,43-46).  Giving every worker time to pass that check
    // before Exit() avoids it; the wall time is taken before the pause.
    std::this_thread::sleep_for(std::chrono::milliseconds(50));
    rm->Exit();

    std::memcpy(out_pos, pos.data(), npx * sizeof(glm::vec4));
    std::memcpy(out_nrm, nrm.data(), npx * sizeof(glm::vec4));
    delete rm;
    delete ds;
    return std::chrono::duration<double>(t3 - t2).count();
}

double ref_march(const float* xyz, int64_t n, float radius, const float* inv_proj_view, const float* cam_pos,
                 int32_t width, int32_t height, const float* depth_in, int32_t max_steps, float step_size,
                 float iso, int32_t box_mode, float* out_pos, float* out_nrm, float* sorted_out, float* grid_out,
                 double* build_seconds)
{
    return ref_march_any(xyz, n, radius, inv_proj_view, cam_pos, width, height, depth_in, max_steps, step_size, iso,
                         box_mode, out_pos, out_nrm, sorted_out, grid_out, build_seconds, 0, 2.0f, 0.5f, 2.0f,
                         2000.0f, 1);
}

// The reference kernel values (Kernel.cpp:16-52) for known-answer tests.
float ref_W(float h, float rx, float ry, float rz)
{
    CubicSplineKernel k(h);
    return k.W(glm::vec3(rx, ry, rz));
}

void ref_gradW(float h, float rx, float ry, float rz, float* out3)
{
    CubicSplineKernel k(h);
    glm::vec3 g = k.gradW(glm::vec3(rx, ry, rz));
    out3[0] = g.x; out3[1] = g.y; out3[2] = g.z;
}

// Frame::QueryDensityGrid (Dataset.cpp:26-47) on a built frame: linear cell
// index of each query point (-1 when outside the grid).
int ref_query_cells(const float* xyz, int64_t n, float radius, const float* queries, int64_t nq, int64_t* out)
{
    fm_shim_box_mode = 0;
    Dataset* ds = new Dataset();
    ds->ParticleRadius = radius;
    ds->ParticleRadiusExt = 2.0f * radius;
    ds->ParticleRadiusInv = 1.0f / radius;
    ds->ParticleRadiusExtInv = 1.0f / ds->ParticleRadiusExt;
    ds->m_IsotropicKernel = CubicSplineKernel(radius);
    ds->m_AnisotropicKernel = AnisotropicKernel(radius);
    std::vector<Particle> particles(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) particles[i] = Particle(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    ds->Frames.reserve(1);
    ds->Frames.emplace_back(ds, particles, ds->ParticleRadius, ds->ParticleRadiusExt);
    Frame& fr = ds->Frames[0];
    for (int64_t i = 0; i < nq; ++i)
    {
        OctreeNode* node = fr.QueryDensityGrid(glm::vec3(queries[3 * i], queries[3 * i + 1], queries[3 * i + 2]));
        out[i] = node ? int64_t(node - fr.m_DensityGrid.m_Nodes.data()) : -1;
    }
    delete ds;
    return 0;
}

// ---- particle files --------------------------------------------------------

// Partio::read + the copy of Dataset::ReadFile (Dataset.cpp:292-306): the
// "position" of every particle, in file order.  Returns the particle count
// (positions written up to cap), -1 when Partio returns no file.
int64_t ref_bgeo_positions(const char* path, float* xyz, int64_t cap)
{
    Partio::ParticlesDataMutable* file = Partio::read(path, false);
    if (!file) return -1;
    Partio::ParticleAttribute attr;
    file->attributeInfo("position", attr);
    const int64_t n = file->numParticles();
    for (int64_t i = 0; i < n && i < cap; ++i)
    {
        const float* p = file->data<float>(attr, int(i));
        xyz[3 * i] = p[0];
        xyz[3 * i + 1] = p[1];
        xyz[3 * i + 2] = p[2];
    }
    file->release();
    return n;
}

// Partio's writer: n positions as a BGEO file (gzip-compressed when
// compressed != 0, Partio::write's forceCompressed).  0 on success.
int ref_bgeo_write(const char* path, const float* xyz, int64_t n, int32_t compressed)
{
    Partio::ParticlesDataMutable* p = Partio::create();
    Partio::ParticleAttribute attr = p->addAttribute("position", Partio::VECTOR, 3);
    p->addParticles(int(n));
    for (int64_t i = 0; i < n; ++i)
    {
        float* d = p->dataWrite<float>(attr, int(i));
        d[0] = xyz[3 * i];
        d[1] = xyz[3 * i + 1];
        d[2] = xyz[3 * i + 2];
    }
    Partio::write(path, *p, compressed != 0, false);
    p->release();
    return 0;
}

// The reference's Dataset constructor over prefix + i + suffix (count < 0: no
// limit), radius multiplier 2.  Returns the frame count (-1 when !Loaded);
// counts[i] = particles of frame i (up to max_frames), *max_particles =
// Dataset::MaxParticles, and xyz (cap floats) the frames' particles one after
// another in the order the Frame keeps them (the search's spatial order).
int32_t ref_dataset_load(const char* prefix, const char* suffix, int32_t count, float radius, int64_t* counts,
                         int32_t max_frames, int64_t* max_particles, float* xyz, int64_t cap)
{
    Dataset ds(prefix, suffix, radius, 2.0f, count);
    if (!ds.Loaded) return -1;
    int64_t at = 0;
    for (size_t f = 0; f < ds.Frames.size(); ++f)
    {
        const auto& ps = ds.Frames[f].m_Particles;
        if (int32_t(f) < max_frames) counts[f] = int64_t(ps.size());
        for (const auto& q : ps)
        {
            if (at + 3 > cap) break;
            xyz[at++] = q.x;
            xyz[at++] = q.y;
            xyz[at++] = q.z;
        }
    }
    *max_particles = int64_t(ds.MaxParticles);
    return int32_t(ds.Frames.size());
}

}  // extern "C"
