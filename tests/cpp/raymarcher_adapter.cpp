// Drives fluidmarch::RayMarcher (include/fluidmarch.hpp) the way the
// reference's AdvancedRenderer drives its CPU RayMarcher: Prepare, Start,
// poll IsDone, Exit.  Input and output are raw binary files written and read
// by tests/test_gpu_cpp_adapter.py.
//   argv[1] input:  int32 n, W, H, max_steps; float radius, step, iso;
//                   float camera[16+16+16+3]; float xyz[3n]; float depth[W*H]
//   argv[2] output: float positions[4*W*H], normals[4*W*H]
#include <cstdio>
#include <cstring>
#include <vector>

#include "fluidmarch.hpp"

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int hdr[4];
    float par[3];
    fm_camera cam{};
    if (std::fread(hdr, 4, 4, f) != 4 || std::fread(par, 4, 3, f) != 3) return 4;
    if (std::fread(cam.view, 4, 16, f) != 16 || std::fread(cam.proj, 4, 16, f) != 16 ||
        std::fread(cam.inv_proj_view, 4, 16, f) != 16 || std::fread(cam.position, 4, 3, f) != 3)
        return 4;
    const int n = hdr[0];
    cam.width = hdr[1];
    cam.height = hdr[2];
    const size_t npx = (size_t)cam.width * cam.height;
    std::vector<float> xyz(3 * (size_t)n), depth(npx), pos(4 * npx, 0.0f), nrm(4 * npx, 0.0f);
    if (std::fread(xyz.data(), 4, xyz.size(), f) != xyz.size() || std::fread(depth.data(), 4, npx, f) != npx) return 4;
    std::fclose(f);
    try {
        fluidmarch::RayMarcher marcher(0);
        fluidmarch::Frame frame(marcher.context(), xyz.data(), (size_t)n, par[0]);
        fluidmarch::VisualizationSettings s;
        s.EnableAnisotropy = false;  // the isotropic march, compared with the oracle's
        s.MaxSteps = hdr[3];
        s.StepSize = par[1];
        s.IsoDensity = par[2];
        s.SkipMode = FM_SKIP_OFF;
        marcher.Prepare(s, cam, frame, pos.data(), nrm.data(), depth.data());
        marcher.Start();
        while (!marcher.IsDone()) {
        }
        marcher.Exit();
    } catch (const fluidmarch::Error& e) {
        std::fprintf(stderr, "fluidmarch error %d: %s\n", e.code, e.what());
        return 5;
    }
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 6;
    std::fwrite(pos.data(), 4, pos.size(), o);
    std::fwrite(nrm.data(), 4, nrm.size(), o);
    std::fclose(o);
    return 0;
}
