// fm_oracle.cpp -- CPU restatement of the reference's isotropic SPH ray march.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the CUDA
// path in bachelor-thesis_gb300/csrc.  Only the tests, the smoke check and the
// CPU-baseline leg of bench.py load it; the product library never links it.
//
// What it restates (file:line in Fruup/bachelor-thesis):
//   * grid origin / dims / cell index ..... src/app/Dataset.cpp:78-104 (ComputeAABB,
//                                           BuildDensityGrid) and :26-47 (QueryDensityGrid)
//   * cubic spline W, gradW ............... src/app/Kernel.cpp:9-52
//   * ray setup, march loop, hit test ...... src/app/AdvancedRenderer/RayMarcher.cpp:256-344
//   * empty-space skip (reference flags) ... RayMarcher.cpp:281-306, intersectAABB :51-62,
//                                           flags Dataset.cpp:137-164
//   * splat depth .......................... AdvancedRenderer.cpp:447-485,
//                                           assets/shaders/advanced/depth.vert:20-28, depth.frag:19-34
//   * shading .............................. assets/shaders/advanced/composition.frag:37-46,59-66,79-122
// Additions that the reference does not have (and that the CUDA path shares):
//   * bisection between the last outside and first inside sample,
//   * the normal taken at the refined hit point,
//   * hit distance output, r == 0 guard in gradW (the reference would return NaN).
//
// Arithmetic: every FP32 operation is written out in the order glm 0.9.9 uses
// (dot = (x*x + y*y) + z*z, normalize = v * (1/sqrt(dot)), mat4*vec4 =
// (m0*v0 + m1*v1) + (m2*v2 + m3*v3)).  Build with -ffp-contract=off so that no
// multiply-add is fused; then the FP32 march is bit-identical to the reference
// translation units compiled the same way, given the same neighbour order.
//
// Neighbour order (canonical order): the 27 cells around the sample's cell in
// increasing linear cell index (z outer, y, x inner); inside a cell by 2x2x2
// sub-cell (sx + 2 sy + 4 sz), inside a sub-cell by increasing input index
// (a stable counting sort).  Particles are stored in that order, so the
// canonical order is the increasing sorted index.
//
// The FP64 twin runs the same march in double precision from the same inputs
// (it keeps the FP32 cell table) and is the "FP64 re-evaluation" the parity
// tests state errors against.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {

struct OrcCamera {
    float view[16];           // glm column-major: m[col*4 + row]
    float proj[16];
    float inv_proj_view[16];
    float position[3];
    int32_t width;
    int32_t height;
};

struct OrcGrid {
    float min[3];     // AABB min - support radius  (Frame::m_Min)
    float max[3];     // AABB max + support radius  (Frame::m_Max)
    float cell;       // cell width = support radius
    float inv;        // 1.0f / cell
    int32_t dims[3];  // ceil((max - min) / cell)
    int32_t pad;
};

struct OrcParams {
    float iso;            // VisualizationSettings::IsoDensity
    float step;           // VisualizationSettings::StepSize
    int32_t max_steps;    // VisualizationSettings::MaxSteps
    int32_t bisect_iters; // 0 = reference behaviour (first sample with rho >= iso)
    int32_t skip_mode;    // 0 off, 1 exact density-bound skip (same result as off), 2 reference flags
    int32_t flags;        // unused by the oracle
};

}  // extern "C"

namespace {

template <typename T> struct V3 { T x, y, z; };

template <typename T> inline V3<T> add(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> inline V3<T> sub(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> inline V3<T> mul(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T> inline V3<T> mul(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T> inline V3<T> divs(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
// glm compute_dot<vec3>: tmp = a*b; return tmp.x + tmp.y + tmp.z
template <typename T> inline T dot(V3<T> a, V3<T> b) {
    T tx = a.x * b.x, ty = a.y * b.y, tz = a.z * b.z;
    return (tx + ty) + tz;
}
// glm normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
template <typename T> inline V3<T> normalize(V3<T> v) {
    T inv = T(1) / std::sqrt(dot(v, v));
    return mul(v, inv);
}

// glm mat4 * vec4 (column-major m[col*4+row]):
// ((m[0]*v0 + m[1]*v1) + (m[2]*v2 + m[3]*v3))
template <typename T> inline void mat4_mul(const float* mf, const T v[4], T out[4]) {
    for (int r = 0; r < 4; ++r) {
        T m0 = T(mf[0 * 4 + r]), m1 = T(mf[1 * 4 + r]), m2 = T(mf[2 * 4 + r]), m3 = T(mf[3 * 4 + r]);
        T mul0 = m0 * v[0], mul1 = m1 * v[1];
        T add0 = mul0 + mul1;
        T mul2 = m2 * v[2], mul3 = m3 * v[3];
        T add1 = mul2 + mul3;
        out[r] = add0 + add1;
    }
}

// ---------------------------------------------------------------------------
// Cubic spline kernel, src/app/Kernel.cpp:9-52.  h is the SUPPORT radius.
template <typename T> struct Cubic {
    T h, h2, hinv, sig;
    explicit Cubic(float hf) {
        h = T(hf);
        h2 = h * h;
        hinv = T(1) / h;
        // sig_d = 8 / (pi * h * h * h), evaluated left to right
        const T pi = std::is_same<T, float>::value ? T(3.14159265358979323846f) : T(3.14159265358979323846);
        sig = T(8) / (((pi * h) * h) * h);
    }
    // W(r) given q2 = dot(r, r) < h2
    inline T W_in(T q2) const {
        T q = std::sqrt(q2) * hinv;
        if (q >= T(0.5)) {
            T q_ = T(1) - q;
            return sig * (((T(2) * q_) * q_) * q_);
        }
        return sig * (T(6) * (((q * q) * q) - (q * q)) + T(1));
    }
    // gradW(r) given rn = dot(r, r) < h2, rn > 0
    inline V3<T> gradW_in(V3<T> r, T rn) const {
        T rl = std::sqrt(rn);
        T q = rl * hinv;
        // gradQ = normalize(r) / (r_length * h)
        V3<T> gq = divs(normalize(r), rl * h);
        if (q >= T(0.5)) {
            T q_ = T(1) - q;
            // -sig_d * gradQ * (6 q_ q_): (-sig * gradQ) * (6*q_*q_)
            T s = (T(6) * q_) * q_;
            V3<T> a = mul(-sig, gq);
            return mul(a, s);
        }
        // sig * gradQ * (6 * (3 q q - 2 q))
        T s = T(6) * (((T(3) * q) * q) - (T(2) * q));
        V3<T> a = mul(sig, gq);
        return mul(a, s);
    }
};

struct Scene {
    const float* sorted;     // xyz(w) cell-sorted, stride 4
    const uint32_t* start;   // ncells + 1
    OrcGrid g;
    float H;                 // support radius
    const uint8_t* ref_flag; // reference skip flags (mode 2) or null
};

// Sample -> cell coordinates with the FP32 formula of QueryDensityGrid.
// Returns false when the sample is so far outside the grid that its 27
// neighbourhood is empty (also for non-finite samples).
inline bool sample_cell_f32(const OrcGrid& g, float px, float py, float pz, int& cx, int& cy, int& cz) {
    float fx = std::floor((px - g.min[0]) * g.inv);
    float fy = std::floor((py - g.min[1]) * g.inv);
    float fz = std::floor((pz - g.min[2]) * g.inv);
    if (!(fx >= -2.0f && fx <= float(g.dims[0]) + 1.0f)) return false;
    if (!(fy >= -2.0f && fy <= float(g.dims[1]) + 1.0f)) return false;
    if (!(fz >= -2.0f && fz <= float(g.dims[2]) + 1.0f)) return false;
    cx = int(fx); cy = int(fy); cz = int(fz);
    return true;
}

template <typename T> inline bool sample_cell(const OrcGrid& g, V3<T> p, int& cx, int& cy, int& cz) {
    if (std::is_same<T, float>::value) return sample_cell_f32(g, float(p.x), float(p.y), float(p.z), cx, cy, cz);
    T fx = std::floor((p.x - T(g.min[0])) * (T(1) / T(g.cell)));
    T fy = std::floor((p.y - T(g.min[1])) * (T(1) / T(g.cell)));
    T fz = std::floor((p.z - T(g.min[2])) * (T(1) / T(g.cell)));
    if (!(fx >= -2 && fx <= T(g.dims[0]) + 1)) return false;
    if (!(fy >= -2 && fy <= T(g.dims[1]) + 1)) return false;
    if (!(fz >= -2 && fz <= T(g.dims[2]) + 1)) return false;
    cx = int(fx); cy = int(fy); cz = int(fz);
    return true;
}

struct EvalStats { int64_t evals = 0; int64_t candidates = 0; };

// The grid is the particles' box padded by the support radius H
// (Dataset.cpp:89-92), so farther than H beyond that box (plus a rounding
// slack of 1e-4 H + 1e-6 max|coordinate|) no particle is within H and the
// density is exactly 0.  True when p is out there on an axis the step moves
// further out on: with iso > 0 no later sample can hit.
template <typename T> inline bool leaving_zero_box(const OrcGrid& g, V3<T> p, V3<T> s) {
    float amax = 0.0f;
    for (int a = 0; a < 3; ++a) amax = std::max(amax, std::max(std::fabs(g.min[a]), std::fabs(g.max[a])));
    const float H = g.cell;
    const float slack = 1.0e-4f * H + 1.0e-6f * amax;
    const T pa[3] = {p.x, p.y, p.z}, sa[3] = {s.x, s.y, s.z};
    for (int a = 0; a < 3; ++a) {
        const float lo = g.min[a] - slack, hi = g.max[a] + slack;
        if (pa[a] > T(hi) && sa[a] >= T(0)) return true;
        if (pa[a] < T(lo) && sa[a] <= T(0)) return true;
    }
    return false;
}

// floor((p - min) * inv) leaves [-2, dims + 1] on an axis and the step moves
// further out on it (monotone FP addition): all later densities are 0.
template <typename T> inline bool outside_forever(const OrcGrid& g, V3<T> p, V3<T> s) {
    const T pa[3] = {p.x, p.y, p.z}, sa[3] = {s.x, s.y, s.z};
    for (int a = 0; a < 3; ++a) {
        T f = std::is_same<T, float>::value ? T(std::floor((float(pa[a]) - g.min[a]) * g.inv))
                                            : std::floor((pa[a] - T(g.min[a])) * (T(1) / T(g.cell)));
        if (f > T(g.dims[a]) + T(1) && sa[a] >= T(0)) return true;
        if (f < T(-2) && sa[a] <= T(0)) return true;
    }
    return false;
}

// Visit the canonical neighbour list of cell (cx,cy,cz): rows (z, y) in
// increasing order, each row a contiguous sorted range over x-1..x+1.
template <typename F> inline void for_rows(const Scene& s, int cx, int cy, int cz, F&& f) {
    const int W = s.g.dims[0], Hh = s.g.dims[1], D = s.g.dims[2];
    int x0 = std::max(cx - 1, 0), x1 = std::min(cx + 1, W - 1);
    if (x0 > x1) return;
    for (int z = cz - 1; z <= cz + 1; ++z) {
        if (z < 0 || z >= D) continue;
        for (int y = cy - 1; y <= cy + 1; ++y) {
            if (y < 0 || y >= Hh) continue;
            int64_t row = (int64_t(z) * Hh + y) * W;
            f(s.start[row + x0], s.start[row + x1 + 1]);
        }
    }
}

template <typename T> inline T density(const Scene& s, const Cubic<T>& k, V3<T> p, EvalStats& st) {
    int cx, cy, cz;
    st.evals++;
    if (!sample_cell(s.g, p, cx, cy, cz)) return T(0);
    T rho = T(0);
    for_rows(s, cx, cy, cz, [&](uint32_t b, uint32_t e) {
        st.candidates += int64_t(e - b);
        for (uint32_t j = b; j < e; ++j) {
            const float* q = s.sorted + 4 * size_t(j);
            V3<T> r{T(q[0]) - p.x, T(q[1]) - p.y, T(q[2]) - p.z};
            T q2 = dot(r, r);
            if (q2 < k.h2) rho = rho + k.W_in(q2);
        }
    });
    return rho;
}

template <typename T> inline V3<T> grad_sum(const Scene& s, const Cubic<T>& k, V3<T> p) {
    int cx, cy, cz;
    V3<T> g{T(0), T(0), T(0)};
    if (!sample_cell(s.g, p, cx, cy, cz)) return g;
    for_rows(s, cx, cy, cz, [&](uint32_t b, uint32_t e) {
        for (uint32_t j = b; j < e; ++j) {
            const float* q = s.sorted + 4 * size_t(j);
            V3<T> r{T(q[0]) - p.x, T(q[1]) - p.y, T(q[2]) - p.z};
            T q2 = dot(r, r);
            if (q2 < k.h2 && q2 > T(0)) g = add(g, k.gradW_in(r, q2));
        }
    });
    return g;
}

// intersectAABB, RayMarcher.cpp:51-62 with glm's min/max semantics:
// glm::min(x, y) = (y < x) ? y : x, glm::max(x, y) = (x < y) ? y : x,
// std::max(a, b) = (a < b) ? b : a.
inline float gmin(float x, float y) { return (y < x) ? y : x; }
inline float gmax(float x, float y) { return (x < y) ? y : x; }
inline V3<float> intersect_aabb(V3<float> o, V3<float> d, V3<float> bmin, V3<float> bmax) {
    V3<float> tmin{(bmin.x - o.x) / d.x, (bmin.y - o.y) / d.y, (bmin.z - o.z) / d.z};
    V3<float> tmax{(bmax.x - o.x) / d.x, (bmax.y - o.y) / d.y, (bmax.z - o.z) / d.z};
    V3<float> t1{gmin(tmin.x, tmax.x), gmin(tmin.y, tmax.y), gmin(tmin.z, tmax.z)};
    V3<float> t2{gmax(tmin.x, tmax.x), gmax(tmin.y, tmax.y), gmax(tmin.z, tmax.z)};
    float tnear = gmax(gmax(t1.x, t1.y), t1.z);
    float tfar = gmin(gmin(t2.x, t2.y), t2.z);
    float t = (tnear < tfar) ? tfar : tnear;
    return t >= 0.0f ? add(o, mul(d, t)) : o;
}

// Reference skip loop (mode 2), RayMarcher.cpp:284-306.  QueryDensityGrid
// returns the cell only when 0 <= x < W etc.; the loop is capped so that a
// degenerate input cannot spin forever (the reference has no cap).
inline V3<float> ref_skip(const Scene& s, V3<float> p, V3<float> step) {
    const OrcGrid& g = s.g;
    for (int it = 0; it < (1 << 20); ++it) {
        float fx = std::floor((p.x - g.min[0]) * g.inv);
        float fy = std::floor((p.y - g.min[1]) * g.inv);
        float fz = std::floor((p.z - g.min[2]) * g.inv);
        if (!(fx >= 0.0f && fx < float(g.dims[0]) && fy >= 0.0f && fy < float(g.dims[1]) && fz >= 0.0f &&
              fz < float(g.dims[2])))
            return p;
        int x = int(fx), y = int(fy), z = int(fz);
        int64_t c = x + int64_t(y) * g.dims[0] + int64_t(z) * g.dims[0] * g.dims[1];
        if (s.ref_flag[c]) return p;
        // node->Min = m_Min + vec3(x, y, z) * cellWidth; node->Max = Min + vec3(cellWidth)
        V3<float> bmin{g.min[0] + float(x) * g.cell, g.min[1] + float(y) * g.cell, g.min[2] + float(z) * g.cell};
        V3<float> bmax{bmin.x + g.cell, bmin.y + g.cell, bmin.z + g.cell};
        p = add(intersect_aabb(p, step, bmin, bmax), step);
    }
    return p;
}

// composition.frag:99-108 sampleFloor(a, r)
template <typename T> inline void sample_floor(V3<T> a, V3<T> r, T out[4]) {
    const T FLOOR_HEIGHT = T(-1);
    // b = a + r * (FLOOR_HEIGHT - a.y) / r.y
    T s = FLOOR_HEIGHT - a.y;
    V3<T> t = mul(r, s);
    t = divs(t, r.y);
    V3<T> b = add(a, t);
    // f = step(mod(b.xz, 2), 1): mod(x, y) = x - y * floor(x / y); step(e, x) = x < e ? 0 : 1
    T mx = b.x - T(2) * std::floor(b.x / T(2));
    T mz = b.z - T(2) * std::floor(b.z / T(2));
    T fx = (T(1) < mx) ? T(0) : T(1);
    T fz = (T(1) < mz) ? T(0) : T(1);
    T c = T(0.25) + (fx + fz) / T(4);
    out[0] = c; out[1] = c; out[2] = c; out[3] = T(0.5);
}

// composition.frag:121-128 viewRay(): far-plane point under pixel centre UV
template <typename T> inline V3<T> view_ray(const OrcCamera& cam, int px, int py) {
    T u = (T(px) + T(0.5)) / T(cam.width);
    T v = (T(py) + T(0.5)) / T(cam.height);
    T in[4] = {T(2) * u - T(1), T(2) * v - T(1), T(1), T(1)};
    T o[4];
    mat4_mul<T>(cam.inv_proj_view, in, o);
    return V3<T>{o[0] / o[3], o[1] / o[3], o[2] / o[3]};
}

// composition.frag:132-184, the active branch.
template <typename T> inline void shade(const OrcCamera& cam, int px, int py, bool hit, V3<T> world, V3<T> n,
                                        T out[4]) {
    V3<T> cam_pos{T(cam.position[0]), T(cam.position[1]), T(cam.position[2])};
    V3<T> vr = view_ray<T>(cam, px, py);
    if (!hit) {
        T fl[4];
        sample_floor<T>(cam_pos, vr, fl);
        for (int i = 0; i < 4; ++i) out[i] = T(0.75) * fl[i];
        return;
    }
    // refract(normalize(viewRay()), normal, 1.333), glm compute_refract order
    V3<T> I = normalize(vr);
    const T eta = T(1.333f);
    T dv = dot(n, I);
    T k = T(1) - (eta * eta) * (T(1) - dv * dv);
    V3<T> refr{T(0), T(0), T(0)};
    if (k >= T(0)) {
        T c = eta * dv + std::sqrt(k);
        refr = sub(mul(eta, I), mul(c, n));
    }
    T fl[4];
    sample_floor<T>(world, refr, fl);
    // CameraDirection = System[2] = row 2 of the view matrix's 3x3 block
    V3<T> cdir{T(cam.view[2]), T(cam.view[6]), T(cam.view[10])};
    T f = -dot(cdir, n);
    const T diffuse[4] = {T(120.0f / 255.0f), T(185.0f / 255.0f), T(255.0f / 255.0f), T(255.0f / 255.0f)};
    T kd = (T(0.15f) + T(1)) - f * f;
    for (int i = 0; i < 4; ++i) out[i] = f * fl[i] + kd * diffuse[i];
}

struct MarchOut {
    float* pos;      // 4 per pixel or null
    float* nrm;      // 4 per pixel or null
    float* depth;    // 1 per pixel or null (hit distance, 0 on miss)
    float* colour;   // 4 per pixel or null
    int32_t* evals;  // per pixel density evaluations or null
    int64_t* cand;   // per pixel candidates scanned or null
    double* rho;     // per pixel density at the reported hit point or null
};

// ivl (optional, 2 per pixel): a proposed interval (ks, kf) of the learned
// march: start at sample ks of this ray's lattice (ks additions of the step),
// evaluate samples ks+1 .. kf, and restart as the full march when the first of
// them is already inside or none of them is (the GPU's FM_MARCH_PROPOSAL).
template <typename T>
void march_pixel(const Scene& s, const OrcCamera& cam, const OrcParams& P, const float* depth_in, int64_t idx,
                 const MarchOut& o, const int32_t* ivl = nullptr) {
    const int W = cam.width, Hh = cam.height;
    const int px = int(idx % W), py = int(idx / W);
    Cubic<T> k(s.H);
    EvalStats st;
    bool hit = false;
    V3<T> hp{0, 0, 0}, nn{0, 0, 0};
    T hit_rho = T(0);
    const float z = depth_in[idx];
    if (z != 1.0f) {
        // RayMarcher.cpp:268-274
        T twoWinv = T(2) / T(W), twoHinv = T(2) / T(Hh);
        if (std::is_same<T, float>::value) { twoWinv = T(2.0f / float(W)); twoHinv = T(2.0f / float(Hh)); }
        T clip[4] = {T(float(px)) * twoWinv - T(1), T(float(py)) * twoHinv - T(1), T(z), T(1)};
        T wh[4];
        mat4_mul<T>(cam.inv_proj_view, clip, wh);
        V3<T> p{wh[0] / wh[3], wh[1] / wh[3], wh[2] / wh[3]};
        V3<T> cam_pos{T(cam.position[0]), T(cam.position[1]), T(cam.position[2])};
        V3<T> step = mul(T(P.step), normalize(sub(p, cam_pos)));
        const V3<T> p0 = p;
        int ks = 0, kf = -1;
        if (ivl) {
            ks = ivl[2 * idx];
            kf = ivl[2 * idx + 1];
            if (!(ks >= 1 && ks < kf && kf <= P.max_steps)) { ks = 0; kf = -1; }
        }
    attempt:
        p = p0;
        int i0 = 0;
        if (kf >= 0) {
            for (int k = 0; k < ks; ++k) p = add(p, step);
            i0 = ks;
        }
        V3<T> prev = p;
        bool restart = false;
        for (int i = i0; i < (kf >= 0 ? kf : P.max_steps); ++i) {
            p = add(p, step);
            if (P.skip_mode == 2 && s.ref_flag) {
                if (std::is_same<T, float>::value) {
                    V3<float> pf{float(p.x), float(p.y), float(p.z)};
                    V3<float> sf{float(step.x), float(step.y), float(step.z)};
                    pf = ref_skip(s, pf, sf);
                    p = V3<T>{T(pf.x), T(pf.y), T(pf.z)};
                }
            }
            // Past the grid's evaluation range, or (iso > 0) past the zero-density box, on an
            // axis the step moves away from: every later sample has density 0, so stop (same
            // outputs as marching on).
            if (outside_forever(s.g, p, step) || (P.iso > 0.0f && leaving_zero_box(s.g, p, step))) break;
            T rho = density(s, k, p, st);
            if (rho >= T(P.iso)) {
                if (kf >= 0 && i == ks) { restart = true; break; }
                hit = true;
                hit_rho = rho;
                break;
            }
            prev = p;
        }
        if (kf >= 0 && !hit) restart = true;
        if (restart) {
            kf = -1;
            ks = 0;
            goto attempt;
        }
        if (hit) {
            V3<T> lo = prev, hi = p;
            for (int b = 0; b < P.bisect_iters; ++b) {
                V3<T> mid{(lo.x + hi.x) * T(0.5), (lo.y + hi.y) * T(0.5), (lo.z + hi.z) * T(0.5)};
                T rho = density(s, k, mid, st);
                if (rho >= T(P.iso)) { hi = mid; hit_rho = rho; }
                else lo = mid;
            }
            hp = hi;
            nn = normalize(grad_sum(s, k, hp));
        }
    }
    if (o.pos) {
        float* d = o.pos + 4 * idx;
        d[0] = hit ? float(hp.x) : 0.f; d[1] = hit ? float(hp.y) : 0.f; d[2] = hit ? float(hp.z) : 0.f;
        d[3] = hit ? 1.f : 0.f;
    }
    if (o.nrm) {
        float* d = o.nrm + 4 * idx;
        d[0] = hit ? float(nn.x) : 0.f; d[1] = hit ? float(nn.y) : 0.f; d[2] = hit ? float(nn.z) : 0.f;
        d[3] = hit ? 1.f : 0.f;
    }
    if (o.depth) {
        T dd = T(0);
        if (hit) {
            V3<T> cam_pos{T(cam.position[0]), T(cam.position[1]), T(cam.position[2])};
            V3<T> r = sub(hp, cam_pos);
            dd = std::sqrt(dot(r, r));
        }
        o.depth[idx] = float(dd);
    }
    if (o.colour) {
        T c[4];
        shade<T>(cam, px, py, hit, hp, nn, c);
        for (int i = 0; i < 4; ++i) o.colour[4 * idx + i] = float(c[i]);
    }
    if (o.evals) o.evals[idx] = int32_t(st.evals);
    if (o.cand) o.cand[idx] = st.candidates;
    if (o.rho) o.rho[idx] = double(hit_rho);
}

// ---- anisotropic march (RayMarcher.cpp:114-254, 346-423; Kernel.cpp:55-107) ----

struct OrcAniso {
    float radius_mult;  // ParticleRadiusExt / ParticleRadius (Dataset.cpp:175)
    float k_n, k_r, k_s;
    int32_t n_eps;
    int32_t pad;
};

// Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations
// (Jacobi's method; Golub & Van Loan, Matrix Computations, 8.5), in double:
// A = V diag(w) V^T, V's columns the eigenvectors.
inline void eig3_jacobi(const double Ain[3][3], double w[3], double V[3][3]) {
    double A[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            A[i][j] = Ain[i][j];
            V[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 32; ++sweep) {
        const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        const double diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (A[p][q] == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; ++k) {  // A <- J^T A J
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - sn * akq;
                    A[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - sn * aqk;
                    A[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - sn * vkq;
                    V[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

// WPCA at p over the extended neighbours x (RayMarcher.cpp:114-249): CubicKernel
// weights 1 - (|r| / Hext)^3, weighted mean and covariance, eigen-decomposition,
// the [YT13] eq. 15 clamp, G = (1/H) R Sigma^-1 R^T.  glm / Eigen FP32 order for
// the sums; the eigen-decomposition in double.  G as glm's mat3: G[col][row].
inline void wpca(V3<float> p, const std::vector<V3<float>>& x, float Hext, float Hinv, const OrcAniso& a,
                 float G[3][3]) {
    const size_t N = x.size();
    std::vector<float> wts(N);
    float wsum = 0.0f;
    V3<float> mean{0.0f, 0.0f, 0.0f};
    const float hinv_ext = 1.0f / Hext;
    for (size_t j = 0; j < N; ++j) {
        const V3<float> r = sub(x[j], p);
        const float d = std::sqrt(dot(r, r));
        float w = 0.0f;
        if (d < Hext) {
            const float k = d * hinv_ext;
            w = 1.0f - k * k * k;
        }
        wts[j] = w;
        wsum += w;
        mean = add(mean, mul(w, x[j]));
    }
    const float inv = 1.0f / wsum;
    mean = mul(mean, inv);
    float C[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (size_t j = 0; j < N; ++j) {
        const V3<float> d = sub(x[j], mean);
        const float v[3] = {d.x, d.y, d.z};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) C[r][c] += (wts[j] * v[r]) * v[c];  // (w x) x^T
    }
    double Cd[3][3], sig[3], R[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Cd[r][c] = double(C[r][c] * inv);
    eig3_jacobi(Cd, sig, R);
    float S[3];
    if (int64_t(N) <= int64_t(a.n_eps)) {
        S[0] = S[1] = S[2] = a.k_n;
    } else {
        const float mx = std::max(float(sig[0]), std::max(float(sig[1]), float(sig[2])));
        const float mn = mx / a.k_r;
        for (int k = 0; k < 3; ++k) S[k] = std::max(float(sig[k]), mn) * a.k_s;
    }
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            double g = 0.0;
            for (int k = 0; k < 3; ++k) g += R[r][k] * R[c][k] / double(S[k]);
            G[c][r] = float(double(Hinv) * g);
        }
}

// glm::determinant(mat3) cofactor expansion along the first column.
inline float det3(const float m[3][3]) {
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
           m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

// glm mat3 * vec3 (column-major): out_i = sum_j m[j][i] r_j, glm's add order.
inline V3<float> mat_vec(const float m[3][3], V3<float> r) {
    return {m[0][0] * r.x + m[1][0] * r.y + m[2][0] * r.z, m[0][1] * r.x + m[1][1] * r.y + m[2][1] * r.z,
            m[0][2] * r.x + m[1][2] * r.y + m[2][2] * r.z};
}

// AnisotropicKernel::W / gradW (Kernel.cpp:55-107): h = H, sig = 8 / pi.
inline float aniso_W(float H, const float G[3][3], float detG, V3<float> r0) {
    const V3<float> r = mat_vec(G, r0);
    float q = dot(r, r);
    if (q >= H * H) return 0.0f;
    q = std::sqrt(q) * (1.0f / H);
    const float sig = 8.0f / 3.14159265358979323846f;
    if (q >= 0.5f) {
        const float q_ = 1.0f - q;
        return sig * detG * (2.0f * q_ * q_ * q_);
    }
    return sig * detG * (6.0f * (q * q * q - q * q) + 1.0f);
}

inline V3<float> aniso_gradW(float H, const float G[3][3], float detG, V3<float> r0) {
    const V3<float> r = mat_vec(G, r0);
    const float rn = dot(r, r);
    if (rn >= H * H || rn == 0.0f) return {0.0f, 0.0f, 0.0f};
    const float rl = std::sqrt(rn);
    const float q = rl * (1.0f / H);
    const V3<float> gq = divs(normalize(r), rl * H);
    const float sig = 8.0f / 3.14159265358979323846f;
    if (q >= 0.5f) {
        const float q_ = 1.0f - q;
        return mul(mul(-sig * detG, gq), 6.0f * q_ * q_);
    }
    return mul(mul(sig * detG, gq), 6.0f * (3.0f * q * q - 2.0f * q));
}

// Neighbours of p within the extended radius (5x5x5 cells of width H in
// increasing linear index, each cell in sorted order), and the ones within H.
inline void aniso_neighbours(const Scene& s, V3<float> p, float Hext, std::vector<V3<float>>& ext,
                             std::vector<V3<float>>& rel) {
    ext.clear();
    rel.clear();
    int cx, cy, cz;
    if (!sample_cell_f32(s.g, p.x, p.y, p.z, cx, cy, cz)) return;
    const int W = s.g.dims[0], Hh = s.g.dims[1], D = s.g.dims[2];
    const float he2 = Hext * Hext, h2 = s.H * s.H;
    for (int z = std::max(cz - 2, 0); z <= std::min(cz + 2, D - 1); ++z)
        for (int y = std::max(cy - 2, 0); y <= std::min(cy + 2, Hh - 1); ++y) {
            const int x0 = std::max(cx - 2, 0), x1 = std::min(cx + 2, W - 1);
            if (x0 > x1) continue;
            const int64_t row = (int64_t(z) * Hh + y) * W;
            for (uint32_t j = s.start[row + x0]; j < s.start[row + x1 + 1]; ++j) {
                const float* q = s.sorted + 4 * size_t(j);
                const V3<float> xj{q[0], q[1], q[2]};
                const V3<float> r = sub(xj, p);
                const float d2 = dot(r, r);
                if (d2 < he2 && ext.size() < 8192) {
                    ext.push_back(xj);
                    if (d2 < h2) rel.push_back(r);
                }
            }
        }
}

// Density and G at p; false when p has no extended neighbour.
inline bool aniso_density(const Scene& s, V3<float> p, const OrcAniso& a, float& rho, float G[3][3], float& detG,
                          std::vector<V3<float>>& ext, std::vector<V3<float>>& rel) {
    const float Hext = a.radius_mult * s.H;
    aniso_neighbours(s, p, Hext, ext, rel);
    rho = 0.0f;
    if (ext.empty()) return false;
    wpca(p, ext, Hext, 1.0f / s.H, a, G);
    detG = det3(G);
    for (const auto& r : rel) rho += aniso_W(s.H, G, detG, r);
    return true;
}

void march_pixel_aniso(const Scene& s, const OrcCamera& cam, const OrcParams& P, const OrcAniso& A,
                       const float* depth_in, int64_t idx, const MarchOut& o) {
    const int W = cam.width, Hh = cam.height;
    const int px = int(idx % W), py = int(idx / W);
    bool hit = false;
    V3<float> hp{0, 0, 0}, nn{0, 0, 0};
    const float z = depth_in[idx];
    int64_t evals = 0;
    if (z != 1.0f) {
        const float twoWinv = 2.0f / float(W), twoHinv = 2.0f / float(Hh);
        float clip[4] = {float(px) * twoWinv - 1.0f, float(py) * twoHinv - 1.0f, z, 1.0f};
        float wh[4];
        mat4_mul<float>(cam.inv_proj_view, clip, wh);
        V3<float> p{wh[0] / wh[3], wh[1] / wh[3], wh[2] / wh[3]};
        V3<float> cam_pos{cam.position[0], cam.position[1], cam.position[2]};
        V3<float> step = mul(P.step, normalize(sub(p, cam_pos)));
        std::vector<V3<float>> ext, rel;
        float G[3][3], detG = 0.0f, rho = 0.0f;
        V3<float> prev = p;
        for (int i = 0; i < P.max_steps; ++i) {
            p = add(p, step);
            if (P.skip_mode == 2 && s.ref_flag) p = ref_skip(s, p, step);
            if (outside_forever(s.g, p, step)) break;
            ++evals;
            aniso_density(s, p, A, rho, G, detG, ext, rel);
            if (rho >= P.iso) {
                hit = true;
                break;
            }
            prev = p;
        }
        if (hit) {
            V3<float> lo = prev, hi = p;
            for (int b = 0; b < P.bisect_iters; ++b) {
                V3<float> mid{(lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f};
                ++evals;
                aniso_density(s, mid, A, rho, G, detG, ext, rel);
                if (rho >= P.iso) hi = mid;
                else lo = mid;
            }
            hp = hi;
            // RayMarcher.cpp:411-416: gradient sum with G at the hit point
            ++evals;
            aniso_density(s, hp, A, rho, G, detG, ext, rel);
            V3<float> g{0, 0, 0};
            for (const auto& r : rel) g = add(g, aniso_gradW(s.H, G, detG, r));
            nn = normalize(g);
        }
    }
    if (o.pos) {
        float* d = o.pos + 4 * idx;
        d[0] = hit ? hp.x : 0.f; d[1] = hit ? hp.y : 0.f; d[2] = hit ? hp.z : 0.f; d[3] = hit ? 1.f : 0.f;
    }
    if (o.nrm) {
        float* d = o.nrm + 4 * idx;
        d[0] = hit ? nn.x : 0.f; d[1] = hit ? nn.y : 0.f; d[2] = hit ? nn.z : 0.f; d[3] = hit ? 1.f : 0.f;
    }
    if (o.depth) {
        float dd = 0.0f;
        if (hit) {
            V3<float> r{hp.x - cam.position[0], hp.y - cam.position[1], hp.z - cam.position[2]};
            dd = std::sqrt(dot(r, r));
        }
        o.depth[idx] = dd;
    }
    if (o.evals) o.evals[idx] = int32_t(evals);
}

// Pi/2 as the depth shader writes it (1.57079632679), rounded to float.
constexpr float kHalfPi = 1.57079632679f;

// cos(t) for t in [0, pi/2] from its Taylor series (degree 16, Horner in t^2).
// Written out here and in the CUDA splat kernel with the same operation order,
// so both produce the same bits.  |error| < 2e-7 on the interval.
inline float cos_poly(float t) {
    // coefficients 1/(2k)! rounded to float, written as exact hex literals
    float x = t * t;
    float p = 0x1.ae7f3ep-45f;   // 1/16!
    p = p * x - 0x1.93974ap-37f; // 1/14!
    p = p * x + 0x1.1eed8ep-29f; // 1/12!
    p = p * x - 0x1.27e4fcp-22f; // 1/10!
    p = p * x + 0x1.a01a02p-16f; // 1/8!
    p = p * x - 0x1.6c16c2p-10f; // 1/6!
    p = p * x + 0x1.555556p-5f;  // 1/4!
    p = p * x - 0x1.0p-1f;       // 1/2!
    p = p * x + 1.0f;
    return p;
}

}  // namespace

extern "C" {

int orc_version() { return 1; }

float orc_cos_poly(float t) { return cos_poly(t); }

// W and gradW for known-answer tests (FP32, reference formulas).
float orc_W(float h, float rx, float ry, float rz) {
    Cubic<float> k(h);
    V3<float> r{rx, ry, rz};
    float q2 = dot(r, r);
    if (q2 >= k.h2) return 0.0f;
    return k.W_in(q2);
}
void orc_gradW(float h, float rx, float ry, float rz, float* out3) {
    Cubic<float> k(h);
    V3<float> r{rx, ry, rz};
    float q2 = dot(r, r);
    V3<float> g{0, 0, 0};
    if (q2 < k.h2 && q2 > 0.0f) g = k.gradW_in(r, q2);
    out3[0] = g.x; out3[1] = g.y; out3[2] = g.z;
}
float orc_sigma(float h) { return Cubic<float>(h).sig; }

// Frame::ComputeAABB + the grid part of BuildDensityGrid (Dataset.cpp:78-104).
int orc_grid_params(const float* xyz, int64_t n, int32_t stride, float H, OrcGrid* g) {
    if (n <= 0 || stride < 3 || !(H > 0.0f)) return 1;
    float mn[3] = {xyz[0], xyz[1], xyz[2]}, mx[3] = {xyz[0], xyz[1], xyz[2]};
    for (int64_t i = 0; i < n; ++i) {
        const float* p = xyz + i * stride;
        for (int a = 0; a < 3; ++a) {
            mx[a] = gmax(mx[a], p[a]);
            mn[a] = gmin(mn[a], p[a]);
        }
    }
    const float pad = 1.0f * H;
    for (int a = 0; a < 3; ++a) {
        g->max[a] = mx[a] + pad;
        g->min[a] = mn[a] - pad;
    }
    g->cell = 1.0f * H;
    g->inv = 1.0f / g->cell;
    for (int a = 0; a < 3; ++a) {
        float ext = g->max[a] - g->min[a];
        g->dims[a] = int32_t(std::ceil(ext / g->cell));
    }
    g->pad = 0;
    return 0;
}

// Per-particle linear cell index, QueryDensityGrid formula (Dataset.cpp:28-40),
// and the sort key cell * 8 + sub-cell: each cell is split into 2x2x2
// sub-cells at half the cell width, sx = (f - floor(f) >= 0.5) per axis with
// f = (p - min) * inv, sub = sx + 2 sy + 4 sz.  key may be null.
void orc_cells(const float* xyz, int64_t n, int32_t stride, const OrcGrid* g, uint32_t* cell, uint32_t* key) {
    for (int64_t i = 0; i < n; ++i) {
        const float* p = xyz + i * stride;
        int c[3];
        uint32_t sub = 0;
        for (int a = 0; a < 3; ++a) {
            float f = (p[a] - g->min[a]) * g->inv;
            // clamped into the grid; the support-radius padding keeps finite input inside
            c[a] = std::min(std::max(int(std::floor(f)), 0), g->dims[a] - 1);
            if (f - float(c[a]) >= 0.5f) sub |= 1u << a;
        }
        cell[i] = uint32_t(c[0]) + uint32_t(c[1]) * uint32_t(g->dims[0]) +
                  uint32_t(c[2]) * uint32_t(g->dims[0]) * uint32_t(g->dims[1]);
        if (key) key[i] = cell[i] * 8u + sub;
    }
}

// Stable counting sort by key: perm[k] = input index of the k-th sorted
// particle, start[c] .. start[c+1] the sorted range of key c.
void orc_sort(const uint32_t* key, int64_t n, int64_t nkeys, uint32_t* perm, uint32_t* start) {
    std::vector<uint32_t> cnt(size_t(nkeys) + 1, 0);
    for (int64_t i = 0; i < n; ++i) cnt[key[i]]++;
    uint32_t acc = 0;
    for (int64_t c = 0; c < nkeys; ++c) {
        start[c] = acc;
        acc += cnt[c];
    }
    start[nkeys] = acc;
    std::vector<uint32_t> cur(start, start + nkeys);
    for (int64_t i = 0; i < n; ++i) perm[cur[key[i]]++] = uint32_t(i);
}

// Reference skip flags (Dataset.cpp:137-164) with each cell's particle count
// as the find_neighbors_box result: Flag = (sum_27 exp(-1000*L1) * count) * W0 > 1.
void orc_ref_flags(const uint32_t* start, const OrcGrid* g, float H, uint8_t* flag) {
    const int W = g->dims[0], Hh = g->dims[1], D = g->dims[2];
    const float W0 = Cubic<float>(H).sig;
    for (int x = 0; x < W; ++x)
        for (int y = 0; y < Hh; ++y)
            for (int z = 0; z < D; ++z) {
                float Nc = 0.0f;
                for (int dx = -1; dx <= 1; ++dx)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dz = -1; dz <= 1; ++dz) {
                            int xx = x + dx, yy = y + dy, zz = z + dz;
                            if (xx < 0 || xx >= W || yy < 0 || yy >= Hh || zz < 0 || zz >= D) continue;
                            int64_t c = xx + int64_t(yy) * W + int64_t(zz) * W * Hh;
                            const float C = 1000.0f;
                            const float r = float(std::abs(dx) + std::abs(dy) + std::abs(dz));
                            const float w = std::exp(-C * r);
                            Nc += w * float(start[c + 1] - start[c]);
                        }
                float rho = Nc * W0;
                flag[x + int64_t(y) * W + int64_t(z) * W * Hh] = rho > 1.0f ? 1 : 0;
            }
}

// Sphere-splat depth (restated raster of depth.vert/depth.frag).  For every
// pixel centre whose view ray meets the particle's camera-facing disc of radius
// R (l2 = |UV|^2 <= 1), depth = proj_z(view_z - R*cos(pi/2*sqrt(l2))); LESS
// test against a buffer cleared to 1.0.  Particles whose disc is not entirely
// in front of the camera (view_z - R <= 0) and fragments outside [0, 1) are
// dropped.  depth must hold width*height floats and is overwritten.
void orc_splat(const float* xyz, int64_t n, int32_t stride, float R, const OrcCamera* cam, float* depth) {
    const int W = cam->width, Hh = cam->height;
    for (int64_t i = 0; i < int64_t(W) * Hh; ++i) depth[i] = 1.0f;
    const float* V = cam->view;
    const float* P = cam->proj;
    const float P00 = P[0], P11 = P[5], P22 = P[10], P32 = P[14], P23 = P[11], P33 = P[15];
    const float invR = 1.0f / R;
    const float twoWinv = 2.0f / float(W), twoHinv = 2.0f / float(Hh);
    for (int64_t i = 0; i < n; ++i) {
        const float* pp = xyz + i * stride;
        if (!std::isfinite(pp[0]) || !std::isfinite(pp[1]) || !std::isfinite(pp[2])) continue;
        float v[4] = {pp[0], pp[1], pp[2], 1.0f}, c[4];
        mat4_mul<float>(V, v, c);
        float cx = c[0] / c[3], cy = c[1] / c[3], cz = c[2] / c[3];
        if (!(cz - R > 0.0f)) continue;
        // conservative pixel bounding box of the disc
        float nx0 = P00 * (cx - R) / cz, nx1 = P00 * (cx + R) / cz;
        float ny0 = P11 * (cy - R) / cz, ny1 = P11 * (cy + R) / cz;
        float xa = std::min(nx0, nx1), xb = std::max(nx0, nx1);
        float ya = std::min(ny0, ny1), yb = std::max(ny0, ny1);
        float fx0 = std::floor((xa + 1.0f) * 0.5f * float(W) - 0.5f) - 1.0f;
        float fx1 = std::ceil((xb + 1.0f) * 0.5f * float(W) - 0.5f) + 1.0f;
        float fy0 = std::floor((ya + 1.0f) * 0.5f * float(Hh) - 0.5f) - 1.0f;
        float fy1 = std::ceil((yb + 1.0f) * 0.5f * float(Hh) - 0.5f) + 1.0f;
        if (fx1 < 0.0f || fy1 < 0.0f || fx0 > float(W - 1) || fy0 > float(Hh - 1)) continue;
        int x0 = std::max(0, int(std::max(fx0, -1.0f))), x1 = std::min(W - 1, int(std::min(fx1, float(W))));
        int y0 = std::max(0, int(std::max(fy0, -1.0f))), y1 = std::min(Hh - 1, int(std::min(fy1, float(Hh))));
        for (int y = y0; y <= y1; ++y) {
            float ny = (float(y) + 0.5f) * twoHinv - 1.0f;
            float vy = (ny * cz) / P11;
            float vv = (vy - cy) * invR;
            for (int x = x0; x <= x1; ++x) {
                float nx = (float(x) + 0.5f) * twoWinv - 1.0f;
                float vx = (nx * cz) / P00;
                float uu = (vx - cx) * invR;
                float l2 = uu * uu + vv * vv;
                if (l2 > 1.0f) continue;
                float off = cos_poly(kHalfPi * std::sqrt(l2));
                float zv = cz - R * off;
                float d = (P22 * zv + P32) / (P23 * zv + P33);
                if (!(d >= 0.0f && d < 1.0f)) continue;
                d = d + 0.0f;  // -0 -> +0
                float& dst = depth[int64_t(y) * W + x];
                if (d < dst) dst = d;
            }
        }
    }
}

// March the given pixels (or all when pixels == null) on `threads` threads
// (<= 0: hardware_concurrency - 1, as RayMarcher.cpp:67).  precision 32 or 64.
// sorted: cell-sorted xyz with stride 4; start: ncells + 1 offsets.
int orc_march_ivl(const float* sorted, const uint32_t* start, const OrcGrid* g, float H, const uint8_t* ref_flag,
                  const OrcCamera* cam, const OrcParams* P, const float* depth_in, const int64_t* pixels, int64_t npix,
                  int32_t threads, int32_t precision, float* out_pos, float* out_nrm, float* out_depth,
                  float* out_col, int32_t* out_evals, int64_t* out_cand, double* out_rho, const int32_t* ivl) {
    Scene s{sorted, start, *g, H, ref_flag};
    MarchOut o{out_pos, out_nrm, out_depth, out_col, out_evals, out_cand, out_rho};
    const int64_t total = pixels ? npix : int64_t(cam->width) * cam->height;
    int nt = threads > 0 ? threads : std::max(1, int(std::thread::hardware_concurrency()) - 1);
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            int64_t k = next.fetch_add(1);
            if (k >= total) break;
            int64_t idx = pixels ? pixels[k] : k;
            if (precision == 64) march_pixel<double>(s, *cam, *P, depth_in, idx, o, ivl);
            else march_pixel<float>(s, *cam, *P, depth_in, idx, o, ivl);
        }
    };
    if (nt == 1) { worker(); return 0; }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    return 0;
}

int orc_march(const float* sorted, const uint32_t* start, const OrcGrid* g, float H, const uint8_t* ref_flag,
              const OrcCamera* cam, const OrcParams* P, const float* depth_in, const int64_t* pixels, int64_t npix,
              int32_t threads, int32_t precision, float* out_pos, float* out_nrm, float* out_depth, float* out_col,
              int32_t* out_evals, int64_t* out_cand, double* out_rho) {
    return orc_march_ivl(sorted, start, g, H, ref_flag, cam, P, depth_in, pixels, npix, threads, precision, out_pos,
                         out_nrm, out_depth, out_col, out_evals, out_cand, out_rho, nullptr);
}

// Anisotropic march (RayMarcher.cpp:346-423) of the given pixels (or all),
// bisect_iters refining the hit as in the isotropic march.
int orc_march_aniso(const float* sorted, const uint32_t* start, const OrcGrid* g, float H, const uint8_t* ref_flag,
                    const OrcCamera* cam, const OrcParams* P, const OrcAniso* A, const float* depth_in,
                    const int64_t* pixels, int64_t npix, int32_t threads, float* out_pos, float* out_nrm,
                    float* out_depth, int32_t* out_evals) {
    Scene s{sorted, start, *g, H, ref_flag};
    MarchOut o{out_pos, out_nrm, out_depth, nullptr, out_evals, nullptr, nullptr};
    const int64_t total = pixels ? npix : int64_t(cam->width) * cam->height;
    int nt = threads > 0 ? threads : std::max(1, int(std::thread::hardware_concurrency()) - 1);
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            int64_t k = next.fetch_add(1);
            if (k >= total) break;
            march_pixel_aniso(s, *cam, *P, *A, depth_in, pixels ? pixels[k] : k, o);
        }
    };
    if (nt == 1) { worker(); return 0; }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    return 0;
}

// Anisotropic density at arbitrary points.
void orc_density_aniso(const float* sorted, const uint32_t* start, const OrcGrid* g, float H, const OrcAniso* A,
                       const float* pts, int64_t n, float* out) {
    Scene s{sorted, start, *g, H, nullptr};
    std::vector<V3<float>> ext, rel;
    float G[3][3], detG, rho;
    for (int64_t i = 0; i < n; ++i) {
        aniso_density(s, V3<float>{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, *A, rho, G, detG, ext, rel);
        out[i] = rho;
    }
}

// Density at arbitrary points (FP32 canonical order, or FP64).
void orc_density(const float* sorted, const uint32_t* start, const OrcGrid* g, float H, const float* pts, int64_t n,
                 int32_t precision, double* out) {
    Scene s{sorted, start, *g, H, nullptr};
    EvalStats st;
    for (int64_t i = 0; i < n; ++i) {
        if (precision == 64) {
            Cubic<double> k(H);
            out[i] = density<double>(s, k, V3<double>{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, st);
        } else {
            Cubic<float> k(H);
            out[i] = density<float>(s, k, V3<float>{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, st);
        }
    }
}

// ---- depth Gaussian blur (GaussRenderPass.cpp:13-57,347-355, gauss.frag) ----

// ComputeGaussKernel (GaussRenderPass.cpp:24-57): weights for i, j = 0..N at
// out[j + i (N + 1)], normalised over the whole (2N+1)^2 grid.
void orc_gauss_weights(int32_t N, float* out) {
    const float e = 2.71828182845904523536f;
    float sum = 0.0f;
    for (int i = 0; i <= N; ++i)
        for (int j = 0; j <= N; ++j) {
            const float r = std::sqrt((float)i * (float)i + (float)j * (float)j);
            const float y = std::pow(e, -0.5f * r * r);
            out[j + i * (N + 1)] = y;
            if (i == 0 && j == 0) sum += y;
            else if (i != 0 && j != 0) sum += 4.0f * y;
            else sum += 2.0f * y;
        }
    for (int k = 0; k < (N + 1) * (N + 1); ++k) out[k] /= sum;
}

// gauss.frag: sum over i (outer) and j (inner) of weight(|i|, |j|) times the
// depth texture at UV + (i, j) * (spread / W, spread / H), UV the pixel centre;
// linear filtering (texel coordinate u W - 1/2, floor, fraction kept to 8
// sub-texel bits), clamp-to-edge.  FP32, every operation rounded separately.
void orc_depth_blur(const float* in, float* out, int32_t W, int32_t H, int32_t N, float spread) {
    std::vector<float> w((size_t)(N + 1) * (N + 1));
    orc_gauss_weights(N, w.data());
    const float tw = spread / (float)W, th = spread / (float)H;
    auto texel = [&](int x, int y) {
        x = std::min(std::max(x, 0), W - 1);
        y = std::min(std::max(y, 0), H - 1);
        return in[(size_t)y * W + x];
    };
    auto sample = [&](float s, float t) {
        const float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
        const float fu = std::floor(u), fv = std::floor(v);
        float al = u - fu, be = v - fv;
        al = std::nearbyint(al * 256.0f) * 0.00390625f;
        be = std::nearbyint(be * 256.0f) * 0.00390625f;
        const int i0 = (int)std::fmax(std::fmin(fu, (float)W), -1.0f);
        const int j0 = (int)std::fmax(std::fmin(fv, (float)H), -1.0f);
        const float t00 = texel(i0, j0), t10 = texel(i0 + 1, j0), t01 = texel(i0, j0 + 1), t11 = texel(i0 + 1, j0 + 1);
        const float ia = 1.0f - al, ib = 1.0f - be;
        return (ia * ib) * t00 + (al * ib) * t10 + (ia * be) * t01 + (al * be) * t11;
    };
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const float u0 = ((float)x + 0.5f) / (float)W, v0 = ((float)y + 0.5f) / (float)H;
            float sum = 0.0f;
            for (int i = -N; i <= N; ++i) {
                const float s = u0 + (float)i * tw;
                for (int j = -N; j <= N; ++j) {
                    const float t = v0 + (float)j * th;
                    sum = sum + w[(size_t)std::abs(i) * (N + 1) + std::abs(j)] * sample(s, t);
                }
            }
            out[(size_t)y * W + x] = sum;
        }
}

}  // extern "C"
