// Stand-in for the CompactNSearch neighbourhood search that the reference
// calls (src/app/Dataset.cpp:54-73, 128, 277, 287).  The library is an
// un-vendored submodule in the reference (vendor/CompactNSearch is empty), so
// this header is written from the library's documented behaviour, not from its
// source:
//   * NeighborhoodSearch(r): uniform-grid radius search with cell width r;
//   * add_point_set(x, n, ...): registers n xyz points (not copied);
//   * z_sort() + point_set(i).sort_field(a): reorders arrays into the
//     search's spatial order; update_point_sets() rebuilds the cell table;
//   * find_neighbors(p, out): out[0] = indices of points with |x - p| < r.
// Choices this stand-in makes (the real ordering is unpinned):
//   * the spatial order is a stable counting sort by the linear cell index of
//     the reference's density grid (origin = AABB min - r, width r, index
//     x + y*W + z*W*H, Dataset.cpp:26-47,78-104), then by 2x2x2 sub-cell
//     (half-width slabs, sx + 2 sy + 4 sz), so point i of the sorted set is at
//     sorted position i;
//   * find_neighbors lists the 27 cells around p in increasing linear index,
//     each cell in sorted order (the canonical order of the CUDA path);
//   * find_neighbors_box (a call of the reference's fork, Dataset.cpp:128)
//     answers by the global mode fm_shim_box_mode: 0 = one dummy index for every
//     cell (every skip flag true: skipping off), 1 = the points of the density
//     cell that contains p.
// Oracle build only.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

extern int fm_shim_box_mode;

namespace CompactNSearch
{

class PointSet
{
public:
    template <typename T>
    void sort_field(T* field) const
    {
        std::vector<T> tmp(field, field + m_Perm.size());
        for (std::size_t k = 0; k < m_Perm.size(); ++k) field[k] = tmp[m_Perm[k]];
    }

    std::size_t n_points() const { return m_N; }

    const float* m_X = nullptr;
    std::size_t m_N = 0;
    std::vector<uint32_t> m_Perm;
};

class NeighborhoodSearch
{
public:
    NeighborhoodSearch() = default;
    explicit NeighborhoodSearch(float r, bool = false) : m_R(r) {}

    unsigned int add_point_set(float const* x, std::size_t n, bool = true, bool = true, bool = true,
                               void* = nullptr)
    {
        PointSet ps;
        ps.m_X = x;
        ps.m_N = n;
        m_Sets.push_back(ps);
        return unsigned(m_Sets.size() - 1);
    }

    PointSet& point_set(unsigned int i) { return m_Sets[i]; }

    void z_sort()
    {
        for (auto& ps : m_Sets)
        {
            Build(ps);
            const std::size_t nkeys = 8 * m_NumCells;
            std::vector<uint32_t> cnt(nkeys + 1, 0);
            std::vector<uint32_t> cell(ps.m_N);
            for (std::size_t i = 0; i < ps.m_N; ++i) { cell[i] = KeyOf(ps.m_X + 3 * i); cnt[cell[i]]++; }
            std::vector<uint32_t> cur(nkeys + 1, 0);
            uint32_t acc = 0;
            for (std::size_t c = 0; c < nkeys; ++c) { cur[c] = acc; acc += cnt[c]; }
            ps.m_Perm.assign(ps.m_N, 0);
            for (std::size_t i = 0; i < ps.m_N; ++i) ps.m_Perm[cur[cell[i]]++] = uint32_t(i);
        }
    }

    void update_point_sets()
    {
        for (auto& ps : m_Sets) Build(ps);
        if (m_Sets.empty()) return;
        const PointSet& ps = m_Sets[0];
        m_Start.assign(m_NumCells + 1, 0);
        std::vector<uint32_t> cnt(m_NumCells, 0);
        for (std::size_t i = 0; i < ps.m_N; ++i) cnt[CellOf(ps.m_X + 3 * i)]++;
        uint32_t acc = 0;
        for (std::size_t c = 0; c < m_NumCells; ++c) { m_Start[c] = acc; acc += cnt[c]; }
        m_Start[m_NumCells] = acc;
    }

    void find_neighbors(float const* p, std::vector<std::vector<unsigned int>>& out) const
    {
        out.assign(1, {});
        if (m_Sets.empty()) return;
        const float* X = m_Sets[0].m_X;
        const float r2 = m_R * m_R;
        int cx, cy, cz;
        if (!SampleCell(p, cx, cy, cz)) return;
        int x0 = std::max(cx - 1, 0), x1 = std::min(cx + 1, m_Dims[0] - 1);
        if (x0 > x1) return;
        for (int z = cz - 1; z <= cz + 1; ++z)
        {
            if (z < 0 || z >= m_Dims[2]) continue;
            for (int y = cy - 1; y <= cy + 1; ++y)
            {
                if (y < 0 || y >= m_Dims[1]) continue;
                std::size_t row = (std::size_t(z) * m_Dims[1] + y) * m_Dims[0];
                for (uint32_t j = m_Start[row + x0]; j < m_Start[row + x1 + 1]; ++j)
                {
                    const float* q = X + 3 * std::size_t(j);
                    float rx = q[0] - p[0], ry = q[1] - p[1], rz = q[2] - p[2];
                    float tx = rx * rx, ty = ry * ry, tz = rz * rz;
                    if ((tx + ty) + tz < r2) out[0].push_back(j);
                }
            }
        }
    }

    void find_neighbors_box(float const* p, std::vector<std::vector<unsigned int>>& out) const
    {
        out.assign(1, {});
        if (fm_shim_box_mode == 0) { out[0].push_back(0); return; }
        int cx, cy, cz;
        if (!SampleCell(p, cx, cy, cz)) return;
        if (cx < 0 || cy < 0 || cz < 0 || cx >= m_Dims[0] || cy >= m_Dims[1] || cz >= m_Dims[2]) return;
        std::size_t c = cx + std::size_t(cy) * m_Dims[0] + std::size_t(cz) * m_Dims[0] * m_Dims[1];
        for (uint32_t j = m_Start[c]; j < m_Start[c + 1]; ++j) out[0].push_back(j);
    }

private:
    void Build(const PointSet& ps)
    {
        if (ps.m_N == 0) { m_Dims[0] = m_Dims[1] = m_Dims[2] = 1; m_NumCells = 1; return; }
        float mn[3] = {ps.m_X[0], ps.m_X[1], ps.m_X[2]}, mx[3] = {mn[0], mn[1], mn[2]};
        for (std::size_t i = 0; i < ps.m_N; ++i)
            for (int a = 0; a < 3; ++a)
            {
                float v = ps.m_X[3 * i + a];
                mx[a] = (mx[a] < v) ? v : mx[a];
                mn[a] = (v < mn[a]) ? v : mn[a];
            }
        for (int a = 0; a < 3; ++a)
        {
            m_Min[a] = mn[a] - 1.0f * m_R;
            float top = mx[a] + 1.0f * m_R;
            m_Dims[a] = int(std::ceil((top - m_Min[a]) / (1.0f * m_R)));
        }
        m_Inv = 1.0f / (1.0f * m_R);
        m_NumCells = std::size_t(m_Dims[0]) * m_Dims[1] * m_Dims[2];
    }

    uint32_t CellOf(const float* p) const
    {
        int x = int(std::floor((p[0] - m_Min[0]) * m_Inv));
        int y = int(std::floor((p[1] - m_Min[1]) * m_Inv));
        int z = int(std::floor((p[2] - m_Min[2]) * m_Inv));
        return uint32_t(x) + uint32_t(y) * uint32_t(m_Dims[0]) + uint32_t(z) * uint32_t(m_Dims[0]) * uint32_t(m_Dims[1]);
    }

    // cell * 8 + 2x2x2 sub-cell (sx + 2 sy + 4 sz, sx = frac >= 0.5)
    uint32_t KeyOf(const float* p) const
    {
        int c[3];
        uint32_t sub = 0;
        for (int a = 0; a < 3; ++a)
        {
            float f = (p[a] - m_Min[a]) * m_Inv;
            c[a] = std::min(std::max(int(std::floor(f)), 0), m_Dims[a] - 1);
            if (f - float(c[a]) >= 0.5f) sub |= 1u << a;
        }
        uint32_t lin = uint32_t(c[0]) + uint32_t(c[1]) * uint32_t(m_Dims[0]) +
                       uint32_t(c[2]) * uint32_t(m_Dims[0]) * uint32_t(m_Dims[1]);
        return lin * 8u + sub;
    }

    bool SampleCell(const float* p, int& cx, int& cy, int& cz) const
    {
        float fx = std::floor((p[0] - m_Min[0]) * m_Inv);
        float fy = std::floor((p[1] - m_Min[1]) * m_Inv);
        float fz = std::floor((p[2] - m_Min[2]) * m_Inv);
        if (!(fx >= -2.0f && fx <= float(m_Dims[0]) + 1.0f)) return false;
        if (!(fy >= -2.0f && fy <= float(m_Dims[1]) + 1.0f)) return false;
        if (!(fz >= -2.0f && fz <= float(m_Dims[2]) + 1.0f)) return false;
        cx = int(fx); cy = int(fy); cz = int(fz);
        return true;
    }

    float m_R = 0.0f;
    float m_Min[3] = {0, 0, 0};
    float m_Inv = 1.0f;
    int m_Dims[3] = {1, 1, 1};
    std::size_t m_NumCells = 1;
    std::vector<PointSet> m_Sets;
    std::vector<uint32_t> m_Start;
};

}  // namespace CompactNSearch
