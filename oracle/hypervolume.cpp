/*
 * CPU oracle for the hypervolume indicator of 2 and 3 objectives (TEST
 * INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU leg of the
 * benchmark use it; the product library never links or loads it).
 *
 * Restates what pagmo's hypervolume::compute returns for 2 and 3 objectives
 * (src/utils/hypervolume.cpp:203-228 choosing hv2d / hv3d,
 * src/utils/hv_algos/hv_hv2d.cpp:48-68, hv_hv3d.cpp:75-116): the measure of the
 * region dominated by the points and bounded by the reference point, in long
 * double, as a sum of non-negative slabs: 2D, sorted by the second objective,
 * the width of the staircase (largest r0 - x0 so far) times the height of each
 * step; 3D, sorted by the third objective, the 2D area of the points below
 * each level times the thickness of the level. tests/test_oracle_hypervolume.py
 * pins it to the compiled reference (and to the reference's own test cases
 * where its tree is present).
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace
{
using ld = long double;

// 2D area dominated by the points idx[0..k) of p (x = coordinate 0, y = 1).
ld area_2d(const double *p, uint64_t m, std::vector<uint64_t> idx, const double *r)
{
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return p[a * m + 1] < p[b * m + 1]; });
    ld area = 0, w = 0;
    for (size_t t = 0; t < idx.size(); ++t) {
        const uint64_t q = idx[t];
        w = std::max(w, static_cast<ld>(r[0]) - static_cast<ld>(p[q * m]));
        const ld ynext = t + 1 < idx.size() ? static_cast<ld>(p[idx[t + 1] * m + 1]) : static_cast<ld>(r[1]);
        area += (ynext - static_cast<ld>(p[q * m + 1])) * w;
    }
    return area;
}
} // namespace

extern "C" {

int orc_hypervolume_ld(const double *pts, uint64_t n, uint64_t m, const double *r, double *out)
{
    if (n == 0 || (m != 2 && m != 3)) return 1;
    std::vector<uint64_t> idx(n);
    std::iota(idx.begin(), idx.end(), uint64_t(0));
    if (m == 2) {
        *out = static_cast<double>(area_2d(pts, m, idx, r));
        return 0;
    }
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return pts[a * m + 2] < pts[b * m + 2]; });
    ld v = 0;
    std::vector<uint64_t> prefix;
    prefix.reserve(n);
    for (uint64_t i = 0; i < n; ++i) {
        prefix.push_back(idx[i]);
        const ld znext = i + 1 < n ? static_cast<ld>(pts[idx[i + 1] * m + 2]) : static_cast<ld>(r[2]);
        const ld dz = znext - static_cast<ld>(pts[idx[i] * m + 2]);
        if (dz != 0) v += dz * area_2d(pts, m, prefix, r);
    }
    *out = static_cast<double>(v);
    return 0;
}

} // extern "C"

/*
 * WFG (pagmo's hvwfg with stop dimension 2, src/utils/hv_algos/hv_hvwfg.cpp),
 * in double and in the reference's order of operations, so that the values
 * are the reference's bit for bit:
 *  - vol(p, d) = |prod over k = d-1 .. 0 of (r_k - p_k)|
 *    (hv_algorithm::volume_between on pointers, hv_algorithm.cpp:73-82);
 *  - the limit set of p over candidates q: the points max(q, p) over the first
 *    d coordinates, filtered to the non-dominated ones, one copy of equal
 *    points (hvwfg::limitset, hv_hvwfg.cpp:134-193);
 *  - hv of a frame: one point -> vol; two -> vol + vol - intersection
 *    (coordinates in ascending order); two coordinates -> hv2d's sweep after
 *    sorting by the second coordinate (hv_hv2d.cpp:76-95); else the frame
 *    sorted by hvwfg::cmp_points (descending, last coordinate first) and
 *    H += |(p_j[d-1] - r[d-1]) * exclusive_j| in that order, exclusive_j =
 *    vol(p_j, d-1) - hv(limit set of p_j over the later points, d-1)
 *    (hvwfg::compute_hv and exclusive_hv, hv_hvwfg.cpp:196-272);
 *  - the contribution of point i: vol(p_i, m) - hv(limit set of p_i over
 *    every other point, m) (hvwfg::contributions, hv_hvwfg.cpp:79-105).
 * Frames hold rows of `stride` doubles, the first d of them in use.
 */
namespace
{
struct wfg_state {
    const double *r;

    static double dmax(double a, double b)
    {
        return a < b ? b : a; // std::max
    }

    double vol(const double *p, uint64_t d) const
    {
        double v = 1.0;
        for (uint64_t k = d; k-- > 0;) v *= (r[k] - p[k]);
        return v < 0 ? -v : v;
    }

    // rows src[t] for t in [begin, end) but skip, max'd with p over d
    // coordinates; the non-dominated ones, in the order they survive
    std::vector<double> limit(const double *src, uint64_t stride, uint64_t begin, uint64_t end, uint64_t skip,
                              const double *p, uint64_t d) const
    {
        std::vector<double> kept;
        std::vector<double> s(d);
        for (uint64_t t = begin; t < end; ++t) {
            if (t == skip) continue;
            for (uint64_t k = 0; k < d; ++k) s[k] = dmax(src[t * stride + k], p[k]);
            const uint64_t cnt = kept.size() / d;
            bool beaten = false; // a kept point is <= s everywhere and < s somewhere
            for (uint64_t q = 0; q < cnt && !beaten; ++q) {
                bool le = true, lt = false;
                for (uint64_t k = 0; k < d; ++k) {
                    le &= kept[q * d + k] <= s[k];
                    lt |= kept[q * d + k] < s[k];
                }
                beaten = le && lt;
            }
            if (beaten) continue;
            std::vector<double> next;
            next.reserve(kept.size() + d);
            for (uint64_t q = 0; q < cnt; ++q) {
                bool covered = true; // s <= kept point everywhere: s replaces it
                for (uint64_t k = 0; k < d; ++k) covered &= s[k] <= kept[q * d + k];
                if (!covered) next.insert(next.end(), kept.begin() + q * d, kept.begin() + (q + 1) * d);
            }
            next.insert(next.end(), s.begin(), s.end());
            kept.swap(next);
        }
        return kept;
    }

    double hv(std::vector<double> f, uint64_t d) const
    {
        const uint64_t k = f.size() / d;
        if (k == 1) return vol(f.data(), d);
        if (k == 2) {
            const double h = vol(f.data(), d) + vol(f.data() + d, d);
            double isect = 1.0;
            for (uint64_t i = 0; i < d; ++i) isect *= (r[i] - dmax(f[i], f[d + i]));
            return h - isect;
        }
        std::vector<uint64_t> ord(k);
        for (uint64_t i = 0; i < k; ++i) ord[i] = i;
        if (d == 2) {
            std::sort(ord.begin(), ord.end(), [&](uint64_t a, uint64_t b) { return f[a * d + 1] < f[b * d + 1]; });
            double area = 0.0, w = r[0] - f[ord[0] * d];
            for (uint64_t t = 0; t + 1 < k; ++t) {
                area += (f[ord[t + 1] * d + 1] - f[ord[t] * d + 1]) * w;
                w = dmax(w, r[0] - f[ord[t + 1] * d]);
            }
            return area + (r[1] - f[ord[k - 1] * d + 1]) * w;
        }
        std::sort(ord.begin(), ord.end(), [&](uint64_t a, uint64_t b) {
            for (uint64_t c = d; c-- > 0;) {
                if (f[a * d + c] != f[b * d + c]) return f[a * d + c] > f[b * d + c];
            }
            return false;
        });
        std::vector<double> sorted(k * d);
        for (uint64_t t = 0; t < k; ++t) std::copy(f.begin() + ord[t] * d, f.begin() + (ord[t] + 1) * d, sorted.begin() + t * d);
        double H = 0.0;
        for (uint64_t j = 0; j < k; ++j) {
            const double *p = sorted.data() + j * d;
            const std::vector<double> child = limit(sorted.data(), d, j + 1, k, k, p, d - 1);
            double ex = vol(p, d - 1);
            if (!child.empty()) ex -= hv(child, d - 1);
            H += std::fabs((p[d - 1] - r[d - 1]) * ex);
        }
        return H;
    }
};
} // namespace

extern "C" {

int orc_hvwfg(const double *pts, uint64_t n, uint64_t m, const double *ref, double *out)
{
    if (n == 0 || m < 2) return 1;
    const wfg_state w{ref};
    *out = w.hv(std::vector<double>(pts, pts + n * m), m);
    return 0;
}

int orc_hvwfg_contributions(const double *pts, uint64_t n, uint64_t m, const double *ref, double *out)
{
    if (n == 0 || m < 2) return 1;
    const wfg_state w{ref};
    for (uint64_t i = 0; i < n; ++i) {
        const double *p = pts + i * m;
        const std::vector<double> child = w.limit(pts, m, 0, n, i, p, m);
        double ex = w.vol(p, m);
        if (!child.empty()) ex -= w.hv(child, m);
        out[i] = ex;
    }
    return 0;
}

} // extern "C"
