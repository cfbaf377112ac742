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
