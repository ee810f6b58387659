// Nearest skeleton pixel at a given distance: the search of
// utils::distanceToNearestWallIndex (include/utils.hpp:116-135) as called by
// Shape::calculateProperties (include/shape.hpp:227-236), shared by the host
// code and the GPU kernel.
//
// The reference scans the window rows [trunc(i - D - 2), i + D + 2) x columns
// [trunc(j - D - 2), j + D + 2) in raster order and returns the first pixel
// (r, c) with skel[r][c] set and |sqrt((i - r)^2 + (j - c)^2) - D| < 1e-4
// (the square root of the integer s = (i - r)^2 + (j - c)^2 in double), or -1.
// That costs O(D^2) double square roots per pixel.
//
// Here the test is decided on s alone: the double square root is monotonic in
// s, so the passing values of s form one interval [s_lo, s_hi], found once
// per pixel with the reference's own expression (a few evaluations next to
// (D -+ 1e-4)^2).  A row r (di = i - r) can then only pass at |j - c| = m with
// s_lo - di^2 <= m^2 <= s_hi - di^2, an integer-square-root range, visited in
// increasing column order (c = j - m for falling m, then c = j + m for rising
// m) under the reference's window bounds.  The passing pixels are exactly the
// reference's, in the same order, so the first hit is the reference's first
// hit.  Cost O(D) integer work per pixel.
#pragma once
#include <math.h>

#include <cstdint>

#if defined(__CUDACC__)
#define MANTIIS_HD __host__ __device__
#else
#define MANTIIS_HD
#endif

namespace mantiis
{
// floor(sqrt(x)) for 0 <= x < 2^53, exact: a float estimate corrected by
// integer comparisons
MANTIIS_HD inline int64_t isqrt_floor(int64_t x)
{
    int64_t r = (int64_t)sqrtf((float)x);
    while (r > 0 && r * r > x) r--;
    while ((r + 1) * (r + 1) <= x) r++;
    return r;
}

MANTIIS_HD inline bool within_distance(int64_t s, double D)
{
    return fabs(sqrt((double)s) - D) < 1.0e-4;
}

// skel: n*n row-major, non-zero on skeleton pixels.  Returns the linear index
// r * n + c of the hit, or -1.  D larger than any distance inside the image
// (no skeleton pixel at all gives the float maximum) returns -1 at once.
template <typename Pixel>
MANTIIS_HD inline int64_t nearest_skeleton_at(const Pixel *skel, int n, int i, int j, double D)
{
    const double tol = 1.0e-4;
    if (!(D >= 0.0 && D <= 2.0 * (double)n)) return -1;
    // the interval of passing squared distances: sqrt(s) - D rises with s
    const double lo = D - tol > 0.0 ? D - tol : 0.0;
    int64_t s_lo = (int64_t)(lo * lo);
    while (s_lo > 0 && sqrt((double)(s_lo - 1)) - D > -tol) s_lo--;
    while (!(sqrt((double)s_lo) - D > -tol)) s_lo++;
    int64_t s_hi = (int64_t)((D + tol) * (D + tol)) + 1;
    while (s_hi >= 0 && !(sqrt((double)s_hi) - D < tol)) s_hi--;
    while (sqrt((double)(s_hi + 1)) - D < tol) s_hi++;
    if (s_lo > s_hi || !within_distance(s_lo, D)) return -1;

    const int64_t r0 = (int64_t)(i - D - 2), c0 = (int64_t)(j - D - 2);
    const double r_end = i + D + 2, c_end = j + D + 2;
    for (int64_t r = r0 < 0 ? 0 : r0; r < n && (double)r < r_end; r++)
    {
        const int64_t di = (int64_t)i - r;
        const int64_t b = s_hi - di * di;
        if (b < 0) continue;
        const int64_t a = s_lo - di * di;
        const int64_t m_hi = isqrt_floor(b);
        int64_t m_lo = a > 0 ? isqrt_floor(a - 1) + 1 : 0; // ceil(sqrt(a))
        if (m_lo > m_hi) continue;
        // left side (c = j - m, m falling), then the right side (c = j + m, m
        // rising); m = 0 (c = j) once, on the left pass
        for (int side = 0; side < 2; side++)
            for (int64_t s = 0; s <= m_hi - m_lo; s++)
            {
                const int64_t m = side == 0 ? m_hi - s : m_lo + s;
                if (side == 1 && m == 0) continue;
                const int64_t c = side == 0 ? (int64_t)j - m : (int64_t)j + m;
                if (c < c0 || !((double)c < c_end) || c < 0 || c >= n) continue;
                if (skel[r * n + c]) return r * n + c;
            }
    }
    return -1;
}
} // namespace mantiis
