/*
 * ALGLIB stand-in used only to compile the reference solver as a CPU oracle
 * (test infrastructure; never linked into the product).
 *
 * The reference calls two routines of ALGLIB's 2-D spline unit (version not
 * pinned: README.md:8,17-53; call sites include/coreLB.hpp:1217-1224 and
 * :1535-1540):
 *   spline2dbuildbicubicv(x, n, y, m, f, d, s)  with f[d*(n*j+i)] = F(x[i], y[j])
 *   spline2dcalc(s, x, y)
 * This file restates ALGLIB's published bicubic spline:
 *   - the nodes are sorted ascending in x and in y (the value table is permuted
 *     with them);
 *   - the node derivatives dF/dx, dF/dy and d2F/dxdy are the node slopes of 1-D
 *     cubic splines with "parabolically terminated" ends (ALGLIB boundary type
 *     0), built along each row, each column, and along each column of dF/dx;
 *     with only two nodes such a spline degenerates to the straight line;
 *   - evaluation is bicubic Hermite interpolation on the cell found by a binary
 *     search clamped to the first/last cell, so points outside the node range are
 *     extrapolated with the boundary cell's polynomial.
 */
#pragma once
#include <vector>
#include <stdexcept>
#include <cstddef>

namespace alglib
{
class real_1d_array
{
public:
    std::vector<double> v;
    void setlength(long n) { v.assign((size_t)n, 0.0); }
    long length() const { return (long)v.size(); }
    double &operator[](long i) { return v.at((size_t)i); }
    const double &operator[](long i) const { return v.at((size_t)i); }
};

struct spline2dinterpolant
{
    int n = 0, m = 0;
    std::vector<double> x, y;            // sorted nodes
    std::vector<double> f, fx, fy, fxy;  // [j*n + i]
};

namespace detail
{
// Node slopes of the 1-D cubic spline through (t[k], v[k]), k < cnt, with
// parabolically terminated ends (the end intervals are parabolas).
static inline void spline_slopes(const double *t, const double *v, int cnt, double *d)
{
    if (cnt == 2)
    {
        double s = (v[1] - v[0]) / (t[1] - t[0]);
        d[0] = s;
        d[1] = s;
        return;
    }
    // tridiagonal system a[k] d[k-1] + b[k] d[k] + c[k] d[k+1] = r[k]
    std::vector<double> a(cnt), b(cnt), c(cnt), r(cnt);
    // left end: d0 + d1 = 2 (v1 - v0) / h0
    a[0] = 0;
    b[0] = 1;
    c[0] = 1;
    r[0] = 2 * (v[1] - v[0]) / (t[1] - t[0]);
    for (int k = 1; k < cnt - 1; k++)
    {
        double h0 = t[k] - t[k - 1], h1 = t[k + 1] - t[k];
        a[k] = 1 / h0;
        b[k] = 2 * (1 / h0 + 1 / h1);
        c[k] = 1 / h1;
        r[k] = 3 * ((v[k] - v[k - 1]) / (h0 * h0) + (v[k + 1] - v[k]) / (h1 * h1));
    }
    int e = cnt - 1;
    a[e] = 1;
    b[e] = 1;
    c[e] = 0;
    r[e] = 2 * (v[e] - v[e - 1]) / (t[e] - t[e - 1]);
    // Thomas algorithm
    for (int k = 1; k < cnt; k++)
    {
        double w = a[k] / b[k - 1];
        b[k] -= w * c[k - 1];
        r[k] -= w * r[k - 1];
    }
    d[e] = r[e] / b[e];
    for (int k = e - 1; k >= 0; k--) d[k] = (r[k] - c[k] * d[k + 1]) / b[k];
}
} // namespace detail

static inline void spline2dbuildbicubicv(const real_1d_array &xa, long n, const real_1d_array &ya, long m,
                                         const real_1d_array &fa, long d, spline2dinterpolant &s)
{
    if (n < 2 || m < 2 || d != 1) throw std::runtime_error("alglib shim: unsupported spline size");
    s.n = (int)n;
    s.m = (int)m;
    s.x.assign(xa.v.begin(), xa.v.begin() + n);
    s.y.assign(ya.v.begin(), ya.v.begin() + m);
    s.f.assign(fa.v.begin(), fa.v.begin() + n * m);
    // selection sort of the x nodes (columns), then of the y nodes (rows)
    for (int j = 0; j < n; j++)
    {
        int k = j;
        for (int i = j + 1; i < n; i++)
            if (s.x[i] < s.x[k]) k = i;
        if (k != j)
        {
            std::swap(s.x[j], s.x[k]);
            for (int r = 0; r < m; r++) std::swap(s.f[r * n + j], s.f[r * n + k]);
        }
    }
    for (int i = 0; i < m; i++)
    {
        int k = i;
        for (int j = i + 1; j < m; j++)
            if (s.y[j] < s.y[k]) k = j;
        if (k != i)
        {
            std::swap(s.y[i], s.y[k]);
            for (int c = 0; c < n; c++) std::swap(s.f[i * n + c], s.f[k * n + c]);
        }
    }
    s.fx.assign(n * m, 0.0);
    s.fy.assign(n * m, 0.0);
    s.fxy.assign(n * m, 0.0);
    std::vector<double> row(n), drow(n), col(m), dcol(m);
    for (int r = 0; r < m; r++)
    {
        for (int c = 0; c < n; c++) row[c] = s.f[r * n + c];
        detail::spline_slopes(s.x.data(), row.data(), (int)n, drow.data());
        for (int c = 0; c < n; c++) s.fx[r * n + c] = drow[c];
    }
    for (int c = 0; c < n; c++)
    {
        for (int r = 0; r < m; r++) col[r] = s.f[r * n + c];
        detail::spline_slopes(s.y.data(), col.data(), (int)m, dcol.data());
        for (int r = 0; r < m; r++) s.fy[r * n + c] = dcol[r];
        for (int r = 0; r < m; r++) col[r] = s.fx[r * n + c];
        detail::spline_slopes(s.y.data(), col.data(), (int)m, dcol.data());
        for (int r = 0; r < m; r++) s.fxy[r * n + c] = dcol[r];
    }
}

static inline double spline2dcalc(const spline2dinterpolant &s, double x, double y)
{
    int l = 0, r = s.n - 1;
    while (l != r - 1)
    {
        int h = (l + r) / 2;
        if (s.x[h] >= x) r = h;
        else l = h;
    }
    int ix = l;
    l = 0;
    r = s.m - 1;
    while (l != r - 1)
    {
        int h = (l + r) / 2;
        if (s.y[h] >= y) r = h;
        else l = h;
    }
    int iy = l;
    double hx = s.x[ix + 1] - s.x[ix], hy = s.y[iy + 1] - s.y[iy];
    double t = (x - s.x[ix]) / hx, u = (y - s.y[iy]) / hy;
    double t2 = t * t, t3 = t2 * t, u2 = u * u, u3 = u2 * u;
    // cubic Hermite basis: value weights H0, H1 and slope weights G0, G1 (scaled by the spacing)
    double H[2] = {2 * t3 - 3 * t2 + 1, -2 * t3 + 3 * t2};
    double G[2] = {(t3 - 2 * t2 + t) * hx, (t3 - t2) * hx};
    double K[2] = {2 * u3 - 3 * u2 + 1, -2 * u3 + 3 * u2};
    double L[2] = {(u3 - 2 * u2 + u) * hy, (u3 - u2) * hy};
    double v = 0;
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
        {
            int k = (iy + b) * s.n + (ix + a);
            v += H[a] * K[b] * s.f[k] + G[a] * K[b] * s.fx[k] + H[a] * L[b] * s.fy[k] + G[a] * L[b] * s.fxy[k];
        }
    return v;
}
} // namespace alglib
