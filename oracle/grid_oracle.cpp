// CPU restatement of the reference's grid construction -- TEST INFRASTRUCTURE
// ONLY (see grid_oracle.h for the reference functions it follows).
//
// The reference builds its grid with hash maps and searches over every cell
// (Grid2D::rebuildGrid scans all cells for each interface cell); the same
// steps here use per-row lists of cells and dense position tables so that a
// 1024 x 1024 three-level image builds in seconds.  Every decision, every loop
// order that fixes a cell or table order, and every floating-point expression
// whose value reaches a table is kept as the reference has it.

#include "grid_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include <omp.h>

// the reference's boundary-type tables (include/system_files/*.txt), compiled in
#include "reference_tables.h"

namespace
{
using i64 = int64_t;

thread_local std::string g_error;

const int EX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1}; // include/globalParameters.hpp lattice e_x
const int EY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1}; // e_y

// ------------------------------------------------------------------ distances
// cv::distanceTransform(DIST_L2, DIST_MASK_PRECISE) as the reference calls it
// (include/shape.hpp:190-213, include/grid.hpp:367-380): the Euclidean
// distance of every non-zero pixel to the nearest zero pixel, in float.  The
// squared distance is found exactly in integers with the linear-time algorithm
// of Meijster, Roerdink and Hesselink ("A general algorithm for computing
// distance transforms in linear time", 2000), then rounded by a
// single-precision square root.  No zero pixel at all gives 3.4e38.
i64 floor_div(i64 a, i64 b) // b > 0
{
    i64 q = a / b;
    return (a % b != 0 && a < 0) ? q - 1 : q;
}

std::vector<float> distance_transform(const std::vector<uint8_t> &nonzero, int rows, int cols)
{
    const i64 INF = (i64)rows + cols; // above every in-image distance along a line
    std::vector<i64> g((size_t)rows * cols);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < cols; c++)
    {
        // phase 1: distance to the nearest zero of the same column
        g[c] = nonzero[c] ? INF : 0;
        for (int r = 1; r < rows; r++)
            g[(size_t)r * cols + c] = nonzero[(size_t)r * cols + c] ? 1 + g[(size_t)(r - 1) * cols + c] : 0;
        for (int r = rows - 2; r >= 0; r--)
        {
            i64 &v = g[(size_t)r * cols + c];
            const i64 below = g[(size_t)(r + 1) * cols + c];
            if (below < v) v = 1 + below;
        }
    }
    std::vector<float> out((size_t)rows * cols);
#pragma omp parallel
    {
        std::vector<i64> s(cols), t(cols);
#pragma omp for schedule(static)
        for (int r = 0; r < rows; r++)
        {
            // phase 2: lower envelope of the parabolas (x - u)^2 + g(u)^2 along the row
            const i64 *gr = &g[(size_t)r * cols];
            auto f = [&](i64 x, i64 i) { return (x - i) * (x - i) + gr[i] * gr[i]; };
            auto sep = [&](i64 i, i64 u) { return floor_div(u * u - i * i + gr[u] * gr[u] - gr[i] * gr[i], 2 * (u - i)); };
            int q = 0;
            s[0] = 0;
            t[0] = 0;
            for (int u = 1; u < cols; u++)
            {
                while (q >= 0 && f(t[q], s[q]) > f(t[q], u)) q--;
                if (q < 0)
                {
                    q = 0;
                    s[0] = u;
                }
                else
                {
                    const i64 w = 1 + sep(s[q], u);
                    if (w < cols)
                    {
                        q++;
                        s[q] = u;
                        t[q] = w;
                    }
                }
            }
            for (int u = cols - 1; u >= 0; u--)
            {
                const i64 d2 = f(u, s[q]);
                out[(size_t)r * cols + u] = d2 >= INF * INF ? 3.4e38f : std::sqrt((float)d2);
                if (u == t[q]) q--;
            }
        }
    }
    return out;
}

// ------------------------------------------------------------------ thinning
// utils::thinning (include/utils.hpp:436-537): Zhang-Suen sub-iterations 0 and
// 1, each marking over the image as it stands and then clearing the marks,
// repeated until a pair of sub-iterations changes nothing; the outermost rows
// and columns are never examined.  Only a foreground pixel with a background
// 8-neighbour can be marked (A == 1 needs a 0 -> 1 transition), so each
// sub-iteration examines just those: the survivors of the last list plus the
// foreground neighbours of the pixels just cleared.
void zhang_suen(std::vector<uint8_t> &im, int rows, int cols)
{
    if (rows <= 3 || cols <= 3) throw std::runtime_error("thinning needs an image larger than 3x3");
    auto px = [&](int r, int c) -> int { return im[(size_t)r * cols + c]; };
    std::vector<uint8_t> listed((size_t)rows * cols, 0);
    std::vector<i64> border, marks, grown;
    for (int r = 1; r < rows - 1; r++)
        for (int c = 1; c < cols - 1; c++)
        {
            if (!px(r, c)) continue;
            bool bg = false;
            for (int k = 1; k < 9 && !bg; k++) bg = !px(r + EY[k], c + EX[k]);
            if (bg)
            {
                border.push_back((i64)r * cols + c);
                listed[(size_t)r * cols + c] = 1;
            }
        }
    for (;;)
    {
        bool changed = false;
        for (int iter = 0; iter < 2; iter++)
        {
            marks.clear();
            for (i64 p : border)
            {
                const int r = (int)(p / cols), c = (int)(p % cols);
                const int no = px(r - 1, c), ne = px(r - 1, c + 1), ea = px(r, c + 1), se = px(r + 1, c + 1);
                const int so = px(r + 1, c), sw = px(r + 1, c - 1), we = px(r, c - 1), nw = px(r - 1, c - 1);
                const int A = (no == 0 && ne == 1) + (ne == 0 && ea == 1) + (ea == 0 && se == 1) + (se == 0 && so == 1) +
                              (so == 0 && sw == 1) + (sw == 0 && we == 1) + (we == 0 && nw == 1) + (nw == 0 && no == 1);
                const int B = no + ne + ea + se + so + sw + we + nw;
                const int m1 = iter == 0 ? no * ea * so : no * ea * we;
                const int m2 = iter == 0 ? ea * so * we : no * so * we;
                if (A == 1 && B >= 2 && B <= 5 && m1 == 0 && m2 == 0) marks.push_back(p);
            }
            if (marks.empty()) continue;
            changed = true;
            for (i64 p : marks) im[(size_t)p] = 0;
            grown.clear();
            for (i64 p : border)
            {
                if (im[(size_t)p]) grown.push_back(p);
                else listed[(size_t)p] = 0;
            }
            for (i64 p : marks)
            {
                const int r = (int)(p / cols), c = (int)(p % cols);
                for (int k = 1; k < 9; k++)
                {
                    const int rr = r + EY[k], cc = c + EX[k];
                    if (rr < 1 || rr > rows - 2 || cc < 1 || cc > cols - 2) continue;
                    const size_t pp = (size_t)rr * cols + cc;
                    if (im[pp] && !listed[pp])
                    {
                        listed[pp] = 1;
                        grown.push_back((i64)pp);
                    }
                }
            }
            border.swap(grown);
        }
        if (!changed) break;
    }
}

// utils::distanceToNearestWallIndex (include/utils.hpp:116-134): the first
// skeleton pixel, row by row over the square of half-width D + 2 around (i, j),
// whose distance from (i, j) is within 1e-4 of D.  The loop bounds are the
// reference's: a double start truncated to an integer, a double end.
i64 nearest_skeleton(const std::vector<uint8_t> &skel, int n, int i, int j, double D)
{
    if (!(D >= 0.0 && D <= 4.0 * n)) return -1; // no skeleton pixel anywhere
    for (i64 row = (i64)(i - D - 2); (double)row < i + D + 2; row++)
    {
        if (row < 0 || row >= n) continue;
        for (i64 col = (i64)(j - D - 2); (double)col < j + D + 2; col++)
        {
            if (col < 0 || col >= n || !skel[(size_t)row * n + col]) continue;
            const double di = (double)(i - row), dj = (double)(j - col);
            const double distance = std::sqrt(di * di + dj * dj);
            if (std::fabs(distance - D) < 1.0e-4) return row * n + col;
        }
    }
    return -1;
}

// Shape::calculateProperties (include/shape.hpp:127-251) for an n x n domain.
i64 pore_properties(const std::vector<int> &domain, int n, double resolution, double mfp, std::vector<double> &locpore,
                    std::vector<double> &kn)
{
    // the image in the middle of a 3n x 3n frame whose side bands (rows 1 .. n-2) are void
    const int ne = n + 2 * n, st = n;
    std::vector<uint8_t> ex((size_t)ne * ne, 0);
    for (int i = -st; i < n + st; i++)
        for (int j = -st; j < n + st; j++)
        {
            uint8_t v = 0;
            if (i >= 0 && i < n && j >= 0 && j < n) v = domain[(size_t)i * n + j] == 1;
            else if (i >= 1 && i < n - 1 && (j < 0 || j >= n)) v = 1;
            ex[(size_t)(i + st) * ne + (j + st)] = v;
        }
    zhang_suen(ex, ne, ne);
    std::vector<uint8_t> skel((size_t)n * n), dom((size_t)n * n), off_skel((size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            const size_t k = (size_t)i * n + j;
            skel[k] = ex[(size_t)(i + st) * ne + (j + st)] != 0;
            dom[k] = domain[k] != 0;
            off_skel[k] = !skel[k];
        }
    const std::vector<float> to_wall = distance_transform(dom, n, n);
    const std::vector<float> to_skel = distance_transform(off_skel, n, n);
    locpore.assign((size_t)n * n, 0.0);
    kn.assign((size_t)n * n, 0.0);
    i64 failed = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : failed)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            const size_t k = (size_t)i * n + j;
            if (domain[k] != 1) continue;
            const i64 hit = nearest_skeleton(skel, n, i, j, (double)to_skel[k]);
            double mid;
            if (hit >= 0) mid = domain[(size_t)hit] == 1 ? (double)to_wall[(size_t)hit] * (double)skel[(size_t)hit] : 0.0;
            else
            {
                // the reference would index outside its arrays here; never seen
                failed++;
                mid = (double)to_wall[k];
            }
            locpore[k] = 2.0 * mid;
            kn[k] = mfp / locpore[k] / resolution;
        }
    return failed;
}

// utils::resizeBinaryImage (include/utils.hpp:539-568) by a power-of-two
// factor: bilinear sampling at (x + 0.5) f - 0.5 falls midway between source
// pixels f x + f/2 - 1 and f x + f/2 in each axis, so the output is the rounded
// mean (s + 2) >> 2 of that 2 x 2 block of 0/255 values, kept where above 128
// (three or four void pixels of the four).
std::vector<int> resize_binary(const std::vector<int> &img, int n, int f)
{
    if (f == 1)
    {
        std::vector<int> out(img.size());
        for (size_t k = 0; k < img.size(); k++) out[k] = img[k] ? 1 : 0;
        return out;
    }
    const int m = n / f, o = f / 2 - 1;
    std::vector<int> out((size_t)m * m);
    for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++)
        {
            const int r = f * i + o, c = f * j + o;
            const int s = 255 * ((img[(size_t)r * n + c] != 0) + (img[(size_t)r * n + c + 1] != 0) +
                                 (img[(size_t)(r + 1) * n + c] != 0) + (img[(size_t)(r + 1) * n + c + 1] != 0));
            out[(size_t)i * m + j] = ((s + 2) >> 2) > 128 ? 1 : 0;
        }
    return out;
}

// ------------------------------------------------------------------ the grid
struct Tables
{
    int n = 0, max_level = 1;
    i64 N = 0;
    std::vector<int32_t> x, y, level, type, is_buffer, bnd;
    std::vector<i64> lin, conn;
    std::vector<double> tau, kn, locpore;
    std::vector<i64> stream_id, stream_loc, wall_id, per_id, per_i2;
    std::vector<int32_t> stream_ic, wall_ic, per_ic;
    std::vector<i64> coarse_rows, fine_rows, parent_child; // 6, 6 and 5 per row
    i64 inlet = -1, inlet2 = -1, outlet = -1, outlet2 = -1;
    i64 buffer_wall_links = 0;
};

struct GridBuilder
{
    const int32_t *pore;
    const double *kn_in, *lp_in;
    int n;
    OracleGridOptions opt;
    Tables T;

    GridBuilder(const int32_t *p, const double *k, const double *lp, int size, const OracleGridOptions &o)
        : pore(p), kn_in(k), lp_in(lp), n(size), opt(o)
    {
    }

    // original cells (every quadtree leaf, solid ones too) in the order of
    // Grid2D::rebuildGrid: raster order of their top-left pixels
    std::vector<int32_t> oc, orow, olvl;
    std::vector<uint8_t> opore;

    i64 sub2ind(int col, int row, int lvl0) const { return (i64)col + (i64)row * n + (i64)lvl0 * n * n; }

    // ---- Grid2D::processMultigrid / quadtreeDecompose / backwardsQuadTree
    // (include/grid.hpp:313-399, 1160-1266): leaf numbers per pixel, the
    // leaves numbered 1, 2, ... depth first over the quadrants top-left,
    // top-right, bottom-left, bottom-right; negative for solid leaves.
    std::vector<i64> leaf;
    std::vector<int> leaf_side;
    std::vector<float> dwall;
    std::vector<i64> solid_sum; // (n+1)^2 summed-area table of solid pixels
    i64 leaves = 0;

    void quadtree(int r0, int c0, int size, int min_dist)
    {
        const double alpha = 0.99;
        const int h = size / 2;
        const int qr[4] = {r0, r0, r0 + h, r0 + h}, qc[4] = {c0, c0 + h, c0, c0 + h};
        for (int k = 0; k < 4; k++)
        {
            const int R = qr[k], Cc = qc[k];
            auto S = [&](int r, int c) { return solid_sum[(size_t)r * (n + 1) + c]; };
            const i64 solids = S(R + h, Cc + h) - S(R, Cc + h) - S(R + h, Cc) + S(R, Cc);
            const double beta = (double)solids / (double)((i64)h * h); // utils::calculateRatio
            bool divide = false;
            if (h > 1)
            {
                float mn = FLT_MAX;
                for (int r = R; r < R + h; r++)
                    for (int c = Cc; c < Cc + h; c++) mn = std::min(mn, dwall[(size_t)r * n + c]);
                if ((double)mn < (double)((size_t)min_dist * (size_t)h)) divide = true;
            }
            if (std::log2((double)h) + 1 > opt.max_allowed_level) divide = true;
            // this build's option: quadrants on an x edge are refined to single pixels
            if (opt.edge_fine && h > 1 && (Cc == 0 || Cc + h == n)) divide = true;
            if (((1.0 - alpha) < beta && beta < alpha) || divide)
            {
                quadtree(R, Cc, h, min_dist);
                continue;
            }
            leaves++;
            const i64 v = beta > alpha ? -leaves : leaves;
            for (int r = R; r < R + h; r++)
                for (int c = Cc; c < Cc + h; c++) leaf[(size_t)r * n + c] = v;
            leaf_side.push_back(h);
        }
    }

    void original_cells()
    {
        const size_t nn = (size_t)n * n;
        leaf.assign(nn, 0);
        if (!opt.multiblock)
        {
            // Grid2D::processSinglegrid (include/grid.hpp:401-424): one leaf per pixel
            for (size_t k = 0; k < nn; k++) leaf[k] = pore[k] == 0 ? -(i64)(k + 1) : (i64)(k + 1);
            leaf_side.assign(nn + 1, 1);
        }
        else
        {
            if (n < 2 || (n & (n - 1))) throw std::runtime_error("Matrix dimensions must be divisible by 2 in each direction.");
            std::vector<uint8_t> nz(nn);
            solid_sum.assign((size_t)(n + 1) * (n + 1), 0);
            for (int r = 0; r < n; r++)
                for (int c = 0; c < n; c++)
                {
                    const int sol = pore[(size_t)r * n + c] == 0;
                    nz[(size_t)r * n + c] = !sol;
                    solid_sum[(size_t)(r + 1) * (n + 1) + c + 1] = solid_sum[(size_t)r * (n + 1) + c + 1] +
                                                                   solid_sum[(size_t)(r + 1) * (n + 1) + c] -
                                                                   solid_sum[(size_t)r * (n + 1) + c] + sol;
                }
            dwall = distance_transform(nz, n, n);
            leaf_side.assign(1, 0); // numbers start at 1
            const int min_dist = (int)std::ceil(std::pow(2, opt.max_allowed_level - 1) * std::sqrt(2));
            quadtree(0, 0, n, min_dist);
        }
        // Grid2D::rebuildGrid (include/grid.hpp:427-558): a cell per leaf at its
        // first pixel in raster order, level log2(sqrt(pixels)) + 1
        std::vector<uint8_t> seen(leaf_side.size(), 0);
        int maxl = 1;
        for (int r = 0; r < n; r++)
            for (int c = 0; c < n; c++)
            {
                const i64 v = leaf[(size_t)r * n + c];
                const size_t a = (size_t)(v < 0 ? -v : v);
                if (opt.multiblock)
                {
                    if (seen[a]) continue;
                    seen[a] = 1;
                }
                const int s = opt.multiblock ? leaf_side[a] : 1;
                const int lvl = (int)(std::log2(std::sqrt((double)s * s)) + 1);
                maxl = std::max(maxl, lvl);
                oc.push_back(c);
                orow.push_back(r);
                olvl.push_back(lvl);
                opore.push_back(v > 0);
            }
        T.max_level = maxl;
    }

    void build();
};

void GridBuilder::build()
{
    T.n = n;
    original_cells();
    const int L = T.max_level;
    const size_t nn = (size_t)n * n, space = nn * (size_t)L;
    const i64 n_orig = (i64)oc.size();

    // position tables over (level, row, col): original cell there, and
    // "a cell exists there" (originals, then the buffers as they are made)
    std::vector<int32_t> orig_at(space, -1);
    for (i64 k = 0; k < n_orig; k++) orig_at[(size_t)sub2ind(oc[k], orow[k], olvl[k] - 1)] = (int32_t)k;
    std::vector<uint8_t> taken(space, 0);
    for (i64 k = 0; k < n_orig; k++) taken[(size_t)sub2ind(oc[k], orow[k], olvl[k] - 1)] = 1;

    // original cells per top-left row, ascending column (= ascending cell id)
    std::vector<std::vector<int32_t>> by_row(n);
    for (i64 k = 0; k < n_orig; k++) by_row[orow[k]].push_back((int32_t)k);

    // ---- buffer cells (include/grid.hpp:600-805)
    std::vector<i64> new_ids;
    std::vector<int32_t> new_types;
    const float base_range = (float)std::pow(2, L - 1);
    const float range = base_range;
    auto ind2sub = [&](i64 idx, int &c, int &r, int &l) {
        // utils::ind2sub with sizes {n, n, max_level}: C++ remainder and quotient
        c = (int)(idx % n);
        idx /= n;
        r = (int)(idx % n);
        idx /= n;
        l = (int)(idx % L);
    };
    for (i64 i = 0; i < n_orig; i++)
    {
        const int lv = olvl[i];
        const float shift = (float)(std::pow(2, lv - 2) - 0.5);
        const int jump = (int)std::pow(2, lv - 1);
        const float sx = (float)oc[i] + shift, sy = (float)orow[i] + shift;
        // DistantNeighborMap and MissingKeysMap of this cell (:600-650): same-level
        // positions within the base range, x outer, y inner
        std::vector<i64> neighbour_map, missing;
        for (float ic = sx - base_range; ic <= sx + base_range; ic += jump)
            for (float jc = sy - base_range; jc <= sy + base_range; jc += jump)
            {
                i64 idx;
                if (ic - shift < 0 || jc - shift < 0 || ic - shift >= n || jc - shift >= n) idx = -1;
                else idx = sub2ind((int)(ic - shift), (int)(jc - shift), lv - 1);
                if (idx >= 0 && orig_at[(size_t)idx] >= 0) neighbour_map.push_back(idx);
                else if (ic < 0 || jc < 0 || ic >= n || jc >= n) neighbour_map.push_back(-1);
                else
                {
                    neighbour_map.push_back(idx);
                    missing.push_back(idx);
                }
            }
        if (missing.empty() || lv <= 1) continue;
        // original cells whose top-left lies within the range, in cell order
        const float maxI = sx + range, maxJ = sy + range, minI = sx - range, minJ = sy - range;
        std::vector<int32_t> in_range;
        int max_level_in = 0;
        for (int r = std::max(0, (int)std::floor(minJ - shift)); r < n && (float)r + shift <= maxJ; r++)
        {
            if ((float)r + shift < minJ) continue;
            const auto &row = by_row[r];
            auto it = std::lower_bound(row.begin(), row.end(), 0, [&](int32_t k, int) { return (float)oc[k] + shift < minI; });
            for (; it != row.end() && (float)oc[*it] + shift <= maxI; ++it)
            {
                in_range.push_back(*it);
                max_level_in = std::max(max_level_in, (int)olvl[*it]);
            }
        }
        // rows were visited in ascending order and columns ascending within a
        // row, which is ascending cell id
        for (int32_t k : in_range)
        {
            const i64 idk = sub2ind(oc[k], orow[k], olvl[k] - 1);
            if (std::find(neighbour_map.begin(), neighbour_map.end(), idk) != neighbour_map.end())
            {
                // break this cell up into four cells of the level below
                const float shift_upper = (float)(std::pow(2, lv - 2) - 0.5);
                const int half = (int)std::pow(2, lv - 2);
                const int il = (int)(sx - shift_upper), jl = (int)(sy - shift_upper);
                const int kids[4][2] = {{il, jl}, {il + half, jl}, {il, jl + half}, {il + half, jl + half}};
                for (auto &kd : kids)
                {
                    const i64 id = sub2ind(kd[0], kd[1], lv - 2);
                    if (taken[(size_t)id]) continue;
                    taken[(size_t)id] = 1;
                    new_ids.push_back(id);
                    new_types.push_back(10 * (lv - 1) + lv);
                }
            }
            else if (max_level_in <= lv)
            {
                // upscale: the missing position nearest to this finer cell
                const float gx = (float)oc[k] + shift, gy = (float)orow[k] + shift;
                int best = 0;
                double best_d = std::numeric_limits<double>::max();
                for (size_t m = 0; m < missing.size(); m++)
                {
                    int mc, mr, ml;
                    ind2sub(missing[m], mc, mr, ml);
                    const float mx = (float)mc + shift, my = (float)mr + shift;
                    const double d = std::sqrt(static_cast<double>(std::pow(gx - mx, 2) + std::pow(gy - my, 2)));
                    if (d < best_d)
                    {
                        best_d = d;
                        best = (int)m;
                    }
                }
                const i64 id = missing[(size_t)best];
                if (id != -1 && !taken[(size_t)id])
                {
                    taken[(size_t)id] = 1;
                    new_ids.push_back(id);
                    new_types.push_back(10 * lv + lv - 1);
                    missing[(size_t)best] = -1;
                }
            }
        }
    }

    // ---- the grid: void original cells, then the buffers (:806-889)
    for (i64 k = 0; k < n_orig; k++)
    {
        if (!opore[k]) continue;
        T.lin.push_back(sub2ind(oc[k], orow[k], olvl[k] - 1));
        T.x.push_back(oc[k]);
        T.y.push_back(orow[k]);
        T.level.push_back(olvl[k]);
        T.type.push_back(0);
        T.is_buffer.push_back(0);
    }
    for (size_t b = 0; b < new_ids.size(); b++)
    {
        int c, r, l;
        ind2sub(new_ids[b], c, r, l);
        T.lin.push_back(new_ids[b]);
        T.x.push_back(c);
        T.y.push_back(r);
        T.level.push_back(l + 1);
        T.type.push_back(new_types[b]);
        T.is_buffer.push_back(1);
    }
    const i64 N = (i64)T.lin.size();
    T.N = N;

    // ---- Grid2D::getProperties (:891-898): inputs at each cell's top-left pixel
    T.kn.resize(N);
    T.locpore.resize(N);
    for (i64 c = 0; c < N; c++)
    {
        const size_t p = (size_t)T.y[c] * n + T.x[c];
        T.kn[c] = kn_in[p];
        T.locpore[c] = lp_in[p];
    }

    // ---- Grid2D::buildConnections (:916-972)
    std::vector<i64> cell_at(space, -1);
    for (i64 c = 0; c < N; c++) cell_at[(size_t)T.lin[c]] = c;
    T.conn.assign((size_t)N * 9, -2);
#pragma omp parallel for schedule(static)
    for (i64 c = 0; c < N; c++)
    {
        const int jump = (int)std::pow(2, T.level[c] - 1);
        for (int q = 0; q < 9; q++)
        {
            int ip = T.x[c] + EX[q] * jump, jp = T.y[c] + EY[q] * jump;
            jp = (jp <= -1) ? jp + n : jp;
            jp = (jp >= n) ? jp - n : jp;
            ip = (ip <= -1) ? ip + n : ip;
            ip = (ip >= n) ? ip - n : ip;
            const i64 ng = sub2ind(ip, jp, T.level[c] - 1);
            i64 v;
            if (cell_at[(size_t)ng] >= 0) v = cell_at[(size_t)ng];
            else if (orig_at[(size_t)ng] >= 0) v = -1; // a (solid) original cell: a wall
            else v = -2;                               // no cell at that level: interpolated
            T.conn[(size_t)c * 9 + q] = v;
        }
    }

    if (opt.multiblock)
    {
        // ---- Grid2D::determineParentChild (:974-1038)
        for (i64 c = 0; c < N; c++)
        {
            if (T.level[c] <= 1) continue;
            const int jump = (int)std::pow(2, T.level[c] - 1);
            const int i = T.x[c], j = T.y[c], d = T.level[c];
            const int kids[4][2] = {{i, j}, {i + jump / 2, j}, {i, j + jump / 2}, {i + jump / 2, j + jump / 2}};
            T.parent_child.push_back(c);
            for (auto &kd : kids) T.parent_child.push_back(cell_at[(size_t)sub2ind(kd[0], kd[1], d - 2)]);
        }
        const i64 npc = (i64)T.parent_child.size() / 5;
        // first row (rows in order, columns in order) holding an id anywhere / as a child
        std::vector<i64> first_any(N, -1), first_child(N, -1);
        for (i64 r = npc - 1; r >= 0; r--)
            for (int k = 4; k >= 0; k--)
            {
                const i64 id = T.parent_child[(size_t)r * 5 + k];
                if (id < 0) continue;
                first_any[id] = r;
                if (k > 0) first_child[id] = r;
            }
        // ---- Grid2D::orderBufferIndex (:1041-1108)
        for (int lv = L; lv >= 2; lv--)
        {
            const int key = 10 * lv + lv - 1;
            for (i64 c = 0; c < N; c++)
                if (T.type[c] == key)
                {
                    const i64 r = first_any[c];
                    T.coarse_rows.push_back(key);
                    for (int k = 0; k < 5; k++) T.coarse_rows.push_back(T.parent_child[(size_t)r * 5 + k]);
                }
        }
        for (int lv = 1; lv < L; lv++)
        {
            const int key = 10 * lv + lv + 1;
            std::vector<i64> ids;
            for (i64 c = 0; c < N; c++)
                if (T.type[c] == key) ids.push_back(c);
            for (size_t s = 0; s + 4 <= ids.size(); s += 4)
            {
                i64 best = -1;
                for (int k = 0; k < 4; k++)
                {
                    const i64 r = first_child[ids[s + k]];
                    if (r >= 0 && (best < 0 || r < best)) best = r;
                }
                if (best < 0) continue; // the reference would use an unset parent here; never seen
                T.fine_rows.push_back(key);
                T.fine_rows.push_back(T.parent_child[(size_t)best * 5]);
                for (int k = 0; k < 4; k++) T.fine_rows.push_back(ids[s + k]);
            }
        }
    }

    // ---- Grid2D::getBoundaryTypes (:1111-1157)
    const int order[9] = {7, 3, 6, 4, 0, 2, 8, 1, 5};
    T.bnd.assign(N, -1);
    for (i64 c = 0; c < N; c++)
    {
        if (T.is_buffer[c]) continue;
        int code = 0;
        for (int k = 0; k < 9; k++) code = code * 2 + (T.conn[(size_t)c * 9 + order[k]] == -1 ? 0 : 1);
        if (code == 511) continue;
        int t = 0;
        while (t < ORACLE_N_BND_TYPES && ORACLE_BND_CODES[t] != code) t++;
        if (t == ORACLE_N_BND_TYPES) throw std::runtime_error("[ERROR]: Boundary type is not contained.");
        T.bnd[c] = t;
    }

    // ---- LB2D link lists and inlet/outlet cells (include/coreLB.hpp:280-366, one rank)
    const int thr = (int)std::pow(2, L - 1);
    const int ny_c = (n % 2 == 1) ? (n + 1) / 2 - 1 : n / 2 - 1;
    for (i64 i = 0; i < N; i++)
    {
        const int b = T.bnd[i];
        for (int q = 0; q < 9; q++)
        {
            const i64 nb = T.conn[(size_t)i * 9 + q];
            // a buffer cell has no boundary type; its wall links read ifStream[-1]
            // in the reference and are taken as walls here
            const bool streams = b == -1 ? (nb != -1) : ORACLE_IFSTREAM[b][q] != 0;
            if (nb >= 0 && nb < N)
            {
                const bool xp = std::abs(T.x[i] - T.x[nb]) > thr, yp = std::abs(T.y[i] - T.y[nb]) > thr;
                if (!xp && !yp)
                {
                    if (b == -1 || streams)
                    {
                        T.stream_id.push_back(i);
                        T.stream_ic.push_back(q);
                        T.stream_loc.push_back(nb);
                    }
                    else
                    {
                        T.wall_id.push_back(i);
                        T.wall_ic.push_back(q);
                    }
                }
                else if (xp)
                {
                    T.per_id.push_back(i);
                    T.per_i2.push_back(nb);
                    T.per_ic.push_back(q);
                }
            }
            else if (nb != -1)
            {
                if (!(b == -1 || streams))
                {
                    T.wall_id.push_back(i);
                    T.wall_ic.push_back(q);
                }
            }
            else if (!streams)
            {
                if (b == -1) T.buffer_wall_links++;
                T.wall_id.push_back(i);
                T.wall_ic.push_back(q);
            }
        }
        // one cell each is kept (the last that matches)
        if (T.y[i] == ny_c && T.x[i] == 0) T.inlet = i;
        else if (T.y[i] == ny_c && T.x[i] == n - 1) T.outlet = i;
        else if (T.y[i] == ny_c && T.x[i] == 1) T.inlet2 = i;
        else if (T.y[i] == ny_c && T.x[i] == n - 2) T.outlet2 = i;
    }

    // ---- relaxation times (include/coreLB.hpp:432-502)
    T.tau.assign(N, 0.0);
    const double k6pi = std::sqrt(6.0 / M_PI);
    if (!opt.multiblock)
    {
        for (i64 c = 0; c < N; c++) T.tau[c] = 0.5 + k6pi * T.locpore[c] * T.kn[c] / (1 + 2 * T.kn[c]);
        return;
    }
    std::vector<int> img(nn);
    for (size_t k = 0; k < nn; k++) img[k] = pore[k];
    std::vector<std::vector<double>> tau_level(L);
    for (int lv = 0; lv < L; lv++)
    {
        const double factor = std::pow(0.5, lv);
        const int m = (int)(n * factor);
        const std::vector<int> small = resize_binary(img, n, n / m);
        // a Shape of the resized size with solid first and last rows
        std::vector<int> dom((size_t)m * m, 1);
        for (int j = 0; j < m; j++)
        {
            dom[j] = 0;
            dom[(size_t)(m - 1) * m + j] = 0;
        }
        for (int i = 1; i < m - 1; i++)
            for (int j = 0; j < m; j++) dom[(size_t)i * m + j] = small[(size_t)i * m + j];
        std::vector<double> lp, knl;
        pore_properties(dom, m, opt.dx / factor, opt.mfp, lp, knl);
        tau_level[lv].resize((size_t)m * m);
        for (size_t k = 0; k < (size_t)m * m; k++) tau_level[lv][k] = 0.5 + k6pi * lp[k] * knl[k] / (1 + 2 * knl[k]);
    }
    for (i64 c = 0; c < N; c++)
    {
        const int lv = T.level[c];
        const int f = (int)std::pow(2, lv - 1);
        const int m = n / f;
        T.tau[c] = tau_level[lv - 1][(size_t)(T.y[c] / f) * m + (T.x[c] / f)];
    }
}

const void *ptr(const std::vector<int32_t> &v) { return v.empty() ? nullptr : v.data(); }
} // namespace

extern "C" {

int64_t oracle_pore_properties(const int32_t *domain, int n, double resolution, double mfp, double *locpore, double *kn)
{
    try
    {
        if (n <= 1) throw std::runtime_error("image too small");
        std::vector<int> dom(domain, domain + (size_t)n * n);
        std::vector<double> lp, k;
        const i64 failed = pore_properties(dom, n, resolution, mfp, lp, k);
        std::memcpy(locpore, lp.data(), lp.size() * sizeof(double));
        std::memcpy(kn, k.data(), k.size() * sizeof(double));
        return failed;
    }
    catch (const std::exception &e)
    {
        g_error = e.what();
        return -1;
    }
}

void *oracle_grid_create(const int32_t *pore, const double *kn, const double *locpore, int n,
                         const OracleGridOptions *opt)
{
    try
    {
        GridBuilder b(pore, kn, locpore, n, *opt);
        b.build();
        return new Tables(std::move(b.T)); // only the tables are kept
    }
    catch (const std::exception &e)
    {
        g_error = e.what();
        return nullptr;
    }
}

void oracle_grid_view(void *h, OracleGrid *g, OracleGridExtra *extra)
{
    const Tables &T = *static_cast<Tables *>(h);
    std::memset(g, 0, sizeof(*g));
    g->n = T.n;
    g->max_level = T.max_level;
    g->n_cells = T.N;
    g->x = T.x.data();
    g->y = T.y.data();
    g->level = T.level.data();
    g->type = T.type.data();
    g->is_buffer = T.is_buffer.data();
    g->bnd = T.bnd.data();
    g->conn = T.conn.data();
    g->tau = T.tau.data();
    g->kn = T.kn.data();
    g->n_stream = (int64_t)T.stream_id.size();
    g->stream_id = T.stream_id.data();
    g->stream_loc = T.stream_loc.data();
    g->stream_ic = static_cast<const int32_t *>(ptr(T.stream_ic));
    g->n_wall = (int64_t)T.wall_id.size();
    g->wall_id = T.wall_id.data();
    g->wall_ic = static_cast<const int32_t *>(ptr(T.wall_ic));
    g->n_per = (int64_t)T.per_id.size();
    g->per_id = T.per_id.data();
    g->per_i2 = T.per_i2.data();
    g->per_ic = static_cast<const int32_t *>(ptr(T.per_ic));
    g->n_coarse = (int64_t)T.coarse_rows.size() / 6;
    g->n_fine = (int64_t)T.fine_rows.size() / 6;
    g->coarse_rows = T.coarse_rows.data();
    g->fine_rows = T.fine_rows.data();
    g->inlet = T.inlet;
    g->inlet2 = T.inlet2;
    g->outlet = T.outlet;
    g->outlet2 = T.outlet2;
    if (extra)
    {
        extra->lin = T.lin.data();
        extra->locpore = T.locpore.data();
        extra->n_parent_child = (int64_t)T.parent_child.size() / 5;
        extra->parent_child = T.parent_child.data();
        extra->buffer_wall_links = T.buffer_wall_links;
    }
}

void oracle_grid_destroy(void *h) { delete static_cast<Tables *>(h); }

const char *oracle_grid_error(void) { return g_error.c_str(); }
}
