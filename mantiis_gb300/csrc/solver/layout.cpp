#include "layout.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "../boundary_tables.h"
#include "../d2q9.h"

namespace mantiis
{
namespace
{
// ordering key of a special record's site (x | y << 16): 8x4 blocks in row-major
// order, then row-major inside the block
// a special record is light when only missing arrivals (with their constant
// row) and buffer status make it special: no wall link, no x-periodic override,
// no quirk link, no inlet / outlet role
inline bool special_is_light(const SpecialRec &r)
{
    const uint32_t over = (r.m0 >> 9) & 0x1FFu, wall = (r.m0 >> 18) & 0x1FFu, quirk = r.m1 & 0x1FFu;
    const uint32_t flags = (r.m1 >> 17) & 0xFu;
    return !wall && !over && !quirk && !(flags & (SF_INLET | SF_OUTLET));
}

inline uint64_t special_order_key(int32_t xy)
{
    const uint64_t x = (uint64_t)(xy & 0xFFFF), y = (uint64_t)((uint32_t)xy >> 16);
    return ((y >> 2) << 40) | ((x >> 3) << 20) | ((y & 3) << 8) | (x & 7);
}
} // namespace

namespace
{
// Node slopes of the three-node cubic spline with parabolically terminated
// ends (the end intervals are parabolas): closed-form solution of
//   d0 + d1 = 2 s0,  d0/h0 + 2 (1/h0 + 1/h1) d1 + d2/h1 = 3 (s0/h0 + s1/h1),  d1 + d2 = 2 s1
// with s = secant slopes.
void slopes3(const double t[3], const double v[3], double d[3])
{
    double h0 = t[1] - t[0], h1 = t[2] - t[1];
    double s0 = (v[1] - v[0]) / h0, s1 = (v[2] - v[1]) / h1;
    double r0 = 2 * s0, r2 = 2 * s1, r1 = 3 * (s0 / h0 + s1 / h1);
    d[1] = (r1 - r0 / h0 - r2 / h1) / (1 / h0 + 1 / h1);
    d[0] = r0 - d[1];
    d[2] = r2 - d[1];
}

// Bicubic Hermite evaluation on the 3 (x) by 2 (y) node grid; F[j][i] at
// (x[i], y[j]); x and y ascending.  Node slopes: 3-node spline along x,
// straight line along y (a 2-node spline with parabolic ends is a line).
double bicubic32(const double x[3], const double y[2], const double F[2][3], double qx, double qy)
{
    double Fx[2][3], Fy[2][3], Fxy[2][3];
    for (int j = 0; j < 2; j++) slopes3(x, F[j], Fx[j]);
    for (int i = 0; i < 3; i++)
    {
        double sy = (F[1][i] - F[0][i]) / (y[1] - y[0]);
        Fy[0][i] = Fy[1][i] = sy;
        double sxy = (Fx[1][i] - Fx[0][i]) / (y[1] - y[0]);
        Fxy[0][i] = Fxy[1][i] = sxy;
    }
    // cell search clamped to the first/last interval (points outside extrapolate)
    int ix = (qx <= x[1]) ? 0 : 1;
    double hx = x[ix + 1] - x[ix], hy = y[1] - y[0];
    double t = (qx - x[ix]) / hx, u = (qy - y[0]) / hy;
    auto h00 = [](double s) { return 2 * s * s * s - 3 * s * s + 1; };
    auto h01 = [](double s) { return -2 * s * s * s + 3 * s * s; };
    auto g00 = [](double s) { return s * s * s - 2 * s * s + s; };
    auto g01 = [](double s) { return s * s * s - s * s; };
    double Hx[2] = {h00(t), h01(t)}, Gx[2] = {g00(t) * hx, g01(t) * hx};
    double Hy[2] = {h00(u), h01(u)}, Gy[2] = {g00(u) * hy, g01(u) * hy};
    double v = 0;
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
        {
            int i = ix + a;
            v += Hx[a] * Hy[b] * F[b][i] + Gx[a] * Hy[b] * Fx[b][i] + Hx[a] * Gy[b] * Fy[b][i] +
                 Gx[a] * Gy[b] * Fxy[b][i];
        }
    return v;
}

int tiles_of(int W) { return (W + 31) / 32; }
} // namespace

void spline_weights(const double xin[3], const double yin[2], double qx, double qy, double w[6])
{
    // sort nodes ascending, remembering where each input node went
    int px[3] = {0, 1, 2}, py[2] = {0, 1};
    std::sort(px, px + 3, [&](int a, int b) { return xin[a] < xin[b]; });
    if (yin[1] < yin[0]) std::swap(py[0], py[1]);
    double x[3] = {xin[px[0]], xin[px[1]], xin[px[2]]}, y[2] = {yin[py[0]], yin[py[1]]};
    for (int k = 0; k < 6; k++)
    {
        double F[2][3] = {{0, 0, 0}, {0, 0, 0}};
        int i = k % 3, j = k / 3; // input node (x index i, y index j) carries the unit value
        int si = (int)(std::find(px, px + 3, i) - px), sj = (py[0] == j) ? 0 : 1;
        F[sj][si] = 1.0;
        w[k] = bicubic32(x, y, F, qx, qy);
    }
}

ImageLayout build_layout(const Grid &g, const LayoutParams &p)
{
    using namespace d2q9;
    ImageLayout L;
    L.n = g.n;
    L.max_level = g.max_level;
    const int ML = g.max_level;
    L.levels.resize(ML);
    for (int l = 1; l <= ML; l++)
    {
        LevelLayout &lv = L.levels[l - 1];
        lv.level = l;
        lv.W = lv.H = g.n >> (l - 1);
        lv.pitch = ((lv.W + 31) / 32) * 32;
        lv.plane = (int64_t)lv.pitch * lv.H;
        lv.omega.assign((size_t)lv.plane, 0.0f);
        if (p.adsorption || p.collision == COLL_MRT) lv.tau_d.assign((size_t)lv.plane, 0.0f);
        lv.spec.assign((size_t)lv.plane, 0u);
        lv.substeps = 1 << (ML - l);
        lv.snapshot_all = g.multiblock;
        lv.tiles_x = tiles_of(lv.W);
        lv.tiles_y = (lv.H + 7) / 8;
    }
    const int64_t N = g.n_cells;
    L.cell_level.resize(N);
    L.cell_site.resize(N);
    for (int64_t c = 0; c < N; c++)
    {
        int l = g.level[c];
        const LevelLayout &lv = L.levels[l - 1];
        int sx = g.x[c] >> (l - 1), sy = g.y[c] >> (l - 1);
        L.cell_level[c] = l;
        L.cell_site[c] = sy * lv.pitch + sx;
    }
    auto torus_site = [&](int64_t c, int q) {
        int l = g.level[c];
        const LevelLayout &lv = L.levels[l - 1];
        int sx = (g.x[c] >> (l - 1)) + CX[q], sy = (g.y[c] >> (l - 1)) + CY[q];
        sx = (sx + lv.W) % lv.W;
        sy = (sy + lv.H) % lv.H;
        return sy * lv.pitch + sx;
    };

    // masks from the reference link lists
    std::vector<uint32_t> arrive(N, 0), over(N, 0), wall(N, 0), quirk(N, 0), out(N, 0);
    for (size_t k = 0; k < g.stream_id.size(); k++)
    {
        int64_t src = g.stream_id[k], dst = g.stream_loc[k];
        int q = g.stream_ic[k];
        if (torus_site(src, q) != L.cell_site[dst] || g.level[src] != g.level[dst])
            throw std::runtime_error("layout: stream link does not land on its torus neighbour");
        arrive[dst] |= 1u << q;
        out[src] |= 1u << q;
    }
    for (size_t k = 0; k < g.per_id.size(); k++)
    {
        int64_t src = g.per_id[k], dst = g.per_i2[k];
        int q = g.per_ic[k];
        if (torus_site(src, q) != L.cell_site[dst] || g.level[src] != g.level[dst])
            throw std::runtime_error("layout: periodic link does not land on its torus neighbour");
        arrive[dst] |= 1u << q;
        over[dst] |= 1u << q;
        out[src] |= 1u << q;
    }
    for (size_t k = 0; k < g.wall_id.size(); k++)
    {
        int64_t c = g.wall_id[k];
        int q = g.wall_ic[k];
        wall[c] |= 1u << q;
        if (g.conn[(size_t)c * 9 + q] >= 0) quirk[c] |= 1u << q;
    }

    // interpolation buffer targets
    std::vector<int32_t> buf_of(N, -1);
    auto want_buf = [&](int64_t c) {
        if (c < 0) return;
        if (buf_of[c] < 0)
        {
            buf_of[c] = (int32_t)L.n_buffers++;
            L.buf_level.push_back(g.level[c]);
            L.buf_site.push_back(L.cell_site[c]);
        }
    };
    for (auto &row : g.coarse_rows)
        if (row[0] >= 0 && g.is_buffer[row[0]]) want_buf(row[0]);
    for (auto &row : g.fine_rows)
        for (int k = 1; k < 5; k++)
            if (row[k] >= 0 && g.is_buffer[row[k]]) want_buf(row[k]);

    const uint32_t ALL = 0x1FFu;
    std::vector<int> spec_level;
    std::vector<char> plain_buffer(N, 0);
    for (int64_t c = 0; c < N; c++)
    {
        int l = g.level[c];
        LevelLayout &lv = L.levels[l - 1];
        int s = L.cell_site[c];
        if (lv.omega[(size_t)s] != 0.0f) throw std::runtime_error("layout: two cells share a site");
        if (!(g.tau[c] > 0.0)) throw std::runtime_error("layout: non-positive relaxation time");
        const float omega = (float)(1.0 / g.tau[c]);
        uint32_t flags = 0;
        if (p.adsorption && c == g.inlet && g.outlet >= 0) flags |= SF_INLET;
        if (p.adsorption && c == g.outlet && g.inlet >= 0) flags |= SF_OUTLET;
        bool special = arrive[c] != ALL || wall[c] != 0 || flags != 0 || (p.adsorption && out[c] != ALL);
        // an interpolation target that streams like a plain cell stays plain:
        // the interface exchange writes its values into the slots it reads next
        if (buf_of[c] >= 0)
        {
            if (special) flags |= SF_BUFFER;
            else plain_buffer[c] = 1;
        }
        if (p.adsorption || p.collision == COLL_MRT)
        {
            // include/coreLB.hpp:710 (tau_d of the plain MRT from the cell's Kn)
            double a = p.mfp_over_cl * 1.0 / (1.0 + 2.0 * g.kn[c]);
            lv.tau_d[(size_t)s] = (float)(0.5 + (3.0 / 2.0) * std::sqrt(3.0) * 1.0 / std::pow((1.0 / std::sqrt(a)) * 2.0, 2.0));
        }
        lv.n_active++;
        if (!g.is_buffer[c]) lv.n_active_real++;
        if (!special)
        {
            lv.omega[(size_t)s] = omega;
            continue;
        }
        SpecialRec rec{};
        int b = g.bnd[c];
        rec.m0 = arrive[c] | (over[c] << 9) | (wall[c] << 18);
        rec.m1 = quirk[c] | ((uint32_t)(b < 0 ? 0xFF : b) << 9) | (flags << 17) | (out[c] << 21);
        double kn = g.kn[c];
        double r = 0.0;
        if (wall[c])
        {
            if (b < 0) r = 1.0; // wall link of a cell with no boundary type: full bounce-back
            else if (p.wall == WALL_SRBB) r = 0.4987 * std::pow(kn, -0.131) - 0.25;
            else if (p.wall == WALL_MDBB) r = 0.3222 * std::pow(kn, -0.217) - 0.25;
        }
        rec.r = (float)r;
        rec.quirk_base = -1;
        if (quirk[c])
        {
            rec.quirk_base = (int32_t)L.n_quirk;
            L.n_quirk += __builtin_popcount(quirk[c]);
        }
        rec.buf = buf_of[c];
        // constant part of each population's deviation: rho0 * K_p
        double K[9] = {0};
        for (int q = 0; q < 9; q++)
            if (!((arrive[c] >> q) & 1)) K[q] -= W[q];
        if (p.wall == WALL_SRBB)
        {
            for (int q = 0; q < 9; q++)
            {
                if (!((wall[c] >> q) & 1)) continue;
                int p1 = OPP[q];
                int p2 = (b >= 0) ? MANTIIS_ICSR[b][q] : OPP[q];
                if (!((over[c] >> p1) & 1)) K[p1] += r * W[q];
                if (!((over[c] >> p2) & 1)) K[p2] += (1 - r) * W[q];
            }
        }
        else
        {
            // BB / MDBB assign the reflected population outright
            for (int q = 0; q < 9; q++)
                if (((wall[c] >> q) & 1) && !((over[c] >> OPP[q]) & 1)) K[OPP[q]] = 0.0;
        }
        bool hasK = false;
        for (int q = 0; q < 9; q++)
            if (std::fabs(K[q]) > 1e-15) hasK = true;
        rec.k_row = -1;
        if (hasK)
        {
            rec.k_row = (int32_t)(L.ktab.size() / 9);
            for (int q = 0; q < 9; q++) L.ktab.push_back((float)(p.rho0 * K[q]));
            rec.m1 |= (uint32_t)SF_HAS_K << 17;
        }
        rec.xy = (int32_t)((s % lv.pitch) | ((s / lv.pitch) << 16));
        rec.omega = omega;
        lv.omega[(size_t)s] = -omega;
        L.specials.push_back(rec);
        spec_level.push_back(l);
    }
    // special records grouped by level, heavy before light, then by whether they
    // have wall links, then ordered by 8x4 block of sites (row-major blocks,
    // row-major inside a block), so a warp of the special-cell kernel takes one
    // path over a compact patch
    {
        std::vector<int64_t> order(L.specials.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = (int64_t)i;
        std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
            if (spec_level[a] != spec_level[b]) return spec_level[a] < spec_level[b];
            // heavy records first, light ones last (the 8x4 plain kernel can take
            // those); cells with wall links apart from the others, so the warps of
            // the special-cell kernel take one path
            const bool la = special_is_light(L.specials[a]), lb = special_is_light(L.specials[b]);
            if (la != lb) return la < lb;
            const bool wa = ((L.specials[a].m0 >> 18) & 0x1FFu) != 0, wb = ((L.specials[b].m0 >> 18) & 0x1FFu) != 0;
            if (wa != wb) return wa < wb;
            return special_order_key(L.specials[a].xy) < special_order_key(L.specials[b].xy);
        });
        std::vector<SpecialRec> sorted(order.size());
        for (size_t i = 0; i < order.size(); i++) sorted[i] = L.specials[order[i]];
        L.specials.swap(sorted);
        for (auto &lv : L.levels) lv.spec_count = lv.spec_heavy = 0;
        for (size_t i = 0; i < L.specials.size(); i++)
        {
            int l = spec_level[order[i]];
            LevelLayout &lv = L.levels[l - 1];
            if (lv.spec_count == 0) lv.spec_begin = (int64_t)i;
            lv.spec_count++;
            if (!special_is_light(L.specials[i])) lv.spec_heavy++;
            const int32_t xy = L.specials[i].xy;
            lv.spec[(size_t)(xy >> 16) * lv.pitch + (xy & 0xFFFF)] = (uint32_t)i;
        }
    }

    // active tiles (32 x 8 sites): the x-interior ones first, then the two
    // border columns
    for (auto &lv : L.levels)
    {
        std::vector<std::pair<int, int>> order;
        for (int pass = 0; pass < 2; pass++)
            for (int ty = 0; ty < lv.tiles_y; ty++)
                for (int tx = 0; tx < lv.tiles_x; tx++)
                {
                    const bool interior = tx > 0 && tx + 1 < lv.tiles_x;
                    if (interior == (pass == 0)) order.push_back({tx, ty});
                }
        for (const auto &tt : order)
        {
            const int tx = tt.first, ty = tt.second;
            bool any = false;
            for (int yy = ty * 8; yy < std::min(lv.H, ty * 8 + 8) && !any; yy++)
                for (int xx = tx * 32; xx < std::min(lv.W, tx * 32 + 32); xx++)
                    if (lv.omega[(size_t)yy * lv.pitch + xx] != 0.0f)
                    {
                        any = true;
                        break;
                    }
            if (!any) continue;
            if (tx > 0 && tx + 1 < lv.tiles_x) lv.n_tiles_interior++;
            lv.tile_list.push_back(tx | ty << 16);
            for (int r = 0; r < 8; r++)
            {
                uint32_t m = 0;
                int yy = ty * 8 + r;
                for (int k = 0; k < 32 && yy < lv.H; k++)
                {
                    int xx = tx * 32 + k;
                    if (xx < lv.W && lv.omega[(size_t)yy * lv.pitch + xx] > 0.0f) m |= 1u << k;
                }
                lv.tile_mask.push_back(m);
            }
        }
    }

    // 8x4 tiles holding a plain or light cell, row-major (one warp per tile in the
    // 8x4 kernel: sparse levels fill them better than 32x8 tiles), with the mask
    // of their light cells
    for (auto &lv : L.levels)
    {
        const int t8x = (lv.W + 7) / 8, t8y = (lv.H + 3) / 4;
        for (int ty = 0; ty < t8y; ty++)
            for (int tx = 0; tx < t8x; tx++)
            {
                uint32_t m = 0, light = 0;
                for (int r = 0; r < 4; r++)
                {
                    const int yy = ty * 4 + r;
                    if (yy >= lv.H) break;
                    for (int k = 0; k < 8; k++)
                    {
                        const int xx = tx * 8 + k;
                        if (xx >= lv.W) break;
                        const size_t site = (size_t)yy * lv.pitch + xx;
                        const float om = lv.omega[site];
                        if (om > 0.0f) m |= 1u << (8 * r + k);
                        else if (om < 0.0f && special_is_light(L.specials[lv.spec[site]]))
                        {
                            m |= 1u << (8 * r + k);
                            light |= 1u << (8 * r + k);
                        }
                    }
                }
                if (!m) continue;
                lv.tile8_list.push_back(tx | ty << 16);
                lv.tile8_mask.push_back(m);
                lv.tile8_light.push_back(light);
            }
    }

    // interfaces (include/coreLB.hpp:1101-1231)
    auto is_coarse_buffer = [&](int64_t c) { return g.is_buffer[c] && g.type[c] == 10 * g.level[c] + g.level[c] - 1; };
    for (int l1 = 1; l1 < ML; l1++)
    {
        int l2 = l1 + 1;
        InterfaceLayout itf;
        itf.l1 = l1;
        itf.l2 = l2;
        int ckey = 10 * l2 + l1, fkey = 10 * l1 + l2;
        for (size_t r = 0; r < g.coarse_rows.size(); r++)
        {
            if (g.coarse_key[r] != ckey) continue;
            const auto &row = g.coarse_rows[r];
            if (row[0] < 0 || buf_of[row[0]] < 0) continue;
            // with three levels the reference also files some rows of the pair
            // (l2, l2 + 1) under this key (target one level up); the same target
            // has its row under the right key, which is processed later and sets
            // the final value, so the stray copy is left out
            bool same_levels = g.level[row[0]] == l2;
            for (int k = 1; k < 5; k++)
                if (row[k] >= 0 && g.level[row[k]] != l1) same_levels = false;
            if (!same_levels) continue;
            CoarseRowDev d{};
            d.site = L.cell_site[row[0]];
            d.buf = buf_of[row[0]];
            double tsum = 0;
            int cnt = 0;
            for (int k = 0; k < 4; k++)
            {
                int64_t ch = row[k + 1];
                d.child[k] = ch >= 0 ? L.cell_site[ch] : -1;
                d.child_buf[k] = (ch >= 0 && is_coarse_buffer(ch) && g.level[ch] <= l2) ? buf_of[ch] : -1;
                if (ch >= 0)
                {
                    tsum += g.tau[ch];
                    cnt++;
                }
            }
            if (cnt == 0) continue;
            d.ratio = (float)(2 * g.tau[row[0]] / (tsum / cnt));
            d.inv_nchild = 1.0f / cnt;
            d.plain_target = plain_buffer[row[0]];
            itf.coarse.push_back(d);
        }
        const int top_order[9] = {7, 4, 8, 3, 0, 1, 6, 2, 5};
        const int bottom_order[9] = {6, 2, 5, 3, 0, 1, 7, 4, 8};
        double parent_shift = std::pow(2.0, l2 - 2) - 0.5;
        double child_shift = (l1 == 1) ? 0 : std::pow(2.0, l1 - 2) - 0.5;
        for (size_t r = 0; r < g.fine_rows.size(); r++)
        {
            if (g.fine_key[r] != fkey) continue;
            const auto &row = g.fine_rows[r];
            int64_t pc = row[0];
            int lvp = g.level[pc];
            int thr = 1 << (lvp - 1);
            double X[9], Y[9];
            int64_t nb_cell[9];
            for (int q = 0; q < 9; q++)
            {
                int64_t nb = g.conn[(size_t)pc * 9 + q];
                nb_cell[q] = nb;
                // neighbour position on the parent's level (periodic), which is
                // also where a wall / missing neighbour is taken to sit (it then
                // carries the parent's populations)
                int ny = ((g.y[pc] + CY[q] * thr) % g.n + g.n) % g.n;
                int nx = ((g.x[pc] + CX[q] * thr) % g.n + g.n) % g.n;
                if (nb >= 0 && (g.y[nb] != ny || g.x[nb] != nx))
                    throw std::runtime_error("layout: neighbour off its lattice position");
                int dy = g.y[pc] - ny, dxv = g.x[pc] - nx;
                if (std::abs(dy) > thr && dy < 0) X[q] = g.y[pc] + parent_shift + 1 - 2;
                else if (std::abs(dy) > thr && dy > 0) X[q] = g.y[pc] + parent_shift + 1 + 2;
                else X[q] = ny + parent_shift + 1;
                if (std::abs(dxv) > thr && dxv < 0) Y[q] = g.x[pc] + parent_shift + 1 - 2;
                else if (std::abs(dxv) > thr && dxv > 0) Y[q] = g.x[pc] + parent_shift + 1 + 2;
                else Y[q] = nx + parent_shift + 1;
            }
            std::vector<double> xs(X, X + 9), ys(Y, Y + 9);
            std::sort(xs.begin(), xs.end());
            xs.erase(std::unique(xs.begin(), xs.end()), xs.end());
            std::sort(ys.begin(), ys.end());
            ys.erase(std::unique(ys.begin(), ys.end()), ys.end());
            if (xs.size() != 3 || ys.size() != 3) throw std::runtime_error("layout: spline nodes are not a 3x3 lattice");
            bool top = g.y[pc] < g.n / 2;
            double ynode[2] = {top ? xs[0] : xs[2], xs[1]};
            double xnode[3] = {ys[0], ys[1], ys[2]};
            const int *order = top ? top_order : bottom_order;
            FineRowDev d{};
            for (int k = 0; k < 6; k++)
            {
                int64_t nb = nb_cell[order[k]];
                int64_t src = nb >= 0 ? nb : pc;
                d.node_site[k] = L.cell_site[src];
                d.node_buf[k] = (is_coarse_buffer(src) && g.level[src] <= l2) ? buf_of[src] : -1;
            }
            for (int k = 0; k < 4; k++)
            {
                int64_t ch = row[k + 1];
                d.child_site[k] = L.cell_site[ch];
                d.child_buf[k] = buf_of[ch];
                if (plain_buffer[ch]) d.plain_mask |= 1 << k;
                double w[6];
                spline_weights(xnode, ynode, g.x[ch] + child_shift + 1, g.y[ch] + child_shift + 1, w);
                double sum = 0;
                for (int j = 0; j < 6; j++)
                {
                    d.weight[k][j] = (float)w[j];
                    sum += w[j];
                }
                if (std::fabs(sum - 1.0) > 1e-9) throw std::runtime_error("layout: spline weights do not sum to one");
                d.ratio[k] = (float)(g.tau[ch] / (2 * g.tau[pc]));
            }
            itf.fine.push_back(d);
        }
        L.interfaces.push_back(std::move(itf));
    }

    // statistics: mean tau, pixel area, lattice updates per coarse step
    double ts = 0;
    int64_t nt = 0;
    for (int64_t c = 0; c < N; c++)
    {
        int l = g.level[c];
        double lu = (double)(1 << (ML - l));
        if (g.is_buffer[c])
        {
            L.buffer_lu_per_coarse_step += lu;
            continue;
        }
        ts += g.tau[c];
        nt++;
        L.pixel_area_cells += (int64_t)1 << (2 * (l - 1));
        L.lu_per_coarse_step += lu;
    }
    L.tau_mean = nt ? ts / nt : 0.0;
    return L;
}
} // namespace mantiis
