#include "grid.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <unordered_map>

#include "../boundary_tables.h"
#include "../d2q9.h"

namespace mantiis
{
namespace
{
constexpr int kDirOrder[9] = {7, 3, 6, 4, 0, 2, 8, 1, 5}; // include/grid.hpp:1113

struct Builder
{
    const PoreImage &img;
    GridOptions opt;
    int n;
    Grid g;

    // quadtree output: raster image of signed leaf numbers and leaf side per number
    std::vector<int64_t> leafimg;
    std::vector<int32_t> leafside; // index = |leaf number|
    int64_t leafcount = 1;

    std::vector<int64_t> solid_prefix; // summed-area table of solid pixels
    std::vector<double> dwall;

    explicit Builder(const PoreImage &im, const GridOptions &o) : img(im), opt(o), n(im.n) {}

    int64_t lin_of(int col, int row, int lvl) const { return (int64_t)col + (int64_t)row * n + (int64_t)(lvl - 1) * n * n; }

    int64_t solids_in(int r0, int c0, int h) const
    {
        auto S = [&](int r, int c) { return solid_prefix[(size_t)r * (n + 1) + c]; };
        return S(r0 + h, c0 + h) - S(r0, c0 + h) - S(r0 + h, c0) + S(r0, c0);
    }

    // include/grid.hpp:1160-1238 (decision) and :1241-1266 (numbering)
    void decompose(int r0, int c0, int size, int min_dist)
    {
        const double alpha = 0.99;
        int h = size / 2;
        const int quad[4][2] = {{r0, c0}, {r0, c0 + h}, {r0 + h, c0}, {r0 + h, c0 + h}};
        for (auto &qd : quad)
        {
            int qr = qd[0], qc = qd[1];
            bool divide = false;
            double beta = (double)solids_in(qr, qc, h) / (double)((int64_t)h * h);
            if (h > 1)
            {
                double mn = std::numeric_limits<double>::max();
                for (int r = qr; r < qr + h; r++)
                    for (int c = qc; c < qc + h; c++) mn = std::min(mn, dwall[(size_t)r * n + c]);
                if (mn < (double)((size_t)min_dist * (size_t)h)) divide = true;
            }
            if (std::log2((double)h) + 1 > opt.max_allowed_level) divide = true;
            if (opt.edge_fine && h > 1 && (qc == 0 || qc + h == n)) divide = true;
            if (((1.0 - alpha) < beta && beta < alpha) || divide)
            {
                decompose(qr, qc, h, min_dist);
                continue;
            }
            int64_t v = beta > alpha ? -leafcount : leafcount;
            for (int r = qr; r < qr + h; r++)
                for (int c = qc; c < qc + h; c++) leafimg[(size_t)r * n + c] = v;
            leafside.push_back(h);
            leafcount++;
        }
    }

    void build_cells();
    void build_connections();
    void build_parent_child_and_buffers();
    void build_boundary_types();
    void build_links();
    void build_taus();
};

void Builder::build_cells()
{
    const size_t nn = (size_t)n * n;
    std::vector<int64_t> value(nn);
    std::vector<int32_t> side_of_value; // by leaf number
    if (!opt.multiblock)
    {
        // include/grid.hpp:401-424: every pixel its own cell
        for (size_t k = 0; k < nn; k++) value[k] = img.pore[k] == 0 ? -(int64_t)(k + 1) : (int64_t)(k + 1);
    }
    else
    {
        if (n < 2 || (n & (n - 1))) throw std::invalid_argument("Matrix dimensions must be divisible by 2 in each direction.");
        // pore image as +-1 and its wall distance (include/grid.hpp:313-399)
        std::vector<uint8_t> vmask(nn);
        solid_prefix.assign((size_t)(n + 1) * (n + 1), 0);
        for (int r = 0; r < n; r++)
            for (int c = 0; c < n; c++)
            {
                int solid = img.pore[(size_t)r * n + c] == 0;
                vmask[(size_t)r * n + c] = !solid;
                solid_prefix[(size_t)(r + 1) * (n + 1) + (c + 1)] = solid_prefix[(size_t)r * (n + 1) + (c + 1)] +
                                                                     solid_prefix[(size_t)(r + 1) * (n + 1) + c] -
                                                                     solid_prefix[(size_t)r * (n + 1) + c] + solid;
            }
        std::vector<float> dw = distance_to_zero(vmask, n, n);
        dwall.assign(dw.begin(), dw.end());
        leafimg.assign(nn, 0);
        leafside.assign(1, 0);
        int min_dist = (int)std::ceil(std::pow(2, opt.max_allowed_level - 1) * std::sqrt(2));
        decompose(0, 0, n, min_dist);
        value = leafimg;
    }
    g.reconstructed = value;

    // include/grid.hpp:427-558: cells in raster order of first occurrence
    auto side_of = [&](int64_t v) -> int {
        if (!opt.multiblock) return 1;
        return leafside[(size_t)(v < 0 ? -v : v)];
    };
    int max_level = 1;
    for (size_t k = 0; k < nn; k++)
    {
        int s = side_of(value[k]);
        int lvl = (int)(std::log2(std::sqrt((double)s * s)) + 1);
        max_level = std::max(max_level, lvl);
    }
    g.max_level = max_level;
    g.n = n;
    g.multiblock = opt.multiblock;

    struct Orig
    {
        int32_t col, row, lvl;
        bool pore;
    };
    std::vector<Orig> orig;
    std::vector<uint8_t> seen(opt.multiblock ? (size_t)leafcount + 1 : 0, 0);
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++)
        {
            int64_t v = value[(size_t)r * n + c];
            if (opt.multiblock)
            {
                size_t a = (size_t)(v < 0 ? -v : v);
                if (seen[a]) continue;
                seen[a] = 1;
            }
            int s = side_of(v);
            int lvl = (int)(std::log2(std::sqrt((double)s * s)) + 1);
            orig.push_back({c, r, lvl, v > 0});
        }

    // lookup over the (level, row, col) index space
    const size_t space = nn * (size_t)max_level;
    std::vector<int32_t> orig_at(space, -1);       // original cell id at an exact (lvl,row,col)
    std::vector<int32_t> orig_topleft(nn, -1);     // original cell whose top-left pixel this is
    for (size_t k = 0; k < orig.size(); k++)
    {
        orig_at[(size_t)lin_of(orig[k].col, orig[k].row, orig[k].lvl)] = (int32_t)k;
        orig_topleft[(size_t)orig[k].row * n + orig[k].col] = (int32_t)k;
    }
    std::vector<uint8_t> exists(space, 0);
    for (auto &o : orig) exists[(size_t)lin_of(o.col, o.row, o.lvl)] = 1;

    // include/grid.hpp:560-795: buffer cells
    struct Buf
    {
        int64_t lin;
        int32_t type;
    };
    std::vector<Buf> bufs;
    const int base_range = 1 << (max_level - 1);
    auto decode = [&](int64_t id, int &col, int &row, int &lvlidx) {
        // utils::ind2sub with sizes {n, n, max_level}, C++ truncating division
        col = (int)(id % n);
        id /= n;
        row = (int)(id % n);
        id /= n;
        lvlidx = (int)(id % max_level);
    };
    for (size_t i = 0; i < orig.size(); i++)
    {
        const Orig &ci = orig[i];
        if (ci.lvl <= 1) continue;
        const int jump = 1 << (ci.lvl - 1);
        const int kmax = base_range / jump;
        // missing same-level positions, x-major then y (include/grid.hpp:577-611)
        std::vector<int64_t> missing;
        for (int kx = -kmax; kx <= kmax; kx++)
            for (int ky = -kmax; ky <= kmax; ky++)
            {
                int cc = ci.col + kx * jump, rr = ci.row + ky * jump;
                if (cc < 0 || rr < 0 || cc >= n || rr >= n) continue;
                int64_t id = lin_of(cc, rr, ci.lvl);
                if (!exists[(size_t)id] || orig_at[(size_t)id] < 0) missing.push_back(id);
            }
        if (missing.empty()) continue;
        const float shift = (float)(std::pow(2, ci.lvl - 2) - 0.5);
        // original cells with top-left in the window, in cell order (= raster order)
        std::vector<int32_t> win;
        int max_level_in = 0;
        for (int rr = std::max(0, ci.row - base_range); rr <= std::min(n - 1, ci.row + base_range); rr++)
            for (int cc = std::max(0, ci.col - base_range); cc <= std::min(n - 1, ci.col + base_range); cc++)
            {
                int32_t k = orig_topleft[(size_t)rr * n + cc];
                if (k < 0) continue;
                win.push_back(k);
                max_level_in = std::max(max_level_in, (int)orig[k].lvl);
            }
        for (int32_t k : win)
        {
            const Orig &cw = orig[k];
            if (cw.lvl == ci.lvl)
            {
                // break the coarse cell into 4 finer buffer cells (TL, TR, BL, BR)
                int half = 1 << (ci.lvl - 2);
                const int kids[4][2] = {{ci.col, ci.row}, {ci.col + half, ci.row}, {ci.col, ci.row + half},
                                        {ci.col + half, ci.row + half}};
                for (auto &kd : kids)
                {
                    int64_t id = lin_of(kd[0], kd[1], ci.lvl - 1);
                    if (exists[(size_t)id]) continue;
                    exists[(size_t)id] = 1;
                    bufs.push_back({id, 10 * (ci.lvl - 1) + ci.lvl});
                }
            }
            else if (max_level_in <= ci.lvl)
            {
                // upscale: the missing position nearest to this finer cell
                float ngx = (float)cw.col + shift, ngy = (float)cw.row + shift;
                int best = 0;
                double bestd = std::numeric_limits<double>::max();
                for (size_t m = 0; m < missing.size(); m++)
                {
                    int mc, mr, ml;
                    decode(missing[m], mc, mr, ml);
                    float sx = (float)mc + shift, sy = (float)mr + shift;
                    double d = std::sqrt(std::pow(ngx - sx, 2) + std::pow(ngy - sy, 2));
                    if (d < bestd)
                    {
                        bestd = d;
                        best = (int)m;
                    }
                }
                int64_t id = missing[(size_t)best];
                if (id != -1 && !exists[(size_t)id])
                {
                    exists[(size_t)id] = 1;
                    bufs.push_back({id, 10 * ci.lvl + ci.lvl - 1});
                    missing[(size_t)best] = -1;
                }
            }
        }
    }

    // include/grid.hpp:800-889: pore cells, then buffer cells
    for (auto &o : orig)
    {
        if (o.pore)
        {
            g.lin.push_back(lin_of(o.col, o.row, o.lvl));
            g.x.push_back(o.col);
            g.y.push_back(o.row);
            g.level.push_back(o.lvl);
            g.type.push_back(0);
            g.is_buffer.push_back(0);
        }
    }
    for (auto &b : bufs)
    {
        int c, r, l;
        decode(b.lin, c, r, l);
        g.lin.push_back(b.lin);
        g.x.push_back(c);
        g.y.push_back(r);
        g.level.push_back(l + 1);
        g.type.push_back(b.type);
        g.is_buffer.push_back(1);
    }
    g.n_cells = (int64_t)g.lin.size();
    for (size_t k = 0; k < nn; k++)
        if (img.pore[k] == 0) g.solid_pixels.push_back((int64_t)k);

    // properties from the input fields at the top-left pixel (include/grid.hpp:891-898)
    g.kn.resize(g.n_cells);
    g.locpore.resize(g.n_cells);
    for (int64_t c = 0; c < g.n_cells; c++)
    {
        size_t p = (size_t)g.y[c] * n + g.x[c];
        g.kn[c] = img.kn[p];
        g.locpore[c] = img.locpore[p];
    }

    // neighbour table (include/grid.hpp:916-972)
    std::vector<int64_t> cell_at(space, -1);
    for (int64_t c = 0; c < g.n_cells; c++) cell_at[(size_t)g.lin[c]] = c;
    g.conn.assign((size_t)g.n_cells * 9, -2);
    for (int64_t c = 0; c < g.n_cells; c++)
    {
        int jump = 1 << (g.level[c] - 1);
        for (int q = 0; q < 9; q++)
        {
            int ip = g.x[c] + d2q9::CX[q] * jump, jp = g.y[c] + d2q9::CY[q] * jump;
            if (jp <= -1) jp += n;
            if (jp >= n) jp -= n;
            if (ip <= -1) ip += n;
            if (ip >= n) ip -= n;
            int64_t ng = lin_of(ip, jp, g.level[c]);
            int64_t v;
            if (cell_at[(size_t)ng] >= 0) v = cell_at[(size_t)ng];
            else if (orig_at[(size_t)ng] >= 0) v = -1;
            else v = -2;
            g.conn[(size_t)c * 9 + q] = v;
        }
    }

    // parent-child rows for every coarse cell (include/grid.hpp:974-1038)
    for (int64_t c = 0; c < g.n_cells; c++)
    {
        if (g.level[c] <= 1) continue;
        int half = (1 << (g.level[c] - 1)) / 2;
        std::array<int64_t, 5> row;
        row[0] = c;
        const int kids[4][2] = {{0, 0}, {half, 0}, {0, half}, {half, half}};
        for (int k = 0; k < 4; k++)
        {
            int64_t id = lin_of(g.x[c] + kids[k][0], g.y[c] + kids[k][1], g.level[c] - 1);
            row[k + 1] = cell_at[(size_t)id];
        }
        g.parent_child.push_back(row);
    }

    // interface tables (include/grid.hpp:1041-1108)
    if (opt.multiblock)
    {
        // first (row, column) occurrence of each id in the parent-child table
        std::unordered_map<int64_t, int64_t> first_row;
        std::unordered_map<int64_t, int64_t> first_row_as_child;
        for (size_t r = 0; r < g.parent_child.size(); r++)
            for (int k = 0; k < 5; k++)
            {
                first_row.emplace(g.parent_child[r][k], (int64_t)r);
                if (k > 0) first_row_as_child.emplace(g.parent_child[r][k], (int64_t)r);
            }
        for (int lvl = max_level; lvl >= 2; lvl--)
        {
            int key = 10 * lvl + lvl - 1;
            for (int64_t c = 0; c < g.n_cells; c++)
                if (g.type[c] == key)
                {
                    auto it = first_row.find(c);
                    std::array<int64_t, 5> row = g.parent_child[(size_t)it->second];
                    for (int k = 1; k < 5; k++)
                        if (row[k] < 0) g.diag.coarse_missing_child++;
                    g.coarse_key.push_back(key);
                    g.coarse_rows.push_back(row);
                }
        }
        for (int lvl = 1; lvl < max_level; lvl++)
        {
            int key = 10 * lvl + lvl + 1;
            std::vector<int64_t> ids;
            for (int64_t c = 0; c < g.n_cells; c++)
                if (g.type[c] == key) ids.push_back(c);
            if (ids.size() % 4) g.diag.fine_group_unmatched++;
            for (size_t s = 0; s + 4 <= ids.size(); s += 4)
            {
                // parent = owner of the earliest parent-child row holding any of the four
                int64_t best = -1;
                for (int k = 0; k < 4; k++)
                {
                    auto it = first_row_as_child.find(ids[s + k]);
                    if (it != first_row_as_child.end() && (best < 0 || it->second < best)) best = it->second;
                }
                if (best < 0)
                {
                    g.diag.fine_group_unmatched++;
                    continue;
                }
                std::array<int64_t, 5> row{g.parent_child[(size_t)best][0], ids[s], ids[s + 1], ids[s + 2], ids[s + 3]};
                for (int q = 0; q < 9; q++)
                    if (g.conn[(size_t)row[0] * 9 + q] < 0)
                    {
                        g.diag.fine_parent_missing_nbr++;
                        break;
                    }
                g.fine_key.push_back(key);
                g.fine_rows.push_back(row);
            }
        }
    }
}

void Builder::build_boundary_types()
{
    g.bnd.assign(g.n_cells, -1);
    for (int64_t c = 0; c < g.n_cells; c++)
        if (g.is_buffer[c] == 0) g.bnd[c] = boundary_type_of(&g.conn[(size_t)c * 9]);
}

void Builder::build_links()
{
    // include/coreLB.hpp:293-366 (one rank: every neighbour is local)
    const int thr = 1 << (g.max_level - 1);
    int ny_c = (n % 2 == 1) ? (n + 1) / 2 - 1 : n / 2 - 1;
    for (int64_t i = 0; i < g.n_cells; i++)
    {
        int b = g.bnd[i];
        for (int q = 0; q < 9; q++)
        {
            int64_t nb = g.conn[(size_t)i * 9 + q];
            auto streams = [&]() {
                if (b == -1) return true;
                return MANTIIS_IFSTREAM[b][q] != 0;
            };
            if (nb >= 0)
            {
                bool xp = std::abs(g.x[i] - g.x[nb]) > thr;
                bool yp = std::abs(g.y[i] - g.y[nb]) > thr;
                if (!xp && !yp)
                {
                    if (streams())
                    {
                        g.stream_id.push_back(i);
                        g.stream_ic.push_back(q);
                        g.stream_loc.push_back(nb);
                    }
                    else
                    {
                        g.wall_id.push_back(i);
                        g.wall_ic.push_back(q);
                    }
                }
                else if (xp)
                {
                    g.per_id.push_back(i);
                    g.per_i2.push_back(nb);
                    g.per_ic.push_back(q);
                }
            }
            else if (nb != -1)
            {
                if (!streams())
                {
                    g.wall_id.push_back(i);
                    g.wall_ic.push_back(q);
                }
            }
            else
            {
                // a wall neighbour; with no boundary type the reference reads
                // ifStream[-1]: treat the link as a wall
                bool wall = (b == -1) ? true : MANTIIS_IFSTREAM[b][q] == 0;
                if (b == -1) g.diag.buffer_wall_links++;
                if (wall)
                {
                    g.wall_id.push_back(i);
                    g.wall_ic.push_back(q);
                }
            }
        }
        if (g.y[i] == ny_c && g.x[i] == 0) g.inlet = i;
        else if (g.y[i] == ny_c && g.x[i] == n - 1) g.outlet = i;
        else if (g.y[i] == ny_c && g.x[i] == 1) g.inlet2 = i;
        else if (g.y[i] == ny_c && g.x[i] == n - 2) g.outlet2 = i;
    }
}

void Builder::build_taus()
{
    g.tau.assign(g.n_cells, 0.0);
    const double k6pi = std::sqrt(6.0 / M_PI);
    if (!opt.multiblock)
    {
        // include/coreLB.hpp:482-502
        for (int64_t c = 0; c < g.n_cells; c++)
            g.tau[c] = 0.5 + k6pi * g.locpore[c] * g.kn[c] / (1 + 2 * g.kn[c]);
        return;
    }
    // include/coreLB.hpp:432-480: per level, properties of the shrunk image
    std::vector<std::vector<double>> tau_lvl(g.max_level);
    for (int l = 0; l < g.max_level; l++)
    {
        int f = 1 << l;
        int m = n / f;
        std::vector<int> shr = shrink_binary(img.pore, n, f);
        std::vector<int> dom((size_t)m * m, 1);
        for (int i = 1; i < m - 1; i++)
            for (int j = 0; j < m; j++) dom[(size_t)i * m + j] = shr[(size_t)i * m + j];
        for (int j = 0; j < m; j++)
        {
            dom[j] = 0;
            dom[(size_t)(m - 1) * m + j] = 0;
        }
        std::vector<double> lp, kn;
        local_pore_properties(dom, m, opt.dx / std::pow(0.5, l), opt.mfp, lp, kn);
        tau_lvl[l].resize((size_t)m * m);
        for (size_t k = 0; k < (size_t)m * m; k++) tau_lvl[l][k] = 0.5 + k6pi * lp[k] * kn[k] / (1 + 2 * kn[k]);
    }
    for (int64_t c = 0; c < g.n_cells; c++)
    {
        int l = g.level[c];
        int f = 1 << (l - 1);
        int m = n / f;
        g.tau[c] = tau_lvl[l - 1][(size_t)(g.y[c] / f) * m + (g.x[c] / f)];
    }
}
} // namespace

int boundary_type_of(const int64_t *conn9)
{
    int code = 0;
    for (int k = 0; k < 9; k++) code = (code << 1) | (conn9[kDirOrder[k]] == -1 ? 0 : 1);
    if (code == 511) return -1;
    for (int t = 0; t < MANTIIS_N_BND_TYPES; t++)
        if (MANTIIS_BND_CODES[t] == code) return t;
    throw std::runtime_error("[ERROR]: Boundary type is not contained.");
}

Grid build_grid(const PoreImage &img, const GridOptions &opt)
{
    if ((size_t)img.n * img.n != img.pore.size()) throw std::runtime_error("pore image size mismatch");
    Builder b(img, opt);
    b.build_cells();
    b.build_boundary_types();
    b.build_links();
    b.build_taus();
    return std::move(b.g);
}
} // namespace mantiis
