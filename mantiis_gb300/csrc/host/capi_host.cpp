// Host-only part of the C ABI (include/mantiis_gpu.h): grid construction,
// unit system, pore properties and the disk generator.  No CUDA calls.
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../../../include/mantiis_gpu.h"
#include "geometry.hpp"
#include "grid.hpp"
#include "units.hpp"

using namespace mantiis;

struct mgpu_grid
{
    Grid g;
};

namespace
{
thread_local std::string h_error;

template <typename F> int host_guard(F &&fn)
{
    try
    {
        return fn();
    }
    catch (const std::invalid_argument &e)
    {
        h_error = e.what();
        return MGPU_E_INPUT;
    }
    catch (const std::runtime_error &e)
    {
        h_error = e.what();
        return std::string(e.what()).rfind("[ERROR]", 0) == 0 ? MGPU_E_INPUT : MGPU_E_ARG;
    }
    catch (const std::exception &e)
    {
        h_error = e.what();
        return MGPU_E_ARG;
    }
}

GridOptions options_of(const mgpu_params *p)
{
    UnitSystem u;
    u.Cl = p->dx;
    u.T_phy = p->T;
    u.P_phy = p->P;
    u.recompute();
    GridOptions o;
    o.multiblock = p->multiblock != 0;
    o.max_allowed_level = p->max_allowed_level;
    o.dx = p->dx;
    o.mfp = u.mfp;
    o.edge_fine = p->edge_fine != 0;
    return o;
}
} // namespace

extern "C" {

const char *mgpu_host_error(void) { return h_error.c_str(); }

int mgpu_grid_build(const int32_t *pore, const double *kn, const double *locpore, int n, const mgpu_params *p,
                    mgpu_grid **out)
{
    return host_guard([&]() {
        if (!pore || !kn || !locpore || !p || !out || n <= 0) throw std::invalid_argument("bad argument");
        PoreImage img;
        img.n = n;
        img.pore.assign(pore, pore + (size_t)n * n);
        img.kn.assign(kn, kn + (size_t)n * n);
        img.locpore.assign(locpore, locpore + (size_t)n * n);
        auto *g = new mgpu_grid();
        try
        {
            g->g = build_grid(img, options_of(p));
        }
        catch (...)
        {
            delete g;
            throw;
        }
        *out = g;
        return MGPU_OK;
    });
}

int mgpu_grid_build_from_folder(const char *folder, int n, const mgpu_params *p, mgpu_grid **out)
{
    return host_guard([&]() {
        if (!folder || !p || !out) throw std::invalid_argument("bad argument");
        PoreImage img = load_pore_image(folder, n);
        auto *g = new mgpu_grid();
        try
        {
            g->g = build_grid(img, options_of(p));
        }
        catch (...)
        {
            delete g;
            throw;
        }
        *out = g;
        return MGPU_OK;
    });
}

int mgpu_grid_sizes(const mgpu_grid *gh, int64_t s[12])
{
    if (!gh || !s) return MGPU_E_ARG;
    const Grid &g = gh->g;
    s[0] = g.n_cells;
    s[1] = g.max_level;
    s[2] = (int64_t)g.stream_id.size();
    s[3] = (int64_t)g.wall_id.size();
    s[4] = (int64_t)g.per_id.size();
    s[5] = (int64_t)g.coarse_rows.size();
    s[6] = (int64_t)g.fine_rows.size();
    s[7] = (int64_t)g.parent_child.size();
    s[8] = g.inlet;
    s[9] = g.inlet2;
    s[10] = g.outlet;
    s[11] = g.outlet2;
    return MGPU_OK;
}

int mgpu_grid_cells(const mgpu_grid *gh, int32_t *x, int32_t *y, int32_t *level, int32_t *type, int32_t *is_buffer,
                    int32_t *bnd, int64_t *conn, double *tau, double *kn, double *locpore, int64_t *lin)
{
    if (!gh) return MGPU_E_ARG;
    const Grid &g = gh->g;
    if (x) std::copy(g.x.begin(), g.x.end(), x);
    if (y) std::copy(g.y.begin(), g.y.end(), y);
    if (level) std::copy(g.level.begin(), g.level.end(), level);
    if (type) std::copy(g.type.begin(), g.type.end(), type);
    if (is_buffer) std::copy(g.is_buffer.begin(), g.is_buffer.end(), is_buffer);
    if (bnd) std::copy(g.bnd.begin(), g.bnd.end(), bnd);
    if (conn) std::copy(g.conn.begin(), g.conn.end(), conn);
    if (tau) std::copy(g.tau.begin(), g.tau.end(), tau);
    if (kn) std::copy(g.kn.begin(), g.kn.end(), kn);
    if (locpore) std::copy(g.locpore.begin(), g.locpore.end(), locpore);
    if (lin) std::copy(g.lin.begin(), g.lin.end(), lin);
    return MGPU_OK;
}

int mgpu_grid_links(const mgpu_grid *gh, int64_t *stream_id, int32_t *stream_ic, int64_t *stream_loc, int64_t *wall_id,
                    int32_t *wall_ic, int64_t *per_id, int64_t *per_i2, int32_t *per_ic)
{
    if (!gh) return MGPU_E_ARG;
    const Grid &g = gh->g;
    if (stream_id) std::copy(g.stream_id.begin(), g.stream_id.end(), stream_id);
    if (stream_ic) std::copy(g.stream_ic.begin(), g.stream_ic.end(), stream_ic);
    if (stream_loc) std::copy(g.stream_loc.begin(), g.stream_loc.end(), stream_loc);
    if (wall_id) std::copy(g.wall_id.begin(), g.wall_id.end(), wall_id);
    if (wall_ic) std::copy(g.wall_ic.begin(), g.wall_ic.end(), wall_ic);
    if (per_id) std::copy(g.per_id.begin(), g.per_id.end(), per_id);
    if (per_i2) std::copy(g.per_i2.begin(), g.per_i2.end(), per_i2);
    if (per_ic) std::copy(g.per_ic.begin(), g.per_ic.end(), per_ic);
    return MGPU_OK;
}

int mgpu_grid_interfaces(const mgpu_grid *gh, int64_t *coarse_rows, int64_t *fine_rows, int64_t *parent_child)
{
    if (!gh) return MGPU_E_ARG;
    const Grid &g = gh->g;
    if (coarse_rows)
        for (size_t r = 0; r < g.coarse_rows.size(); r++)
        {
            coarse_rows[r * 6] = g.coarse_key[r];
            for (int k = 0; k < 5; k++) coarse_rows[r * 6 + 1 + k] = g.coarse_rows[r][k];
        }
    if (fine_rows)
        for (size_t r = 0; r < g.fine_rows.size(); r++)
        {
            fine_rows[r * 6] = g.fine_key[r];
            for (int k = 0; k < 5; k++) fine_rows[r * 6 + 1 + k] = g.fine_rows[r][k];
        }
    if (parent_child)
        for (size_t r = 0; r < g.parent_child.size(); r++)
            for (int k = 0; k < 5; k++) parent_child[r * 5 + k] = g.parent_child[r][k];
    return MGPU_OK;
}

int mgpu_grid_diagnostics(const mgpu_grid *gh, int64_t out[5])
{
    if (!gh || !out) return MGPU_E_ARG;
    const GridDiagnostics &d = gh->g.diag;
    out[0] = d.buffer_wall_links;
    out[1] = d.fine_parent_missing_nbr;
    out[2] = d.coarse_missing_child;
    out[3] = d.fine_group_unmatched;
    out[4] = d.pore_search_failed;
    return MGPU_OK;
}

int mgpu_grid_destroy(mgpu_grid *g)
{
    delete g;
    return MGPU_OK;
}

int mgpu_units(double dx, double T, double P, double out[6])
{
    if (!out) return MGPU_E_ARG;
    UnitSystem u;
    u.Cl = dx;
    u.T_phy = T;
    u.P_phy = P;
    u.recompute();
    out[0] = u.rhoin;
    out[1] = u.mfp;
    out[2] = u.T_lu;
    out[3] = u.a_alpha_lu;
    out[4] = u.Cu;
    out[5] = u.Cf;
    return MGPU_OK;
}

int mgpu_pore_properties(const int32_t *pore, int n, double dx, double mfp, double *locpore, double *kn)
{
    return host_guard([&]() {
        if (!pore || !locpore || !kn || n <= 3) throw std::invalid_argument("bad argument");
        std::vector<int> dom(pore, pore + (size_t)n * n);
        std::vector<double> lp, k;
        local_pore_properties(dom, n, dx, mfp, lp, k);
        std::copy(lp.begin(), lp.end(), locpore);
        std::copy(k.begin(), k.end(), kn);
        return MGPU_OK;
    });
}

int mgpu_generate_disks(int n, double rmin, double rmax, double porosity, uint64_t seed, int32_t *pore_out)
{
    return mgpu_generate_disks_ex(n, rmin, rmax, porosity, seed, 0, pore_out);
}

int mgpu_generate_disks_ex(int n, double rmin, double rmax, double porosity, uint64_t seed, int flags,
                           int32_t *pore_out)
{
    return host_guard([&]() {
        if (!pore_out || n <= 0 || rmin <= 0 || rmax < rmin) throw std::invalid_argument("bad argument");
        std::vector<int> img =
            generate_disk_image(n, rmin, rmax, porosity, seed, (flags & MGPU_DISKS_PERIODIC_X) != 0,
                                (flags & (MGPU_DISKS_OPEN_X_EDGES | MGPU_DISKS_WIDE_X_EDGES)) != 0,
                                (flags & MGPU_DISKS_WIDE_X_EDGES) != 0 ? 3 : 2);
        std::copy(img.begin(), img.end(), pore_out);
        return MGPU_OK;
    });
}
} // extern "C"
