// Kernels of the lattice Boltzmann step (sm_103a): the fused AA-pattern
// collide-and-stream, the output/residual pass, the coarse/fine interface
// exchange and the equilibrium initialisation.
#pragma once
#include <cuda_runtime.h>

#include "device.cuh"

namespace mantiis
{
namespace dev
{
constexpr int kMaxLevels = 4;

struct AllLevels
{
    LevelView lv[kMaxLevels];
    int parity[kMaxLevels]; // parity of the next step of each level
    int direct[kMaxLevels]; // level holds f itself (no step since initialisation)
};

// Sum of two doubles over the block, then one atomic per block.
__device__ __forceinline__ void block_add2(double a, double b, double *dst)
{
    __shared__ double sa[32], sb[32];
    for (int o = 16; o > 0; o >>= 1)
    {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
    {
        sa[wid] = a;
        sb[wid] = b;
    }
    __syncthreads();
    if (wid == 0)
    {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sa[lane] : 0.0;
        b = lane < nw ? sb[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1)
        {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if (lane == 0)
        {
            if (a != 0.0) atomicAdd(dst, a);
            if (b != 0.0) atomicAdd(dst + 1, b);
        }
    }
    __syncthreads();
}

// Loads the populations of a cell of level view L for a step (or a read) at
// parity P.  Returns 1/tau_s and, for special cells, a copy of the record.
template <int P>
__device__ __forceinline__ float load_cell(const LevelView &L, const Common &C, int x, int y, int direct, int first_sub,
                                           float df[9], bool &special, SpecialRec &rec)
{
    const int64_t s = site_of(L, x, y);
    float om = L.omega[s];
    special = om < 0.0f;
    if (!special)
    {
        if (direct) load_raw<0>(L, x, y, df);
        else load_raw<P>(L, x, y, df);
        return om;
    }
    rec = C.specials[L.spec[s]];
    const uint32_t flags = (rec.m1 >> 17) & 0xFu;
    if ((flags & SF_BUFFER) && (first_sub || direct))
    {
#pragma unroll
        for (int q = 0; q < 9; q++) df[q] = C.ibuf[(size_t)q * C.n_buf + rec.buf];
    }
    else if (direct)
        load_raw<0>(L, x, y, df);
    else
        load_special<P>(L, C, rec, x, y, df);
    return -om;
}

// Collision and streaming of one cell whose populations df are loaded:
// macroscopic moments (and the residual / snapshot side outputs), equilibrium,
// regularized MRT / MRT / BGK collision, the wall values of special cells and
// the AA-pattern store (include/coreLB.hpp:420-430, 646-792, 834-977, 1018-1054).
template <int P>
__device__ __forceinline__ void step_cell(const LevelView &L, const Common &C, const StepOpt &o, int x, int y, int64_t s,
                                          const float df[9], float omega, bool special, const SpecialRec &rec,
                                          double &r_diff, double &r_norm, bool interior = false)
{
    float drho, rho, ux, uy;
    macro(df, C.rho0, L.fshift, 0.0f, drho, rho, ux, uy);
    if (o.diff | o.store_u)
    {
        const float un = sqrtf(ux * ux + uy * uy);
        if (o.diff)
        {
            r_diff = (double)fabsf(un - L.unorm[s]);
            r_norm = (double)un;
        }
        if (o.store_u) L.unorm[s] = un;
    }
    if (o.snap_store)
    {
        L.snap[s] = drho;
        L.snap[L.plane + s] = ux;
        L.snap[2 * L.plane + s] = uy;
    }
    float edrho = drho, erho = rho, eux = ux, euy = uy;
    if (o.snap_use)
    {
        edrho = L.snap[s];
        erho = C.rho0 + edrho;
        eux = L.snap[L.plane + s];
        euy = L.snap[2 * L.plane + s];
    }
    float feq[9], fs[9];
    equilibrium(edrho, erho, eux, euy, feq);
    if (C.collision == COLL_RMRT) collide_rmrt(df, feq, edrho, erho, eux, euy, omega, fs);
    else if (C.collision == COLL_MRT) collide_mrt(df, feq, 1.0f / omega, L.tau2 ? L.tau2[s] : 1.0f, fs);
    else
    {
        const float inv_tau = 1.0f; // 1 / tau_SRT, tau_SRT = 1 (include/globalParameters.hpp:140)
#pragma unroll
        for (int q = 0; q < 9; q++) fs[q] = df[q] - inv_tau * (df[q] - feq[q]);
    }
    if (special)
    {
        const uint32_t wall = (rec.m0 >> 18) & 0x1FFu, quirk = rec.m1 & 0x1FFu;
        if (wall && C.wall == WALL_MDBB)
        {
            // include/coreLB.hpp:936-967: reflected value
            //   r f*_q + (1 - r) (sum_{c.n<0} f / sum_{c.n>0} f_eq) f_eq,opp(q)
            // in deviation form; both sums share the weight total A.
            const uint32_t bnd = (rec.m1 >> 9) & 0xFFu;
            const uint32_t pos = bnd == 0xFFu ? 0u : c_npos[bnd], neg = bnd == 0xFFu ? 0u : c_nneg[bnd];
            float a = 0.f, ap = 0.f, A = 0.f;
#pragma unroll
            for (int q = 0; q < 9; q++)
            {
                if ((neg >> q) & 1u) a += df[q];
                if ((pos >> q) & 1u)
                {
                    ap += feq[q];
                    A += wq(q) * C.rho0;
                }
            }
            const float g = (A + ap) != 0.f ? (a - ap) / (A + ap) : 0.f;
            const float r = rec.r;
#pragma unroll
            for (int q = 0; q < 9; q++)
                if ((wall >> q) & 1u)
                {
                    const int po = d2q9::opp(q);
                    fs[q] = r * fs[q] + (1.0f - r) * (feq[po] + (wq(po) * C.rho0 + feq[po]) * g);
                }
        }
        if (quirk)
        {
            float *side_now = C.side + (size_t)P * C.n_quirk;
            int qi = 0;
#pragma unroll
            for (int q = 0; q < 9; q++)
                if ((quirk >> q) & 1u) side_now[rec.quirk_base + qi++] = fs[q];
        }
    }
    store_post<P>(L, x, y, fs, interior);
}

// Plain cells of one level (all nine populations stream in, no wall link):
// one thread per site, 32x8 sites per block, blocks over the active tiles.
// Each slot a thread reads is written by that thread alone in this launch (AA
// ownership), so the loads take the read-only path.
template <int P> __global__ void __launch_bounds__(256, 6) k_plain(LevelView L, Common C, StepOpt o)
{
    // the tile id and this row's plain-cell mask are independent loads, so the
    // relaxation rate and the populations are then fetched together
    const int tile = __ldg(&L.tiles[blockIdx.x]);
    const uint32_t mask = __ldg(&L.tile_mask[blockIdx.x * 8 + (threadIdx.x >> 5)]);
    const int tx = tile % L.tiles_x, ty = tile / L.tiles_x;
    const int x = tx * 32 + (threadIdx.x & 31);
    const int y = ty * 8 + (threadIdx.x >> 5);
    // tiles off the border reach their neighbours without wrapping
    const bool interior = tx > 0 && tx + 1 < L.tiles_x && ty > 0 && ty + 1 < (L.H + 7) / 8;
    double r_diff = 0.0, r_norm = 0.0;
    if ((mask >> (threadIdx.x & 31)) & 1u)
    {
        const int64_t s = site_of(L, x, y);
        float df[9];
        if (o.direct) load_raw_ro<0>(L, x, y, df);
        else load_raw_ro<P>(L, x, y, df, interior);
        const float om = __ldg(&L.omega[s]);
        SpecialRec none;
        step_cell<P>(L, C, o, x, y, s, df, om, false, none, r_diff, r_norm, interior);
    }
    if (o.diff) block_add2(r_diff, r_norm, C.red + o.red_slot);
}

// Persistent, software-pipelined variant of k_plain: each block walks the
// tiles blockIdx.x, blockIdx.x + gridDim.x, ... and issues the loads of its
// next tile before colliding and storing the current one, so that memory
// requests stay in flight during the arithmetic.  The next tile's slots are
// disjoint from the current tile's (AA ownership), so the early loads are safe.
template <int P> __global__ void __launch_bounds__(256, 4) k_plain_pipe(LevelView L, Common C, StepOpt o)
{
    double r_diff = 0.0, r_norm = 0.0;
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    int t = blockIdx.x;
    float cur[9], nxt[9];
    float ctau = 0.0f;
    int cx = 0, cy = 0;
    auto fetch = [&](int tile, float v[9], float &tau, int &x, int &y) {
        const int tt = __ldg(&L.tiles[tile]);
        x = (tt % L.tiles_x) * 32 + lx;
        y = (tt / L.tiles_x) * 8 + ly;
        tau = 0.0f;
        if (x < L.W && y < L.H)
        {
            tau = __ldg(&L.omega[site_of(L, x, y)]);
            if (tau > 0.0f)
            {
                if (o.direct) load_raw_ro<0>(L, x, y, v);
                else load_raw_ro<P>(L, x, y, v);
            }
        }
    };
    if (t < L.ntiles) fetch(t, cur, ctau, cx, cy);
    for (; t < L.ntiles; t += gridDim.x)
    {
        const int tn = t + gridDim.x;
        float ntau = 0.0f;
        int nx = 0, ny = 0;
        if (tn < L.ntiles) fetch(tn, nxt, ntau, nx, ny);
        if (ctau > 0.0f)
        {
            SpecialRec none;
            double rd = 0.0, rn = 0.0;
            step_cell<P>(L, C, o, cx, cy, site_of(L, cx, cy), cur, ctau, false, none, rd, rn);
            r_diff += rd;
            r_norm += rn;
        }
#pragma unroll
        for (int q = 0; q < 9; q++) cur[q] = nxt[q];
        ctau = ntau;
        cx = nx;
        cy = ny;
    }
    if (o.diff) block_add2(r_diff, r_norm, C.red + o.red_slot);
}

// Special cells of one level, from the level's site-sorted record range.
template <int P>
__global__ void __launch_bounds__(128) k_special(LevelView L, Common C, StepOpt o, int64_t begin, int count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double r_diff = 0.0, r_norm = 0.0;
    if (i < count)
    {
        const SpecialRec rec = C.specials[begin + i];
        const int x = rec.site % L.pitch, y = rec.site / L.pitch;
        float df[9];
        const uint32_t flags = (rec.m1 >> 17) & 0xFu;
        if ((flags & SF_BUFFER) && (o.first_sub || o.direct))
        {
#pragma unroll
            for (int q = 0; q < 9; q++) df[q] = C.ibuf[(size_t)q * C.n_buf + rec.buf];
        }
        else if (o.direct)
            load_raw<0>(L, x, y, df);
        else
            load_special<P>(L, C, rec, x, y, df);
        step_cell<P>(L, C, o, x, y, (int64_t)rec.site, df, rec.omega, true, rec, r_diff, r_norm);
    }
    if (o.diff) block_add2(r_diff, r_norm, C.red + o.red_slot);
}

// Maximum of a non-negative double over the block, then one atomic per block
// (non-negative doubles order like their bit patterns).
__device__ __forceinline__ void block_max(double v, double *dst)
{
    __shared__ double sm[32];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (wid == 0)
    {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? sm[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0)
            atomicMax(reinterpret_cast<unsigned long long *>(dst), (unsigned long long)__double_as_longlong(v));
    }
    __syncthreads();
}

// Adsorption, first pass of a step (include/mantiisApp.hpp:248-252,
// include/coreLB.hpp:1056-1067, 515-531, 1269-1283): density of every cell from
// its streamed populations, its pseudopotential, and the relative density change
// since the previous step (maximum over the cells).
template <int P> __global__ void __launch_bounds__(256) k_ads_psi(LevelView L, Common C, StepOpt o)
{
    const int tile = L.tiles[blockIdx.x];
    const int x = (tile % L.tiles_x) * 32 + (threadIdx.x & 31);
    const int y = (tile / L.tiles_x) * 8 + (threadIdx.x >> 5);
    double rmax = 0.0;
    if (x < L.W && y < L.H && L.omega[site_of(L, x, y)] != 0.0f)
    {
        const int64_t s = site_of(L, x, y);
        float df[9];
        bool special;
        SpecialRec rec;
        load_cell<P>(L, C, x, y, o.direct, o.first_sub, df, special, rec);
        float drho = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) drho += df[q];
        const float rho = C.rho0 + drho;
        L.psi[s] = pseudo_potential((float)C.psi_form, C.psi_rho0, C.eos_a, C.eos_b, C.eos_T, C.g_ff, rho);
        const float old = L.rho_prev[s];
        rmax = (double)(fabsf(rho - old) / old);
        L.rho_prev[s] = rho;
    }
    if (o.diff) block_max(rmax, C.red + o.red_slot);
}

// Adsorption, second pass: Shan-Chen force (include/coreLB.hpp:533-566),
// velocity with the half-force shift (:1069-1099), equilibrium, plain MRT
// (:694-742), Guo source term (:568-630), AA store.  Bounce-back walls, the
// x-periodic links and the inlet/outlet overwrite (:859-865, 969-1009) are
// applied when the populations are read in the next step.
template <int P> __global__ void __launch_bounds__(256) k_ads_step(LevelView L, Common C, StepOpt o)
{
    const int tile = L.tiles[blockIdx.x];
    const int x = (tile % L.tiles_x) * 32 + (threadIdx.x & 31);
    const int y = (tile / L.tiles_x) * 8 + (threadIdx.x >> 5);
    if (x >= L.W || y >= L.H) return;
    const int64_t s = site_of(L, x, y);
    if (L.omega[s] == 0.0f) return;
    float df[9];
    bool special;
    SpecialRec rec;
    const float omega = load_cell<P>(L, C, x, y, o.direct, o.first_sub, df, special, rec);
    const uint32_t out = special ? ((rec.m1 >> 21) & 0x1FFu) : 0x1FFu;
    const uint32_t wall = special ? ((rec.m0 >> 18) & 0x1FFu) : 0u;
    // sum over the streaming links of w_f psi(x + c) c, formed from psi differences
    const float psx = L.psi[s];
    float sx = 0.f, sy = 0.f, cwx = 0.f, cwy = 0.f, wwx = 0.f, wwy = 0.f;
#pragma unroll
    for (int q = 1; q < 9; q++)
    {
        const float w = (float)d2q9::wf(q);
        if ((out >> q) & 1u)
        {
            const int xn = wrapx(x + d2q9::cx(q), L.W), yn = wrapx(y + d2q9::cy(q), L.H);
            const float dpsi = L.psi[site_of(L, xn, yn)] - psx;
            sx += w * dpsi * (float)d2q9::cx(q);
            sy += w * dpsi * (float)d2q9::cy(q);
            cwx += w * (float)d2q9::cx(q);
            cwy += w * (float)d2q9::cy(q);
        }
        if ((wall >> q) & 1u)
        {
            wwx += w * (float)d2q9::cx(q);
            wwy += w * (float)d2q9::cy(q);
        }
    }
    const float kff = -6.0f * C.g_ff * psx;
    const float Fx = kff * (sx + psx * cwx) - C.g_fs * psx * psx * wwx + C.fbody;
    const float Fy = kff * (sy + psx * cwy) - C.g_fs * psx * psx * wwy;
    float drho = 0.0f, jx = 0.0f, jy = 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        drho += df[q];
        jx += (float)d2q9::cx(q) * df[q];
        jy += (float)d2q9::cy(q) * df[q];
    }
    const float rho = C.rho0 + drho;
    const float ux = (jx + 0.5f * Fx) / rho, uy = (jy + 0.5f * Fy) / rho;
    if (o.snap_store)
    {
        L.snap[s] = drho;
        L.snap[L.plane + s] = ux;
        L.snap[2 * L.plane + s] = uy;
    }
    float feq[9], fs[9];
    equilibrium(drho, rho, ux, uy, feq);
    const float tau_s = 1.0f / omega, tau_d = L.tau2[s];
    collide_mrt(df, feq, tau_s, tau_d, fs);
    add_source(fs, ux, uy, Fx, Fy, tau_s, tau_d);
    if (special && (rec.m1 & 0x1FFu))
    {
        const uint32_t quirk = rec.m1 & 0x1FFu;
        float *side_now = C.side + (size_t)P * C.n_quirk;
        int qi = 0;
#pragma unroll
        for (int q = 0; q < 9; q++)
            if ((quirk >> q) & 1u) side_now[rec.quirk_base + qi++] = fs[q];
    }
    store_post<P>(L, x, y, fs);
}

// Reads the current state of every reference cell (no update): FP64 density,
// velocity and populations in reference cell order, plus the residual terms
// against the stored |u| and the pixel-area sums of u_x and rho.
__global__ void __launch_bounds__(256) k_cells(AllLevels A, Common C, const int32_t *cell_level, const int32_t *cell_site,
                                               int64_t n, double *rho_out, double *ux_out, double *uy_out, double *f_out,
                                               int diff, int store_u, int red_slot)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double r_diff = 0.0, r_norm = 0.0, r_ux = 0.0, r_rho = 0.0;
    if (c < n)
    {
        const int l = cell_level[c] - 1;
        const LevelView &L = A.lv[l];
        const int s = cell_site[c];
        const int x = s % L.pitch, y = s / L.pitch;
        float df[9];
        bool special;
        SpecialRec rec;
        // after a coarse step every interface buffer holds its interpolated values
        if (A.parity[l] == 0) load_cell<0>(L, C, x, y, A.direct[l], 1, df, special, rec);
        else load_cell<1>(L, C, x, y, A.direct[l], 1, df, special, rec);
        float drho, rho, ux, uy;
        macro(df, C.rho0, L.fshift, 0.0f, drho, rho, ux, uy);
        if (diff | store_u)
        {
            const float un = sqrtf(ux * ux + uy * uy);
            if (diff)
            {
                r_diff = (double)fabsf(un - L.unorm[s]);
                r_norm = (double)un;
            }
            if (store_u) L.unorm[s] = un;
        }
        // FP64 outputs from the FP32 deviations
        double ddr = 0, jx = 0, jy = 0;
        for (int q = 0; q < 9; q++)
        {
            ddr += (double)df[q];
            jx += (double)d2q9::cx(q) * (double)df[q];
            jy += (double)d2q9::cy(q) * (double)df[q];
        }
        double r = (double)C.rho0 + ddr;
        double vx = (jx + (double)L.fshift) / r, vy = jy / r;
        if (C.adsorption)
        {
            // the reference reports the density and velocity computed at the
            // start of the last step (include/mantiisApp.hpp:248-265)
            r = (double)C.rho0 + (double)L.snap[s];
            vx = (double)L.snap[L.plane + s];
            vy = (double)L.snap[2 * L.plane + s];
        }
        if (rho_out) rho_out[c] = r;
        if (ux_out) ux_out[c] = vx;
        if (uy_out) uy_out[c] = vy;
        if (f_out)
            for (int q = 0; q < 9; q++) f_out[c * 9 + q] = d2q9::w(q) * (double)C.rho0 + (double)df[q];
        const bool buffer = special && (((rec.m1 >> 17) & 0xFu) & SF_BUFFER);
        if (!buffer)
        {
            const double area = (double)(1 << (2 * l));
            r_ux = vx * area;
            r_rho = r * area;
        }
    }
    if (red_slot >= 0)
    {
        block_add2(r_diff, r_norm, C.red + red_slot);
        block_add2(r_ux, r_rho, C.red + red_slot + 2);
    }
}

// Coarse buffer cells <- rescaled mean of their 4 children
// (include/coreLB.hpp:1104-1135): f_c = f_eq,c + 2 tau_c / mean(tau_f) (mean(f_f) - f_eq,c).
template <int PF>
__global__ void __launch_bounds__(128) k_coarse(LevelView Lf, LevelView Lc, Common C, const CoarseRowDev *rows, int nrows)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const CoarseRowDev row = rows[r];
    float mean[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 4; k++)
    {
        if (row.child[k] < 0) continue;
        float df[9];
        if (row.child_buf[k] >= 0)
        {
#pragma unroll
            for (int q = 0; q < 9; q++) df[q] = C.ibuf[(size_t)q * C.n_buf + row.child_buf[k]];
        }
        else
        {
            bool special;
            SpecialRec rec;
            load_cell<PF>(Lf, C, row.child[k] % Lf.pitch, row.child[k] / Lf.pitch, 0, 0, df, special, rec);
        }
#pragma unroll
        for (int q = 0; q < 9; q++) mean[q] += df[q];
    }
    const float drho = Lc.snap[row.site], ux = Lc.snap[Lc.plane + row.site], uy = Lc.snap[2 * Lc.plane + row.site];
    float feq[9];
    equilibrium(drho, C.rho0 + drho, ux, uy, feq);
#pragma unroll
    for (int q = 0; q < 9; q++)
        C.ibuf[(size_t)q * C.n_buf + row.buf] = feq[q] + row.ratio * (mean[q] * row.inv_nchild - feq[q]);
}

// Fine buffer cells <- bicubic spline of the parent neighbourhood
// (include/coreLB.hpp:1137-1230); the spline is linear in the node values, so
// each child holds 6 precomputed weights.  f = f_eq + tau_f / (2 tau_c) (f_spline - f_eq).
template <int PC>
__global__ void __launch_bounds__(128) k_fine(LevelView Lf, LevelView Lc, Common C, const FineRowDev *rows, int nrows)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const FineRowDev &row = rows[r];
    float z[6][9];
    for (int k = 0; k < 6; k++)
    {
        if (row.node_buf[k] >= 0)
        {
#pragma unroll
            for (int q = 0; q < 9; q++) z[k][q] = C.ibuf[(size_t)q * C.n_buf + row.node_buf[k]];
        }
        else
        {
            bool special;
            SpecialRec rec;
            load_cell<PC>(Lc, C, row.node_site[k] % Lc.pitch, row.node_site[k] / Lc.pitch, 0, 0, z[k], special, rec);
        }
    }
    for (int c = 0; c < 4; c++)
    {
        const int s = row.child_site[c];
        const float drho = Lf.snap[s], ux = Lf.snap[Lf.plane + s], uy = Lf.snap[2 * Lf.plane + s];
        float feq[9];
        equilibrium(drho, C.rho0 + drho, ux, uy, feq);
        const float rat = row.ratio[c];
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < 6; k++) v += row.weight[c][k] * z[k][q];
            C.ibuf[(size_t)q * C.n_buf + row.child_buf[c]] = feq[q] + rat * (v - feq[q]);
        }
    }
}

// f = f_eq(rho, u) per reference cell, written into its own slots (state then
// reads "direct") and, for interface buffers, into the interpolation buffer.
__global__ void k_set_equilibrium(AllLevels A, Common C, const int32_t *cell_level, const int32_t *cell_site, int64_t n,
                                  const double *rho, const double *ux, const double *uy)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int l = cell_level[c] - 1;
    const LevelView &L = A.lv[l];
    const int s = cell_site[c];
    const double r = rho[c], vx = ux[c], vy = uy[c];
    const double usq = vx * vx + vy * vy;
    float df[9];
    for (int q = 0; q < 9; q++)
    {
        const double cu = d2q9::cx(q) * vx + d2q9::cy(q) * vy;
        // deviation from w rho0, formed in FP64 before rounding
        const double feq = d2q9::w(q) * r * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
        df[q] = (float)(feq - d2q9::w(q) * (double)C.rho0);
        L.f[(size_t)q * L.plane + s] = df[q];
    }
    if (L.rho_prev)
    {
        // the same FP32 sum as the first step's density, so an unchanged state
        // reads as no change
        float drho = 0.0f;
        for (int q = 0; q < 9; q++) drho += df[q];
        L.rho_prev[s] = C.rho0 + drho;
    }
    if (L.snap)
    {
        L.snap[s] = (float)(r - (double)C.rho0);
        L.snap[L.plane + s] = (float)vx;
        L.snap[2 * L.plane + s] = (float)vy;
    }
    if (L.omega[s] < 0.0f)
    {
        const SpecialRec rec = C.specials[L.spec[s]];
        if (((rec.m1 >> 17) & 0xFu) & SF_BUFFER)
            for (int q = 0; q < 9; q++) C.ibuf[(size_t)q * C.n_buf + rec.buf] = df[q];
    }
}
} // namespace dev
} // namespace mantiis
