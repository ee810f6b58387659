// Kernels of the lattice Boltzmann step (sm_103a): the fused AA-pattern
// collide-and-stream, the output/residual pass, the coarse/fine interface
// exchange and the equilibrium initialisation.
#pragma once
#include <cuda_runtime.h>

#include "device.cuh"
#include "tma.cuh"

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

// The coarse-step-start moments (drho, u_x, u_y) of site s.  In a launch that
// uses them nothing writes them (phase 0 stored them), so the step kernels may
// take the read-only path (NC); the persistent step, where phase 0 ran earlier
// in the same launch, takes ordinary loads.
template <bool NC> __device__ __forceinline__ void load_snap(const LevelView &L, int64_t s, float sn[3])
{
    sn[0] = ldf<NC>(&L.snap[s]);
    sn[1] = ldf<NC>(&L.snap[L.plane + s]);
    sn[2] = ldf<NC>(&L.snap[2 * L.plane + s]);
}

// Collision and streaming of one cell whose populations df are loaded:
// macroscopic moments (and the residual / snapshot side outputs), equilibrium,
// regularized MRT / MRT / BGK collision, the wall values of special cells and
// the AA-pattern store (include/coreLB.hpp:420-430, 646-792, 834-977, 1018-1054).
template <int P>
__device__ __forceinline__ void step_cell(const LevelView &L, const Common &C, const StepOpt &o, int diff, int store_u,
                                          int x, int y, int64_t s, const float df[9], float omega, bool special,
                                          const SpecialRec &rec, double &r_diff, double &r_norm, bool interior = false,
                                          const float *unorm_prev = nullptr, const float *snap_prev = nullptr)
{
    float drho, rho, ux, uy;
    macro(df, C.rho0, L.fshift, 0.0f, drho, rho, ux, uy);
    if (diff | store_u)
    {
        const float un = sqrtf(ux * ux + uy * uy);
        if (diff)
        {
            r_diff = (double)fabsf(un - (unorm_prev ? *unorm_prev : L.unorm[s]));
            r_norm = (double)un;
        }
        if (store_u) L.unorm[s] = un;
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
        // the coarse-step-start moments: loaded by the caller with the populations
        // where it can (a load here is one more dependent round trip per cell)
        edrho = snap_prev ? snap_prev[0] : L.snap[s];
        erho = C.rho0 + edrho;
        eux = snap_prev ? snap_prev[1] : L.snap[L.plane + s];
        euy = snap_prev ? snap_prev[2] : L.snap[2 * L.plane + s];
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

// Plain cells of one active tile (all nine populations stream in, no wall
// link): one thread per site of a 32x8 tile, the row masks of plain cells let
// the relaxation rate and the nine populations load together.  Each slot a
// thread reads is written by that thread alone in this launch (AA ownership),
// so the loads take the read-only path.  Special cells (walls, missing
// arrivals, buffers) go to their own kernel: in the same warps their longer
// path would hold the plain lanes.
template <int P>
__device__ __forceinline__ void plain_tile(const LevelView &L, const Common &C, const StepOpt &o, int t, int diff,
                                           int store_u, double &r_diff, double &r_norm)
{
    // the tile id and this row's plain-cell mask are independent loads
    const int tile = __ldg(&L.tiles[t]); // tx | ty << 16
    const uint32_t mask = __ldg(&L.tile_mask[t * 8 + (threadIdx.x >> 5)]);
    const int tx = tile & 0xFFFF, ty = tile >> 16;
    const int x = tx * 32 + (threadIdx.x & 31);
    const int y = ty * 8 + (threadIdx.x >> 5);
    // tiles off the border reach their neighbours without wrapping
    const bool interior = tx > 0 && tx + 1 < L.tiles_x && ty > 0 && ty + 1 < (L.H + 7) / 8;
    if ((mask >> (threadIdx.x & 31)) & 1u)
    {
        const int64_t s = site_of(L, x, y);
        // (a "direct" state is read like an even step: own slots)
        float df[9], sn[3] = {0.f, 0.f, 0.f};
        const float uprev = diff ? __ldg(&L.unorm[s]) : 0.0f; // with the populations, as in plain_tile8
        if (o.snap_use) load_snap<true>(L, s, sn);
        load_raw_ro<P>(L, x, y, df, interior);
        const float om = __ldg(&L.omega[s]);
        SpecialRec none;
        step_cell<P>(L, C, o, diff, store_u, x, y, s, df, om, false, none, r_diff, r_norm, interior, &uprev,
                     o.snap_use ? sn : nullptr);
    }
}

// Plain cells of one 8x4 tile, one warp per tile (lane = 8 * row + column):
// the same cell update as plain_tile; on sparse levels these tiles hold a
// larger share of active cells than 32x8 tiles, so fewer lanes idle and fewer
// sectors are fetched for inactive sites.  The tile's light cells (special only
// through missing arrivals and buffer status: most of the interface ring of a
// finer level) are stepped here too, with the reads of special_cell for such a
// record (interpolated values at the first substep, else the arrivals plus the
// constant row), so the special-cell kernel keeps only the cells with walls.
template <int P, bool NC = true>
__device__ __forceinline__ void plain_tile8(const LevelView &L, const Common &C, const StepOpt &o, int t, int diff,
                                            int store_u, double &r_diff, double &r_norm)
{
    const int lane = threadIdx.x & 31;
    const int tile = __ldg(&L.tiles8[t]); // tx | ty << 16, in 8- and 4-site units
    const uint32_t mask = __ldg(&L.tile8_mask[t]);
    if (!((mask >> lane) & 1u)) return;
    const bool light = (__ldg(&L.tile8_light[t]) >> lane) & 1u;
    const int tx = tile & 0xFFFF, ty = tile >> 16;
    const int x = tx * 8 + (lane & 7), y = ty * 4 + (lane >> 3);
    // tiles off the border reach their neighbours without wrapping
    const bool interior = tx > 0 && tx + 1 < (L.W + 7) / 8 && ty > 0 && ty + 1 < (L.H + 3) / 4;
    const int64_t s = site_of(L, x, y);
    float df[9];
    float om;
    // the |u| the residual compares with, loaded with the populations (the
    // cell's own site: this thread alone writes it, after reading it)
    const float uprev = diff ? ldf<NC>(&L.unorm[s]) : 0.0f;
    float sn[3] = {0.f, 0.f, 0.f};
    if (o.snap_use) load_snap<NC>(L, s, sn);
    if (!light)
    {
        load_raw_ro<P, NC>(L, x, y, df, interior);
        om = __ldg(&L.omega[s]);
    }
    else
    {
        const SpecialRec rec = C.specials[__ldg(&L.spec[s])];
        const uint32_t arrive = rec.m0 & 0x1FFu, flags = (rec.m1 >> 17) & 0xFu;
        om = rec.omega;
        if ((flags & SF_BUFFER) && (o.first_sub || o.direct))
        {
#pragma unroll
            for (int q = 0; q < 9; q++) df[q] = C.ibuf[(size_t)q * C.n_buf + rec.buf];
        }
        else
        {
            // a direct state has parity 0: own slots, as load_raw<0>
            load_raw_ro<P, NC>(L, x, y, df, interior);
            if (!o.direct)
            {
                const bool has_k = (flags & SF_HAS_K) != 0;
                const float *k = C.ktab + (size_t)(has_k ? rec.k_row : 0) * 9;
#pragma unroll
                for (int q = 0; q < 9; q++)
                {
                    float v = ((arrive >> q) & 1u) ? df[q] : 0.0f;
                    if (has_k) v += __ldg(&k[q]);
                    df[q] = v;
                }
            }
        }
    }
    SpecialRec none;
    step_cell<P>(L, C, o, diff, store_u, x, y, s, df, om, false, none, r_diff, r_norm, interior, &uprev,
                 o.snap_use ? sn : nullptr);
}

// One special cell (wall links, missing arrivals, interface buffer, inlet /
// outlet) from its record.
template <int P>
__device__ __forceinline__ void special_cell(const LevelView &L, const Common &C, const StepOpt &o, int64_t i, int diff,
                                             int store_u, double &r_diff, double &r_norm)
{
    const SpecialRec rec = C.specials[i];
    const int x = rec.xy & 0xFFFF, y = rec.xy >> 16;
    const int64_t s = site_of(L, x, y);
    // the |u| the residual compares with, in flight with the populations
    const float uprev = diff ? L.unorm[s] : 0.0f;
    float sn[3] = {0.f, 0.f, 0.f};
    if (o.snap_use) load_snap<false>(L, s, sn);
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
    step_cell<P>(L, C, o, diff, store_u, x, y, s, df, rec.omega, true, rec, r_diff, r_norm, false, &uprev,
                 o.snap_use ? sn : nullptr);
}

// ---- phase kernels.  A coarse time step is a sequence of phases; a phase
// steps every (image, level) whose next substep falls on it.  All levels of an
// image are independent within a coarse step (they meet only in the interface
// exchange that closes it), so one launch covers them all.  The descriptors
// travel in the launch parameters: each owns a contiguous block range, so the
// descriptor index and its fields are block-uniform.

// One (image, level) in one phase: where its state is and how to step it.
struct StepDesc
{
    LevelView L;
    Common C;
    StepOpt o;
    int64_t spec_begin; // the level's special records
    int spec_count;
    int tile_base;      // first tile of the level's list this descriptor covers
};

// Per-launch residual switches: the residual terms (and the |u| store) apply
// to the first substep of each level, which falls on phase 0.
struct PhaseArgs
{
    int diff, store_u, red_slot;
};

constexpr int kMaxPhaseDescs = 24;

struct PhaseLaunch
{
    int ndesc;
    int start[kMaxPhaseDescs + 1]; // first block of each descriptor; start[ndesc] = blocks
    int grid;                      // blocks launched (k_phase_plain8: may be fewer; they loop)
    PhaseArgs a;
    StepDesc d[kMaxPhaseDescs];
};

// descriptor owning block b (block-uniform)
__device__ __forceinline__ int owner(const int *start, int n, int b)
{
    int j = 0;
#pragma unroll 1
    while (j + 1 < n && b >= start[j + 1]) j++;
    return j;
}

// plain cells with direct loads: blocks of a descriptor walk its tiles
__global__ void __launch_bounds__(256, 5) k_phase_plain(const __grid_constant__ PhaseLaunch P)
{
    const int j = owner(P.start, P.ndesc, (int)blockIdx.x);
    const StepDesc &d = P.d[j];
    const int t = d.tile_base + (int)blockIdx.x - P.start[j];
    const int diff = P.a.diff & d.o.first_sub, store_u = P.a.store_u & d.o.first_sub;
    double r_diff = 0.0, r_norm = 0.0;
    if (d.o.parity) plain_tile<1>(d.L, d.C, d.o, t, diff, store_u, r_diff, r_norm);
    else plain_tile<0>(d.L, d.C, d.o, t, diff, store_u, r_diff, r_norm);
    if (diff) block_add2(r_diff, r_norm, d.C.red + P.a.red_slot);
}

// plain cells in 8x4 tiles: 8 tiles (warps) per block-sized unit of work; a
// block walks units blockIdx.x, blockIdx.x + gridDim.x, ...  Alone the launch
// has a block per unit; when other images' kernels run beside it (batch
// streams) it has at most 4 blocks per SM, so they find room on every SM.
__global__ void __launch_bounds__(256, 5) k_phase_plain8(const __grid_constant__ PhaseLaunch P)
{
    const int units = P.start[P.ndesc];
    for (int u = (int)blockIdx.x; u < units; u += (int)gridDim.x)
    {
        const int j = owner(P.start, P.ndesc, u);
        const StepDesc &d = P.d[j];
        const int t = (u - P.start[j]) * 8 + (int)(threadIdx.x >> 5);
        const int diff = P.a.diff & d.o.first_sub, store_u = P.a.store_u & d.o.first_sub;
        double r_diff = 0.0, r_norm = 0.0;
        if (t < d.L.ntiles8)
        {
            if (d.o.parity) plain_tile8<1>(d.L, d.C, d.o, t, diff, store_u, r_diff, r_norm);
            else plain_tile8<0>(d.L, d.C, d.o, t, diff, store_u, r_diff, r_norm);
        }
        if (diff) block_add2(r_diff, r_norm, d.C.red + P.a.red_slot);
    }
}

// special cells: blocks of a descriptor walk its records, kSpecialBlock per block
// special records per block of k_phase_special (64 and 32 measured slower: config-2
// batch 338 / 343 / 353 us per coarse step for 128 / 64 / 32)
constexpr int kSpecialBlock = 128;

__global__ void __launch_bounds__(kSpecialBlock) k_phase_special(const __grid_constant__ PhaseLaunch P)
{
    const int j = owner(P.start, P.ndesc, (int)blockIdx.x);
    const StepDesc &d = P.d[j];
    const int i = ((int)blockIdx.x - P.start[j]) * kSpecialBlock + (int)threadIdx.x;
    const int diff = P.a.diff & d.o.first_sub, store_u = P.a.store_u & d.o.first_sub;
    double r_diff = 0.0, r_norm = 0.0;
    if (i < d.spec_count)
    {
        if (d.o.parity) special_cell<1>(d.L, d.C, d.o, d.spec_begin + i, diff, store_u, r_diff, r_norm);
        else special_cell<0>(d.L, d.C, d.o, d.spec_begin + i, diff, store_u, r_diff, r_norm);
    }
    if (diff) block_add2(r_diff, r_norm, d.C.red + P.a.red_slot);
}

// ---- plain cells through a TMA pipeline.  A persistent block walks the
// x-interior tiles of its descriptors; for each tile one bulk tensor copy
// brings the 9 planes with a halo of 4 columns and 1 row (a 40 x 10 x 9 box,
// x start 16-byte aligned), a second the tile's 32 x 8 relaxation rates and a
// bulk copy its 8 row masks into shared memory, two tiles ahead of the one
// being stepped.  Cells read their slots from shared memory (odd steps index
// the shifted neighbours there) and store as in plain_tile.
constexpr int kTmaW = 40, kTmaH = 10, kTmaStages = 2;
constexpr uint32_t kTmaFBytes = kTmaW * kTmaH * 9 * 4;
constexpr uint32_t kTmaOmOff = (kTmaFBytes + 127) / 128 * 128; // 128-byte aligned
constexpr uint32_t kTmaMaskOff = kTmaOmOff + 32 * 8 * 4;
constexpr uint32_t kTmaTxBytes = kTmaFBytes + 32 * 8 * 4 + 32;         // bytes the copies of one tile deliver
constexpr uint32_t kTmaStageBytes = (kTmaMaskOff + 32 + 127) / 128 * 128; // stage stride
constexpr int kMaxTmaDescs = 8;
constexpr uint32_t kWaitPolls = 1u << 26;

struct TmaLaunch
{
    CUtensorMap map[kMaxTmaDescs];    // per descriptor: its level's 9 planes as (x, y, q)
    CUtensorMap om_map[kMaxTmaDescs]; // per descriptor: its level's relaxation rates as (x, y)
    int grid;                         // persistent blocks of the launch (host side)
    int ndesc;
    int start[kMaxTmaDescs + 1];      // first tile (in launch order) of each descriptor
    PhaseArgs a;
    StepDesc d[kMaxTmaDescs];
};

template <int P>
__device__ __forceinline__ void plain_tile_smem(const LevelView &L, const Common &C, const StepOpt &o, int tile,
                                                const unsigned char *stage, int diff, int store_u, double &r_diff,
                                                double &r_norm)
{
    const float *sb = reinterpret_cast<const float *>(stage);
    const float *som = reinterpret_cast<const float *>(stage + kTmaOmOff);
    const uint32_t *smask = reinterpret_cast<const uint32_t *>(stage + kTmaMaskOff);
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    if (!((smask[ly] >> lx) & 1u)) return;
    const int x = (tile & 0xFFFF) * 32 + lx, y = (tile >> 16) * 8 + ly;
    const int64_t s = site_of(L, x, y);
    const float om = som[ly * 32 + lx];
    const float uprev = diff ? L.unorm[s] : 0.0f;
    float sn[3] = {0.f, 0.f, 0.f};
    if (o.snap_use) load_snap<true>(L, s, sn);
    float df[9];
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        // even: own slot (x, q); odd: slot (x - c_q, opp q)
        const int pq = P == 0 ? q : d2q9::opp(q);
        const int sy = ly + 1 - (P == 0 ? 0 : d2q9::cy(q)), sx = lx + 4 - (P == 0 ? 0 : d2q9::cx(q));
        df[q] = sb[(pq * kTmaH + sy) * kTmaW + sx];
    }
    SpecialRec none;
    step_cell<P>(L, C, o, diff, store_u, x, y, s, df, om, false, none, r_diff, r_norm, true, &uprev,
                 o.snap_use ? sn : nullptr);
}

__global__ void __launch_bounds__(256, 4) k_phase_plain_tma(const __grid_constant__ TmaLaunch P)
{
    __shared__ __align__(128) unsigned char sbuf[kTmaStages][kTmaStageBytes];
    __shared__ __align__(8) uint64_t full[kTmaStages];
    __shared__ int s_tile[kTmaStages];
    __shared__ int s_fail;
    static_assert(kTmaStageBytes % 128 == 0 && kTmaOmOff % 128 == 0 && kTmaMaskOff % 16 == 0, "stage layout");
    const int total = P.start[P.ndesc];
    if (threadIdx.x == 0)
    {
        for (int st = 0; st < kTmaStages; st++) mbar_init(&full[st], 1);
        s_fail = 0;
        fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int g, int st) {
        const int j = owner(P.start, P.ndesc, g);
        const int t = P.d[j].tile_base + g - P.start[j];
        const int tile = P.d[j].L.tiles[t];
        const int x0 = (tile & 0xFFFF) * 32, y0 = (tile >> 16) * 8;
        s_tile[st] = tile;
        mbar_arrive_expect_tx(&full[st], kTmaTxBytes);
        tma_load_3d(sbuf[st], &P.map[j], x0 - 4, y0 - 1, 0, &full[st]);
        tma_load_2d(sbuf[st] + kTmaOmOff, &P.om_map[j], x0, y0, &full[st]);
        bulk_load(sbuf[st] + kTmaMaskOff, P.d[j].L.tile_mask + (size_t)t * 8, 32, &full[st]);
    };
    if (threadIdx.x == 0)
        for (int st = 0; st < kTmaStages; st++)
        {
            const int g = (int)blockIdx.x + st * (int)gridDim.x;
            if (g < total) issue(g, st);
        }
    double r_diff = 0.0, r_norm = 0.0;
    int red_desc = -1;
    int it = 0;
    for (int g = (int)blockIdx.x; g < total; g += (int)gridDim.x, it++)
    {
        const int st = it % kTmaStages;
        const uint32_t parity = (uint32_t)(it / kTmaStages) & 1u;
        if (!mbar_wait_bounded(&full[st], parity, kWaitPolls)) atomicOr(&s_fail, 1);
        __syncthreads();
        if (s_fail) break;
        const int j = owner(P.start, P.ndesc, g);
        const StepDesc &d = P.d[j];
        const int diff = P.a.diff & d.o.first_sub, store_u = P.a.store_u & d.o.first_sub;
        if (diff) red_desc = j;
        const int tile = s_tile[st];
        if (d.o.parity) plain_tile_smem<1>(d.L, d.C, d.o, tile, sbuf[st], diff, store_u, r_diff, r_norm);
        else plain_tile_smem<0>(d.L, d.C, d.o, tile, sbuf[st], diff, store_u, r_diff, r_norm);
        // every thread is done with this stage before it is refilled
        __syncthreads();
        if (threadIdx.x == 0)
        {
            const int gn = g + kTmaStages * (int)gridDim.x;
            if (gn < total) issue(gn, st);
        }
    }
    if (s_fail)
    {
        if (threadIdx.x == 0)
        {
            atomicOr(P.d[0].C.err, kErrTmaTimeout);
            // let copies still in flight land before the block's shared memory goes
            for (int st = 0; st < kTmaStages; st++) mbar_wait_bounded(&full[st], 0u, 1024u);
        }
        return;
    }
    // residual terms: only single-image launches ask for them (one accumulator)
    if (P.a.diff)
    {
        const int rd = __syncthreads_or(red_desc >= 0) ? 0 : -1;
        if (rd == 0) block_add2(r_diff, r_norm, P.d[0].C.red + P.a.red_slot);
    }
}

// Maximum of a non-negative float over the block, then one atomic per block on
// the double it converts to: the conversion is exact and monotone, so this is
// the maximum of the converted values, with the shuffles on the FP32 pipe
// (non-negative doubles order like their bit patterns).
__device__ __forceinline__ void block_max(float v, double *dst)
{
    __shared__ float sm[32];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (wid == 0)
    {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? sm[lane] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0f)
            atomicMax(reinterpret_cast<unsigned long long *>(dst), (unsigned long long)__double_as_longlong((double)v));
    }
    __syncthreads();
}

// Adsorption, first pass of a step (include/mantiisApp.hpp:248-252,
// include/coreLB.hpp:1056-1067, 515-531, 1269-1283): density of every cell from
// its streamed populations, its pseudopotential, and the relative density change
// since the previous step (maximum over the cells).
// density and pseudopotential of one cell (pass 1), the density change against
// the previous step's density for the residual
template <int P, bool SPEC>
__device__ __forceinline__ float ads_density(const LevelView &L, const Common &C, const StepOpt &o, int x, int y)
{
    const int64_t s = site_of(L, x, y);
    float df[9];
    if (SPEC)
    {
        bool special;
        SpecialRec rec;
        load_cell<P>(L, C, x, y, o.direct, o.first_sub, df, special, rec);
    }
    else if (o.direct)
        load_raw<0>(L, x, y, df);
    else
        load_raw<P>(L, x, y, df);
    float drho = 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++) drho += df[q];
    const float rho = C.rho0 + drho;
    L.psi[s] = pseudo_potential((float)C.psi_form, C.psi_rho0, C.eos_a, C.eos_b, C.eos_T, C.g_ff, rho);
    const float old = L.rho_prev[s];
    L.rho_prev[s] = rho;
    return fabsf(rho - old) / old;
}

// pass 1 over the plain cells of active 32x8 tile t (row masks): one block
template <int P> __device__ __forceinline__ float ads_psi_tile(const LevelView &L, const Common &C, const StepOpt &o, int t)
{
    const int tile = L.tiles[t]; // tx | ty << 16
    const uint32_t mask = L.tile_mask[t * 8 + (threadIdx.x >> 5)];
    const int x = (tile & 0xFFFF) * 32 + (threadIdx.x & 31);
    const int y = (tile >> 16) * 8 + (threadIdx.x >> 5);
    return ((mask >> (threadIdx.x & 31)) & 1u) ? ads_density<P, false>(L, C, o, x, y) : 0.0f;
}

// pass 1 of special record i of the level (i < spec_count)
template <int P>
__device__ __forceinline__ float ads_psi_record(const LevelView &L, const Common &C, const StepOpt &o, int64_t rec)
{
    const int32_t xy = C.specials[rec].xy;
    return ads_density<P, true>(L, C, o, xy & 0xFFFF, xy >> 16);
}

template <int P> __global__ void __launch_bounds__(256) k_ads_psi(LevelView L, Common C, StepOpt o)
{
    const float rmax = ads_psi_tile<P>(L, C, o, (int)blockIdx.x);
    if (o.diff) block_max(rmax, C.red + o.red_slot);
}

// pass 1 over the special cells, from their records (128 per block)
template <int P> __global__ void __launch_bounds__(128) k_ads_psi_special(LevelView L, Common C, StepOpt o,
                                                                          int64_t spec_begin, int spec_count)
{
    const int i = (int)blockIdx.x * 128 + (int)threadIdx.x;
    const float rmax = i < spec_count ? ads_psi_record<P>(L, C, o, spec_begin + i) : 0.0f;
    if (o.diff) block_max(rmax, C.red + o.red_slot);
}

// Adsorption, second pass: Shan-Chen force (include/coreLB.hpp:533-566),
// velocity with the half-force shift (:1069-1099), equilibrium, plain MRT
// (:694-742), Guo source term (:568-630), AA store.  Bounce-back walls, the
// x-periodic links and the inlet/outlet overwrite (:859-865, 969-1009) are
// applied when the populations are read in the next step.
// The coupling phase of the coupled run (include/mantiisApp.hpp:267-284) takes
// the same body with the regularized MRT, SRBB walls, no inlet / outlet and the
// velocity residual (C.collision, C.wall, C.inlet_outlet; o.diff accumulates
// sum |u| for both terms, as its |u| of the previous step is never stored).
// psi[r][c]: the pseudopotential at (x + c - 1, y + r - 1); SPEC: the cell may
// be special (its record applies), else it is a plain cell
template <int P, bool SPEC>
__device__ __forceinline__ void ads_cell(const LevelView &L, const Common &C, const StepOpt &o, int x, int y,
                                         const float psi[3][3], double &r_diff, double &r_norm)
{
    const int64_t s = site_of(L, x, y);
    float df[9];
    bool special = false;
    SpecialRec rec;
    float omega;
    if (SPEC) omega = load_cell<P>(L, C, x, y, o.direct, o.first_sub, df, special, rec);
    else
    {
        if (o.direct) load_raw<0>(L, x, y, df);
        else load_raw<P>(L, x, y, df);
        omega = L.omega[s];
    }
    const uint32_t out = special ? ((rec.m1 >> 21) & 0x1FFu) : 0x1FFu;
    const uint32_t wall = special ? ((rec.m0 >> 18) & 0x1FFu) : 0u;
    // sum over the streaming links of w_f psi(x + c) c, formed from psi differences
    const float psx = psi[1][1];
    float sx = 0.f, sy = 0.f, cwx = 0.f, cwy = 0.f, wwx = 0.f, wwy = 0.f;
#pragma unroll
    for (int q = 1; q < 9; q++)
    {
        const float w = (float)d2q9::wf(q);
        if ((out >> q) & 1u)
        {
            const float dpsi = psi[1 + d2q9::cy(q)][1 + d2q9::cx(q)] - psx;
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
    if (o.diff)
    {
        const float un = sqrtf(ux * ux + uy * uy);
        r_diff = (double)un;
        r_norm = (double)un;
    }
    float feq[9], fs[9];
    equilibrium(drho, rho, ux, uy, feq);
    const float tau_s = 1.0f / omega, tau_d = L.tau2[s];
    if (C.collision == COLL_RMRT) collide_rmrt(df, feq, drho, rho, ux, uy, omega, fs);
    else collide_mrt(df, feq, tau_s, tau_d, fs);
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

// Pass 2 over the plain cells of active 32x8 tile t: one block.  The
// neighbour pseudopotentials come by warp shuffles: a warp holds one row of
// the tile, each lane loads psi of its column in the rows y-1, y, y+1
// (coalesced), and takes the x-neighbours from the adjacent lanes; the lanes at
// the ends of the row (and the last image column) load their outer neighbours.
template <int P>
__device__ __forceinline__ void ads_step_tile(const LevelView &L, const Common &C, const StepOpt &o, int t, double &r_diff,
                                              double &r_norm)
{
    const int tile = L.tiles[t]; // tx | ty << 16
    const int lane = threadIdx.x & 31;
    const int x = (tile & 0xFFFF) * 32 + lane;
    const int y = (tile >> 16) * 8 + (threadIdx.x >> 5);
    const bool inside = x < L.W && y < L.H;
    float psi[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
    {
        const int yr = wrapx(y + r - 1, L.H);
        psi[r][1] = inside ? L.psi[site_of(L, x, yr)] : 0.0f;
        psi[r][0] = __shfl_up_sync(0xffffffffu, psi[r][1], 1);
        psi[r][2] = __shfl_down_sync(0xffffffffu, psi[r][1], 1);
        if (inside && lane == 0) psi[r][0] = L.psi[site_of(L, wrapx(x - 1, L.W), yr)];
        if (inside && (lane == 31 || x + 1 == L.W)) psi[r][2] = L.psi[site_of(L, wrapx(x + 1, L.W), yr)];
    }
    const uint32_t mask = L.tile_mask[t * 8 + (threadIdx.x >> 5)];
    if ((mask >> lane) & 1u) ads_cell<P, false>(L, C, o, x, y, psi, r_diff, r_norm);
}

// pass 2 of special record rec; the neighbour pseudopotentials are read directly
template <int P>
__device__ __forceinline__ void ads_step_record(const LevelView &L, const Common &C, const StepOpt &o, int64_t rec,
                                                double &r_diff, double &r_norm)
{
    const int32_t xy = C.specials[rec].xy;
    const int x = xy & 0xFFFF, y = xy >> 16;
    float psi[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            psi[r][c] = L.psi[site_of(L, wrapx(x + c - 1, L.W), wrapx(y + r - 1, L.H))];
    ads_cell<P, true>(L, C, o, x, y, psi, r_diff, r_norm);
}

template <int P> __global__ void __launch_bounds__(256) k_ads_step(LevelView L, Common C, StepOpt o)
{
    double r_diff = 0.0, r_norm = 0.0;
    ads_step_tile<P>(L, C, o, (int)blockIdx.x, r_diff, r_norm);
    if (o.diff) block_add2(r_diff, r_norm, C.red + o.red_slot);
}

// pass 2 over the special cells, from their records (128 per block)
template <int P> __global__ void __launch_bounds__(128) k_ads_step_special(LevelView L, Common C, StepOpt o,
                                                                           int64_t spec_begin, int spec_count)
{
    const int i = (int)blockIdx.x * 128 + (int)threadIdx.x;
    double r_diff = 0.0, r_norm = 0.0;
    if (i < spec_count) ads_step_record<P>(L, C, o, spec_begin + i, r_diff, r_norm);
    if (o.diff) block_add2(r_diff, r_norm, C.red + o.red_slot);
}

// Reads the current state of every reference cell (no update): FP64 density,
// velocity and populations in reference cell order, plus the residual terms
// against the stored |u| and the pixel-area sums of u_x and rho.
__global__ void __launch_bounds__(256) k_cells(AllLevels A, Common C, const int32_t *cell_level, const int32_t *cell_site,
                                               const uint8_t *cell_buffer, int64_t n, double *rho_out, double *ux_out,
                                               double *uy_out, double *f_out, int diff, int store_u, int red_slot)
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
        // interface buffer cells cover pixels of finer cells: left out of the
        // pixel-area sums (also those that step like plain cells)
        if (!cell_buffer[c])
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

// Writes populations df of cell (x, y) into the slots its next step reads at
// parity P: its own slots (even) or the neighbours' opposite slots (odd).
// These slots belong to the cell (AA ownership), so nothing else touches them
// before that step.
__device__ __forceinline__ void store_for_load(const LevelView &L, int x, int y, const float df[9], int parity)
{
    if (parity == 0)
    {
        const int64_t s = site_of(L, x, y);
#pragma unroll
        for (int q = 0; q < 9; q++) L.f[q * L.plane + s] = df[q];
    }
    else
    {
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            const int xs = wrapx(x - d2q9::cx(q), L.W), ys = wrapx(y - d2q9::cy(q), L.H);
            L.f[d2q9::opp(q) * L.plane + site_of(L, xs, ys)] = df[q];
        }
    }
}

// The interface rows are handled by groups of 4 adjacent lanes (lane & 3 = k):
// each lane loads one child (coarse rows) or one or two spline nodes (fine
// rows), and the group exchanges the loaded populations with shuffles, so the
// loads of a row are in flight together and each is made once.  Sums run in
// the same order as one lane summing alone.

// populations of an interface source cell: its interpolation buffer, or the
// cell's own slots after streaming and its rules
template <int P>
__device__ __forceinline__ void load_source(const LevelView &L, const Common &C, int site, int buf, float z[9])
{
    if (buf >= 0)
    {
#pragma unroll
        for (int q = 0; q < 9; q++) z[q] = C.ibuf[(size_t)q * C.n_buf + buf];
    }
    else
    {
        bool special;
        SpecialRec rec;
        load_cell<P>(L, C, site % L.pitch, site / L.pitch, 0, 0, z, special, rec);
    }
}

// Coarse buffer cells <- rescaled mean of their 4 children
// (include/coreLB.hpp:1104-1135): f_c = f_eq,c + 2 tau_c / mean(tau_f) (mean(f_f) - f_eq,c).
// Lane k of the group loads child k; lane 0 writes the result.
template <int PF>
__device__ __forceinline__ void coarse_row(const LevelView &Lf, const LevelView &Lc, const Common &C,
                                           const CoarseRowDev &row, int k, bool valid, int pc)
{
    const int lane = threadIdx.x & 31, base = lane & ~3;
    const bool has = valid && row.child[k] >= 0;
    float df[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (has) load_source<PF>(Lf, C, row.child[k], row.child_buf[k], df);
    float mean[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
    {
        const bool present = __shfl_sync(0xffffffffu, has ? 1 : 0, base + kk) != 0;
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            const float v = __shfl_sync(0xffffffffu, df[q], base + kk);
            if (present) mean[q] += v;
        }
    }
    if (!valid || k != 0) return;
    const float drho = Lc.snap[row.site], ux = Lc.snap[Lc.plane + row.site], uy = Lc.snap[2 * Lc.plane + row.site];
    float feq[9];
    equilibrium(drho, C.rho0 + drho, ux, uy, feq);
    float v[9];
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        v[q] = feq[q] + row.ratio * (mean[q] * row.inv_nchild - feq[q]);
        C.ibuf[(size_t)q * C.n_buf + row.buf] = v[q];
    }
    if (row.plain_target) store_for_load(Lc, row.site % Lc.pitch, row.site / Lc.pitch, v, pc);
}

// Fine buffer cells <- bicubic spline of the parent neighbourhood
// (include/coreLB.hpp:1137-1230); the spline is linear in the node values, so
// each child holds 6 precomputed weights.  f = f_eq + tau_f / (2 tau_c) (f_spline - f_eq).
// Lane c of the group loads nodes c and c + 4 (c < 2) and computes child c.
template <int PC>
__device__ __forceinline__ void fine_child(const LevelView &Lf, const LevelView &Lc, const Common &C,
                                           const FineRowDev &row, int c, bool valid, int pf)
{
    const int lane = threadIdx.x & 31, base = lane & ~3;
    float za[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, zb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (valid)
    {
        load_source<PC>(Lc, C, row.node_site[c], row.node_buf[c], za);
        if (c < 2) load_source<PC>(Lc, C, row.node_site[c + 4], row.node_buf[c + 4], zb);
    }
    float acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 6; k++)
    {
        const float w = valid ? row.weight[c][k] : 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            const float z = __shfl_sync(0xffffffffu, k < 4 ? za[q] : zb[q], base + (k & 3));
            acc[q] += w * z;
        }
    }
    if (!valid) return;
    const int s = row.child_site[c];
    const float drho = Lf.snap[s], ux = Lf.snap[Lf.plane + s], uy = Lf.snap[2 * Lf.plane + s];
    float feq[9];
    equilibrium(drho, C.rho0 + drho, ux, uy, feq);
    const float rat = row.ratio[c];
    const int cb = row.child_buf[c];
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        acc[q] = feq[q] + rat * (acc[q] - feq[q]);
        C.ibuf[(size_t)q * C.n_buf + cb] = acc[q];
    }
    if ((row.plain_mask >> c) & 1) store_for_load(Lf, s % Lf.pitch, s / Lf.pitch, acc, pf);
}


// One level pair of one image in the interface exchange: the two levels'
// states (at their parities after the coarse step) and the pair's rows.
struct PairDesc
{
    LevelView Lf, Lc;
    Common C;
    const CoarseRowDev *coarse;
    const FineRowDev *fine;
    int pf, pc;  // parity of the next step of the fine / coarse level
    int kind;    // rows of this entry: 0 coarse, 1 fine
    int nrows;
};

constexpr int kMaxWaveDescs = 16;

struct WaveLaunch
{
    int ndesc;
    int start[kMaxWaveDescs + 1];
    PairDesc d[kMaxWaveDescs];
};

// Interface exchange wave: coarse rows of some pairs and fine rows of others
// (independent within a wave), 32 rows per block, 4 lanes per row.
__global__ void __launch_bounds__(128) k_wave(const __grid_constant__ WaveLaunch W)
{
    const int j = owner(W.start, W.ndesc, (int)blockIdx.x);
    const PairDesc &d = W.d[j];
    const int u = ((int)blockIdx.x - W.start[j]) * 128 + (int)threadIdx.x;
    const int r = u >> 2, k = u & 3;
    // lanes past the last row stay for the group shuffles
    const bool valid = r < d.nrows;
    const int rr = valid ? r : 0;
    if (d.kind == 0)
    {
        const CoarseRowDev &row = d.coarse[rr];
        if (d.pf) coarse_row<1>(d.Lf, d.Lc, d.C, row, k, valid, d.pc);
        else coarse_row<0>(d.Lf, d.Lc, d.C, row, k, valid, d.pc);
    }
    else
    {
        const FineRowDev &row = d.fine[rr];
        if (d.pc) fine_child<1>(d.Lf, d.Lc, d.C, row, k, valid, d.pf);
        else fine_child<0>(d.Lf, d.Lc, d.C, row, k, valid, d.pf);
    }
}

// ---- persistent step: one launch runs whole coarse steps of a group of
// images.  The work is a list of units (one block of 256 threads each) in claim
// order: 8 x tiles_per_warp tiles of 8x4 plain and light cells, 256 special
// records with walls, or 64 interface rows.  Units are grouped in segments,
// and the segments of one image form stages: the phases of its coarse step,
// then its interface waves.  A stage starts only when the image's previous
// stage is complete (the level substeps and the exchange that the phase engine
// orders by stream order), which a block learns from that stage's completion
// counter.  Blocks claim units with one atomic counter; every segment waits
// only on units earlier in claim order, so the unit with the lowest unfinished
// index can always run and the launch never deadlocks, whatever its grid size.
// Stages of different images interleave in the claim order, so while one image
// waits on its last units another image's work fills the GPU.
struct PersistSeg
{
    int kind;        // 0 plain8 tiles, 1 special records, 2 coarse rows, 3 fine rows
    int desc;        // StepDesc (kinds 0, 1) or PairDesc (2, 3) index
    int unit0;       // first unit of the segment in claim order
    int nunits;
    int wait_ctr;    // counter that must reach wait_target first (-1: none)
    unsigned wait_target;
    int done_ctr;    // counter each finished unit increments
    int pad;
};

constexpr int kPersistThreads = 256;
constexpr int kPersistRecords = kPersistThreads; // special records per unit
constexpr int kPersistRows = kPersistThreads / 4; // interface rows per unit (4 lanes each)
constexpr unsigned kErrDepTimeout = 2u;
// polls of a stage counter before a block gives up (an L2 round trip and a
// 64 ns sleep each: about a second); a normal wait takes microseconds
constexpr uint32_t kDepPolls = 1u << 22;

struct PersistLaunch
{
    const PersistSeg *segs;
    const StepDesc *sd;
    const PairDesc *pd;
    unsigned int *sync;   // [0] claim counter, [1 + c] stage counter c; zero at launch
    unsigned int *err;    // device error word
    int nseg, total_units;
    int tiles_per_warp;   // 8x4 tiles each warp of a plain-cell unit steps
};

__device__ __forceinline__ bool wait_counter(const unsigned int *c, unsigned int target)
{
    for (uint32_t i = 0; i < kDepPolls; i++)
    {
        unsigned int v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(c) : "memory");
        if (v >= target) return true;
        __nanosleep(64);
    }
    return false;
}

// Stage-counter update with release semantics: after the block barrier, every
// thread's stores of the unit are ordered before it (cumulativity).
__device__ __forceinline__ void add_release(unsigned int *c, unsigned int v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(c), "r"(v) : "memory");
}

// The descriptor of a segment, staged in shared memory once per segment (the
// array is read-only during the launch, so it takes the read-only path).
template <typename T> __device__ __forceinline__ void stage_desc(T *dst, const T *src)
{
    static_assert(sizeof(T) % 4 == 0, "descriptor size");
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    for (int i = (int)threadIdx.x; i < (int)(sizeof(T) / 4); i += (int)blockDim.x) d[i] = __ldg(&s[i]);
}

// MINB: blocks per SM the register budget is sized for (more blocks, fewer
// registers: the special-record and interface paths then spill a little; 5
// blocks of 48 registers measured best).
template <int MINB>
__global__ void __launch_bounds__(kPersistThreads, MINB) k_step_persistent(const __grid_constant__ PersistLaunch P)
{
    __shared__ union
    {
        StepDesc sd;
        PairDesc pd;
    } s_desc;
    __shared__ int s_unit, s_seg, s_next;
    int seg_cache = 0;        // thread 0: segment of the last claim (claims only grow)
    int ok_ctr = -1;          // thread 0: a counter already seen complete by this block
    unsigned ok_target = 0u;
    int staged = -1;          // segment whose descriptor is in shared memory
    if (threadIdx.x == 0) s_next = (int)atomicAdd(P.sync, 1u);
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            const int u = s_next;
            int seg = -1;
            if (u < P.total_units)
            {
                while (seg_cache + 1 < P.nseg && __ldg(&P.segs[seg_cache + 1].unit0) <= u) seg_cache++;
                seg = seg_cache;
                const int wc = __ldg(&P.segs[seg].wait_ctr);
                const unsigned wt = __ldg(&P.segs[seg].wait_target);
                if (wc >= 0 && !(wc == ok_ctr && wt <= ok_target))
                {
                    if (wait_counter(P.sync + 1 + wc, wt))
                    {
                        ok_ctr = wc;
                        ok_target = wt;
                    }
                    else
                    {
                        // an earlier unit never finished: stop (its waiters stop too)
                        atomicOr(P.err, kErrDepTimeout);
                        seg = -1;
                    }
                }
                // the next claim is in flight while this unit runs
                if (seg >= 0) s_next = (int)atomicAdd(P.sync, 1u);
            }
            s_unit = u;
            s_seg = seg;
        }
        __syncthreads();
        const int u = s_unit, seg = s_seg;
        if (seg < 0) break;
        const int kind = __ldg(&P.segs[seg].kind), desc = __ldg(&P.segs[seg].desc);
        const int k = u - __ldg(&P.segs[seg].unit0);
        if (seg != staged)
        {
            if (kind < 2) stage_desc(&s_desc.sd, &P.sd[desc]);
            else stage_desc(&s_desc.pd, &P.pd[desc]);
            staged = seg;
            __syncthreads();
        }
        double r_diff = 0.0, r_norm = 0.0;
        if (kind == 0)
        {
            const StepDesc &d = s_desc.sd;
            const int t0 = (k * 8 + (int)(threadIdx.x >> 5)) * P.tiles_per_warp;
#pragma unroll 1
            for (int j = 0; j < P.tiles_per_warp; j++)
            {
                const int t = t0 + j;
                if (t < d.L.ntiles8)
                {
                    if (d.o.parity) plain_tile8<1, false>(d.L, d.C, d.o, t, 0, 0, r_diff, r_norm);
                    else plain_tile8<0, false>(d.L, d.C, d.o, t, 0, 0, r_diff, r_norm);
                }
            }
        }
        else if (kind == 1)
        {
            const StepDesc &d = s_desc.sd;
            const int i = k * kPersistRecords + (int)threadIdx.x;
            if (i < d.spec_count)
            {
                if (d.o.parity) special_cell<1>(d.L, d.C, d.o, d.spec_begin + i, 0, 0, r_diff, r_norm);
                else special_cell<0>(d.L, d.C, d.o, d.spec_begin + i, 0, 0, r_diff, r_norm);
            }
        }
        else
        {
            // 4 lanes per row, as k_wave
            const PairDesc &d = s_desc.pd;
            const int v = k * kPersistThreads + (int)threadIdx.x;
            const int r = v >> 2, c = v & 3;
            const bool valid = r < d.nrows;
            const int rr = valid ? r : 0;
            if (kind == 2)
            {
                const CoarseRowDev &row = d.coarse[rr];
                if (d.pf) coarse_row<1>(d.Lf, d.Lc, d.C, row, c, valid, d.pc);
                else coarse_row<0>(d.Lf, d.Lc, d.C, row, c, valid, d.pc);
            }
            else
            {
                const FineRowDev &row = d.fine[rr];
                if (d.pc) fine_child<1>(d.Lf, d.Lc, d.C, row, c, valid, d.pf);
                else fine_child<0>(d.Lf, d.Lc, d.C, row, c, valid, d.pf);
            }
        }
        // the unit's stores, then its count (release): a waiter's acquire load
        // of the counter then sees them
        __syncthreads();
        if (threadIdx.x == 0) add_release(P.sync + 1 + __ldg(&P.segs[seg].done_ctr), 1u);
    }
}

// ---- the adsorption step as one cooperative launch over many steps.  Each
// step is the two passes of k_ads_psi / k_ads_psi_special and k_ads_step /
// k_ads_step_special over the same units (32x8 tiles, then runs of 256 special
// records), walked by a grid that is resident as a whole (cooperative launch);
// a grid barrier closes each pass.  The per-cell arithmetic is the same code,
// so the states are bit-identical to the launch-per-pass engine.
struct AdsPersist
{
    LevelView L;
    Common C;
    int64_t spec_begin;
    int spec_count, ntiles;
    int nsteps, parity0, direct0;
    int slot0, ring;        // residual of step k in slot (slot0 + k) mod ring
    int psi_diff, step_diff; // the residual terms of pass 1 (density change) / pass 2 (|u|)
    unsigned int *bar;      // arrivals at the grid barriers; zero at launch
};

// Grid barrier `target` = (barriers passed) x gridDim.x: every block adds one
// arrival with release semantics after its block barrier, then waits (bounded)
// for all of them; a wait that runs out sets the error word and the block stops.
__device__ __forceinline__ bool grid_barrier(unsigned int *bar, unsigned int target, unsigned int *err)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        add_release(bar, 1u);
        const bool ok = wait_counter(bar, target);
        if (!ok) atomicOr(err, kErrDepTimeout);
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    return s_ok != 0;
}

constexpr int kAdsRecords = 256; // special records per unit of k_ads_persistent

__global__ void __launch_bounds__(256) k_ads_persistent(const __grid_constant__ AdsPersist A)
{
    const int units = A.ntiles + (A.spec_count + kAdsRecords - 1) / kAdsRecords;
    unsigned int target = 0;
    for (int k = 0; k < A.nsteps; k++)
    {
        StepOpt o{};
        o.parity = (A.parity0 + k) & 1;
        o.direct = k == 0 ? A.direct0 : 0;
        o.red_slot = ((A.slot0 + k) % A.ring) * 4;
        o.snap_store = 1;
        StepOpt o1 = o, o2 = o;
        o1.diff = A.psi_diff;
        o2.diff = A.step_diff;
        for (int u = (int)blockIdx.x; u < units; u += (int)gridDim.x)
        {
            float rmax = 0.0f;
            if (u < A.ntiles) rmax = o.parity ? ads_psi_tile<1>(A.L, A.C, o1, u) : ads_psi_tile<0>(A.L, A.C, o1, u);
            else
            {
                const int i = (u - A.ntiles) * kAdsRecords + (int)threadIdx.x;
                if (i < A.spec_count)
                    rmax = o.parity ? ads_psi_record<1>(A.L, A.C, o1, A.spec_begin + i)
                                    : ads_psi_record<0>(A.L, A.C, o1, A.spec_begin + i);
            }
            if (o1.diff) block_max(rmax, A.C.red + o1.red_slot);
        }
        target += gridDim.x;
        if (!grid_barrier(A.bar, target, A.C.err)) return;
        for (int u = (int)blockIdx.x; u < units; u += (int)gridDim.x)
        {
            double r_diff = 0.0, r_norm = 0.0;
            if (u < A.ntiles)
            {
                if (o.parity) ads_step_tile<1>(A.L, A.C, o2, u, r_diff, r_norm);
                else ads_step_tile<0>(A.L, A.C, o2, u, r_diff, r_norm);
            }
            else
            {
                const int i = (u - A.ntiles) * kAdsRecords + (int)threadIdx.x;
                if (i < A.spec_count)
                {
                    if (o.parity) ads_step_record<1>(A.L, A.C, o2, A.spec_begin + i, r_diff, r_norm);
                    else ads_step_record<0>(A.L, A.C, o2, A.spec_begin + i, r_diff, r_norm);
                }
            }
            if (o2.diff) block_add2(r_diff, r_norm, A.C.red + o2.red_slot);
        }
        target += gridDim.x;
        if (!grid_barrier(A.bar, target, A.C.err)) return;
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
// Restart: the populations f (FP64, 9 per cell in cell order) become the state
// in the slots the first step reads directly, as after k_set_equilibrium; the
// residual side arrays take the moments of f with the FP32 arithmetic of a step.
__global__ void k_set_distributions(AllLevels A, Common C, const int32_t *cell_level, const int32_t *cell_site,
                                    int64_t n, const double *f)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int l = cell_level[c] - 1;
    const LevelView &L = A.lv[l];
    const int s = cell_site[c];
    float df[9];
    for (int q = 0; q < 9; q++)
    {
        df[q] = (float)(f[c * 9 + q] - d2q9::w(q) * (double)C.rho0);
        L.f[(size_t)q * L.plane + s] = df[q];
    }
    float drho, rho, ux, uy;
    macro(df, C.rho0, L.fshift, 0.0f, drho, rho, ux, uy);
    if (L.unorm) L.unorm[s] = sqrtf(ux * ux + uy * uy);
    if (L.rho_prev)
    {
        float sum = 0.0f;
        for (int q = 0; q < 9; q++) sum += df[q];
        L.rho_prev[s] = C.rho0 + sum;
    }
    if (L.snap)
    {
        L.snap[s] = drho;
        L.snap[L.plane + s] = ux;
        L.snap[2 * L.plane + s] = uy;
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
