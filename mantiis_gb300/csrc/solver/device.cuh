// Device-side data views and per-cell building blocks of the lattice
// Boltzmann step (sm_103a).  Shared by the step, interface and output kernels.
//
// Storage: df_q = f_q - w_q rho0 (FP32) in 9 SoA planes per level, AA pattern:
//   even step (parity 0): cell x reads slot (x, q), writes f*_q to (x, opp q)
//   odd step  (parity 1): cell x reads slot (x - c_q, opp q), writes f*_q to (x + c_q, q)
// so after either step the value streamed into f_q(x) sits where the next
// step looks for it.  A wall link q of cell x leaves f*_q(x) in its natural
// slot, which belongs to an inactive site, and the reflection is applied when x
// reads its populations in the next step.  Wall links to an active neighbour
// (the table's fluid-to-fluid "wall" links) keep the value in a side buffer.
#pragma once
#include <cstdint>

#include "../boundary_tables.h"
#include "../d2q9.h"
#include "layout.hpp"

namespace mantiis
{
namespace dev
{
// boundary tables in constant memory: specular target per (type, direction),
// and per type the directions with c.n > 0 and c.n < 0 (MDBB)
// specular targets per boundary type, in global memory: lanes of a warp index it
// with different types, which the constant cache would serialize
__device__ unsigned char c_icsr[MANTIIS_N_BND_TYPES * 9];
__constant__ unsigned short c_npos[MANTIIS_N_BND_TYPES];
__constant__ unsigned short c_nneg[MANTIIS_N_BND_TYPES];
struct LevelView
{
    float *f;             // 9 * plane
    const float *omega;   // per site 1/tau_s: 0 inactive, >0 plain, <0 special
    const uint32_t *spec; // per site special index
    const float *tau2;    // per site second relaxation time (plain MRT: tau_d), may be null
    float *snap;          // 3 * plane: coarse-step-start (drho, ux, uy), may be null
    float *unorm;         // per site |u| of the last stored state, may be null
    float *psi;           // per site pseudopotential (adsorption), may be null
    float *rho_prev;      // per site density at the start of the previous step (adsorption), may be null
    const int32_t *tiles; // active 32x8 tiles
    const uint32_t *tile_mask; // 8 row masks of plain cells per active tile
    const int32_t *tiles8;     // 8x4 tiles holding a plain or light cell
    const uint32_t *tile8_mask;// their plain and light cells (bit = 8 * row + column)
    const uint32_t *tile8_light;// their light cells (special only by missing arrivals / buffer status)
    int ntiles, tiles_x;
    int ntiles8;
    int W, H, pitch;
    int64_t plane;
    float fshift;         // F_body / 2 * 2^(l-1): u_x = j_x / rho + fshift / rho
    int level;
};

struct Common
{
    const SpecialRec *specials;
    const float *ktab;
    float *side;          // 2 * n_quirk (double-buffered by step parity)
    int64_t n_quirk;
    float *ibuf;          // 9 * n_buf, interpolated buffer-cell populations [q][b]
    int64_t n_buf;
    float rho0;           // reference density of the deviation storage
    float inlet_axis;     // w_1 rho_in - w_1 rho0: inlet/outlet axis population deviation
    float inlet_diag;     // w_2 rho_in - w_5 rho0: inlet/outlet diagonal deviation (the reference uses W[2])
    int wall;             // WallMode
    int collision;        // CollisionMode
    float fbody;
    // Shan-Chen (adsorption)
    int psi_form;         // 0: Peng-Robinson pseudopotential, 1: rho0 (1 - exp(-rho/rho0))
    float psi_rho0;       // rho0 of the exponential form
    float eos_a, eos_b, eos_T; // a_alpha_lu, b_lu, T_lu
    float g_ff, g_fs;
    int adsorption;       // Shan-Chen step (outputs come from the snapshot planes)
    int inlet_outlet;     // apply the adsorption inlet / outlet values (not in the coupling phase)
    double *red;          // reduction accumulators
    unsigned int *err;    // device error word
};

// per-launch step options
struct StepOpt
{
    int parity;        // 0 even, 1 odd
    int direct;        // state holds f itself (after initialisation): read own slots unmasked
    int first_sub;     // first substep of this level in the coarse step: buffers read the interpolation buffer
    int snap_store;    // store (drho, ux, uy) of the loaded state
    int snap_use;      // use the stored snapshot for the equilibrium (stale f_eq of the fine substeps)
    int diff;          // accumulate the residual terms of the loaded state (needs unorm)
    int store_u;       // store |u| of the loaded state
    int red_slot;      // accumulator base index
};

constexpr float kW0 = 4.0f / 9.0f, kW1 = 1.0f / 9.0f, kW2 = 1.0f / 36.0f;
__device__ __forceinline__ float wq(int q) { return q == 0 ? kW0 : (q < 5 ? kW1 : kW2); }

__device__ __forceinline__ int wrapx(int x, int W) { return x < 0 ? x + W : (x >= W ? x - W : x); }

// density deviation and velocity of a population set: u = j / rho + F / (2 rho) * 2^(l-1)
// (include/coreLB.hpp:1018-1054, 1069-1099); fx, fy are the level-scaled half forces
__device__ __forceinline__ void macro(const float df[9], float rho0, float fx, float fy, float &drho, float &rho,
                                      float &ux, float &uy)
{
    drho = ((df[0] + df[1]) + (df[2] + df[3])) + ((df[4] + df[5]) + (df[6] + df[7])) + df[8];
    rho = rho0 + drho;
    const float jx = (df[1] - df[3]) + (df[5] - df[6]) + (df[8] - df[7]);
    const float jy = (df[2] - df[4]) + (df[5] + df[6]) - (df[7] + df[8]);
    const float inv = 1.0f / rho;
    ux = (jx + fx) * inv;
    uy = (jy + fy) * inv;
}

// equilibrium deviation of direction q: w_q (rho - rho0) + w_q rho (3 cu + 4.5 cu^2 - 1.5 u^2)
__device__ __forceinline__ void equilibrium(float drho, float rho, float ux, float uy, float feq[9])
{
    const float usq = ux * ux + uy * uy;
    const float base = 1.5f * usq;
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        const float cu = (float)d2q9::cx(q) * ux + (float)d2q9::cy(q) * uy;
        feq[q] = wq(q) * drho + wq(q) * rho * (3.0f * cu + 4.5f * cu * cu - base);
    }
}

// Regularized MRT (include/coreLB.hpp:646-675, 744-792): the non-equilibrium
// part f - f_eq is projected on its second-order Hermite content
// Pi = sum c c (f - f_eq), then relaxed in moment space with
// diag(1, 1/1.1, 1/1.2, 1, 1/tau_q, 1, 1/tau_q, 1/tau_s, 1/tau_s).  The
// projection has only e = 3T, epsilon = -3T, p_xx = N, p_xy = Pxy non-zero
// (T = Pxx + Pyy, N = Pxx - Pyy), so M^-1 applied to the relaxed moments
// reduces to
//   f* = f_eq + k0 T                      (rest)
//   f* = f_eq + ka T +- (1 - omega) N / 4   (axes x / y)
//   f* = f_eq + kd T +- (1 - omega) Pxy / 4 (diagonals +- c_x c_y)
// with k0 = -2/3 + (3/1.1 + 2.5)/9, ka = 1/12 + 3/39.6 - 2.5/18,
// kd = 1/12 - 3/19.8 + 2.5/36 (the bulk moments relax at 1/1.1 and 1/1.2).
// Pi comes from the moments of f minus those of f_eq, rho (cs^2 I + u u).
__device__ __forceinline__ void collide_rmrt(const float df[9], const float feq[9], float drho_e, float rho_e, float ux,
                                             float uy, float omega, float out[9])
{
    constexpr float k0 = (float)(-2.0 / 3.0 + (3.0 / 1.1 + 2.5) / 9.0);
    constexpr float ka = (float)(1.0 / 12.0 + 3.0 / 39.6 - 2.5 / 18.0);
    constexpr float kd = (float)(1.0 / 12.0 - 3.0 / 19.8 + 2.5 / 36.0);
    const float sd = (df[5] + df[6]) + (df[7] + df[8]);
    const float sxx = (df[1] + df[3]) + sd;
    const float syy = (df[2] + df[4]) + sd;
    const float sxy = (df[5] - df[6]) + (df[7] - df[8]);
    const float d3 = drho_e * (1.0f / 3.0f);
    const float Pxx = sxx - (d3 + rho_e * ux * ux);
    const float Pyy = syy - (d3 + rho_e * uy * uy);
    const float Pxy = sxy - rho_e * ux * uy;
    const float T = Pxx + Pyy, N = Pxx - Pyy;
    const float g = 0.25f * (1.0f - omega);
    const float at = ka * T, gn = g * N, dt = kd * T, gp = g * Pxy;
    out[0] = feq[0] + k0 * T;
    out[1] = feq[1] + (at + gn);
    out[3] = feq[3] + (at + gn);
    out[2] = feq[2] + (at - gn);
    out[4] = feq[4] + (at - gn);
    out[5] = feq[5] + (dt + gp);
    out[7] = feq[7] + (dt + gp);
    out[6] = feq[6] + (dt - gp);
    out[8] = feq[8] + (dt - gp);
}

// Pseudopotential (include/coreLB.hpp:515-531): from the lattice Peng-Robinson
// pressure, psi = sqrt((p_EOS - rho/3) / (3 G_ff)), kept negative (unrooted)
// where the radicand is negative as the reference does; psi_form 1 is the
// exponential form rho_psi (1 - exp(-rho / rho_psi)).
__device__ __forceinline__ float pseudo_potential(float psi_form_exp, float rho_psi, float a, float b, float T,
                                                  float g_ff, float rho)
{
    if (psi_form_exp != 0.0f) return rho_psi * (1.0f - expf(-rho / rho_psi));
    const float md = rho; // molar density, Mw_lu = 1
    const float p = md * T / (1.0f - b * md) - a * md * md / (1.0f + 2.0f * b * md - b * b * md * md);
    const float acc = (p - rho * (1.0f / 3.0f)) / (3.0f * g_ff);
    return acc < 0.0f ? acc : sqrtf(acc);
}

// Moment matrix M and its inverse (include/globalParameters.hpp:154-175).
__device__ __forceinline__ void moments(const float v[9], float m[9])
{
    m[0] = v[0] + v[1] + v[2] + v[3] + v[4] + v[5] + v[6] + v[7] + v[8];
    m[1] = -4.f * v[0] - v[1] - v[2] - v[3] - v[4] + 2.f * (v[5] + v[6] + v[7] + v[8]);
    m[2] = 4.f * v[0] - 2.f * (v[1] + v[2] + v[3] + v[4]) + v[5] + v[6] + v[7] + v[8];
    m[3] = v[1] - v[3] + v[5] - v[6] - v[7] + v[8];
    m[4] = -2.f * v[1] + 2.f * v[3] + v[5] - v[6] - v[7] + v[8];
    m[5] = v[2] - v[4] + v[5] + v[6] - v[7] - v[8];
    m[6] = -2.f * v[2] + 2.f * v[4] + v[5] + v[6] - v[7] - v[8];
    m[7] = v[1] - v[2] + v[3] - v[4];
    m[8] = v[5] - v[6] + v[7] - v[8];
}
__device__ __forceinline__ void inv_moments(const float m[9], float v[9])
{
    const float a = m[0] * (1.f / 9.f);
    v[0] = a - m[1] * (1.f / 9.f) + m[2] * (1.f / 9.f);
    const float ax = a - m[1] * (1.f / 36.f) - m[2] * (1.f / 18.f);
    const float ad = a + m[1] * (1.f / 18.f) + m[2] * (1.f / 36.f);
    v[1] = ax + (m[3] - m[4]) * (1.f / 6.f) + m[7] * 0.25f;
    v[3] = ax - (m[3] - m[4]) * (1.f / 6.f) + m[7] * 0.25f;
    v[2] = ax + (m[5] - m[6]) * (1.f / 6.f) - m[7] * 0.25f;
    v[4] = ax - (m[5] - m[6]) * (1.f / 6.f) - m[7] * 0.25f;
    const float jx = m[3] * (1.f / 6.f) + m[4] * (1.f / 12.f);
    const float jy = m[5] * (1.f / 6.f) + m[6] * (1.f / 12.f);
    v[5] = ad + jx + jy + m[8] * 0.25f;
    v[6] = ad - jx + jy - m[8] * 0.25f;
    v[7] = ad - jx - jy + m[8] * 0.25f;
    v[8] = ad + jx - jy - m[8] * 0.25f;
}

// relaxation rates diag(1, 1/1.1, 1/1.2, 1/tau_d, 1/tau_q, 1/tau_d, 1/tau_q, 1/tau_s, 1/tau_s)
__device__ __forceinline__ void rates(float tau_s, float tau_d, float s[9])
{
    const float t = 2.0f * tau_s - 1.0f;
    const float tau_q = 0.5f + (3.0f + 3.14159265358979f * t * t * 0.9f) / (8.0f * t);
    s[0] = 1.0f;
    s[1] = 1.0f / 1.1f;
    s[2] = 1.0f / 1.2f;
    s[3] = s[5] = 1.0f / tau_d;
    s[4] = s[6] = 1.0f / tau_q;
    s[7] = s[8] = 1.0f / tau_s;
}

// Plain MRT (include/coreLB.hpp:694-742): f* = f - M^-1 R M (f - f_eq)
__device__ __forceinline__ void collide_mrt(const float df[9], const float feq[9], float tau_s, float tau_d, float out[9])
{
    float fn[9], m[9], s[9], dv[9];
#pragma unroll
    for (int q = 0; q < 9; q++) fn[q] = df[q] - feq[q];
    moments(fn, m);
    rates(tau_s, tau_d, s);
#pragma unroll
    for (int k = 0; k < 9; k++) m[k] *= s[k];
    inv_moments(m, dv);
#pragma unroll
    for (int q = 0; q < 9; q++) out[q] = df[q] - dv[q];
}

// Guo-type MRT source term (include/coreLB.hpp:568-630): f += M^-1 (I - R/2) M S,
// S_q = w_q [c.F / cs^2 + (u F) : (c c - cs^2 I) / cs^4] with the reference's
// pairing of the mixed terms (uF[2] with c_x c_y, uF[1] with c_y c_x).
__device__ __forceinline__ void add_source(float out[9], float ux, float uy, float Fx, float Fy, float tau_s, float tau_d)
{
    float S[9], m[9], s[9], dv[9];
    const float uFxx = ux * Fx, uFxy = ux * Fy, uFyx = uy * Fx, uFyy = uy * Fy;
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        const float cx = (float)d2q9::cx(q), cy = (float)d2q9::cy(q);
        const float cF = cx * Fx + cy * Fy;
        const float cc = uFxx * (cx * cx - (1.f / 3.f)) + uFyx * (cx * cy) + uFxy * (cy * cx) + uFyy * (cy * cy - (1.f / 3.f));
        S[q] = wq(q) * (cF * 3.0f + cc * 9.0f);
    }
    moments(S, m);
    rates(tau_s, tau_d, s);
#pragma unroll
    for (int k = 0; k < 9; k++) m[k] *= (1.0f - 0.5f * s[k]);
    inv_moments(m, dv);
#pragma unroll
    for (int q = 0; q < 9; q++) out[q] += dv[q];
}

__device__ __forceinline__ int64_t site_of(const LevelView &L, int x, int y) { return (int64_t)y * L.pitch + x; }

// raw slot reads of cell (x, y) at the given parity
template <int P> __device__ __forceinline__ void load_raw(const LevelView &L, int x, int y, float raw[9])
{
    if (P == 0)
    {
        const int64_t s = site_of(L, x, y);
#pragma unroll
        for (int q = 0; q < 9; q++) raw[q] = L.f[q * L.plane + s];
    }
    else
    {
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            const int xs = wrapx(x - d2q9::cx(q), L.W), ys = wrapx(y - d2q9::cy(q), L.H);
            raw[q] = L.f[d2q9::opp(q) * L.plane + site_of(L, xs, ys)];
        }
    }
}

// population load: through the read-only data path (NC: the slot is written by
// no other thread during the launch) or an ordinary load (the persistent step,
// where other blocks of the same launch wrote it in an earlier stage, which the
// reading warp has acquired)
template <bool NC> __device__ __forceinline__ float ldf(const float *p) { return NC ? __ldg(p) : *p; }

// same reads through the read-only data path (the slots read by a thread are
// written only by that thread in the same launch), or with NC = false through L2
template <int P, bool NC = true>
__device__ __forceinline__ void load_raw_ro(const LevelView &L, int x, int y, float raw[9], bool interior = false)
{
    if (P == 0)
    {
        const int64_t s = site_of(L, x, y);
#pragma unroll
        for (int q = 0; q < 9; q++) raw[q] = ldf<NC>(&L.f[q * L.plane + s]);
    }
    else if (interior)
    {
        // no neighbour wraps around the torus: plain offsets
        const int64_t s = site_of(L, x, y);
#pragma unroll
        for (int q = 0; q < 9; q++)
            raw[q] = ldf<NC>(&L.f[d2q9::opp(q) * L.plane + s - d2q9::cy(q) * (int64_t)L.pitch - d2q9::cx(q)]);
    }
    else
    {
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            const int xs = wrapx(x - d2q9::cx(q), L.W), ys = wrapx(y - d2q9::cy(q), L.H);
            raw[q] = ldf<NC>(&L.f[d2q9::opp(q) * L.plane + site_of(L, xs, ys)]);
        }
    }
}

template <int P>
__device__ __forceinline__ void store_post(const LevelView &L, int x, int y, const float fs[9], bool interior = false)
{
    if (P == 0)
    {
        const int64_t s = site_of(L, x, y);
#pragma unroll
        for (int q = 0; q < 9; q++) L.f[d2q9::opp(q) * L.plane + s] = fs[q];
    }
    else if (interior)
    {
        const int64_t s = site_of(L, x, y);
#pragma unroll
        for (int q = 0; q < 9; q++) L.f[q * L.plane + s + d2q9::cy(q) * (int64_t)L.pitch + d2q9::cx(q)] = fs[q];
    }
    else
    {
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            const int xd = wrapx(x + d2q9::cx(q), L.W), yd = wrapx(y + d2q9::cy(q), L.H);
            L.f[q * L.plane + site_of(L, xd, yd)] = fs[q];
        }
    }
}

// value of wall link q of cell (x, y) left by the previous step (parity 1-P)
template <int P> __device__ __forceinline__ float wall_slot(const LevelView &L, int x, int y, int q)
{
    if (P == 1) return L.f[d2q9::opp(q) * L.plane + site_of(L, x, y)];
    const int xd = wrapx(x + d2q9::cx(q), L.W), yd = wrapx(y + d2q9::cy(q), L.H);
    return L.f[q * L.plane + site_of(L, xd, yd)];
}

// Populations of a special cell after streaming and the wall rules:
//   stream (=) -> wall (SRBB +=, BB/MDBB =) -> x-periodic (=) -> inlet/outlet (=)
// (include/mantiisApp.hpp:239-265, include/coreLB.hpp:834-1009).  `raw` holds
// the slots the cell reads at parity P; `wall(q)` gives the value its wall
// link q left in the previous step.
template <int P, typename WallSlot>
__device__ __forceinline__ void special_rules(const Common &C, const SpecialRec &rec, const float raw[9], WallSlot wall_of,
                                              float df[9])
{
    const uint32_t arrive = rec.m0 & 0x1FFu, over = (rec.m0 >> 9) & 0x1FFu, wall = (rec.m0 >> 18) & 0x1FFu;
    const uint32_t quirk = rec.m1 & 0x1FFu, bnd = (rec.m1 >> 9) & 0xFFu, flags = (rec.m1 >> 17) & 0xFu;
    // every load first (wall values, quirk values, constant terms, specular
    // targets), so they are in flight together; then the arithmetic in the
    // reference's order
    const float *side_prev = C.side + (size_t)(P ^ 1) * C.n_quirk;
    float v[9], kq[9];
    int p2s[9];
#pragma unroll
    for (int q = 0; q < 9; q++)
    {
        v[q] = 0.0f;
        p2s[q] = d2q9::opp(q);
        if ((wall >> q) & 1u)
        {
            v[q] = ((quirk >> q) & 1u) ? side_prev[rec.quirk_base + __popc(quirk & ((1u << q) - 1u))] : wall_of(q);
            if (bnd != 0xFFu) p2s[q] = (int)__ldg(&c_icsr[bnd * 9 + q]);
        }
    }
    const bool has_k = (flags & SF_HAS_K) != 0;
    const float *k = C.ktab + (size_t)(has_k ? rec.k_row : 0) * 9;
#pragma unroll
    for (int q = 0; q < 9; q++) kq[q] = has_k ? __ldg(&k[q]) : 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++) df[q] = ((arrive >> q) & 1u) ? raw[q] : 0.0f;
    if (wall)
    {
        const float r = rec.r;
        // unrolled with fixed indices (the specular target is matched against
        // each population), so df stays in registers
#pragma unroll
        for (int q = 0; q < 9; q++)
        {
            if (!((wall >> q) & 1u)) continue;
            const int p1 = d2q9::opp(q);
            if (C.wall == WALL_SRBB)
            {
                const int p2 = p2s[q];
                if (!((over >> p1) & 1u)) df[p1] += r * v[q];
                const float rv = (((over >> p2) & 1u) ? 0.0f : (1.0f - r) * v[q]);
#pragma unroll
                for (int p = 0; p < 9; p++)
                    if (p == p2) df[p] += rv;
            }
            else if (!((over >> p1) & 1u))
                df[p1] = v[q];
        }
    }
    if (has_k)
    {
#pragma unroll
        for (int q = 0; q < 9; q++) df[q] += kq[q];
    }
    if ((flags & SF_INLET) && C.inlet_outlet)
    {
        df[1] = C.inlet_axis;
        df[5] = df[8] = C.inlet_diag;
    }
    if ((flags & SF_OUTLET) && C.inlet_outlet)
    {
        df[3] = C.inlet_axis;
        df[6] = df[7] = C.inlet_diag;
    }
}

template <int P>
__device__ __forceinline__ void load_special(const LevelView &L, const Common &C, const SpecialRec &rec, int x, int y,
                                             float df[9])
{
    float raw[9];
    load_raw<P>(L, x, y, raw);
    special_rules<P>(C, rec, raw, [&](int q) { return wall_slot<P>(L, x, y, q); }, df);
}
} // namespace dev
} // namespace mantiis
