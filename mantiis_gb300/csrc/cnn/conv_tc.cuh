// 3x3 convolution as an implicit GEMM on the fifth-generation tensor cores
// (tcgen05, sm_103a): one CTA of 128 threads computes 128 consecutive pixels
// of one image for up to 256 output channels.  Per chunk of 16 input channels
// the CTA gathers the 128 x 144 patch matrix A (pixel x (channel, tap)) into
// shared memory and the weights B (output channel x (channel, tap)); one
// thread issues the MMAs into a 128 x N FP32 accumulator in tensor memory.
// The activations are FP32: each one is split into a BF16 high part and a BF16
// remainder, and both are multiplied by the BF16 weights (two MMAs per K step),
// so the products carry about 16 bits of the activation's mantissa and the sum
// stays within FP32 rounding of the CUDA-core result.  Operands are staged in
// the no-swizzle K-major layout of 8 x 16-byte core matrices.  Every wait is
// bounded; a wait that runs out sets the error word and the CTA frees its
// tensor memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace cnn_tc
{
constexpr int kM = 128;              // pixels per CTA = accumulator lanes
constexpr int kCC = 16;              // input channels per K chunk
constexpr int kKK = kCC * 9;         // K per chunk: 144 = 9 MMA steps of 16
constexpr int kNMax = 256;           // output channels per CTA
constexpr uint32_t kPolls = 1u << 24; // polls of the MMA barrier before giving up

constexpr uint32_t kABytes = kM * kKK * 2;                  // one BF16 patch matrix
constexpr uint32_t kBBytesMax = kNMax * kKK * 2;            // the weight matrix
constexpr uint32_t kSmemBytes = 2 * kABytes + kBBytesMax + 64; // A hi, A lo, B, barrier, TMEM address

__device__ unsigned int g_tc_error; // set when a wait ran out

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row r, k) in a K-major no-swizzle operand of `rows`
// rows: core matrix (r / 8, k / 8) of 8 rows x 16 bytes, K-adjacent core
// matrices rows / 8 * 128 bytes apart, row-adjacent ones 128 bytes apart
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int rows)
{
    return (uint32_t)(((k >> 3) * (rows >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (between core matrices along K), stride byte offset (between core
// matrices along M / N), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N / 8 and M / 16
__host__ __device__ constexpr uint32_t instr_desc(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}

__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity, uint32_t polls)
{
    for (uint32_t i = 0; i < polls; i++)
        if (bar_try_wait(bar, parity)) return true;
    return false;
}

// 16 accumulator columns of this thread's lane (warp w reads lanes 32w .. 32w + 31)
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint16_t bf16_bits(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }

// 8 BF16 values packed for one 16-byte store (a core-matrix row)
__device__ __forceinline__ uint4 pack8(const uint16_t v[8])
{
    uint4 r;
    r.x = (uint32_t)v[0] | ((uint32_t)v[1] << 16);
    r.y = (uint32_t)v[2] | ((uint32_t)v[3] << 16);
    r.z = (uint32_t)v[4] | ((uint32_t)v[5] << 16);
    r.w = (uint32_t)v[6] | ((uint32_t)v[7] << 16);
    return r;
}

constexpr int kThreads = 256; // two threads per pixel row when staging A

// y[co] = b[co] + sum_ci sum_k w[co][ci][k] x[ci](p + offset(k)), as k_conv3x3;
// TRANSPOSE: the data gradient (w[ci][co][8 - k], channels swapped, taps
// flipped).  grid = (ceil(h wd / 128), ceil(cout / ntile), n), 256 threads,
// kSmemBytes of dynamic shared memory; ntile (a multiple of 16, at most 256)
// output channels per CTA.  Staging: the two threads of a pixel row each build
// 9 core-matrix rows (72 of the chunk's 144 K values) and store each with one
// 16-byte store per operand.
template <bool TRANSPOSE>
__global__ void __launch_bounds__(kThreads, 1) k_conv3x3_tc(const float *__restrict__ x, const uint16_t *__restrict__ w,
                                                            const float *__restrict__ b, float *__restrict__ y, int cin,
                                                            int cout, int h, int wd, int relu, int ntile)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *a_hi = smem, *a_lo = smem + kABytes, *bmat = smem + 2 * kABytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * kABytes + kBBytesMax);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 2 * kABytes + kBBytesMax + 16);

    const int tid = (int)threadIdx.x, warp = tid >> 5;
    const int row = tid & (kM - 1), half = tid >> 7;
    const int hw = h * wd;
    const int p0 = (int)blockIdx.x * kM;
    const int co0 = (int)blockIdx.y * ntile;
    const int n_img = (int)blockIdx.z;
    const int nco = min(ntile, cout - co0);
    const int N = (nco + 15) & ~15;                 // MMA N: a multiple of 16
    uint32_t ncols = 32;                            // tensor-memory columns: a power of 2 >= 32
    while ((int)ncols < N) ncols <<= 1;

    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const int p = p0 + row; // this thread's pixel (row of A)
    const int py = p / wd, px = p - py * wd;
    const bool pin = p < hw;
    const float *xn = x + (size_t)n_img * cin * hw;
    // the 9 taps of this pixel: offsets and validity
    int toff[9];
    bool tok[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
    {
        const int yy = py + k / 3 - 1, xx = px + k % 3 - 1;
        tok[k] = pin && yy >= 0 && yy < h && xx >= 0 && xx < wd;
        toff[k] = tok[k] ? yy * wd + xx : 0;
    }
    const uint32_t idesc = instr_desc(kM, N);
    const uint32_t a_hi_u = smem_u32(a_hi), a_lo_u = smem_u32(a_lo), b_u = smem_u32(bmat);
    const uint32_t lbo_a = (kM / 8) * 128, lbo_b = (uint32_t)(N / 8) * 128;
    bool ok = true;
    int chunk = 0;
    for (int ci0 = 0; ci0 < cin; ci0 += kCC, chunk++)
    {
        // A: this thread's half of its row, 9 core-matrix rows of 8 K values
#pragma unroll 1
        for (int g = half * 9; g < half * 9 + 9; g++)
        {
            uint16_t hv[8], lv[8];
#pragma unroll
            for (int e = 0; e < 8; e++)
            {
                const int kk = g * 8 + e, c = kk / 9, k = kk - c * 9;
                const int ci = ci0 + c;
                const float v = (ci < cin && tok[k]) ? __ldg(&xn[(size_t)ci * hw + toff[k]]) : 0.f;
                hv[e] = bf16_bits(v);
                lv[e] = bf16_bits(v - __bfloat162float(__ushort_as_bfloat16(hv[e])));
            }
            const uint32_t off = kmajor_offset(row, g * 8, kM);
            *reinterpret_cast<uint4 *>(a_hi + off) = pack8(hv);
            *reinterpret_cast<uint4 *>(a_lo + off) = pack8(lv);
        }
        // B: N rows (output channels) x 144, one core-matrix row (8 K values) per item
        for (int i = tid; i < N * (kKK / 8); i += kThreads)
        {
            const int nrow = i / (kKK / 8), g = i - nrow * (kKK / 8);
            const int gco = co0 + nrow;
            uint16_t v[8];
#pragma unroll
            for (int e = 0; e < 8; e++)
            {
                const int kk = g * 8 + e, c = kk / 9, k = kk - c * 9;
                const int gci = ci0 + c;
                v[e] = 0;
                if (nrow < nco && gci < cin)
                    v[e] = TRANSPOSE ? __ldg(&w[((size_t)gci * cout + gco) * 9 + (8 - k)])
                                     : __ldg(&w[((size_t)gco * cin + gci) * 9 + k]);
            }
            *reinterpret_cast<uint4 *>(bmat + kmajor_offset(nrow, g * 8, N)) = pack8(v);
        }
        // the generic-proxy stores become visible to the tensor cores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0)
        {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
            for (int s = 0; s < kKK / 16; s++)
            {
                // K step s covers core-matrix columns 2s and 2s + 1
                const uint64_t ad_hi = smem_desc(a_hi_u + (uint32_t)(2 * s) * lbo_a, lbo_a, 128);
                const uint64_t ad_lo = smem_desc(a_lo_u + (uint32_t)(2 * s) * lbo_a, lbo_a, 128);
                const uint64_t bd = smem_desc(b_u + (uint32_t)(2 * s) * lbo_b, lbo_b, 128);
                mma_bf16(tmem, ad_hi, bd, idesc, (chunk > 0 || s > 0) ? 1 : 0);
                mma_bf16(tmem, ad_lo, bd, idesc, 1);
            }
            mma_commit(bar);
        }
        // the operands may be overwritten once the MMAs have read them
        if (!bar_wait(bar, (uint32_t)(chunk & 1), kPolls))
        {
            atomicOr(&g_tc_error, 1u);
            ok = false;
        }
        ok = __syncthreads_and(ok);
        if (!ok) break;
    }
    if (ok && warp < 4)
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // accumulator row tid = pixel p; warp w reads lanes 32w .. 32w + 31
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        float *yn = y + (size_t)n_img * cout * hw;
        for (int c0 = 0; c0 < N; c0 += 16)
        {
            float v[16];
            tmem_load16(lane_addr + (uint32_t)c0, v);
            if (!pin) continue;
#pragma unroll
            for (int j = 0; j < 16; j++)
            {
                const int co = c0 + j;
                if (co >= nco) break;
                float o = v[j] + (b ? b[co0 + co] : 0.f);
                if (relu) o = fmaxf(o, 0.f);
                yn[(size_t)(co0 + co) * hw + p] = o;
            }
        }
    }
    else if (!ok)
    {
        // let MMAs still in flight finish before the tensor memory goes
        bar_wait(bar, (uint32_t)(chunk & 1), 1024u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// ---- weight gradient: dw[co][ci][k] += sum over pixels of dy[co](p) x[ci](p +
// offset(k)), a GEMM with M = output channels (128 per CTA), N = 16 input
// channels x 9 taps = 144 columns, K = pixels.  Each CTA takes one slice of
// the batch's pixels (split K) and adds its 128 x 144 partial sums to dw with
// atomics.  Both operands are FP32 here, so three MMAs per K step (dy_hi x_hi,
// dy_hi x_lo, dy_lo x_hi) keep the products to about 16 bits of mantissa.
constexpr int kWN = kCC * 9;                 // 144 columns
constexpr int kWK = 64;                      // pixels per K chunk
constexpr uint32_t kWABytes = kM * kWK * 2;  // 16 KB
constexpr uint32_t kWBBytes = kWN * kWK * 2; // 18 KB
constexpr uint32_t kWSmemBytes = 2 * kWABytes + 2 * kWBBytes + 64;

// grid = (ceil(cout / 128), ceil(cin / 16), slices), 256 threads, kWSmemBytes
// of dynamic shared memory; each slice covers `slice` consecutive pixels of the
// flattened batch (n h wd)
__global__ void __launch_bounds__(kThreads, 1) k_conv3x3_wgrad_tc(const float *__restrict__ x, const float *__restrict__ dy,
                                                             float *__restrict__ dw, int n, int cin, int cout, int h,
                                                             int wd, int slice)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *a_hi = smem, *a_lo = smem + kWABytes;
    unsigned char *b_hi = smem + 2 * kWABytes, *b_lo = smem + 2 * kWABytes + kWBBytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * kWABytes + 2 * kWBBytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 2 * kWABytes + 2 * kWBBytes + 16);

    const int tid = (int)threadIdx.x, warp = tid >> 5;
    const int hw = h * wd;
    const int64_t total = (int64_t)n * hw;
    const int co0 = (int)blockIdx.x * kM, ci0 = (int)blockIdx.y * kCC;
    const int64_t g0 = (int64_t)blockIdx.z * slice;
    const int64_t g1 = min(total, g0 + slice);
    const uint32_t ncols = 256;

    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const uint32_t idesc = instr_desc(kM, kWN);
    const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo), bh = smem_u32(b_hi), bl = smem_u32(b_lo);
    const uint32_t lbo_a = (kM / 8) * 128, lbo_b = (kWN / 8) * 128;
    bool ok = true;
    int chunk = 0;
    for (int64_t k0 = g0; k0 < g1; k0 += kWK, chunk++)
    {
        // A: dy of 128 output channels x 64 pixels, one core-matrix row (8
        // consecutive pixels of one channel) per item
        for (int i = tid; i < kM * (kWK / 8); i += kThreads)
        {
            const int r = i / (kWK / 8), g = i - r * (kWK / 8);
            const int co = co0 + r;
            uint16_t hv[8], lv[8];
#pragma unroll
            for (int e = 0; e < 8; e++)
            {
                const int64_t gp = k0 + g * 8 + e;
                float v = 0.f;
                if (gp < g1 && co < cout)
                {
                    const int64_t img = gp / hw, pix = gp - img * hw;
                    v = __ldg(&dy[(img * cout + co) * hw + pix]);
                }
                hv[e] = bf16_bits(v);
                lv[e] = bf16_bits(v - __bfloat162float(__ushort_as_bfloat16(hv[e])));
            }
            const uint32_t off = kmajor_offset(r, g * 8, kM);
            *reinterpret_cast<uint4 *>(a_hi + off) = pack8(hv);
            *reinterpret_cast<uint4 *>(a_lo + off) = pack8(lv);
        }
        // B: x of 16 input channels x 9 taps (shifted) x 64 pixels, same items
        for (int i = tid; i < kWN * (kWK / 8); i += kThreads)
        {
            const int r = i / (kWK / 8), g = i - r * (kWK / 8);
            const int c = r / 9, k = r - c * 9;
            const int ci = ci0 + c;
            uint16_t hv[8], lv[8];
#pragma unroll
            for (int e = 0; e < 8; e++)
            {
                const int64_t gp = k0 + g * 8 + e;
                float v = 0.f;
                if (gp < g1 && ci < cin)
                {
                    const int64_t img = gp / hw, pix = gp - img * hw;
                    const int py = (int)(pix / wd), px = (int)(pix - (int64_t)py * wd);
                    const int yy = py + k / 3 - 1, xx = px + k % 3 - 1;
                    if (yy >= 0 && yy < h && xx >= 0 && xx < wd)
                        v = __ldg(&x[(img * cin + ci) * hw + (int64_t)yy * wd + xx]);
                }
                hv[e] = bf16_bits(v);
                lv[e] = bf16_bits(v - __bfloat162float(__ushort_as_bfloat16(hv[e])));
            }
            const uint32_t off = kmajor_offset(r, g * 8, kWN);
            *reinterpret_cast<uint4 *>(b_hi + off) = pack8(hv);
            *reinterpret_cast<uint4 *>(b_lo + off) = pack8(lv);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0)
        {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
            for (int s = 0; s < kWK / 16; s++)
            {
                const uint32_t da = (uint32_t)(2 * s) * lbo_a, db = (uint32_t)(2 * s) * lbo_b;
                const uint64_t dah = smem_desc(ah + da, lbo_a, 128), dal = smem_desc(al + da, lbo_a, 128);
                const uint64_t dbh = smem_desc(bh + db, lbo_b, 128), dbl = smem_desc(bl + db, lbo_b, 128);
                mma_bf16(tmem, dah, dbh, idesc, (chunk > 0 || s > 0) ? 1 : 0);
                mma_bf16(tmem, dah, dbl, idesc, 1);
                mma_bf16(tmem, dal, dbh, idesc, 1);
            }
            mma_commit(bar);
        }
        if (!bar_wait(bar, (uint32_t)(chunk & 1), kPolls))
        {
            atomicOr(&g_tc_error, 1u);
            ok = false;
        }
        ok = __syncthreads_and(ok);
        if (!ok) break;
    }
    if (ok && chunk > 0 && warp < 4)
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        const int co = co0 + tid;
        for (int c0 = 0; c0 < kWN; c0 += 16)
        {
            float v[16];
            tmem_load16(lane_addr + (uint32_t)c0, v);
            if (co >= cout) continue;
#pragma unroll
            for (int j = 0; j < 16; j++)
            {
                const int col = c0 + j, c = col / 9;
                if (ci0 + c < cin) atomicAdd(&dw[((size_t)co * cin + ci0) * 9 + col], v[j]);
            }
        }
    }
    else if (!ok)
    {
        bar_wait(bar, (uint32_t)(chunk & 1), 1024u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// db[co] += sum over the batch's pixels of dy[co]: one block per channel
__global__ void __launch_bounds__(256) k_bias_grad(const float *__restrict__ dy, float *__restrict__ db, int n, int cout,
                                                   int hw)
{
    const int co = (int)blockIdx.x;
    float s = 0.f;
    for (int img = 0; img < n; img++)
        for (int p = (int)threadIdx.x; p < hw; p += (int)blockDim.x) s += dy[((size_t)img * cout + co) * hw + p];
    __shared__ float red[8];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        float t = 0.f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
        atomicAdd(&db[co], t);
    }
}
} // namespace cnn_tc
