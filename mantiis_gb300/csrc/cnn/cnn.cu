// Kernels of the warm-start encoder-decoder network (include/mantiis_cnn.h):
// 3x3 convolutions (forward, data gradient, weight gradient) with BF16
// weights and FP32 accumulation, pooling / upsampling / ReLU adjoints, the
// masked loss and the Adam update.  sm_103a.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../../include/mantiis_cnn.h"
#include "conv_tc.cuh"

namespace
{
constexpr int TS = 16;  // pixel tile side
constexpr int COB = 16; // output channels per block
constexpr int CIB = 16; // input channels per shared-memory chunk

__device__ __forceinline__ float bf(const uint16_t v) { return __bfloat162float(__ushort_as_bfloat16(v)); }

// y[co] = sum_ci sum_k w[co][ci][k] x[ci](p + offset(k)), offsets (kx - 1, ky - 1)
// with k = 3 ky + kx.  TRANSPOSE: the data gradient of such a convolution, i.e.
// the same with w[ci][co][8 - k] (channels swapped, kernel flipped); `cin` and
// `cout` are this convolution's own input / output channel counts.
template <bool TRANSPOSE>
__global__ void __launch_bounds__(256) k_conv3x3(const float *__restrict__ x, const uint16_t *__restrict__ w,
                                                 const float *__restrict__ b, float *__restrict__ y, int cin,
                                                 int cout, int h, int wd, int relu)
{
    __shared__ float sx[CIB][TS + 2][TS + 2];
    __shared__ float sw[COB][CIB][9];
    const int tiles_x = (wd + TS - 1) / TS;
    const int tx0 = ((int)blockIdx.x % tiles_x) * TS, ty0 = ((int)blockIdx.x / tiles_x) * TS;
    const int co0 = (int)blockIdx.y * COB;
    const int n = (int)blockIdx.z;
    const int lx = threadIdx.x % TS, ly = threadIdx.x / TS;
    const size_t plane = (size_t)h * wd;
    float acc[COB];
#pragma unroll
    for (int c = 0; c < COB; c++) acc[c] = 0.f;
    for (int ci0 = 0; ci0 < cin; ci0 += CIB)
    {
        for (int i = threadIdx.x; i < CIB * (TS + 2) * (TS + 2); i += blockDim.x)
        {
            const int c = i / ((TS + 2) * (TS + 2)), r = i % ((TS + 2) * (TS + 2));
            const int yy = r / (TS + 2), xx = r % (TS + 2);
            const int gy = ty0 + yy - 1, gx = tx0 + xx - 1, gc = ci0 + c;
            float v = 0.f;
            if (gc < cin && gy >= 0 && gy < h && gx >= 0 && gx < wd)
                v = x[((size_t)n * cin + gc) * plane + (size_t)gy * wd + gx];
            sx[c][yy][xx] = v;
        }
        for (int i = threadIdx.x; i < COB * CIB * 9; i += blockDim.x)
        {
            const int co = i / (CIB * 9), r = i % (CIB * 9), c = r / 9, k = r % 9;
            const int gco = co0 + co, gci = ci0 + c;
            float v = 0.f;
            if (gco < cout && gci < cin)
                v = TRANSPOSE ? bf(w[((size_t)gci * cout + gco) * 9 + (8 - k)]) : bf(w[((size_t)gco * cin + gci) * 9 + k]);
            sw[co][c][k] = v;
        }
        __syncthreads();
        const int cmax = min(CIB, cin - ci0);
        for (int c = 0; c < cmax; c++)
        {
#pragma unroll
            for (int k = 0; k < 9; k++)
            {
                const float xv = sx[c][ly + k / 3][lx + k % 3];
#pragma unroll
                for (int co = 0; co < COB; co++) acc[co] = fmaf(sw[co][c][k], xv, acc[co]);
            }
        }
        __syncthreads();
    }
    const int px = tx0 + lx, py = ty0 + ly;
    if (px >= wd || py >= h) return;
#pragma unroll
    for (int co = 0; co < COB; co++)
    {
        const int gco = co0 + co;
        if (gco >= cout) break;
        float v = acc[co] + (b ? b[gco] : 0.f);
        if (relu) v = fmaxf(v, 0.f);
        y[((size_t)n * cout + gco) * plane + (size_t)py * wd + px] = v;
    }
}

// dw[co][ci][k] += sum_pixels dy[co](p) x[ci](p + offset(k)); db[co] += sum dy[co]
__global__ void __launch_bounds__(256) k_conv3x3_bw(const float *__restrict__ x, const float *__restrict__ dy,
                                                    float *__restrict__ dw, float *__restrict__ db, int cin, int cout,
                                                    int h, int wd)
{
    __shared__ float sdy[COB][TS][TS];
    __shared__ float sx[CIB][TS + 2][TS + 2];
    const int tiles_x = (wd + TS - 1) / TS;
    const int tx0 = ((int)blockIdx.x % tiles_x) * TS, ty0 = ((int)blockIdx.x / tiles_x) * TS;
    const int nci = (cin + CIB - 1) / CIB;
    const int co0 = ((int)blockIdx.y / nci) * COB, ci0 = ((int)blockIdx.y % nci) * CIB;
    const int n = (int)blockIdx.z;
    const size_t plane = (size_t)h * wd;
    for (int i = threadIdx.x; i < COB * TS * TS; i += blockDim.x)
    {
        const int c = i / (TS * TS), r = i % (TS * TS), yy = r / TS, xx = r % TS;
        const int gy = ty0 + yy, gx = tx0 + xx, gc = co0 + c;
        float v = 0.f;
        if (gc < cout && gy < h && gx < wd) v = dy[((size_t)n * cout + gc) * plane + (size_t)gy * wd + gx];
        sdy[c][yy][xx] = v;
    }
    for (int i = threadIdx.x; i < CIB * (TS + 2) * (TS + 2); i += blockDim.x)
    {
        const int c = i / ((TS + 2) * (TS + 2)), r = i % ((TS + 2) * (TS + 2));
        const int yy = r / (TS + 2), xx = r % (TS + 2);
        const int gy = ty0 + yy - 1, gx = tx0 + xx - 1, gc = ci0 + c;
        float v = 0.f;
        if (gc < cin && gy >= 0 && gy < h && gx >= 0 && gx < wd)
            v = x[((size_t)n * cin + gc) * plane + (size_t)gy * wd + gx];
        sx[c][yy][xx] = v;
    }
    __syncthreads();
    const int co = threadIdx.x / CIB, ci = threadIdx.x % CIB;
    float acc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] = 0.f;
    for (int yy = 0; yy < TS; yy++)
        for (int xx = 0; xx < TS; xx++)
        {
            const float g = sdy[co][yy][xx];
#pragma unroll
            for (int k = 0; k < 9; k++) acc[k] = fmaf(g, sx[ci][yy + k / 3][xx + k % 3], acc[k]);
        }
    const int gco = co0 + co, gci = ci0 + ci;
    if (gco < cout && gci < cin)
    {
#pragma unroll
        for (int k = 0; k < 9; k++) atomicAdd(&dw[((size_t)gco * cin + gci) * 9 + k], acc[k]);
    }
    if (db && ci0 == 0 && (int)threadIdx.x < COB && co0 + (int)threadIdx.x < cout)
    {
        float s = 0.f;
        for (int yy = 0; yy < TS; yy++)
            for (int xx = 0; xx < TS; xx++) s += sdy[threadIdx.x][yy][xx];
        atomicAdd(&db[co0 + threadIdx.x], s);
    }
}

__global__ void k_relu_bw(float *dy, const float *y, int64_t count)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count && !(y[i] > 0.f)) dy[i] = 0.f;
}

// per (image * channel) plane: y (h/2, wd/2) = mean of the 2x2 blocks
__global__ void k_pool_fw(const float *x, float *y, int nc, int h, int wd)
{
    const int ho = h / 2, wo = wd / 2;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nc * ho * wo) return;
    const int64_t c = i / ((int64_t)ho * wo);
    const int r = (int)(i % ((int64_t)ho * wo)), yy = r / wo, xx = r % wo;
    const float *p = x + c * h * wd + (int64_t)(2 * yy) * wd + 2 * xx;
    y[i] = 0.25f * (p[0] + p[1] + p[wd] + p[wd + 1]);
}

__global__ void k_pool_bw(const float *dy, float *dx, int nc, int h, int wd)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nc * h * wd) return;
    const int64_t c = i / ((int64_t)h * wd);
    const int r = (int)(i % ((int64_t)h * wd)), yy = r / wd, xx = r % wd;
    dx[i] = 0.25f * dy[c * (h / 2) * (wd / 2) + (int64_t)(yy / 2) * (wd / 2) + xx / 2];
}

// nearest upsampling of an (h, wd) map to (2h, 2wd)
__global__ void k_up_fw(const float *x, float *y, int nc, int h, int wd)
{
    const int ho = 2 * h, wo = 2 * wd;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nc * ho * wo) return;
    const int64_t c = i / ((int64_t)ho * wo);
    const int r = (int)(i % ((int64_t)ho * wo)), yy = r / wo, xx = r % wo;
    y[i] = x[c * h * wd + (int64_t)(yy / 2) * wd + xx / 2];
}

__global__ void k_up_bw(const float *dy, float *dx, int nc, int h, int wd)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nc * h * wd) return;
    const int64_t c = i / ((int64_t)h * wd);
    const int r = (int)(i % ((int64_t)h * wd)), yy = r / wd, xx = r % wd;
    const int wo = 2 * wd;
    const float *p = dy + c * (4 * (int64_t)h * wd) + (int64_t)(2 * yy) * wo + 2 * xx;
    dx[i] = p[0] + p[1] + p[wo] + p[wo + 1];
}

__global__ void k_add(float *y, const float *x, int64_t count)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) y[i] += x[i];
}

__global__ void __launch_bounds__(256) k_mse(const float *p, const float *t, const float *mask, float *dp, float *loss,
                                             int n, int c, int h, int wd, float norm)
{
    __shared__ float red[256];
    const int64_t plane = (int64_t)h * wd, count = (int64_t)n * c * plane;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < count)
    {
        const int64_t img = i / (c * plane), pix = i % plane;
        const float m = mask[img * plane + pix];
        const float d = m * (p[i] - t[i]);
        dp[i] = 2.f * d / norm;
        l = d * d / norm;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

__global__ void k_adam(float *w, const float *g, float *m, float *v, uint16_t *w16, int64_t count, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(wi));
}

__global__ void k_to_bf16(const float *x, uint16_t *y, int64_t count)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) y[i] = __bfloat16_as_ushort(__float2bfloat16_rn(x[i]));
}

int done()
{
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : -(int)e;
}

unsigned blocks(int64_t count) { return (unsigned)((count + 255) / 256); }

// the tensor-core convolutions take more than 48 KB of dynamic shared memory
int tc_attributes()
{
    static int rc = 1;
    if (rc == 1)
    {
        cudaError_t e = cudaFuncSetAttribute(cnn_tc::k_conv3x3_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)cnn_tc::kSmemBytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(cnn_tc::k_conv3x3_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)cnn_tc::kSmemBytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(cnn_tc::k_conv3x3_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)cnn_tc::kWSmemBytes);
        rc = e == cudaSuccess ? 0 : -(int)e;
    }
    return rc;
}

// output channels per CTA of the tensor-core convolutions: all (up to 256) when
// the pixel tiles alone fill the GPU, else fewer (multiples of 16), so that the
// launch has about two CTAs per SM
int tc_ntile(int pixel_ctas, int cout)
{
    static int sms = 0;
    if (!sms)
    {
        int dev = 0;
        sms = 148;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    int nt = std::min(cout, cnn_tc::kNMax);
    nt = (nt + 15) & ~15;
    while (nt > 16 && (int64_t)pixel_ctas * ((cout + nt - 1) / nt) < 2 * sms) nt = ((nt / 2) + 15) & ~15;
    return nt;
}

dim3 conv_grid(int h, int wd, int groups, int n)
{
    return dim3((unsigned)(((wd + TS - 1) / TS) * ((h + TS - 1) / TS)), (unsigned)groups, (unsigned)n);
}
} // namespace

extern "C" {

int cnn_conv3x3_forward(const float *x, const uint16_t *w, const float *b, float *y, int n, int cin, int cout, int h,
                        int wd, int relu, void *stream)
{
    if (n <= 0 || cin <= 0 || cout <= 0 || h <= 0 || wd <= 0) return -1;
    k_conv3x3<false><<<conv_grid(h, wd, (cout + COB - 1) / COB, n), 256, 0, (cudaStream_t)stream>>>(x, w, b, y, cin,
                                                                                                   cout, h, wd, relu);
    return done();
}

int cnn_conv3x3_backward_data(const float *dy, const uint16_t *w, float *dx, int n, int cin, int cout, int h, int wd,
                              void *stream)
{
    if (n <= 0 || cin <= 0 || cout <= 0 || h <= 0 || wd <= 0) return -1;
    // a convolution from the cout gradient channels to the cin input channels
    k_conv3x3<true><<<conv_grid(h, wd, (cin + COB - 1) / COB, n), 256, 0, (cudaStream_t)stream>>>(dy, w, nullptr, dx,
                                                                                                  cout, cin, h, wd, 0);
    return done();
}

int cnn_conv3x3_forward_tc(const float *x, const uint16_t *w, const float *b, float *y, int n, int cin, int cout,
                           int h, int wd, int relu, void *stream)
{
    if (n <= 0 || cin <= 0 || cout <= 0 || h <= 0 || wd <= 0) return -1;
    const int rc = tc_attributes();
    if (rc) return rc;
    const int tiles = (h * wd + cnn_tc::kM - 1) / cnn_tc::kM;
    const int nt = tc_ntile(tiles * n, cout);
    const dim3 grid((unsigned)tiles, (unsigned)((cout + nt - 1) / nt), (unsigned)n);
    cnn_tc::k_conv3x3_tc<false><<<grid, cnn_tc::kThreads, cnn_tc::kSmemBytes, (cudaStream_t)stream>>>(
        x, w, b, y, cin, cout, h, wd, relu, nt);
    return done();
}

int cnn_conv3x3_backward_data_tc(const float *dy, const uint16_t *w, float *dx, int n, int cin, int cout, int h, int wd,
                                 void *stream)
{
    if (n <= 0 || cin <= 0 || cout <= 0 || h <= 0 || wd <= 0) return -1;
    const int rc = tc_attributes();
    if (rc) return rc;
    const int tiles = (h * wd + cnn_tc::kM - 1) / cnn_tc::kM;
    const int nt = tc_ntile(tiles * n, cin);
    const dim3 grid((unsigned)tiles, (unsigned)((cin + nt - 1) / nt), (unsigned)n);
    // a convolution from the cout gradient channels to the cin input channels
    cnn_tc::k_conv3x3_tc<true><<<grid, cnn_tc::kThreads, cnn_tc::kSmemBytes, (cudaStream_t)stream>>>(
        dy, w, nullptr, dx, cout, cin, h, wd, 0, nt);
    return done();
}

int cnn_conv3x3_backward_weight_tc(const float *x, const float *dy, float *dw, float *db, int n, int cin, int cout,
                                   int h, int wd, void *stream)
{
    if (n <= 0 || cin <= 0 || cout <= 0 || h <= 0 || wd <= 0) return -1;
    const int rc = tc_attributes();
    if (rc) return rc;
    const int64_t total = (int64_t)n * h * wd;
    const int mt = (cout + cnn_tc::kM - 1) / cnn_tc::kM, nt = (cin + cnn_tc::kCC - 1) / cnn_tc::kCC;
    // split K: about four CTAs per SM over the whole launch, slices of at least
    // 1024 pixels (a multiple of the 64-pixel chunk)
    int sms = 148;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t slices = std::max<int64_t>(1, (int64_t)4 * sms / (mt * nt));
    int64_t slice = (total + slices - 1) / slices;
    slice = std::max<int64_t>(1024, (slice + cnn_tc::kWK - 1) / cnn_tc::kWK * cnn_tc::kWK);
    slices = (total + slice - 1) / slice;
    const dim3 grid((unsigned)mt, (unsigned)nt, (unsigned)slices);
    cnn_tc::k_conv3x3_wgrad_tc<<<grid, cnn_tc::kThreads, cnn_tc::kWSmemBytes, (cudaStream_t)stream>>>(
        x, dy, dw, n, cin, cout, h, wd, (int)slice);
    if (db) cnn_tc::k_bias_grad<<<cout, 256, 0, (cudaStream_t)stream>>>(dy, db, n, cout, h * wd);
    return done();
}

int cnn_tc_error(void)
{
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, cnn_tc::g_tc_error, sizeof(v)) != cudaSuccess) return -1;
    if (v && cudaMemcpyToSymbol(cnn_tc::g_tc_error, &zero, sizeof(zero)) != cudaSuccess) return -1;
    return (int)v;
}

int cnn_conv3x3_backward_weight(const float *x, const float *dy, float *dw, float *db, int n, int cin, int cout, int h,
                                int wd, void *stream)
{
    if (n <= 0 || cin <= 0 || cout <= 0 || h <= 0 || wd <= 0) return -1;
    const int groups = ((cout + COB - 1) / COB) * ((cin + CIB - 1) / CIB);
    k_conv3x3_bw<<<conv_grid(h, wd, groups, n), 256, 0, (cudaStream_t)stream>>>(x, dy, dw, db, cin, cout, h, wd);
    return done();
}

int cnn_relu_backward(float *dy, const float *y, int64_t count, void *stream)
{
    if (count <= 0) return 0;
    k_relu_bw<<<blocks(count), 256, 0, (cudaStream_t)stream>>>(dy, y, count);
    return done();
}

int cnn_avgpool2_forward(const float *x, float *y, int nc, int h, int wd, void *stream)
{
    if (nc <= 0 || h <= 0 || wd <= 0 || h % 2 || wd % 2) return -1;
    k_pool_fw<<<blocks((int64_t)nc * h * wd / 4), 256, 0, (cudaStream_t)stream>>>(x, y, nc, h, wd);
    return done();
}

int cnn_avgpool2_backward(const float *dy, float *dx, int nc, int h, int wd, void *stream)
{
    if (nc <= 0 || h <= 0 || wd <= 0 || h % 2 || wd % 2) return -1;
    k_pool_bw<<<blocks((int64_t)nc * h * wd), 256, 0, (cudaStream_t)stream>>>(dy, dx, nc, h, wd);
    return done();
}

int cnn_upsample2_forward(const float *x, float *y, int nc, int h, int wd, void *stream)
{
    if (nc <= 0 || h <= 0 || wd <= 0) return -1;
    k_up_fw<<<blocks((int64_t)nc * h * wd * 4), 256, 0, (cudaStream_t)stream>>>(x, y, nc, h, wd);
    return done();
}

int cnn_upsample2_backward(const float *dy, float *dx, int nc, int h, int wd, void *stream)
{
    if (nc <= 0 || h <= 0 || wd <= 0) return -1;
    k_up_bw<<<blocks((int64_t)nc * h * wd), 256, 0, (cudaStream_t)stream>>>(dy, dx, nc, h, wd);
    return done();
}

int cnn_add(float *y, const float *x, int64_t count, void *stream)
{
    if (count <= 0) return 0;
    k_add<<<blocks(count), 256, 0, (cudaStream_t)stream>>>(y, x, count);
    return done();
}

int cnn_mse(const float *p, const float *t, const float *mask, float *dp, float *loss, int n, int c, int h, int wd,
            float norm, void *stream)
{
    if (n <= 0 || c <= 0 || h <= 0 || wd <= 0 || !(norm > 0.f)) return -1;
    k_mse<<<blocks((int64_t)n * c * h * wd), 256, 0, (cudaStream_t)stream>>>(p, t, mask, dp, loss, n, c, h, wd, norm);
    return done();
}

int cnn_adam(float *w, const float *g, float *m, float *v, uint16_t *w16, int64_t count, float lr, float beta1,
             float beta2, float eps, int step, void *stream)
{
    if (count <= 0) return 0;
    if (step < 1) return -1;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    k_adam<<<blocks(count), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, w16, count, lr, beta1, beta2, eps, c1, c2);
    return done();
}

int cnn_to_bf16(const float *x, uint16_t *y, int64_t count, void *stream)
{
    if (count <= 0) return 0;
    k_to_bf16<<<blocks(count), 256, 0, (cudaStream_t)stream>>>(x, y, count);
    return done();
}
} // extern "C"
