// Local pore size and Knudsen number of a pore image on the GPU: the pipeline
// of Shape::calculateProperties (include/shape.hpp:127-251), kernel by kernel.
//
//   1. The image is padded by n columns on each side (void beside rows
//      1..n-2, include/shape.hpp:131-147) and thinned with the Zhang-Suen rule
//      of utils::thinning (include/utils.hpp:438-536).  Of the 3n x 3n padded
//      image only rows n-1..2n can ever be non-zero, so the kernels keep that
//      band of n+2 rows, bit-packed: bit k of word w of a row is column
//      32 w + k.  One thread evaluates the deletion rule for 32 pixels at
//      once with bitwise logic (the neighbour counts A and B come from a
//      bit-sliced adder over the eight neighbour masks).  Each sub-iteration
//      reads one buffer and writes the other, which is the reference's
//      "mark, then delete" order.  The loop stops after the first iteration
//      (pair of sub-iterations) that deletes nothing; iterations are issued
//      in chunks with a per-iteration change flag, and the extra iterations
//      of the last chunk change nothing.
//   2. Exact Euclidean distance transforms (the float distance of the exact
//      integer squared distance) to the nearest solid pixel and to the
//      nearest skeleton pixel, in two separable passes: the vertical distance
//      to the nearest zero pixel of the column, then the row minimum of
//      t^2 + g(j +- t)^2 scanned outwards from the pixel until t^2 exceeds
//      the best value found.
//   3. Per void pixel, the first skeleton pixel in raster order at the
//      skeleton distance (utils::distanceToNearestWallIndex,
//      include/utils.hpp:116-135, visited in O(D) by nearest_skeleton_at),
//      LocPore = 2 x its wall distance and Kn = mfp / LocPore / dx.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../host/medial_search.hpp"
#include "pore_props.hpp"

namespace mantiis
{
namespace
{
struct GeomCudaError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

#define GK(call)                                                                                                       \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess)                                                                                         \
            throw GeomCudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" +         \
                                std::to_string(__LINE__) + ")");                                                       \
    } while (0)

template <typename T> struct GBuf
{
    T *p = nullptr;
    explicit GBuf(size_t n) { GK(cudaMalloc(&p, (n ? n : 1) * sizeof(T))); }
    ~GBuf() { cudaFree(p); }
    GBuf(const GBuf &) = delete;
    GBuf &operator=(const GBuf &) = delete;
};

constexpr int kThreads = 256;
// iterations issued between two reads of the change flags
constexpr int kChunk = 16;

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// ---------------------------------------------------------------- thinning

// band row b (0..n+1) is padded row n-1+b, i.e. image row i = b-1; band
// column c (0..3n-1) is image column j = c-n.  Void image pixels, and the
// padding beside image rows 1..n-2, are 1.
__global__ void k_band_init(const int32_t *__restrict__ pore, uint32_t *__restrict__ band, int n, int wpr)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)(n + 2) * wpr) return;
    const int b = (int)(t / wpr), w = (int)(t % wpr);
    const int i = b - 1;
    uint32_t word = 0;
    if (i >= 0 && i < n)
    {
        const bool pad = i >= 1 && i <= n - 2;
        for (int k = 0; k < 32; k++)
        {
            const int c = 32 * w + k;
            if (c >= 3 * n) break;
            const int j = c - n;
            const bool v = (j >= 0 && j < n) ? pore[(int64_t)i * n + j] == 1 : pad;
            word |= (uint32_t)v << k;
        }
    }
    band[t] = word;
}

__device__ __forceinline__ void full_add(uint32_t a, uint32_t b, uint32_t c, uint32_t &s, uint32_t &carry)
{
    const uint32_t x = a ^ b;
    s = x ^ c;
    carry = (a & b) | (c & x);
}

// bit-sliced population count of eight masks: per bit position, the count is
// b0 + 2 b1 + 4 b2 + 8 b3
__device__ __forceinline__ void count8(const uint32_t x[8], uint32_t &b0, uint32_t &b1, uint32_t &b2, uint32_t &b3)
{
    uint32_t s0, c0, s1, c1, c3, t, c4;
    full_add(x[0], x[1], x[2], s0, c0);
    full_add(x[3], x[4], x[5], s1, c1);
    const uint32_t s2 = x[6] ^ x[7], c2 = x[6] & x[7];
    full_add(s0, s1, s2, b0, c3);
    full_add(c0, c1, c2, t, c4);
    b1 = t ^ c3;
    const uint32_t c5 = t & c3;
    b2 = c4 ^ c5;
    b3 = c4 & c5;
}

// One Zhang-Suen sub-iteration (include/utils.hpp:438-514) over band rows
// 1..n: a pixel is deleted when A == 1, 2 <= B <= 5 and both of the
// sub-iteration's triple products are zero.  Padded columns 0 and 3n-1 are
// never examined by the reference's raster loop and are never deleted.
template <int ITER>
__global__ void __launch_bounds__(kThreads) k_thin(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, int n,
                                                   int wpr, uint32_t *__restrict__ changed)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = t < (int64_t)n * wpr;
    uint32_t del = 0;
    if (active)
    {
        const int b = 1 + (int)(t / wpr), w = (int)(t % wpr);
        const uint32_t *up = src + (int64_t)(b - 1) * wpr, *cu = up + wpr, *dn = cu + wpr;
        const uint32_t P = cu[w];
        if (P)
        {
            const uint32_t uC = up[w], dC = dn[w];
            const uint32_t uL = w > 0 ? up[w - 1] : 0u, cL = w > 0 ? cu[w - 1] : 0u, dL = w > 0 ? dn[w - 1] : 0u;
            const bool r = w + 1 < wpr;
            const uint32_t uR = r ? up[w + 1] : 0u, cR = r ? cu[w + 1] : 0u, dR = r ? dn[w + 1] : 0u;
            // neighbour masks: bit k holds the neighbour of column 32 w + k
            const uint32_t no = uC, so = dC;
            const uint32_t ne = (uC >> 1) | (uR << 31), nw = (uC << 1) | (uL >> 31);
            const uint32_t ea = (P >> 1) | (cR << 31), we = (P << 1) | (cL >> 31);
            const uint32_t se = (dC >> 1) | (dR << 31), sw = (dC << 1) | (dL >> 31);
            // 0 -> 1 transitions around the ring no, ne, ea, se, so, sw, we, nw
            const uint32_t tr[8] = {~no & ne, ~ne & ea, ~ea & se, ~se & so, ~so & sw, ~sw & we, ~we & nw, ~nw & no};
            const uint32_t nb[8] = {no, ne, ea, se, so, sw, we, nw};
            uint32_t a0, a1, a2, a3, q0, q1, q2, q3;
            count8(tr, a0, a1, a2, a3);
            count8(nb, q0, q1, q2, q3);
            const uint32_t a_is_one = a0 & ~a1 & ~a2 & ~a3;
            const uint32_t b_in_2_5 = ~q3 & (q1 ^ q2);
            const uint32_t m1 = ITER == 0 ? (no & ea & so) : (no & ea & we);
            const uint32_t m2 = ITER == 0 ? (ea & so & we) : (no & so & we);
            del = P & a_is_one & b_in_2_5 & ~m1 & ~m2;
            if (w == 0) del &= ~1u;
            const int last = 3 * n - 1;
            if (w == last / 32) del &= ~(1u << (last % 32));
        }
        dst[t + wpr] = P & ~del;
    }
    if (__any_sync(0xffffffffu, del != 0) && (threadIdx.x & 31) == 0) atomicOr(changed, 1u);
}

// skeleton of the image: the band's image columns n..2n-1 of rows 1..n
__global__ void k_cut_skeleton(const uint32_t *__restrict__ band, uint8_t *__restrict__ skel, int n, int wpr)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    const int c = j + n;
    skel[t] = (uint8_t)((band[(int64_t)(i + 1) * wpr + c / 32] >> (c % 32)) & 1u);
}

// ---------------------------------------------------------- distance transform

// foreground of the two transforms: mode 0, non-zero image pixels (distance
// to the nearest solid pixel, include/shape.hpp:183-196); mode 1, pixels off
// the skeleton (distance to the skeleton, :198-212)
__global__ void k_foreground(const int32_t *__restrict__ pore, const uint8_t *__restrict__ skel,
                             uint8_t *__restrict__ fg, int64_t count, int mode)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    fg[t] = (uint8_t)(mode == 0 ? pore[t] != 0 : skel[t] == 0);
}

// vertical distance to the nearest zero pixel of the column, -1 if none
__global__ void k_edt_columns(const uint8_t *__restrict__ fg, int32_t *__restrict__ g, int n)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    int d = -1;
    if (!fg[t]) d = 0;
    else
        for (int s = 1; s < n; s++)
        {
            const bool up = i - s >= 0, down = i + s < n;
            if (!up && !down) break;
            if ((up && !fg[(int64_t)(i - s) * n + j]) || (down && !fg[(int64_t)(i + s) * n + j]))
            {
                d = s;
                break;
            }
        }
    g[t] = d;
}

// exact squared distance = min over columns c of (j - c)^2 + g(c)^2, scanned
// outwards from j until (j - c)^2 reaches the best value; float distance as
// sqrtf of it, the float maximum where the image has no zero pixel
__global__ void k_edt_rows(const int32_t *__restrict__ g, float *__restrict__ out, int n)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    const int32_t *row = g + (int64_t)i * n;
    const int64_t none = INT64_MAX;
    int64_t best = row[j] >= 0 ? (int64_t)row[j] * row[j] : none;
    for (int s = 1; s < n; s++)
    {
        const int64_t s2 = (int64_t)s * s;
        if (s2 >= best) break;
        const bool left = j - s >= 0, right = j + s < n;
        if (!left && !right) break;
        if (left && row[j - s] >= 0) best = min(best, s2 + (int64_t)row[j - s] * row[j - s]);
        if (right && row[j + s] >= 0) best = min(best, s2 + (int64_t)row[j + s] * row[j + s]);
    }
    out[t] = best == none ? FLT_MAX : sqrtf((float)best);
}

// ------------------------------------------------------------ local pore size

__global__ void k_local_pore(const int32_t *__restrict__ pore, const uint8_t *__restrict__ skel,
                             const float *__restrict__ dwall, const float *__restrict__ dskel,
                             double *__restrict__ locpore, double *__restrict__ kn, int n, double dx, double mfp)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    if (pore[t] != 1)
    {
        locpore[t] = 0.0;
        kn[t] = 0.0;
        return;
    }
    const int i = (int)(t / n), j = (int)(t % n);
    const int64_t hit = nearest_skeleton_at(skel, n, i, j, (double)dskel[t]);
    const double mid = hit >= 0 ? (double)dwall[hit] * (double)skel[hit] : (double)dwall[t];
    const double lp = 2.0 * mid;
    locpore[t] = lp;
    kn[t] = mfp / lp / dx;
}
} // namespace

void gpu_pore_properties(const int32_t *pore, int n, double dx, double mfp, double *locpore, double *kn,
                         int64_t *iterations, cudaStream_t stream)
{
    if (!pore || !locpore || !kn) throw std::invalid_argument("gpu_pore_properties: null argument");
    if (n <= 3 || n > kMaxPorePropsSide)
        throw std::invalid_argument("gpu_pore_properties: image side must be in 4.." +
                                    std::to_string(kMaxPorePropsSide));
    const int64_t nn = (int64_t)n * n;
    const int wpr = (3 * n + 31) / 32;
    const int64_t band_words = (int64_t)(n + 2) * wpr;
    GBuf<int32_t> d_pore(nn), d_g(nn);
    GBuf<uint32_t> band_a(band_words), band_b(band_words), flags(kChunk);
    GBuf<uint8_t> d_skel(nn), d_fg(nn);
    GBuf<float> d_wall(nn), d_sk(nn);
    GBuf<double> d_lp(nn), d_kn(nn);
    GK(cudaMemcpyAsync(d_pore.p, pore, nn * sizeof(int32_t), cudaMemcpyHostToDevice, stream));

    k_band_init<<<blocks_for(band_words), kThreads, 0, stream>>>(d_pore.p, band_a.p, n, wpr);
    GK(cudaGetLastError());
    // rows 0 and n+1 of the second buffer stay zero; the kernels write rows 1..n
    GK(cudaMemcpyAsync(band_b.p, band_a.p, band_words * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
    // each iteration deletes at least one pixel of the band or ends the loop
    const int64_t max_iterations = (int64_t)(n + 2) * 3 * n + kChunk;
    std::vector<uint32_t> host_flags(kChunk);
    int64_t done = 0, converged_at = -1;
    const unsigned grid = blocks_for((int64_t)n * wpr);
    while (converged_at < 0)
    {
        if (done > max_iterations) throw std::runtime_error("gpu_pore_properties: thinning did not converge");
        GK(cudaMemsetAsync(flags.p, 0, kChunk * sizeof(uint32_t), stream));
        for (int k = 0; k < kChunk; k++)
        {
            k_thin<0><<<grid, kThreads, 0, stream>>>(band_a.p, band_b.p, n, wpr, flags.p + k);
            k_thin<1><<<grid, kThreads, 0, stream>>>(band_b.p, band_a.p, n, wpr, flags.p + k);
        }
        GK(cudaGetLastError());
        GK(cudaMemcpyAsync(host_flags.data(), flags.p, kChunk * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        GK(cudaStreamSynchronize(stream));
        for (int k = 0; k < kChunk && converged_at < 0; k++)
            if (!host_flags[k]) converged_at = done + k + 1;
        done += kChunk;
    }
    if (iterations) *iterations = converged_at;

    const unsigned gp = blocks_for(nn);
    k_cut_skeleton<<<gp, kThreads, 0, stream>>>(band_a.p, d_skel.p, n, wpr);
    for (int mode = 0; mode < 2; mode++)
    {
        k_foreground<<<gp, kThreads, 0, stream>>>(d_pore.p, d_skel.p, d_fg.p, nn, mode);
        k_edt_columns<<<gp, kThreads, 0, stream>>>(d_fg.p, d_g.p, n);
        k_edt_rows<<<gp, kThreads, 0, stream>>>(d_g.p, mode == 0 ? d_wall.p : d_sk.p, n);
    }
    k_local_pore<<<gp, kThreads, 0, stream>>>(d_pore.p, d_skel.p, d_wall.p, d_sk.p, d_lp.p, d_kn.p, n, dx, mfp);
    GK(cudaGetLastError());
    GK(cudaMemcpyAsync(locpore, d_lp.p, nn * sizeof(double), cudaMemcpyDeviceToHost, stream));
    GK(cudaMemcpyAsync(kn, d_kn.p, nn * sizeof(double), cudaMemcpyDeviceToHost, stream));
    GK(cudaStreamSynchronize(stream));
}

bool is_geometry_cuda_error(const std::exception &e) { return dynamic_cast<const GeomCudaError *>(&e) != nullptr; }
} // namespace mantiis
