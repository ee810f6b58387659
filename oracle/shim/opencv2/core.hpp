/*
 * Minimal OpenCV stand-in used only to compile the reference solver as a CPU
 * oracle (test infrastructure; never linked into the product).
 *
 * It implements the handful of calls the reference makes, from their published
 * definitions:
 *   - cv::Mat for 8-bit and 32-bit-float single-channel images;
 *   - distanceTransform(DIST_L2, DIST_MASK_PRECISE): the exact Euclidean
 *     distance from each non-zero pixel to the nearest zero pixel, as float
 *     (exact integer squared distance, then a correctly rounded sqrtf);
 *   - resize (default INTER_LINEAR) for the power-of-two shrink factors the
 *     reference uses (1, 1/2, 1/4): the output pixel is the rounded mean
 *     (s + 2) >> 2 of the 2x2 source pixels that bilinear sampling at
 *     (dx + 0.5) * scale - 0.5 straddles;
 *   - threshold(THRESH_BINARY), absdiff, countNonZero, element-wise ops;
 *   - GUI calls are no-ops.
 * OpenCV's version is not pinned by the reference (Makefile:39-42).
 */
#pragma once
#include <vector>
#include <memory>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <stdexcept>
#include <string>
#include <algorithm>

typedef unsigned char uchar;

#define CV_8U 0
#define CV_32F 5
#define CV_8UC1 CV_8U
#define CV_32FC1 CV_32F
#define CV_Assert(expr) do { if (!(expr)) throw std::runtime_error("CV_Assert failed: " #expr); } while (0)

namespace cv
{
enum { DIST_L2 = 2 };
enum { DIST_MASK_PRECISE = 0 };
enum { THRESH_BINARY = 0 };
enum { WINDOW_NORMAL = 0 };
enum { INTER_LINEAR = 1 };

struct Size
{
    int width = 0, height = 0;
    Size() {}
    Size(int w, int h) : width(w), height(h) {}
};

class Mat
{
public:
    int rows = 0, cols = 0;
    int kind = CV_8U;
    std::shared_ptr<std::vector<uint8_t>> buf;

    Mat() {}
    Mat(int r, int c, int type) : rows(r), cols(c), kind(type)
    {
        buf = std::make_shared<std::vector<uint8_t>>((size_t)r * c * elem(), 0);
    }
    size_t elem() const { return kind == CV_32F ? 4 : 1; }
    static Mat zeros(Size s, int type) { return Mat(s.height, s.width, type); }
    Size size() const { return Size(cols, rows); }
    int channels() const { return 1; }
    int depth() const { return kind; }
    int type() const { return kind; }
    bool isContinuous() const { return true; }
    bool empty() const { return !buf || rows == 0 || cols == 0; }
    template <typename T> T &at(int i, int j) { return reinterpret_cast<T *>(buf->data())[(size_t)i * cols + j]; }
    template <typename T> const T &at(int i, int j) const
    {
        return reinterpret_cast<const T *>(buf->data())[(size_t)i * cols + j];
    }
    template <typename T> T *ptr(int i) { return reinterpret_cast<T *>(buf->data()) + (size_t)i * cols; }
    Mat clone() const
    {
        Mat m;
        m.rows = rows;
        m.cols = cols;
        m.kind = kind;
        if (buf) m.buf = std::make_shared<std::vector<uint8_t>>(*buf);
        return m;
    }
    void copyTo(Mat &dst) const { dst = clone(); }
    void release() { buf.reset(); rows = cols = 0; }
    size_t total() const { return (size_t)rows * cols; }

    Mat &operator/=(double s)
    {
        CV_Assert(kind == CV_8U);
        for (auto &v : *buf) v = (uint8_t)std::lround(std::min(255.0, std::max(0.0, v / s)));
        return *this;
    }
    Mat &operator*=(double s)
    {
        CV_Assert(kind == CV_8U);
        for (auto &v : *buf) v = (uint8_t)std::lround(std::min(255.0, std::max(0.0, v * s)));
        return *this;
    }
    Mat &operator&=(const Mat &o)
    {
        CV_Assert(kind == CV_8U && o.kind == CV_8U && o.total() == total());
        for (size_t k = 0; k < total(); k++) (*buf)[k] &= (*o.buf)[k];
        return *this;
    }
    Mat operator~() const
    {
        CV_Assert(kind == CV_8U);
        Mat m = clone();
        for (auto &v : *m.buf) v = (uint8_t)~v;
        return m;
    }
};

static inline void absdiff(const Mat &a, const Mat &b, Mat &dst)
{
    CV_Assert(a.kind == CV_8U && b.kind == CV_8U && a.total() == b.total());
    Mat m(a.rows, a.cols, CV_8U);
    for (size_t k = 0; k < a.total(); k++)
    {
        int d = (int)(*a.buf)[k] - (int)(*b.buf)[k];
        (*m.buf)[k] = (uint8_t)(d < 0 ? -d : d);
    }
    dst = m;
}

static inline int countNonZero(const Mat &a)
{
    int n = 0;
    for (size_t k = 0; k < a.total() * a.elem(); k += a.elem())
    {
        bool nz = false;
        for (size_t e = 0; e < a.elem(); e++) nz |= (*a.buf)[k + e] != 0;
        n += nz;
    }
    return n;
}

// Exact Euclidean distance transform: two passes of the 1-D squared-distance
// lower envelope (Felzenszwalb & Huttenlocher, 2012) in exact integer arithmetic.
static inline void edt_1d(const std::vector<int64_t> &f, std::vector<int64_t> &d, int n)
{
    const int64_t INF = (int64_t)1 << 60;
    std::vector<int> v(n);
    std::vector<double> z(n + 1);
    int k = -1;
    for (int q = 0; q < n; q++)
    {
        if (f[q] >= INF) continue;
        if (k < 0)
        {
            k = 0;
            v[0] = q;
            z[0] = -1e300;
            z[1] = 1e300;
            continue;
        }
        while (true)
        {
            int p = v[k];
            // intersection of parabolas rooted at p and q (exact rational compare below)
            double s = ((double)(f[q] + (int64_t)q * q) - (double)(f[p] + (int64_t)p * p)) / (2.0 * (q - p));
            if (s <= z[k])
            {
                k--;
                if (k < 0) break;
                continue;
            }
            k++;
            v[k] = q;
            z[k] = s;
            z[k + 1] = 1e300;
            break;
        }
        if (k < 0)
        {
            k = 0;
            v[0] = q;
            z[0] = -1e300;
            z[1] = 1e300;
        }
    }
    if (k < 0)
    {
        for (int q = 0; q < n; q++) d[q] = INF;
        return;
    }
    int j = 0;
    for (int q = 0; q < n; q++)
    {
        while (z[j + 1] < q) j++;
        // take the exact minimum over the envelope neighbourhood to absorb any
        // rounding in the intersection abscissae
        int64_t best = INF;
        for (int jj = std::max(0, j - 1); jj <= std::min(k, j + 1); jj++)
        {
            int64_t dq = (int64_t)(q - v[jj]);
            best = std::min(best, dq * dq + f[v[jj]]);
        }
        d[q] = best;
    }
}

static inline void distanceTransform(const Mat &src, Mat &dst, int, int)
{
    CV_Assert(src.kind == CV_8U);
    const int64_t INF = (int64_t)1 << 60;
    int R = src.rows, C = src.cols;
    std::vector<int64_t> g((size_t)R * C);
    std::vector<int64_t> f, d;
    f.resize(R);
    d.resize(R);
    for (int c = 0; c < C; c++)
    {
        for (int r = 0; r < R; r++) f[r] = src.at<uchar>(r, c) ? INF : 0;
        edt_1d(f, d, R);
        for (int r = 0; r < R; r++) g[(size_t)r * C + c] = d[r];
    }
    Mat out(R, C, CV_32F);
    f.resize(C);
    d.resize(C);
    for (int r = 0; r < R; r++)
    {
        for (int c = 0; c < C; c++) f[c] = g[(size_t)r * C + c];
        edt_1d(f, d, C);
        for (int c = 0; c < C; c++)
            out.at<float>(r, c) = d[c] >= INF ? 3.4e38f : std::sqrt((float)d[c]);
    }
    dst = out;
}

static inline void resize(const Mat &src, Mat &dst, Size s)
{
    CV_Assert(src.kind == CV_8U);
    if (s.width == src.cols && s.height == src.rows)
    {
        dst = src.clone();
        return;
    }
    CV_Assert(src.cols % s.width == 0 && src.rows % s.height == 0);
    int kx = src.cols / s.width, ky = src.rows / s.height;
    CV_Assert(kx == ky && (kx & (kx - 1)) == 0);
    // bilinear sample point (dx + 0.5) * k - 0.5 lies midway between source
    // pixels k*dx + k/2 - 1 and k*dx + k/2, so the result is their 2x2 rounded mean
    int o = kx / 2 - 1;
    Mat out(s.height, s.width, CV_8U);
    for (int i = 0; i < s.height; i++)
        for (int j = 0; j < s.width; j++)
        {
            int r0 = ky * i + o, c0 = kx * j + o;
            int sum = src.at<uchar>(r0, c0) + src.at<uchar>(r0, c0 + 1) + src.at<uchar>(r0 + 1, c0) +
                      src.at<uchar>(r0 + 1, c0 + 1);
            out.at<uchar>(i, j) = (uchar)((sum + 2) >> 2);
        }
    dst = out;
}

static inline double threshold(const Mat &src, Mat &dst, double thr, double maxv, int)
{
    CV_Assert(src.kind == CV_8U);
    Mat out(src.rows, src.cols, CV_8U);
    for (size_t k = 0; k < src.total(); k++) (*out.buf)[k] = (*src.buf)[k] > thr ? (uchar)maxv : 0;
    dst = out;
    return thr;
}

static inline void imshow(const std::string &, const Mat &) {}
static inline int waitKey(int = 0) { return 0; }
static inline void namedWindow(const std::string &, int = 0) {}
static inline bool imwrite(const std::string &, const Mat &) { return true; }
} // namespace cv
