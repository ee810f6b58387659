#include "geometry.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <random>
#include <stdexcept>

#include "../boundary_tables.h"
#include "medial_search.hpp"

namespace mantiis
{
namespace
{
std::vector<double> read_numbers(const std::string &path, size_t count)
{
    std::ifstream in(path);
    if (!in.is_open())
    {
        std::cout << "Tried loading " << path << std::endl;
        throw std::runtime_error("[ERROR]: File not found.");
    }
    std::vector<double> v(count);
    for (size_t k = 0; k < count; k++)
        if (!(in >> v[k])) throw std::runtime_error("[ERROR]: Insufficient data in the file.");
    return v;
}

// 1-D squared distance transform (lower envelope of parabolas rooted at the
// finite samples), integer arithmetic throughout; `inf` marks empty samples.
void sq_dist_1d(const int64_t *f, int64_t *out, int n, int64_t inf, std::vector<int> &root, std::vector<int64_t> &num,
                std::vector<int64_t> &den)
{
    // envelope: parabola k is rooted at root[k]; it is lowest from the
    // abscissa num[k]/den[k] (a rational) up to the next one's start.
    int k = -1;
    for (int q = 0; q < n; q++)
    {
        if (f[q] >= inf) continue;
        while (k >= 0)
        {
            int p = root[k];
            // intersection s = ((f[q] + q^2) - (f[p] + p^2)) / (2 (q - p))
            int64_t sn = (f[q] + (int64_t)q * q) - (f[p] + (int64_t)p * p);
            int64_t sd = 2 * (int64_t)(q - p);
            // pop parabola k when s <= start of k  (compare sn/sd <= num/den; both denominators > 0)
            if (k > 0 && (__int128)sn * den[k] <= (__int128)num[k] * sd) k--;
            else
            {
                k++;
                root[k] = q;
                num[k] = sn;
                den[k] = sd;
                break;
            }
        }
        if (k < 0)
        {
            k = 0;
            root[0] = q;
            num[0] = 0;
            den[0] = 0; // unbounded to the left
        }
    }
    if (k < 0)
    {
        for (int q = 0; q < n; q++) out[q] = inf;
        return;
    }
    int j = 0;
    for (int q = 0; q < n; q++)
    {
        // advance while the next parabola starts at or before q  (num/den <= q)
        while (j < k && num[j + 1] <= (int64_t)q * den[j + 1]) j++;
        int64_t d = (int64_t)(q - root[j]);
        out[q] = d * d + f[root[j]];
    }
}
} // namespace

PoreImage load_pore_image(const std::string &folder, int n)
{
    if (n <= 0) throw std::runtime_error("[ERROR]: grid size must be positive.");
    PoreImage im;
    im.n = n;
    size_t nn = (size_t)n * n;
    auto pore = read_numbers(folder + "pore.dat", nn);
    auto kn = read_numbers(folder + "Kn.dat", nn);
    auto lp = read_numbers(folder + "localporesize.dat", nn);
    im.pore.resize(nn);
    im.kn.resize(nn);
    im.locpore.resize(nn);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            size_t src = (size_t)j * n + i, dst = (size_t)i * n + j;
            im.pore[dst] = static_cast<int>(pore[src]);
            im.kn[dst] = kn[src];
            im.locpore[dst] = lp[src];
        }
    return im;
}

template <typename T> static void write_any(const std::string &path, const std::vector<T> &v)
{
    std::ofstream out(path);
    if (!out.is_open())
    {
        std::cout << "Tried writing " << path << std::endl;
        throw std::runtime_error("[ERROR]: Unable to open file for writing.");
    }
    out << std::setprecision(15);
    for (const auto &x : v) out << x << '\n';
}

void write_values(const std::string &path, const std::vector<double> &v) { write_any(path, v); }
void write_values(const std::string &path, const std::vector<int64_t> &v) { write_any(path, v); }

void zhang_suen_thin(std::vector<uint8_t> &img, int rows, int cols)
{
    if (rows <= 3 || cols <= 3) throw std::runtime_error("thinning needs an image larger than 3x3");
    auto at = [&](int r, int c) -> int { return img[(size_t)r * cols + c]; };
    auto touches_bg = [&](int r, int c) {
        for (int dr = -1; dr <= 1; dr++)
            for (int dc = -1; dc <= 1; dc++)
                if ((dr || dc) && !at(r + dr, c + dc)) return true;
        return false;
    };
    std::vector<uint8_t> queued((size_t)rows * cols, 0);
    std::vector<int64_t> cand, next, del;
    for (int r = 1; r < rows - 1; r++)
        for (int c = 1; c < cols - 1; c++)
            if (at(r, c) && touches_bg(r, c))
            {
                cand.push_back((int64_t)r * cols + c);
                queued[(size_t)r * cols + c] = 1;
            }
    bool changed = true;
    while (changed)
    {
        changed = false;
        for (int sub = 0; sub < 2; sub++)
        {
            del.clear();
            for (int64_t p : cand)
            {
                int r = (int)(p / cols), c = (int)(p % cols);
                if (!img[p]) continue;
                int no = at(r - 1, c), ne = at(r - 1, c + 1), ea = at(r, c + 1), se = at(r + 1, c + 1);
                int so = at(r + 1, c), sw = at(r + 1, c - 1), we = at(r, c - 1), nw = at(r - 1, c - 1);
                int A = (!no && ne) + (!ne && ea) + (!ea && se) + (!se && so) + (!so && sw) + (!sw && we) +
                        (!we && nw) + (!nw && no);
                int B = no + ne + ea + se + so + sw + we + nw;
                int m1 = sub == 0 ? no * ea * so : no * ea * we;
                int m2 = sub == 0 ? ea * so * we : no * so * we;
                if (A == 1 && B >= 2 && B <= 5 && m1 == 0 && m2 == 0) del.push_back(p);
            }
            if (del.empty()) continue;
            changed = true;
            for (int64_t p : del) img[p] = 0;
            // next candidates: surviving old ones plus foreground neighbours of deleted pixels
            next.clear();
            for (int64_t p : cand)
            {
                if (img[p]) next.push_back(p);
                else queued[p] = 0;
            }
            for (int64_t p : del)
            {
                int r = (int)(p / cols), c = (int)(p % cols);
                for (int dr = -1; dr <= 1; dr++)
                    for (int dc = -1; dc <= 1; dc++)
                    {
                        int rr = r + dr, cc = c + dc;
                        if (rr < 1 || rr >= rows - 1 || cc < 1 || cc >= cols - 1) continue;
                        int64_t pp = (int64_t)rr * cols + cc;
                        if (img[pp] && !queued[pp])
                        {
                            queued[pp] = 1;
                            next.push_back(pp);
                        }
                    }
            }
            cand.swap(next);
        }
    }
}

std::vector<float> distance_to_zero(const std::vector<uint8_t> &img, int rows, int cols)
{
    const int64_t inf = std::numeric_limits<int64_t>::max() / 4;
    int m = std::max(rows, cols);
    std::vector<int> root(m);
    std::vector<int64_t> num(m), den(m), f(m), o(m);
    std::vector<int64_t> g((size_t)rows * cols);
    for (int c = 0; c < cols; c++)
    {
        for (int r = 0; r < rows; r++) f[r] = img[(size_t)r * cols + c] ? inf : 0;
        sq_dist_1d(f.data(), o.data(), rows, inf, root, num, den);
        for (int r = 0; r < rows; r++) g[(size_t)r * cols + c] = o[r];
    }
    std::vector<float> out((size_t)rows * cols);
    for (int r = 0; r < rows; r++)
    {
        sq_dist_1d(&g[(size_t)r * cols], o.data(), cols, inf, root, num, den);
        for (int c = 0; c < cols; c++)
            out[(size_t)r * cols + c] = o[c] >= inf ? std::numeric_limits<float>::max() : std::sqrt((float)o[c]);
    }
    return out;
}

void local_pore_properties(const std::vector<int> &domain, int n, double dx, double mfp, std::vector<double> &locpore,
                           std::vector<double> &kn)
{
    const int ne = 3 * n, s = n;
    std::vector<uint8_t> ex((size_t)ne * ne, 0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) ex[(size_t)(i + s) * ne + (j + s)] = domain[(size_t)i * n + j] == 1;
    for (int i = 1; i < n - 1; i++)
        for (int j = -s; j < n + s; j++)
            if (j < 0 || j >= n) ex[(size_t)(i + s) * ne + (j + s)] = 1;
    zhang_suen_thin(ex, ne, ne);

    std::vector<uint8_t> skel((size_t)n * n), dom((size_t)n * n), notskel((size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            size_t k = (size_t)i * n + j;
            skel[k] = ex[(size_t)(i + s) * ne + (j + s)] != 0;
            dom[k] = domain[k] != 0;
            notskel[k] = !skel[k];
        }
    std::vector<float> dwall = distance_to_zero(dom, n, n);
    std::vector<float> dskel = distance_to_zero(notskel, n, n);

    locpore.assign((size_t)n * n, 0.0);
    kn.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            size_t k = (size_t)i * n + j;
            if (domain[k] != 1) continue;
            double D = (double)dskel[k];
            int64_t hit = nearest_skeleton_at(skel.data(), n, i, j, D);
            // a void pixel always has a skeleton pixel at its skeleton distance;
            // fall back to its own wall distance should that ever fail
            double mid = hit >= 0 ? (double)dwall[hit] * (double)skel[hit] : (double)dwall[k];
            locpore[k] = 2.0 * mid;
            kn[k] = mfp / locpore[k] / dx;
        }
}

std::vector<int> shrink_binary(const std::vector<int> &img, int n, int factor)
{
    if (factor == 1)
    {
        std::vector<int> out(img.size());
        for (size_t k = 0; k < img.size(); k++) out[k] = img[k] ? 1 : 0;
        return out;
    }
    if (factor <= 0 || (factor & (factor - 1)) || n % factor) throw std::runtime_error("bad shrink factor");
    int m = n / factor, o = factor / 2 - 1;
    std::vector<int> out((size_t)m * m);
    for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++)
        {
            int r = factor * i + o, c = factor * j + o;
            int cnt = (img[(size_t)r * n + c] != 0) + (img[(size_t)r * n + c + 1] != 0) +
                      (img[(size_t)(r + 1) * n + c] != 0) + (img[(size_t)(r + 1) * n + c + 1] != 0);
            out[(size_t)i * m + j] = cnt >= 3;
        }
    return out;
}

int64_t fill_untabulated_pixels(std::vector<int> &img, int n)
{
    static const int dx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1}, dy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    static const int order[9] = {7, 3, 6, 4, 0, 2, 8, 1, 5};
    std::vector<uint8_t> ok(512, 0);
    ok[511] = 1;
    for (int t = 0; t < MANTIIS_N_BND_TYPES; t++) ok[MANTIIS_BND_CODES[t]] = 1;
    int64_t filled = 0;
    bool changed = true;
    while (changed)
    {
        changed = false;
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++)
            {
                if (!img[(size_t)y * n + x]) continue;
                int code = 0;
                for (int k = 0; k < 9; k++)
                {
                    int q = order[k];
                    int xx = (x + dx[q] + n) % n, yy = (y + dy[q] + n) % n;
                    code = (code << 1) | (img[(size_t)yy * n + xx] ? 1 : 0);
                }
                if (!ok[code])
                {
                    img[(size_t)y * n + x] = 0;
                    filled++;
                    changed = true;
                }
            }
    }
    return filled;
}

std::vector<int> generate_disk_image(int n, double rmin, double rmax, double porosity, uint64_t seed, bool periodic_x,
                                     bool open_x_edges, int edge_margin)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> ur(rmin, rmax), uc(0.0, (double)n);
    std::vector<int> img((size_t)n * n, 1);
    int64_t voids = (int64_t)n * n;
    for (int j = 0; j < n; j++)
    {
        img[j] = 0;
        img[(size_t)(n - 1) * n + j] = 0;
    }
    voids -= 2 * n;
    const int64_t target = (int64_t)std::floor(porosity * (double)n * n);
    int guard = 0;
    while (voids > target && guard++ < 100000000)
    {
        double r = ur(rng), cx = uc(rng), cy = uc(rng);
        int r0 = std::max(0, (int)std::floor(cy - r)), r1 = std::min(n - 1, (int)std::ceil(cy + r));
        int c0 = (int)std::floor(cx - r), c1 = (int)std::ceil(cx + r);
        if (!periodic_x)
        {
            c0 = std::max(0, c0);
            c1 = std::min(n - 1, c1);
        }
        else if (c1 - c0 >= n)
        {
            c0 = 0;
            c1 = n - 1;
        }
        for (int i = r0; i <= r1; i++)
            for (int jj = c0; jj <= c1; jj++)
            {
                // x-periodic disks also cover the columns they reach across the edge
                const int j = ((jj % n) + n) % n;
                if (open_x_edges && (j < edge_margin || j >= n - edge_margin)) continue;
                double dy = i - cy, dxv = std::fabs(j - cx);
                if (periodic_x) dxv = std::min(dxv, (double)n - dxv);
                if (dy * dy + dxv * dxv <= r * r && img[(size_t)i * n + j])
                {
                    img[(size_t)i * n + j] = 0;
                    voids--;
                }
            }
    }
    fill_untabulated_pixels(img, n);
    return img;
}
} // namespace mantiis
