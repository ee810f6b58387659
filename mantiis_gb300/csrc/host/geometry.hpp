// Pore-image geometry on the host: input/output files, skeleton, distance
// transforms, local pore size and Knudsen number, image shrinking, and the
// seeded disk-packing generator used for synthetic workloads.
//
// Images are row-major, [row * width + col], with row = y and col = x as in
// the reference's Shape::domain[i][j] (include/shape.hpp:55-60).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mantiis
{
struct PoreImage
{
    int n = 0;                  // square side (the reference sets Ny = Nx)
    std::vector<int> pore;      // 1 = void, 0 = solid
    std::vector<double> kn;     // local Knudsen number per pixel
    std::vector<double> locpore;// local pore size (lattice units) per pixel
};

// Reads pore.dat, Kn.dat and localporesize.dat from `folder` (string-joined,
// as the reference does): N*N whitespace-separated numbers each, stored
// column-major (value k belongs to row k % N, column k / N);
// include/shape.hpp:253-285, include/io.hpp:53-72.  Throws std::runtime_error
// with the reference's messages on a missing or short file.
PoreImage load_pore_image(const std::string &folder, int n);

// Writes one value per line with 15 significant digits (include/io.hpp:75-92).
void write_values(const std::string &path, const std::vector<double> &v);
void write_values(const std::string &path, const std::vector<int64_t> &v);

// Zhang-Suen thinning of a 0/1 image in place, with the reference's deletion
// rule A == 1, 2 <= B <= 5 (include/utils.hpp:438-536).  Only pixels that
// touch background are examined, which gives the same result as the full
// raster scan because no other pixel can meet the rule.
void zhang_suen_thin(std::vector<uint8_t> &img, int rows, int cols);

// Exact Euclidean distance from every non-zero pixel to the nearest zero pixel
// (zero pixels get 0), as float: exact integer squared distance, then sqrtf.
std::vector<float> distance_to_zero(const std::vector<uint8_t> &img, int rows, int cols);

// Local pore size and Knudsen number of every void pixel, following
// Shape::calculateProperties (include/shape.hpp:127-251): skeleton of the
// image padded by N on each side (void beside rows 1..N-2), distance to wall,
// distance to the skeleton, the nearest skeleton pixel at that distance
// (first in raster order within 1e-4), LocPore = 2 * its wall distance,
// Kn = mfp / LocPore / dx.  Solid pixels get 0 for both.
void local_pore_properties(const std::vector<int> &domain, int n, double dx, double mfp,
                           std::vector<double> &locpore, std::vector<double> &kn);

// Shrinks a 0/1 image by a power-of-two factor the way the reference's
// resizeBinaryImage does it (include/utils.hpp:539-568): an output pixel is
// void when the rounded mean of the 2x2 source pixels straddling its
// bilinear sample point exceeds 128 of 255, i.e. when at least 3 of them are
// void.  factor 1 returns the image unchanged.
std::vector<int> shrink_binary(const std::vector<int> &img, int n, int factor);

// Seeded disk packing: solid disks of radius uniform in [rmin, rmax] at
// uniform centres are stamped into an all-void n x n image (rows 0 and n-1
// solid) until the porosity is at most `porosity`.  Void pixels whose
// 9-neighbour wall pattern is not one of the 52 tabulated boundary types are
// then filled (the reference rejects such images, include/grid.hpp:1146-1150).
// periodic_x: disks wrap across the x-periodic edge; open_x_edges: no disk
// covers the `edge_margin` columns on either x edge (2 by default), which keeps
// the periodic seam free of solid pixels unless the fill of untabulated
// neighbourhoods puts some back there
std::vector<int> generate_disk_image(int n, double rmin, double rmax, double porosity, uint64_t seed,
                                     bool periodic_x = false, bool open_x_edges = false, int edge_margin = 2);

// Fills void pixels whose neighbour pattern (periodic in x and y, as the
// grid's neighbour table) is not tabulated, until none is left; returns the
// number of pixels filled.
int64_t fill_untabulated_pixels(std::vector<int> &img, int n);
} // namespace mantiis
