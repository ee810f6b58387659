// Device data layout of one pore image, built on the host from a Grid.
//
// Every refinement level l (1 = finest) is a dense torus of W_l x W_l sites,
// W_l = n >> (l-1); the cell whose top-left pixel is (x, y) sits at site
// (x >> (l-1), y >> (l-1)).  Populations are FP32 deviations from the lattice
// weights, df_q = f_q - w_q * rho0, in 9 SoA planes per level, updated in place
// with the AA access pattern.  Solid and other-level positions are inactive
// sites: they are never stepped, but their slots exist, which is where wall
// links park their post-collision value for the reflection in the next step.
//
// A cell is "special" when anything but plain streaming feeds its
// populations: a missing arrival (wall, dropped y-wrap, missing neighbour), a
// wall link, buffer status (multi-block interface) or an inlet/outlet role.
// The per-site relaxation rate 1/tau_s is stored negated for special cells, which then carry a
// 32-byte record with their masks.
#pragma once
#include <cstdint>
#include <vector>

#include "../host/grid.hpp"

namespace mantiis
{
enum WallMode
{
    WALL_BB = 0,   // include/coreLB.hpp:859-865
    WALL_MDBB = 1, // include/coreLB.hpp:936-967
    WALL_SRBB = 2, // include/coreLB.hpp:918-933
};
enum CollisionMode
{
    COLL_BGK = 0,    // include/coreLB.hpp:678-691
    COLL_MRT = 1,    // include/coreLB.hpp:694-742
    COLL_RMRT = 2,   // include/coreLB.hpp:744-792
};

// flags of a special cell record
enum SpecialFlags : uint32_t
{
    SF_BUFFER = 1u,   // multi-block buffer cell that is special anyway: the first substep of a coarse step
                      // reads the interpolated values from the interpolation buffer (a buffer cell
                      // that is otherwise plain gets them written into the slots it reads)
    SF_INLET = 2u,    // adsorption inlet (include/coreLB.hpp:980-1009)
    SF_OUTLET = 4u,
    SF_HAS_K = 8u,    // has a constant term row in the K table
};

struct alignas(16) SpecialRec
{
    uint32_t m0;       // arrive mask | override mask << 9 | wall mask << 18
                       //   arrive bit p: f_p streams in from the neighbour at -c_p
                       //   override bit p: that arrival is x-periodic (it wins over walls)
                       //   wall bit q: link q of this cell is a wall link
    uint32_t m1;       // quirk mask | boundary type << 9 (8 bits, 0xFF = none) | flags << 17 (4 bits)
                       //   | out mask << 21
                       //   quirk bit q: wall link whose neighbour site is an active cell
                       //   out bit q: link q streams (or wraps in x) to a live neighbour
    float r;           // wall coefficient (SRBB / MDBB), from the cell's Kn
    int32_t quirk_base;// side-buffer slot of this cell's first quirk link
    int32_t k_row;     // row of the constant-term table (SF_HAS_K)
    int32_t buf;       // interpolation buffer index (SF_BUFFER), else -1
    int32_t xy;        // position of the cell on its level: x | y << 16
    float omega;       // 1/tau_s of the cell
};

struct LevelLayout
{
    int level = 1;
    int W = 0, H = 0;       // sites
    int pitch = 0;          // floats per row (multiple of 32)
    int64_t plane = 0;      // floats per plane
    std::vector<float> omega;        // per site 1/tau_s: 0 inactive, >0 plain, <0 special
    std::vector<float> tau_d;        // per site tau_d of the plain MRT (adsorption), else empty
    std::vector<uint32_t> spec;      // per site: special record index (valid when tau < 0)
    std::vector<int32_t> tile_list;  // active 32x8 tiles: tx | ty << 16; x-interior tiles first
    int n_tiles_interior = 0;        // tiles with tx in [1, tiles_x - 2] (no x wrap within one cell)
    std::vector<uint32_t> tile_mask; // per active tile, 8 row masks of its plain cells (bit = x offset)
    int tiles_x = 0, tiles_y = 0;
    std::vector<int32_t> tile8_list;  // 8x4 tiles holding a plain or light cell: tx | ty << 16 (x in 8s, y in 4s)
    std::vector<uint32_t> tile8_mask; // per such tile, its plain and light cells (bit = 8 * row + column)
    std::vector<uint32_t> tile8_light;// per such tile, its light cells (subset of tile8_mask)
    int64_t n_active = 0, n_active_real = 0;
    int substeps = 1;                // per coarse step, 2^(L-l)
    int64_t spec_begin = 0, spec_count = 0; // this level's special records (sorted by site)
    // the first spec_heavy records of the level have wall links, x-periodic
    // overrides or inlet / outlet roles; the rest ("light": missing arrivals and
    // buffer status only) can be stepped by the 8x4 plain kernel
    int64_t spec_heavy = 0;
    bool snapshot_all = false;       // level keeps the coarse-step-start (rho,u) of all cells
};

// Coarse-buffer row: coarse buffer cell <- rescaled mean of its 4 children
struct CoarseRowDev
{
    int32_t site;        // coarse cell site (level l2)
    int32_t buf;         // its interpolation buffer index
    int32_t child[4];    // child sites (level l1), -1 if absent
    int32_t child_buf[4];// >= 0: read that child from the interpolation buffer (it was refreshed earlier in this phase)
    float ratio;         // 2 tau_c / mean(tau_children)
    float inv_nchild;    // 1 / number of children present
    int32_t plain_target;// the coarse cell steps as a plain cell: its values also go to the slots it reads next
    int32_t pad_[3];     // 64 bytes: rows stay 16-byte aligned in an array
};
static_assert(sizeof(CoarseRowDev) % 16 == 0, "coarse row size");

// Fine-buffer row: 4 fine buffer cells <- spline of the parent neighbourhood
struct FineRowDev
{
    int32_t node_site[6];// parent-level sites of the 3x2 spline nodes
    int32_t node_buf[6]; // >= 0: read from the interpolation buffer
    int32_t child_site[4];
    int32_t child_buf[4];
    float weight[4][6];  // interpolation weights per child
    float ratio[4];      // tau_child / (2 tau_parent)
    int32_t plain_mask;  // bit c: child c steps as a plain cell (values also go to the slots it reads next)
    int32_t pad_[3];
};
static_assert(sizeof(FineRowDev) % 16 == 0, "fine row size");

struct InterfaceLayout
{
    int l1 = 1, l2 = 2;
    std::vector<CoarseRowDev> coarse;
    std::vector<FineRowDev> fine;
};

struct LayoutParams
{
    int wall = WALL_SRBB;
    int collision = COLL_RMRT;
    double rho0 = 0.0;   // reference density of the deviation storage (= initial density)
    bool adsorption = false;
    double mfp_over_cl = 0.0; // mean free path / lattice spacing (tau_d of the plain MRT)
};

struct ImageLayout
{
    int n = 0, max_level = 1;
    std::vector<LevelLayout> levels;        // index l-1
    std::vector<SpecialRec> specials;
    std::vector<float> ktab;                // 9 floats per row: rho0 * K_p
    int64_t n_quirk = 0;
    int64_t n_buffers = 0;
    std::vector<int32_t> buf_level, buf_site; // per interpolation buffer entry
    std::vector<InterfaceLayout> interfaces;  // (1,2), (2,3), ...
    // per reference cell: level and site, for outputs
    std::vector<int32_t> cell_level, cell_site;
    double tau_mean = 0.0;                    // mean tau_s over non-buffer cells
    int64_t pixel_area_cells = 0;             // sum over non-buffer cells of their pixel area
    double lu_per_coarse_step = 0.0;          // sum_l N_l * 2^(L-l), non-buffer cells
    double buffer_lu_per_coarse_step = 0.0;
};

ImageLayout build_layout(const Grid &g, const LayoutParams &p);

// Interpolation weights of the reference's fine-buffer bicubic spline for one
// parent (exposed for tests): nodes x[3], y[2] and the query points (qx, qy),
// result w[6] in the reference's Z order (x fastest, then y).
void spline_weights(const double x[3], const double y[2], double qx, double qy, double w[6]);
} // namespace mantiis
