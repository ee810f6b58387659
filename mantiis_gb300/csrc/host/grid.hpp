// Host-side grid construction: the cell list, neighbour table, boundary types,
// relaxation times and interface tables of the reference's Grid2D, plus the
// link classification of the LB2D constructor.
//
// Single-block (include/grid.hpp:401-424): one cell per void pixel, raster
// order.  Multi-block (include/grid.hpp:313-399, 427-889): quadtree leaves of
// the +-1 image under the wall-distance rule, linearised in raster order of
// their top-left pixel, followed by the buffer cells created at coarse/fine
// interfaces in the order the reference creates them.  Everything the
// reference does by whole-grid searches (O(N^2)) is done here with dense
// per-level lookup arrays, so the cell order and every table come out the
// same at O(N) cost.
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "geometry.hpp"

namespace mantiis
{
// Cases where the reference's behaviour is undefined (it reads outside an
// array).  The builder gives each a defined meaning and counts it here.
struct GridDiagnostics
{
    int64_t buffer_wall_links = 0;       // -1 link of a cell with no boundary type (ifStream[-1])
    int64_t fine_parent_missing_nbr = 0; // fine-buffer parent with a wall/missing neighbour (gridIJ[-1])
    int64_t coarse_missing_child = 0;    // coarse-buffer row with a -1 child (f[-9..])
    int64_t fine_group_unmatched = 0;    // fine-buffer group of 4 with no parent / ragged tail
    int64_t pore_search_failed = 0;      // no skeleton pixel found in local pore size search
};

struct Grid
{
    int n = 0;              // image side (Nx = Ny)
    int max_level = 1;      // 1 = single block
    bool multiblock = false;
    int64_t n_cells = 0;    // globalGridSize

    // per cell, in the reference's cell order
    std::vector<int32_t> x, y;        // top-left pixel (gridIJ[0], gridIJ[1])
    std::vector<int32_t> level;       // 1 = finest
    std::vector<int32_t> type;        // 0 real cell, 10*a+b buffer of the a/b interface
    std::vector<int32_t> is_buffer;
    std::vector<int32_t> bnd;         // boundary type index into the 52 tables, -1 = none
    std::vector<int64_t> lin;         // gridID = x + y*n + (level-1)*n*n
    std::vector<int64_t> conn;        // 9 per cell: neighbour cell, -1 wall, -2 missing
    std::vector<double> kn, locpore, tau;

    std::vector<int64_t> solid_pixels; // sorted raster ids of solid pixels
    std::vector<int64_t> reconstructed; // quadtree image: +leaf number (void), -leaf number (solid)

    // interface tables (rows of 5 ids; key = buffer type)
    std::vector<std::array<int64_t, 5>> parent_child;
    std::vector<int32_t> coarse_key, fine_key;
    std::vector<std::array<int64_t, 5>> coarse_rows; // [coarse buffer, 4 children]
    std::vector<std::array<int64_t, 5>> fine_rows;   // [parent, 4 fine buffers]

    // reference link lists (include/coreLB.hpp:293-366)
    std::vector<int64_t> stream_id, stream_loc;
    std::vector<int32_t> stream_ic;
    std::vector<int64_t> wall_id;
    std::vector<int32_t> wall_ic;
    std::vector<int64_t> per_id, per_i2;
    std::vector<int32_t> per_ic;
    // adsorption inlet/outlet cells (include/coreLB.hpp:281-291, 357-365), -1 if absent
    int64_t inlet = -1, inlet2 = -1, outlet = -1, outlet2 = -1;

    GridDiagnostics diag;
};

struct GridOptions
{
    bool multiblock = false;
    int max_allowed_level = 2; // quadtree depth limit (include/grid.hpp:1180)
    double dx = 1.0e-9;        // lattice spacing, m (multi-block relaxation times)
    double mfp = 0.0;          // mean free path, m
    // Keep every quadrant that touches column 0 or column n-1 at the finest
    // level.  The reference builds no buffer cells across the x-periodic
    // boundary, so a coarse cell facing finer cells across it loses those
    // populations every step and the solution diverges; with this option no
    // coarse/fine interface crosses the boundary.  Off = the reference's grid.
    bool edge_fine = false;
};

Grid build_grid(const PoreImage &img, const GridOptions &opt);

// Boundary-type index of a 9-direction connection row (-1 = interior),
// include/grid.hpp:1111-1157; throws on a pattern that is not in the tables.
int boundary_type_of(const int64_t *conn9);
} // namespace mantiis
