/*
 * CPU restatement of the reference's grid construction -- TEST INFRASTRUCTURE
 * ONLY.  Used by tests/ and by bench.py's CPU arm, which with it builds its
 * grid tables, steps them with lbm_oracle.cpp and loads no product library;
 * never by the product.
 *
 * It follows, step by step:
 *   Shape::calculateProperties        include/shape.hpp:127-251
 *   utils::thinning (Zhang-Suen)      include/utils.hpp:436-537
 *   utils::distanceToNearestWallIndex include/utils.hpp:116-134
 *   utils::resizeBinaryImage          include/utils.hpp:539-568
 *   Grid2D (quadtree, cells, buffers,
 *     neighbours, parent-child,
 *     interface tables, boundary types) include/grid.hpp:313-1266
 *   LB2D link lists and inlet/outlet  include/coreLB.hpp:280-366
 *   LB2D relaxation times             include/coreLB.hpp:432-502
 * The tables come out in the layout of OracleGrid (lbm_oracle.h).
 */
#ifndef GRID_ORACLE_H
#define GRID_ORACLE_H
#include <stdint.h>

#include "lbm_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleGridOptions
{
    int multiblock;        /* is_multiblock of the mantiis executable */
    int max_allowed_level; /* quadtree depth limit (include/grid.hpp:1180 holds 2) */
    int edge_fine;         /* 1: quadrants touching an x edge are split to single pixels */
    double dx, mfp;        /* lattice spacing and mean free path, m (per-level relaxation times) */
} OracleGridOptions;

/* Tables that OracleGrid does not carry, for checks. */
typedef struct OracleGridExtra
{
    const int64_t *lin;          /* col + row n + (level - 1) n^2 per cell */
    const double *locpore;       /* input local pore size at each cell's top-left pixel */
    int64_t n_parent_child;
    const int64_t *parent_child; /* 5 per row: cell, 4 children (-1 absent) */
    int64_t buffer_wall_links;   /* wall links of buffer cells (no boundary type) */
} OracleGridExtra;

/* Local pore size and Kn of every pixel of an n x n binary image (1 void,
 * 0 solid), as Shape::calculateProperties(resolution, mfp).  Returns the
 * number of void pixels whose skeleton search failed (0 on every image tried),
 * or -1 on error (oracle_grid_error). */
int64_t oracle_pore_properties(const int32_t *domain, int n, double resolution, double mfp, double *locpore,
                               double *kn);

/* Grid tables of an n x n image with per-pixel Kn and local pore size (the
 * inputs Grid2D reads from its Shape).  NULL on error (oracle_grid_error). */
void *oracle_grid_create(const int32_t *pore, const double *kn, const double *locpore, int n,
                         const OracleGridOptions *opt);
/* Pointers into the handle's tables, valid until oracle_grid_destroy. */
void oracle_grid_view(void *h, OracleGrid *g, OracleGridExtra *extra);
void oracle_grid_destroy(void *h);
const char *oracle_grid_error(void);

#ifdef __cplusplus
}
#endif
#endif
