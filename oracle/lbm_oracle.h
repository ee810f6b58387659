/*
 * FP64 CPU restatement of the reference solver's time step -- TEST
 * INFRASTRUCTURE ONLY.  Used by tests/, by __graft_entry__.smoke() as the
 * checker and by bench.py's CPU-baseline leg; never by the product.
 *
 * It follows LB2D (include/coreLB.hpp) loop by loop: array-of-structures
 * f[cell*9+q], f_eq once per coarse step, collide -> copy -> zero -> push
 * stream -> walls -> x-periodic per level, the interface exchange, and the
 * macroscopic/residual pass.  The grid tables (cells, neighbours, boundary
 * types, link lists, interface rows) are inputs: they are produced by the
 * reference's Grid2D / LB2D constructor or by an equivalent builder.
 *
 * Parity: pinned against the reference's golden files
 * test/test_input_output/gold/{transport,adsorption}/{ux,uy,rho}.txt (64x64,
 * 100 steps, 1e-10) and against the reference's own code compiled in
 * oracle/_ref (multi-block cases without undefined behaviour).
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleGrid
{
    int n, max_level;
    int64_t n_cells;
    const int32_t *x, *y, *level, *type, *is_buffer, *bnd;
    const int64_t *conn; /* 9 per cell */
    const double *tau, *kn;
    int64_t n_stream;
    const int64_t *stream_id, *stream_loc;
    const int32_t *stream_ic;
    int64_t n_wall;
    const int64_t *wall_id;
    const int32_t *wall_ic;
    int64_t n_per;
    const int64_t *per_id, *per_i2;
    const int32_t *per_ic;
    int64_t n_coarse, n_fine;
    const int64_t *coarse_rows; /* 6 per row: key, coarse, 4 children */
    const int64_t *fine_rows;   /* 6 per row: key, parent, 4 fine */
    int64_t inlet, inlet2, outlet, outlet2;
} OracleGrid;

typedef struct OracleParams
{
    int simulation; /* 0 transport, 1 adsorption, 2 coupled */
    int collision;  /* 0 BGK, 1 MRT, 2 regularized MRT */
    int wall;       /* 0 BB, 1 MDBB, 2 SRBB */
    double fbody, rhoin, mfp, Cl, T_lu, a_alpha_lu;
    double tol;
    int psi_form;   /* 0 PR-EOS, 1 rho_psi (1 - exp(-rho/rho_psi)) */
    double rho_psi, g_ff, g_fs;
} OracleParams;

void *oracle_create(const OracleGrid *g, const OracleParams *p, const double *rho_init);
/* runs up to n steps; with break_on_tol stops after the first step whose
 * residual is below tol (the breaking step is executed); returns steps run */
int oracle_run(void *o, int n, int break_on_tol);
void oracle_fields(void *o, double *rho, double *ux, double *uy, double *f);
int64_t oracle_residuals(void *o, double *out, int64_t cap);
void oracle_destroy(void *o);
int oracle_threads(int n); /* OpenMP threads for the stepping loops; returns the previous value */

#ifdef __cplusplus
}
#endif
#endif
