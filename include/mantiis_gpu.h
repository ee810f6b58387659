/*
 * C ABI of the GB300 lattice Boltzmann solver (libmantiis_gpu.so).
 *
 * The reference (nnrustamo/mantiis) is a header-only C++ program with no FFI;
 * its hot path is the per-time-step loop body of MantiisApp and the LB2D
 * methods it calls.  Each entry point below names the reference code it
 * replaces.  All functions return 0 on success or a negative MGPU_E* code;
 * mgpu_last_error() then describes the failure.  A context is single-threaded
 * and owns one CUDA stream (its own, or one set with mgpu_set_stream).
 */
#ifndef MANTIIS_GPU_H
#define MANTIIS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGPU_OK 0
#define MGPU_E_ARG (-1)      /* bad argument */
#define MGPU_E_CUDA (-2)     /* CUDA runtime error */
#define MGPU_E_INPUT (-3)    /* unreadable / short input file, unknown boundary pattern */
#define MGPU_E_DEVICE (-4)   /* device-side error flag (non-finite state, bounds) */
#define MGPU_E_STATE (-5)    /* call not valid in the current state */

#define MGPU_SIM_TRANSPORT 0
#define MGPU_SIM_ADSORPTION 1
#define MGPU_SIM_COUPLED 2

typedef struct mgpu_ctx mgpu_ctx;

/* Simulation settings: the reference's Settings struct
 * (include/mantiisApp.hpp:46-64) plus the executable arguments
 * (include/mantiisApp.hpp:131-142) and the knobs of the GPU build. */
typedef struct mgpu_params
{
    int simulation;        /* MGPU_SIM_*                      (Settings::simulation_type) */
    int collision;         /* 0 BGK, 1 MRT, 2 regularized MRT (Settings::collision_method) */
    int wall;              /* 0 BB, 1 MDBB, 2 SRBB            (Settings::wall_boundary) */
    int multiblock;        /* argv[2] == "true" */
    int max_allowed_level; /* quadtree depth limit, 2 in the reference (include/grid.hpp:1180) */
    double dx;             /* Settings::dx, m */
    double fbody;          /* Settings::Fbody, lattice units */
    double T, P;           /* Settings::T (K), Settings::P (Pa) */
    double tol;            /* Settings::threshold: stop when the residual drops below */
    /* adsorption variants; the defaults are the reference's */
    int psi_form;          /* 0: Peng-Robinson pseudopotential (include/coreLB.hpp:515-531),
                              1: psi = rho_psi (1 - exp(-rho / rho_psi)) */
    double rho_psi;        /* rho0 of psi_form 1 */
    double g_ff, g_fs;     /* fluid-fluid and fluid-solid strengths (reference: -1, -12.7) */
    double rho_init;       /* initial density; 0 = the PR-EOS inlet density rho_in */
    double rho_noise;      /* half-width of uniform initial density noise (0 = none) */
    uint64_t seed;         /* seed of that noise */
    int check_every;       /* residual evaluated every k coarse steps (1 = every step, as the reference) */
    int edge_fine;         /* 1: keep the quadtree at the finest level on the x-periodic edges (the
                              reference's grid, 0, leaves coarse/fine interfaces across that boundary
                              without buffer cells, which makes the multi-block solution diverge) */
    int plain_path;        /* plain-cell kernels: 1 = TMA pipeline through shared memory for x-interior
                              32x8 tiles, 0 = direct loads over 32x8 tiles, 2 = direct loads over 8x4
                              tiles, one warp each (fits sparse levels better); -1 (default) = pick the
                              fastest per image by timing all three over a few coarse steps at creation
                              (the state is put back; results are bit-identical on every path) */
    int concurrent;        /* 1: other contexts step on this GPU at the same time (several host threads or
                              streams); the 8x4 plain kernel then leaves room on every SM for their kernels
                              (a batch does this by itself).  0 (default): this context has the GPU */
} mgpu_params;

/* Static description of a built context. */
typedef struct mgpu_info
{
    int n;                 /* image side */
    int max_level;         /* quadtree levels in use (1 = single block) */
    int64_t n_cells;       /* reference cell count incl. buffer cells (globalGridSize) */
    int64_t n_buffer_cells;
    int64_t n_special;     /* cells fed by anything but plain streaming */
    double lu_per_step;    /* lattice updates per coarse step, sum_l N_l 2^(L-l), buffers excluded */
    double buffer_lu_per_step;
    double rho_in;         /* PR-EOS inlet density (lattice units) */
    double mfp;            /* mean free path, m */
    double tau_mean;       /* mean tau_s over non-buffer cells (permeability viscosity) */
    int64_t device_bytes;  /* device memory held by the context */
    int64_t grid_undefined_cases; /* reference-undefined cases given a defined meaning */
    int plain_path;        /* plain-cell path in use: 1 TMA pipeline, 0 direct 32x8, 2 direct 8x4 */
    int pad_;
    double autotune_us[3]; /* plain_path -1: measured microseconds per coarse step of paths 0, 1, 2 (else 0) */
} mgpu_info;

void mgpu_default_params(mgpu_params *p);

/* Builds the grid on the host and uploads it: replaces MantiisApp::init
 * (include/mantiisApp.hpp:158-237), i.e. Grid2D::initialize
 * (include/grid.hpp:271-311), the LB2D constructor (include/coreLB.hpp:231-378)
 * and LB2D::initialize (include/coreLB.hpp:381-417).  pore/kn/locpore are
 * n*n row-major images (row = y); the caller keeps ownership. */
int mgpu_create(const int32_t *pore, const double *kn, const double *locpore, int n, const mgpu_params *p,
                mgpu_ctx **out);

/* Same, reading pore.dat, Kn.dat and localporesize.dat (column-major text)
 * from `folder` (string-joined as in Shape::loadExistingModel,
 * include/shape.hpp:253-285). */
int mgpu_create_from_folder(const char *folder, int n, const mgpu_params *p, mgpu_ctx **out);

int mgpu_destroy(mgpu_ctx *ctx);
int mgpu_get_info(const mgpu_ctx *ctx, mgpu_info *info);

/* Runs up to n_steps coarse time steps of MantiisApp::run's loop
 * (include/mantiisApp.hpp:294-352) with the step body of
 * transport_simulation_loop / adsorption_simulation_loop
 * (include/mantiisApp.hpp:239-265), stopping after the first step whose
 * residual is below tol, exactly like the reference's break.  *steps_done
 * receives the number of steps executed in this call.  A coupled run
 * (MGPU_SIM_COUPLED, include/mantiisApp.hpp:376-392) spends its first steps
 * (100, or fewer if the residual test ends that phase) in the adsorption step
 * without body force, then takes coupled_simulation_loop's step
 * (include/mantiisApp.hpp:267-284); only a break in the coupling phase stops. */
int mgpu_run(mgpu_ctx *ctx, int n_steps, int *steps_done);

/* Runs exactly n_steps coarse steps with no residual and no break; the
 * throughput path.  Residual / permeability are evaluated every
 * p->check_every steps into the history. */
int mgpu_advance(mgpu_ctx *ctx, int n_steps);

/* Same as mgpu_advance with no residual at all, replayed from a CUDA graph of
 * two coarse steps (captured on first use); enqueues the work and returns
 * without waiting.  The throughput path. */
int mgpu_advance_graph(mgpu_ctx *ctx, int n_steps);

/* Profiling aid: enqueues n substeps of one level alone (the step kernel of
 * that level, no interface exchange).  It leaves the multi-level state
 * inconsistent, so use it on a context kept for timing only. */
int mgpu_step_level(mgpu_ctx *ctx, int level, int n);

/* Per level: active cells (incl. buffers), active non-buffer cells, active
 * 32x8 tiles, substeps per coarse step. */
int mgpu_level_info(const mgpu_ctx *ctx, int level, int64_t out[4]);

/* Waits for all work enqueued on the context's stream. */
int mgpu_sync(mgpu_ctx *ctx);

/* Reference step counter lb->t (steps executed, without the step that broke). */
int mgpu_time(const mgpu_ctx *ctx, int64_t *t);

/* Residual history (LB2D::diff_over_time, include/coreLB.hpp:1248-1283):
 * copies up to cap values, *count = total available. */
int mgpu_residuals(mgpu_ctx *ctx, double *out, int64_t cap, int64_t *count);

/* Per-cell fields in the reference cell order, FP64 (rho, ux, uy: n_cells
 * each, may be NULL; f: 9 * n_cells, may be NULL): LB2D::rho/ux/uy/f. */
int mgpu_download_cells(mgpu_ctx *ctx, double *rho, double *ux, double *uy, double *f);

/* n*n pixel fields, row-major (y * n + x), solids 0: completeSingleGridDomain
 * (include/coreLB.hpp:1344-1411); a multi-block cell fills its
 * 2^(l-1) x 2^(l-1) pixels (the piecewise-constant fill of
 * include/coreLB.hpp:1463-1578).  f (9 * n*n, may be NULL): prepareDistributions
 * (include/coreLB.hpp:1619-1641). */
int mgpu_download_pixels(mgpu_ctx *ctx, double *rho, double *ux, double *uy, double *f);

/* Permeability and mass of the current state (no reference counterpart):
 * out[0] = mean u_x over all n*n pixels, out[1] = k = <u_x> nu / F_body with
 * nu = (tau_mean - 1/2) / 3, out[2] = total mass over pixels, out[3] = last residual. */
int mgpu_observables(mgpu_ctx *ctx, double out[4]);

/* Top-left pixel (x, y) and level of every reference cell, in reference
 * cell order (Grid2D::gridIJ / gridLevel, include/grid.hpp:167-264); any
 * pointer may be NULL. */
int mgpu_cell_positions(const mgpu_ctx *ctx, int32_t *x, int32_t *y, int32_t *level);

/* The quadtree image the grid was built from (n*n row-major, +cell number for
 * void leaves, -cell number for solid ones), as Grid2D::initialize writes it
 * to reconstructed.dat (include/grid.hpp:281-287). */
int mgpu_reconstructed(const mgpu_ctx *ctx, int64_t *out);

/* Overwrites the state with f = f_eq(rho, u) per cell (warm start); arrays in
 * reference cell order. */
int mgpu_set_equilibrium(mgpu_ctx *ctx, const double *rho, const double *ux, const double *uy);

/* Restart from saved populations; no counterpart in the reference, which
 * writes f.txt (include/mantiisApp.hpp:412, LB2D::prepareDistributions) but
 * never reads it back.  f becomes the state and the step counter is set to t
 * (lb->t), so that stepping continues as if the run had not stopped: with the
 * populations of mgpu_download_cells the continued run equals the
 * uninterrupted one up to the FP64 rounding of the saved f = w rho0 + df (a
 * deviation df below ~1e-9 may come back one FP32 ulp off).  Layouts:
 *   MGPU_LAYOUT_CELLS   9 * n_cells, cell order (mgpu_download_cells);
 *   MGPU_LAYOUT_PIXELS  9 * n * n, f.txt's order (mgpu_download_pixels): every
 *                       cell takes the populations of its top-left pixel,
 *                       exact on single-block grids; on multi-block grids the
 *                       interface buffer cells take the values of the cells
 *                       that cover the same pixel.
 * The residual history starts empty.  The first transport residual after a
 * restart is the uninterrupted run's; the first adsorption (density) residual
 * compares the restart state with itself, as the first step of a fresh run does
 * (the reference's 1e-5 floor).  A coupled run resumes in the phase that t
 * falls in.  Non-finite populations are rejected (MGPU_E_INPUT). */
#define MGPU_LAYOUT_CELLS 0
#define MGPU_LAYOUT_PIXELS 1
int mgpu_set_distributions(mgpu_ctx *ctx, const double *f, int layout, int64_t t);

/* mgpu_set_equilibrium without any allocation; it has no counterpart in the
 * reference.  For callers that must not allocate device or host memory during a
 * run, e.g. a loop that warm-starts contexts while other contexts keep stepping
 * on their own streams (cudaFree synchronizes the whole device), or a process
 * whose device memory is owned by another allocator.  Same arguments, result and
 * error codes as mgpu_set_equilibrium; the inputs are staged through one static
 * device array of MGPU_NOALLOC_MAX_CELLS cells (24 MiB, part of the library's
 * module image), so a grid with more cells is rejected with MGPU_E_ARG.
 * - The context's device must be current.
 * - The first call on a device looks up the array's address (and may load the
 *   module); make it before any stream capture.
 * - All contexts on a device share the array: calls that overlap in time (from
 *   several host threads) race.  Each call returns after its kernel has read the
 *   array, so calls made one after another are safe. */
#define MGPU_NOALLOC_MAX_CELLS (1 << 20)
int mgpu_set_equilibrium_noalloc(mgpu_ctx *ctx, const double *rho, const double *ux, const double *uy);

/* Use an external cudaStream_t for all work of this context (NULL = own stream). */
int mgpu_set_stream(mgpu_ctx *ctx, void *stream);

/* Number of kernel launches issued by this context so far. */
int64_t mgpu_launch_count(const mgpu_ctx *ctx);

/* ---- batched stepping (no reference counterpart: the reference runs one
 * image per process, include/mantiisApp.hpp:286-430) ----
 * A batch steps a group of transport contexts of the current device together:
 * two coarse steps of every image are replayed from one CUDA graph in which the
 * images run on a few concurrent streams (as many as fit twice the L2 cache,
 * at least 2), so one image's small launches overlap another's work.  The
 * contexts keep their state and stay usable on their own; batch work is
 * ordered after earlier work on each context's stream and before later work.
 * A context must not be stepped by two batches at once. */
typedef struct mgpu_batch mgpu_batch;
int mgpu_batch_create(mgpu_ctx *const *ctxs, int n, mgpu_batch **out);
/* n coarse steps of every image, no residual; enqueues and returns */
int mgpu_batch_advance(mgpu_batch *b, int n_steps);
/* mgpu_observables of every image, 4 values per image */
int mgpu_batch_observables(mgpu_batch *b, double *out);
int mgpu_batch_set_stream(mgpu_batch *b, void *stream);
/* How the batch steps: engine 0 = per-image phase launches on the concurrent
 * streams above; engine 1 = one persistent launch per coarse step (two per
 * graph replay) over every image, level, tile, wall record and interface row
 * of the batch: blocks claim units of work in order and a stage of an image
 * (a phase of its coarse step, an interface wave) starts when its previous
 * stage is complete, as device-side counters show; `group` images (0 = all)
 * are interleaved at a time.  Both engines give bit-identical states. */
#define MGPU_ENGINE_STREAMS 0
#define MGPU_ENGINE_PERSISTENT 1
int mgpu_batch_set_engine(mgpu_batch *b, int engine, int group);
/* The adsorption step of one context (single level, not coupled): engine 1
 * (the default) runs the steps of an mgpu_run batch, an mgpu_advance call or an
 * mgpu_advance_graph call in one cooperative launch, all of its blocks resident,
 * each of the two passes of a step closed by a grid barrier whose waits are
 * bounded (about a second, then MGPU_E_DEVICE); engine 0 launches the passes of
 * every step (pairs of steps replayed from a CUDA graph).  Both give
 * bit-identical states; transport contexts are not affected. */
int mgpu_set_engine(mgpu_ctx *ctx, int engine);
int mgpu_batch_sync(mgpu_batch *b);
int64_t mgpu_batch_launch_count(const mgpu_batch *b);
int mgpu_batch_destroy(mgpu_batch *b);

const char *mgpu_last_error(const mgpu_ctx *ctx);
const char *mgpu_global_error(void);

/* ---- host-only entry points (no GPU needed) ---- */

/* Grid construction alone: Grid2D::initialize (include/grid.hpp:271-311) and
 * the link lists of the LB2D constructor (include/coreLB.hpp:293-366). */
typedef struct mgpu_grid mgpu_grid;
int mgpu_grid_build(const int32_t *pore, const double *kn, const double *locpore, int n, const mgpu_params *p,
                    mgpu_grid **out);
int mgpu_grid_build_from_folder(const char *folder, int n, const mgpu_params *p, mgpu_grid **out);
/* sizes: n_cells, max_level, n_stream, n_wall, n_per, n_coarse, n_fine,
 * n_parent_child, inlet, inlet2, outlet, outlet2 (cell ids, -1 if absent) */
int mgpu_grid_sizes(const mgpu_grid *g, int64_t sizes[12]);
/* per cell (reference order); any pointer may be NULL; conn is 9 per cell */
int mgpu_grid_cells(const mgpu_grid *g, int32_t *x, int32_t *y, int32_t *level, int32_t *type, int32_t *is_buffer,
                    int32_t *bnd, int64_t *conn, double *tau, double *kn, double *locpore, int64_t *lin);
int mgpu_grid_links(const mgpu_grid *g, int64_t *stream_id, int32_t *stream_ic, int64_t *stream_loc, int64_t *wall_id,
                    int32_t *wall_ic, int64_t *per_id, int64_t *per_i2, int32_t *per_ic);
/* coarse/fine rows are 6 values each (key, 5 ids); parent-child rows 5 each */
int mgpu_grid_interfaces(const mgpu_grid *g, int64_t *coarse_rows, int64_t *fine_rows, int64_t *parent_child);
/* undefined-in-the-reference cases: -1 link of a buffer cell, fine parent with
 * a wall/missing neighbour, missing coarse child, unmatched fine group, failed
 * pore-size search */
int mgpu_grid_diagnostics(const mgpu_grid *g, int64_t out[5]);
int mgpu_grid_destroy(mgpu_grid *g);
/* message of the last failed host-only call */
const char *mgpu_host_error(void);

/* Unit system of _GLOBAL_::recompute() (include/globalParameters.hpp:180-221):
 * out = rho_in, mfp, T_lu, a_alpha_lu, Cu, Cf */
int mgpu_units(double dx, double T, double P, double out[6]);

/* Local pore size and Knudsen number of an n*n row-major 0/1 image
 * (Shape::calculateProperties, include/shape.hpp:127-251). */
int mgpu_pore_properties(const int32_t *pore, int n, double dx, double mfp, double *locpore, double *kn);

/* The same fields computed on the current GPU (host pointers in and out, one
 * synchronous call on `stream`, a cudaStream_t, NULL = legacy default stream):
 * the Zhang-Suen skeleton of the padded image (utils::thinning,
 * include/utils.hpp:438-536) as bit-packed bitwise kernels, the two exact
 * distance transforms (include/shape.hpp:183-212) and the nearest-skeleton
 * search (utils::distanceToNearestWallIndex, include/utils.hpp:116-135).
 * Results equal mgpu_pore_properties bit for bit.  4 <= n <= 16384;
 * `iterations` (may be NULL) receives the number of thinning iterations. */
int mgpu_pore_properties_gpu(const int32_t *pore, int n, double dx, double mfp, double *locpore, double *kn,
                             int64_t *iterations, void *stream);

/* Seeded disk packing (synthetic pore images): disks of radius U[rmin, rmax]
 * at uniform centres until the porosity is <= porosity; rows 0 and n-1 solid. */
int mgpu_generate_disks(int n, double rmin, double rmax, double porosity, uint64_t seed, int32_t *pore_out);
/* Same with flags: MGPU_DISKS_PERIODIC_X makes the disks wrap across the
 * x-periodic edge, so the image is itself x-periodic; MGPU_DISKS_OPEN_X_EDGES
 * keeps disks off the two columns at either x edge (solid pixels on the
 * x-periodic seam make the reference's wall-then-periodic order lose mass
 * there: a wall link's share lands in a population the periodic copy then
 * overwrites, so such images have no steady state); MGPU_DISKS_WIDE_X_EDGES
 * keeps them off three columns.  The fill of untabulated neighbourhoods can
 * still put solid pixels on the seam: callers check the result. */
#define MGPU_DISKS_PERIODIC_X 1
#define MGPU_DISKS_OPEN_X_EDGES 2
#define MGPU_DISKS_WIDE_X_EDGES 4
int mgpu_generate_disks_ex(int n, double rmin, double rmax, double porosity, uint64_t seed, int flags,
                           int32_t *pore_out);

#ifdef __cplusplus
}
#endif
#endif
