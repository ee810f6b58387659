// Host context of the GB300 lattice Boltzmann solver and its C ABI
// (include/mantiis_gpu.h).  One context = one pore image on one GPU stream.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/mantiis_gpu.h"
#include "../boundary_tables.h"
#include "../geometry/pore_props.hpp"
#include "../host/geometry.hpp"
#include "../host/grid.hpp"
#include "../host/units.hpp"
#include "kernels.cuh"
#include "layout.hpp"

using namespace mantiis;

namespace
{
thread_local std::string g_error;

struct CudaError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};
struct DeviceError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};
struct InputError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

#define CK(call)                                                                                                       \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess)                                                                                         \
            throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" +              \
                            std::to_string(__LINE__) + ")");                                                           \
    } while (0)

template <typename T> struct DevBuf
{
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n)
    {
        o.p = nullptr;
        o.n = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o)
        {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count, int64_t &acct)
    {
        release();
        if (count == 0) return;
        CK(cudaMalloc(&p, count * sizeof(T)));
        n = count;
        acct += (int64_t)(count * sizeof(T));
    }
    void upload(const std::vector<T> &v, int64_t &acct, cudaStream_t s)
    {
        alloc(v.size(), acct);
        if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void zero(cudaStream_t s)
    {
        if (n) CK(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

struct LevelDev
{
    CUtensorMap tmap;    // the 9 planes as a (x, y, q) tensor for the TMA tile loads
    CUtensorMap om_map;  // the relaxation rates as a (x, y) tensor
    bool has_tmap = false;
    bool use8 = false;   // plain cells through the 8x4 warp-tile kernel
    DevBuf<float> f, omega, tau2, snap, unorm, psi, rho_prev;
    DevBuf<uint32_t> spec;
    DevBuf<int32_t> tiles, tiles8;
    DevBuf<uint32_t> tile_mask, tile8_mask, tile8_light;
    int64_t steps = 0; // substeps done at this level
};

struct InterfaceDev
{
    DevBuf<CoarseRowDev> coarse;
    DevBuf<FineRowDev> fine;
    int l1 = 1;
    int ncoarse = 0, nfine = 0;
};

constexpr int kRing = 8192; // residual accumulator slots (4 doubles each)

// Launch parameters of one state of the step parities over a group of
// images: per phase the plain- and special-cell launches (each with up to
// kMaxPhaseDescs level descriptors), per interface wave its launches.
struct PhaseVariant
{
    std::vector<std::vector<dev::PhaseLaunch>> plain; // per phase: plain cells, tiles with direct loads
    std::vector<std::vector<dev::PhaseLaunch>> plain8; // per phase: plain cells, 8x4 warp tiles
    std::vector<std::vector<dev::TmaLaunch>> tma;     // per phase: plain cells, x-interior tiles through TMA
    std::vector<std::vector<dev::PhaseLaunch>> spec;  // per phase: special cells
    std::vector<std::vector<dev::WaveLaunch>> waves;        // per wave
};

// Phase schedule of a group of images: which (image, level, substep) each
// phase steps, and the level pairs of the interface exchange.
struct PhasePlan
{
    int nphase = 1, nwave = 0;
    // per phase: (image, level - 1, substep k, steps the level has taken in
    // this coarse step before this phase)
    std::vector<std::vector<int4>> entries;
    std::vector<int2> pairs; // (image, interface index)
    std::map<std::string, PhaseVariant> variants;
};

// Work list of the persistent step (dev::k_step_persistent) for a state of the
// level parities: segments in claim order and the descriptors they point to.
struct PersistPlan
{
    DevBuf<dev::PersistSeg> segs;
    DevBuf<dev::StepDesc> sd;
    DevBuf<dev::PairDesc> pd;
    int nseg = 0, total_units = 0, nctr = 0;
    int tiles_per_warp = 1;
    int64_t bytes = 0;
};

} // namespace

// Streams that run beside a context's (or a batch's) main stream within a
// phase: the special-cell kernels on one, the x-border plain tiles on the
// other, so both overlap the x-interior tile kernel.  The three sets of cells
// own disjoint slots (AA pattern), so no ordering is needed among them.
struct SideLanes
{
    cudaStream_t special = nullptr, border = nullptr;
    cudaEvent_t fork = nullptr, join_special = nullptr, join_border = nullptr;
    void create()
    {
        CK(cudaStreamCreateWithFlags(&special, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&border, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&join_special, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&join_border, cudaEventDisableTiming));
    }
    void destroy()
    {
        for (cudaStream_t st : {special, border})
            if (st)
            {
                cudaStreamSynchronize(st);
                cudaStreamDestroy(st);
            }
        for (cudaEvent_t e : {fork, join_special, join_border})
            if (e) cudaEventDestroy(e);
        special = border = nullptr;
        fork = join_special = join_border = nullptr;
    }
};

// Captures the work enqueued on `st` between construction and take() into a
// graph; if an exception leaves the scope first, the capture is ended and its
// partial graph dropped, so the stream is usable again.
struct StreamCapture
{
    cudaStream_t st;
    bool open = false;
    explicit StreamCapture(cudaStream_t s) : st(s)
    {
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        open = true;
    }
    cudaGraph_t take()
    {
        cudaGraph_t g = nullptr;
        open = false;
        CK(cudaStreamEndCapture(st, &g));
        return g;
    }
    ~StreamCapture()
    {
        if (!open) return;
        cudaGraph_t g = nullptr;
        if (cudaStreamEndCapture(st, &g) == cudaSuccess && g) cudaGraphDestroy(g);
        cudaGetLastError();
    }
    StreamCapture(const StreamCapture &) = delete;
    StreamCapture &operator=(const StreamCapture &) = delete;
};

struct mgpu_ctx
{
    mgpu_params prm{};
    UnitSystem units;
    Grid grid;
    ImageLayout lay;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    SideLanes lanes; // special cells and x-border tiles beside `stream`
    int64_t bytes = 0;
    int64_t launches = 0;
    std::string err;

    std::vector<LevelDev> lv;
    std::vector<InterfaceDev> itf;
    DevBuf<SpecialRec> specials;
    DevBuf<float> ktab, side, ibuf;
    DevBuf<int32_t> cell_level, cell_site;
    DevBuf<uint8_t> cell_buffer; // 1 for interface buffer cells (Grid2D::gridIsBuffer)
    DevBuf<double> red;     // kRing * 4
    double *red_host = nullptr; // pinned staging copy of the accumulators
    DevBuf<double> out_rho, out_ux, out_uy, out_f;
    DevBuf<double> in_rho, in_ux, in_uy; // staging of mgpu_set_equilibrium, kept between calls
    DevBuf<unsigned int> errword;
    // adsorption step engine: MGPU_ENGINE_PERSISTENT runs many steps in one
    // cooperative launch (k_ads_persistent), MGPU_ENGINE_STREAMS launches the
    // passes (pairs of steps replayed from a CUDA graph)
    int engine = MGPU_ENGINE_PERSISTENT;
    DevBuf<unsigned int> ads_bar; // grid-barrier arrivals of k_ads_persistent
    int ads_grid = 0;             // its blocks: all resident at once
    float rho0f = 0.f;
    bool adsorption = false; // Shan-Chen step body (include/mantiisApp.hpp:248-265)
    // coupled run (include/mantiisApp.hpp:376-392): up to 100 adsorption steps
    // without body force, then coupling steps (regularized MRT, SRBB walls)
    bool coupled = false, coupled_b = false;
    bool last_step_b = false;            // the last executed step was a coupling step
    int coupled_a = 0;                   // adsorption-phase steps done
    DevBuf<SpecialRec> specials_b;       // records with SRBB wall coefficients / constants
    DevBuf<float> ktab_b;

    cudaGraphExec_t graph = nullptr; // two coarse steps, no residual (throughput path)
    std::string graph_key;           // level parities the graph was captured at
    // mgpu_step_level: two substeps of one level, and the kernels they launch
    std::map<std::string, std::pair<cudaGraphExec_t, int64_t>> level_graphs;
    cudaGraphExec_t run_graph = nullptr; // two coarse steps with residuals into the scratch slots
    std::string run_graph_key;
    int64_t run_graph_launches = 0;
    int64_t graph_launches = 0;
    std::unique_ptr<PhasePlan> plan; // phase engine tables of this image
    std::vector<std::unique_ptr<PhasePlan>> level_plans; // single-level tables (mgpu_step_level)
    int sm_count = 1;
    double autotune_us[3] = {0.0, 0.0, 0.0}; // plain_path -1: microseconds per coarse step of paths 0, 1, 2
    int64_t coarse_done = 0;     // coarse steps executed since creation
    int64_t ref_t = 0;           // reference lb->t
    std::vector<double> residuals;
    bool stored_u_valid = false; // |u| of the current state has been stored

    // checkpoint of the mutable state (exact break semantics)
    struct Checkpoint
    {
        std::vector<std::unique_ptr<DevBuf<float>>> f;
        DevBuf<float> ibuf, side;
        std::vector<std::unique_ptr<DevBuf<float>>> unorm;
        std::vector<int64_t> steps;
        int64_t coarse_done = 0;
        int coupled_a = 0;
        bool coupled_b = false, last_step_b = false;
        bool valid = false;
    } ckpt;

    dev::Common common() const
    {
        dev::Common C{};
        C.specials = specials.p;
        C.ktab = ktab.p;
        C.side = side.p;
        C.n_quirk = lay.n_quirk;
        C.ibuf = ibuf.p;
        C.n_buf = lay.n_buffers;
        C.rho0 = rho0f;
        C.inlet_axis = (float)(d2q9::W[1] * units.rhoin - d2q9::W[1] * (double)rho0f);
        C.inlet_diag = (float)(d2q9::W[2] * units.rhoin - d2q9::W[5] * (double)rho0f);
        C.wall = adsorption ? WALL_BB : prm.wall;
        C.collision = adsorption ? COLL_MRT : prm.collision;
        C.adsorption = adsorption ? 1 : 0;
        C.inlet_outlet = 1;
        C.fbody = (float)prm.fbody;
        if (coupled && !coupled_b) C.fbody = 0.0f; // the adsorption phase runs without body force
        // the collision of the next step follows the phase; the boundary rules
        // applied when populations are read belong to the step that streamed them
        if (coupled && coupled_b) C.collision = COLL_RMRT;
        if (coupled && last_step_b)
        {
            C.wall = WALL_SRBB;
            C.inlet_outlet = 0;
            C.specials = specials_b.p;
            C.ktab = ktab_b.p;
        }
        C.psi_form = prm.psi_form;
        C.psi_rho0 = (float)prm.rho_psi;
        C.eos_a = (float)units.a_alpha_lu;
        C.eos_b = (float)UnitSystem::b_lu;
        C.eos_T = (float)units.T_lu;
        C.g_ff = (float)prm.g_ff;
        C.g_fs = (float)prm.g_fs;
        C.red = red.p;
        C.err = errword.p;
        return C;
    }
    dev::LevelView view(int l) const
    {
        const LevelLayout &ll = lay.levels[l];
        const LevelDev &d = lv[l];
        dev::LevelView v{};
        v.f = d.f.p;
        v.omega = d.omega.p;
        v.spec = d.spec.p;
        v.tau2 = d.tau2.p;
        v.snap = d.snap.p;
        v.unorm = d.unorm.p;
        v.psi = d.psi.p;
        v.rho_prev = d.rho_prev.p;
        v.tiles = d.tiles.p;
        v.tile_mask = d.tile_mask.p;
        v.ntiles = (int)ll.tile_list.size();
        v.tiles_x = ll.tiles_x;
        v.tiles8 = d.tiles8.p;
        v.tile8_mask = d.tile8_mask.p;
        v.tile8_light = d.tile8_light.p;
        v.ntiles8 = (int)ll.tile8_list.size();
        v.W = ll.W;
        v.H = ll.H;
        v.pitch = ll.pitch;
        v.plane = ll.plane;
        v.fshift = (float)(prm.fbody / 2.0 * std::pow(2.0, l));
        v.level = l + 1;
        return v;
    }
    dev::AllLevels all() const
    {
        dev::AllLevels A{};
        for (int l = 0; l < (int)lv.size(); l++)
        {
            A.lv[l] = view(l);
            A.parity[l] = (int)(lv[l].steps & 1);
            A.direct[l] = lv[l].steps == 0 ? 1 : 0;
        }
        return A;
    }
};

namespace
{
int fail(mgpu_ctx *ctx, int code, const std::string &msg)
{
    g_error = msg;
    if (ctx) ctx->err = msg;
    return code;
}

template <typename F> int guarded(mgpu_ctx *ctx, F &&fn)
{
    try
    {
        return fn();
    }
    catch (const CudaError &e)
    {
        return fail(ctx, MGPU_E_CUDA, e.what());
    }
    catch (const DeviceError &e)
    {
        return fail(ctx, MGPU_E_DEVICE, e.what());
    }
    catch (const InputError &e)
    {
        return fail(ctx, MGPU_E_INPUT, e.what());
    }
    catch (const std::invalid_argument &e)
    {
        return fail(ctx, MGPU_E_INPUT, e.what());
    }
    catch (const std::runtime_error &e)
    {
        std::string m = e.what();
        bool input = m.rfind("[ERROR]", 0) == 0;
        return fail(ctx, input ? MGPU_E_INPUT : MGPU_E_ARG, m);
    }
    catch (const std::exception &e)
    {
        return fail(ctx, MGPU_E_ARG, e.what());
    }
}

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (no link against libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn)
    {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) throw std::runtime_error("cuTensorMapEncodeTiled is not available");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// the level's 9 planes as a 3-D tensor (x: pitch floats, y: H rows, q: 9
// planes) read in boxes of 40 x 10 x 9 (a 32 x 8 tile with its halo)
// the level's relaxation-rate plane, read in 32 x 8 boxes (one tile)
void encode_omega_map(CUtensorMap *map, const float *om, const LevelLayout &ll)
{
    const cuuint64_t dims[2] = {(cuuint64_t)ll.pitch, (cuuint64_t)ll.H};
    const cuuint64_t strides[1] = {(cuuint64_t)ll.pitch * 4};
    const cuuint32_t box[2] = {32, 8};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(om), dims, strides,
                                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

void encode_level_map(CUtensorMap *map, float *f, const LevelLayout &ll)
{
    const cuuint64_t dims[3] = {(cuuint64_t)ll.pitch, (cuuint64_t)ll.H, 9};
    const cuuint64_t strides[2] = {(cuuint64_t)ll.pitch * 4, (cuuint64_t)ll.plane * 4};
    const cuuint32_t box[3] = {(cuuint32_t)dev::kTmaW, (cuuint32_t)dev::kTmaH, 9};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = tensor_map_encoder()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, f, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

void upload_constants()
{
    unsigned char icsr[MANTIIS_N_BND_TYPES * 9];
    unsigned short npos[MANTIIS_N_BND_TYPES], nneg[MANTIIS_N_BND_TYPES];
    for (int t = 0; t < MANTIIS_N_BND_TYPES; t++)
    {
        npos[t] = nneg[t] = 0;
        for (int q = 0; q < 9; q++)
        {
            icsr[t * 9 + q] = MANTIIS_ICSR[t][q];
            double cn = d2q9::CY[q] * MANTIIS_XY_NORM[t][1] + d2q9::CX[q] * MANTIIS_XY_NORM[t][0];
            if (cn > 0) npos[t] |= (unsigned short)(1u << q);
            else if (cn < 0) nneg[t] |= (unsigned short)(1u << q);
        }
    }
    CK(cudaMemcpyToSymbol(dev::c_icsr, icsr, sizeof(icsr)));
    CK(cudaMemcpyToSymbol(dev::c_npos, npos, sizeof(npos)));
    CK(cudaMemcpyToSymbol(dev::c_nneg, nneg, sizeof(nneg)));
}

// device error word (a bounded wait that ran out, ...): raises MGPU_E_DEVICE
void check_device_error(mgpu_ctx *ctx)
{
    unsigned int w = 0;
    CK(cudaMemcpyAsync(&w, ctx->errword.p, sizeof(w), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (w)
    {
        CK(cudaMemsetAsync(ctx->errword.p, 0, sizeof(w), ctx->stream));
        throw DeviceError("device error flag " + std::to_string(w) +
                          ((w & dev::kErrTmaTimeout) ? ": a tile copy did not complete in time" : ""));
    }
}

void launch_check(mgpu_ctx *ctx)
{
    ctx->launches++;
    CK(cudaGetLastError());
}

// ---- phase engine, host side.  Substep k of level l (0-based) of an image
// with L levels, in a group whose deepest image has Lmax levels, falls on
// phase k * 2^(Lmax - L + l): every level's first substep on phase 0.
std::unique_ptr<PhasePlan> build_plan(const std::vector<mgpu_ctx *> &ctxs, int only_level);
std::string state_key(const std::vector<mgpu_ctx *> &ctxs, int ahead);
PhaseVariant &plan_variant(PhasePlan &P, const std::vector<mgpu_ctx *> &ctxs, int ahead);
void launch_phase(const PhaseVariant &V, int ph, const dev::PhaseArgs &a, cudaStream_t main, SideLanes &lanes,
                  int64_t &launches, bool share = false);
void phase_step(PhasePlan &P, const std::vector<mgpu_ctx *> &ctxs, cudaStream_t main, SideLanes &lanes,
                dev::PhaseArgs a, int64_t &launches, bool share = false);

// ---- one coarse time step (include/mantiisApp.hpp:239-246, include/coreLB.hpp:1310-1331)
void coarse_step(mgpu_ctx *ctx, bool diff, bool store_u, int red_slot)
{
    dev::Common C = ctx->common();
    if (ctx->adsorption)
    {
        // single level: density and pseudopotential of every cell first (the
        // force needs the neighbours'), then the collision and streaming
        const LevelLayout &ll = ctx->lay.levels[0];
        dev::LevelView V = ctx->view(0);
        dev::StepOpt o{};
        o.parity = (int)(ctx->lv[0].steps & 1);
        o.direct = ctx->lv[0].steps == 0 ? 1 : 0;
        o.red_slot = red_slot;
        o.snap_store = 1;
        // residual: density change in the adsorption pass, |u| sums in the coupling phase
        const bool vel_res = ctx->coupled && ctx->coupled_b;
        dev::StepOpt o_psi = o, o_step = o;
        o_psi.diff = (diff && !vel_res) ? 1 : 0;
        o_step.diff = (diff && vel_res) ? 1 : 0;
        // plain cells over the tiles on the main stream, special cells from their
        // records on a side stream; pass 2 reads the pseudopotential of every
        // cell, so both pass-1 kernels finish before either pass-2 kernel
        dim3 grid((unsigned)ll.tile_list.size()), block(256);
        const int nspec = (int)ll.spec_count;
        const dim3 sgrid((unsigned)((nspec + 127) / 128));
        cudaStream_t side = ctx->lanes.special;
        auto fork = [&]() {
            CK(cudaEventRecord(ctx->lanes.fork, ctx->stream));
            CK(cudaStreamWaitEvent(side, ctx->lanes.fork, 0));
        };
        auto join = [&]() {
            CK(cudaEventRecord(ctx->lanes.join_special, side));
            CK(cudaStreamWaitEvent(ctx->stream, ctx->lanes.join_special, 0));
        };
        if (!ll.tile_list.empty())
        {
            if (nspec) fork();
            if (o.parity == 0) dev::k_ads_psi<0><<<grid, block, 0, ctx->stream>>>(V, C, o_psi);
            else dev::k_ads_psi<1><<<grid, block, 0, ctx->stream>>>(V, C, o_psi);
            launch_check(ctx);
            if (nspec)
            {
                if (o.parity == 0) dev::k_ads_psi_special<0><<<sgrid, 128, 0, side>>>(V, C, o_psi, ll.spec_begin, nspec);
                else dev::k_ads_psi_special<1><<<sgrid, 128, 0, side>>>(V, C, o_psi, ll.spec_begin, nspec);
                launch_check(ctx);
                join();
                fork();
            }
            if (o.parity == 0) dev::k_ads_step<0><<<grid, block, 0, ctx->stream>>>(V, C, o_step);
            else dev::k_ads_step<1><<<grid, block, 0, ctx->stream>>>(V, C, o_step);
            launch_check(ctx);
            if (nspec)
            {
                if (o.parity == 0)
                    dev::k_ads_step_special<0><<<sgrid, 128, 0, side>>>(V, C, o_step, ll.spec_begin, nspec);
                else dev::k_ads_step_special<1><<<sgrid, 128, 0, side>>>(V, C, o_step, ll.spec_begin, nspec);
                launch_check(ctx);
                join();
            }
        }
        ctx->lv[0].steps++;
        ctx->coarse_done++;
        if (ctx->coupled && !ctx->coupled_b) ctx->coupled_a++;
        if (ctx->coupled) ctx->last_step_b = ctx->coupled_b;
        return;
    }
    dev::PhaseArgs a{diff ? 1 : 0, store_u ? 1 : 0, red_slot};
    phase_step(*ctx->plan, {ctx}, ctx->stream, ctx->lanes, a, ctx->launches, ctx->prm.concurrent != 0);
}

// read pass over all reference cells
void cells_pass(mgpu_ctx *ctx, double *rho, double *ux, double *uy, double *f, bool diff, bool store_u, int red_slot,
                cudaStream_t st = nullptr)
{
    int64_t n = ctx->grid.n_cells;
    if (n == 0) return;
    dim3 grid((unsigned)((n + 255) / 256)), block(256);
    dev::k_cells<<<grid, block, 0, st ? st : ctx->stream>>>(ctx->all(), ctx->common(), ctx->cell_level.p, ctx->cell_site.p,
                                                            ctx->cell_buffer.p, n, rho, ux, uy, f, diff ? 1 : 0,
                                                            store_u ? 1 : 0, red_slot);
    launch_check(ctx);
}

void zero_slots(mgpu_ctx *ctx, int first, int count)
{
    // slots are used cyclically; zero a contiguous (possibly wrapping) range
    // with at most two calls
    first %= kRing;
    count = std::min(count, kRing);
    const int a = std::min(count, kRing - first);
    if (a > 0) CK(cudaMemsetAsync(ctx->red.p + (size_t)first * 4, 0, (size_t)a * 4 * sizeof(double), ctx->stream));
    if (count > a) CK(cudaMemsetAsync(ctx->red.p, 0, (size_t)(count - a) * 4 * sizeof(double), ctx->stream));
}

// the accumulators of `count` consecutive slots from `first` (wrapping) into
// out[4 * count]: at most two copies into the context's pinned staging array,
// then a wait on the stream
void read_slots(mgpu_ctx *ctx, int first, int count, double *out)
{
    first %= kRing;
    if (count <= 0) return;
    if (count > kRing) throw std::logic_error("read_slots: more slots than the ring holds");
    if (!ctx->red_host)
    {
        void *p = nullptr;
        CK(cudaMallocHost(&p, (size_t)kRing * 4 * sizeof(double)));
        ctx->red_host = static_cast<double *>(p);
    }
    const int a = std::min(count, kRing - first);
    CK(cudaMemcpyAsync(ctx->red_host, ctx->red.p + (size_t)first * 4, (size_t)a * 4 * sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->stream));
    if (count > a)
        CK(cudaMemcpyAsync(ctx->red_host + (size_t)a * 4, ctx->red.p, (size_t)(count - a) * 4 * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::copy(ctx->red_host, ctx->red_host + (size_t)count * 4, out);
}

void read_slot(mgpu_ctx *ctx, int slot, double out[4])
{
    CK(cudaMemcpyAsync(out, ctx->red.p + (size_t)(slot % kRing) * 4, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
}

void checkpoint_save(mgpu_ctx *ctx)
{
    auto &k = ctx->ckpt;
    int64_t dummy = 0;
    if (!k.valid && k.f.empty())
    {
        for (auto &l : ctx->lv)
        {
            k.f.emplace_back(new DevBuf<float>());
            k.f.back()->alloc(l.f.n, dummy);
            k.unorm.emplace_back(new DevBuf<float>());
            k.unorm.back()->alloc(l.unorm.n, dummy);
        }
        k.ibuf.alloc(ctx->ibuf.n, dummy);
        k.side.alloc(ctx->side.n, dummy);
        ctx->bytes += dummy;
    }
    for (size_t l = 0; l < ctx->lv.size(); l++)
    {
        if (ctx->lv[l].f.n)
            CK(cudaMemcpyAsync(k.f[l]->p, ctx->lv[l].f.p, ctx->lv[l].f.n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        if (ctx->lv[l].unorm.n)
            CK(cudaMemcpyAsync(k.unorm[l]->p, ctx->lv[l].unorm.p, ctx->lv[l].unorm.n * 4, cudaMemcpyDeviceToDevice,
                               ctx->stream));
    }
    if (ctx->ibuf.n) CK(cudaMemcpyAsync(k.ibuf.p, ctx->ibuf.p, ctx->ibuf.n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (ctx->side.n) CK(cudaMemcpyAsync(k.side.p, ctx->side.p, ctx->side.n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    k.steps.clear();
    for (auto &l : ctx->lv) k.steps.push_back(l.steps);
    k.coarse_done = ctx->coarse_done;
    k.coupled_a = ctx->coupled_a;
    k.coupled_b = ctx->coupled_b;
    k.last_step_b = ctx->last_step_b;
    k.valid = true;
}

// frees the checkpoint buffers (the next save allocates them again)
void checkpoint_release(mgpu_ctx *ctx)
{
    auto &k = ctx->ckpt;
    int64_t held = 0;
    for (auto &b : k.f) held += (int64_t)b->n * 4;
    for (auto &b : k.unorm) held += (int64_t)b->n * 4;
    held += (int64_t)(k.ibuf.n + k.side.n) * 4;
    k.f.clear();
    k.unorm.clear();
    k.ibuf = DevBuf<float>();
    k.side = DevBuf<float>();
    k.valid = false;
    ctx->bytes -= held;
}

void checkpoint_restore(mgpu_ctx *ctx)
{
    auto &k = ctx->ckpt;
    for (size_t l = 0; l < ctx->lv.size(); l++)
    {
        if (ctx->lv[l].f.n)
            CK(cudaMemcpyAsync(ctx->lv[l].f.p, k.f[l]->p, ctx->lv[l].f.n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        if (ctx->lv[l].unorm.n)
            CK(cudaMemcpyAsync(ctx->lv[l].unorm.p, k.unorm[l]->p, ctx->lv[l].unorm.n * 4, cudaMemcpyDeviceToDevice,
                               ctx->stream));
        ctx->lv[l].steps = k.steps[l];
    }
    if (ctx->ibuf.n) CK(cudaMemcpyAsync(ctx->ibuf.p, k.ibuf.p, ctx->ibuf.n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (ctx->side.n) CK(cudaMemcpyAsync(ctx->side.p, k.side.p, ctx->side.n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->coarse_done = k.coarse_done;
    ctx->coupled_a = k.coupled_a;
    ctx->coupled_b = k.coupled_b;
    ctx->last_step_b = k.last_step_b;
}

// Steps [k0+1 .. k0+n] with the residual of every step in slots (step index
// mod kRing).  Kernel of step k reads state k-1, so it evaluates residual k-1;
// the residual of the last step comes from a read pass.
// Two coarse steps with residual terms from a CUDA graph (captured once per
// state of the level parities): the graph zeroes the two scratch slots past the
// ring, both steps accumulate into them, and they are then copied to ring slots
// `first` and `first + 1` (mod kRing).  Launch overhead, not GPU work, limits
// small images stepped one call at a time; the graph takes it off the host.
void run_pair_graph(mgpu_ctx *ctx, bool store_u, int first)
{
    const std::string key = state_key({ctx}, 0) + (ctx->adsorption ? "a" : "t");
    if (ctx->run_graph && ctx->run_graph_key != key)
    {
        CK(cudaGraphExecDestroy(ctx->run_graph));
        ctx->run_graph = nullptr;
    }
    double *scratch = ctx->red.p + (size_t)kRing * 4;
    if (!ctx->run_graph)
    {
        if (ctx->plan)
        {
            plan_variant(*ctx->plan, {ctx}, 0);
            plan_variant(*ctx->plan, {ctx}, 1);
        }
        std::vector<int64_t> saved;
        for (auto &l : ctx->lv) saved.push_back(l.steps);
        const int64_t saved_done = ctx->coarse_done, saved_launch = ctx->launches;
        // capturing advances the host-side step counters; put them back either way
        auto restore = [&]() {
            for (size_t l = 0; l < ctx->lv.size(); l++) ctx->lv[l].steps = saved[l];
            ctx->coarse_done = saved_done;
            ctx->launches = saved_launch;
        };
        cudaGraph_t g;
        try
        {
            StreamCapture cap(ctx->stream);
            CK(cudaMemsetAsync(scratch, 0, 8 * sizeof(double), ctx->stream));
            coarse_step(ctx, true, store_u, kRing * 4);
            coarse_step(ctx, true, store_u, (kRing + 1) * 4);
            g = cap.take();
        }
        catch (...)
        {
            restore();
            throw;
        }
        const int64_t captured = ctx->launches - saved_launch;
        restore();
        {
            const cudaError_t e_inst = cudaGraphInstantiate(&ctx->run_graph, g, 0);
            cudaGraphDestroy(g);
            CK(e_inst);
        }
        ctx->run_graph_key = key;
        ctx->run_graph_launches = captured;
    }
    CK(cudaGraphLaunch(ctx->run_graph, ctx->stream));
    for (size_t l = 0; l < ctx->lv.size(); l++) ctx->lv[l].steps += 2 * ctx->lay.levels[l].substeps;
    ctx->coarse_done += 2;
    ctx->launches += ctx->run_graph_launches;
    first %= kRing;
    const int a = first + 1 < kRing ? 2 : 1;
    CK(cudaMemcpyAsync(ctx->red.p + (size_t)first * 4, scratch, (size_t)a * 4 * sizeof(double),
                       cudaMemcpyDeviceToDevice, ctx->stream));
    if (a == 1)
        CK(cudaMemcpyAsync(ctx->red.p, scratch + 4, 4 * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
}

// Adsorption steps k .. k + n - 1 of a single-level context (not coupled) in
// one cooperative launch; with diff, the residual of step j lands in slot
// j mod kRing (zeroed by the caller).
bool ads_persistent_ok(const mgpu_ctx *ctx)
{
    return ctx->adsorption && !ctx->coupled && ctx->engine == MGPU_ENGINE_PERSISTENT &&
           !ctx->lay.levels[0].tile_list.empty();
}

void run_ads_persistent(mgpu_ctx *ctx, int n, int64_t k, bool diff)
{
    // the barrier count of one launch stays far below 2^32 (2 per step and block)
    constexpr int kMaxSteps = 100000;
    while (n > kMaxSteps)
    {
        run_ads_persistent(ctx, kMaxSteps, k, diff);
        n -= kMaxSteps;
        k += kMaxSteps;
    }
    const LevelLayout &ll = ctx->lay.levels[0];
    dev::AdsPersist A{};
    A.L = ctx->view(0);
    A.C = ctx->common();
    A.spec_begin = ll.spec_begin;
    A.spec_count = (int)ll.spec_count;
    A.ntiles = (int)ll.tile_list.size();
    A.nsteps = n;
    A.parity0 = (int)(ctx->lv[0].steps & 1);
    A.direct0 = ctx->lv[0].steps == 0 ? 1 : 0;
    A.slot0 = (int)(k % kRing);
    A.ring = kRing;
    A.psi_diff = diff ? 1 : 0; // the density change (the coupling phase, with |u| sums, is not run here)
    A.step_diff = 0;
    A.bar = ctx->ads_bar.p;
    const int units = A.ntiles + (A.spec_count + dev::kAdsRecords - 1) / dev::kAdsRecords;
    if (ctx->ads_grid == 0)
    {
        int per_sm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::k_ads_persistent, 256, 0));
        ctx->ads_grid = std::max(1, per_sm) * ctx->sm_count;
    }
    const int grid = std::min(units, ctx->ads_grid);
    CK(cudaMemsetAsync(A.bar, 0, sizeof(unsigned int), ctx->stream));
    void *args[] = {&A};
    CK(cudaLaunchCooperativeKernel((const void *)dev::k_ads_persistent, dim3((unsigned)grid), dim3(256), args, 0,
                                   ctx->stream));
    ctx->launches++;
    ctx->lv[0].steps += n;
    ctx->coarse_done += n;
}

bool fresh_state(const mgpu_ctx *ctx)
{
    for (auto &l : ctx->lv)
        if (l.steps == 0) return true;
    return false;
}

// Steps [k0+1 .. k0+n] with the residual of every step in slots (step index
// mod kRing).  Kernel of step k reads state k-1, so it evaluates residual k-1;
// the residual of the last step comes from a read pass.  Pairs of steps run
// from a CUDA graph (not for coupled runs, whose phase switch is host-side,
// nor from the initial "direct" state).
void run_batch_with_residuals(mgpu_ctx *ctx, int n)
{
    int64_t k0 = ctx->coarse_done;
    zero_slots(ctx, (int)((k0 + 1) % kRing), n);
    const bool graphs = !ctx->coupled;
    if (ctx->adsorption)
    {
        // the density change of step k is known within step k
        if (ads_persistent_ok(ctx) && n > 0)
        {
            run_ads_persistent(ctx, n, ctx->coarse_done + 1, true);
            return;
        }
        for (int i = 0; i < n;)
        {
            int64_t k = ctx->coarse_done + 1;
            if (graphs && n - i >= 2 && !fresh_state(ctx))
            {
                run_pair_graph(ctx, false, (int)(k % kRing));
                i += 2;
            }
            else
            {
                coarse_step(ctx, true, false, (int)((k % kRing) * 4));
                i++;
            }
        }
        return;
    }
    for (int i = 0; i < n;)
    {
        int64_t k = ctx->coarse_done + 1; // this step
        bool diff = i > 0;                // residual of step k-1 (the previous batch closed its own last one)
        if (diff && graphs && n - i >= 2 && !fresh_state(ctx))
        {
            run_pair_graph(ctx, true, (int)((k - 1) % kRing));
            i += 2;
        }
        else
        {
            coarse_step(ctx, diff, true, (int)(((k - 1) % kRing) * 4));
            i++;
        }
    }
    int64_t last = ctx->coarse_done;
    cells_pass(ctx, nullptr, nullptr, nullptr, nullptr, true, false, (int)((last % kRing) * 4));
}

// residual of one step from its accumulator slot: transport
// sum|d|u|| / sum|u| (include/coreLB.hpp:1248-1267), adsorption max relative
// density change, 1e-5 when below 1e-15 (include/coreLB.hpp:1269-1283)
double residual_of(const mgpu_ctx *ctx, const double *v)
{
    if (ctx->adsorption && !(ctx->coupled && ctx->coupled_b)) return v[0] < 1.0e-15 ? 1.0e-5 : v[0];
    return v[0] / v[1];
}

// the coupled run leaves its adsorption phase (include/mantiisApp.hpp:378-391)
void enter_coupling(mgpu_ctx *ctx) { ctx->coupled_b = true; }

std::unique_ptr<PhasePlan> build_plan(const std::vector<mgpu_ctx *> &ctxs, int only_level)
{
    std::unique_ptr<PhasePlan> P(new PhasePlan());
    int Lmax = 1;
    for (auto *c : ctxs) Lmax = std::max(Lmax, c->lay.max_level);
    P->nphase = only_level >= 0 ? 1 : 1 << (Lmax - 1);
    P->entries.resize(P->nphase);
    for (int ph = 0; ph < P->nphase; ph++)
        for (size_t i = 0; i < ctxs.size(); i++)
        {
            const ImageLayout &lay = ctxs[i]->lay;
            const int L = lay.max_level;
            for (int l = 0; l < L; l++)
            {
                const LevelLayout &ll = lay.levels[l];
                if (ll.tile_list.empty() && ll.spec_count == 0) continue;
                if (only_level >= 0)
                {
                    // flags of a middle substep (snapshot in use, no buffer refresh)
                    if (l == only_level) P->entries[ph].push_back(make_int4((int)i, l, 1, 0));
                    continue;
                }
                const int stride = 1 << (Lmax - L + l);
                if (ph % stride) continue;
                P->entries[ph].push_back(make_int4((int)i, l, ph / stride, ph / stride));
            }
        }
    if (only_level >= 0) return P;
    // interface waves (include/coreLB.hpp:1327-1330 runs pairs (1,2), (2,3), ...
    // each coarse rows first): coarse rows of pair (l, l+1) read level-l cells
    // and buffers refreshed by the coarse rows of (l-1, l); fine rows of (l, l+1)
    // read level-(l+1) cells and buffers refreshed by the coarse rows of (l, l+1).
    // So wave w = coarse rows of pair (w+1, w+2) and fine rows of pair (w, w+1).
    P->nwave = Lmax >= 2 ? Lmax : 0;
    for (size_t i = 0; i < ctxs.size(); i++)
        for (int p = 0; p < (int)ctxs[i]->itf.size(); p++) P->pairs.push_back(make_int2((int)i, p));
    return P;
}

// parity and "never stepped" state of every level, `ahead` coarse steps on
std::string state_key(const std::vector<mgpu_ctx *> &ctxs, int ahead)
{
    std::string key;
    for (auto *c : ctxs)
        for (size_t l = 0; l < c->lv.size(); l++)
        {
            const int64_t st = c->lv[l].steps + (int64_t)ahead * c->lay.levels[l].substeps;
            key.push_back((char)('0' + (int)(st & 1) + (st == 0 ? 2 : 0)));
        }
    return key;
}

// splits a list of descriptors with their block counts into launches
template <typename Launch, typename Desc, int Max>
std::vector<Launch> pack_launches(const std::vector<std::pair<Desc, int>> &items)
{
    std::vector<Launch> out;
    for (size_t i = 0; i < items.size(); i += Max)
    {
        Launch l;
        std::memset(&l, 0, sizeof(l));
        const int n = (int)std::min<size_t>(Max, items.size() - i);
        l.ndesc = n;
        int blocks = 0;
        for (int j = 0; j < n; j++)
        {
            l.start[j] = blocks;
            l.d[j] = items[i + j].first;
            blocks += items[i + j].second;
        }
        l.start[n] = blocks;
        out.push_back(l);
    }
    return out;
}

// Launch parameters for the state `ahead` coarse steps after the current one.
PhaseVariant &plan_variant(PhasePlan &P, const std::vector<mgpu_ctx *> &ctxs, int ahead)
{
    const std::string key = state_key(ctxs, ahead);
    auto found = P.variants.find(key);
    if (found != P.variants.end()) return found->second;
    auto steps_of = [&](const mgpu_ctx *c, int l) {
        return c->lv[l].steps + (int64_t)ahead * c->lay.levels[l].substeps;
    };
    PhaseVariant V;
    V.plain.resize(P.nphase);
    V.plain8.resize(P.nphase);
    V.tma.resize(P.nphase);
    V.spec.resize(P.nphase);
    for (int ph = 0; ph < P.nphase; ph++)
    {
        std::vector<std::pair<dev::StepDesc, int>> pl, p8, tm, sp;
        std::vector<const LevelDev *> tm_map;
        for (const int4 &e : P.entries[ph])
        {
            const mgpu_ctx *c = ctxs[e.x];
            const int l = e.y, k = e.z;
            const LevelLayout &ll = c->lay.levels[l];
            const int64_t st = steps_of(c, l) + e.w;
            const bool mb = c->grid.multiblock;
            dev::StepDesc sd;
            std::memset(&sd, 0, sizeof(sd));
            sd.L = c->view(l);
            sd.C = c->common();
            sd.o.parity = (int)(st & 1);
            sd.o.direct = st == 0 ? 1 : 0;
            sd.o.first_sub = k == 0 ? 1 : 0;
            sd.o.snap_store = (mb && k == 0) ? 1 : 0;
            sd.o.snap_use = (mb && k > 0) ? 1 : 0;
            sd.spec_begin = ll.spec_begin;
            sd.spec_count = (int)ll.spec_count;
            // x-interior tiles through the TMA pipeline (when the image uses it),
            // the others with direct loads
            const int nt = c->lv[l].use8 ? 0 : (int)ll.tile_list.size();
            const int ni = c->lv[l].has_tmap && !c->lv[l].use8 ? ll.n_tiles_interior : 0;
            if (c->lv[l].use8 && !ll.tile8_list.empty())
            {
                sd.tile_base = 0;
                p8.push_back({sd, (int)((ll.tile8_list.size() + 7) / 8)});
            }
            if (ni > 0)
            {
                sd.tile_base = 0;
                tm.push_back({sd, ni});
                tm_map.push_back(&c->lv[l]);
            }
            if (nt > ni)
            {
                sd.tile_base = ni;
                pl.push_back({sd, nt - ni});
            }
            sd.tile_base = 0;
            // with the 8x4 kernel the light records are stepped there: the
            // special-cell kernel takes the level's heavy prefix only
            const int nspec = (int)(c->lv[l].use8 ? ll.spec_heavy : ll.spec_count);
            sd.spec_count = nspec;
            if (nspec) sp.push_back({sd, (nspec + dev::kSpecialBlock - 1) / dev::kSpecialBlock});
        }
        V.plain[ph] = pack_launches<dev::PhaseLaunch, dev::StepDesc, dev::kMaxPhaseDescs>(pl);
        V.plain8[ph] = pack_launches<dev::PhaseLaunch, dev::StepDesc, dev::kMaxPhaseDescs>(p8);
        for (auto &l : V.plain8[ph]) l.grid = std::min(l.start[l.ndesc], ctxs[0]->sm_count * 4);
        V.spec[ph] = pack_launches<dev::PhaseLaunch, dev::StepDesc, dev::kMaxPhaseDescs>(sp);
        V.tma[ph] = pack_launches<dev::TmaLaunch, dev::StepDesc, dev::kMaxTmaDescs>(tm);
        for (size_t k = 0; k < V.tma[ph].size(); k++)
        {
            dev::TmaLaunch &t = V.tma[ph][k];
            for (int j = 0; j < t.ndesc; j++)
            {
                const LevelDev *ld = tm_map[k * dev::kMaxTmaDescs + j];
                t.map[j] = ld->tmap;
                t.om_map[j] = ld->om_map;
            }
            t.grid = std::min(t.start[t.ndesc], ctxs[0]->sm_count * 4);
        }
    }
    std::vector<std::vector<std::pair<dev::PairDesc, int>>> wv(P.nwave);
    for (const int2 &pr : P.pairs)
    {
        const mgpu_ctx *c = ctxs[pr.x];
        const InterfaceDev &it = c->itf[pr.y];
        const int lf = it.l1 - 1, lc = it.l1;
        dev::PairDesc d;
        std::memset(&d, 0, sizeof(d));
        d.Lf = c->view(lf);
        d.Lc = c->view(lc);
        d.C = c->common();
        d.coarse = it.coarse.p;
        d.fine = it.fine.p;
        // parities once the level has taken this coarse step's substeps
        d.pf = (int)((steps_of(c, lf) + c->lay.levels[lf].substeps) & 1);
        d.pc = (int)((steps_of(c, lc) + c->lay.levels[lc].substeps) & 1);
        if (it.ncoarse)
        {
            d.kind = 0;
            d.nrows = it.ncoarse;
            wv[it.l1 - 1].push_back({d, (it.ncoarse + 31) / 32});
        }
        if (it.nfine)
        {
            d.kind = 1;
            d.nrows = it.nfine;
            wv[it.l1].push_back({d, (4 * it.nfine + 127) / 128});
        }
    }
    V.waves.resize(P.nwave);
    for (int w = 0; w < P.nwave; w++) V.waves[w] = pack_launches<dev::WaveLaunch, dev::PairDesc, dev::kMaxWaveDescs>(wv[w]);
    return P.variants.emplace(key, std::move(V)).first->second;
}

// The launches of one phase: plain cells on `main` (TMA tiles, direct-load
// tiles), special cells forked onto `side` (their slot sets are disjoint
// under the AA ownership rule).
// share: other images' kernels run beside this phase (batch streams); the 8x4
// plain kernel then launches at most 4 blocks per SM, which walk its tiles, so
// the special-cell kernel and the other streams' kernels find room on every SM
// (config-2 batch +6 %; alone, the full grid is faster: 16.4 against 19.1 us
// per level-1 substep)
void launch_phase(const PhaseVariant &V, int ph, const dev::PhaseArgs &a, cudaStream_t main, SideLanes &lanes,
                  int64_t &launches, bool share)
{
    const auto &plain = V.plain[ph], &plain8 = V.plain8[ph], &spec = V.spec[ph];
    const auto &tma = V.tma[ph];
    // x-border tiles beside the TMA tile kernel, special cells beside the plain kernels
    const bool border_side = !plain.empty() && !tma.empty();
    const bool special_side = !spec.empty() && (!plain.empty() || !tma.empty() || !plain8.empty());
    if (border_side || special_side)
    {
        CK(cudaEventRecord(lanes.fork, main));
        if (border_side) CK(cudaStreamWaitEvent(lanes.border, lanes.fork, 0));
        if (special_side) CK(cudaStreamWaitEvent(lanes.special, lanes.fork, 0));
    }
    for (const auto &t0 : tma)
    {
        dev::TmaLaunch t = t0;
        t.a = a;
        dev::k_phase_plain_tma<<<(unsigned)t.grid, 256, 0, main>>>(t);
        CK(cudaGetLastError());
        launches++;
    }
    for (const auto &l0 : plain8)
    {
        dev::PhaseLaunch l = l0;
        l.a = a;
        const int blocks = l.start[l.ndesc];
        dev::k_phase_plain8<<<(unsigned)(share ? std::min(blocks, l.grid) : blocks), 256, 0, main>>>(l);
        CK(cudaGetLastError());
        launches++;
    }
    for (const auto &l0 : plain)
    {
        dev::PhaseLaunch l = l0;
        l.a = a;
        dev::k_phase_plain<<<(unsigned)l.start[l.ndesc], 256, 0, border_side ? lanes.border : main>>>(l);
        CK(cudaGetLastError());
        launches++;
    }
    for (const auto &l0 : spec)
    {
        dev::PhaseLaunch l = l0;
        l.a = a;
        dev::k_phase_special<<<(unsigned)l.start[l.ndesc], dev::kSpecialBlock, 0,
                               special_side ? lanes.special : main>>>(l);
        CK(cudaGetLastError());
        launches++;
    }
    if (border_side)
    {
        CK(cudaEventRecord(lanes.join_border, lanes.border));
        CK(cudaStreamWaitEvent(main, lanes.join_border, 0));
    }
    if (special_side)
    {
        CK(cudaEventRecord(lanes.join_special, lanes.special));
        CK(cudaStreamWaitEvent(main, lanes.join_special, 0));
    }
}

// One coarse step of every image of the group: the phases, then the
// interface waves.
void phase_step(PhasePlan &P, const std::vector<mgpu_ctx *> &ctxs, cudaStream_t main, SideLanes &lanes,
                dev::PhaseArgs a, int64_t &launches, bool share)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(main, &cs));
    if (cs != cudaStreamCaptureStatusNone && !P.variants.count(state_key(ctxs, 0)))
        throw std::logic_error("phase launches missing during graph capture");
    PhaseVariant &V = plan_variant(P, ctxs, 0);
    const dev::PhaseArgs none{0, 0, 0};
    for (int ph = 0; ph < P.nphase; ph++)
        launch_phase(V, ph, ph == 0 ? a : none, main, lanes, launches, share);
    for (int w = 0; w < P.nwave; w++)
        for (const auto &l : V.waves[w])
        {
            dev::k_wave<<<(unsigned)l.start[l.ndesc], 128, 0, main>>>(l);
            CK(cudaGetLastError());
            launches++;
        }
    for (auto *c : ctxs)
    {
        for (size_t l = 0; l < c->lv.size(); l++) c->lv[l].steps += c->lay.levels[l].substeps;
        c->coarse_done++;
    }
}

// ---- persistent step, host side.  The work of `ncoarse` coarse steps of the
// images `ctxs`, from the state `ahead` coarse steps on, as one list of units
// for dev::k_step_persistent.  Per image the stages are its phases (the 8x4
// tiles of every level stepping in the phase, with the light special records,
// and the records with walls) and then its interface waves, exactly the work
// and order of phase_step on one image; images are interleaved stage by stage
// in groups of `group` images (0: all), so that the images in flight at once
// can be kept to what shares the L2.
void build_persist(PersistPlan &PP, const std::vector<mgpu_ctx *> &ctxs, int ahead, int ncoarse, int group,
                   int tiles_per_warp, cudaStream_t st)
{
    struct Item
    {
        int kind, desc, units;
    };
    using Stage = std::vector<Item>;
    std::vector<std::vector<Stage>> stages(ctxs.size());
    std::vector<dev::StepDesc> sd;
    std::vector<dev::PairDesc> pd;
    auto units_of = [](int64_t n, int per) { return (int)((n + per - 1) / per); };
    for (size_t i = 0; i < ctxs.size(); i++)
    {
        const mgpu_ctx *c = ctxs[i];
        const PhasePlan &P = *c->plan;
        for (int a = 0; a < ncoarse; a++)
        {
            const int ah = ahead + a;
            auto steps_of = [&](int l) { return c->lv[l].steps + (int64_t)ah * c->lay.levels[l].substeps; };
            for (int ph = 0; ph < P.nphase; ph++)
            {
                Stage stg;
                for (const int4 &e : P.entries[ph])
                {
                    const int l = e.y, k = e.z;
                    const LevelLayout &ll = c->lay.levels[l];
                    const int64_t stp = steps_of(l) + e.w;
                    const bool mb = c->grid.multiblock;
                    dev::StepDesc d;
                    std::memset(&d, 0, sizeof(d));
                    d.L = c->view(l);
                    d.C = c->common();
                    d.o.parity = (int)(stp & 1);
                    d.o.direct = stp == 0 ? 1 : 0;
                    d.o.first_sub = k == 0 ? 1 : 0;
                    d.o.snap_store = (mb && k == 0) ? 1 : 0;
                    d.o.snap_use = (mb && k > 0) ? 1 : 0;
                    d.spec_begin = ll.spec_begin;
                    d.spec_count = (int)ll.spec_heavy; // the light records are stepped with the tiles
                    if (!ll.tile8_list.empty())
                    {
                        sd.push_back(d);
                        stg.push_back({0, (int)sd.size() - 1, units_of((int64_t)ll.tile8_list.size(), 8 * tiles_per_warp)});
                    }
                    if (ll.spec_heavy > 0)
                    {
                        sd.push_back(d);
                        stg.push_back({1, (int)sd.size() - 1, units_of(ll.spec_heavy, dev::kPersistRecords)});
                    }
                }
                if (!stg.empty()) stages[i].push_back(stg);
            }
            // interface waves: wave w = coarse rows of pair (w+1, w+2), fine rows of pair (w, w+1)
            for (int w = 0; w < P.nwave; w++)
            {
                Stage stg;
                for (const int2 &pr : P.pairs)
                {
                    const InterfaceDev &it = c->itf[pr.y];
                    const int lf = it.l1 - 1, lc = it.l1;
                    dev::PairDesc d;
                    std::memset(&d, 0, sizeof(d));
                    d.Lf = c->view(lf);
                    d.Lc = c->view(lc);
                    d.C = c->common();
                    d.coarse = it.coarse.p;
                    d.fine = it.fine.p;
                    d.pf = (int)((steps_of(lf) + c->lay.levels[lf].substeps) & 1);
                    d.pc = (int)((steps_of(lc) + c->lay.levels[lc].substeps) & 1);
                    if (it.ncoarse && it.l1 - 1 == w)
                    {
                        d.kind = 0;
                        d.nrows = it.ncoarse;
                        pd.push_back(d);
                        stg.push_back({2, (int)pd.size() - 1, units_of(it.ncoarse, dev::kPersistRows)});
                    }
                    if (it.nfine && it.l1 == w)
                    {
                        d.kind = 1;
                        d.nrows = it.nfine;
                        pd.push_back(d);
                        stg.push_back({3, (int)pd.size() - 1, units_of(it.nfine, dev::kPersistRows)});
                    }
                }
                if (!stg.empty()) stages[i].push_back(stg);
            }
        }
    }
    // claim order: groups of images one after another; within a group stage s
    // of every image before stage s + 1 of any
    std::vector<dev::PersistSeg> segs;
    std::vector<std::vector<int>> ctr(ctxs.size());
    std::vector<std::vector<unsigned>> stage_units(ctxs.size());
    int nctr = 0;
    for (size_t i = 0; i < ctxs.size(); i++)
        for (const Stage &stg : stages[i])
        {
            ctr[i].push_back(nctr++);
            unsigned u = 0;
            for (const Item &it : stg) u += (unsigned)it.units;
            stage_units[i].push_back(u);
        }
    const size_t G = group > 0 ? (size_t)group : ctxs.size();
    int unit = 0;
    for (size_t g0 = 0; g0 < ctxs.size(); g0 += G)
    {
        const size_t g1 = std::min(ctxs.size(), g0 + G);
        size_t smax = 0;
        for (size_t i = g0; i < g1; i++) smax = std::max(smax, stages[i].size());
        for (size_t sidx = 0; sidx < smax; sidx++)
            for (size_t i = g0; i < g1; i++)
            {
                if (sidx >= stages[i].size()) continue;
                for (const Item &it : stages[i][sidx])
                {
                    dev::PersistSeg sg{};
                    sg.kind = it.kind;
                    sg.desc = it.desc;
                    sg.unit0 = unit;
                    sg.nunits = it.units;
                    sg.wait_ctr = sidx > 0 ? ctr[i][sidx - 1] : -1;
                    sg.wait_target = sidx > 0 ? stage_units[i][sidx - 1] : 0u;
                    sg.done_ctr = ctr[i][sidx];
                    segs.push_back(sg);
                    unit += it.units;
                }
            }
    }
    PP.bytes = 0;
    PP.segs.upload(segs, PP.bytes, st);
    PP.sd.upload(sd, PP.bytes, st);
    PP.pd.upload(pd, PP.bytes, st);
    PP.nseg = (int)segs.size();
    PP.total_units = unit;
    PP.nctr = nctr;
    PP.tiles_per_warp = tiles_per_warp;
}

// the persistent kernel's register budget is sized for this many blocks per SM
constexpr int kPersistMinBlocks = 5;

// blocks of a persistent launch: as many as fit on the GPU at once
int persist_grid(int sm_count, int total_units)
{
    static int per_sm = 0;
    if (!per_sm)
    {
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::k_step_persistent<kPersistMinBlocks>,
                                                         dev::kPersistThreads, 0));
        per_sm = std::max(per_sm, 1);
    }
    return std::max(1, std::min(total_units, sm_count * per_sm));
}

// Enqueues one persistent launch of the plan (its counters zeroed first).
void launch_persist(const PersistPlan &PP, unsigned int *sync, unsigned int *err, int sm_count, cudaStream_t st,
                    int64_t &launches)
{
    if (PP.total_units == 0) return;
    CK(cudaMemsetAsync(sync, 0, (size_t)(1 + PP.nctr) * sizeof(unsigned int), st));
    dev::PersistLaunch L{};
    L.segs = PP.segs.p;
    L.sd = PP.sd.p;
    L.pd = PP.pd.p;
    L.sync = sync;
    L.err = err;
    L.nseg = PP.nseg;
    L.total_units = PP.total_units;
    L.tiles_per_warp = PP.tiles_per_warp;
    dev::k_step_persistent<kPersistMinBlocks>
        <<<(unsigned)persist_grid(sm_count, PP.total_units), dev::kPersistThreads, 0, st>>>(L);
    CK(cudaGetLastError());
    launches++;
}

// plain_path -1: times the three plain-cell paths (0 direct 32x8 tiles, 1 TMA
// pipeline for x-interior 32x8 tiles, 2 direct 8x4 warp tiles) over a few
// coarse steps from the initial state, puts the state back after each and
// keeps the fastest.
void autotune_plain_path(mgpu_ctx *ctx)
{
    std::vector<bool> had;
    for (auto &l : ctx->lv) had.push_back(l.has_tmap);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    checkpoint_save(ctx);
    const int64_t launches0 = ctx->launches;
    // the paths are timed with the GPU to themselves
    const int concurrent = ctx->prm.concurrent;
    ctx->prm.concurrent = 0;
    double us[3] = {0.0, 0.0, 0.0};
    auto select = [&](int path) {
        for (size_t l = 0; l < ctx->lv.size(); l++)
        {
            ctx->lv[l].has_tmap = path == 1 && had[l];
            ctx->lv[l].use8 = path == 2;
        }
        ctx->plan = build_plan({ctx}, -1);
    };
    for (int path = 0; path < 3; path++)
    {
        select(path);
        for (int i = 0; i < 2; i++) coarse_step(ctx, false, false, 0);
        const int n = 6;
        CK(cudaEventRecord(e0, ctx->stream));
        for (int i = 0; i < n; i++) coarse_step(ctx, false, false, 0);
        CK(cudaEventRecord(e1, ctx->stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        us[path] = ms * 1e3 / n;
        checkpoint_restore(ctx);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaEventDestroy(e0));
    CK(cudaEventDestroy(e1));
    int best = 0;
    for (int path = 1; path < 3; path++)
        if (us[path] < us[best]) best = path;
    select(best);
    for (int path = 0; path < 3; path++) ctx->autotune_us[path] = us[path];
    ctx->launches = launches0;
    ctx->prm.concurrent = concurrent;
    checkpoint_release(ctx);
}

void check_supported(mgpu_ctx *ctx)
{
    if (ctx->prm.simulation != MGPU_SIM_TRANSPORT && ctx->grid.max_level > 1)
        throw std::runtime_error("the adsorption step is single-block (include/mantiisApp.hpp:248-265 steps level 1 only)");
}
} // namespace

extern "C" {

void mgpu_default_params(mgpu_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->simulation = MGPU_SIM_TRANSPORT;
    p->collision = 2;
    p->wall = 2;
    p->multiblock = 0;
    p->max_allowed_level = 2;
    p->dx = 1.0e-9;
    p->fbody = 1.0e-8;
    p->T = 300.0;
    p->P = 2.0e6;
    p->tol = 1.0e-10;
    p->psi_form = 0;
    p->rho_psi = 1.0;
    p->g_ff = -1.0;
    p->g_fs = -12.7;
    p->rho_init = 0.0;
    p->rho_noise = 0.0;
    p->seed = 0;
    p->check_every = 1;
    p->edge_fine = 0;
    p->plain_path = -1;
    p->concurrent = 0;
}

static int create_impl(const PoreImage &img, const mgpu_params *p, mgpu_ctx **out)
{
    if (!p || !out) throw std::invalid_argument("null argument");
    if (p->collision < 0 || p->collision > 2)
        throw std::runtime_error("Incorrect keyword for collision: available options are\n\t 2 for regularized MRT\n"
                                 "\t 1 for simple MRT\n\t 0 for simple BGK\n");
    if (p->wall < 0 || p->wall > 2)
        throw std::runtime_error("Incorrect keyword for wall boundary method: available options are\n\t 2 for SRBBWall\n"
                                 "\t 1 for MDBBWall\n\t 0 for BBWall\n");
    if (p->simulation < 0 || p->simulation > 2) throw std::runtime_error("Unknown simulation type");
    if (p->check_every < 1) throw std::invalid_argument("check_every must be >= 1");
    std::unique_ptr<mgpu_ctx> ctx(new mgpu_ctx());
    ctx->prm = *p;
    ctx->units.Cl = p->dx;
    ctx->units.T_phy = p->T;
    ctx->units.P_phy = p->P;
    ctx->units.recompute();
    GridOptions go;
    go.multiblock = p->multiblock != 0;
    go.max_allowed_level = p->max_allowed_level;
    go.dx = p->dx;
    go.mfp = ctx->units.mfp;
    go.edge_fine = p->edge_fine != 0;
    ctx->grid = build_grid(img, go);
    if (ctx->grid.max_level > dev::kMaxLevels) throw std::runtime_error("too many refinement levels");
    ctx->adsorption = p->simulation != MGPU_SIM_TRANSPORT;
    ctx->coupled = p->simulation == MGPU_SIM_COUPLED;
    check_supported(ctx.get());

    double rho_init = p->rho_init > 0 ? p->rho_init : ctx->units.rhoin;
    ctx->rho0f = (float)rho_init;
    LayoutParams lp;
    lp.wall = p->wall;
    lp.collision = p->collision;
    lp.rho0 = (double)ctx->rho0f;
    lp.adsorption = p->simulation != MGPU_SIM_TRANSPORT;
    lp.mfp_over_cl = ctx->units.mfp / ctx->units.Cl;
    if (lp.adsorption)
    {
        // the adsorption loop calls the plain MRT and bounce-back directly
        lp.wall = WALL_BB;
        lp.collision = COLL_MRT;
    }
    ctx->lay = build_layout(ctx->grid, lp);
    ImageLayout lay_b; // coupling phase: SRBB wall coefficients and constants
    if (ctx->coupled)
    {
        LayoutParams lpb = lp;
        lpb.wall = WALL_SRBB;
        lpb.collision = COLL_RMRT;
        lay_b = build_layout(ctx->grid, lpb);
        if (lay_b.specials.size() != ctx->lay.specials.size())
            throw std::logic_error("coupled run: special records differ between the two wall modes");
        for (size_t i = 0; i < lay_b.specials.size(); i++)
            if (lay_b.specials[i].xy != ctx->lay.specials[i].xy)
                throw std::logic_error("coupled run: special records are ordered differently");
    }

    CK(cudaGetDevice(&ctx->device));
    CK(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device));
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
    ctx->lanes.create();
    upload_constants();
    cudaStream_t s = ctx->stream;
    int64_t &acct = ctx->bytes;
    ctx->lv.resize(ctx->lay.levels.size());
    for (size_t l = 0; l < ctx->lv.size(); l++)
    {
        const LevelLayout &ll = ctx->lay.levels[l];
        LevelDev &d = ctx->lv[l];
        d.f.alloc((size_t)ll.plane * 9, acct);
        d.f.zero(s);
        d.omega.upload(ll.omega, acct, s);
        if (p->plain_path != 0 && !ctx->adsorption && ll.n_tiles_interior > 0)
        {
            encode_level_map(&d.tmap, d.f.p, ll);
            encode_omega_map(&d.om_map, d.omega.p, ll);
            d.has_tmap = true;
        }
        d.spec.upload(ll.spec, acct, s);
        d.tiles.upload(ll.tile_list, acct, s);
        d.tile_mask.upload(ll.tile_mask, acct, s);
        d.tiles8.upload(ll.tile8_list, acct, s);
        d.tile8_mask.upload(ll.tile8_mask, acct, s);
        d.tile8_light.upload(ll.tile8_light, acct, s);
        d.use8 = p->plain_path == 2 && !ctx->adsorption;
        d.unorm.alloc((size_t)ll.plane, acct);
        d.unorm.zero(s);
        if (ll.snapshot_all || ctx->adsorption)
        {
            d.snap.alloc((size_t)ll.plane * 3, acct);
            d.snap.zero(s);
        }
        if (!ll.tau_d.empty()) d.tau2.upload(ll.tau_d, acct, s); // plain MRT: tau_d from Kn
        if (ctx->adsorption)
        {
            d.psi.alloc((size_t)ll.plane, acct);
            d.psi.zero(s);
            d.rho_prev.alloc((size_t)ll.plane, acct);
            d.rho_prev.zero(s);
        }
    }
    ctx->specials.upload(ctx->lay.specials, acct, s);
    ctx->ktab.upload(ctx->lay.ktab, acct, s);
    if (ctx->coupled)
    {
        ctx->specials_b.upload(lay_b.specials, acct, s);
        ctx->ktab_b.upload(lay_b.ktab, acct, s);
        CK(cudaStreamSynchronize(s)); // lay_b's host vectors go out of scope
    }
    ctx->side.alloc((size_t)ctx->lay.n_quirk * 2, acct);
    ctx->side.zero(s);
    ctx->ibuf.alloc((size_t)ctx->lay.n_buffers * 9, acct);
    ctx->ibuf.zero(s);
    ctx->cell_level.upload(ctx->lay.cell_level, acct, s);
    ctx->cell_site.upload(ctx->lay.cell_site, acct, s);
    {
        const std::vector<uint8_t> buf(ctx->grid.is_buffer.begin(), ctx->grid.is_buffer.end());
        ctx->cell_buffer.upload(buf, acct, s);
        CK(cudaStreamSynchronize(s)); // buf goes out of scope
    }
    ctx->red.alloc((size_t)(kRing + 2) * 4, acct); // the ring and two scratch slots
    ctx->red.zero(s);
    ctx->errword.alloc(1, acct);
    ctx->errword.zero(s);
    if (ctx->adsorption) ctx->ads_bar.alloc(1, acct);
    for (auto &it : ctx->lay.interfaces)
    {
        ctx->itf.emplace_back();
        InterfaceDev &e = ctx->itf.back();
        e.l1 = it.l1;
        e.ncoarse = (int)it.coarse.size();
        e.nfine = (int)it.fine.size();
        e.coarse.upload(it.coarse, acct, s);
        e.fine.upload(it.fine, acct, s);
    }

    if (!ctx->adsorption) ctx->plan = build_plan({ctx.get()}, -1);

    // initial state: rho = rho_init, u = 0, f = f_eq (include/coreLB.hpp:381-417)
    std::vector<double> rho(ctx->grid.n_cells, rho_init), zero(ctx->grid.n_cells, 0.0);
    if (p->rho_noise > 0)
    {
        std::mt19937_64 rng(p->seed);
        std::uniform_real_distribution<double> u(-p->rho_noise, p->rho_noise);
        for (auto &v : rho) v += u(rng);
    }
    DevBuf<double> dr, du, dv;
    int64_t tmp = 0;
    dr.upload(rho, tmp, s);
    du.upload(zero, tmp, s);
    dv.upload(zero, tmp, s);
    int64_t n = ctx->grid.n_cells;
    if (n > 0)
    {
        dev::k_set_equilibrium<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ctx->all(), ctx->common(), ctx->cell_level.p,
                                                                          ctx->cell_site.p, n, dr.p, du.p, dv.p);
        launch_check(ctx.get());
    }
    CK(cudaStreamSynchronize(s));
    if (p->plain_path < 0 && !ctx->adsorption) autotune_plain_path(ctx.get());
    *out = ctx.release();
    return MGPU_OK;
}

int mgpu_create(const int32_t *pore, const double *kn, const double *locpore, int n, const mgpu_params *p, mgpu_ctx **out)
{
    return guarded(nullptr, [&]() {
        if (!pore || !kn || !locpore || n <= 0) throw std::invalid_argument("null image or bad size");
        PoreImage img;
        img.n = n;
        img.pore.assign(pore, pore + (size_t)n * n);
        img.kn.assign(kn, kn + (size_t)n * n);
        img.locpore.assign(locpore, locpore + (size_t)n * n);
        return create_impl(img, p, out);
    });
}

int mgpu_create_from_folder(const char *folder, int n, const mgpu_params *p, mgpu_ctx **out)
{
    return guarded(nullptr, [&]() {
        if (!folder) throw std::invalid_argument("null folder");
        PoreImage img = load_pore_image(folder, n);
        return create_impl(img, p, out);
    });
}

int mgpu_destroy(mgpu_ctx *ctx)
{
    if (!ctx) return MGPU_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    if (ctx->run_graph) cudaGraphExecDestroy(ctx->run_graph);
    for (auto &kv : ctx->level_graphs) cudaGraphExecDestroy(kv.second.first);
    ctx->lanes.destroy();
    if (ctx->red_host) cudaFreeHost(ctx->red_host);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MGPU_OK;
}

int mgpu_get_info(const mgpu_ctx *ctx, mgpu_info *info)
{
    if (!ctx || !info) return fail(nullptr, MGPU_E_ARG, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->n = ctx->grid.n;
    info->max_level = ctx->grid.max_level;
    info->n_cells = ctx->grid.n_cells;
    int64_t nb = 0;
    for (auto v : ctx->grid.is_buffer) nb += v;
    info->n_buffer_cells = nb;
    info->n_special = (int64_t)ctx->lay.specials.size();
    info->lu_per_step = ctx->lay.lu_per_coarse_step;
    info->buffer_lu_per_step = ctx->lay.buffer_lu_per_coarse_step;
    info->rho_in = ctx->units.rhoin;
    info->mfp = ctx->units.mfp;
    info->tau_mean = ctx->lay.tau_mean;
    info->device_bytes = ctx->bytes;
    const GridDiagnostics &d = ctx->grid.diag;
    info->grid_undefined_cases =
        d.buffer_wall_links + d.fine_parent_missing_nbr + d.coarse_missing_child + d.fine_group_unmatched + d.pore_search_failed;
    bool tma = false;
    for (auto &l : ctx->lv) tma |= l.has_tmap;
    bool use8 = false;
    for (auto &l : ctx->lv) use8 |= l.use8;
    info->plain_path = use8 ? 2 : tma ? 1 : 0;
    for (int k = 0; k < 3; k++) info->autotune_us[k] = ctx->autotune_us[k];
    return MGPU_OK;
}

int mgpu_run(mgpu_ctx *ctx, int n_steps, int *steps_done)
{
    return guarded(ctx, [&]() {
        if (!ctx || n_steps < 0) throw std::invalid_argument("bad argument");
        const double tol = ctx->prm.tol;
        const int batch_max = 1000;
        int done = 0;
        bool broke = false;
        while (done < n_steps && !broke)
        {
            int batch = std::min(batch_max, n_steps - done);
            // a coupled run's adsorption phase ends after 100 steps or on the
            // residual test; batches do not cross that point
            const bool phase_a = ctx->coupled && !ctx->coupled_b;
            if (phase_a) batch = std::min(batch, 100 - ctx->coupled_a);
            checkpoint_save(ctx);
            int64_t k0 = ctx->coarse_done;
            run_batch_with_residuals(ctx, batch);
            std::vector<double> slots((size_t)batch * 4);
            read_slots(ctx, (int)((k0 + 1) % kRing), batch, slots.data());
            int stop = -1;
            for (int i = 0; i < batch; i++)
            {
                double d = residual_of(ctx, &slots[(size_t)i * 4]);
                ctx->residuals.push_back(d);
                if (d < tol)
                {
                    stop = i;
                    break;
                }
            }
            if (stop >= 0)
            {
                // the reference stops right after this step: replay up to it
                if (stop + 1 < batch)
                {
                    checkpoint_restore(ctx);
                    for (int i = 0; i <= stop; i++) coarse_step(ctx, false, true, 0);
                }
                done += stop + 1;
                ctx->ref_t += stop; // the breaking step is not counted (include/mantiisApp.hpp:302-350)
                if (phase_a) enter_coupling(ctx); // the break ends the adsorption phase only
                else broke = true;
            }
            else
            {
                done += batch;
                ctx->ref_t += batch;
                if (phase_a && ctx->coupled_a >= 100) enter_coupling(ctx);
            }
        }
        CK(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
        if (steps_done) *steps_done = done;
        return MGPU_OK;
    });
}

int mgpu_advance(mgpu_ctx *ctx, int n_steps)
{
    return guarded(ctx, [&]() {
        if (!ctx || n_steps < 0) throw std::invalid_argument("bad argument");
        const int K = ctx->prm.check_every;
        std::vector<int64_t> pending;
        auto flush = [&]() {
            if (pending.empty()) return;
            std::vector<double> v(pending.size() * 4);
            // consecutive slots in one read
            size_t a = 0;
            while (a < pending.size())
            {
                size_t b = a + 1;
                while (b < pending.size() && pending[b] == pending[b - 1] + 1 && (int)(b - a) < kRing) b++;
                read_slots(ctx, (int)(pending[a] % kRing), (int)(b - a), &v[a * 4]);
                a = b;
            }
            for (size_t i = 0; i < pending.size(); i++) ctx->residuals.push_back(residual_of(ctx, &v[i * 4]));
            pending.clear();
        };
        // with a residual every step, pairs of steps replay a CUDA graph (not for
        // coupled runs, whose phase switch is host-side, nor from the initial state)
        auto pairs_ok = [&](int i) { return K == 1 && !ctx->coupled && n_steps - i >= 2 && !fresh_state(ctx); };
        for (int i = 0; i < n_steps; i++)
        {
            int64_t k = ctx->coarse_done + 1;
            if (ctx->coupled && !ctx->coupled_b && ctx->coupled_a >= 100)
            {
                flush(); // residuals of the adsorption phase read as such
                enter_coupling(ctx);
            }
            if (ctx->adsorption)
            {
                if (K == 1 && ads_persistent_ok(ctx))
                {
                    // the rest of the call (as many steps as the pending slots hold) in one launch
                    const int m = std::min(n_steps - i, kRing / 2 - (int)pending.size());
                    zero_slots(ctx, (int)(k % kRing), m);
                    run_ads_persistent(ctx, m, k, true);
                    for (int j = 0; j < m; j++) pending.push_back(k + j);
                    i += m - 1;
                }
                else if (pairs_ok(i))
                {
                    run_pair_graph(ctx, false, (int)(k % kRing));
                    pending.push_back(k);
                    pending.push_back(k + 1);
                    i++;
                }
                else
                {
                    bool diff = (k % K == 0);
                    if (diff) zero_slots(ctx, (int)(k % kRing), 1);
                    coarse_step(ctx, diff, false, (int)((k % kRing) * 4));
                    if (diff) pending.push_back(k);
                }
                if ((int)pending.size() >= kRing / 2) flush();
                continue;
            }
            // residual of step s is evaluated by kernel s+1 against |u| stored by kernel s
            bool diff = k >= 2 && ((k - 1) % K == 0);
            bool store = (k % K == 0);
            if (diff && pairs_ok(i))
            {
                run_pair_graph(ctx, true, (int)((k - 1) % kRing));
                pending.push_back(k - 1);
                pending.push_back(k);
                i++;
            }
            else
            {
                int slot = (int)(((k - 1) % kRing) * 4);
                if (diff) zero_slots(ctx, (int)((k - 1) % kRing), 1);
                coarse_step(ctx, diff, store, slot);
                if (diff) pending.push_back(k - 1);
            }
            if ((int)pending.size() >= kRing / 2) flush();
        }
        flush();
        ctx->ref_t += n_steps;
        return MGPU_OK;
    });
}

int mgpu_advance_graph(mgpu_ctx *ctx, int n_steps)
{
    if (ctx && ctx->coupled) return mgpu_advance(ctx, n_steps); // its phase switch is host-side
    return guarded(ctx, [&]() {
        if (!ctx || n_steps < 0) throw std::invalid_argument("bad argument");
        if (ads_persistent_ok(ctx))
        {
            if (n_steps > 0) run_ads_persistent(ctx, n_steps, ctx->coarse_done + 1, false);
            ctx->ref_t += n_steps;
            return MGPU_OK;
        }
        int left = n_steps;
        // the graph starts from a stepped state (not the initial "direct" one)
        bool fresh = false;
        for (auto &l : ctx->lv) fresh |= l.steps == 0;
        if (fresh && left > 0)
        {
            coarse_step(ctx, false, false, 0);
            left--;
        }
        if (left >= 2 && ctx->graph && ctx->graph_key != state_key({ctx}, 0))
        {
            // captured at other step parities
            CK(cudaGraphExecDestroy(ctx->graph));
            ctx->graph = nullptr;
        }
        if (left >= 2 && !ctx->graph)
        {
            ctx->graph_key = state_key({ctx}, 0);
            // capture two coarse steps: every level then returns to its parity
            if (ctx->plan)
            {
                plan_variant(*ctx->plan, {ctx}, 0);
                plan_variant(*ctx->plan, {ctx}, 1);
            }
            std::vector<int64_t> saved;
            for (auto &l : ctx->lv) saved.push_back(l.steps);
            int64_t saved_done = ctx->coarse_done, saved_launch = ctx->launches;
            auto restore = [&]() {
                for (size_t l = 0; l < ctx->lv.size(); l++) ctx->lv[l].steps = saved[l];
                ctx->coarse_done = saved_done;
                ctx->launches = saved_launch;
            };
            cudaGraph_t g;
            try
            {
                StreamCapture cap(ctx->stream);
                coarse_step(ctx, false, false, 0);
                coarse_step(ctx, false, false, 0);
                g = cap.take();
            }
            catch (...)
            {
                restore();
                throw;
            }
            ctx->graph_launches = ctx->launches - saved_launch;
            restore();
            {
                const cudaError_t e_inst = cudaGraphInstantiate(&ctx->graph, g, 0);
                cudaGraphDestroy(g);
                CK(e_inst);
            }
        }
        while (left >= 2)
        {
            CK(cudaGraphLaunch(ctx->graph, ctx->stream));
            for (size_t l = 0; l < ctx->lv.size(); l++) ctx->lv[l].steps += 2 * ctx->lay.levels[l].substeps;
            ctx->coarse_done += 2;
            ctx->launches += ctx->graph_launches;
            left -= 2;
        }
        if (left == 1) coarse_step(ctx, false, false, 0);
        ctx->ref_t += n_steps;
        return MGPU_OK;
    });
}

int mgpu_set_engine(mgpu_ctx *ctx, int engine)
{
    return guarded(ctx, [&]() {
        if (!ctx || (engine != MGPU_ENGINE_STREAMS && engine != MGPU_ENGINE_PERSISTENT))
            throw std::invalid_argument("bad argument");
        ctx->engine = engine;
        return MGPU_OK;
    });
}

int mgpu_step_level(mgpu_ctx *ctx, int level, int n)
{
    return guarded(ctx, [&]() {
        if (!ctx || level < 1 || level > (int)ctx->lv.size() || n < 0) throw std::invalid_argument("bad argument");
        if (ctx->adsorption) throw std::logic_error("mgpu_step_level steps the transport kernels");
        const int l = level - 1;
        if ((int)ctx->level_plans.size() < level) ctx->level_plans.resize(level);
        if (!ctx->level_plans[l]) ctx->level_plans[l] = build_plan({ctx}, l);
        PhasePlan &P = *ctx->level_plans[l];
        const dev::PhaseArgs none{0, 0, 0};
        auto one = [&]() {
            PhaseVariant &V = plan_variant(P, {ctx}, 0);
            launch_phase(V, 0, none, ctx->stream, ctx->lanes, ctx->launches);
            ctx->lv[l].steps++;
        };
        int i = 0;
        if (n > 0 && ctx->lv[l].steps == 0)
        {
            one(); // from the initial state, outside the graphs
            i++;
        }
        // pairs of substeps (the level returns to its parity) replay a CUDA
        // graph, so timing them measures the GPU, not the host's launch rate
        while (n - i >= 2)
        {
            const std::string key = std::to_string(level) + ":" + state_key({ctx}, 0);
            auto it = ctx->level_graphs.find(key);
            if (it == ctx->level_graphs.end())
            {
                plan_variant(P, {ctx}, 0);
                ctx->lv[l].steps++;
                plan_variant(P, {ctx}, 0);
                ctx->lv[l].steps--;
                const int64_t saved = ctx->lv[l].steps, saved_launch = ctx->launches;
                cudaGraph_t g;
                try
                {
                    StreamCapture cap(ctx->stream);
                    one();
                    one();
                    g = cap.take();
                }
                catch (...)
                {
                    ctx->lv[l].steps = saved;
                    ctx->launches = saved_launch;
                    throw;
                }
                const int64_t captured = ctx->launches - saved_launch;
                ctx->lv[l].steps = saved;
                ctx->launches = saved_launch;
                cudaGraphExec_t exec = nullptr;
                const cudaError_t e_inst = cudaGraphInstantiate(&exec, g, 0);
                cudaGraphDestroy(g);
                CK(e_inst);
                it = ctx->level_graphs.emplace(key, std::make_pair(exec, captured)).first;
            }
            CK(cudaGraphLaunch(it->second.first, ctx->stream));
            ctx->lv[l].steps += 2;
            ctx->launches += it->second.second;
            i += 2;
        }
        if (i < n) one();
        return MGPU_OK;
    });
}

int mgpu_level_info(const mgpu_ctx *ctx, int level, int64_t out[4])
{
    if (!ctx || !out || level < 1 || level > (int)ctx->lay.levels.size()) return fail(nullptr, MGPU_E_ARG, "bad argument");
    const LevelLayout &ll = ctx->lay.levels[level - 1];
    out[0] = ll.n_active;
    out[1] = ll.n_active_real;
    out[2] = (int64_t)ll.tile_list.size();
    out[3] = ll.substeps;
    return MGPU_OK;
}

int mgpu_sync(mgpu_ctx *ctx)
{
    return guarded(ctx, [&]() {
        if (!ctx) throw std::invalid_argument("null context");
        CK(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
        return MGPU_OK;
    });
}

int mgpu_time(const mgpu_ctx *ctx, int64_t *t)
{
    if (!ctx || !t) return fail(nullptr, MGPU_E_ARG, "null argument");
    *t = ctx->ref_t;
    return MGPU_OK;
}

int mgpu_residuals(mgpu_ctx *ctx, double *out, int64_t cap, int64_t *count)
{
    if (!ctx) return fail(nullptr, MGPU_E_ARG, "null argument");
    int64_t n = (int64_t)ctx->residuals.size();
    if (count) *count = n;
    if (out)
        for (int64_t i = 0; i < std::min(cap, n); i++) out[i] = ctx->residuals[i];
    return MGPU_OK;
}

int mgpu_download_cells(mgpu_ctx *ctx, double *rho, double *ux, double *uy, double *f)
{
    return guarded(ctx, [&]() {
        if (!ctx) throw std::invalid_argument("null context");
        int64_t n = ctx->grid.n_cells;
        int64_t acct = 0;
        if (ctx->out_rho.n < (size_t)n)
        {
            ctx->out_rho.alloc(n, acct);
            ctx->out_ux.alloc(n, acct);
            ctx->out_uy.alloc(n, acct);
        }
        if (f && ctx->out_f.n < (size_t)n * 9) ctx->out_f.alloc((size_t)n * 9, acct);
        ctx->bytes += acct;
        cells_pass(ctx, ctx->out_rho.p, ctx->out_ux.p, ctx->out_uy.p, f ? ctx->out_f.p : nullptr, false, false, -1);
        if (rho) CK(cudaMemcpyAsync(rho, ctx->out_rho.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        if (ux) CK(cudaMemcpyAsync(ux, ctx->out_ux.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        if (uy) CK(cudaMemcpyAsync(uy, ctx->out_uy.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        if (f) CK(cudaMemcpyAsync(f, ctx->out_f.p, n * 72, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return MGPU_OK;
    });
}

int mgpu_download_pixels(mgpu_ctx *ctx, double *rho, double *ux, double *uy, double *f)
{
    return guarded(ctx, [&]() {
        if (!ctx) throw std::invalid_argument("null context");
        const Grid &g = ctx->grid;
        int64_t n = g.n_cells;
        std::vector<double> r(n), vx(n), vy(n), ff(f ? (size_t)n * 9 : 0);
        int rc = mgpu_download_cells(ctx, r.data(), vx.data(), vy.data(), f ? ff.data() : nullptr);
        if (rc) return rc;
        const size_t nn = (size_t)g.n * g.n;
        if (rho) std::fill(rho, rho + nn, 0.0);
        if (ux) std::fill(ux, ux + nn, 0.0);
        if (uy) std::fill(uy, uy + nn, 0.0);
        if (f) std::fill(f, f + nn * 9, 0.0);
        for (int64_t c = 0; c < n; c++)
        {
            if (g.is_buffer[c]) continue;
            int side = 1 << (g.level[c] - 1);
            for (int yy = g.y[c]; yy < g.y[c] + side; yy++)
                for (int xx = g.x[c]; xx < g.x[c] + side; xx++)
                {
                    size_t p = (size_t)yy * g.n + xx;
                    if (rho) rho[p] = r[c];
                    if (ux) ux[p] = vx[c];
                    if (uy) uy[p] = vy[c];
                    if (f)
                        for (int q = 0; q < 9; q++) f[p * 9 + q] = ff[(size_t)c * 9 + q];
                }
        }
        return MGPU_OK;
    });
}

int mgpu_observables(mgpu_ctx *ctx, double out[4])
{
    return guarded(ctx, [&]() {
        if (!ctx || !out) throw std::invalid_argument("null argument");
        const int slot = kRing - 1;
        zero_slots(ctx, slot, 1);
        cells_pass(ctx, nullptr, nullptr, nullptr, nullptr, false, false, slot * 4);
        double v[4];
        read_slot(ctx, slot, v);
        CK(cudaStreamSynchronize(ctx->stream));
        double npix = (double)ctx->grid.n * ctx->grid.n;
        double mean_ux = v[2] / npix;
        double nu = (ctx->lay.tau_mean - 0.5) / 3.0;
        out[0] = mean_ux;
        out[1] = ctx->prm.fbody != 0 ? mean_ux * nu / ctx->prm.fbody : 0.0;
        out[2] = v[3];
        out[3] = ctx->residuals.empty() ? 1.0 : ctx->residuals.back();
        return MGPU_OK;
    });
}

int mgpu_cell_positions(const mgpu_ctx *ctx, int32_t *x, int32_t *y, int32_t *level)
{
    if (!ctx) return fail(nullptr, MGPU_E_ARG, "null context");
    if (x) std::copy(ctx->grid.x.begin(), ctx->grid.x.end(), x);
    if (y) std::copy(ctx->grid.y.begin(), ctx->grid.y.end(), y);
    if (level) std::copy(ctx->grid.level.begin(), ctx->grid.level.end(), level);
    return MGPU_OK;
}

int mgpu_reconstructed(const mgpu_ctx *ctx, int64_t *out)
{
    if (!ctx || !out) return fail(nullptr, MGPU_E_ARG, "null argument");
    std::copy(ctx->grid.reconstructed.begin(), ctx->grid.reconstructed.end(), out);
    return MGPU_OK;
}

int mgpu_set_equilibrium(mgpu_ctx *ctx, const double *rho, const double *ux, const double *uy)
{
    return guarded(ctx, [&]() {
        if (!ctx || !rho || !ux || !uy) throw std::invalid_argument("null argument");
        const int64_t n = ctx->grid.n_cells;
        if (n == 0) return MGPU_OK;
        if (ctx->in_rho.n < (size_t)n)
        {
            int64_t acct = 0;
            ctx->in_rho.alloc(n, acct);
            ctx->in_ux.alloc(n, acct);
            ctx->in_uy.alloc(n, acct);
            ctx->bytes += acct;
        }
        // straight from the caller's buffers (fast when they are pinned); the
        // call returns after the copies, so the buffers are free again
        CK(cudaMemcpyAsync(ctx->in_rho.p, rho, n * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->in_ux.p, ux, n * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->in_uy.p, uy, n * 8, cudaMemcpyHostToDevice, ctx->stream));
        for (auto &l : ctx->lv) l.steps = 0;
        dev::k_set_equilibrium<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            ctx->all(), ctx->common(), ctx->cell_level.p, ctx->cell_site.p, n, ctx->in_rho.p, ctx->in_ux.p,
            ctx->in_uy.p);
        launch_check(ctx);
        CK(cudaStreamSynchronize(ctx->stream));
        return MGPU_OK;
    });
}

int mgpu_set_distributions(mgpu_ctx *ctx, const double *f, int layout, int64_t t)
{
    return guarded(ctx, [&]() {
        if (!ctx || !f) throw std::invalid_argument("null argument");
        if (layout != MGPU_LAYOUT_CELLS && layout != MGPU_LAYOUT_PIXELS)
            throw std::invalid_argument("mgpu_set_distributions: unknown layout " + std::to_string(layout));
        if (t < 0) throw std::invalid_argument("mgpu_set_distributions: negative time step");
        const Grid &g = ctx->grid;
        const int64_t n = g.n_cells;
        std::vector<double> cells((size_t)n * 9);
        if (layout == MGPU_LAYOUT_CELLS)
            std::copy(f, f + n * 9, cells.begin());
        else
            for (int64_t c = 0; c < n; c++)
            {
                const int64_t px = (int64_t)g.y[c] * g.n + g.x[c];
                std::copy(f + px * 9, f + px * 9 + 9, cells.begin() + c * 9);
            }
        for (double v : cells)
            if (!std::isfinite(v)) throw std::invalid_argument("mgpu_set_distributions: non-finite population");
        int64_t tmp = 0;
        DevBuf<double> df;
        df.upload(cells, tmp, ctx->stream);
        for (auto &l : ctx->lv) l.steps = 0;
        dev::k_set_distributions<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            ctx->all(), ctx->common(), ctx->cell_level.p, ctx->cell_site.p, n, df.p);
        launch_check(ctx);
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->ref_t = t;
        ctx->residuals.clear();
        ctx->ckpt.valid = false;
        if (ctx->coupled)
        {
            // the first 100 steps of a coupled run are adsorption steps
            ctx->coupled_a = (int)std::min<int64_t>(t, 100);
            ctx->coupled_b = t >= 100;
            ctx->last_step_b = t > 100;
        }
        return MGPU_OK;
    });
}

} // extern "C"

namespace
{
// Staging area of mgpu_set_equilibrium_noalloc: rho, u_x, u_y of up to
// MGPU_NOALLOC_MAX_CELLS cells (3 x 8 MiB), part of the module image, so it exists
// once per device and no call allocates it.  Nothing in it has to start at zero:
// each call writes the 3 n values its kernel reads before the kernel runs.
__device__ __align__(256) double g_noalloc_stage[3 * (size_t)MGPU_NOALLOC_MAX_CELLS];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
struct NoallocSlot
{
    unsigned long long context_id = 0; // CUDA context the address belongs to (0 = none yet)
    double *ptr = nullptr;
};
NoallocSlot g_noalloc_slot[kMaxDevices];

// Process-unique id of the CUDA context bound to the calling thread (cuCtxGetId,
// through the runtime's entry-point query).  Ids are never reused, unlike context
// handles: a primary context re-created after cudaDeviceReset gets a new id.
// Returns false when no context is bound to the thread yet.
bool current_context_id(unsigned long long *id)
{
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    if (!get_current || !get_id)
    {
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1 = cudaDriverEntryPointSymbolNotFound, r2 = r1;
        CK(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &r1));
        CK(cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2));
        if (r1 != cudaDriverEntryPointSuccess || r2 != cudaDriverEntryPointSuccess || !p || !q)
            throw CudaError("cuCtxGetCurrent / cuCtxGetId are not available");
        get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(q);
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return false;
    return get_id(c, id) == CUDA_SUCCESS;
}

// The array's device address in the context current on `device`.  It is looked
// up (cudaGetSymbolAddress, which may load the module) once per CUDA context and
// kept with that context's id, so a context created after cudaDeviceReset, whose
// module may sit at another address, gets its own lookup.
double *noalloc_stage(int device)
{
    if (device < 0 || device >= kMaxDevices) throw std::invalid_argument("device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocSlot &s = g_noalloc_slot[device];
    unsigned long long id = 0;
    if (current_context_id(&id) && s.ptr && s.context_id == id) return s.ptr;
    void *p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_stage)); // binds the device's primary context to this thread
    if (!current_context_id(&id)) throw CudaError("no CUDA context is current after cudaGetSymbolAddress");
    s.context_id = id;
    s.ptr = static_cast<double *>(p);
    return s.ptr;
}
} // namespace

extern "C" {

int mgpu_pore_properties_gpu(const int32_t *pore, int n, double dx, double mfp, double *locpore, double *kn,
                             int64_t *iterations, void *stream)
{
    try
    {
        gpu_pore_properties(pore, n, dx, mfp, locpore, kn, iterations, static_cast<cudaStream_t>(stream));
        return MGPU_OK;
    }
    catch (const std::invalid_argument &e)
    {
        return fail(nullptr, MGPU_E_ARG, e.what());
    }
    catch (const std::exception &e)
    {
        return fail(nullptr, is_geometry_cuda_error(e) ? MGPU_E_CUDA : MGPU_E_ARG, e.what());
    }
}

int mgpu_set_equilibrium_noalloc(mgpu_ctx *ctx, const double *rho, const double *ux, const double *uy)
{
    return guarded(ctx, [&]() {
        if (!ctx || !rho || !ux || !uy) throw std::invalid_argument("null argument");
        const int64_t n = ctx->grid.n_cells;
        if (n > MGPU_NOALLOC_MAX_CELLS)
            throw std::length_error("mgpu_set_equilibrium_noalloc: " + std::to_string(n) +
                                        " cells exceed the static staging area of " +
                                        std::to_string(MGPU_NOALLOC_MAX_CELLS) + " cells");
        int prev = -1;
        CK(cudaGetDevice(&prev));
        if (prev != ctx->device)
            throw std::logic_error("mgpu_set_equilibrium_noalloc: the context's device is not current");
        double *stage = noalloc_stage(ctx->device);
        if (n == 0) return MGPU_OK;
        double *dr = stage, *du = stage + MGPU_NOALLOC_MAX_CELLS, *dv = stage + 2 * (size_t)MGPU_NOALLOC_MAX_CELLS;
        CK(cudaMemcpyAsync(dr, rho, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(du, ux, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(dv, uy, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        for (auto &l : ctx->lv) l.steps = 0;
        dev::k_set_equilibrium<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            ctx->all(), ctx->common(), ctx->cell_level.p, ctx->cell_site.p, n, dr, du, dv);
        launch_check(ctx);
        // the staging area is free for the next call once this returns
        CK(cudaStreamSynchronize(ctx->stream));
        return MGPU_OK;
    });
}

int mgpu_set_stream(mgpu_ctx *ctx, void *stream)
{
    return guarded(ctx, [&]() {
        if (!ctx) throw std::invalid_argument("null context");
        CK(cudaStreamSynchronize(ctx->stream));
        if (ctx->own_stream) CK(cudaStreamDestroy(ctx->stream));
        if (ctx->graph)
        {
            CK(cudaGraphExecDestroy(ctx->graph));
            ctx->graph = nullptr;
        }
        if (stream)
        {
            ctx->stream = (cudaStream_t)stream;
            ctx->own_stream = false;
        }
        else
        {
            CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
        return MGPU_OK;
    });
}

int64_t mgpu_launch_count(const mgpu_ctx *ctx) { return ctx ? ctx->launches : 0; }
} // extern "C"

// A group of transport contexts stepped together: each phase of a coarse step
// is one launch over all images, each interface wave one launch.
struct mgpu_batch
{
    std::vector<mgpu_ctx *> ctxs;
    std::unique_ptr<PhasePlan> plan;
    cudaStream_t stream = nullptr;
    SideLanes lanes;
    bool own_stream = false;
    cudaEvent_t ev_done = nullptr;
    // images step on a few concurrent streams (each with its own side lanes),
    // image i on stream i % streams, forked from and joined back to `stream`
    // around their coarse steps
    std::vector<cudaStream_t> img_stream;
    std::vector<SideLanes> img_lanes;
    std::vector<cudaEvent_t> img_done;
    cudaEvent_t ev_start = nullptr;
    std::vector<cudaEvent_t> ctx_ev;
    cudaGraphExec_t graph = nullptr;
    std::string graph_key;
    int64_t graph_launches = 0, launches = 0;
    // engine 1: every coarse step (two inside the graph) is one persistent
    // launch over all images (dev::k_step_persistent), images interleaved in
    // groups of `group` (0: all); engine 0: per-image phase launches on the
    // concurrent streams above
    // 8x4 tiles per warp of a plain-cell unit of the persistent kernel (config-2
    // batch of 4 at 5 blocks per SM: 4 -> 408 us per coarse step, 2 -> 443, 1 -> 459;
    // at 4 blocks per SM 436, at 3 630)
    int engine = 0, group = 0, tiles_per_warp = 4;
    std::map<std::string, std::unique_ptr<PersistPlan>> pplans;
    DevBuf<unsigned int> sync; // claim and stage counters of the persistent launch
    int64_t bytes = 0;
    int sm_count = 1;
};

namespace
{
// the batch's work starts after each context's earlier work ...
void batch_enter(mgpu_batch *b)
{
    for (size_t i = 0; i < b->ctxs.size(); i++)
        if (b->ctxs[i]->stream != b->stream)
        {
            CK(cudaEventRecord(b->ctx_ev[i], b->ctxs[i]->stream));
            CK(cudaStreamWaitEvent(b->stream, b->ctx_ev[i], 0));
        }
}
// ... and each context's later work starts after the batch's
void batch_leave(mgpu_batch *b)
{
    CK(cudaEventRecord(b->ev_done, b->stream));
    for (auto *c : b->ctxs)
        if (c->stream != b->stream) CK(cudaStreamWaitEvent(c->stream, b->ev_done, 0));
}

// the persistent plan of the batch's current state for n coarse steps
PersistPlan &batch_persist_plan(mgpu_batch *b, int n)
{
    const std::string key = state_key(b->ctxs, 0) + "/" + std::to_string(n);
    auto it = b->pplans.find(key);
    if (it != b->pplans.end()) return *it->second;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(b->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) throw std::logic_error("persistent plan missing during graph capture");
    std::unique_ptr<PersistPlan> PP(new PersistPlan());
    build_persist(*PP, b->ctxs, 0, n, b->group, b->tiles_per_warp, b->stream);
    if ((size_t)(1 + PP->nctr) > b->sync.n) throw std::logic_error("persistent plan: too many stage counters");
    b->bytes += PP->bytes;
    return *b->pplans.emplace(key, std::move(PP)).first->second;
}

// n coarse steps of every image: each image on its own stream with its own
// phase launches, so that one image's small launches (interface waves, the
// sparse coarse levels) overlap another's; images share no data.  With the
// persistent engine: one launch for the n steps of all images.
void batch_step(mgpu_batch *b, int n = 1)
{
    const dev::PhaseArgs none{0, 0, 0};
    if (b->engine == 1)
    {
        PersistPlan &PP = batch_persist_plan(b, n);
        launch_persist(PP, b->sync.p, b->ctxs[0]->errword.p, b->sm_count, b->stream, b->launches);
        for (auto *c : b->ctxs)
        {
            for (size_t l = 0; l < c->lv.size(); l++) c->lv[l].steps += (int64_t)n * c->lay.levels[l].substeps;
            c->coarse_done += n;
            c->ref_t += n;
        }
        return;
    }
    if (b->img_stream.empty())
    {
        for (int k = 0; k < n; k++) phase_step(*b->plan, b->ctxs, b->stream, b->lanes, none, b->launches);
    }
    else
    {
        CK(cudaEventRecord(b->ev_start, b->stream));
        const size_t ns = b->img_stream.size();
        for (size_t j = 0; j < ns; j++) CK(cudaStreamWaitEvent(b->img_stream[j], b->ev_start, 0));
        for (size_t i = 0; i < b->ctxs.size(); i++)
            for (int k = 0; k < n; k++)
                phase_step(*b->ctxs[i]->plan, {b->ctxs[i]}, b->img_stream[i % ns], b->img_lanes[i % ns], none,
                           b->launches, ns > 1);
        for (size_t j = 0; j < ns; j++)
        {
            CK(cudaEventRecord(b->img_done[j], b->img_stream[j]));
            CK(cudaStreamWaitEvent(b->stream, b->img_done[j], 0));
        }
    }
    for (auto *c : b->ctxs) c->ref_t += n;
}
} // namespace

extern "C" {

int mgpu_batch_create(mgpu_ctx *const *ctxs, int n, mgpu_batch **out)
{
    return guarded(nullptr, [&]() {
        if (!ctxs || n <= 0 || !out) throw std::invalid_argument("bad argument");
        std::unique_ptr<mgpu_batch> b(new mgpu_batch());
        int dev = -1;
        CK(cudaGetDevice(&dev));
        for (int i = 0; i < n; i++)
        {
            mgpu_ctx *c = ctxs[i];
            if (!c) throw std::invalid_argument("null context in batch");
            if (c->adsorption || !c->plan) throw std::invalid_argument("a batch steps transport contexts only");
            if (c->device != dev) throw std::invalid_argument("batch contexts must live on the current device");
            for (int k = 0; k < i; k++)
                if (ctxs[k] == c) throw std::invalid_argument("context listed twice in batch");
            b->ctxs.push_back(c);
        }
        b->plan = build_plan(b->ctxs, -1);
        CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        b->own_stream = true;
        b->lanes.create();
        CK(cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming));
        // concurrent streams: as many images as fit twice the L2 together (at
        // least 2: one image's small launches then overlap another's work; more
        // large images at once evict each other's levels from L2 -- config-2
        // images, ~110 MB each: 2 streams 13.4 k MLUPS, 4 or 8 streams 12.2 k)
        int l2 = 0;
        CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
        int64_t bytes = 0;
        for (auto *c : b->ctxs) bytes += c->bytes;
        const double per = (double)bytes / (double)b->ctxs.size();
        const int streams = (int)std::max<double>(2.0, std::min<double>((double)b->ctxs.size(),
                                                                        std::floor(2.0 * l2 / std::max(per, 1.0))));
        if (b->ctxs.size() > 1)
        {
            CK(cudaEventCreateWithFlags(&b->ev_start, cudaEventDisableTiming));
            b->img_stream.resize((size_t)streams);
            b->img_lanes.resize((size_t)streams);
            b->img_done.resize((size_t)streams);
            for (int i = 0; i < streams; i++)
            {
                CK(cudaStreamCreateWithFlags(&b->img_stream[i], cudaStreamNonBlocking));
                b->img_lanes[i].create();
                CK(cudaEventCreateWithFlags(&b->img_done[i], cudaEventDisableTiming));
            }
        }
        b->ctx_ev.resize(b->ctxs.size());
        for (auto &e : b->ctx_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->sm_count = b->ctxs[0]->sm_count;
        // stage counters of two coarse steps: at most 2^(L-1) phases and L waves
        // per image and step (L <= 4)
        b->sync.alloc(1 + b->ctxs.size() * 2 * (8 + 4), b->bytes);
        *out = b.release();
        return MGPU_OK;
    });
}

int mgpu_batch_advance(mgpu_batch *b, int n_steps)
{
    return guarded(nullptr, [&]() {
        if (!b || n_steps < 0) throw std::invalid_argument("bad argument");
        batch_enter(b);
        int left = n_steps;
        // the graph starts from a stepped state (not the initial "direct" one)
        bool fresh = false;
        for (auto *c : b->ctxs)
            for (auto &l : c->lv) fresh |= l.steps == 0;
        if (fresh && left > 0)
        {
            batch_step(b);
            left--;
        }
        if (left >= 2 && b->graph && b->graph_key != state_key(b->ctxs, 0))
        {
            CK(cudaGraphExecDestroy(b->graph));
            b->graph = nullptr;
        }
        if (left >= 2 && !b->graph)
        {
            // two coarse steps: every level of every image returns to its parity
            if (b->engine == 1) batch_persist_plan(b, 2);
            plan_variant(*b->plan, b->ctxs, 0);
            plan_variant(*b->plan, b->ctxs, 1);
            for (auto *c : b->ctxs)
            {
                plan_variant(*c->plan, {c}, 0);
                plan_variant(*c->plan, {c}, 1);
            }
            b->graph_key = state_key(b->ctxs, 0);
            std::vector<std::vector<int64_t>> saved;
            std::vector<int64_t> saved_done, saved_t;
            for (auto *c : b->ctxs)
            {
                saved.emplace_back();
                for (auto &l : c->lv) saved.back().push_back(l.steps);
                saved_done.push_back(c->coarse_done);
                saved_t.push_back(c->ref_t);
            }
            const int64_t l0 = b->launches;
            // capturing advances the host-side step counters; put them back either way
            auto restore = [&]() {
                b->launches = l0;
                for (size_t i = 0; i < b->ctxs.size(); i++)
                {
                    for (size_t l = 0; l < b->ctxs[i]->lv.size(); l++) b->ctxs[i]->lv[l].steps = saved[i][l];
                    b->ctxs[i]->coarse_done = saved_done[i];
                    b->ctxs[i]->ref_t = saved_t[i];
                }
            };
            cudaGraph_t g;
            try
            {
                StreamCapture cap(b->stream);
                batch_step(b, 2);
                g = cap.take();
            }
            catch (...)
            {
                restore();
                b->graph_key.clear();
                throw;
            }
            b->graph_launches = b->launches - l0;
            restore();
            {
                const cudaError_t e_inst = cudaGraphInstantiate(&b->graph, g, 0);
                cudaGraphDestroy(g);
                CK(e_inst);
            }
        }
        while (left >= 2)
        {
            CK(cudaGraphLaunch(b->graph, b->stream));
            for (auto *c : b->ctxs)
            {
                for (size_t l = 0; l < c->lv.size(); l++) c->lv[l].steps += 2 * c->lay.levels[l].substeps;
                c->coarse_done += 2;
                c->ref_t += 2;
            }
            b->launches += b->graph_launches;
            left -= 2;
        }
        if (left == 1) batch_step(b);
        batch_leave(b);
        return MGPU_OK;
    });
}

int mgpu_batch_observables(mgpu_batch *b, double *out)
{
    return guarded(nullptr, [&]() {
        if (!b || !out) throw std::invalid_argument("null argument");
        batch_enter(b);
        const int slot = kRing - 1;
        std::vector<double> v(4 * b->ctxs.size());
        for (size_t i = 0; i < b->ctxs.size(); i++)
        {
            mgpu_ctx *c = b->ctxs[i];
            CK(cudaMemsetAsync(c->red.p + (size_t)slot * 4, 0, 4 * sizeof(double), b->stream));
            cells_pass(c, nullptr, nullptr, nullptr, nullptr, false, false, slot * 4, b->stream);
            CK(cudaMemcpyAsync(&v[4 * i], c->red.p + (size_t)slot * 4, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                               b->stream));
        }
        CK(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < b->ctxs.size(); i++)
        {
            const mgpu_ctx *c = b->ctxs[i];
            const double npix = (double)c->grid.n * c->grid.n;
            const double mean_ux = v[4 * i + 2] / npix;
            const double nu = (c->lay.tau_mean - 0.5) / 3.0;
            out[4 * i + 0] = mean_ux;
            out[4 * i + 1] = c->prm.fbody != 0 ? mean_ux * nu / c->prm.fbody : 0.0;
            out[4 * i + 2] = v[4 * i + 3];
            out[4 * i + 3] = c->residuals.empty() ? 1.0 : c->residuals.back();
        }
        return MGPU_OK;
    });
}

int mgpu_batch_set_stream(mgpu_batch *b, void *stream)
{
    return guarded(nullptr, [&]() {
        if (!b) throw std::invalid_argument("null batch");
        CK(cudaStreamSynchronize(b->stream));
        if (b->own_stream) CK(cudaStreamDestroy(b->stream));
        if (b->graph)
        {
            CK(cudaGraphExecDestroy(b->graph));
            b->graph = nullptr;
        }
        if (stream)
        {
            b->stream = (cudaStream_t)stream;
            b->own_stream = false;
        }
        else
        {
            CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
            b->own_stream = true;
        }
        return MGPU_OK;
    });
}

int mgpu_batch_sync(mgpu_batch *b)
{
    return guarded(nullptr, [&]() {
        if (!b) throw std::invalid_argument("null batch");
        CK(cudaStreamSynchronize(b->stream));
        for (auto *c : b->ctxs) check_device_error(c);
        return MGPU_OK;
    });
}

int mgpu_batch_set_engine(mgpu_batch *b, int engine, int group)
{
    return guarded(nullptr, [&]() {
        if (!b || engine < 0 || engine > 1 || group < 0) throw std::invalid_argument("bad argument");
        if (engine == b->engine && group == b->group) return MGPU_OK;
        CK(cudaStreamSynchronize(b->stream));
        if (b->graph)
        {
            CK(cudaGraphExecDestroy(b->graph));
            b->graph = nullptr;
        }
        b->graph_key.clear();
        if (group != b->group) b->pplans.clear();
        b->engine = engine;
        b->group = group;
        return MGPU_OK;
    });
}

int64_t mgpu_batch_launch_count(const mgpu_batch *b) { return b ? b->launches : 0; }

int mgpu_batch_destroy(mgpu_batch *b)
{
    if (!b) return MGPU_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->lanes.destroy();
    for (size_t i = 0; i < b->img_stream.size(); i++)
    {
        if (b->img_stream[i])
        {
            cudaStreamSynchronize(b->img_stream[i]);
            cudaStreamDestroy(b->img_stream[i]);
        }
        b->img_lanes[i].destroy();
        if (b->img_done[i]) cudaEventDestroy(b->img_done[i]);
    }
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    for (auto e : b->ctx_ev) cudaEventDestroy(e);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MGPU_OK;
}


const char *mgpu_last_error(const mgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : g_error.c_str(); }
const char *mgpu_global_error(void) { return g_error.c_str(); }

} // extern "C"
