/*
 * CPU oracle driver around the reference solver's own, unmodified classes
 * (Shape, Grid2D, LB2D from include/*.hpp).  Test infrastructure only: it is
 * built by oracle/Makefile into oracle/_ref/ and is never part of the product.
 *
 * It replays MantiisApp::init (include/mantiisApp.hpp:158-237) and the run
 * loop (include/mantiisApp.hpp:294-352, transport/adsorption/coupled step
 * bodies at :239-284), but instead of only the pixel fields it also dumps the
 * per-cell grid tables, link lists and state in grid order, which the
 * parity tests compare against.  It additionally times the stepping loop alone.
 *
 * Usage:
 *   ref_driver <num_threads> <is_multiblock> <Nx> <input_folder/> <Nt>
 *              [--mode transport|adsorption|coupled] [--dx v] [--fbody v]
 *              [--T v] [--P v] [--collision 0|1|2] [--wall 0|1|2] [--tol v]
 *              [--dump dir] [--dump-steps a,b,c] [--no-break] [--quiet]
 *   --mode properties --mfp v --dx v --dump dir: only Shape::calculateProperties
 *              (include/shape.hpp:127-251) on pore.dat; writes dir/properties.bin
 *              (LocPore then Kn, row-major [row][column], as length-prefixed
 *              float64 vectors).
 */
#include <omp.h>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "mantiisApp.hpp"

namespace
{
template <typename T> void put(std::ofstream &o, const T &v) { o.write((const char *)&v, sizeof(T)); }
template <typename T> void putv(std::ofstream &o, const std::vector<T> &v)
{
    int64_t n = (int64_t)v.size();
    put(o, n);
    if (n) o.write((const char *)v.data(), sizeof(T) * n);
}

void dump_grid(const std::string &dir, Grid2D &g, LB2D &lb)
{
    std::ofstream o(dir + "/grid.bin", std::ios::binary);
    int64_t n = g.globalGridSize;
    put(o, n);
    put(o, (int32_t)g.maxLevel);
    std::vector<int32_t> ij(2 * n), conn32;
    std::vector<int64_t> conn(9 * n);
    for (int64_t i = 0; i < n; i++)
    {
        ij[2 * i] = g.gridIJ[i][0];
        ij[2 * i + 1] = g.gridIJ[i][1];
        for (int q = 0; q < 9; q++) conn[9 * i + q] = g.gridConnect[i][q];
    }
    putv(o, ij);
    putv(o, std::vector<int32_t>(g.gridLevel.begin(), g.gridLevel.end()));
    putv(o, std::vector<int32_t>(g.gridType.begin(), g.gridType.end()));
    putv(o, std::vector<int32_t>(g.gridIsBuffer.begin(), g.gridIsBuffer.end()));
    putv(o, std::vector<int32_t>(g.bndTypes.begin(), g.bndTypes.end()));
    putv(o, conn);
    putv(o, lb.taus);
    putv(o, g.kn);
    putv(o, g.locpore);
    putv(o, g.gridID);
    putv(o, lb.streamID);
    putv(o, std::vector<int32_t>(lb.streamIC.begin(), lb.streamIC.end()));
    putv(o, lb.streamLOC);
    putv(o, lb.boundaryID);
    putv(o, std::vector<int32_t>(lb.boundaryIC.begin(), lb.boundaryIC.end()));
    putv(o, lb.periodicID);
    putv(o, lb.periodicI2);
    putv(o, std::vector<int32_t>(lb.periodicIC.begin(), lb.periodicIC.end()));
    // interface tables: for each buffer type key, rows of 5 ids
    std::vector<int64_t> cb, fb;
    for (int lvl = g.maxLevel; lvl >= 2; lvl--)
    {
        int key = 10 * lvl + lvl - 1;
        for (auto &row : g.coarseBuffer[key])
        {
            cb.push_back(key);
            for (auto v : row) cb.push_back(v);
        }
    }
    for (int lvl = 1; lvl < g.maxLevel; lvl++)
    {
        int key = 10 * lvl + lvl + 1;
        for (auto &row : g.fineBuffer[key])
        {
            fb.push_back(key);
            for (auto v : row) fb.push_back(v);
        }
    }
    putv(o, cb);
    putv(o, fb);
    std::vector<int64_t> pc;
    for (auto &row : g.gridParentChild)
        for (auto v : row) pc.push_back(v);
    putv(o, pc);
}

void dump_state(const std::string &dir, int step, LB2D &lb)
{
    std::ofstream o(dir + "/state_" + std::to_string(step) + ".bin", std::ios::binary);
    put(o, (int64_t)step);
    putv(o, lb.rho);
    putv(o, lb.ux);
    putv(o, lb.uy);
    putv(o, lb.f);
    putv(o, lb.diff_over_time);
}
} // namespace

int main(int argc, char *argv[])
{
    if (argc < 6)
    {
        std::fprintf(stderr, "Usage: %s <num_threads> <is_multiblock> <Nx> <input_folder/> <Nt> [options]\n", argv[0]);
        return 1;
    }
    Settings settings;
    settings.verbose = 1000000000;
    settings.dump_macroscopic_every_timestep = 1000000;
    settings.dump_distributions_first_timestep = -1;
    std::string mode = "transport", dumpdir;
    std::set<int> dump_steps;
    bool nobreak = false, quiet = false;
    double props_mfp = 0.0;
    settings.dx = 1.0e-9;
    settings.Fbody = 1.0e-8;
    for (int a = 6; a < argc; a++)
    {
        std::string k = argv[a];
        auto next = [&]() -> std::string {
            if (a + 1 >= argc) throw std::runtime_error("missing value for " + k);
            return argv[++a];
        };
        if (k == "--mode") mode = next();
        else if (k == "--dx") settings.dx = std::stod(next());
        else if (k == "--fbody") settings.Fbody = std::stod(next());
        else if (k == "--T") settings.T = std::stod(next());
        else if (k == "--P") settings.P = std::stod(next());
        else if (k == "--collision") settings.collision_method = std::stoi(next());
        else if (k == "--wall") settings.wall_boundary = std::stoi(next());
        else if (k == "--tol") settings.threshold = std::stod(next());
        else if (k == "--mfp") props_mfp = std::stod(next());
        else if (k == "--dump") dumpdir = next();
        else if (k == "--dump-steps")
        {
            std::stringstream ss(next());
            std::string tok;
            while (std::getline(ss, tok, ',')) dump_steps.insert(std::stoi(tok));
        }
        else if (k == "--no-break") nobreak = true;
        else if (k == "--quiet") quiet = true;
        else throw std::runtime_error("unknown option " + k);
    }
    if (quiet) std::cout.setstate(std::ios::failbit);

    // ---- MantiisApp constructor (include/mantiisApp.hpp:109-156)
    _GLOBAL_::mfp = settings.mfp;
    _GLOBAL_::Fbody = settings.Fbody;
    _GLOBAL_::Cl = settings.dx;
    _GLOBAL_::T_phy = settings.T;
    _GLOBAL_::P_phy = settings.P;
    _GLOBAL_::recompute();
    int num_threads = std::stoi(argv[1]);
    bool is_multiblock = (std::string(argv[2]) == "true");
    int Nx = std::stoi(argv[3]), Ny = Nx;
    std::string folder = argv[4];
    int iters = std::stoi(argv[5]);
    int proc_id, num_procs;
    mantiis_parallel::launchMPI(proc_id, num_procs, num_threads);

    // ---- MantiisApp::init (include/mantiisApp.hpp:158-237)
    Shape shape(Nx, Ny, _GLOBAL_::Cl);
    shape.loadExistingModel(folder);
    if (mode == "properties")
    {
        shape.calculateProperties(settings.dx, props_mfp);
        std::ofstream o(dumpdir + "/properties.bin", std::ios::binary);
        std::vector<double> lp, kn;
        for (int i = 0; i < Ny; i++)
            for (int j = 0; j < Nx; j++)
            {
                lp.push_back(shape.LocPore[i][j]);
                kn.push_back(shape.Kn[i][j]);
            }
        putv(o, lp);
        putv(o, kn);
        return 0;
    }
    lattice latt;
    Grid2D grid(shape, latt, is_multiblock);
    auto t_setup0 = std::chrono::steady_clock::now();
    grid.initialize(shape);
    grid.MPI_distributeGridData();
    LB2D lb(Nx, Ny, latt, grid, shape);
    lb.initialize();
    auto t_setup1 = std::chrono::steady_clock::now();
    switch (settings.collision_method)
    {
    case 2: lb.setCollision(&LB2D::MRTCollisionRegularized); break;
    case 1: lb.setCollision(&LB2D::MRTCollisionNonRegularized); break;
    case 0: lb.setCollision(&LB2D::SRTCollision); break;
    default: throw std::runtime_error("bad collision method");
    }
    switch (settings.wall_boundary)
    {
    case 2: lb.setWallBoundary(&LB2D::SRBBWall); break;
    case 1: lb.setWallBoundary(&LB2D::MDBBWall); break;
    case 0: lb.setWallBoundary(&LB2D::BBWall); break;
    default: throw std::runtime_error("bad wall boundary");
    }
    lb.setOpenBoundary(&LB2D::periodicBoundary);
    if (!dumpdir.empty())
    {
        dump_grid(dumpdir, grid, lb);
        if (dump_steps.count(0)) dump_state(dumpdir, 0, lb);
    }

    // ---- step bodies (include/mantiisApp.hpp:239-284)
    auto transport = [&]() {
        lb.usq_old = lb.usq;
        lb.equilibrium();
        lb.evolutionStepOfMultiBlock(lb.grid.maxLevel);
        lb.calculateMacroscopicPorperties();
        lb.calculateVelocityDifference();
    };
    auto adsorption = [&]() {
        lb.rho_old = lb.rho;
        lb.calculateDensity();
        lb.getPseudoPotential();
        lb.calculateForces();
        lb.calculateVelocity();
        lb.equilibrium();
        lb.MRTCollisionNonRegularized();
        lb.applySourceTerm();
        lb.ftemp = lb.f;
        lb.zeroDown();
        lb.stream();
        lb.BBWall();
        lb.periodicBoundary();
        lb.generalizedPeriodicBoundaryAdsorption();
        lb.calculateDensityDifference();
    };
    auto coupled = [&]() {
        lb.rho_old = lb.rho;
        lb.calculateDensity();
        lb.getPseudoPotential();
        lb.calculateForces();
        lb.calculateVelocity();
        lb.equilibrium();
        lb.MRTCollisionRegularized();
        lb.applySourceTerm();
        lb.ftemp = lb.f;
        lb.zeroDown();
        lb.stream();
        lb.SRBBWall();
        lb.periodicBoundary();
        lb.calculateVelocityDifference();
    };

    // ---- run loop (include/mantiisApp.hpp:294-352); steps counted 1.. for dumps
    int64_t done = 0;
    auto run_loop = [&](auto step, int n) {
        for (int i = 0; i < n; i++)
        {
            step();
            done++;
            if (!dumpdir.empty() && dump_steps.count((int)done)) dump_state(dumpdir, (int)done, lb);
            if (!nobreak && lb.diff < settings.threshold) break;
            lb.t++;
        }
    };
    auto t0 = std::chrono::steady_clock::now();
    if (mode == "transport") run_loop(transport, iters);
    else if (mode == "adsorption") run_loop(adsorption, iters);
    else if (mode == "coupled")
    {
        // include/mantiisApp.hpp:378-393
        auto fbody = _GLOBAL_::Fbody;
        _GLOBAL_::Fbody = 0;
        run_loop(adsorption, 100);
        _GLOBAL_::Fbody = fbody;
        std::fill(lb.ux.begin(), lb.ux.end(), 0);
        std::fill(lb.ux.begin(), lb.ux.end(), 0);
        std::fill(lb.rho.begin(), lb.rho.end(), _GLOBAL_::rhoin);
        std::fill(lb.feq.begin(), lb.feq.end(), 0);
        run_loop(coupled, iters);
    }
    else throw std::runtime_error("unknown mode " + mode);
    auto t1 = std::chrono::steady_clock::now();

    if (!dumpdir.empty())
    {
        dump_state(dumpdir, -1, lb);
        std::ofstream o(dumpdir + "/run.txt");
        o << std::setprecision(17);
        o << "steps " << done << "\n";
        o << "t " << lb.t << "\n";
        o << "cells " << grid.globalGridSize << "\n";
        o << "maxlevel " << grid.maxLevel << "\n";
        o << "threads " << num_threads << "\n";
        o << "step_seconds " << std::chrono::duration<double>(t1 - t0).count() << "\n";
        o << "setup_seconds " << std::chrono::duration<double>(t_setup1 - t_setup0).count() << "\n";
        o << "rhoin " << _GLOBAL_::rhoin << "\n";
        o << "mfp " << _GLOBAL_::mfp << "\n";
        o << "Cl " << _GLOBAL_::Cl << "\n";
        o << "T_lu " << _GLOBAL_::T_lu << "\n";
        o << "a_alpha_lu " << _GLOBAL_::a_alpha_lu << "\n";
    }
    if (!is_multiblock)
    {
        auto [ux, uy, rho] = lb.completeSingleGridDomain();
        IO::writeVectorToFile(folder + "ux.txt", ux);
        IO::writeVectorToFile(folder + "uy.txt", uy);
        IO::writeVectorToFile(folder + "rho.txt", rho);
        IO::writeVectorToFile(folder + "convergence.txt", lb.diff_over_time);
    }
    if (quiet) std::cout.clear();
    std::printf("{\"steps\": %lld, \"t\": %d, \"cells\": %lld, \"step_seconds\": %.6f, \"setup_seconds\": %.6f}\n",
                (long long)done, lb.t, (long long)grid.globalGridSize, std::chrono::duration<double>(t1 - t0).count(),
                std::chrono::duration<double>(t_setup1 - t_setup0).count());
    return 0;
}
