// Drop-in replacement of the reference's `mantiis` executable
// (mantiis.cpp, include/mantiisApp.hpp): same positional arguments, same input
// files, same output files and console lines; the time stepping runs on the
// GPU through the C ABI of libmantiis_gpu.so.
//
//   mantiis <num_threads> <is_multiblock> <Nx> <input_folder/> <Nt> [options]
//
// The reference compiles its Settings into each executable (mantiis.cpp,
// test/transport_test.cpp, test/adsorption_test.cpp); here they are chosen
// with trailing options:
//   --preset mantiis|transport_test|adsorption_test   (default mantiis)
//   --simulation transport|adsorption  --dx m  --fbody f  --T K  --P Pa
//   --collision 0|1|2  --wall 0|1|2  --tol t  --levels 2|3  --verbose k
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/mantiis_gpu.h"

namespace
{
struct Settings
{
    std::string simulation_type = "transport";
    int verbose = 10;
    double T = 300.0, P = 2.0e6, dx = 5e-10, Fbody = 1.0e-8;
    long long dump_macroscopic_every_timestep = 1000000;
    double threshold = 1.0e-10;
    int collision_method = 2, wall_boundary = 2;
    int levels = 2;
};

template <typename T> void write_vec(const std::string &path, const std::vector<T> &v)
{
    std::ofstream out(path);
    if (!out.is_open())
    {
        std::cout << "Tried writing " << path << std::endl;
        throw std::runtime_error("[ERROR]: Unable to open file for writing.");
    }
    for (const auto &x : v) out << std::setprecision(15) << x << '\n';
}

void check(int rc, mgpu_ctx *ctx)
{
    if (rc != MGPU_OK)
        throw std::runtime_error(ctx ? mgpu_last_error(ctx) : mgpu_global_error());
}
} // namespace

int main(int argc, char *argv[])
{
    Settings st;
    // preset first so that explicit options override it
    for (int a = 6; a + 1 < argc; a++)
        if (std::string(argv[a]) == "--preset")
        {
            std::string p = argv[a + 1];
            if (p == "transport_test") st.dx = 1.0e-9;
            else if (p == "adsorption_test")
            {
                st.simulation_type = "adsorption";
                st.dx = 12.0e-9;
            }
            else if (p != "mantiis")
            {
                std::cerr << "unknown preset " << p << "\n";
                return EXIT_FAILURE;
            }
        }
    for (int a = 6; a < argc; a++)
    {
        std::string k = argv[a];
        if (a + 1 >= argc)
        {
            std::cerr << "missing value for " << k << "\n";
            return EXIT_FAILURE;
        }
        std::string v = argv[++a];
        if (k == "--preset") continue;
        else if (k == "--simulation") st.simulation_type = v;
        else if (k == "--dx") st.dx = std::stod(v);
        else if (k == "--fbody") st.Fbody = std::stod(v);
        else if (k == "--T") st.T = std::stod(v);
        else if (k == "--P") st.P = std::stod(v);
        else if (k == "--collision") st.collision_method = std::stoi(v);
        else if (k == "--wall") st.wall_boundary = std::stoi(v);
        else if (k == "--tol") st.threshold = std::stod(v);
        else if (k == "--levels") st.levels = std::stoi(v);
        else if (k == "--verbose") st.verbose = std::stoi(v);
        else
        {
            std::cerr << "unknown option " << k << "\n";
            return EXIT_FAILURE;
        }
    }

    double u[6];
    mgpu_units(st.dx, st.T, st.P, u);
    // include/mantiisApp.hpp:131-135
    if (argc < 6)
    {
        std::cerr << "Usage: " << argv[0] << " <num_threads> <is_multiblock> <Nx> <input_folder/> <Nt>\n";
        std::exit(EXIT_FAILURE);
    }
    try
    {
        int num_threads = std::stoi(argv[1]);
        (void)num_threads; // host preprocessing is single-threaded here; accepted for compatibility
        bool is_multiblock = (std::string(argv[2]) == "true");
        int Nx = std::stoi(argv[3]);
        std::string folder = argv[4];
        int iters = std::stoi(argv[5]);

        std::cout << "Mean free path: " << u[1] << "\n";
        std::cout << "Cl: " << st.dx << "\n";
        std::cout << "Temperature: " << st.T << "\n";
        std::cout << "Pressure: " << st.P << "\n";
        std::cout << "Fbody: " << st.Fbody << "\n";
        std::cout << "Force conversion factor: " << std::setprecision(15) << u[5] << "\n";
        std::cout << "Input density: " << std::setprecision(15) << u[0] << "\n";

        using clk = std::chrono::high_resolution_clock;
        auto start = clk::now();
        mgpu_params p;
        mgpu_default_params(&p);
        if (st.simulation_type == "transport") p.simulation = MGPU_SIM_TRANSPORT;
        else if (st.simulation_type == "adsorption") p.simulation = MGPU_SIM_ADSORPTION;
        else if (st.simulation_type == "coupled") p.simulation = MGPU_SIM_COUPLED;
        else throw std::runtime_error("Unknown simulation type: " + st.simulation_type);
        p.collision = st.collision_method;
        p.wall = st.wall_boundary;
        p.multiblock = is_multiblock;
        p.max_allowed_level = st.levels;
        p.dx = st.dx;
        p.fbody = st.Fbody;
        p.T = st.T;
        p.P = st.P;
        p.tol = st.threshold;
        std::cout << "Loading input from saved data\n";
        mgpu_ctx *ctx = nullptr;
        check(mgpu_create_from_folder(folder.c_str(), Nx, &p, &ctx), nullptr);
        mgpu_info info;
        mgpu_get_info(ctx, &info);
        {
            std::vector<int64_t> rec((size_t)Nx * Nx);
            mgpu_reconstructed(ctx, rec.data());
            write_vec("reconstructed.dat", rec);
        }
        std::cout << "The number of active cells: " << info.n_cells << "\n";
        std::cout << "Initializing Simulation...\n";

        // run loop (include/mantiisApp.hpp:294-352)
        int64_t t = 0;
        std::vector<double> hist;
        int done_total = 0;
        bool stopped = false;
        auto residuals = [&]() {
            int64_t cnt = 0;
            mgpu_residuals(ctx, nullptr, 0, &cnt);
            hist.resize((size_t)cnt);
            mgpu_residuals(ctx, hist.data(), cnt, &cnt);
        };
        const bool coupled = p.simulation == MGPU_SIM_COUPLED;
        if (coupled)
        {
            // 100 adsorption steps come first (include/mantiisApp.hpp:376-392)
            iters += 100;
            std::cout << "======================= Adsorption ONLY for initial condition =======================\n";
        }
        while (done_total < iters && !stopped)
        {
            // first step alone (its fields are dumped as ux_0 / uy_0), then in chunks
            int chunk = done_total == 0 ? 1 : std::min(iters - done_total, 1000);
            size_t h0 = hist.size();
            int done = 0;
            check(mgpu_run(ctx, chunk, &done), ctx);
            residuals();
            for (size_t k = h0; k < hist.size(); k++)
            {
                if (coupled && t == 100) std::cout << "======================= Coupling =======================\n";
                if (t % st.verbose == 0)
                    std::cout << "Timestep: " << t << ", residual difference: " << hist[k] << "\n";
                if (hist[k] < st.threshold)
                {
                    stopped = true;
                    break;
                }
                if (t % st.dump_macroscopic_every_timestep == 0)
                {
                    std::vector<double> ux((size_t)Nx * Nx), uy((size_t)Nx * Nx);
                    check(mgpu_download_pixels(ctx, nullptr, ux.data(), uy.data(), nullptr), ctx);
                    write_vec(folder + "ux_" + std::to_string(t) + ".txt", ux);
                    write_vec(folder + "uy_" + std::to_string(t) + ".txt", uy);
                }
                t++;
            }
            done_total += done;
            if (done < chunk) stopped = true;
        }

        // final outputs (include/mantiisApp.hpp:399-429)
        size_t nn = (size_t)Nx * Nx;
        std::vector<double> rho(nn), ux(nn), uy(nn), f(nn * 9);
        check(mgpu_download_pixels(ctx, rho.data(), ux.data(), uy.data(), f.data()), ctx);
        write_vec(folder + "f.txt", f);
        write_vec(folder + "ux.txt", ux);
        write_vec(folder + "uy.txt", uy);
        write_vec(folder + "rho.txt", rho);
        write_vec(folder + "convergence.txt", hist);
        std::ofstream det(folder + "SimulationDetails.txt");
        det << "Domain dimension: " << Nx << " x " << Nx << "\n";
        det << "Tolerance was set to " << st.threshold << "\n";
        det << "Number timesteps executed: " << t << "\n";
        det << "The number of active cells: " << info.n_cells << "\n";
        auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(clk::now() - start).count();
        std::cout << "Total run time (milliseconds) " << std::setprecision(15) << ms << std::endl;
        det << "Total run time (milliseconds): " << std::setprecision(15) << ms;
        mgpu_destroy(ctx);
    }
    catch (const std::exception &e)
    {
        std::cerr << "terminate called after throwing an instance of 'std::runtime_error'\n  what():  " << e.what() << "\n";
        return EXIT_FAILURE;
    }
    return 0;
}
