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
// and, beyond the reference:
//   --output text|binary|both   text: the reference's files (default); binary:
//                               ux.bin uy.bin rho.bin f.bin convergence.bin
//                               (raw little-endian float64, same order as the
//                               text files) and f_cells.bin (9 per grid cell,
//                               the exact restart state)
//   --restart file [--restart-step t]  start from saved populations: f.txt,
//                               f.bin (pixel layout) or f_cells.bin (cell
//                               layout, exact on multi-block grids), told
//                               apart by their length; t = the step the file
//                               was written at (SimulationDetails.txt's
//                               "Number timesteps executed"), default 0
// Text files are formatted by num_threads threads (argv[1]).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <thread>
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
    std::string output = "text";
    std::string restart;
    long long restart_step = 0;
};

void format_one(std::string &buf, double x)
{
    char tmp[40];
    int k = std::snprintf(tmp, sizeof tmp, "%.15g\n", x); // = ostream << setprecision(15) << x
    buf.append(tmp, (size_t)k);
}
void format_one(std::string &buf, int64_t x)
{
    char tmp[32];
    int k = std::snprintf(tmp, sizeof tmp, "%lld\n", (long long)x);
    buf.append(tmp, (size_t)k);
}

int g_threads = 1;

// One value per line, 15 significant digits (include/io.hpp:75-92); the text
// is formatted in g_threads slices in parallel and written in order.
template <typename T> void write_vec(const std::string &path, const std::vector<T> &v)
{
    std::FILE *out = std::fopen(path.c_str(), "wb");
    if (!out)
    {
        std::cout << "Tried writing " << path << std::endl;
        throw std::runtime_error("[ERROR]: Unable to open file for writing.");
    }
    const size_t slice = 1 << 18;
    const size_t n_slices = (v.size() + slice - 1) / slice;
    const int nt = (int)std::max<size_t>(1, std::min<size_t>((size_t)g_threads, n_slices));
    bool ok = true;
    for (size_t first = 0; first < n_slices; first += (size_t)nt)
    {
        std::vector<std::string> text((size_t)nt);
        auto work = [&](int w) {
            size_t sl = first + (size_t)w;
            if (sl >= n_slices) return;
            std::string &b = text[(size_t)w];
            b.reserve(slice * 24);
            for (size_t k = sl * slice, end = std::min(v.size(), (sl + 1) * slice); k < end; k++) format_one(b, v[k]);
        };
        std::vector<std::thread> pool;
        for (int w = 1; w < nt; w++) pool.emplace_back(work, w);
        work(0);
        for (auto &th : pool) th.join();
        for (auto &b : text) ok = ok && std::fwrite(b.data(), 1, b.size(), out) == b.size();
    }
    ok = std::fclose(out) == 0 && ok;
    if (!ok) throw std::runtime_error("[ERROR]: Unable to write file " + path);
}

void write_bin(const std::string &path, const std::vector<double> &v)
{
    std::FILE *out = std::fopen(path.c_str(), "wb");
    if (!out) throw std::runtime_error("[ERROR]: Unable to open file for writing.");
    bool ok = std::fwrite(v.data(), sizeof(double), v.size(), out) == v.size();
    ok = std::fclose(out) == 0 && ok;
    if (!ok) throw std::runtime_error("[ERROR]: Unable to write file " + path);
}

// populations of a restart file: raw float64 (.bin) or whitespace-separated text
std::vector<double> read_restart(const std::string &path)
{
    std::FILE *in = std::fopen(path.c_str(), "rb");
    if (!in)
    {
        std::cout << "Tried loading " << path << std::endl;
        throw std::runtime_error("[ERROR]: File not found.");
    }
    std::string raw;
    char chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof chunk, in)) > 0) raw.append(chunk, k);
    std::fclose(in);
    std::vector<double> v;
    const bool binary = path.size() >= 4 && path.compare(path.size() - 4, 4, ".bin") == 0;
    if (binary)
    {
        if (raw.size() % sizeof(double)) throw std::runtime_error("[ERROR]: " + path + " is not a float64 file.");
        v.resize(raw.size() / sizeof(double));
        std::memcpy(v.data(), raw.data(), raw.size());
        return v;
    }
    const char *p = raw.c_str();
    char *end = nullptr;
    for (;;)
    {
        double x = std::strtod(p, &end);
        if (end == p) break;
        v.push_back(x);
        p = end;
    }
    while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') p++;
    if (*p) throw std::runtime_error("[ERROR]: unreadable number in " + path);
    return v;
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
        else if (k == "--output") st.output = v;
        else if (k == "--restart") st.restart = v;
        else if (k == "--restart-step") st.restart_step = std::stoll(v);
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
        g_threads = std::max(1, std::min(num_threads, 256)); // text output formatting
        if (st.output != "text" && st.output != "binary" && st.output != "both")
            throw std::runtime_error("unknown output format " + st.output);
        const bool text_out = st.output != "binary", bin_out = st.output != "text";
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
        if (!st.restart.empty())
        {
            std::vector<double> f0 = read_restart(st.restart);
            const size_t per_cell = 9 * (size_t)info.n_cells, per_pixel = 9 * (size_t)Nx * Nx;
            int layout = f0.size() == per_pixel ? MGPU_LAYOUT_PIXELS : MGPU_LAYOUT_CELLS;
            if (f0.size() != per_pixel && f0.size() != per_cell)
                throw std::runtime_error("[ERROR]: " + st.restart + " holds " + std::to_string(f0.size()) +
                                         " values, expected " + std::to_string(per_pixel) + " (pixels) or " +
                                         std::to_string(per_cell) + " (cells)");
            check(mgpu_set_distributions(ctx, f0.data(), layout, st.restart_step), ctx);
            t = st.restart_step;
            std::cout << "Restarting from " << st.restart << " at timestep " << t << "\n";
        }
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
        if (coupled && t < 100)
        {
            // 100 adsorption steps come first (include/mantiisApp.hpp:376-392)
            iters += (int)(100 - t);
            std::cout << "======================= Adsorption ONLY for initial condition =======================\n";
        }
        while (done_total < iters && !stopped)
        {
            // chunks of up to 1000 steps that end on every step whose fields are
            // dumped (ux_<t>, uy_<t>: t = 0, then every dump_macroscopic_every_timestep)
            const long long every = st.dump_macroscopic_every_timestep;
            const long long to_dump = (every - t % every) % every;
            int chunk = (int)std::min<long long>({(long long)(iters - done_total), 1000LL, to_dump + 1});
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
        if (text_out)
        {
            write_vec(folder + "f.txt", f);
            write_vec(folder + "ux.txt", ux);
            write_vec(folder + "uy.txt", uy);
            write_vec(folder + "rho.txt", rho);
            write_vec(folder + "convergence.txt", hist);
        }
        if (bin_out)
        {
            std::vector<double> fc(9 * (size_t)info.n_cells);
            check(mgpu_download_cells(ctx, nullptr, nullptr, nullptr, fc.data()), ctx);
            write_bin(folder + "f_cells.bin", fc);
            write_bin(folder + "f.bin", f);
            write_bin(folder + "ux.bin", ux);
            write_bin(folder + "uy.bin", uy);
            write_bin(folder + "rho.bin", rho);
            write_bin(folder + "convergence.bin", hist);
        }
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
