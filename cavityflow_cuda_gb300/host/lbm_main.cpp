// lbm_main.cpp -- the lbm_gb300 command: the reference's `lbm <config.xml>`
// program (src/main.cpp:43-80 without MPI, CManager::CManager
// src/CManager.cpp:27-105 for one subdomain, CController::run
// src/CController.cpp:1354-1510) on the C ABI of liblbm_gb300.so.
//
//   lbm_gb300 CONFIG.xml [--storage f64|f32|f16s|bf16s|f16sr] [--fma] [--moving-wall]
//             [--device N] [--fast-variant V | --autotune] [--vtk-binary]
//             [--checkpoint FILE --checkpoint-every N] [--resume FILE]
//
// As the reference: the six faces are obstacles, the lid (y = ny) is driven
// with the configuration's dimensionless x velocity, even steps are alpha and
// odd steps beta, `loops` steps run (forever when negative), VTK files
// <visualization-dir>/visualization_0_<step>.vtk are written at step 0 and
// every `rate` steps, and with benchmarking on <benchmark-dir>/benchmark_0.txt
// gets the reference's five lines (loops, time, iterations, GLUPS, GBytes/s
// with its byte count per update).  With logging on, <logging-dir>/log_0.txt
// records the set-up and every iteration.  Validation compares MPI ranks with
// a single rank in the reference; with one domain it only adds the
// velocity/density bytes to the benchmark's byte count, as there.
//
// Additions: the storage precision is an option (the reference fixes it at
// compile time, float by default, src/constants.h:23); checkpoints are written
// every N steps and on SIGINT/SIGTERM, and --resume continues a run from one
// bit-identically.  Errors print the library's message and exit 1, where the
// reference exit()s with EXIT_FAILURE.
#include <algorithm>
#include <chrono>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

#include "../../include/lbm_gb300.h"

namespace {

volatile std::sig_atomic_t g_stop = 0;

void on_signal(int) { g_stop = 1; }

[[noreturn]] void die(const std::string& what)
{
    std::cerr << "lbm_gb300: " << what << std::endl;
    std::exit(EXIT_FAILURE);
}

void check(int status, const char* call)
{
    if (status != LBM_OK)
        die(std::string(call) + ": " + lbm_status_string(status) + ": " + lbm_last_error());
}

struct Options {
    std::string config;
    int storage = LBM_STORAGE_F32;
    int device = 0;
    int fast_variant = -1;
    bool fma = false;
    int lid_mode = LBM_LID_INJECTION;
    bool autotune = false;
    bool vtk_binary = false;
    std::string checkpoint;
    long long checkpoint_every = 0;
    std::string resume;
};

void usage()
{
    std::cerr << "usage: lbm_gb300 CONFIG.xml [--storage f64|f32|f16s|bf16s|f16sr] [--fma] [--moving-wall]\n"
                 "                 [--device N]\n"
                 "                 [--fast-variant V | --autotune] [--vtk-binary]\n"
                 "                 [--checkpoint FILE --checkpoint-every N] [--resume FILE]\n";
}

Options parse(int argc, char** argv)
{
    Options o;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto value = [&]() -> std::string {
            if (i + 1 >= argc) {
                usage();
                die("option " + a + " needs a value");
            }
            return argv[++i];
        };
        if (a == "--storage") {
            const std::string v = value();
            if (v == "f64") o.storage = LBM_STORAGE_F64;
            else if (v == "f32") o.storage = LBM_STORAGE_F32;
            else if (v == "f16s") o.storage = LBM_STORAGE_F16S;
            else if (v == "bf16s") o.storage = LBM_STORAGE_BF16S;
            else if (v == "f16sr") o.storage = LBM_STORAGE_F16SR;
            else die("unknown storage " + v);
        } else if (a == "--device") {
            o.device = std::atoi(value().c_str());
        } else if (a == "--fast-variant") {
            o.fast_variant = std::atoi(value().c_str());
        } else if (a == "--fma") {
            o.fma = true;  // FP64/FP32: fused multiply-adds (lbm_params.fused_multiply_add)
        } else if (a == "--moving-wall") {
            o.lid_mode = LBM_LID_MOVING_WALL;  // mass-conserving moving top wall instead of the injection lid
        } else if (a == "--autotune") {
            o.autotune = true;
        } else if (a == "--vtk-binary") {
            o.vtk_binary = true;
        } else if (a == "--checkpoint") {
            o.checkpoint = value();
        } else if (a == "--checkpoint-every") {
            o.checkpoint_every = std::atoll(value().c_str());
        } else if (a == "--resume") {
            o.resume = value();
        } else if (a == "-h" || a == "--help") {
            usage();
            std::exit(EXIT_SUCCESS);
        } else if (!a.empty() && a[0] == '-') {
            usage();
            die("unknown option " + a);
        } else if (o.config.empty()) {
            o.config = a;
        } else {
            usage();
            die("exactly one configuration file is expected");
        }
    }
    if (o.config.empty()) {
        usage();
        die("exactly one configuration file is expected");
    }
    if (o.checkpoint_every > 0 && o.checkpoint.empty()) die("--checkpoint-every needs --checkpoint FILE");
    return o;
}

// Appends to <logging-dir>/log_0.txt when logging is on.
class Log {
public:
    Log(bool on, const std::string& dir)
    {
        if (!on) return;
        const std::string path = dir + "/log_0.txt";
        f_.open(path, std::ios::out | std::ios::app);
        if (!f_.is_open()) die("cannot open log file " + path);
    }
    template <class V>
    Log& operator<<(const V& v)
    {
        if (f_.is_open()) f_ << v;
        return *this;
    }
    bool on() const { return f_.is_open(); }

private:
    std::ofstream f_;
};

std::string vec3(const double* v)
{
    std::ostringstream s;
    s << "[" << v[0] << ", " << v[1] << ", " << v[2] << "]";
    return s.str();
}

std::string vec3(const int32_t* v)
{
    std::ostringstream s;
    s << "[" << v[0] << ", " << v[1] << ", " << v[2] << "]";
    return s.str();
}

}  // namespace

int main(int argc, char** argv)
{
    const Options opt = parse(argc, argv);
    lbm_configuration cfg;
    check(lbm_read_configuration(opt.config.c_str(), &cfg), "reading the configuration");
    lbm_physical phys;
    check(lbm_configuration_physical(&cfg, &phys), "lbm_configuration_physical");
    lbm_lattice lat;
    check(lbm_derive_lattice(&phys, opt.storage, &lat), "deriving the lattice parameters");
    Log log(cfg.do_logging != 0, cfg.logging_dir);

    lbm_solver* solver = nullptr;
    if (!opt.resume.empty()) {
        check(lbm_create_from_checkpoint(opt.resume.c_str(), opt.device, &solver), "resuming");
        lbm_info info;
        check(lbm_get_info(solver, &info), "lbm_get_info");
        if (info.storage != opt.storage || info.size[0] != cfg.domain_size[0] || info.size[1] != cfg.domain_size[1] ||
            info.size[2] != cfg.domain_size[2])
            die("checkpoint " + opt.resume + " does not hold this configuration's domain and storage");
    } else {
        lbm_params p;
        std::memset(&p, 0, sizeof(p));
        for (int d = 0; d < 3; ++d) p.size[d] = cfg.domain_size[d];
        p.storage = opt.storage;
        for (int f = 0; f < 6; ++f) p.boundary[f] = LBM_OBSTACLE;  // src/CManager.cpp:91-104, one subdomain
        p.inv_tau = lat.inv_tau;
        p.lid_velocity = lat.velocity[0];
        for (int d = 0; d < 3; ++d) p.gravity[d] = lat.acceleration[d];
        p.device = opt.device;
        p.fast_variant = opt.fast_variant < 0 ? 0 : opt.fast_variant + 1;
        p.fused_multiply_add = opt.fma ? 1 : 0;
        p.lid_mode = opt.lid_mode;
        check(lbm_create(&p, &solver), "lbm_create");
        check(lbm_set_driven_cavity(solver), "lbm_set_driven_cavity");
    }
    if (opt.autotune) {
        int32_t best = 0;
        float ms[64];
        check(lbm_autotune(solver, 4, &best, ms), "lbm_autotune");
    }
    lbm_info info;
    check(lbm_get_info(solver, &info), "lbm_get_info");
    long long step = info.step_counter;

    if (log.on()) {
        log << "----- lbm_gb300 -----\n"
            << "configuration:          " << opt.config << "\n"
            << "domain size:            " << vec3(cfg.domain_size) << "\n"
            << "domain length:          " << vec3(cfg.domain_length) << "\n"
            << "storage:                " << opt.storage << "\n"
            << "tau:                    " << lat.tau << "\n"
            << "lid velocity:           " << lat.velocity[0] << "\n"
            << "gravity:                " << vec3(lat.acceleration) << "\n"
            << "boundaryConditions:     all six faces OBSTACLE (" << LBM_OBSTACLE << ")\n"
            << "launch variant:         " << info.fast_variant << "\n"
            << "starting step:          " << step << "\n"
            << "---------------------\n";
    }

    std::signal(SIGINT, on_signal);
    std::signal(SIGTERM, on_signal);

    const bool vis = cfg.do_visualization != 0;
    const long long rate = cfg.visualization_rate;
    auto render = [&](long long iteration) {
        if (!vis || iteration % rate != 0) return;
        std::ostringstream name;
        name << cfg.visualization_dir << "/visualization_0_" << iteration << ".vtk";
        check(lbm_write_vtk(solver, name.str().c_str(), cfg.domain_length, opt.vtk_binary ? 1 : 0), "lbm_write_vtk");
    };
    auto checkpoint = [&]() {
        if (opt.checkpoint.empty()) return;
        check(lbm_save_checkpoint(solver, opt.checkpoint.c_str()), "lbm_save_checkpoint");
        log << "checkpoint at step " << step << " written to " << opt.checkpoint << "\n";
    };

    // src/CController.cpp:1382-1399: populations read and written, the flag
    // read, and velocity and density written when they are output.
    const int value_bytes = opt.storage == LBM_STORAGE_F64 ? 8 : opt.storage == LBM_STORAGE_F32 ? 4 : 2;
    long long used_bytes = 19 * 2 * value_bytes + 4;
    if (cfg.do_visualization || cfg.do_validation) used_bytes += 4 * (opt.storage == LBM_STORAGE_F64 ? 8 : 4);

    if (opt.resume.empty()) render(0);
    const bool forever = cfg.loops < 0;
    const long long total = cfg.loops;
    const auto t0 = std::chrono::steady_clock::now();
    long long done = 0;
    while ((forever || step < total) && !g_stop) {
        // run up to the next visualization step, checkpoint or the end, so
        // long stretches replay the solver's captured step graph
        long long chunk = forever ? (1LL << 20) : total - step;
        if (vis) chunk = std::min(chunk, rate - step % rate);
        if (opt.checkpoint_every > 0) chunk = std::min(chunk, opt.checkpoint_every - step % opt.checkpoint_every);
        if (log.on()) chunk = 1;
        if (log.on()) log << "Do iteration " << step << ":\n";
        check(lbm_run(solver, chunk, nullptr), "lbm_run");
        step += chunk;
        done += chunk;
        if (log.on()) log << "Iteration " << step - 1 << " successful.\n";
        render(step);
        if (opt.checkpoint_every > 0 && step % opt.checkpoint_every == 0) checkpoint();
    }
    check(lbm_synchronize(solver), "lbm_synchronize");
    const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (g_stop) {
        checkpoint();
        std::cerr << "lbm_gb300: stopped by signal at step " << step << std::endl;
    }

    if (cfg.do_benchmark && done > 0) {
        // src/CController.cpp:1452-1481, in the value type's precision
        const bool dbl = opt.storage == LBM_STORAGE_F64;
        const double cells = (double)cfg.domain_size[0] * cfg.domain_size[1] * cfg.domain_size[2];
        double its = (double)done / elapsed, lups = its * cells * 1e-9, bw = lups * (double)used_bytes;
        if (!dbl) {
            its = (float)((float)done / (float)elapsed);
            lups = (float)((float)its * (float)cfg.domain_size[0] * (float)cfg.domain_size[1] *
                           (float)cfg.domain_size[2] * 0.000000001f);
            bw = (float)((float)lups * (float)used_bytes);
        }
        const std::string path = std::string(cfg.benchmark_dir) + "/benchmark_0.txt";
        std::ofstream b(path, std::ios::out);
        if (!b.is_open()) die("cannot open benchmark file " + path);
        b << "loops:           " << done << std::endl;
        b << "time:            " << (dbl ? elapsed : (double)(float)elapsed) << "s" << std::endl;
        b << "iterations:      " << its << "s^-1" << std::endl;
        b << "lattice updates: " << lups << "GLUPS" << std::endl;
        b << "bandwidth:       " << bw << "GBytes/s" << std::endl;
    }
    log << "---------------------\n";
    std::cout << "lbm_gb300: " << done << " steps of " << cfg.domain_size[0] << "x" << cfg.domain_size[1] << "x"
              << cfg.domain_size[2] << " in " << elapsed << " s (" << (double)done * cfg.domain_size[0] *
                 cfg.domain_size[1] * cfg.domain_size[2] / elapsed * 1e-6 << " MLUPS), final step " << step
              << std::endl;
    check(lbm_destroy(solver), "lbm_destroy");
    return g_stop ? 130 : 0;
}
