// skt_run: a native driver over the C ABI, the caller the reference's start-up and game loop are
// (Game/gameSystem.cpp:43-47 reads the radiosonde archive and initialises the environment,
// Game/game.cpp:56 calls updateGPU once per frame). It reads a sounding from an unpacked archive
// (the members of a KNMI .mwx, or of a DWD zip with the archive's name for the station), sets the
// environment up through the C++ adapter (readTable::initEnvironment), runs the steps and prints
// one JSON line per step and a summary line; --raw writes the 11 prognostic fields at the end;
// --parse-only prints the sounding's rows and stops (no GPU needed).
//
//   skt_run --knmi DIR | --dwd ARCHIVE_NAME --dir DIR  [--grid NX,NY,NZ] [--voxel M] [--steps N]
//           [--dt S] [--speed F] [--mixed] [--textbook] [--no-noise] [--seed K] [--raw OUTDIR]
//           [--parse-only]
//
// NY is the vertical size (the reference's layout).
#include "skewt_env.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace {

// an unpacked archive: the member `name` is the file DIR/name
long long dir_read(void* ctx, const char* name, char* buf, size_t cap) {
    const std::string path = std::string(static_cast<const char*>(ctx)) + "/" + name;
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) return -1;
    const long long size = static_cast<long long>(f.tellg());
    if (buf && cap >= static_cast<size_t>(size)) {
        f.seekg(0);
        f.read(buf, size);
    }
    return size;
}

struct Args {
    std::string knmi, dwd, dir, raw, tune;
    int nx = 64, ny = 32, nz = 64;
    float voxel = 100.0f, dt = 0.5f, speed = 1.0f;
    int steps = 10;
    bool mixed = false, textbook = false, noise = true, parse_only = false, graph = false;
    unsigned seed = 100;
};

[[noreturn]] void usage(const char* msg) {
    std::fprintf(stderr,
                 "skt_run: %s\n"
                 "usage: skt_run --knmi DIR | --dwd ARCHIVE_NAME --dir DIR [--grid NX,NY,NZ] [--voxel M] [--steps N]\n"
                 "               [--dt S] [--speed F] [--mixed] [--textbook] [--no-noise] [--seed K] [--raw OUTDIR]\n"
                 "               [--graph] [--tune CACHE_FILE] [--parse-only]\n",
                 msg);
    std::exit(2);
}

Args parse(int argc, char** argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        auto val = [&]() -> const char* {
            if (i + 1 >= argc) usage(("missing value after " + k).c_str());
            return argv[++i];
        };
        if (k == "--knmi") a.knmi = val();
        else if (k == "--dwd") a.dwd = val();
        else if (k == "--dir") a.dir = val();
        else if (k == "--raw") a.raw = val();
        else if (k == "--grid") {
            if (std::sscanf(val(), "%d,%d,%d", &a.nx, &a.ny, &a.nz) != 3) usage("--grid wants NX,NY,NZ");
        } else if (k == "--voxel") a.voxel = std::strtof(val(), nullptr);
        else if (k == "--steps") a.steps = std::atoi(val());
        else if (k == "--dt") a.dt = std::strtof(val(), nullptr);
        else if (k == "--speed") a.speed = std::strtof(val(), nullptr);
        else if (k == "--seed") a.seed = static_cast<unsigned>(std::strtoul(val(), nullptr, 10));
        else if (k == "--mixed") a.mixed = true;
        else if (k == "--textbook") a.textbook = true;
        else if (k == "--no-noise") a.noise = false;
        else if (k == "--parse-only") a.parse_only = true;
        else if (k == "--graph") a.graph = true;  // each step one launch of the captured CUDA graph
        else if (k == "--tune") a.tune = val();   // the autotuner's launch shapes, cached in this file
        else usage(("unknown option " + k).c_str());
    }
    if (a.knmi.empty() == (a.dwd.empty())) usage("give exactly one of --knmi and --dwd");
    if (!a.dwd.empty() && a.dir.empty()) usage("--dwd needs --dir (the unpacked archive)");
    if (a.steps < 0) usage("--steps must be >= 0");
    return a;
}

struct Field {
    const char* name;
    skt_param param;
    skt_direction dir;
};
constexpr Field kFields[] = {{"th", SKT_POTTEMP, SKT_RIGHT}, {"qv", SKT_QV, SKT_RIGHT},   {"qw", SKT_QW, SKT_RIGHT},
                             {"qc", SKT_QC, SKT_RIGHT},      {"qr", SKT_QR, SKT_RIGHT},   {"qs", SKT_QS, SKT_RIGHT},
                             {"qi", SKT_QI, SKT_RIGHT},      {"u", SKT_WIND, SKT_RIGHT},  {"v", SKT_WIND, SKT_UP},
                             {"w", SKT_WIND, SKT_FORWARD},   {"p", SKT_PRESSURE, SKT_RIGHT}};

}  // namespace

int main(int argc, char** argv) {
    const Args a = parse(argc, argv);
    try {
        skewt::ReadTable table;  // the archive is read before the environment exists, as at start-up
        if (!a.knmi.empty()) table.readKNMIFile(dir_read, const_cast<char*>(a.knmi.c_str()));
        else table.readDWDFile(a.dwd.c_str(), dir_read, const_cast<char*>(a.dir.c_str()));
        if (a.parse_only) {
            const skt_sounding& d = table.data();
            std::printf("{\"sounding_rows\": %zu, \"rows\": [", d.n);
            for (size_t i = 0; i < d.n; ++i)
                std::printf("%s[%.9g, %.9g, %.9g, %.9g, %.9g, %.9g]", i ? ", " : "", d.altitude[i], d.pressure[i], d.temperature[i],
                            d.dew_point[i], d.wind_speed[i], d.wind_dir[i]);
            std::printf("]}\n");
            return 0;
        }
        skt_solver_cfg cfg;
        skt_default_config(&cfg);
        cfg.precision = a.mixed ? SKT_PCG_MIXED : SKT_PCG_PLAIN;
        cfg.semantics = a.textbook ? SKT_SEM_TEXTBOOK : SKT_SEM_REFERENCE;
        cfg.use_graph = a.graph ? 1 : 0;
        skewt::EnvironmentGPU env(a.nx, a.ny, a.nz, a.voxel, &cfg);
        table.initEnvironment(env, a.noise, a.seed);
        std::printf("{\"sounding_rows\": %zu, \"grid\": [%d, %d, %d], \"voxel\": %g, \"precision\": \"%s\", \"semantics\": \"%s\"}\n",
                    table.data().n, a.nx, a.ny, a.nz, a.voxel, a.mixed ? "mixed" : "plain", a.textbook ? "textbook" : "reference");
        if (!a.tune.empty()) {
            skt_tuning t{};
            const skt_status ts = skt_autotune(env.handle(), a.tune.c_str(), 0, &t);
            if (ts != SKT_OK) throw skewt::Error(ts, skt_last_error(env.handle()));
            std::printf("{\"tuning\": {\"diffuse_depth\": %d, \"diffuse_rows\": %d, \"from_cache\": %s}}\n", t.diffuse_depth,
                        t.diffuse_rows, t.from_cache ? "true" : "false");
        }
        const double cells = double(a.nx) * a.ny * a.nz;
        double gpu_ms = 0.0;
        const auto t0 = std::chrono::steady_clock::now();
        for (int s = 0; s < a.steps; ++s) {
            const bool converged = env.updateGPU(a.dt, a.speed);
            const skt_step_stats st = env.stats();
            gpu_ms += st.gpu_ms;
            std::printf("{\"step\": %d, \"pcg_iters\": %d, \"pcg_residual\": %.6g, \"converged\": %s, \"outer_iters\": %d, "
                        "\"sim_time\": %.3f, \"gpu_ms\": %.3f}\n",
                        s + 1, st.pcg_iters, st.pcg_residual, converged ? "true" : "false", st.outer_iters, st.sim_time, st.gpu_ms);
        }
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("{\"steps\": %d, \"cells\": %.0f, \"wall_s\": %.4f, \"gpu_ms\": %.3f, \"cell_steps_per_s\": %.6g, "
                    "\"kernel_launches\": %lld}\n",
                    a.steps, cells, wall, gpu_ms, a.steps > 0 && gpu_ms > 0 ? cells * a.steps / (gpu_ms / 1e3) : 0.0,
                    env.stats().kernel_launches);
        if (!a.raw.empty()) {
            for (const Field& f : kFields) {
                const std::vector<float> v = env.readField(f.param, f.dir);
                const std::string path = a.raw + "/" + f.name + ".f32";
                std::ofstream o(path, std::ios::binary);
                if (!o) throw skewt::Error(SKT_INVALID_ARG, ("cannot write " + path).c_str());
                o.write(reinterpret_cast<const char*>(v.data()), std::streamsize(v.size() * sizeof(float)));
            }
        }
    } catch (const skewt::Error& e) {
        std::fprintf(stderr, "skt_run: %s\n", e.what());
        return 1;
    }
    return 0;
}
