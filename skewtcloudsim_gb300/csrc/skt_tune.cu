// Launch-shape tuning of the stencil kernels (no counterpart in the reference, whose grid and
// launch shapes are compile-time constants, Game/config.h:3-9).
//
// The tunable shapes are those whose best value depends on the grid size and the GPU: the
// diffusion's temporal-blocking depth (one sweep per pass, or two), the two-sweep kernel and its
// tile height (k_diffuse_pair4 with 6 or 14 rows per block, k_diffuse2 with 4 or 8 rows per warp:
// the height sets how much of the intermediate sweep is recomputed at tile edges), and the run lengths of the z and y marches (blocks per SM in the
// grid) of the diffusion and PPM passes. None of them changes a single bit of the results: every
// cell is computed with the same arithmetic from the same neighbour values whatever the shape.
// skt_autotune times each candidate on scratch copies of the environment's own fields and
// checks that it reproduces the default shape's result bit for bit before accepting it (the
// diffusion candidates through a position-weighted hash of the result's bits, the PPM candidates
// cell by cell).
#include "skt_internal.cuh"
#include "../../include/skewt.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

using namespace skt;

namespace {

__global__ void k_count_diff(const unsigned* __restrict__ a, const unsigned* __restrict__ b, size_t n, unsigned* __restrict__ count) {
    unsigned c = 0;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) c += a[i] != b[i];
    if (c) atomicAdd(count, c);
}

// A position-weighted sum of a field's bit patterns modulo 2^64 (integer sums: the same whatever
// the order): two fields with the same hash are taken as equal bit for bit.
__global__ void k_hash_bits(const unsigned* __restrict__ a, size_t n, unsigned long long* __restrict__ h) {
    unsigned long long s = 0;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        s += (unsigned long long)a[i] * (2ull * i + 1ull) + (unsigned long long)(a[i] >> 7) * 0x9E3779B97F4A7C15ull;
    atomicAdd(h, s);
}

void to_abi(const Tuning& t, skt_tuning* o) {
    o->diffuse_depth = t.diffuse_depth;
    o->diffuse_rows = t.diffuse_h;
    o->diffuse_bps = t.diffuse_bps;
    o->diffuse2_bps = t.diffuse2_bps;
    o->ppm_x_bps = t.ppm_bps;
    o->ppm_y_bps = t.ppmy_bps;
    o->ppm_z_bps = t.ppmz_bps;
}

bool from_abi(const skt_tuning* o, Tuning& t) {
    auto in = [](int v, int lo, int hi) { return v >= lo && v <= hi; };
    if (!(o->diffuse_depth == 1 || o->diffuse_depth == 2) || !(o->diffuse_rows == 4 || o->diffuse_rows == 8 || o->diffuse_rows == 6 || o->diffuse_rows == 14) ||
        !in(o->diffuse_bps, 1, 256) || !in(o->diffuse2_bps, 1, 256) || !in(o->ppm_x_bps, 1, 256) || !in(o->ppm_y_bps, 1, 256) ||
        !in(o->ppm_z_bps, 1, 256))
        return false;
    t.diffuse_depth = o->diffuse_depth;
    t.diffuse_h = o->diffuse_rows;
    t.diffuse_bps = o->diffuse_bps;
    t.diffuse2_bps = o->diffuse2_bps;
    t.ppm_bps = o->ppm_x_bps;
    t.ppmy_bps = o->ppm_y_bps;
    t.ppmz_bps = o->ppm_z_bps;
    return true;
}

// The cache is a JSON object with one entry per line, keyed by GPU name and grid:
//   "NVIDIA GB300 512x256x512": {"diffuse_depth": 1, "diffuse_rows": 8, ...},
const char* kFields[] = {"diffuse_depth", "diffuse_rows", "diffuse_bps", "diffuse2_bps", "ppm_x_bps", "ppm_y_bps", "ppm_z_bps"};
constexpr int kNumFields = 7;

int* field_of(skt_tuning& t, int i) {
    int* f[kNumFields] = {&t.diffuse_depth, &t.diffuse_rows, &t.diffuse_bps, &t.diffuse2_bps, &t.ppm_x_bps, &t.ppm_y_bps, &t.ppm_z_bps};
    return f[i];
}

std::string cache_key(const Env& e) {
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, e.device);
    return std::string(prop.name) + " " + std::to_string(e.g.X) + "x" + std::to_string(e.g.Y) + "x" + std::to_string(e.g.Z);
}

bool parse_entry(const std::string& line, skt_tuning& t) {
    for (int i = 0; i < kNumFields; ++i) {
        const std::string tag = std::string("\"") + kFields[i] + "\":";
        const size_t p = line.find(tag);
        if (p == std::string::npos) return false;
        *field_of(t, i) = std::atoi(line.c_str() + p + tag.size());
    }
    return true;
}

std::vector<std::string> read_lines(const char* path) {
    std::vector<std::string> out;
    std::ifstream f(path);
    std::string ln;
    while (std::getline(f, ln)) out.push_back(ln);
    return out;
}

bool cache_lookup(const char* path, const std::string& key, skt_tuning& t) {
    const std::string tag = "\"" + key + "\":";
    for (const std::string& ln : read_lines(path))
        if (ln.find(tag) != std::string::npos && parse_entry(ln, t)) return true;
    return false;
}

bool cache_store(const char* path, const std::string& key, const skt_tuning& t) {
    std::vector<std::string> entries;
    const std::string tag = "\"" + key + "\":";
    for (const std::string& ln : read_lines(path)) {
        if (ln.find('"') == std::string::npos || ln.find(tag) != std::string::npos) continue;  // braces, or the old entry
        std::string e = ln;
        while (!e.empty() && (e.back() == ',' || e.back() == ' ' || e.back() == '\r')) e.pop_back();
        entries.push_back(e);
    }
    std::ostringstream s;
    s << "  " << tag << " {";
    skt_tuning c = t;
    for (int i = 0; i < kNumFields; ++i) s << (i ? ", " : "") << "\"" << kFields[i] << "\": " << *field_of(c, i);
    s << "}";
    entries.push_back(s.str());
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream f(tmp);
        if (!f) return false;
        f << "{\n";
        for (size_t i = 0; i < entries.size(); ++i) f << entries[i] << (i + 1 < entries.size() ? ",\n" : "\n");
        f << "}\n";
        if (!f) return false;
    }
    return std::rename(tmp.c_str(), path) == 0;
}

// Times `run` (queued on e.stream) over reps repetitions after one untimed run; milliseconds per run.
template <class F>
float time_ms(Env& e, int reps, F&& run) {
    run();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, e.stream);
    for (int i = 0; i < reps; ++i) run();
    cudaEventRecord(b, e.stream);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
}

}  // namespace

extern "C" {

skt_status skt_get_tuning(skt_env* env, skt_tuning* out) {
    if (!env || !out) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    to_abi(env->e.tune, out);
    out->from_cache = 0;
    out->diffuse_ms = out->advect_ms = 0.0f;
    return SKT_OK;
}

skt_status skt_set_tuning(skt_env* env, const skt_tuning* t) {
    if (!env || !t) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Tuning nt = env->e.tune;
    if (!from_abi(t, nt))
        return report(&env->e, SKT_INVALID_ARG, "invalid tuning (diffuse_depth 1 or 2, diffuse_rows 4, 6, 8 or 14, blocks per SM 1..256)");
    env->e.tune = nt;
    return SKT_OK;
}

skt_status skt_autotune(skt_env* env, const char* cache_path, int flags, skt_tuning* out) {
    if (!env) return report(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!e.initialized) return report(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    const std::string key = cache_key(e);
    skt_tuning t{};
    if (cache_path && !(flags & SKT_TUNE_FORCE) && cache_lookup(cache_path, key, t)) {
        Tuning nt = e.tune;
        if (!from_abi(&t, nt)) return report(&e, SKT_INVALID_ARG, "the tuning cache holds an invalid entry for this grid");
        e.tune = nt;
        if (out) {
            *out = t;
            out->from_cache = 1;
            out->diffuse_ms = out->advect_ms = 0.0f;
        }
        return SKT_OK;
    }
    const size_t n = size_t(e.g.N);
    const Tuning base = Tuning{};
    unsigned* count = nullptr;
    if (cudaMalloc(&count, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return report(&e, SKT_OUT_OF_MEMORY, "autotune: counter allocation failed");
    }
    // scratch: As holds the field a candidate transforms, r the default shape's result (both are
    // free between steps; the projection fills them again)
    float* work = e.As;
    float* want = e.r;
    const float dtS = 0.5f;
    auto differs = [&]() {
        cudaMemsetAsync(count, 0, sizeof(unsigned), e.stream);
        k_count_diff<<<e.num_sms * 4, 256, 0, e.stream>>>((const unsigned*)work, (const unsigned*)want, n, count);
        unsigned h = 0;
        cudaMemcpyAsync(&h, count, sizeof(unsigned), cudaMemcpyDeviceToHost, e.stream);
        cudaStreamSynchronize(e.stream);
        return h != 0;
    };
    const int reps = 3;
    const long long l0 = e.launches;
    // ---- diffusion: depth, tile height, run length, on theta's boundary table (its row next to
    // the ground reads the ground face) and water vapour's (the one the other fields share) ----
    unsigned long long* hash = reinterpret_cast<unsigned long long*>(want);  // the result hashes
    auto diffuse_hashes = [&](unsigned long long out[2]) {
        cudaMemsetAsync(hash, 0, 2 * sizeof(unsigned long long), e.stream);
        const float* src[2] = {e.th, e.qv};
        for (int t = 0; t < 2; ++t) {
            cudaMemcpyAsync(work, src[t], n * 4, cudaMemcpyDeviceToDevice, e.stream);
            launch_diffuse(e, work, t, dtS);
            k_hash_bits<<<e.num_sms * 4, 256, 0, e.stream>>>((const unsigned*)work, n, hash + t);
        }
        cudaMemcpyAsync(out, hash, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, e.stream);
        cudaStreamSynchronize(e.stream);
    };
    e.tune = base;
    unsigned long long ref_hash[2];
    diffuse_hashes(ref_hash);
    struct Cand { int depth, h, bps; };
    std::vector<Cand> cands;
    for (int bps : {16, 32, 64}) cands.push_back({1, base.diffuse_h, bps});
    if (e.flat && (e.g.X % 4) == 0 && e.cfg.diffuse_sweeps >= 2)
    {
        for (int bps : {2, 4, 8}) cands.push_back({2, 14, bps});
        for (int bps : {4, 8}) cands.push_back({2, 6, bps});
        for (int h : {4, 8})
            for (int bps : {4, 8, 16}) cands.push_back({2, h, bps});
    }
    Tuning best = base;
    float best_ms = 1e30f;
    for (const Cand& c : cands) {
        Tuning tr = base;
        tr.diffuse_depth = c.depth;
        tr.diffuse_h = c.h;
        if (c.depth == 1) tr.diffuse_bps = c.bps;
        else tr.diffuse2_bps = c.bps;
        e.tune = tr;
        unsigned long long hh[2];
        diffuse_hashes(hh);
        if (hh[0] != ref_hash[0] || hh[1] != ref_hash[1]) continue;  // never accept a shape that changes the numbers
        const float ms = time_ms(e, reps, [&]() {
            launch_diffuse(e, work, 0, dtS);
            launch_diffuse(e, work, 1, dtS);
        });
        if (ms < best_ms) {
            best_ms = ms;
            best.diffuse_depth = tr.diffuse_depth;
            best.diffuse_h = tr.diffuse_h;
            best.diffuse_bps = tr.diffuse_bps;
            best.diffuse2_bps = tr.diffuse2_bps;
        }
    }
    // ---- PPM passes: each march's run length in turn (the water-vapour advection) ----
    float adv_ms = 0.0f;
    if (e.flat && (e.g.X % 4) == 0) {
        auto advect_once = [&]() {
            cudaMemcpyAsync(work, e.qv, n * 4, cudaMemcpyDeviceToDevice, e.stream);
            launch_advect(e, work, e.isenQv, CUSTOM, CUSTOM, dtS, 4, true);
        };
        e.tune = best;
        advect_once();
        cudaMemcpyAsync(want, work, n * 4, cudaMemcpyDeviceToDevice, e.stream);
        int* knobs[3] = {&best.ppm_bps, &best.ppmy_bps, &best.ppmz_bps};
        const int opts[3][3] = {{8, 16, 32}, {16, 32, 64}, {4, 8, 16}};
        for (int kk = 0; kk < 3; ++kk) {
            int pick = *knobs[kk];
            float pick_ms = 1e30f;
            for (int v : opts[kk]) {
                Tuning tr = best;
                int* kn[3] = {&tr.ppm_bps, &tr.ppmy_bps, &tr.ppmz_bps};
                *kn[kk] = v;
                e.tune = tr;
                advect_once();
                if (differs()) continue;
                const float ms = time_ms(e, reps, [&]() { launch_advect(e, work, e.isenQv, CUSTOM, CUSTOM, dtS, 4, true); });
                if (ms < pick_ms) {
                    pick_ms = ms;
                    pick = v;
                }
            }
            *knobs[kk] = pick;
            adv_ms = pick_ms;
        }
    }
    cudaFree(count);
    e.tune = best;
    e.launches = l0;  // tuning launches are not the step's
    e.adv_nsub = -1;  // the scratch advection touched the cached Courant count
    const skt_status st = check_cuda(e, "autotune");
    if (st != SKT_OK) return st;
    to_abi(best, &t);
    t.from_cache = 0;
    t.diffuse_ms = best_ms;
    t.advect_ms = adv_ms;
    if (cache_path && !cache_store(cache_path, key, t)) return report(&e, SKT_INVALID_ARG, "autotune: could not write the cache file");
    if (out) *out = t;
    return SKT_OK;
}

}  // extern "C"
