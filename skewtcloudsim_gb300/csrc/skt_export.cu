// Headless view and volume export: the editor's voxel view (editor::viewSky / viewGround,
// Game/editor.cpp:1041-1171, with the colour schemes of editor::setColors :53-112 evaluated as
// bee::colorScheme::getColor does, Engine/source/rendering/colors.cpp:28-67) computed per cell
// on the device, and a sparse brick export of any field (8^3 bricks, only those holding a value
// off the background are written: the leaf layout of VDB-style volumes).
//
// Both are read-only passes over the fields between steps, HBM-bound: the view reads the one to
// five fields its parameter needs and writes 13 bytes per cell; the brick export reads the field
// twice (activity, then the packing of active bricks) and writes the active bricks.
#include "skt_internal.cuh"

#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>

namespace skt {
namespace {

constexpr int kBrick = 8;             // brick edge in cells
constexpr int kBrickCells = 512;      // kBrick^3
constexpr int kRampMax = 13;

// One colour scheme: keys ascending (ties in the order the reference adds them: its std::sort
// of at most 13 entries is an insertion sort, which keeps that order), RGB per key.
struct Ramp {
    int n;
    float key[kRampMax];
    float rgb[kRampMax][3];
};
enum { R_TEMP = 0, R_MIX = 1, R_VEL = 2, R_DEBUG = 3, R_REAL = 4, R_PRESS = 5, R_COUNT = 6 };
__constant__ Ramp c_ramps[R_COUNT];

// bee::Colors (Engine/include/rendering/colors.hpp:34-47), alpha dropped as glm::vec3 does
#define C_BLACK {0.0f, 0.0f, 0.0f}
#define C_WHITE {1.0f, 1.0f, 1.0f}
#define C_RED {1.0f, 0.0f, 0.0f}
#define C_GREEN {0.0f, 1.0f, 0.0f}
#define C_BLUE {0.0f, 0.0f, 1.0f}
#define C_DODGER {0.0f, 0.5f, 1.0f}
#define C_ORANGE {1.0f, 0.66f, 0.0f}
#define C_CYAN {0.0f, 1.0f, 1.0f}
#define C_YELLOW {1.0f, 1.0f, 0.0f}
#define C_PURPLE {0.55f, 0.0f, 0.65f}

// editor::setColors (Game/editor.cpp:53-112), sorted
const Ramp kRamps[R_COUNT] = {
    // TemperatureSky
    {5, {-40 + 273.15f, -10 + 273.15f, 10 + 273.15f, 20 + 273.15f, 40 + 273.15f}, {C_BLUE, C_CYAN, C_GREEN, C_YELLOW, C_RED}},
    // mixingRatio
    {5, {0.0f, 0.0005f, 0.001f, 0.01f, 1.0f}, {C_BLUE, C_CYAN, C_GREEN, C_YELLOW, C_RED}},
    // velField
    {5, {0.0f, 10.0f, 25.0f, 50.0f, 100.0f}, {C_BLUE, C_CYAN, C_GREEN, C_YELLOW, C_RED}},
    // debugColor: Purple * 0.2 at -1, two keys at -0.01 (Purple, then Blue), Pink + (0, 0.8, 0) at 0.1
    {11, {-1.0f, -0.01f, -0.01f, -0.001f, -0.0001f, 0.0f, 0.0001f, 0.001f, 0.01f, 0.1f, 1.0f},
     {{0.55f * 0.2f, 0.0f * 0.2f, 0.65f * 0.2f}, C_PURPLE, C_BLUE, C_DODGER, C_CYAN, C_GREEN, C_YELLOW, C_ORANGE, C_RED,
      {1.0f + 0.0f, 0.0f + 0.8f, 0.72f + 0.0f}, C_WHITE}},
    // realistic
    {6, {0.0f, 0.0005f, 0.001f, 0.005f, 0.01f, 1.0f},
     {C_BLUE, {0.6f, 0.9f, 1.0f}, C_WHITE, {0.8f, 0.8f, 0.8f}, {0.4f, 0.4f, 0.4f}, C_BLACK}},
    // pressure
    {13, {0.0f, 100.0f, 200.0f, 300.0f, 400.0f, 600.0f, 700.0f, 800.0f, 900.0f, 950.0f, 975.0f, 1000.0f, 1050.0f},
     {C_PURPLE, {0.3f, 0.0f, 0.75f}, {0.1f, 0.8f, 0.9f}, {0.0f, 0.8f, 1.0f}, {0.0f, 0.4f, 1.0f}, {0.0f, 0.8f, 0.8f},
      {0.0f, 1.0f, 0.0f}, {0.4f, 0.8f, 0.0f}, {0.8f, 0.0f, 0.0f}, {1.0f, 0.6f, 0.6f}, {0.6f, 0.5f, 0.5f},
      {0.2f, 0.2f, 0.2f}, C_WHITE}},
};

// getColor: lower_bound on the keys; the end and the first key return a key colour; otherwise
// Lerp (Engine/include/math/math.hpp:11-15) of the two neighbouring colours by the clamped
// fraction, a * (1 - t) + b * t, every operation rounded on its own (no contraction).
__device__ __forceinline__ void ramp_color(const Ramp* ramps, int which, float v, float* out) {
    const Ramp& r = ramps[which];
    int it = 0;
    while (it < r.n && r.key[it] < v) it++;
    int pick = -1;
    if (it == r.n) pick = r.n - 1;
    else if (it == 0 || r.key[it] == v) pick = it;
    else if (v == r.key[it - 1]) pick = it - 1;
    if (pick >= 0) {
        out[0] = r.rgb[pick][0];
        out[1] = r.rgb[pick][1];
        out[2] = r.rgb[pick][2];
        return;
    }
    float t = __fdiv_rn(__fsub_rn(v, r.key[it - 1]), __fsub_rn(r.key[it], r.key[it - 1]));
    t = (1.0f < t) ? 1.0f : t;  // std::min(t, 1)
    t = (0.0f < t) ? t : 0.0f;  // std::max(0, t)
    const float s = __fsub_rn(1.0f, t);
#pragma unroll
    for (int c = 0; c < 3; c++) out[c] = __fadd_rn(__fmul_rn(r.rgb[it - 1][c], s), __fmul_rn(r.rgb[it][c], t));
}

struct ViewArgs {
    const float *th, *qv, *qw, *qc, *qr, *qs, *qi, *u, *v, *w, *p, *dbg, *Pg;
    const float* gfield;  // the ground view's array (nullptr: no ground view)
    int sky_param, ground_param;
    int lo[3], hi[3];     // view box in (x, y, z), reference layout
};

// editor::viewSky and viewGround for every cell. kind: 0 not drawn, 1 sky voxel, 2 ground below
// the surface (brown), 3 the ground surface voxel (the ground view's colour). A block covers 128
// cells of one row and walks z; the schemes sit in shared memory (threads of a warp search them
// at different keys, which constant memory would serve one address at a time).
__global__ void __launch_bounds__(128) k_view(Grid g, ViewArgs a, float* __restrict__ rgb, uint8_t* __restrict__ kind) {
    __shared__ Ramp ramps[R_COUNT];
    for (int i = threadIdx.x; i < (int)(sizeof(ramps) / sizeof(int)); i += blockDim.x)
        reinterpret_cast<int*>(ramps)[i] = reinterpret_cast<const int*>(c_ramps)[i];
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    const int zlen = (g.Z + gridDim.z - 1) / gridDim.z, zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    if (x >= g.X) return;
    for (int z = zs; z < ze; ++z) {
        const int c = x + y * g.X + z * g.XY;
        const long long i = c;
        const int cg = x + z * g.X;
        const int gh = g.gh[cg];
        float col[3] = {0.0f, 0.0f, 0.0f};
        uint8_t k = 0;
        const bool in_box = x >= a.lo[0] && x < a.hi[0] && y >= a.lo[1] && y < a.hi[1] && z >= a.lo[2] && z < a.hi[2];
        if (y == gh) {
            if (a.gfield) {  // viewGround draws the surface voxel of every column
                ramp_color(ramps, a.ground_param == 0 ? R_TEMP : R_MIX, a.gfield[cg], col);
                k = 3;
            }
        } else if (in_box && y < gh) {
            col[0] = 0.5f; col[1] = 0.3f; col[2] = 0.0f;  // Colors::Brown
            k = 2;
        } else if (in_box) {
            k = 1;
            switch (a.sky_param) {
                case SKT_POTTEMP: {  // temperature: potentialTemp(theta - 273.15, ground P, p) + 273.15
                    const float tz = __fsub_rn(a.th[c], 273.15f);
                    const float kappa = 287.0528f / 1003.5f;
                    const float f = powf(__fdiv_rn(a.p[c], a.Pg[cg]), kappa);
                    const float t = __fadd_rn(__fsub_rn(__fmul_rn(__fadd_rn(tz, 273.15f), f), 273.15f), 273.15f);
                    ramp_color(ramps, R_TEMP, t, col);
                    break;
                }
                case SKT_QV: ramp_color(ramps, R_MIX, a.qv[c], col); break;
                case SKT_QW: ramp_color(ramps, R_MIX, a.qw[c], col); break;
                case SKT_QC: ramp_color(ramps, R_MIX, a.qc[c], col); break;
                case SKT_QR: ramp_color(ramps, R_MIX, a.qr[c], col); break;
                case SKT_QS: ramp_color(ramps, R_MIX, a.qs[c], col); break;
                case SKT_QI: ramp_color(ramps, R_MIX, a.qi[c], col); break;
                case SKT_WIND: {  // |getUV| (Game/environment.cpp:2083-2095): the z term averages w
                                  // with the v of the cell behind, as the reference does
                    const float uc = a.u[c], vc = a.v[c], wc = a.w[c];
                    const float pu = x == 0 ? uc : a.u[c - 1];
                    const float pv = y == 0 ? 0.0f : a.v[c - g.X];
                    const float pw = z == 0 ? 0.0f : a.v[c - g.XY];
                    const float cx = __fdiv_rn(__fadd_rn(pu, uc), 2.0f);
                    const float cy = __fdiv_rn(__fadd_rn(pv, vc), 2.0f);
                    const float cz = __fdiv_rn(__fadd_rn(pw, wc), 2.0f);
                    const float d = __fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz));
                    ramp_color(ramps, R_VEL, __fsqrt_rn(d), col);
                    break;
                }
                case SKT_PRESSURE: ramp_color(ramps, R_PRESS, a.p[c], col); break;
                case SKT_DEBUG1: {  // the "realistic" view of all condensate; faint cells are not drawn
                    const float s = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.qw[c], a.qc[c]), a.qr[c]), a.qs[c]), a.qi[c]);
                    ramp_color(ramps, R_REAL, s, col);
                    if ((double)s < 0.0001) {  // float against a double literal, as in the reference
                        k = 0;
                        col[0] = col[1] = col[2] = 0.0f;
                    }
                    break;
                }
                case SKT_DEBUG2:
                case SKT_DEBUG3: ramp_color(ramps, R_DEBUG, a.dbg[c], col); break;
                default: k = 0; break;
            }
        }
        rgb[3 * i + 0] = col[0];
        rgb[3 * i + 1] = col[1];
        rgb[3 * i + 2] = col[2];
        kind[i] = k;
    }
}

// ---- sparse bricks -------------------------------------------------------------------------

struct BrickGrid {
    int nbx, nby, nbz, nb;
};

__device__ __forceinline__ bool off_background(float v, float bg, float thr) {
    return !(fabsf(__fsub_rn(v, bg)) <= thr);  // NaN is off the background
}

// one warp per brick: does any cell differ from the background by more than the threshold
__global__ void __launch_bounds__(256) k_brick_flag(Grid g, BrickGrid b, const float* __restrict__ f, float bg, float thr,
                                                    int* __restrict__ flags) {
    const int lane = threadIdx.x & 31;
    for (int br = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; br < b.nb; br += (gridDim.x * blockDim.x) >> 5) {
        const int bx = br % b.nbx, by = (br / b.nbx) % b.nby, bz = br / (b.nbx * b.nby);
        bool any = false;
        for (int k = lane; k < kBrickCells; k += 32) {
            const int x = bx * kBrick + (k & 7), y = by * kBrick + ((k >> 3) & 7), z = bz * kBrick + (k >> 6);
            if (x < g.X && y < g.Y && z < g.Z) any |= off_background(f[x + y * g.X + (size_t)z * g.XY], bg, thr);
        }
        any = __any_sync(0xffffffffu, any);
        if (lane == 0) flags[br] = any ? 1 : 0;
    }
}

// exclusive scan of the flags into output slots, in two levels: k_brick_scan_blocks scans each
// run of 1024 flags in one block (slots within the run; the run's total to totals[run]),
// k_brick_scan_totals scans the run totals into run offsets (one block; *count = all bricks)
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int ws = lane < nw ? warp_sums[lane] : 0;
        int wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) warp_sums[lane] = wi - ws;
        if (lane == 31) warp_sums[32] = wi;
    }
    __syncthreads();
    total = warp_sums[32];
    const int r = warp_sums[wid] + incl - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_brick_scan_blocks(int nb, int* __restrict__ flags, int* __restrict__ totals) {
    __shared__ int warp_sums[33];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int f = i < nb ? flags[i] : 0;
    int total;
    const int slot = block_exclusive_scan(f, warp_sums, total);
    if (i < nb) flags[i] = f ? slot : -1;
    if (threadIdx.x == 0) totals[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_brick_scan_totals(int nruns, int* __restrict__ totals, int* __restrict__ count) {
    __shared__ int warp_sums[33];
    int carry = 0;
    for (int base = 0; base < nruns; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nruns ? totals[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, warp_sums, total);
        if (i < nruns) totals[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *count = carry;
}

// one warp per active brick: its cells in brick order (x fastest), cells past the grid edge hold
// the background; coordinates as three uint32
template <typename T>
__global__ void __launch_bounds__(256) k_brick_pack(Grid g, BrickGrid b, const float* __restrict__ f, float bg,
                                                    const int* __restrict__ slots, const int* __restrict__ run_offsets,
                                                    T* __restrict__ out, uint32_t* __restrict__ coords) {
    const int lane = threadIdx.x & 31;
    for (int br = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; br < b.nb; br += (gridDim.x * blockDim.x) >> 5) {
        int slot = slots[br];
        if (slot < 0) continue;
        slot += run_offsets[br >> 10];
        const int bx = br % b.nbx, by = (br / b.nbx) % b.nby, bz = br / (b.nbx * b.nby);
        T* dst = out + (size_t)slot * kBrickCells;
        for (int k = lane; k < kBrickCells; k += 32) {
            const int x = bx * kBrick + (k & 7), y = by * kBrick + ((k >> 3) & 7), z = bz * kBrick + (k >> 6);
            const float v = (x < g.X && y < g.Y && z < g.Z) ? f[x + y * g.X + (size_t)z * g.XY] : bg;
            if constexpr (sizeof(T) == 2) dst[k] = __float2half_rn(v);
            else dst[k] = v;
        }
        if (lane < 3) coords[3 * (size_t)slot + lane] = lane == 0 ? bx : lane == 1 ? by : bz;
    }
}

int grid_blocks(const Env& e, long long work_threads) {
    const long long b = (work_threads + 255) / 256;
    const long long cap = (long long)e.num_sms * 8;
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

}  // namespace
}  // namespace skt

using namespace skt;

extern "C" {

skt_status skt_view_volume(skt_env* env, int sky_param, int ground_param, const int lo[3], const int hi[3], float* rgb,
                           uint8_t* kind, size_t n) {
    if (!env || !rgb || !kind) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (!e.initialized) return report(&e, SKT_NOT_INITIALIZED, "skt_init first");
    if (n != (size_t)e.g.N) return report(&e, SKT_INVALID_ARG, "size mismatch (n must be nx*ny*nz)");
    ViewArgs a{};
    a.th = e.th; a.qv = e.qv; a.qw = e.qw; a.qc = e.qc; a.qr = e.qr; a.qs = e.qs; a.qi = e.qi;
    a.u = e.u; a.v = e.v; a.w = e.w; a.p = e.p; a.Pg = e.Pg;
    a.sky_param = sky_param;
    a.ground_param = ground_param;
    switch (sky_param) {
        case SKT_POTTEMP: case SKT_QV: case SKT_QW: case SKT_QC: case SKT_QR: case SKT_QS: case SKT_QI:
        case SKT_WIND: case SKT_PRESSURE: case SKT_DEBUG1: break;
        case SKT_DEBUG2:
        case SKT_DEBUG3:
            a.dbg = field_ptr(e, sky_param, 0);
            if (!a.dbg) return report(&e, SKT_INVALID_ARG, "the DEBUG2 view needs skt_set_diagnostics(env, SKT_DIAG_BUOYANCY)");
            break;
        default: return report(&e, SKT_INVALID_ARG, "no view for this parameter");
    }
    // ground views (Game/editor.cpp:1147-1164): 0 temperature, 1 Qrs, 2 Qgr, 3 Qgs, 4 Qgi; -1 none
    static const int gsel[5] = {SKT_G_T, SKT_G_QRS, SKT_G_QGR, SKT_G_QGS, SKT_G_QGI};
    if (ground_param < -1 || ground_param > 4) return report(&e, SKT_INVALID_ARG, "ground view must be -1..4");
    a.gfield = ground_param >= 0 ? ground_field_ptr(e, gsel[ground_param]) : nullptr;
    const int dims[3] = {e.g.X, e.g.Y, e.g.Z};
    for (int d = 0; d < 3; d++) {
        a.lo[d] = lo ? lo[d] : 0;
        a.hi[d] = hi ? hi[d] : dims[d];
    }
    const size_t bytes_rgb = (size_t)e.g.N * 12, bytes_kind = (size_t)e.g.N;
    // staging: the brick scratch doubles as the view's output buffer
    if (e.brick_out_bytes < bytes_rgb + bytes_kind) {
        if (e.brick_out) cudaFree(e.brick_out);
        e.brick_out = nullptr;
        e.brick_out_bytes = 0;
        if (cudaMalloc(&e.brick_out, bytes_rgb + bytes_kind) != cudaSuccess) {
            cudaGetLastError();
            return report(&e, SKT_OUT_OF_MEMORY, "view buffer allocation failed");
        }
        e.brick_out_bytes = bytes_rgb + bytes_kind;
    }
    cudaMemcpyToSymbolAsync(c_ramps, kRamps, sizeof(kRamps), 0, cudaMemcpyHostToDevice, e.stream);
    float* d_rgb = (float*)e.brick_out;
    uint8_t* d_kind = (uint8_t*)e.brick_out + bytes_rgb;
    const int vx = (e.g.X + 127) / 128;
    const int vz = std::max(1, std::min(e.g.Z, (e.num_sms * 64 + vx * e.g.Y - 1) / (vx * e.g.Y)));  // ~64 blocks per SM
    k_view<<<dim3(vx, e.g.Y, vz), 128, 0, e.stream>>>(e.g, a, d_rgb, d_kind);
    e.launches += 1;
    cudaMemcpyAsync(rgb, d_rgb, bytes_rgb, cudaMemcpyDeviceToHost, e.stream);
    cudaMemcpyAsync(kind, d_kind, bytes_kind, cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    return check_cuda(e, "view_volume");
}

skt_status skt_export_bricks(skt_env* env, int param, int dir, float background, float threshold, int half,
                             uint32_t* coords, void* values, size_t capacity, size_t* count) {
    if (!env || !count) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    *count = 0;
    const float* f = field_ptr(e, param, dir);
    if (!f) return report(&e, SKT_INVALID_ARG, "unknown field selector (debug fields need skt_set_diagnostics)");
    BrickGrid b{(e.g.X + kBrick - 1) / kBrick, (e.g.Y + kBrick - 1) / kBrick, (e.g.Z + kBrick - 1) / kBrick, 0};
    b.nb = b.nbx * b.nby * b.nbz;
    const int nruns = (b.nb + 1023) / 1024;
    if (!e.brick_flags) {  // flags, the run totals/offsets, the count
        if (cudaMalloc(&e.brick_flags, sizeof(int) * ((size_t)b.nb + nruns + 1)) != cudaSuccess) {
            cudaGetLastError();
            e.brick_flags = nullptr;
            return report(&e, SKT_OUT_OF_MEMORY, "brick flag allocation failed");
        }
        e.brick_count = e.brick_flags + b.nb + nruns;
    }
    int* runs = e.brick_flags + b.nb;
    const int nblk = grid_blocks(e, (long long)b.nb * 32);
    k_brick_flag<<<nblk, 256, 0, e.stream>>>(e.g, b, f, background, threshold, e.brick_flags);
    k_brick_scan_blocks<<<nruns, 1024, 0, e.stream>>>(b.nb, e.brick_flags, runs);
    k_brick_scan_totals<<<1, 1024, 0, e.stream>>>(nruns, runs, e.brick_count);
    e.launches += 3;
    int n = 0;
    cudaMemcpyAsync(&n, e.brick_count, sizeof(int), cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    skt_status st = check_cuda(e, "export_bricks");
    if (st != SKT_OK) return st;
    *count = (size_t)n;
    if (!coords || !values || capacity < (size_t)n || n == 0) return SKT_OK;  // the count alone
    const size_t elem = half ? 2 : 4;
    const size_t vbytes = (size_t)n * kBrickCells * elem, cbytes = (size_t)n * 3 * sizeof(uint32_t);
    if (e.brick_out_bytes < vbytes + cbytes) {
        if (e.brick_out) cudaFree(e.brick_out);
        e.brick_out = nullptr;
        e.brick_out_bytes = 0;
        if (cudaMalloc(&e.brick_out, vbytes + cbytes) != cudaSuccess) {
            cudaGetLastError();
            return report(&e, SKT_OUT_OF_MEMORY, "brick buffer allocation failed");
        }
        e.brick_out_bytes = vbytes + cbytes;
    }
    uint32_t* d_coords = (uint32_t*)((char*)e.brick_out + vbytes);
    if (half)
        k_brick_pack<__half><<<nblk, 256, 0, e.stream>>>(e.g, b, f, background, e.brick_flags, runs, (__half*)e.brick_out, d_coords);
    else
        k_brick_pack<float><<<nblk, 256, 0, e.stream>>>(e.g, b, f, background, e.brick_flags, runs, (float*)e.brick_out, d_coords);
    e.launches += 1;
    cudaMemcpyAsync(values, e.brick_out, vbytes, cudaMemcpyDeviceToHost, e.stream);
    cudaMemcpyAsync(coords, d_coords, cbytes, cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    return check_cuda(e, "export_bricks");
}

}  // extern "C"
