// C ABI of libskewt_gb300 and the host orchestration of one step
// (environmentGPU, Game/environment.cu:71-1300).
#include "skt_internal.cuh"
#include "../../include/skewt.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

using namespace skt;

namespace {

thread_local std::string g_create_err;

skt_status fail(Env* e, skt_status st, const std::string& msg) {
    if (e) e->err = msg;
    else g_create_err = msg;
    return st;
}

skt_status cuda_check(Env& e, const char* where) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        e.err = std::string(where) + ": " + cudaGetErrorString(err);
        return err == cudaErrorMemoryAllocation ? SKT_OUT_OF_MEMORY : SKT_CUDA_ERROR;
    }
    return SKT_OK;
}

// irridianceGPU Game/environment.cu:1021-1034 (host, float)
float irradiance(float time, int day, float longitude, float sun) {
    const float Gs = 1361.0f * sun;
    const float rd = 1 + 0.034f * cosf(2 * 3.14159265359f * day / 365);
    const float sd = 0.409f * sinf(2 * 3.14159265359f / 365 * (day - 81));
    const float th = time / 3600;
    const float lr = longitude * 0.01745329251994329576923690768489f;  // glm::radians
    const float sr = (th - (6.0f + 14.0f / 2.0f)) * (3.14159265359f / 12.0f);
    const float v = Gs * rd * (sinf(lr) * sinf(sd) + cosf(lr) * cosf(sd) * cosf(sr));
    return v > 0.0f ? v : 0.0f;
}

__global__ void k_fill(float* a, float v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

float* sky_ptr(Env& e, int param, int dir) {
    switch (param) {
        case SKT_POTTEMP: return e.th;
        case SKT_QV: return e.qv;
        case SKT_QW: return e.qw;
        case SKT_QC: return e.qc;
        case SKT_QR: return e.qr;
        case SKT_QS: return e.qs;
        case SKT_QI: return e.qi;
        case SKT_WIND:
            if (dir == SKT_LEFT || dir == SKT_RIGHT) return e.u;
            if (dir == SKT_UP || dir == SKT_DOWN) return e.v;
            if (dir == SKT_FORWARD || dir == SKT_BACKWARD) return e.w;
            return nullptr;
        case SKT_PRESSURE: return e.p;
        case SKT_DENSITY: return e.rho;
        case SKT_DEBUG1: return e.dbg_zero;
        case SKT_DEBUG2: return e.dbg_buoy;
        case SKT_DEBUG3: return e.pp;  // the projection's correction, left in pp by every step
        default: return nullptr;
    }
}
float* ground_ptr(Env& e, int which) {
    switch (which) {
        case SKT_G_QRS: return e.Qrs;
        case SKT_G_QGR: return e.Qgr;
        case SKT_G_QGS: return e.Qgs;
        case SKT_G_QGI: return e.Qgi;
        case SKT_G_P: return e.Pg;
        case SKT_G_TIME_WET: return e.tg;
        case SKT_G_T: return e.Tg;
        case SKT_G_CLOUD_COVER: return e.cover;
        default: return nullptr;
    }
}
float* column_ptr(Env& e, int which) {
    switch (which) {
        case SKT_C_ISEN_T: return e.isenT;
        case SKT_C_ISEN_QV: return e.isenQv;
        case SKT_C_DEF_U: return e.defU;
        case SKT_C_DEF_W: return e.defW;
        case SKT_C_PRESSURE: return e.pcol;
        default: return nullptr;
    }
}

// The launches of one step in the reference's stage order (Game/environment.cu:391-555); the
// ground kernel takes irr, or in graph mode reads it from the graph's first node.
void queue_step(Env& e, float dt, float speed, float irr) {
    const float dtS = dt * speed;
    const bool hs = true;
    // ground, then setTempsAtGround (fused into the ground column kernel)
    launch_ground(e, dt, speed, irr);
    // theta
    launch_diffuse(e, e.th, 0, dtS);
    e.last_nsub[0] = launch_advect(e, e.th, e.isenT, CUSTOM, CUSTOM, dtS, 0, hs);
    // momentum
    launch_buoyancy(e, dtS);
    launch_diffuse(e, e.u, 2, dtS);
    launch_diffuse(e, e.v, 3, dtS);
    launch_diffuse(e, e.w, 4, dtS);
    e.last_nsub[1] = launch_advect(e, e.u, e.defU, CUSTOM, DIRICHLET, dtS, 1, hs);
    e.last_nsub[2] = launch_advect(e, e.v, e.zeroY, DIRICHLET, DIRICHLET, dtS, 2, hs);
    e.last_nsub[3] = launch_advect(e, e.w, e.defW, CUSTOM, DIRICHLET, dtS, 3, hs);
    launch_init_density(e);
    launch_project(e, dtS);
    launch_new_pressure(e);
    // moisture
    launch_diffuse(e, e.qv, 1, dtS);
    e.last_nsub[4] = launch_advect(e, e.qv, e.isenQv, CUSTOM, CUSTOM, dtS, 4, hs);
    // the wind is the same for every moisture field: its substep count is computed once
    launch_diffuse(e, e.qw, 5, dtS);
    e.last_nsub[5] = launch_advect(e, e.qw, e.zeroY, DIRICHLET, DIRICHLET, dtS, 5, hs, true);
    launch_diffuse(e, e.qc, 5, dtS);
    e.last_nsub[6] = launch_advect(e, e.qc, e.zeroY, DIRICHLET, DIRICHLET, dtS, 6, hs, true);
    // rain, snow and ice: diffuse, fall, advect each (the reference's order per species; the
    // species do not read one another here, so the three falls run as one column march)
    launch_diffuse(e, e.qr, 5, dtS);
    launch_diffuse(e, e.qs, 5, dtS);
    launch_diffuse(e, e.qi, 5, dtS);
    launch_precip3(e, dtS);
    e.last_nsub[7] = launch_advect(e, e.qr, e.zeroY, DIRICHLET, DIRICHLET, dtS, 7, hs, true);
    e.last_nsub[8] = launch_advect(e, e.qs, e.zeroY, DIRICHLET, DIRICHLET, dtS, 8, hs, true);
    e.last_nsub[9] = launch_advect(e, e.qi, e.zeroY, DIRICHLET, DIRICHLET, dtS, 9, hs, true);
    // microphysics + latent heat
    launch_micro(e, dt, speed);
}

// the host clock (m_time, Game/environment.cu:550-551)
void advance_clock(Env& e, float dt, float speed) {
    e.sim_time += speed * dt * float(!e.pause);
    if (e.sim_time > 86400.0f) e.sim_time = 0.0f;
}

// One step in the reference's stage order (Game/environment.cu:391-555), stream-ordered.
skt_status run_step(Env& e, float dt, float speed) {
    const float irr = irradiance(e.sim_time, e.day, e.longitude, e.sun);
    // editorDataGPU at the start of updateGPU (Game/environment.cu:398): after a ground edit
    if (e.ground_changed) launch_editor_block(e);
    queue_step(e, dt, speed, irr);
    advance_clock(e, dt, speed);
    return cuda_check(e, "step");
}

// ---- graph mode: the step captured once, its loops as conditional WHILE nodes ----------------

__global__ void k_set_irr(float* dst, float irr) { *dst = irr; }

#define GCHECK(call)                                                                  \
    do {                                                                              \
        const cudaError_t err_ = (call);                                              \
        if (err_ != cudaSuccess && !e.graph_fail) {                                   \
            e.graph_fail = true;                                                      \
            e.graph_err = std::string(#call) + ": " + cudaGetErrorString(err_);        \
        }                                                                             \
    } while (0)

Env::GraphKey graph_key(const Env& e, float dt, float speed) {
    Env::GraphKey k{};
    k.dt = dt;
    k.speed = speed;
    k.flat = e.flat;
    k.rates_on = e.rates_on;
    for (int i = 0; i < 3; ++i) {
        k.rate_lo[i] = e.rates_on ? e.rate_lo[i] : 0;
        k.rate_hi[i] = e.rates_on ? e.rate_hi[i] : 0;
    }
    k.diag_flags = e.diag_flags;
    k.stencil_sms = stencil_sms(e);
    k.tune = e.tune;
    return k;
}
bool same_key(const Env::GraphKey& a, const Env::GraphKey& b) {
    const Tuning &s = a.tune, &t = b.tune;
    return a.dt == b.dt && a.speed == b.speed && a.flat == b.flat && a.rates_on == b.rates_on && a.diag_flags == b.diag_flags &&
           a.stencil_sms == b.stencil_sms &&
           a.rate_lo[0] == b.rate_lo[0] && a.rate_lo[1] == b.rate_lo[1] && a.rate_lo[2] == b.rate_lo[2] && a.rate_hi[0] == b.rate_hi[0] &&
           a.rate_hi[1] == b.rate_hi[1] && a.rate_hi[2] == b.rate_hi[2] && s.diffuse_depth == t.diffuse_depth && s.diffuse_h == t.diffuse_h &&
           s.diffuse_bps == t.diffuse_bps && s.diffuse2_bps == t.diffuse2_bps && s.ppm_bps == t.ppm_bps && s.ppmy_bps == t.ppmy_bps &&
           s.ppmz_bps == t.ppmz_bps;
}

void drop_graph(Env& e) {
    if (e.graph_exec) cudaGraphExecDestroy(e.graph_exec);
    if (e.graph) cudaGraphDestroy(e.graph);
    e.graph_exec = nullptr;
    e.graph = nullptr;
    e.book = GraphBook{};
}

skt_status ensure_side_streams(Env& e) {
    for (int i = 0; i < 4; ++i)
        if (!e.side[i] && cudaStreamCreateWithFlags(&e.side[i], cudaStreamNonBlocking) != cudaSuccess)
            return fail(&e, SKT_CUDA_ERROR, "graph: side stream creation failed");
    return SKT_OK;
}

// Queues one step of e into the capture that e.stream takes part in (its own, or an ensemble's),
// with the irradiance node first, and fills `book`.
void capture_into(Env& e, float dt, float speed, GraphBook& book) {
    e.graph_loops = 0;
    e.body_acc = 0;
    e.graph_depth = 0;
    const long long l0 = e.launches;
    e.capturing = true;
    e.irr_dev = &e.sc->irr;
    k_set_irr<<<1, 1, 0, e.stream>>>(e.irr_dev, 0.0f);
    e.launches += 1;
    {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        GCHECK(cudaStreamGetCaptureInfo(e.stream, &cs, nullptr, nullptr, &deps, nullptr, &nd));
        book.irr_node = (nd == 1 && deps) ? deps[0] : nullptr;
    }
    queue_step(e, dt, speed, 0.0f);
    e.capturing = false;
    const long long captured = e.launches - l0;
    e.launches = l0;
    book.statics = captured - e.body_acc;
    book.loops = e.graph_loops;
    for (int l = 0; l < e.graph_loops; ++l) book.body[l] = e.loop_body[l];
    if (!e.graph_fail && !book.irr_node) {
        e.graph_fail = true;
        e.graph_err = "graph: the irradiance node was not found";
    }
}

// the device's trip counters as they stand (a captured step's loops count on from there)
void read_trips(Env& e) {
    cudaMemcpyAsync(e.trips_seen, e.sc->trips, sizeof(e.trips_seen), cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
}

// Captures one step (as queue_step queues it) into e.graph_exec.
skt_status capture_step(Env& e, float dt, float speed) {
    drop_graph(e);
    if (ensure_side_streams(e) != SKT_OK) return SKT_CUDA_ERROR;
    e.graph_fail = false;
    e.graph_err.clear();
    GCHECK(cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeRelaxed));
    GraphBook book;
    capture_into(e, dt, speed, book);
    cudaGraph_t graph = nullptr;
    GCHECK(cudaStreamEndCapture(e.stream, &graph));
    e.graph = graph;
    if (!e.graph_fail) GCHECK(cudaGraphInstantiate(&e.graph_exec, graph, 0));
    if (e.graph_fail) {
        cudaGetLastError();
        const std::string m = e.graph_err;
        drop_graph(e);
        return fail(&e, SKT_CUDA_ERROR, m);
    }
    e.book = book;
    e.gkey = graph_key(e, dt, speed);
    read_trips(e);
    return cuda_check(e, "graph capture");
}

// Before a launch of a captured step: the ground block after an edit (queued on `before`, which the
// launch follows) and this step's irradiance into the step's irradiance node.
skt_status prepare_launch(Env& e, cudaGraphExec_t exec, const GraphBook& book, cudaStream_t before) {
    if (e.ground_changed) {
        cudaStream_t own = e.stream;
        e.stream = before;
        launch_editor_block(e);
        e.stream = own;
    }
    e.ground_changed = 0;
    float irr = irradiance(e.sim_time, e.day, e.longitude, e.sun);
    cudaKernelNodeParams kp{};
    void* args[2] = {&e.irr_dev, &irr};
    kp.func = (void*)k_set_irr;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.kernelParams = args;
    if (cudaGraphExecKernelNodeSetParams(exec, book.irr_node, &kp) != cudaSuccess) return cuda_check(e, "graph irradiance update");
    return SKT_OK;
}

// After launches of a captured step (the stream synchronised): the solver scalars, the stats and
// the kernel count from the trip counters.
void finish_graph_steps(Env& e, const GraphBook& book, int nsteps) {
    fetch_scalars(e);
    const Scalars& h = *e.host_sc;
    long long ran = book.statics * nsteps;
    for (int l = 0; l < book.loops; ++l) {
        ran += (long long)(h.trips[l] - e.trips_seen[l]) * book.body[l];
        e.trips_seen[l] = h.trips[l];
    }
    e.launches += ran;
    for (int f = 0; f < 10; ++f) e.last_nsub[f] = h.nsub_f[f];
    if (e.cfg.precision == 1) {
        e.last_outer = h.outer;
        e.last_iters = h.outer_inner_total;
        e.last_residual = float(h.rnorm0 > 0 ? h.rnorm / h.rnorm0 : 0.0);
        e.last_converged = h.refine_done == 1;
    } else {
        e.last_iters = h.iters;
        e.last_residual = h.residual;
        e.last_converged = h.converged == 1;
    }
}

// the status a graph step left on the device, turned into the call's result (and cleared)
skt_status graph_status(Env& e) {
    const int dev_status = e.host_sc->status;
    if (dev_status != 0) {
        cudaMemsetAsync(&e.sc->status, 0, sizeof(int), e.stream);
        cudaStreamSynchronize(e.stream);
        e.host_sc->status = 0;
        return fail(&e, skt_status(dev_status),
                    dev_status == SKT_TIMEOUT ? "a kernel's wait for its streamed data ran out (the state is not valid)"
                                              : "a step of this call met a NaN or Inf (in the wind or in a pressure-solver "
                                                "reduction: a non-finite field value or a zero-density cell); the state is not valid");
    }
    return e.last_converged ? SKT_OK : SKT_NOT_CONVERGED;
}

// nsteps launches of the captured step; the host reads the solver scalars once at the end
// Waits for the graph steps queued by skt_step_async and accounts for them (solver scalars, stats,
// kernel count, device time since the first of them); the status they left on the device.
skt_status collect_async(Env& e) {
    if (e.async_steps == 0) return SKT_OK;
    const int n = e.async_steps;
    e.async_steps = 0;
    cudaEventRecord(e.ev1, e.stream);
    cudaEventSynchronize(e.ev1);
    cudaEventElapsedTime(&e.last_gpu_ms, e.ev0, e.ev1);
    const skt_status st = cuda_check(e, "graph step");
    if (st != SKT_OK) return st;
    finish_graph_steps(e, e.book, n);
    return graph_status(e);
}

// Queues nsteps launches of the captured step (capturing it first when dt, speed, the terrain's
// flatness, the diagnostics or the tuning changed); the steps are collected by collect_async.
skt_status launch_graph_steps(Env& e, float dt, float speed, int nsteps) {
    if (!e.graph_exec || !same_key(e.gkey, graph_key(e, dt, speed))) {
        // a new capture replaces the graph and its bookkeeping: collect what the old one queued
        if (e.async_steps > 0) {
            const skt_status pst = collect_async(e);
            if (pst != SKT_OK && pst != SKT_NOT_CONVERGED) return pst;
        }
        const skt_status st = capture_step(e, dt, speed);
        if (st != SKT_OK) return st;
    }
    if (!e.ev0) { cudaEventCreate(&e.ev0); cudaEventCreate(&e.ev1); }
    if (e.async_steps == 0) cudaEventRecord(e.ev0, e.stream);
    for (int i = 0; i < nsteps; ++i) {
        const skt_status ps = prepare_launch(e, e.graph_exec, e.book, e.stream);
        if (ps != SKT_OK) return ps;
        if (cudaGraphLaunch(e.graph_exec, e.stream) != cudaSuccess) return cuda_check(e, "graph launch");
        advance_clock(e, dt, speed);
        ++e.async_steps;
    }
    return SKT_OK;
}

skt_status step_graph(Env& e, float dt, float speed, int nsteps) {
    const skt_status st = launch_graph_steps(e, dt, speed, nsteps);
    if (st != SKT_OK) return st;
    const skt_status cs = collect_async(e);
    return cs == SKT_NOT_CONVERGED ? SKT_OK : cs;  // skt_step turns the solver state into its status
}

}  // namespace

namespace skt {
void graph_while(Env& e, const std::function<void(cudaGraphConditionalHandle)>& init,
                 const std::function<void(cudaGraphConditionalHandle, int)>& body) {
    if (e.graph_loops >= kMaxGraphLoops || e.graph_depth >= 4) {
        if (!e.graph_fail) {
            e.graph_fail = true;
            e.graph_err = "graph: too many or too deeply nested loops";
        }
        return;
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    GCHECK(cudaStreamGetCaptureInfo(e.stream, &cs, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphConditionalHandle h{};
    GCHECK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    init(h);
    GCHECK(cudaStreamGetCaptureInfo(e.stream, &cs, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    GCHECK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    GCHECK(cudaStreamUpdateCaptureDependencies(e.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    const int loop = e.graph_loops++;
    cudaStream_t outer = e.stream, side = e.side[e.graph_depth++];
    GCHECK(cudaStreamBeginCaptureToGraph(side, p.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    e.stream = side;
    const long long l0 = e.launches, acc0 = e.body_acc;
    e.body_acc = 0;
    body(h, loop);
    const long long all = e.launches - l0;
    e.loop_body[loop] = all - e.body_acc;  // this body's own kernels, nested bodies excluded
    e.body_acc = acc0 + all;               // the enclosing level sees the whole body as looped
    e.stream = outer;
    cudaGraph_t done = nullptr;
    GCHECK(cudaStreamEndCapture(side, &done));
    e.graph_depth--;
}

void set_global_error(const char* msg) { g_create_err = msg ? msg : ""; }
skt_status report(Env* e, skt_status st, const char* msg) { return fail(e, st, msg); }
float* field_ptr(Env& e, int param, int dir) { return sky_ptr(e, param, dir); }
float* ground_field_ptr(Env& e, int which) { return ground_ptr(e, which); }
skt_status check_cuda(Env& e, const char* where) { return cuda_check(e, where); }
__global__ void k_fetch_sc(const unsigned* __restrict__ src, unsigned* dst, int nwords) {
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
}
// AoS (u, v, w per cell, Game/environment.cu:263-281) to the three SoA fields on the device. The
// AoS array of 3n floats arrives in three pieces of n floats (float f of the array is float
// f % n of piece f / n).
__global__ void k_aos_to_soa(size_t n, const float* __restrict__ p0, const float* __restrict__ p1, const float* __restrict__ p2,
                             float* __restrict__ u, float* __restrict__ v, float* __restrict__ w) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        float out[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const size_t f = 3 * i + c, piece = f / n, off = f - piece * n;
            out[c] = (piece == 0 ? p0 : (piece == 1 ? p1 : p2))[off];
        }
        u[i] = out[0];
        v[i] = out[1];
        w[i] = out[2];
    }
}
__global__ void k_snapshot(const float4* __restrict__ src, float4* __restrict__ dst, size_t n4) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n4; i += size_t(gridDim.x) * blockDim.x) dst[i] = src[i];
}

constexpr int kHostCopyBlocks = 32;  // blocks of the kernel that writes a snapshot to mapped host memory (176 GB/s alone)

void fetch_scalars(Env& e) {
    static_assert(sizeof(Scalars) % 4 == 0, "Scalars is copied as 32-bit words");
    k_fetch_sc<<<1, 32, 0, e.stream>>>(reinterpret_cast<const unsigned*>(e.sc), reinterpret_cast<unsigned*>(e.host_sc_dev),
                                       int(sizeof(Scalars) / 4));
    e.launches += 1;
    cudaStreamSynchronize(e.stream);
}

}  // namespace skt

extern "C" {

void skt_default_config(skt_solver_cfg* c) {
    if (!c) return;
    c->semantics = SKT_SEM_REFERENCE;
    c->diffuse_sweeps = 20;
    c->pcg_tol = 1e-5f;
    c->pcg_max_iter = 200;
    c->max_substeps = 100;
    c->precision = SKT_PCG_PLAIN;
    c->refine_tol = 1e-8f;
    c->inner_max_iter = 60;
    c->inner_rtol = 1e-4f;
    c->use_graph = 0;
    c->mg_half = 1;
    c->pcg_fused = 1;
}

skt_status skt_set_rate_region(skt_env* env, int enable, const int lo[3], const int hi[3]) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!enable) {
        e.rates_on = 0;
        return SKT_OK;
    }
    if (!lo || !hi) return fail(&e, SKT_INVALID_ARG, "null region bounds");
    if (!e.rates_dev) {
        if (cudaMalloc(&e.rates_dev, sizeof(double) * SKT_RATE_COUNT) != cudaSuccess) {
            cudaGetLastError();
            e.rates_dev = nullptr;
            return fail(&e, SKT_OUT_OF_MEMORY, "rate accumulator allocation failed");
        }
        cudaMemsetAsync(e.rates_dev, 0, sizeof(double) * SKT_RATE_COUNT, e.stream);
    }
    for (int k = 0; k < 3; ++k) {
        e.rate_lo[k] = lo[k];
        e.rate_hi[k] = hi[k];
    }
    e.rates_on = 1;
    return cuda_check(e, "set_rate_region");
}

skt_status skt_read_rates(skt_env* env, float* dst, size_t n) {
    if (!env || !dst) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (n != SKT_RATE_COUNT) return fail(&e, SKT_INVALID_ARG, "n must be SKT_RATE_COUNT");
    if (!e.rates_dev) return fail(&e, SKT_INVALID_ARG, "the rate region was never enabled");
    double h[SKT_RATE_COUNT];
    cudaMemcpyAsync(h, e.rates_dev, sizeof(h), cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    for (size_t k = 0; k < n; ++k) dst[k] = float(h[k]);
    return cuda_check(e, "read_rates");
}

skt_status skt_set_diagnostics(skt_env* env, int flags) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (flags & ~SKT_DIAG_BUOYANCY) return fail(&e, SKT_INVALID_ARG, "unknown diagnostics flag");
    const size_t bytes = sizeof(float) * size_t(e.g.N);
    if ((flags & SKT_DIAG_BUOYANCY) && !e.dbg_buoy) {
        if (cudaMalloc(&e.dbg_buoy, bytes) != cudaSuccess || cudaMalloc(&e.dbg_zero, bytes) != cudaSuccess) {
            cudaGetLastError();
            if (e.dbg_buoy) cudaFree(e.dbg_buoy);
            e.dbg_buoy = nullptr;
            return fail(&e, SKT_OUT_OF_MEMORY, "debug field allocation failed");
        }
        cudaMemsetAsync(e.dbg_buoy, 0, bytes, e.stream);
        cudaMemsetAsync(e.dbg_zero, 0, bytes, e.stream);
    }
    e.diag_flags = flags;
    return cuda_check(e, "set_diagnostics");
}

const char* skt_version(void) { return "skewt-gb300 0.1 (sm_103a)"; }

const char* skt_last_error(const skt_env* env) { return env ? env->e.err.c_str() : g_create_err.c_str(); }

skt_status skt_create(const skt_grid_desc* grid, const skt_solver_cfg* cfg, skt_env** out) {
    if (!grid || !out) return fail(nullptr, SKT_INVALID_ARG, "null argument");
    *out = nullptr;
    const long long n = (long long)grid->nx * grid->ny * grid->nz;
    if (grid->nx < 1 || grid->ny < 2 || grid->nz < 1 || n >= (1ll << 31) || !(grid->voxel > 0.0f))
        return fail(nullptr, SKT_INVALID_ARG, "invalid grid (need nx,nz >= 1, ny >= 2, nx*ny*nz < 2^31, voxel > 0)");
    skt_solver_cfg c;
    skt_default_config(&c);
    if (cfg) c = *cfg;
    if (c.diffuse_sweeps < 0 || c.pcg_max_iter < 0 || c.max_substeps < 1 || (c.semantics != 0 && c.semantics != 1) ||
        (c.precision != 0 && c.precision != 1))
        return fail(nullptr, SKT_INVALID_ARG, "invalid solver configuration");
    if (c.use_graph != 0 && c.use_graph != 1) return fail(nullptr, SKT_INVALID_ARG, "use_graph must be 0 or 1");
    skt_env* h = new (std::nothrow) skt_env();
    if (!h) return fail(nullptr, SKT_OUT_OF_MEMORY, "host allocation failed");
    Env& e = h->e;
    cudaGetDevice(&e.device);
    cudaDeviceGetAttribute(&e.num_sms, cudaDevAttrMultiProcessorCount, e.device);
    e.g.X = grid->nx;
    e.g.Y = grid->ny;
    e.g.Z = grid->nz;
    e.g.XY = grid->nx * grid->ny;
    e.g.N = int(n);
    e.g.vox = grid->voxel;
    e.cfg = SolverCfg{c.semantics, c.diffuse_sweeps, c.pcg_tol, c.pcg_max_iter, c.max_substeps, c.precision, c.refine_tol, c.inner_max_iter,
                      c.inner_rtol, c.use_graph, c.mg_half, c.pcg_fused};
    const size_t N = size_t(n), NG = size_t(grid->nx) * grid->nz, NY = size_t(grid->ny);
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const int nsky = 12 + 2 + 4 + 4;
    size_t bytes = al(N * 4) * nsky + al(N * 8) * 2 + al(NG * 4) * 10 + al(NG * 4) + al(NY * 4) * 6 + al(sizeof(Scalars)) +
                   al(sizeof(double) * 2 * kMaxPartials);
    if (cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking) != cudaSuccess) {
        const std::string m = std::string("stream: ") + cudaGetErrorString(cudaGetLastError());
        delete h;
        return fail(nullptr, SKT_CUDA_ERROR, m);
    }
    if (cudaMalloc(&e.pool, bytes) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(e.stream);
        delete h;
        return fail(nullptr, SKT_OUT_OF_MEMORY, "device allocation of " + std::to_string(bytes) + " bytes failed");
    }
    e.pool_bytes = bytes;
    char* p = (char*)e.pool;
    auto take = [&](size_t b) { char* r = p; p += al(b); return r; };
    float** sky[nsky] = {&e.th, &e.qv, &e.qw, &e.qc, &e.qr, &e.qs, &e.qi, &e.u, &e.v, &e.w, &e.p, &e.rho,
                         &e.tA, &e.tB, &e.r, &e.s, &e.As, &e.pp, &e.ax, &e.ay, &e.az, &e.aw};
    for (int i = 0; i < nsky; ++i) *sky[i] = (float*)take(N * 4);
    e.xd = (double*)take(N * 8);
    e.rd = (double*)take(N * 8);
    float** gr[10] = {&e.Qrs, &e.Qgr, &e.Qgs, &e.Qgi, &e.Pg, &e.tg, &e.Tg, &e.cover, &e.g2a, &e.g2b};
    for (int i = 0; i < 10; ++i) *gr[i] = (float*)take(NG * 4);
    e.gh = (int*)take(NG * 4);
    float** co[6] = {&e.isenT, &e.isenQv, &e.defU, &e.defW, &e.zeroY, &e.pcol};
    for (int i = 0; i < 6; ++i) *co[i] = (float*)take(NY * 4);
    e.sc = (Scalars*)take(sizeof(Scalars));
    e.partials = (double*)take(sizeof(double) * 2 * kMaxPartials);
    cudaMemsetAsync(e.pool, 0, bytes, e.stream);
    e.g.gh = e.gh;
    if (cudaMallocHost(&e.host_sc, sizeof(Scalars)) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&e.host_sc_dev, e.host_sc, 0) != cudaSuccess) {
        cudaGetLastError();
        if (e.host_sc) cudaFreeHost(e.host_sc);
        cudaFree(e.pool);
        cudaStreamDestroy(e.stream);
        delete h;
        return fail(nullptr, SKT_OUT_OF_MEMORY, "pinned allocation failed");
    }
    // the constructor's ground defaults (Game/environment.cu:162-168)
    const int ng = int(NG);
    k_fill<<<(ng + 255) / 256, 256, 0, e.stream>>>(e.Qrs, 0.001f, ng);
    k_fill<<<(ng + 255) / 256, 256, 0, e.stream>>>(e.Pg, 1000.0f, ng);
    k_fill<<<(ng + 255) / 256, 256, 0, e.stream>>>(e.Tg, 315.15f, ng);
    // gammas (initGammasMicroPhysics Game/microPhysics.cu:31-61, initKernelSky Game/kernelSky.cu:30-37)
    const float b = 0.8f, d = 0.25f;
    e.gam.R = tgammaf(3 + b);
    e.gam.ER = tgammaf((b + 5.0f) / 2.0f);
    e.gam.S = tgammaf(3 + d);
    e.gam.RC = tgammaf(6 + b);
    e.gam.SS = tgammaf((d + 5.0f) / 2.0f);
    e.gam.I = tgammaf(3.5f);
    e.gam.RI = tgammaf(2.75f);
    e.gam.Qr = tgammaf(4.0f + b);
    e.gam.Qs = tgammaf(4.0f + d);
    e.gam.Qi = e.gam.Qs;
    if (e.cfg.precision == 1) {
        e.cfg.semantics = SKT_SEM_TEXTBOOK;  // CG needs the symmetric operator
        if (!mg_allocate(e)) {
            g_create_err = "mixed precision needs grid sizes that halve down to <= 4096 cells (even nx, ny, nz at every level)";
            skt_destroy(h);
            return SKT_INVALID_ARG;
        }
    }
    const skt_status st = cuda_check(e, "create");
    if (st != SKT_OK) {
        g_create_err = e.err;
        skt_destroy(h);
        return st;
    }
    cudaStreamSynchronize(e.stream);
    *out = h;
    return SKT_OK;
}

void skt_destroy(skt_env* env) {
    if (!env) return;
    Env& e = env->e;
    if (e.stream) cudaStreamSynchronize(e.stream);
    if (e.ev0) cudaEventDestroy(e.ev0);
    if (e.ev1) cudaEventDestroy(e.ev1);
    if (e.pool) cudaFree(e.pool);
    if (e.mg_pool) cudaFree(e.mg_pool);
    if (e.rates_dev) cudaFree(e.rates_dev);
    if (e.dbg_buoy) cudaFree(e.dbg_buoy);
    if (e.dbg_zero) cudaFree(e.dbg_zero);
    if (e.copy_stream) cudaStreamSynchronize(e.copy_stream);
    if (e.snap) cudaFree(e.snap);
    if (e.ev_snap) cudaEventDestroy(e.ev_snap);
    if (e.ev_copy) cudaEventDestroy(e.ev_copy);
    if (e.copy_stream) cudaStreamDestroy(e.copy_stream);
    if (e.brick_flags) cudaFree(e.brick_flags);
    if (e.brick_out) cudaFree(e.brick_out);
    drop_graph(e);
    for (cudaStream_t side : e.side)
        if (side) cudaStreamDestroy(side);
    if (e.host_sc) cudaFreeHost(e.host_sc);
    if (e.stream) cudaStreamDestroy(e.stream);
    delete env;
}

skt_status skt_init(skt_env* env, const float* theta, const float* vel, const float* qv, const float* ground_T, const float* ground_p,
                    const float* p3d, const float* p_column, const int32_t* gh, uint32_t flags, uint32_t noise_seed) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!theta || !vel || !qv || !ground_T || !ground_p || !p3d || !gh) return fail(&e, SKT_INVALID_ARG, "null input array");
    // the reference keeps the pressure column for the editor's resets (m_defaultPressure)
    const size_t N = size_t(e.g.N), NG = size_t(e.g.X) * e.g.Z;
    for (size_t i = 0; i < NG; ++i)
        if (gh[i] < 0 || gh[i] >= e.g.Y - 1)
            return fail(&e, SKT_INVALID_ARG, "ground_height must lie in [0, ny-2] so every column has sky above the ground layer");
    int flat = 1;
    for (size_t i = 0; i < NG; ++i) flat &= gh[i] == 0;
    e.flat = flat;
    // AoS -> SoA (Game/environment.cu:263-281) on the device: the velocity array is copied as it
    // is, in three pieces, into scratch fields that are free before the first step
    float* piece[3] = {e.tA, e.tB, e.As};
    for (int j = 0; j < 3; ++j) cudaMemcpyAsync(piece[j], vel + size_t(j) * N, N * 4, cudaMemcpyHostToDevice, e.stream);
    k_aos_to_soa<<<int(std::min<size_t>((N + 255) / 256, size_t(e.num_sms) * 16)), 256, 0, e.stream>>>(N, piece[0], piece[1], piece[2],
                                                                                                    e.u, e.v, e.w);
    e.launches += 1;
    cudaMemcpyAsync(e.th, theta, N * 4, cudaMemcpyHostToDevice, e.stream);
    cudaMemcpyAsync(e.qv, qv, N * 4, cudaMemcpyHostToDevice, e.stream);
    cudaMemcpyAsync(e.Tg, ground_T, NG * 4, cudaMemcpyHostToDevice, e.stream);
    cudaMemcpyAsync(e.Pg, ground_p, NG * 4, cudaMemcpyHostToDevice, e.stream);
    cudaMemcpyAsync(e.p, p3d, N * 4, cudaMemcpyHostToDevice, e.stream);
    cudaMemcpyAsync(e.gh, gh, NG * 4, cudaMemcpyHostToDevice, e.stream);
    if (p_column) cudaMemcpyAsync(e.pcol, p_column, size_t(e.g.Y) * 4, cudaMemcpyHostToDevice, e.stream);
    else cudaMemsetAsync(e.pcol, 0, size_t(e.g.Y) * 4, e.stream);
    e.ground_changed = 0;  // the init does the first editorDataGPU pass itself
    launch_init_state(e, (flags & SKT_INIT_NOISE) ? 1 : 0, noise_seed);
    cudaStreamSynchronize(e.stream);
    const skt_status st = cuda_check(e, "init");
    if (st == SKT_OK) e.initialized = true;
    return st;
}

skt_status skt_step(skt_env* env, float dt, float speed, int nsteps) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!e.initialized) return fail(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    if (!(dt > 0.0f) || !(speed > 0.0f) || nsteps < 0) return fail(&e, SKT_INVALID_ARG, "dt and speed must be > 0, nsteps >= 0");
    if (e.async_steps > 0 && !(e.cfg.use_graph && !e.prof && nsteps > 0)) {
        // stream-ordered steps after graph steps queued by skt_step_async: collect those first
        const skt_status ps = collect_async(e);
        if (ps != SKT_OK && ps != SKT_NOT_CONVERGED) return ps;
    }
    if (e.cfg.use_graph && !e.prof && nsteps > 0) {
        // graph mode: the status is read once after the nsteps launches
        const skt_status gs = step_graph(e, dt, speed, nsteps);
        if (gs != SKT_OK) return gs;
        return graph_status(e);
    }
    skt_status worst = SKT_OK;
    if (!e.ev0) { cudaEventCreate(&e.ev0); cudaEventCreate(&e.ev1); }
    cudaEventRecord(e.ev0, e.stream);
    int done = 0;
    for (int i = 0; i < nsteps; ++i) {
        const skt_status st = run_step(e, dt, speed);
        if (st != SKT_OK) return st;
        ++done;
        e.ground_changed = 0;  // Game/environment.cu:554
        if (!e.last_converged) worst = SKT_NOT_CONVERGED;
        // the step's own scalar reads (Courant counts, solver stop tests) already brought the
        // device status to the host: a step that met a NaN or Inf ends the call
        if (e.host_sc->status != 0) break;
    }
    cudaEventRecord(e.ev1, e.stream);
    cudaEventSynchronize(e.ev1);
    cudaEventElapsedTime(&e.last_gpu_ms, e.ev0, e.ev1);
    const skt_status st = cuda_check(e, "step");
    if (st != SKT_OK) return st;
    fetch_scalars(e);
    const int dev_status = e.host_sc->status;
    if (dev_status != 0) {
        cudaMemsetAsync(&e.sc->status, 0, sizeof(int), e.stream);
        cudaStreamSynchronize(e.stream);
        e.host_sc->status = 0;
        return fail(&e, skt_status(dev_status),
                    dev_status == SKT_TIMEOUT
                        ? "step " + std::to_string(done) + " of this call: a kernel's wait for its streamed data ran out (the state is not valid)"
                        : "step " + std::to_string(done) + " of this call met a NaN or Inf (in the wind or in a pressure-solver "
                          "reduction: a non-finite field value or a zero-density cell); the remaining steps were not run and "
                          "the state is not valid");
    }
    return worst;
}

}  // extern "C"

// An ensemble captured as one CUDA graph: every member's whole step is an independent branch of
// the graph (forked from and joined to the ensemble's stream), so one graph launch advances all
// members and the GPU runs their kernels side by side; no host thread per member and no host
// synchronisation inside a step.
struct skt_ensemble {
    std::vector<skt_env*> members;
    std::vector<GraphBook> books;
    std::vector<Env::GraphKey> keys;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> joins;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    float last_ms = 0.0f;
};

namespace {
void drop_ensemble_graph(skt_ensemble* s) {
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->exec = nullptr;
    s->graph = nullptr;
}

skt_status capture_ensemble(skt_ensemble* s, const std::vector<float>& dts, const std::vector<float>& sps) {
    drop_ensemble_graph(s);
    const int n = int(s->members.size());
    for (int i = 0; i < n; ++i) {
        Env& e = s->members[i]->e;
        if (ensure_side_streams(e) != SKT_OK) return fail(nullptr, SKT_CUDA_ERROR, "ensemble: member " + std::to_string(i) + ": " + e.err);
        e.graph_fail = false;
        e.graph_err.clear();
    }
    if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess || cudaEventRecord(s->fork, s->stream) != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, SKT_CUDA_ERROR, "ensemble: capture could not begin");
    }
    for (int i = 0; i < n; ++i) {
        Env& e = s->members[i]->e;
        cudaStreamWaitEvent(e.stream, s->fork, 0);
        capture_into(e, dts[i], sps[i], s->books[i]);
        cudaEventRecord(s->joins[i], e.stream);
        cudaStreamWaitEvent(s->stream, s->joins[i], 0);
        s->keys[i] = graph_key(e, dts[i], sps[i]);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(s->stream, &graph);
    s->graph = graph;
    std::string err;
    for (int i = 0; i < n && err.empty(); ++i)
        if (s->members[i]->e.graph_fail) err = "ensemble: member " + std::to_string(i) + ": " + s->members[i]->e.graph_err;
    if (err.empty() && end != cudaSuccess) err = std::string("ensemble: capture: ") + cudaGetErrorString(end);
    if (err.empty() && cudaGraphInstantiate(&s->exec, graph, 0) != cudaSuccess) err = "ensemble: graph instantiation failed";
    if (!err.empty()) {
        cudaGetLastError();
        drop_ensemble_graph(s);
        return fail(nullptr, SKT_CUDA_ERROR, err);
    }
    for (int i = 0; i < n; ++i) read_trips(s->members[i]->e);
    return SKT_OK;
}
}  // namespace

extern "C" {

skt_status skt_ensemble_create(skt_env* const* envs, int n, skt_ensemble** out) {
    if (!envs || n < 1 || !out) return fail(nullptr, SKT_INVALID_ARG, "invalid ensemble arguments");
    *out = nullptr;
    int device = -1;
    for (int i = 0; i < n; ++i) {
        if (!envs[i]) return fail(nullptr, SKT_INVALID_ARG, "null member");
        for (int j = 0; j < i; ++j)
            if (envs[j] == envs[i]) return fail(nullptr, SKT_INVALID_ARG, "a member appears twice");
        if (device >= 0 && envs[i]->e.device != device) return fail(nullptr, SKT_INVALID_ARG, "members on different devices");
        device = envs[i]->e.device;
    }
    skt_ensemble* s = new (std::nothrow) skt_ensemble();
    if (!s) return fail(nullptr, SKT_OUT_OF_MEMORY, "host allocation failed");
    s->members.assign(envs, envs + n);
    // the members run side by side: each member's per-cell kernels are sized for twice its share of
    // the SMs in proportion to its cells (at least one SM), instead of for the whole GPU. Measured on
    // 48 members of four sizes (69M cells): 130 ms per ensemble step sized for the whole GPU, 110 ms
    // at the share, 101 ms at twice it, 103 ms at four times it.
    double total = 0.0;
    for (int i = 0; i < n; ++i) total += double(envs[i]->e.g.N);
    for (int i = 0; i < n; ++i) {
        Env& e = envs[i]->e;
        e.stencil_sms = std::min(e.num_sms, std::max(1, int(std::lround(2.0 * e.num_sms * double(e.g.N) / total))));
    }
    s->books.resize(n);
    s->keys.resize(n);
    s->joins.resize(n, nullptr);
    bool ok = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming) == cudaSuccess && cudaEventCreate(&s->ev0) == cudaSuccess &&
              cudaEventCreate(&s->ev1) == cudaSuccess;
    for (int i = 0; ok && i < n; ++i) ok = cudaEventCreateWithFlags(&s->joins[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        skt_ensemble_destroy(s);
        return fail(nullptr, SKT_CUDA_ERROR, "ensemble: stream or event creation failed");
    }
    *out = s;
    return SKT_OK;
}

void skt_ensemble_destroy(skt_ensemble* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (skt_env* m : s->members) m->e.stencil_sms = 0;  // stepped alone again: the whole GPU
    drop_ensemble_graph(s);
    for (cudaEvent_t ev : s->joins)
        if (ev) cudaEventDestroy(ev);
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

skt_status skt_ensemble_step(skt_ensemble* s, const float* dt, float dt0, const float* speed, int nsteps, int* statuses) {
    if (!s || nsteps < 0) return fail(nullptr, SKT_INVALID_ARG, "invalid ensemble step arguments");
    const int n = int(s->members.size());
    std::vector<float> dts(n), sps(n);
    for (int i = 0; i < n; ++i) {
        Env& e = s->members[i]->e;
        if (!e.initialized) return fail(nullptr, SKT_NOT_INITIALIZED, "member " + std::to_string(i) + ": skt_init has not run");
        dts[i] = dt ? dt[i] : dt0;
        sps[i] = speed ? speed[i] : 1.0f;
        if (!(dts[i] > 0.0f) || !(sps[i] > 0.0f)) return fail(nullptr, SKT_INVALID_ARG, "dt and speed must be > 0");
    }
    if (nsteps == 0) return SKT_OK;
    bool stale = !s->exec;
    for (int i = 0; i < n && !stale; ++i) stale = !same_key(s->keys[i], graph_key(s->members[i]->e, dts[i], sps[i]));
    if (stale) {
        const skt_status st = capture_ensemble(s, dts, sps);
        if (st != SKT_OK) return st;
    }
    cudaEventRecord(s->ev0, s->stream);
    for (int k = 0; k < nsteps; ++k) {
        for (int i = 0; i < n; ++i) {
            const skt_status ps = prepare_launch(s->members[i]->e, s->exec, s->books[i], s->stream);
            if (ps != SKT_OK) return fail(nullptr, ps, "member " + std::to_string(i) + ": " + s->members[i]->e.err);
        }
        if (cudaGraphLaunch(s->exec, s->stream) != cudaSuccess) {
            const std::string m = cudaGetErrorString(cudaGetLastError());
            return fail(nullptr, SKT_CUDA_ERROR, "ensemble: graph launch: " + m);
        }
        for (int i = 0; i < n; ++i) advance_clock(s->members[i]->e, dts[i], sps[i]);
    }
    cudaEventRecord(s->ev1, s->stream);
    cudaEventSynchronize(s->ev1);
    cudaEventElapsedTime(&s->last_ms, s->ev0, s->ev1);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(nullptr, SKT_CUDA_ERROR, std::string("ensemble step: ") + cudaGetErrorString(err));
    skt_status first = SKT_OK;
    for (int i = 0; i < n; ++i) {
        Env& e = s->members[i]->e;
        finish_graph_steps(e, s->books[i], nsteps);
        e.last_gpu_ms = s->last_ms;
        const skt_status st = graph_status(e);
        if (statuses) statuses[i] = st;
        if (st != SKT_OK && st != SKT_NOT_CONVERGED && first == SKT_OK) {
            first = st;
            fail(nullptr, st, "member " + std::to_string(i) + ": " + e.err);
        }
    }
    return first;
}

skt_status skt_step_ensemble(skt_env* const* envs, int n, const float* dt, float dt0, const float* speed, int nsteps,
                             int threads, int* statuses) {
    if (!envs || n < 0 || nsteps < 0) return fail(nullptr, SKT_INVALID_ARG, "invalid ensemble arguments");
    for (int i = 0; i < n; ++i)
        if (!envs[i]) return fail(nullptr, SKT_INVALID_ARG, "null member");
    if (n == 0) return SKT_OK;
    int device = 0;
    cudaGetDevice(&device);
    const int nt = std::min(n, threads > 0 ? threads : std::min(n, 64));
    std::vector<int> st(n, SKT_OK);
    std::atomic<int> next(0);
    auto work = [&]() {
        cudaSetDevice(device);  // the calling thread's device, for every worker
        for (int i = next++; i < n; i = next++)
            st[i] = skt_step(envs[i], dt ? dt[i] : dt0, speed ? speed[i] : 1.0f, nsteps);
    };
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    skt_status first = SKT_OK;
    for (int i = 0; i < n; ++i) {
        if (statuses) statuses[i] = st[i];
        if (first == SKT_OK && st[i] != SKT_OK && st[i] != SKT_NOT_CONVERGED) first = skt_status(st[i]);
    }
    if (first != SKT_OK) {
        for (int i = 0; i < n; ++i)
            if (st[i] == first) { g_create_err = "member " + std::to_string(i) + ": " + envs[i]->e.err; break; }
    }
    return first;
}

skt_status skt_sync(skt_env* env) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    if (env->e.async_steps > 0) return collect_async(env->e);
    cudaStreamSynchronize(env->e.stream);
    return cuda_check(env->e, "sync");
}

skt_status skt_step_async(skt_env* env, float dt, float speed, int nsteps) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!e.initialized) return fail(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    if (!(dt > 0.0f) || !(speed > 0.0f) || nsteps < 0) return fail(&e, SKT_INVALID_ARG, "dt and speed must be > 0, nsteps >= 0");
    if (!e.cfg.use_graph || e.prof) return skt_step(env, dt, speed, nsteps);  // stream-ordered steps read their loop counts on the host
    if (nsteps == 0) return SKT_OK;
    return launch_graph_steps(e, dt, speed, nsteps);
}

skt_status skt_read_field(skt_env* env, int param, int dir, float* dst, size_t n) {
    if (!env || !dst) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    float* src = sky_ptr(e, param, dir);
    if (!src && (param == SKT_DEBUG1 || param == SKT_DEBUG2))
        return fail(&e, SKT_INVALID_ARG, "debug fields need skt_set_diagnostics(env, SKT_DIAG_BUOYANCY) first");
    if (!src) return fail(&e, SKT_INVALID_ARG, "unknown field selector");
    if (n != size_t(e.g.N)) return fail(&e, SKT_INVALID_ARG, "size mismatch");
    cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    return cuda_check(e, "read_field");
}

skt_status skt_read_fields_async(skt_env* env, int nfields, const int* params, const int* dirs, float* const* dst, size_t n) {
    if (!env || nfields < 0 || (nfields > 0 && (!params || !dst))) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (n != size_t(e.g.N)) return fail(&e, SKT_INVALID_ARG, "size mismatch");
    std::vector<float*> src(nfields);
    for (int i = 0; i < nfields; ++i) {
        src[i] = sky_ptr(e, params[i], dirs ? dirs[i] : 0);
        if (!src[i] || !dst[i]) return fail(&e, SKT_INVALID_ARG, "unknown field selector or null destination");
    }
    if (!e.copy_stream) {
        if (cudaStreamCreateWithFlags(&e.copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&e.ev_snap, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&e.ev_copy, cudaEventDisableTiming) != cudaSuccess)
            return cuda_check(e, "read_fields_async");
    }
    if (e.snap_fields < size_t(nfields)) {
        if (e.copy_pending) cudaEventSynchronize(e.ev_copy);
        if (e.snap) cudaFree(e.snap);
        e.snap = nullptr;
        e.snap_fields = 0;
        if (cudaMalloc(&e.snap, sizeof(float) * n * size_t(nfields)) != cudaSuccess) {
            cudaGetLastError();
            return fail(&e, SKT_OUT_OF_MEMORY, "snapshot allocation failed");
        }
        e.snap_fields = size_t(nfields);
        e.copy_pending = false;
    }
    // the snapshot waits for the copies of the previous one, then follows the queued work
    if (e.copy_pending) cudaStreamWaitEvent(e.stream, e.ev_copy, 0);
    // the snapshot is an SM copy (a kernel on the step's stream), so it never waits for a copy engine
    for (int i = 0; i < nfields; ++i) {
        float* d = e.snap + size_t(i) * n;
        if (n % 4 == 0) {
            const size_t n4 = n / 4;
            const int blocks = int(std::min<size_t>((n4 + 255) / 256, size_t(e.num_sms) * 8));
            k_snapshot<<<blocks, 256, 0, e.stream>>>(reinterpret_cast<const float4*>(src[i]), reinterpret_cast<float4*>(d), n4);
        } else {
            cudaMemcpyAsync(d, src[i], sizeof(float) * n, cudaMemcpyDeviceToDevice, e.stream);
        }
    }
    // a failed snapshot launch is reported here, before the attribute queries below clear errors
    {
        const skt_status snap_st = cuda_check(e, "read_fields_async (snapshot)");
        if (snap_st != SKT_OK) return snap_st;
    }
    cudaEventRecord(e.ev_snap, e.stream);
    cudaStreamWaitEvent(e.copy_stream, e.ev_snap, 0);
    // Stream-ordered steps read small scalars back through the copy engine and would queue behind
    // bulk copies there: for them, pinned destinations are written by a narrow kernel through
    // their mapped addresses (it takes a few SMs beside the next step's kernels). Graph steps read
    // nothing back until the call ends, so the copy engine takes every field and leaves the SMs to
    // the step (measured at 512x512x256: a step beside the readback 163.7 ms with the copy engine,
    // 166.5 ms with the writer kernel, 162.7 ms alone). Pageable destinations: the copy engine.
    const bool writer_kernel = !e.cfg.use_graph || e.prof;
    for (int i = 0; i < nfields; ++i) {
        const float* s = e.snap + size_t(i) * n;
        cudaPointerAttributes at{};
        const bool known = writer_kernel && cudaPointerGetAttributes(&at, dst[i]) == cudaSuccess;
        if (writer_kernel && !known) cudaGetLastError();  // an unregistered host pointer: clear only the query's own error
        const bool mapped = known && at.type == cudaMemoryTypeHost && at.devicePointer &&
                            (reinterpret_cast<uintptr_t>(at.devicePointer) % 16) == 0 && n % 4 == 0;
        if (mapped) {
            k_snapshot<<<kHostCopyBlocks, 256, 0, e.copy_stream>>>(reinterpret_cast<const float4*>(s), static_cast<float4*>(at.devicePointer), n / 4);
            e.launches += 1;
        } else {
            cudaMemcpyAsync(dst[i], s, sizeof(float) * n, cudaMemcpyDeviceToHost, e.copy_stream);
        }
    }
    cudaEventRecord(e.ev_copy, e.copy_stream);
    e.copy_pending = true;
    return cuda_check(e, "read_fields_async");
}

skt_status skt_read_wait(skt_env* env) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (e.copy_pending) {
        cudaEventSynchronize(e.ev_copy);
        e.copy_pending = false;
    }
    return cuda_check(e, "read_wait");
}

skt_status skt_write_field(skt_env* env, int param, int dir, const float* src, size_t n) {
    if (!env || !src) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    float* dst = sky_ptr(e, param, dir);
    if (!dst) return fail(&e, SKT_INVALID_ARG, "unknown field selector");
    if (n != size_t(e.g.N)) return fail(&e, SKT_INVALID_ARG, "size mismatch");
    cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyHostToDevice, e.stream);
    cudaStreamSynchronize(e.stream);
    return cuda_check(e, "write_field");
}

skt_status skt_field_device_ptr(skt_env* env, int param, int dir, float** out) {
    if (!env || !out) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    float* p = sky_ptr(env->e, param, dir);
    if (!p) return fail(&env->e, SKT_INVALID_ARG, "unknown field selector");
    *out = p;
    return SKT_OK;
}

skt_status skt_read_ground(skt_env* env, int which, float* dst, size_t n) {
    if (!env || !dst) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    float* src = ground_ptr(e, which);
    if (!src || n != size_t(e.g.X) * e.g.Z) return fail(&e, SKT_INVALID_ARG, "bad ground selector or size");
    cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    return cuda_check(e, "read_ground");
}

skt_status skt_write_ground(skt_env* env, int which, const float* src, size_t n) {
    if (!env || !src) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    float* dst = ground_ptr(e, which);
    if (!dst || n != size_t(e.g.X) * e.g.Z) return fail(&e, SKT_INVALID_ARG, "bad ground selector or size");
    cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyHostToDevice, e.stream);
    cudaStreamSynchronize(e.stream);
    return cuda_check(e, "write_ground");
}

skt_status skt_read_column(skt_env* env, int which, float* dst, size_t n) {
    if (!env || !dst) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    float* src = column_ptr(e, which);
    if (!src || n != size_t(e.g.Y)) return fail(&e, SKT_INVALID_ARG, "bad column selector or size");
    cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    return cuda_check(e, "read_column");
}

skt_status skt_write_column(skt_env* env, int which, const float* src, size_t n) {
    if (!env || !src) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    float* dst = column_ptr(e, which);
    if (!dst || n != size_t(e.g.Y)) return fail(&e, SKT_INVALID_ARG, "bad column selector or size");
    cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyHostToDevice, e.stream);
    cudaStreamSynchronize(e.stream);
    return cuda_check(e, "write_column");
}

skt_status skt_set_clock(skt_env* env, double sim_time, int day, float longitude, float sun, int pause) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    e.sim_time = float(sim_time);
    e.day = day;
    e.longitude = longitude;
    e.sun = sun;
    e.pause = pause;
    return SKT_OK;
}

skt_status skt_stats(skt_env* env, skt_step_stats* out) {
    if (!env || !out) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    out->pcg_iters = e.last_iters;
    out->pcg_residual = e.last_residual;
    out->pcg_converged = e.last_converged;
    for (int i = 0; i < 10; ++i) out->nsub[i] = e.last_nsub[i];
    out->outer_iters = e.last_outer;
    out->sim_time = e.sim_time;
    out->kernel_launches = e.launches;
    out->gpu_ms = e.last_gpu_ms;
    return SKT_OK;
}

skt_status skt_profile_enable(skt_env* env, int on) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    env->e.prof = on != 0;
    return SKT_OK;
}

skt_status skt_profile_read(skt_env* env, char* buf, size_t n) {
    if (!env || !buf || n == 0) return fail(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    cudaStreamSynchronize(e.stream);
    struct Acc { std::string name; double ms; long long nk; int scopes; };
    std::vector<Acc> acc;
    for (auto& r : e.recs) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
        size_t i = 0;
        for (; i < acc.size(); ++i)
            if (acc[i].name == r.name) break;
        if (i == acc.size()) acc.push_back({r.name, 0.0, 0, 0});
        acc[i].ms += ms;
        acc[i].nk += r.nk;
        acc[i].scopes += 1;
    }
    e.recs.clear();
    std::string js = "{";
    for (size_t i = 0; i < acc.size(); ++i) {
        char tmp[256];
        snprintf(tmp, sizeof tmp, "%s\"%s\": [%.6f, %lld, %d]", i ? ", " : "", acc[i].name.c_str(), acc[i].ms, acc[i].nk, acc[i].scopes);
        js += tmp;
    }
    js += "}";
    if (js.size() + 1 > n) return fail(&e, SKT_INVALID_ARG, "buffer too small");
    memcpy(buf, js.c_str(), js.size() + 1);
    return cuda_check(e, "profile_read");
}

skt_status skt_run_stage(skt_env* env, int stage, int arg, float dt, float speed, skt_step_stats* out) {
    if (!env) return fail(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!e.initialized) return fail(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    switch (stage) {
        case 0: {
            float* f[6] = {e.th, e.qv, e.u, e.v, e.w, e.qw};
            if (arg < 0 || arg > 5) return fail(&e, SKT_INVALID_ARG, "diffuse type");
            launch_diffuse(e, f[arg], arg, dt);
            break;
        }
        case 1: {
            if (arg < 0 || arg > 5) return fail(&e, SKT_INVALID_ARG, "advect field");
            float* f[6] = {e.th, e.u, e.v, e.w, e.qv, e.qw};
            const float* df[6] = {e.isenT, e.defU, e.zeroY, e.defW, e.isenQv, e.zeroY};
            const int sd[6] = {CUSTOM, CUSTOM, DIRICHLET, CUSTOM, CUSTOM, DIRICHLET};
            const int gd[6] = {CUSTOM, DIRICHLET, DIRICHLET, DIRICHLET, CUSTOM, DIRICHLET};
            e.last_nsub[0] = launch_advect(e, f[arg], df[arg], sd[arg], gd[arg], dt, 0, true);
            break;
        }
        case 2: launch_buoyancy(e, dt); break;
        case 3: launch_init_density(e); launch_project(e, dt); break;
        case 4: launch_micro(e, dt, speed); break;
        case 5: {
            if (arg < 0 || arg > 2) return fail(&e, SKT_INVALID_ARG, "precip type");
            float* f[3] = {e.qr, e.qs, e.qi};
            launch_precip(e, f[arg], arg, dt);
            break;
        }
        case 6: launch_ground(e, dt, speed, irradiance(e.sim_time, e.day, e.longitude, e.sun)); break;
        case 8: launch_init_density(e); break;
        case 9: launch_new_pressure(e); break;
        default: return fail(&e, SKT_INVALID_ARG, "unknown stage");
    }
    cudaStreamSynchronize(e.stream);
    const skt_status st = cuda_check(e, "stage");
    if (out) skt_stats(env, out);
    if (st != SKT_OK) return st;
    fetch_scalars(e);
    if (e.host_sc->status != 0) {  // as skt_step: a NaN or Inf met by the wind maximum or a solver reduction
        const int dev_status = e.host_sc->status;
        cudaMemsetAsync(&e.sc->status, 0, sizeof(int), e.stream);
        cudaStreamSynchronize(e.stream);
        e.host_sc->status = 0;
        return fail(&e, skt_status(dev_status), "the stage met a NaN or Inf (wind maximum or pressure-solver reduction)");
    }
    return st;
}

}  // extern "C"
