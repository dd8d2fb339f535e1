// Internal declarations shared by the CUDA translation units of libskewt_gb300.
//
// Data layout in HBM: structure-of-arrays FP32 fields of X*Y*Z cells, idx = x + y*X + z*X*Y
// with y vertical (the reference's layout, Game/utils.cuh:8-11); 2D ground arrays of X*Z
// cells, idxG = x + z*X; per-level columns of Y values. A cell is ground when
// y <= gh[x + z*X] (Game/kernelSky.cu:1709-1712). All fields live in one allocation carved into
// 256-byte aligned slices.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <functional>
#include <vector>

#include "skt_physics.cuh"
#include "../../include/skewt.h"

namespace skt {

enum BC : int { NEUMANN = 0, DIRICHLET = 1, CUSTOM = 2 };

struct Grid {
    int X, Y, Z;  // Y vertical
    int XY;       // X*Y
    int N;        // X*Y*Z (< 2^31)
    const int* __restrict__ gh;
    float vox;
};

__device__ __forceinline__ int cidx(const Grid& g, int x, int y, int z) { return x + y * g.X + z * g.XY; }
__device__ __forceinline__ bool is_ground(const Grid& g, int x, int y, int z) { return y <= __ldg(g.gh + x + z * g.X); }
__device__ __forceinline__ bool in_dom(const Grid& g, int x, int y, int z) {
    return (unsigned)x < (unsigned)g.X && (unsigned)y < (unsigned)g.Y && (unsigned)z < (unsigned)g.Z;
}
__device__ __forceinline__ float bc_val(int bc, float own, float custom) {
    return bc == NEUMANN ? own : (bc == DIRICHLET ? 0.0f : custom);
}

// Value of field q seen by a sky-cell stencil at (x,y,z), which may be outside the domain or a
// ground cell. Outside: the condition of the nearest in-domain cell ("ground" if that cell is
// ground, else "sides"; the top boundary also uses "sides") with that cell's value and the
// default column at its height. In-domain ground: the "ground" condition with the default at
// that height. This one rule restates the reference's Neigh records plus fillNeighbourData,
// fillSharedNeigh and getValueExtra* (Game/kernelSky.cu:1765-2042).
__device__ __forceinline__ float ghost(const Grid& g, const float* __restrict__ q, int x, int y, int z, int sides, int ground,
                                       const float* __restrict__ def) {
    if (!in_dom(g, x, y, z)) {
        const int xc = min(max(x, 0), g.X - 1), yc = min(max(y, 0), g.Y - 1), zc = min(max(z, 0), g.Z - 1);
        const int bc = is_ground(g, xc, yc, zc) ? ground : sides;
        return bc_val(bc, q[cidx(g, xc, yc, zc)], def ? def[yc] : 0.0f);
    }
    if (is_ground(g, x, y, z)) return bc_val(ground, q[cidx(g, x, y, z)], def ? def[y] : 0.0f);
    return q[cidx(g, x, y, z)];
}

// Face value through fillNeighbourData with an explicit custom value (the velocity of the
// face behind a cell and the boundary densities/pressures of the projection).
__device__ __forceinline__ float face_nb(const Grid& g, const float* __restrict__ q, int x, int y, int z, int dx, int dy, int dz,
                                         int sides, int ground, float custom) {
    const int xn = x + dx, yn = y + dy, zn = z + dz;
    const float own = q[cidx(g, x, y, z)];
    if (!in_dom(g, xn, yn, zn)) return bc_val(sides, own, custom);
    if (is_ground(g, xn, yn, zn)) return bc_val(ground, own, custom);
    return q[cidx(g, xn, yn, zn)];
}

constexpr int kMaxGraphLoops = 16;  // conditional loops of one captured step

// Device-resident scalars of the solver (one per environment).
struct Scalars {
    double sigma0, sigma1, beta;      // PCG scalars (FP64)
    float alpha, beta_f;              // the FP32 step lengths applied to the vectors
    float alpha_pp;                   // plain PCG: the step length of the pressure update still to apply
    unsigned int maxbits;             // float bits of a max-reduction (atomicMax on uint)
    int converged;                    // PCG stop flag
    int iters;                        // PCG iterations done
    float residual;                   // last max residual
    unsigned int done_blocks;         // last-block reduction ticket
    unsigned int done_blocks2;
    int nsub;                         // Courant substeps of the current advection
    int status;                       // 0 ok, otherwise an skt_status
    double rnorm0;                    // mixed mode: initial residual norm
    double rnorm;                     // mixed mode: current residual norm
    int outer;                        // mixed mode: refinement steps
    float inner_tol;                  // mixed mode: max residual at the start of the inner solve
    int outer_inner_total;            // mixed mode: inner iterations summed over the refinement
    int refine_done;                  // mixed mode: relative FP64 residual met refine_tol
    int edit_changed;                 // an edit changed the ground store
    // graph mode (the step captured as a CUDA graph, conditional nodes for the loops)
    float irr;                        // the step's irradiance, set by the graph's first node
    int slot;                         // advection: substeps done in the current field's loop
    int nsub_f[10];                   // advection: substep count of each field in the last step
    unsigned int trips[kMaxGraphLoops];  // completed trips of each captured loop body (cumulative)
};

// A non-finite total of a solver reduction (a dot product or squared norm over every sky cell)
// means a NaN or Inf reached the projection: a non-finite field value or a zero density. The
// reduction's last block records it for skt_step, which stops stepping and reports
// SKT_NAN_DETECTED; the solver loops stop at their next host check. The reference traps only on
// CUDA errors (Game/environment.cu:394-403) and would carry the NaNs on.
__device__ __forceinline__ void note_nonfinite(Scalars* sc, double tot) {
    if (!isfinite(tot)) sc->status = SKT_NAN_DETECTED;
}
// the same test on one float (the wind maximum's inputs)
__device__ __forceinline__ bool nonfinite(float v) { return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u; }

// one coarse level of the multigrid preconditioner (A-form coefficients and work vectors)
struct MgLevel {
    int X = 0, Y = 0, Z = 0;
    float *ax = nullptr, *ay = nullptr, *az = nullptr, *aw = nullptr, *x = nullptr, *x2 = nullptr, *b = nullptr;
};
constexpr int kMaxMgLevels = 12;

constexpr int kMaxPartials = 4096;

// Kernel-level configuration (from skt_solver_cfg)
struct SolverCfg {
    int semantics;       // 0 reference, 1 textbook
    int diffuse_sweeps;
    float pcg_tol;
    int pcg_max_iter;
    int max_substeps;
    int precision;       // 0 plain, 1 mixed
    float refine_tol;
    int inner_max_iter;
    float inner_rtol;
    int use_graph;
    int mg_half;         // mixed: FP16 finest-level coefficients in the V-cycle
    int pcg_fused;       // plain: search step and pressure update fused into the operator
};

// Launch shapes of the kernels whose best shape depends on the grid and the GPU, chosen by
// skt_autotune (skt_tune.cu) and otherwise these defaults (hand-measured at 512x256x512).
struct Tuning {
    int diffuse_depth = 1;   // sweeps per diffusion pass: 1, or 2 (temporal blocking, k_diffuse2)
    int diffuse_h = 8;       // two-sweep kernel: k_diffuse_pair4 rows per block (6, 14), k_diffuse2 rows per warp (4, 8)
    int diffuse_bps = 32;    // k_diffuse4: blocks per SM in the grid (z-run length)
    int diffuse2_bps = 8;    // k_diffuse2: blocks per SM in the grid (z-run length)
    int ppm_bps = 16;        // k_ppm4x: blocks per SM (z-run length)
    int ppmz_bps = 8;        // k_ppm4z: blocks per SM (z-run length)
    int ppmy_bps = 32;       // k_ppm4y: blocks per SM (y-run length)
};

// What a captured step needs at launch and afterwards: the irradiance node to update, and the
// kernel counts (outside the loops, and per trip of each loop) to count the launches from the
// device's trip counters.
struct GraphBook {
    cudaGraphNode_t irr_node = nullptr;
    long long statics = 0;
    int loops = 0;
    long long body[kMaxGraphLoops] = {0};
};

struct Env {
    Grid g{};
    SolverCfg cfg{};
    Tuning tune{};
    int device = 0;
    cudaStream_t stream = nullptr;
    void* pool = nullptr;
    size_t pool_bytes = 0;
    // sky fields
    float *th, *qv, *qw, *qc, *qr, *qs, *qi, *u, *v, *w, *p, *rho;
    // scratch sky fields
    float *tA, *tB;               // ping-pong for diffusion/advection
    float *r, *s, *As, *pp;       // PCG vectors
    float *ax, *ay, *az, *aw;     // Poisson coefficients (+x, +y, +z faces, diagonal)
    double *xd, *rd;              // mixed mode FP64 solution and residual
    // ground (X*Z)
    float *Qrs, *Qgr, *Qgs, *Qgi, *Pg, *tg, *Tg, *cover, *g2a, *g2b;
    int* gh;
    // columns (Y)
    float *isenT, *isenQv, *defU, *defW, *zeroY;
    float* pcol = nullptr;        // the init's pressure column (the editor's pressure reset)
    int ground_changed = 0;       // the ground changed since the last step (m_groundChanged)
    int adv_nsub = -1;            // Courant substeps of the last advection's wind (host copy; 0 = on the device only)
    // reductions
    Scalars* sc;
    double* partials;
    Scalars* host_sc = nullptr;      // pinned mirror, written by fetch_scalars
    Scalars* host_sc_dev = nullptr;  // the mirror's device-side address (mapped pinned memory)
    // host clock (environmentGPU::m_time etc.)
    float sim_time = 43200.0f;
    int day = 130;
    float longitude = 52.37f;
    float sun = 1.0f;
    int pause = 0;
    bool initialized = false;
    Gammas gam{};
    // last-step diagnostics
    int last_iters = 0;
    float last_residual = 0.0f;
    int last_converged = 1;
    int last_nsub[10] = {0};
    int last_outer = 0;
    int num_sms = 148;
    // SMs the grids of the per-cell kernels are sized for (0: all of them). An ensemble gives each
    // member a share in proportion to its cells, since the members run side by side. Only kernels
    // whose results do not depend on their grid use it; the reductions keep num_sms, so a member's
    // bits are the same inside an ensemble and alone.
    int stencil_sms = 0;
    std::string err;
    int flat = 1;  // all gh == 0
    // graph mode: the step captured once per key, the loops as conditional WHILE nodes
    bool capturing = false;              // launches go into a stream capture (no host reads)
    cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr};  // capture streams of nested loop bodies
    int graph_depth = 0;
    cudaGraphExec_t graph_exec = nullptr;
    cudaGraph_t graph = nullptr;
    float* irr_dev = nullptr;            // the irradiance the ground kernel reads in graph mode
    struct GraphKey {
        float dt, speed;
        int flat, rates_on, rate_lo[3], rate_hi[3], diag_flags, stencil_sms;
        Tuning tune;
    } gkey{};
    GraphBook book;                      // the bookkeeping of the environment's own captured step
    int graph_loops = 0;                 // capture in progress: loops captured so far
    long long loop_body[kMaxGraphLoops] = {0};  // capture in progress: kernels of one trip of each loop body
    unsigned int trips_seen[kMaxGraphLoops] = {0};
    long long body_acc = 0;              // capture bookkeeping: kernels inside loop bodies at the current level
    bool graph_fail = false;             // a capture call failed
    std::string graph_err;
    // graph
    // multigrid hierarchy of the mixed-precision solve (level 0 = the grid itself)
    int mg_levels = 0;
    void* mg_pool = nullptr;
    MgLevel mg[kMaxMgLevels];
    void* mg_h = nullptr;         // FP16 ax, ay, az, aw of the finest level (4 x N halves, in mg_pool)
    // diagnostics (allocated when enabled, never during a step)
    int rates_on = 0;
    int rate_lo[3] = {0, 0, 0}, rate_hi[3] = {0, 0, 0};
    double* rates_dev = nullptr;  // the 33 region-summed process amounts of the last step
    // volume export scratch (allocated by the first export, never during a step)
    int* brick_flags = nullptr;   // per 8^3 brick: active, then its output slot
    int* brick_count = nullptr;
    void* brick_out = nullptr;    // packed brick values and coordinates
    // asynchronous readback: a device snapshot of the fields and the stream that copies it out
    float* snap = nullptr;
    size_t snap_fields = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_snap = nullptr, ev_copy = nullptr;
    bool copy_pending = false;
    size_t brick_out_bytes = 0;
    int diag_flags = 0;
    float* dbg_buoy = nullptr;    // buoyancy velocity change per cell (the second debug field)
    float* dbg_zero = nullptr;    // the first debug field, which the step never writes
    // launch accounting and optional per-stage event timing
    long long launches = 0;
    float last_gpu_ms = 0.0f;
    int async_steps = 0;  // graph steps queued by skt_step_async and not yet collected by skt_sync
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool prof = false;
    struct ProfRec { const char* name; cudaEvent_t a, b; int nk; };
    std::vector<ProfRec> recs;
};

// Times the kernels queued between construction and destruction when profiling is on.
struct ProfScope {
    Env& e;
    const char* name;
    cudaEvent_t a = nullptr;
    long long l0;
    ProfScope(Env& env, const char* n) : e(env), name(n), l0(env.launches) {
        if (e.prof && !e.capturing) { cudaEventCreate(&a); cudaEventRecord(a, e.stream); }
    }
    ~ProfScope() {
        if (e.prof && !e.capturing) {
            cudaEvent_t b;
            cudaEventCreate(&b);
            cudaEventRecord(b, e.stream);
            e.recs.push_back({name, a, b, int(e.launches - l0)});
        }
    }
};

// ---- launchers (defined in the kernel translation units) --------------------------------------
void launch_diffuse(Env& e, float* f, int type, float dtS);
int launch_advect(Env& e, float* f, const float* def, int sides, int ground, float dtS, int field_slot, bool host_sync,
                  bool same_wind = false);
void launch_precip(Env& e, float* q, int type, float dtS);
void launch_precip3(Env& e, float dtS);  // rain, snow and ice in one column march
void launch_buoyancy(Env& e, float dtS);
void launch_init_density(Env& e);
void launch_new_pressure(Env& e);
void launch_project(Env& e, float dtS);
void launch_micro(Env& e, float dt, float speed);
void launch_ground(Env& e, float dt, float speed, float irr);
void launch_init_state(Env& e, int noise, uint32_t seed);
void launch_isen_ground(Env& e);  // computeIsenTempGroundGPU on the current heightfield
void launch_editor_block(Env& e);  // editorDataGPU's ground block (after a ground edit)
inline int stencil_sms(const Env& e) { return e.stencil_sms > 0 ? e.stencil_sms : e.num_sms; }
bool mg_allocate(Env& e);
// Graph capture: inside a capture of e.stream, adds a WHILE conditional node. `init` queues the
// kernel that sets the node's condition for the first trip (before the node); `body` queues the
// body's launches (e.stream then points at a side stream that captures into the node's body graph)
// and must end with a kernel that counts the trip (note_trip) and sets the condition again. Both get
// the node's handle; body also gets the loop's index into Scalars::trips.
void graph_while(Env& e, const std::function<void(cudaGraphConditionalHandle)>& init,
                 const std::function<void(cudaGraphConditionalHandle, int)>& body);
__device__ __forceinline__ void note_trip(Scalars* sc, int loop) { sc->trips[loop] += 1; }
void launch_matvec_textbook(Env& e, const float* s, float* As);
void mg_solve(Env& e);

// C-ABI helpers of skt_api.cu: record the error text on e (or, for e == nullptr, the thread's
// create error) and return st; turn a pending CUDA error into a status
skt_status report(Env* e, skt_status st, const char* msg);
skt_status check_cuda(Env& e, const char* where);
// the device array behind a field selector (skt_read_field's mapping), nullptr if none
// Copies the device scalars into the pinned mirror e.host_sc with a one-warp kernel (stores to
// mapped host memory) and waits for the stream: the step's control reads never queue behind
// bulk copies on the copy engines.
void fetch_scalars(Env& e);
float* field_ptr(Env& e, int param, int dir);
float* ground_field_ptr(Env& e, int which);

}  // namespace skt

// the opaque handle of include/skewt.h
struct skt_env {
    skt::Env e;
};
