/*
 * skewt.h — C ABI of libskewt_gb300, a GB300 (sm_103a) implementation of skewTCloudSim's
 * per-timestep 3D atmosphere solver: colour-split diffusion, PPM advection, sedimentation,
 * buoyancy, a PCG pressure projection, bulk six-species microphysics and the ground/surface
 * kernels.
 *
 * It replaces the reference's `environmentGPU` class (Game/environment.cuh:9-183,
 * Game/environment.cu:71-1300). Plain pointers and sizes only. The library owns every device
 * buffer; host arrays passed in are copied.
 *
 * Layout: fields are float32 arrays of nx*ny*nz cells, idx = x + y*nx + z*nx*ny with y
 * VERTICAL (the reference's layout, Game/utils.cuh:8-11). Ground arrays hold nx*nz values,
 * idxG = x + z*nx. Cell (x,y,z) is ground when y <= ground_height[idxG].
 *
 * Threading: calls on one skt_env are not thread-safe; different environments are
 * independent. Work is queued on the environment's own CUDA stream. Nothing aborts the process:
 * every call returns an skt_status, and skt_last_error() describes the last failure.
 */
#ifndef SKEWT_GB300_H
#define SKEWT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct skt_env skt_env;

typedef enum {
    SKT_OK = 0,
    SKT_INVALID_ARG = 1,
    SKT_CUDA_ERROR = 2,
    SKT_NOT_CONVERGED = 3, /* the PCG hit its iteration cap; the step still completed */
    SKT_NAN_DETECTED = 4,  /* a step met a NaN or Inf (wind maximum or pressure-solver reduction); stepping stopped */
    SKT_TIMEOUT = 5,       /* a kernel's bounded wait for its own streamed data (TMA copies) ran out */
    SKT_OUT_OF_MEMORY = 6,
    SKT_NOT_INITIALIZED = 7,
    SKT_COURANT_LIMIT = 8  /* reserved, never returned: a step runs any substep count up to max_substeps */
} skt_status;

/* Field selector, the reference's `parameter` enum (Game/config.h:62-65) plus DENSITY. */
typedef enum {
    SKT_POTTEMP = 0, SKT_QV = 1, SKT_QW = 2, SKT_QC = 3, SKT_QR = 4, SKT_QS = 5, SKT_QI = 6,
    SKT_WIND = 7, SKT_PGROUND = 8, SKT_PRESSURE = 9, SKT_DEBUG1 = 10, SKT_DEBUG2 = 11, SKT_DEBUG3 = 12,
    SKT_DENSITY = 100
} skt_param;

/* Wind component selector, the reference's `direction` enum (Game/config.h:36-39):
 * LEFT/RIGHT = u (x), UP/DOWN = v (vertical), FORWARD/BACKWARD = w (z). */
typedef enum { SKT_LEFT = 0, SKT_RIGHT = 1, SKT_UP = 2, SKT_DOWN = 3, SKT_FORWARD = 4, SKT_BACKWARD = 5 } skt_direction;

/* Ground (nx*nz) arrays, gridDataGroundGPU (Game/environment.cuh:28-37) plus cloud cover. */
typedef enum {
    SKT_G_QRS = 0, SKT_G_QGR = 1, SKT_G_QGS = 2, SKT_G_QGI = 3, SKT_G_P = 4, SKT_G_TIME_WET = 5, SKT_G_T = 6,
    SKT_G_CLOUD_COVER = 7
} skt_ground_field;

/* Per-level default columns (ny values) taken at init; SKT_C_PRESSURE is the pressure column
 * skt_init received (the editor's pressure reset, m_defaultPressure). */
typedef enum { SKT_C_ISEN_T = 0, SKT_C_ISEN_QV = 1, SKT_C_DEF_U = 2, SKT_C_DEF_W = 3, SKT_C_PRESSURE = 4 } skt_column;

typedef struct {
    int nx, ny, nz; /* ny is vertical */
    float voxel;    /* cell size in metres (the reference's VOXELSIZE, Game/config.h:9) */
} skt_grid_desc;

typedef enum { SKT_SEM_REFERENCE = 0, SKT_SEM_TEXTBOOK = 1 } skt_semantics;
typedef enum { SKT_PCG_PLAIN = 0, SKT_PCG_MIXED = 1 } skt_precision;

typedef struct {
    int semantics;      /* skt_semantics: REFERENCE reproduces the reference's PCG quirks */
    int diffuse_sweeps; /* Jacobi sweeps per field (20, Game/environment.cu:649) */
    float pcg_tol;      /* stop when the max residual <= tol (1e-5, Game/environment.cu:906) */
    int pcg_max_iter;   /* 200 (Game/environment.cu:907) */
    int max_substeps;   /* Courant substep cap (100, Game/environment.cu:727) */
    int precision;      /* skt_precision */
    float refine_tol;   /* MIXED: relative residual target of the FP64 refinement (1e-8) */
    int inner_max_iter; /* MIXED: FP32 iterations per refinement step */
    float inner_rtol;   /* MIXED: relative tolerance of each FP32 inner solve */
    int use_graph;      /* 1: each step is one launch of a CUDA graph captured at the first step (and
                           again when dt, speed, the tuning, the diagnostics or the terrain's flatness
                           change), its loops (advection substeps, PCG iterations, the mixed
                           refinement) as conditional nodes decided on the device: no host
                           synchronisation inside a step; the solver's status is read once per
                           skt_step call. Not used while per-stage profiling is on. 0: launches
                           issued stream-ordered, the loop counts read back by the host. */
    int mg_half;        /* MIXED: the V-cycle smooths with FP16 copies of the finest coefficients */
    int pcg_fused;      /* PLAIN, nx % 4 == 0: two launches per iteration (search step and pressure
                           update fused into the operator's march) instead of three; same values up
                           to the dot products' summation order */
} skt_solver_cfg;

typedef struct {
    int pcg_iters;        /* iterations of the last step's projection (total inner for MIXED) */
    float pcg_residual;   /* final max residual */
    int pcg_converged;    /* 1 when the tolerance was met */
    int nsub[10];         /* Courant substeps per advected field (theta,u,v,w,qv,qw,qc,qr,qs,qi) */
    int outer_iters;      /* MIXED: refinement steps */
    double sim_time;      /* environmentGPU::m_time */
    long long kernel_launches; /* kernels this environment has launched since skt_create */
    float gpu_ms;         /* device time of the last skt_step call (CUDA events on its stream) */
} skt_step_stats;

/* Fills cfg with the reference's settings (reference semantics, plain PCG, no graph). */
void skt_default_config(skt_solver_cfg* cfg);

/* Replaces environmentGPU::environmentGPU() (Game/environment.cu:71-185): allocates all device
 * state for one grid on the current CUDA device and sets the ground stores as the reference
 * constructor does (Qrs = 0.001, P = 1000 hPa, T = 315.15 K, others 0). */
skt_status skt_create(const skt_grid_desc* grid, const skt_solver_cfg* cfg, skt_env** out);

/* Replaces environmentGPU::~environmentGPU() (Game/environment.cu:187-247). NULL is accepted. */
void skt_destroy(skt_env* env);

#define SKT_INIT_NOISE 1u /* add the reference's init noise (Game/environment.cu:308-313) */

/* Replaces environmentGPU::init (Game/environment.cu:249-389, declared
 * Game/environment.cuh:42). vel_aos3 holds (u, v, w) per cell on MAC faces like the reference's
 * glm::vec3 array; ground_height replaces the Perlin heightfield (which rounds to a flat ground
 * layer in the reference); noise_seed is the first of the five randomArray seeds (100). */
skt_status skt_init(skt_env* env, const float* theta, const float* vel_aos3, const float* qv, const float* ground_T,
                    const float* ground_p, const float* p3d, const float* p_column, const int32_t* ground_height,
                    uint32_t flags, uint32_t noise_seed);

/* Replaces environmentGPU::updateGPU(dt, speed) (Game/environment.cu:391-555), nsteps times.
 * Returns SKT_NOT_CONVERGED when a projection hit its iteration cap (the step is still done, as
 * in the reference). Returns SKT_NAN_DETECTED when a step met a NaN or Inf: the Courant wind
 * maximum saw a non-finite wind, or a dot product of the pressure solve came out non-finite (a
 * non-finite field value or a zero-density cell reaches it within the step); the steps after it
 * are not run and the fields are not valid (the reference runs on with NaNs). Does not read fields back (the reference's per-step GPUSetEnv copy,
 * Game/environment.cu:553, is explicit here: skt_read_field). */
skt_status skt_step(skt_env* env, float dt, float speed, int nsteps);

/* skt_step without waiting (graph mode, cfg.use_graph = 1): queues nsteps launches of the captured
 * step on the environment's stream and returns; the host may work meanwhile, and further calls
 * queue more steps. skt_sync waits for them and returns what skt_step would have returned for all
 * of them (SKT_NOT_CONVERGED, SKT_NAN_DETECTED, ...); skt_stats describes them after skt_sync.
 * Field reads, writes and edits queue behind the steps on the same stream. Without graph mode the
 * steps read their loop counts on the host, and the call runs them as skt_step does. */
skt_status skt_step_async(skt_env* env, float dt, float speed, int nsteps);

/* Waits for the environment's stream; after skt_step_async, the status of the queued steps. */
skt_status skt_sync(skt_env* env);

/* Ensemble stepping: advances n independent environments (members of any grid sizes, each with
 * its own state) by nsteps steps each. Every member already runs on its own CUDA stream; here up
 * to `threads` host threads (0: one per member, at most 64) drive the members' steps at once, so
 * the kernels of small members run side by side on the GPU instead of one member after another.
 * dt and speed hold one value per member (NULL: dt0 / 1 for all). Returns SKT_OK, or the first
 * failing member's status (SKT_NOT_CONVERGED counts as OK, as for skt_step); statuses, when not
 * NULL, receives every member's own status. Results equal stepping the members one by one. */
skt_status skt_step_ensemble(skt_env* const* envs, int n, const float* dt, float dt0, const float* speed, int nsteps,
                             int threads, int* statuses);

/* Ensemble as one CUDA graph (no counterpart in the reference, which runs one environment): every
 * member's whole step, its loops as conditional nodes decided on the device, is captured as an
 * independent branch of one graph at the first skt_ensemble_step (and again when a member's dt,
 * speed, tuning, diagnostics or terrain flatness change), so each ensemble step is a single graph
 * launch from the calling thread: the GPU runs the members' kernels side by side and the host
 * synchronises once per call. Results equal stepping the members one by one, bit for bit. While a
 * member belongs to an ensemble, the grids of its per-cell kernels are sized for its share of the
 * SMs (twice its proportion of the cells), since the members run side by side; skt_ensemble_destroy gives
 * it the whole GPU again. Members keep their own state and may still be stepped alone; they must
 * outlive the ensemble and must not be stepped from another thread while the ensemble steps. */
typedef struct skt_ensemble skt_ensemble;
skt_status skt_ensemble_create(skt_env* const* envs, int n, skt_ensemble** out);
void skt_ensemble_destroy(skt_ensemble* ens);
/* nsteps steps of every member (dt and speed per member, or dt0 and 1 for all when NULL).
 * Returns SKT_OK, or the first member's failure (SKT_NOT_CONVERGED counts as OK); statuses, when
 * not NULL, receives every member's own status (read once, after the last step). Failure text:
 * skt_last_error(NULL). */
skt_status skt_ensemble_step(skt_ensemble* ens, const float* dt, float dt0, const float* speed, int nsteps, int* statuses);

/* Field readback: the per-field copies of editor::GPUSetEnv (Game/editor.cpp:226-260).
 * dir selects the wind component for SKT_WIND. n must equal nx*ny*nz. Synchronous. */
skt_status skt_read_field(skt_env* env, int param, int dir, float* host_dst, size_t n);

/* The per-frame readback of editor::GPUSetEnv (Game/editor.cpp:226-260, all 11 sky fields after
 * every step), without stalling the step loop.
 * Asynchronous readback of several fields (same selectors): the fields as they stand after the
 * work queued so far are snapshot on the device, then copied to host_dsts[i] on a second stream,
 * so that the next steps can run while the copies proceed; the call returns at once. A new
 * snapshot first waits for the previous one's copies. The host buffers (n floats each, n =
 * nx*ny*nz) must stay valid until skt_read_wait. In graph mode (cfg.use_graph = 1) every buffer is
 * copied by the copy engine, beside the next steps; with stream-ordered steps, whose small scalar
 * reads would queue behind those copies, pinned buffers (cudaHostAlloc / cudaHostRegister) are
 * written by a small kernel through their mapped addresses instead, alongside the next steps'
 * kernels, and pageable ones by the copy engine.
 * The snapshot memory (nfields fields) is allocated by the first call that needs it. */
skt_status skt_read_fields_async(skt_env* env, int nfields, const int* params, const int* dirs, float* const* host_dsts,
                                 size_t n);

/* Waits for the copies of the last skt_read_fields_async. */
skt_status skt_read_wait(skt_env* env);

/* Field upload (state injection); same selectors. Synchronous. */
skt_status skt_write_field(skt_env* env, int param, int dir, const float* host_src, size_t n);

/* Replaces environmentGPU::getParamArray (Game/environment.cu:1076-1125): the device pointer of
 * a field, valid until skt_destroy. */
skt_status skt_field_device_ptr(skt_env* env, int param, int dir, float** out);

/* Ground arrays (nx*nz) and default columns (ny). Synchronous. */
skt_status skt_read_ground(skt_env* env, int which, float* host_dst, size_t n);
skt_status skt_write_ground(skt_env* env, int which, const float* host_src, size_t n);
skt_status skt_read_column(skt_env* env, int which, float* host_dst, size_t n);
skt_status skt_write_column(skt_env* env, int which, const float* host_src, size_t n);

/* Diurnal clock of environmentGPU (m_time, m_day, m_longitude, m_sunStrength, m_pauseDiurnal). */
skt_status skt_set_clock(skt_env* env, double sim_time, int day, float longitude, float sun, int pause);

/* Diagnostics of the last step (PCG iterations/residual, substeps). */
skt_status skt_stats(skt_env* env, skt_step_stats* out);

/* Runs one stage of the step alone, for per-stage parity tests:
 * 0 diffuse (arg = type 0..5 on theta,qv,u,v,w,qw), 1 advect (arg 0..5 on theta,u,v,w,qv,qw),
 * 2 buoyancy, 3 density + projection, 4 microphysics, 5 sedimentation (arg 0..2 on qr,qs,qi),
 * 6 ground stage, 8 density, 9 pressure from density. dt is dt*speed except for 4 and 6. */
skt_status skt_run_stage(skt_env* env, int stage, int arg, float dt, float speed, skt_step_stats* out);

/* Per-stage CUDA-event timing of the kernels queued while enabled (no reference
 * counterpart; the reference's own timing code is commented out, Game/environment.cu:697-702).
 * skt_profile_read synchronises, then writes a JSON object {stage: [ms, kernels, scopes]} into
 * buf and clears the records. */
skt_status skt_profile_enable(skt_env* env, int on);
skt_status skt_profile_read(skt_env* env, char* buf, size_t n);

/* Allocation-free diffusion (no counterpart in the reference). For callers that cannot
 * allocate device memory: a host framework that owns the device memory pool and forbids other
 * allocations, or a running loop where a cudaMalloc would stall the device. It runs the
 * diffusion stage (diffuseGPU's sweeps and boundary table, field_type 0..5 as there) on
 * caller-owned device buffers: in_dev is read, out_dev receives the result (ground cells copied
 * from in_dev). The one intermediate buffer lives in a static device array of
 * SKT_NOALLOC_MAX_CELLS floats (8 MiB) that every GPU loading the library holds until exit;
 * larger grids are rejected with SKT_INVALID_ARG (message in skt_last_error(NULL)), as are
 * nz > 65535 and ny > 524280 (CUDA grid limits). The first call in each CUDA context (a device's
 * primary context, or a driver-API context the caller made current) looks up that array's address,
 * so make it before any stream capture, with the context the later calls will use current.
 * Buffers: in_dev and out_dev hold nx*ny*nz floats, ground_height_dev, ground_T_dev and
 * ground_p_dev nx*nz values, default_column_dev ny floats (the level defaults of this field type:
 * the isentrope for theta and Qv, the default u or w column for u and w; unused for types 3 and 5,
 * may be NULL there), p_dev nx*ny*nz floats (theta only; the others may pass NULL).
 * Calls share the array: calls whose work overlaps on the GPU race. Work is queued on `stream`
 * (a cudaStream_t; NULL = default stream); the call does not synchronise. Nothing in the array
 * needs clearing between calls (every value is written before it is read). */
#define SKT_NOALLOC_MAX_CELLS (1u << 21)
skt_status skt_diffuse_noalloc(int nx, int ny, int nz, float voxel, int field_type, float dt_speed, int sweeps,
                               const float* in_dev, float* out_dev, const int32_t* ground_height_dev,
                               const float* default_column_dev, const float* p_dev, const float* ground_T_dev,
                               const float* ground_p_dev, void* stream);

/* ---- Launch-shape tuning (no counterpart in the reference: its launch shapes are fixed) ---- */

/* Launch shapes of the stencil kernels. None of them changes the results (every cell is computed
 * with the same arithmetic from the same neighbour values); they change only the speed.
 * diffuse_depth: sweeps per diffusion pass, 1 or 2 (temporal blocking: two Jacobi sweeps per trip
 * through HBM, input planes streamed by TMA, flat terrain); diffuse_rows selects the two-sweep
 * kernel and its tile height: 6 or 14 output rows per block of four-cell lanes, or 4 or 8 rows per
 * warp of one-cell lanes (the intermediate sweep is recomputed on the tile's edge rows);
 * *_bps: blocks per SM in the grid of the diffusion (one-sweep and two-sweep) and PPM (x, y, z
 * pass) marches, which sets their run lengths. from_cache and the times are outputs of
 * skt_autotune. */
typedef struct {
    int diffuse_depth;
    int diffuse_rows;
    int diffuse_bps;
    int diffuse2_bps;
    int ppm_x_bps;
    int ppm_y_bps;
    int ppm_z_bps;
    int from_cache;   /* skt_autotune: 1 when the shapes came from the cache file */
    float diffuse_ms; /* skt_autotune: theta's and water vapour's diffusions (all sweeps) with the chosen shapes */
    float advect_ms;  /* skt_autotune: one advection (all passes and substeps) with the chosen shapes */
} skt_tuning;

#define SKT_TUNE_FORCE 1 /* skt_autotune: measure even when the cache has an entry */

/* The environment's current launch shapes. */
skt_status skt_get_tuning(skt_env* env, skt_tuning* out);

/* Sets the launch shapes (the output fields are ignored). SKT_INVALID_ARG for values out of range. */
skt_status skt_set_tuning(skt_env* env, const skt_tuning* t);

/* Chooses the launch shapes for this grid on this GPU: with cache_path set and an entry for the GPU
 * name and grid in that file (and no SKT_TUNE_FORCE), the entry is applied; otherwise every
 * candidate shape is timed on scratch copies of the environment's own fields (a few hundred
 * milliseconds at 512x256x512), candidates whose results differ from the default shapes' in any
 * bit are rejected, the fastest are applied and, with cache_path set, written to the cache (a JSON
 * object, one entry per line). Call between steps; the fields are not changed. Allocates one small
 * device counter while measuring. */
skt_status skt_autotune(skt_env* env, const char* cache_path, int flags, skt_tuning* out);

/* ---- Diagnostics (the reference's data graph and debug views) ---------------------------- */

/* Region-summed microphysics process amounts: the reference's data graph
 * (Game/microPhysics.cu:1356-1413, reset each step at Game/environment.cu:571, read back by
 * dataClass::setMicroPhysicsData Game/dataClass.cu:42). While enabled, every step sums over the
 * sky cells with lo <= (x, y, z) <= hi (inclusive, reference layout, y vertical) the 33 amounts
 * of each cell after its update, PVCON and PVDEP split by sign into PVCON/PVVAP and PVDEP/PVSUB,
 * PGWET times WTerm and PGDRY times (1 - WTerm); the reference sums with float atomics, here in
 * FP64. enable = 0 turns it off. The first enable allocates 33 doubles on the device. */
#define SKT_RATE_COUNT 33
/* PVCON PVDEP PIMLT PIDW PIHOM PIACR PRACI PRAUT PRACW PREVP PRACS PSACW PSACR PSACI PSAUT PSFW
 * PSFI PSDEP PSSUB PSMLT PGAUT PGFR PGACW PGACI PGACR PGDRY PGACS PGSUB PGMLT PGWET PGACR1 PVVAP
 * PVSUB (the order of microPhysicsParams, Game/microPhysics.cuh:7-21) */
skt_status skt_set_rate_region(skt_env* env, int enable, const int lo[3], const int hi[3]);

/* The region sums of the last step (n must be SKT_RATE_COUNT). Synchronous. */
skt_status skt_read_rates(skt_env* env, float* host_dst, size_t n);

/* Debug fields, read with skt_read_field / skt_field_device_ptr as the reference's editor reads
 * its three debug arrays (Game/editor.cpp:190-224, shown as DEBUG1..3): SKT_DEBUG1 is never
 * written by the reference's GPU step and reads as zeros; SKT_DEBUG2 is buoyancyGPU's velocity
 * change per sky cell (Game/kernelSky.cu:1128,1244; 0 where no side neighbour is sky), produced
 * while SKT_DIAG_BUOYANCY is set; SKT_DEBUG3 is the projection's pressure correction
 * (Game/environment.cu:883). Enabling allocates the debug arrays; a step allocates nothing. */
#define SKT_DIAG_BUOYANCY 1
skt_status skt_set_diagnostics(skt_env* env, int flags);

/* ---- Editing between steps (the reference's editor tools) -------------------------------- */

/* Replaces environmentGPU::prepareBrushGPU (Game/environment.cu:1127-1186, kernel applyBrushGPU
 * Game/kernelSky.cu:1476-1549). param: SKT_POTTEMP, SKT_QV..SKT_QI, SKT_WIND (the amount split by
 * dir[3] into u, v, w) or SKT_PGROUND (raise the heightfield to the brushed cells, or with
 * ground_erase lower it to the lowest brushed ground cell; cells an erase frees take the default
 * columns). Adds (1 - d^2/r^2)^smoothness * dt * intensity * value to the sky cells at squared
 * distance d^2 <= r^2 = brush_size^2 from pos (reference layout x, y vertical, z); the brush box
 * reaches -ceil(r) .. ceil(r)-1 in x and y, as the reference's. *ground_changed (optional) tells
 * whether the heightfield changed. SKT_PRESSURE is rejected (the reference has no pressure array
 * for it). Synchronous. */
skt_status skt_apply_brush(skt_env* env, int param, float brush_size, const int pos[3], float smoothness, float dt, float intensity,
                           float value, const float dir[3], int ground_erase, int* ground_changed);

/* Replaces environmentGPU::prepareSelectionGPU (Game/environment.cu:1188-1262, kernel
 * applySelectionGPU Game/kernelSky.cu:1551-1595): sets value (wind: split by dir) on the sky cells
 * of the box lo..hi (inclusive; an empty x or y extent becomes one cell, as the reference's host
 * code does), or edits the heightfield as skt_apply_brush. Synchronous. */
skt_status skt_apply_selection(skt_env* env, int param, const int lo[3], const int hi[3], float value, const float dir[3], int ground_erase,
                               int* ground_changed);

/* Replaces environmentGPU::resetParameterGPU (Game/environment.cu:1264-1285): theta, Qv, wind
 * (u, w) and pressure back to their default columns (each (x, y) column of cells stops at its
 * first ground cell, as the reference's setToDefault does), v and Qw..Qi to 0 everywhere.
 * Synchronous. */
skt_status skt_reset_parameter(skt_env* env, int param);

/* The boundary class of every cell's six neighbours as the library's kernels derive it from the
 * heightfield, written as the reference's Neigh records (computeNeighbourGPU,
 * Game/kernelSky.cu:1284-1316, which the reference stores per cell and this library does not):
 * 12 bytes per cell, for left (-x), right (+x), up (+y), down (-y), forward (+z), backward (-z)
 * a byte `outside` (the neighbour lies outside the grid) and a byte `type` (0 sky, 1 ground).
 * n is the cell count nx*ny*nz; host_dst holds 12*n bytes. Allocates a temporary device buffer.
 * Synchronous. */
skt_status skt_read_neighbours(skt_env* env, uint8_t* host_dst, size_t n);

/* The current heightfield (nx*nz values). Synchronous. */
skt_status skt_read_ground_height(skt_env* env, int32_t* host_dst, size_t n);

/* ---- Sounding ingestion: the radiosonde readers and column interpolation of readTable ---- */

/* One radiosonde ascent, radioSondeData (Game/readTable.h:9-47): n rows in file order (bottom
 * up). Arrays filled by skt_sounding_read_* belong to the library (skt_sounding_free); a caller
 * may also point them at its own arrays to feed skt_sounding_to_init. */
typedef struct {
    size_t n;
    float* altitude;    /* m above sea level */
    float* pressure;    /* hPa */
    float* temperature; /* deg C */
    float* dew_point;   /* deg C */
    float* wind_speed;  /* m/s */
    float* wind_dir;    /* degrees (the direction the wind blows from) */
} skt_sounding;

/* Archive access: the two calls readTable makes on its zip archive (miniz_cpp::zip_file::has_file
 * and read, Game/zip_file.hpp:5286,5459). Returns the size in bytes of the member `name`, or -1
 * when the archive has no such member; when buf is not NULL and cap is at least that size, the
 * member's bytes are copied to buf first. */
typedef long long (*skt_archive_read_fn)(void* ctx, const char* name, char* buf, size_t cap);

/* Replaces readTable::readKNMIFile (Game/readTable.cpp:27-132): parses the member
 * SynchronizedSoundingData.xml of a KNMI .mwx archive. As there: the first line is skipped; on
 * every later line the whitespace-separated tokens 4..8 are pressure (hPa), temperature (K),
 * relative humidity (%), wind direction and wind speed, each read after a fixed-length
 * attribute prefix (10, 13, 10, 9, 11 characters) with its closing quote dropped, and any other
 * token that starts with "Altitude" is the altitude; the dew point is
 * T - (100 - RH) * 0.2 * (T + 273.15) * 0.01 (deg C); the last line read is not a row.
 * Where the reference's reads would go out of bounds (short tokens, missing columns) or std::stof
 * would throw, this returns SKT_INVALID_ARG. On error *out is left empty. */
skt_status skt_sounding_read_knmi(skt_archive_read_fn read, void* ctx, skt_sounding* out);

/* Replaces readTable::readDWDFile (Game/readTable.cpp:134-354) for a DWD "sekundenwerte aero"
 * archive. archive_name is the string the reference splits on '_' for the station number (its
 * third field). As there: the member Metadaten_Sekunde_Aero_<station>.txt lists the ascents
 * (field 1 less its two last characters is a date); the ascent read is the one of date 161 at
 * 12 UTC, from the member produkt_sec_aero_<first date>_<last date>_<station>.txt, found with the
 * reference's search (100000-byte forward probes, then a scan from 100000 bytes back), which
 * decides which rows are read: it can miss the first rows of an ascent or an ascent near the
 * end of the member. Fields 6, 7, 8, 10, 11, 12 are altitude, pressure, temperature, dew point,
 * wind speed and direction. Returns SKT_INVALID_ARG where the reference prints an error and
 * reads nothing (missing member, date not found) and where it would read out of bounds. */
skt_status skt_sounding_read_dwd(const char* archive_name, skt_archive_read_fn read, void* ctx, skt_sounding* out);

/* Frees the arrays of a sounding filled by skt_sounding_read_*; leaves it empty. */
void skt_sounding_free(skt_sounding* s);

/* Replaces readTable::initEnvironment (Game/readTable.cpp:364-474) for a run-time grid: the
 * arrays skt_init takes, every column a copy of the sounding interpolated to the level heights
 * y*voxel above the first row (theta relative to the first row's pressure, Qv = ws(dew point,
 * p), wind from direction and speed on MAC faces, ground T and p from the first row). The
 * outputs are nx*ny*nz (vel_aos3 three times that), nx*nz (ground) and ny (p_column) floats.
 * SKT_INVALID_ARG when the sounding ends below the grid top. */
skt_status skt_sounding_to_init(const skt_sounding* s, const skt_grid_desc* grid, float* theta, float* vel_aos3,
                                float* qv, float* ground_T, float* ground_p, float* p3d, float* p_column);

/* ---- Headless view and volume export (the editor's voxel view, without a renderer) ---- */

#define SKT_VOXEL_HIDDEN 0         /* not drawn */
#define SKT_VOXEL_SKY 1            /* a sky voxel in the view's colour */
#define SKT_VOXEL_GROUND 2         /* ground below the surface (brown) */
#define SKT_VOXEL_GROUND_SURFACE 3 /* the surface voxel of a column, in the ground view's colour */

/* Replaces the per-frame voxel drawing of editor::viewSky and editor::viewGround
 * (Game/editor.cpp:1041-1171) with the colour schemes of editor::setColors (:53-112), evaluated
 * per cell on the device as bee::colorScheme::getColor does (Engine/source/rendering/colors.cpp:28-67).
 * sky_param selects the sky view like the editor's buttons: SKT_POTTEMP (the temperature
 * theta * (p / ground p)^(Rsd/Cpd)), SKT_QV..SKT_QI, SKT_WIND (the cell-centred speed of
 * environment::getUV), SKT_PRESSURE, SKT_DEBUG1 (the "realistic" view of all condensate, cells
 * below 1e-4 kg/kg not drawn), SKT_DEBUG2 and SKT_DEBUG3 (the debug fields). ground_param selects
 * the ground view (0 temperature, 1 Qrs, 2 Qgr, 3 Qgs, 4 Qgi; -1 none). lo/hi (x, y, z, y vertical)
 * bound the sky view like the editor's slice (NULL: the whole grid). Writes n = nx*ny*nz RGB
 * triples (floats, 0..1) and voxel kinds (SKT_VOXEL_*) to host memory. Synchronous. */
skt_status skt_view_volume(skt_env* env, int sky_param, int ground_param, const int lo[3], const int hi[3], float* rgb,
                           uint8_t* kind, size_t n);

/* Sparse export of one field (same selectors as skt_read_field) in bricks of 8x8x8 cells: a
 * brick is written when one of its cells differs from `background` by more than `threshold`
 * (NaN always; threshold < 0 writes every brick). Bricks go out in brick order (x fastest), each
 * as 512 values in x-fastest order (cells past the grid edge hold the background), as float or,
 * with half != 0, IEEE half (round to nearest even), with their brick coordinates (3 uint32 each).
 * *count receives the number of bricks; nothing is copied when coords or values is NULL or
 * capacity (in bricks) is below the count, so a first call with capacity 0 sizes the buffers.
 * Synchronous. */
skt_status skt_export_bricks(skt_env* env, int param, int dir, float background, float threshold, int half,
                             uint32_t* coords, void* values, size_t capacity, size_t* count);

/* Text of the last error on env (or, when env is NULL, of the last skt_create, skt_ensemble_*,
 * skt_diffuse_noalloc or skt_sounding_* failure on this thread). */
const char* skt_last_error(const skt_env* env);

/* Library version string. */
const char* skt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SKEWT_GB300_H */
