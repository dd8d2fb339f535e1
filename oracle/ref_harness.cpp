// ORACLE — test infrastructure only (generates golden fixtures; never part of the product).
//
// Drives skewTCloudSim's OWN CUDA kernels (Game/kernelSky.cu, Game/microPhysics.cu,
// Game/kernelGround.cu, Game/kernelMaths.cu, compiled unmodified into a cubin by
// oracle/build_ref.py) through the CUDA driver API. The host side restates
// environmentGPU::updateGPU and its helpers (Game/environment.cu:391-987, 1021-1069): the same
// launches, launch shapes, buffers, memsets and host read-backs, in the same order. The
// kernels' compile-time grid size and voxel size are the ones the cubin was built for.
//
// State in/out is the oracle's layout (tests pass the same arrays to both).
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

#define CK(x)                                                                          \
    do {                                                                               \
        CUresult r_ = (x);                                                             \
        if (r_ != CUDA_SUCCESS) {                                                      \
            const char* s_ = nullptr;                                                  \
            cuGetErrorString(r_, &s_);                                                 \
            g_err = std::string(#x) + ": " + (s_ ? s_ : "?") + " line " + std::to_string(__LINE__); \
            throw 1;                                                                   \
        }                                                                              \
    } while (0)

enum BC { NEUMANN = 0, DIRICHLET = 1, CUSTOM = 2 };
struct Bounds { int sides, up, ground; };  // boundsEnv (Game/config.h:50-58)
struct I3 { int x, y, z; };

struct Dim { unsigned x, y, z; };

struct H {
    int X, Y, Z;
    float VOX;
    CUmodule mod = nullptr;
    std::vector<std::pair<std::string, CUfunction>> fns;
    size_t N, NG;
    // device buffers of environmentGPU (Game/environment.cu:81-149)
    CUdeviceptr Qv = 0, Qw = 0, Qc = 0, Qr = 0, Qs = 0, Qi = 0, th = 0, u = 0, v = 0, w = 0, p = 0;
    CUdeviceptr Qrs = 0, Qgr = 0, Qgs = 0, Qgi = 0, P = 0, t = 0, T = 0, dGround = 0, dGround2 = 0, GH = 0;
    CUdeviceptr arr = 0, out = 0, density = 0, densityAir = 0, oldDensityAir = 0, neigh = 0, microRes = 0;
    CUdeviceptr isenT = 0, isenQv = 0, defU = 0, defW = 0, dummy = 0, dummySky2 = 0;
    CUdeviceptr condens = 0, depos = 0, freeze = 0, single0 = 0, sigma0 = 0, sigma1 = 0;
    CUdeviceptr stor0 = 0, stor1 = 0, stor2 = 0, A = 0, precon = 0;
    float time_ = 43200.0f;
    int day = 130;
    float lon = 52.37f, sun = 1.0f;
    int pause = 0;
    float pcg_tol = 1e-5f;
    int pcg_max = 200;
    int last_iters = 0;

    CUfunction fn(const char* tag) {
        for (auto& kv : fns)
            if (kv.first.find(tag) != std::string::npos) return kv.second;
        g_err = std::string("kernel not found: ") + tag;
        throw 1;
    }
    template <class... A>
    void launch(const char* tag, Dim g, Dim b, A... args) {
        void* pr[] = {(void*)&args...};
        CK(cuLaunchKernel(fn(tag), g.x, g.y, g.z, b.x, b.y, b.z, 0, nullptr, pr, nullptr));
    }
    void sync() { CK(cuCtxSynchronize()); }
    CUdeviceptr alloc(size_t bytes) {
        CUdeviceptr d;
        CK(cuMemAlloc(&d, bytes));
        CK(cuMemsetD8(d, 0, bytes));
        return d;
    }
    void zero(CUdeviceptr d, size_t bytes) { CK(cuMemsetD8(d, 0, bytes)); }
    void copy(CUdeviceptr dst, CUdeviceptr src, size_t bytes) { CK(cuMemcpyDtoD(dst, src, bytes)); }
    float readf(CUdeviceptr d) {
        float v;
        CK(cuMemcpyDtoH(&v, d, 4));
        return v;
    }

    // ---- environmentGPU helpers ----
    Dim T16() const { return {unsigned((X + 15) / 16), unsigned((Y + 15) / 16), 1}; }
    Dim B16() const { return {unsigned(X < 16 ? X : 16), unsigned(Y < 16 ? Y : 16), 1}; }

    void diffuse(CUdeviceptr f, int type, float dt) {  // :597-673
        CUdeviceptr def = 0;
        Bounds b{NEUMANN, DIRICHLET, DIRICHLET};
        switch (type) {
            case 0: def = isenT; b.ground = CUSTOM; b.sides = CUSTOM; b.up = CUSTOM; break;
            case 1: def = isenQv; b.ground = DIRICHLET; b.sides = CUSTOM; b.up = CUSTOM; break;
            case 2: def = defU; b.sides = CUSTOM; b.up = CUSTOM; break;
            case 3: def = 0; b.sides = NEUMANN; b.up = DIRICHLET; break;
            case 4: def = defW; b.sides = CUSTOM; b.up = CUSTOM; break;
            case 5: zero(dummy, Y * 4); def = dummy; break;
        }
        copy(arr, f, N * 4);
        const float k = 0.005f * dt / (VOX * VOX);
        for (int L = 0; L < 10; ++L) {
            launch("diffuseRedBlack", T16(), B16(), neigh, T, p, P, def, arr, out, k, type, b, true);
            sync();
            launch("diffuseRedBlack", T16(), B16(), neigh, T, p, P, def, arr, out, k, type, b, false);
            sync();
            launch("diffuseRedBlack", T16(), B16(), neigh, T, p, P, def, out, arr, k, type, b, true);
            sync();
            launch("diffuseRedBlack", T16(), B16(), neigh, T, p, P, def, out, arr, k, type, b, false);
            sync();
        }
        copy(f, arr, N * 4);
    }

    int advect(CUdeviceptr f, CUdeviceptr def, Bounds b, float dt) {  // :692-824
        zero(out, N * 4);
        zero(stor0, N * 4);
        launch("10setToValue", Dim{1, 1, 1}, Dim{unsigned(Y), 1, 1}, dummySky2, 1.0f, 1, 0);
        sync();
        zero(single0, 4);
        launch("getMaxDivergence", Dim{unsigned(Y), 1, 1}, Dim{unsigned(X), 1, 1}, single0, u);
        launch("getMaxDivergence", Dim{unsigned(Y), 1, 1}, Dim{unsigned(X), 1, 1}, single0, v);
        launch("getMaxDivergence", Dim{unsigned(Y), 1, 1}, Dim{unsigned(X), 1, 1}, single0, w);
        const float maxVel = readf(single0);
        const float C = maxVel * dt / VOX;
        const int sub = int(fminf(ceilf(fabsf(C)), 100.0f));
        const float dts = dt / sub;
        const Dim YX{unsigned(Y), 1, 1}, XT{unsigned(X), 1, 1};
        for (int i = 0; i < sub; ++i) {
            launch("10advectPPMX", T16(), B16(), density, stor0, dummySky2, u, neigh, b, dts * 0.5f);
            launch("10advectPPMX", T16(), B16(), f, out, def, u, neigh, b, dts * 0.5f);
            sync();
            launch("12divideValues", YX, XT, out, stor0, Z);
            launch("10setToValue", YX, XT, density, 1.0f, Z, 0);
            sync();
            launch("10advectPPMY", T16(), B16(), density, stor0, dummySky2, v, neigh, b, dts * 0.5f);
            launch("10advectPPMY", T16(), B16(), out, f, def, v, neigh, b, dts * 0.5f);
            sync();
            launch("12divideValues", YX, XT, f, stor0, Z);
            launch("10setToValue", YX, XT, density, 1.0f, Z, 0);
            sync();
            launch("10advectPPMZ", T16(), B16(), density, stor0, dummySky2, w, neigh, b, dts);
            launch("10advectPPMZ", T16(), B16(), f, out, def, w, neigh, b, dts);
            sync();
            launch("12divideValues", YX, XT, out, stor0, Z);
            launch("10setToValue", YX, XT, density, 1.0f, Z, 0);
            sync();
            launch("10advectPPMY", T16(), B16(), density, stor0, dummySky2, v, neigh, b, dts * 0.5f);
            launch("10advectPPMY", T16(), B16(), out, f, def, v, neigh, b, dts * 0.5f);
            sync();
            launch("12divideValues", YX, XT, f, stor0, Z);
            launch("10setToValue", YX, XT, density, 1.0f, Z, 0);
            sync();
            launch("10advectPPMX", T16(), B16(), density, stor0, dummySky2, u, neigh, b, dts * 0.5f);
            launch("10advectPPMX", T16(), B16(), f, out, def, u, neigh, b, dts * 0.5f);
            sync();
            launch("12divideValues", YX, XT, out, stor0, Z);
            launch("10setToValue", YX, XT, density, 1.0f, Z, 0);
            sync();
            copy(f, out, N * 4);
        }
        return sub;
    }

    void precip(CUdeviceptr f, int type, float dt) {  // :826-849
        const float maxVel = type == 0 ? 5.0f : (type == 1 ? 1.0f : 8.0f);
        const float C = maxVel * dt / VOX;
        const int sub = int(fminf(ceilf(fabsf(C)), 100.0f));
        const float dts = dt / sub;
        for (int i = 0; i < sub; ++i) {
            launch("advectPrecipGPU", Dim{unsigned(X), 1, 1}, Dim{unsigned(Y), 1, 1}, f, neigh, th, Qv, p, P, type, dts);
            sync();
        }
    }

    void pcg(CUdeviceptr outP, float dt) {  // calculatePressureProject :898-987
        const Bounds bD{NEUMANN, NEUMANN, DIRICHLET}, bA{DIRICHLET, DIRICHLET, DIRICHLET}, bV{CUSTOM, CUSTOM, DIRICHLET};
        zero(stor0, N * 4);
        zero(stor1, N * 4);
        zero(stor2, N * 4);
        zero(outP, N * 4);
        zero(single0, 4);
        zero(sigma0, 4);
        zero(sigma1, 4);
        last_iters = 0;
        launch("calculateDivergenceGPU", T16(), B16(), stor0, neigh, u, v, w, densityAir, oldDensityAir, dummySky2, bD, bV, dt);
        sync();
        const Dim YX{unsigned(Y), 1, 1}, XT{unsigned(X), 1, 1};
        launch("getMaxDivergence", YX, XT, single0, stor0);
        sync();
        float maxr = readf(single0);
        if (maxr == 0.0f) return;
        launch("applyPreconditionerGPU", YX, XT, stor1, precon, stor0, A);
        sync();
        copy(stor2, stor1, N * 4);
        launch("dotProductGPU", YX, XT, sigma0, stor1, stor0);
        sync();
        for (int i = 0; i < pcg_max; ++i) {
            launch("applyAGPU", T16(), B16(), stor1, stor2, neigh, A, bA);
            sync();
            launch("dotProductGPU", YX, XT, sigma1, stor1, stor2);
            sync();
            launch("updatePandDiv", YX, XT, sigma0, sigma1, outP, stor0, stor2, stor1);
            sync();
            last_iters = i + 1;
            zero(single0, 4);
            launch("getMaxDivergence", YX, XT, single0, stor0);
            sync();
            maxr = readf(single0);
            if (maxr <= pcg_tol) return;
            launch("applyPreconditionerGPU", YX, XT, stor1, precon, stor0, A);
            zero(sigma1, 4);
            sync();
            launch("dotProductGPU", YX, XT, sigma1, stor1, stor0);
            sync();
            launch("endIteration", YX, XT, sigma0, sigma1, stor2, stor1);
            sync();
        }
    }

    void project(float dt) {  // pressureProject :851-896
        const Bounds bD{NEUMANN, NEUMANN, DIRICHLET}, bA{NEUMANN, DIRICHLET, DIRICHLET};
        const Dim YX{unsigned(Y), 1, 1}, XT{unsigned(X), 1, 1};
        launch("10setToValue", Dim{1, 1, 1}, Dim{unsigned(Y), 1, 1}, dummySky2, 1.0f, 1, 0);
        launch("resetVelPressProj", YX, XT, neigh, u, v, w);
        sync();
        launch("initAMatrix", T16(), B16(), A, neigh, densityAir, dummySky2, bA);
        sync();
        launch("initPrecon", YX, XT, precon, A);
        sync();
        pcg(out, dt);
        launch("updatePressure", YX, XT, p, out);
        launch("initDensity", YX, XT, densityAir, th, p, Qv, P);
        sync();
        launch("applyPresProjGPU", YX, XT, out, neigh, u, v, w, densityAir, p, bD, dt);
        sync();
    }

    float irradiance() const {  // :1021-1034
        const float Gs = 1361.0f * sun;
        const float rd = 1 + 0.034f * cosf(2 * 3.14159265359f * day / 365);
        const float sd = 0.409f * sinf(2 * 3.14159265359f / 365 * (day - 81));
        const float th_ = time_ / 3600;
        const float lr = lon * 0.01745329251994329576923690768489f;
        const float sr = (th_ - (6.0f + 14.0f / 2.0f)) * (3.14159265359f / 12.0f);
        const float vv = Gs * rd * (sinf(lr) * sinf(sd) + cosf(lr) * cosf(sd) * cosf(sr));
        return vv > 0.0f ? vv : 0.0f;
    }

    void step(float dt, float speed, int* nsub) {  // updateGPU :391-555
        const Dim YX{unsigned(Y), 1, 1}, XT{unsigned(X), 1, 1}, ZX{unsigned(Z), 1, 1};
        const float dtS = dt * speed;
        launch("10setToValue", YX, XT, density, 1.0f, Z, 0);
        const float irr = irradiance();
        launch("advectGroundWaterGPU", Dim{unsigned((X + 15) / 16), unsigned((Z + 15) / 16), 1},
               Dim{unsigned(X < 16 ? X : 16), unsigned(Z < 16 ? Z : 16), 1}, Qrs, Qgr, dt, speed);
        sync();
        launch("calculateCloudCoverGPU", ZX, XT, dGround, Qc, Qw, GH);
        sync();
        launch("calculateGroundTempGPU", ZX, XT, T, dtS, irr, dGround);
        sync();
        launch("calculatePrecipHittingGroundMicroPhysicsGPU", ZX, XT, Qv, Qr, Qs, Qi, Qgr, Qgs, Qgi, dt, speed, T, th, densityAir, p, P, u, GH);
        launch("calculateGroundMicroPhysicsGPU", ZX, XT, Qrs, Qv, Qgr, Qgs, Qgi, dt, speed, T, th, densityAir, p, P, t, irr, u, dGround, GH);
        sync();
        launch("setTempsAtGroundGPU", ZX, XT, th, T, p, P, dtS);
        sync();
        diffuse(th, 0, dtS);
        nsub[0] = advect(th, isenT, Bounds{CUSTOM, CUSTOM, CUSTOM}, dtS);
        launch("buoyancyGPU", T16(), B16(), v, neigh, th, Qv, Qr, Qs, Qi, isenT, isenQv, p, P, stor0, 1.0f,
               Bounds{DIRICHLET, DIRICHLET, DIRICHLET}, Bounds{DIRICHLET, DIRICHLET, DIRICHLET}, dtS);
        sync();
        diffuse(u, 2, dtS);
        diffuse(v, 3, dtS);
        diffuse(w, 4, dtS);
        nsub[1] = advect(u, defU, Bounds{CUSTOM, CUSTOM, DIRICHLET}, dtS);
        zero(dummy, Y * 4);
        nsub[2] = advect(v, dummy, Bounds{DIRICHLET, DIRICHLET, DIRICHLET}, dtS);
        nsub[3] = advect(w, defW, Bounds{CUSTOM, CUSTOM, DIRICHLET}, dtS);
        launch("initDensity", YX, XT, densityAir, th, p, Qv, P);
        sync();
        copy(oldDensityAir, densityAir, N * 4);
        project(dtS);
        launch("calculateNewPressure", YX, XT, p, densityAir, th, Qv, P);
        sync();
        const Bounds bm{DIRICHLET, DIRICHLET, DIRICHLET};
        diffuse(Qv, 1, dtS);
        nsub[4] = advect(Qv, isenQv, Bounds{CUSTOM, CUSTOM, CUSTOM}, dtS);
        diffuse(Qw, 5, dtS);
        nsub[5] = advect(Qw, dummy, bm, dtS);
        diffuse(Qc, 5, dtS);
        nsub[6] = advect(Qc, dummy, bm, dtS);
        diffuse(Qr, 5, dtS);
        precip(Qr, 0, dtS);
        nsub[7] = advect(Qr, dummy, bm, dtS);
        diffuse(Qs, 5, dtS);
        precip(Qs, 1, dtS);
        nsub[8] = advect(Qs, dummy, bm, dtS);
        diffuse(Qi, 5, dtS);
        precip(Qi, 2, dtS);
        nsub[9] = advect(Qi, dummy, bm, dtS);
        // microPhysicsSkyGPU :568-595 (graph region off)
        zero(microRes, 33 * 4);
        const bool graph = false;
        const I3 mn{0, 0, 0}, mx{0, 0, 0};
        launch("calculateEnvMicroPhysicsGPU", YX, XT, Qv, Qw, Qc, Qr, Qs, Qi, dt, speed, th, densityAir, p, GH, P, condens, depos, freeze, graph,
               mn, mx, microRes);
        sync();
        launch("addHeatGPU", YX, XT, Qv, th, condens, depos, freeze);
        sync();
        time_ += speed * dt * float(!pause);
        if (time_ > 86400.0f) time_ = 0.0f;
    }
};

}  // namespace

extern "C" {

typedef struct {
    void *th, *qv, *qw, *qc, *qr, *qs, *qi, *u, *v, *w, *p, *rho;
    void *Qrs, *Qgr, *Qgs, *Qgi, *Pg, *tg, *Tg;
    void *isenT, *isenQv, *defU, *defW;
    int32_t* gh;
    double sim_time;
    int day;
    float longitude, sun;
    int pause;
} rh_state;

const char* rh_last_error(void) { return g_err.c_str(); }

namespace {

// Allocates environmentGPU's buffers, uploads the state and the kernels' constants and builds the
// Neigh records (computeNeighbourGPU), as environmentGPU::environmentGPU and init do.
void open_session(H& h, const char* cubin, int X, int Y, int Z, float vox, const rh_state* st, float pcg_tol, int pcg_max) {
    h.X = X; h.Y = Y; h.Z = Z; h.VOX = vox;
    h.N = size_t(X) * Y * Z;
    h.NG = size_t(X) * Z;
    h.pcg_tol = pcg_tol;
    h.pcg_max = pcg_max;
    CUcontext ctx = nullptr;
    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CK(cuModuleLoad(&h.mod, cubin));
    unsigned int nf = 0;
    CK(cuModuleGetFunctionCount(&nf, h.mod));
    std::vector<CUfunction> fs(nf);
    CK(cuModuleEnumerateFunctions(fs.data(), nf, h.mod));
    for (auto f : fs) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, f));
        h.fns.push_back({name, f});
    }
    // compile-time grid of the cubin must match
    CUdeviceptr gsym;
    size_t gsz = 0;
    CK(cuModuleGetGlobal(&gsym, &gsz, h.mod, "GHeight"));
    if (gsz != h.NG * 4) { g_err = "cubin grid size does not match"; throw 1; }
    const size_t N = h.N, NG = h.NG;
    CUdeviceptr* sky[] = {&h.Qv, &h.Qw, &h.Qc, &h.Qr, &h.Qs, &h.Qi, &h.th, &h.u, &h.v, &h.w, &h.p, &h.arr, &h.out, &h.density,
                          &h.densityAir, &h.oldDensityAir, &h.condens, &h.depos, &h.freeze, &h.stor0, &h.stor1, &h.stor2, &h.precon};
    for (auto* d : sky) *d = h.alloc(N * 4);
    h.A = h.alloc(N * 16);
    h.neigh = h.alloc(N * 12);
    CUdeviceptr* gr[] = {&h.Qrs, &h.Qgr, &h.Qgs, &h.Qgi, &h.P, &h.t, &h.T, &h.dGround, &h.dGround2, &h.GH};
    for (auto* d : gr) *d = h.alloc(NG * 4);
    CUdeviceptr* col[] = {&h.isenT, &h.isenQv, &h.defU, &h.defW, &h.dummy, &h.dummySky2};
    for (auto* d : col) *d = h.alloc(size_t(Y) * 4);
    h.microRes = h.alloc(33 * 4);
    h.single0 = h.alloc(4);
    h.sigma0 = h.alloc(4);
    h.sigma1 = h.alloc(4);
    auto up = [&](CUdeviceptr d, const void* s, size_t b) { CK(cuMemcpyHtoD(d, s, b)); };
    up(h.th, st->th, N * 4); up(h.Qv, st->qv, N * 4); up(h.Qw, st->qw, N * 4); up(h.Qc, st->qc, N * 4);
    up(h.Qr, st->qr, N * 4); up(h.Qs, st->qs, N * 4); up(h.Qi, st->qi, N * 4); up(h.u, st->u, N * 4);
    up(h.v, st->v, N * 4); up(h.w, st->w, N * 4); up(h.p, st->p, N * 4); up(h.densityAir, st->rho, N * 4);
    up(h.Qrs, st->Qrs, NG * 4); up(h.Qgr, st->Qgr, NG * 4); up(h.Qgs, st->Qgs, NG * 4); up(h.Qgi, st->Qgi, NG * 4);
    up(h.P, st->Pg, NG * 4); up(h.t, st->tg, NG * 4); up(h.T, st->Tg, NG * 4); up(h.GH, st->gh, NG * 4);
    up(h.isenT, st->isenT, Y * 4); up(h.isenQv, st->isenQv, Y * 4); up(h.defU, st->defU, Y * 4); up(h.defW, st->defW, Y * 4);
    // initKernelSky (Game/kernelSky.cu:23-38) and initGammasMicroPhysics (Game/microPhysics.cu:31-61)
    auto setsym = [&](const char* nm, const void* src, size_t b) {
        CUdeviceptr d;
        size_t sz;
        CK(cuModuleGetGlobal(&d, &sz, h.mod, nm));
        if (sz != b) { g_err = std::string("symbol size mismatch ") + nm; throw 1; }
        CK(cuMemcpyHtoD(d, src, b));
    };
    setsym("GHeight", st->gh, NG * 4);
    setsym("defaultVelX", st->defU, Y * 4);
    setsym("defaultVelZ", st->defW, Y * 4);
    const float b = 0.8f, d = 0.25f;
    const float gR = tgammaf(4.0f + b), gS = tgammaf(4.0f + d);
    setsym("gammaR", &gR, 4); setsym("gammaS", &gS, 4); setsym("gammaI", &gS, 4);
    const float m_gR = tgammaf(3 + b), m_gER = tgammaf((b + 5.0f) / 2.0f), m_gS = tgammaf(3 + d), m_gRC = tgammaf(6 + b);
    const float m_gSS = tgammaf((d + 5.0f) / 2.0f), m_gI = tgammaf(3.5f), m_gRI = tgammaf(2.75f);
    setsym("m_gammaR", &m_gR, 4); setsym("m_gammaER", &m_gER, 4); setsym("m_gammaS", &m_gS, 4); setsym("m_gammaRC", &m_gRC, 4);
    setsym("m_gammaSS", &m_gSS, 4); setsym("m_gammaI", &m_gI, 4); setsym("m_gammaRI", &m_gRI, 4);
    setsym("m_gammaQr", &gR, 4); setsym("m_gammaQs", &gS, 4); setsym("m_gammaQi", &gS, 4);
    h.launch("computeNeighbourGPU", Dim{unsigned(Y), 1, 1}, Dim{unsigned(X), 1, 1}, h.neigh);
    h.sync();
    h.time_ = float(st->sim_time);
    h.day = st->day; h.lon = st->longitude; h.sun = st->sun; h.pause = st->pause;
}

void read_back(H& h, rh_state* st) {
    const size_t N = h.N, NG = h.NG;
    auto down = [&](void* dst, CUdeviceptr s, size_t bb) { CK(cuMemcpyDtoH(dst, s, bb)); };
    down(st->th, h.th, N * 4); down(st->qv, h.Qv, N * 4); down(st->qw, h.Qw, N * 4); down(st->qc, h.Qc, N * 4);
    down(st->qr, h.Qr, N * 4); down(st->qs, h.Qs, N * 4); down(st->qi, h.Qi, N * 4); down(st->u, h.u, N * 4);
    down(st->v, h.v, N * 4); down(st->w, h.w, N * 4); down(st->p, h.p, N * 4); down(st->rho, h.densityAir, N * 4);
    down(st->Qrs, h.Qrs, NG * 4); down(st->Qgr, h.Qgr, NG * 4); down(st->Qgs, h.Qgs, NG * 4); down(st->Qgi, h.Qgi, NG * 4);
    down(st->tg, h.t, NG * 4); down(st->Tg, h.T, NG * 4);
    st->sim_time = h.time_;
}

void close_session(H& h) {
    CUdeviceptr all[] = {h.Qv, h.Qw, h.Qc, h.Qr, h.Qs, h.Qi, h.th, h.u, h.v, h.w, h.p, h.arr, h.out, h.density, h.densityAir,
                         h.oldDensityAir, h.condens, h.depos, h.freeze, h.stor0, h.stor1, h.stor2, h.precon, h.A, h.neigh,
                         h.Qrs, h.Qgr, h.Qgs, h.Qgi, h.P, h.t, h.T, h.dGround, h.dGround2, h.GH, h.isenT, h.isenQv, h.defU,
                         h.defW, h.dummy, h.dummySky2, h.microRes, h.single0, h.sigma0, h.sigma1};
    for (auto d : all)
        if (d) cuMemFree(d);
    if (h.mod) cuModuleUnload(h.mod);
    h.mod = nullptr;
}

}  // namespace

// Runs nsteps reference steps from the given state (float32 arrays, oracle layout) and writes
// the state back. pcg_iters[step] and nsub[step*10+i] receive the per-step diagnostics.
int rh_run(const char* cubin, int X, int Y, int Z, float vox, rh_state* st, float dt, float speed, int nsteps, float pcg_tol,
           int pcg_max, int* pcg_iters, int* nsub) {
    H h;
    try {
        open_session(h, cubin, X, Y, Z, vox, st, pcg_tol, pcg_max);
        for (int s = 0; s < nsteps; ++s) {
            h.step(dt, speed, nsub + 10 * s);
            pcg_iters[s] = h.last_iters;
        }
        read_back(h, st);
    } catch (...) {
        close_session(h);
        return 1;
    }
    close_session(h);
    return 0;
}

// Runs one stage of updateGPU alone from the given state, with the stage numbering of the
// library's skt_run_stage: 0 diffuseGPU (arg = type 0..5 on theta, Qv, u, v, w, Qw), 1
// advectPPMWGPU (arg 0..5 on theta, u, v, w, Qv, Qw with their bounds and default columns), 2
// buoyancyGPU, 3 initDensity + pressureProject, 4 microphysics and addHeatGPU (dt and speed
// apart), 5 advectPrecip (arg 0..2 on Qr, Qs, Qi), 6 the ground kernels through
// setTempsAtGroundGPU (dt and speed apart). dt is dt*speed for the other stages.
// diag[0] = PCG iterations, diag[1] = Courant substeps.
int rh_stage(const char* cubin, int X, int Y, int Z, float vox, rh_state* st, int stage, int arg, float dt, float speed,
             float pcg_tol, int pcg_max, int* diag) {
    H h;
    try {
        open_session(h, cubin, X, Y, Z, vox, st, pcg_tol, pcg_max);
        const Dim YX{unsigned(Y), 1, 1}, XT{unsigned(X), 1, 1}, ZX{unsigned(Z), 1, 1};
        diag[0] = 0;
        diag[1] = 0;
        switch (stage) {
            case 0: {
                CUdeviceptr f[6] = {h.th, h.Qv, h.u, h.v, h.w, h.Qw};
                if (arg < 0 || arg > 5) { g_err = "diffuse type"; throw 1; }
                h.diffuse(f[arg], arg, dt);
                break;
            }
            case 1: {
                if (arg < 0 || arg > 5) { g_err = "advect field"; throw 1; }
                h.zero(h.dummy, size_t(Y) * 4);
                CUdeviceptr f[6] = {h.th, h.u, h.v, h.w, h.Qv, h.Qw};
                CUdeviceptr df[6] = {h.isenT, h.defU, h.dummy, h.defW, h.isenQv, h.dummy};
                const Bounds bb[6] = {{CUSTOM, CUSTOM, CUSTOM}, {CUSTOM, CUSTOM, DIRICHLET}, {DIRICHLET, DIRICHLET, DIRICHLET},
                                      {CUSTOM, CUSTOM, DIRICHLET}, {CUSTOM, CUSTOM, CUSTOM}, {DIRICHLET, DIRICHLET, DIRICHLET}};
                diag[1] = h.advect(f[arg], df[arg], bb[arg], dt);
                break;
            }
            case 2:
                h.launch("buoyancyGPU", h.T16(), h.B16(), h.v, h.neigh, h.th, h.Qv, h.Qr, h.Qs, h.Qi, h.isenT, h.isenQv, h.p, h.P,
                         h.stor0, 1.0f, Bounds{DIRICHLET, DIRICHLET, DIRICHLET}, Bounds{DIRICHLET, DIRICHLET, DIRICHLET}, dt);
                h.sync();
                break;
            case 3:
                h.launch("initDensity", YX, XT, h.densityAir, h.th, h.p, h.Qv, h.P);
                h.sync();
                h.copy(h.oldDensityAir, h.densityAir, h.N * 4);
                h.project(dt);
                diag[0] = h.last_iters;
                break;
            case 4:
                h.zero(h.microRes, 33 * 4);
                h.launch("calculateEnvMicroPhysicsGPU", YX, XT, h.Qv, h.Qw, h.Qc, h.Qr, h.Qs, h.Qi, dt, speed, h.th, h.densityAir, h.p,
                         h.GH, h.P, h.condens, h.depos, h.freeze, false, I3{0, 0, 0}, I3{0, 0, 0}, h.microRes);
                h.sync();
                h.launch("addHeatGPU", YX, XT, h.Qv, h.th, h.condens, h.depos, h.freeze);
                h.sync();
                break;
            case 5: {
                if (arg < 0 || arg > 2) { g_err = "precip type"; throw 1; }
                CUdeviceptr f[3] = {h.Qr, h.Qs, h.Qi};
                h.precip(f[arg], arg, dt);
                break;
            }
            case 6: {
                const float dtS = dt * speed, irr = h.irradiance();
                h.launch("advectGroundWaterGPU", Dim{unsigned((X + 15) / 16), unsigned((Z + 15) / 16), 1},
                         Dim{unsigned(X < 16 ? X : 16), unsigned(Z < 16 ? Z : 16), 1}, h.Qrs, h.Qgr, dt, speed);
                h.sync();
                h.launch("calculateCloudCoverGPU", ZX, XT, h.dGround, h.Qc, h.Qw, h.GH);
                h.sync();
                h.launch("calculateGroundTempGPU", ZX, XT, h.T, dtS, irr, h.dGround);
                h.sync();
                h.launch("calculatePrecipHittingGroundMicroPhysicsGPU", ZX, XT, h.Qv, h.Qr, h.Qs, h.Qi, h.Qgr, h.Qgs, h.Qgi, dt, speed, h.T,
                         h.th, h.densityAir, h.p, h.P, h.u, h.GH);
                h.launch("calculateGroundMicroPhysicsGPU", ZX, XT, h.Qrs, h.Qv, h.Qgr, h.Qgs, h.Qgi, dt, speed, h.T, h.th, h.densityAir,
                         h.p, h.P, h.t, irr, h.u, h.dGround, h.GH);
                h.sync();
                h.launch("setTempsAtGroundGPU", ZX, XT, h.th, h.T, h.p, h.P, dtS);
                h.sync();
                break;
            }
            default: g_err = "unknown stage"; throw 1;
        }
        read_back(h, st);
    } catch (...) {
        close_session(h);
        return 1;
    }
    close_session(h);
    return 0;
}

// The Neigh records computeNeighbourGPU (Game/kernelSky.cu:1284-1316) builds for the state's
// heightfield: 12 bytes per cell (Game/config.h:24-38: left, right, up, down, forward,
// backward, each {bool outside, envType type}), cell order idx = x + y*X + z*X*Y.
int rh_neighbours(const char* cubin, int X, int Y, int Z, float vox, rh_state* st, uint8_t* out) {
    H h;
    try {
        open_session(h, cubin, X, Y, Z, vox, st, 1e-5f, 1);
        CK(cuMemcpyDtoH(out, h.neigh, h.N * 12));
    } catch (...) {
        close_session(h);
        return 1;
    }
    close_session(h);
    return 0;
}

}  // extern "C"
