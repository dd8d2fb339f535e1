// ORACLE — test infrastructure only (tests/, the smoke check and bench.py's CPU baseline).
// The product library never links, includes or calls this file.
//
// CPU restatement of skewTCloudSim's per-timestep 3D atmosphere solver, following
// Game/environment.cu:249-987 (init, updateGPU, diffuse, advect, project), Game/kernelSky.cu,
// Game/kernelGround.cu, Game/kernelMaths.cu and Game/microPhysics.cu. Templated on float (the
// reference's FP32 arithmetic) and double (the FP64 oracle of the same method). Every grid
// loop is written cell by cell; the boundary handling of the reference (Neigh records plus
// fillNeighbourData / fillSharedNeigh / getValueExtra*) is restated as one ghost-value rule,
// see ghost() below.
//
// Semantics switch: REFERENCE reproduces the reference's quirks (char-truncated lower PCG
// coefficients, the accumulating PCG denominator, the signed max residual, the early return in
// resetVelPressProj); TEXTBOOK removes them.
#include "skt_oracle_physics.hpp"

#include <cstdint>
#include <cstring>
#include <vector>
#include <cstdio>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace skt_oracle {

enum BC { NEUMANN = 0, DIRICHLET = 1, CUSTOM = 2 };
struct Bounds { BC sides, ground; };

struct Grid {
    int X, Y, Z;  // Y is vertical, idx = x + y*X + z*X*Y (Game/utils.cuh:8)
    const int32_t* gh;
    int64_t n() const { return int64_t(X) * Y * Z; }
    int64_t id(int x, int y, int z) const { return int64_t(x) + int64_t(y) * X + int64_t(z) * X * Y; }
    bool inside(int x, int y, int z) const { return x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z; }
    bool ground(int x, int y, int z) const { return y <= gh[x + z * X]; }  // Game/kernelSky.cu:1709
};

template <class T> inline T cond(BC bc, T own, T custom) {  // fillDataBoundCon, Game/kernelSky.cu:1876
    return bc == NEUMANN ? own : (bc == DIRICHLET ? T(0) : custom);
}

// Ghost value of field q at a possibly out-of-domain or ground position, as every sky-cell
// stencil of the reference sees it (fillNeighbourData :1844, fillSharedNeigh :1765,
// getValueExtraDirShared :1894, getValueExtraForward :1983):
//  * outside the domain: the boundary condition of the nearest in-domain (clamped) cell, with that
//    cell's value and the default column at that cell's height. The condition is the "sides" one
//    unless the clamped cell is ground (then "ground"), because Neigh marks an outside neighbour
//    GROUND only when the current cell is ground (:1299-1314) and fillNeighbourData never passes
//    up=true, so the top boundary also uses "sides".
//  * an in-domain ground cell: the "ground" condition with the default at that cell's height.
//  * an in-domain sky cell: its value.
template <class T> inline T ghost(const Grid& g, const T* q, int x, int y, int z, Bounds b, const T* def) {
    if (!g.inside(x, y, z)) {
        int xc = std::min(std::max(x, 0), g.X - 1), yc = std::min(std::max(y, 0), g.Y - 1), zc = std::min(std::max(z, 0), g.Z - 1);
        T d = def ? def[yc] : T(0);
        BC bc = g.ground(xc, yc, zc) ? b.ground : b.sides;
        return cond(bc, q[g.id(xc, yc, zc)], d);
    }
    if (g.ground(x, y, z)) return cond(b.ground, q[g.id(x, y, z)], def ? def[y] : T(0));
    return q[g.id(x, y, z)];
}

// Face value via fillNeighbourData with an explicit custom value, seen from sky cell (x,y,z).
template <class T> inline T face_nb(const Grid& g, const T* q, int x, int y, int z, int dx, int dy, int dz, Bounds b, T custom) {
    const int xn = x + dx, yn = y + dy, zn = z + dz;
    const T own = q[g.id(x, y, z)];
    if (!g.inside(xn, yn, zn)) return cond(b.sides, own, custom);
    if (g.ground(xn, yn, zn)) return cond(b.ground, own, custom);
    return q[g.id(xn, yn, zn)];
}

struct Config {
    int semantics;  // 0 reference, 1 textbook
    int diffuse_sweeps;
    float pcg_tol;
    int pcg_max_iter;
    int max_substeps;
    float voxel;
};

template <class T> struct State {
    T *th, *qv, *qw, *qc, *qr, *qs, *qi, *u, *v, *w, *p, *rho;   // sky, X*Y*Z
    T *Qrs, *Qgr, *Qgs, *Qgi, *Pg, *tg, *Tg;                      // ground, X*Z
    T *isenT, *isenQv, *defU, *defW;                              // columns, Y
    int32_t* gh;
    double sim_time;
    int day;
    float longitude, sun;
    int pause;
};

struct Diag {
    int pcg_iters;
    double pcg_residual;
    int nsub[10];
    int converged;
};

// ---------------------------------------------------------------------------------------------
// Diffusion, Game/environment.cu:597-673 + diffuseRedBlack Game/kernelSky.cu:43-115.
// Both colours read the same input, so one "sweep" (red + black launch) is a Jacobi sweep over
// all sky cells; LOOPS=10 double sweeps (input->output, output->input) = 20 sweeps.
// ---------------------------------------------------------------------------------------------
template <class T>
void diffuse(const Grid& g, const Config& cfg, State<T>& s, T* f, int type, T dt) {
    const T* def = nullptr;
    Bounds b{NEUMANN, DIRICHLET};
    std::vector<T> zero(g.Y, T(0));
    switch (type) {
        case 0: def = s.isenT; b = {CUSTOM, CUSTOM}; break;
        case 1: def = s.isenQv; b = {CUSTOM, DIRICHLET}; break;
        case 2: def = s.defU; b = {CUSTOM, DIRICHLET}; break;
        case 3: def = nullptr; b = {NEUMANN, DIRICHLET}; break;
        case 4: def = s.defW; b = {CUSTOM, DIRICHLET}; break;
        default: def = zero.data(); b = {NEUMANN, DIRICHLET}; break;
    }
    const T vox = T(cfg.voxel);
    const T k = T(0.005) * dt / (vox * vox);
    std::vector<T> a(f, f + g.n()), o(f, f + g.n());
    // theta's ground-face value, potentialTempGPU(groundT-273.15, p_cell, groundP)+273.15 (:95-100)
    auto thg = [&](int64_t idx, int idxg) {
        return potentialTemp(s.Tg[idxg] - T(273.15), s.p[idx], s.Pg[idxg]) + T(273.15);
    };
    const int BX = std::min(16, g.X);
    auto isGroundLevel = [&](int x, int z) {  // Q5, Game/kernelSky.cu:1684-1694 under the T16 launch
        int gi = (x % BX) + z * g.Z;
        if (gi >= g.X * g.Z) gi = g.X * g.Z - 1;
        return (x / BX) == g.gh[gi] + 1;
    };
    const int sweeps = cfg.diffuse_sweeps;
    for (int sw = 0; sw < sweeps; ++sw) {
        const std::vector<T>& in = (sw % 2 == 0) ? a : o;
        std::vector<T>& out = (sw % 2 == 0) ? o : a;
        const T* q = in.data();
#pragma omp parallel for collapse(2) schedule(static)
        for (int z = 0; z < g.Z; ++z)
            for (int y = 0; y < g.Y; ++y)
                for (int x = 0; x < g.X; ++x) {
                    if (g.ground(x, y, z)) continue;
                    const int64_t idx = g.id(x, y, z);
                    T l = ghost(g, q, x - 1, y, z, b, def), r = ghost(g, q, x + 1, y, z, b, def);
                    T d = ghost(g, q, x, y - 1, z, b, def), u = ghost(g, q, x, y + 1, z, b, def);
                    T fw = ghost(g, q, x, y, z + 1, b, def), bw = ghost(g, q, x, y, z - 1, b, def);
                    if (type == 0) {
                        const int idxG = x + z * g.X;
                        const int idxGL = x > 0 ? idxG - 1 : idxG;
                        const int idxGR = x + 1 < g.X ? idxG + 1 : idxG;
                        const int idxGF = z + g.X < g.Z ? idxG + g.X : idxG;  // reference compares z + X < Z
                        const int idxGB = z > 0 ? idxG - g.X : idxG;
                        const bool gl = g.inside(x - 1, y, z) && g.ground(x - 1, y, z);
                        const bool gr = g.inside(x + 1, y, z) && g.ground(x + 1, y, z);
                        const bool gd = y > 0 && g.ground(x, y - 1, z);
                        const bool gf = g.inside(x, y, z + 1) && g.ground(x, y, z + 1);
                        const bool gb = g.inside(x, y, z - 1) && g.ground(x, y, z - 1);
                        if (gl && isGroundLevel(x, z)) l = thg(idx, idxGL);
                        if (gr && isGroundLevel(x, z)) r = thg(idx, idxGR);
                        if (gd) d = thg(idx, idxG);
                        if (gf && isGroundLevel(x, z)) fw = thg(idx, idxGF);
                        if (gb && isGroundLevel(x, z)) bw = thg(idx, idxGB);
                    }
                    out[idx] = (q[idx] + k * (l + r + u + d + fw + bw)) / (1 + 6 * k);
                }
    }
    const std::vector<T>& res = (sweeps % 2 == 0) ? a : o;
    std::memcpy(f, res.data(), sizeof(T) * g.n());
}

// ---------------------------------------------------------------------------------------------
// PPM advection, advectPPMFlux Game/kernelSky.cu:270-366
// ---------------------------------------------------------------------------------------------
template <class T> inline T ppm_flux(T veli, T vL, T vC, T vR, T dt, T vox) {
    T C = veli * dt / vox;
    C = C > T(1) ? T(1) : (C < T(-1) ? T(-1) : C);
    const T qMin = Fmin(vL, Fmin(vC, vR));
    const T qMax = Fmax(vL, Fmax(vC, vR));
    T s = 0;
    const T dl = vC - vL, dr = vR - vC;
    if (dl * dr > T(0)) {
        const T db = vR - vL;
        const T lim = Fmin(T(0.5) * Fabs(db), Fmin(Fabs(dr), Fabs(dl)));
        s = db >= T(0) ? lim : -lim;
    }
    const T qLS = vC - T(0.5) * s, qRS = vC + T(0.5) * s;
    T B = 1;
    if (qRS > qMax) { const T den = qRS - vC; if (den > T(1e-16)) B = Fmin(B, (qMax - vC) / den); }
    if (qLS < qMin) { const T den = vC - qLS; if (den > T(1e-16)) B = Fmin(B, (vC - qMin) / den); }
    T qR = vC + B * (qRS - vC);
    T qL = vC + B * (qLS - vC);
    if ((qR - vC) * (vC - qL) <= T(0)) { qR = qL = vC; }
    T qq;
    if (C > T(0)) qq = qR + C * (-qL - 2 * qR + 3 * vC) + C * C * (qL + qR - 2 * vC);
    else qq = qR + C * (-2 * qL - qR + 3 * vC) + C * C * (qL + qR - 2 * vC);
    return veli * qq;
}

// One directional pass of advectPPMX/Y/Z (Game/kernelSky.cu:368-574) on q and on the density
// companion (a field of ones advected with the same bounds and custom value 1), then the
// division divideValues (Game/kernelMaths.cu:38). axis 0=x (vel u, face custom defU[y]),
// 1=y (vel v, custom 0), 2=z (vel w, custom defW[y]). Writes sky cells of out only.
template <class T>
void ppm_pass(const Grid& g, const State<T>& s, int axis, const T* q, T* out, const T* def, Bounds b, const T* vel, T dt, T vox) {
    const int ax = axis == 0, ay = axis == 1, az = axis == 2;
    std::vector<T> ones(g.Y, T(1));
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y) {
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                auto G = [&](int o) { return ghost(g, q, x + o * ax, y + o * ay, z + o * az, b, def); };
                // density companion: ones everywhere, ghost with custom 1 (m_dummyArraySky2)
                auto G1 = [&](int o) {
                    const int xn = x + o * ax, yn = y + o * ay, zn = z + o * az;
                    if (!g.inside(xn, yn, zn)) {
                        int xc = std::min(std::max(xn, 0), g.X - 1), yc = std::min(std::max(yn, 0), g.Y - 1), zc = std::min(std::max(zn, 0), g.Z - 1);
                        return cond(g.ground(xc, yc, zc) ? b.ground : b.sides, T(1), T(1));
                    }
                    if (g.ground(xn, yn, zn)) return cond(b.ground, T(1), T(1));
                    return T(1);
                };
                const T custom = axis == 0 ? s.defU[y] : (axis == 1 ? T(0) : s.defW[y]);
                const T vc = vel[idx];
                const T vm = face_nb(g, vel, x, y, z, -ax, -ay, -az, b, custom);
                T fq[2], fr[2];
                for (int comp = 0; comp < 2; ++comp) {
                    auto V = [&](int o) { return comp == 0 ? G(o) : G1(o); };
                    const T c0 = comp == 0 ? q[idx] : T(1);
                    // +face: upwind triple, mirrored when the face velocity is negative
                    T L, Cc, R;
                    if (vc >= T(0)) { L = V(-1); Cc = c0; R = V(1); }
                    else { L = V(2); Cc = V(1); R = c0; }
                    const T fplus = ppm_flux(vc, L, Cc, R, dt, vox);
                    if (vm < T(0)) { L = V(1); Cc = c0; R = V(-1); }
                    else { L = V(-2); Cc = V(-1); R = c0; }
                    const T fminus = ppm_flux(vm, L, Cc, R, dt, vox);
                    (comp == 0 ? fq[0] : fr[0]) = fplus;
                    (comp == 0 ? fq[1] : fr[1]) = fminus;
                }
                const T nq = q[idx] - (dt / vox) * (fq[0] - fq[1]);
                const T nr = T(1) - (dt / vox) * (fr[0] - fr[1]);
                out[idx] = nq / nr;
            }
        }
}

// Max "velocity" used for the Courant substeps and the PCG stop test: getMaxDivergence
// (Game/kernelSky.cu:910-953). REFERENCE: |a| at z=0, signed a for z>=1 (Q4), floored at 0 by
// the integer atomicMax; TEXTBOOK: max |a|.
template <class T> double quirky_max(const Grid& g, const T* a, bool reference) {
    double m = 0;
#pragma omp parallel for schedule(static) reduction(max : m)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const T v = a[g.id(x, y, z)];
                const T c = (!reference || z == 0) ? Fabs(v) : v;
                if (c > m) m = c;
            }
    return m;
}

// advectPPMWGPU, Game/environment.cu:692-824. Returns the substep count.
template <class T>
int advect_field(const Grid& g, const Config& cfg, State<T>& s, T* f, const T* def, Bounds b, T dt) {
    const bool ref = cfg.semantics == 0;
    double mv = std::max(quirky_max(g, s.u, ref), std::max(quirky_max(g, s.v, ref), quirky_max(g, s.w, ref)));
    T maxVel = T(mv);
    const T vox = T(cfg.voxel);
    const T C = maxVel * dt / vox;
    const T MAXSUB = T(cfg.max_substeps);
    const int sub = int(Fmin(Ceil(Fabs(C)), MAXSUB));
    const T dts = dt / T(sub);
    std::vector<T> o(g.n(), T(0));
    // A = the field array itself, O = scratch; passes alternate A->O, O->A. The velocity arrays
    // are read at pass start, so when f is itself a velocity component its pass-2/4 velocity is
    // the stale content of A (the reference's behaviour minus its in-kernel race).
    std::vector<T> a_snapshot;
    for (int i = 0; i < sub; ++i) {
        auto velp = [&](int axis) -> const T* { return axis == 0 ? s.u : (axis == 1 ? s.v : s.w); };
        // pass 1: X half, A -> O
        ppm_pass(g, s, 0, f, o.data(), def, b, velp(0), dts * T(0.5), vox);
        // pass 2: Y half, O -> A; velocity snapshot taken before A is overwritten
        {
            const T* vy = velp(1);
            std::vector<T> vsnap;
            if (vy == f) { vsnap.assign(f, f + g.n()); vy = vsnap.data(); }
            std::vector<T> tmp(f, f + g.n());
            ppm_pass(g, s, 1, o.data(), tmp.data(), def, b, vy, dts * T(0.5), vox);
            std::memcpy(f, tmp.data(), sizeof(T) * g.n());
        }
        // pass 3: Z full, A -> O
        ppm_pass(g, s, 2, f, o.data(), def, b, velp(2), dts, vox);
        // pass 4: Y half, O -> A
        {
            const T* vy = velp(1);
            std::vector<T> vsnap;
            if (vy == f) { vsnap.assign(f, f + g.n()); vy = vsnap.data(); }
            std::vector<T> tmp(f, f + g.n());
            ppm_pass(g, s, 1, o.data(), tmp.data(), def, b, vy, dts * T(0.5), vox);
            std::memcpy(f, tmp.data(), sizeof(T) * g.n());
        }
        // pass 5: X half, A -> O, then A = O
        ppm_pass(g, s, 0, f, o.data(), def, b, velp(0), dts * T(0.5), vox);
        for (int64_t c = 0; c < g.n(); ++c) {
            const int x = int(c % g.X), y = int((c / g.X) % g.Y), z = int(c / (int64_t(g.X) * g.Y));
            if (!g.ground(x, y, z)) f[c] = o[c];
        }
    }
    return sub;
}

// Sedimentation, advectPrecip Game/environment.cu:826-849 + advectPrecipGPU Game/kernelSky.cu:576-657
template <class T>
void advect_precip(const Grid& g, const Config& cfg, State<T>& s, T* q, int type, T dt, const Gammas<T>& G) {
    const T vox = T(cfg.voxel);
    const T maxVel = type == 0 ? T(5) : (type == 1 ? T(1) : T(8));
    const T C = maxVel * dt / vox;
    const int sub = int(Fmin(Ceil(Fabs(C)), T(cfg.max_substeps)));
    const T dts = dt / T(sub);
    const T kap = kappa<T>();
    for (int it = 0; it < sub; ++it) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int z = 0; z < g.Z; ++z)
            for (int x = 0; x < g.X; ++x) {
                std::vector<T> col(g.Y);
                for (int y = 0; y < g.Y; ++y) col[y] = q[g.id(x, y, z)];
                const int idxG = x + z * g.X;
                auto fall = [&](T Q, int64_t i) {
                    const T Tt = s.th[i] * Pow(s.p[i] / s.Pg[idxG], kap);
                    const T Tv = Tt * (T(0.608) * s.qv[i] + 1);
                    const T dens = s.p[i] * 100 / (K<T>::Rsd * Tv);
                    T UR, US, UI;
                    fallingVelocity(Q, Q, Q, dens, type, G.Qr, G.Qs, G.Qi, UR, US, UI);
                    return type == 0 ? UR : (type == 1 ? US : UI);
                };
                for (int y = 0; y < g.Y; ++y) {
                    if (g.ground(x, y, z)) continue;
                    const int64_t idx = g.id(x, y, z);
                    const bool up = y < g.Y - 1;
                    const T QC = col[y];
                    const T QU = up ? col[y + 1] : T(0);
                    const T fv = fall(QC, idx);
                    const T fvu = up ? fall(QU, idx + g.X) : T(0);
                    T val = q[idx];
                    val -= dts * Fmin((fv / vox) * QC, QC);
                    if (up) val += dts * Fmin((fvu / vox) * QU, QU);
                    q[idx] = val;
                }
            }
    }
}

// buoyancyGPU, Game/kernelSky.cu:1061-1247 (bounds DIRICHLET everywhere, Game/environment.cu:1056)
// dbg (optional): the velocity change of each sky cell, 0 where no neighbour is sky (the
// reference's buoyancyStor, shown as its second debug field)
template <class T> void buoyancy(const Grid& g, State<T>& s, T dt, T* dbg = nullptr) {
    const Bounds b{DIRICHLET, DIRICHLET};
    const T kap = kappa<T>();
    const T gg = K<T>::g;
    std::vector<T> v0(s.v, s.v + g.n());
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const T vel = v0[idx];
                const bool up = y < g.Y - 1;
                const bool down = y > 0 && !g.ground(x, y - 1, z);
                const T Pgs = s.Pg[x + z * g.X];
                const T psC = s.p[idx];
                const T psU = up ? s.p[idx + g.X] : psC;
                const T psD = down ? s.p[idx - g.X] : psC;
                auto valid = [&](int dx, int dz) { return g.inside(x + dx, y, z + dz) && !g.ground(x + dx, y, z + dz); };
                const bool l = valid(-1, 0), r = valid(1, 0), bb = valid(0, -1), f = valid(0, 1);
                const int nv = int(l) + int(r) + int(bb) + int(f);
                if (nv == 0) {
                    if (dbg) dbg[idx] = 0;
                    continue;
                }
                auto Q = [&](int dx, int dy, int dz) { return ghost(g, s.qv, x + dx, y + dy, z + dz, b, s.isenQv); };
                auto TH = [&](int dx, int dy, int dz) { return ghost(g, s.th, x + dx, y + dy, z + dz, b, s.isenT); };
                const T QP = s.qv[idx];
                const T Qenv = (Q(1, 0, 0) + Q(-1, 0, 0) + Q(0, 0, 1) + Q(0, 0, -1)) / T(nv);
                const T QenvUp = Q(0, 1, 0), QenvDown = Q(0, -1, 0);
                const T thc = s.th[idx];
                const T TDown = TH(0, -1, 0) * Pow(psD / Pgs, kap);
                const T Tc = thc * Pow(psC / Pgs, kap);
                const T TUp = TH(0, 1, 0) * Pow(psU / Pgs, kap);
                T Tad = thc, TadUp = thc, TadDown = thc;
                const T Tenv = (TH(1, 0, 0) + TH(-1, 0, 0) + TH(0, 0, 1) + TH(0, 0, -1)) / T(nv);
                const T TenvUp = TH(0, 1, 0), TenvDown = TH(0, -1, 0);
                if (down) {
                    if ((Tc < T(0) && QP >= wi(TDown - T(273.15), psD)) || QP >= ws(TDown - T(273.15), psD)) {
                        TadDown = Tc - MLR(Tc - T(273.15), psC) * (psC - psD);
                        TadDown = TadDown * Pow(Pgs / psD, kap);
                    }
                }
                if (up) {
                    if ((Tc < T(0) && QP >= wi(TUp - T(273.15), psU)) || QP >= ws(TUp - T(273.15), psU)) {
                        TadUp = MLR(Tc - T(273.15), psC) * (psU - psC) + Tc;
                        TadUp = TadUp * Pow(Pgs / psU, kap);
                    }
                }
                T B = 0, BUp = 0, BDown = 0;
                const T totalQ = s.qr[idx] + s.qs[idx] + s.qi[idx];
                if (down) {
                    const T VTP = TadDown * (T(1) + T(0.608) * QP), VTE = TenvDown * (T(1) + T(0.608) * QenvDown);
                    BDown = gg * ((VTP - VTE) / VTE) - totalQ * gg;
                }
                {
                    const T VTP = Tad * (T(1) + T(0.608) * QP), VTE = Tenv * (T(1) + T(0.608) * Qenv);
                    B = gg * ((VTP - VTE) / VTE) - totalQ * gg;
                }
                if (up) {
                    const T VTP = TadUp * (T(1) + T(0.608) * QP), VTE = TenvUp * (T(1) + T(0.608) * QenvUp);
                    BUp = gg * ((VTP - VTE) / VTE) - totalQ * gg;
                }
                T fin = B;
                if (vel > T(0)) fin = BUp;
                else if (vel < T(0)) fin = BDown;
                T change = fin * dt;
                if ((up && vel > T(0) && -change > vel) || (down && vel < T(0) && -change < vel)) change = -vel;
                if (dbg) dbg[idx] = change;
                s.v[idx] = vel + change;
            }
}

// initDensity Game/kernelSky.cu:1432-1452 (glm::pow on floats == powf)
template <class T> void init_density(const Grid& g, State<T>& s) {
    const T kap = kappa<T>();
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const T Tt = s.th[idx] * Pow(s.p[idx] / s.Pg[x + z * g.X], kap);
                const T Tv = Tt * (T(0.608) * s.qv[idx] + 1);
                s.rho[idx] = s.p[idx] * 100 / (K<T>::Rsd * Tv);
            }
}

// calculateNewPressure Game/kernelSky.cu:1454-1474
template <class T> void new_pressure(const Grid& g, State<T>& s) {
    const T kap = kappa<T>();
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const T Tt = s.th[idx] * Pow(s.p[idx] / s.Pg[x + z * g.X], kap);
                const T Tv = Tt * (T(0.608) * s.qv[idx] + 1);
                s.p[idx] = s.rho[idx] * K<T>::Rsd * Tv / T(100);
            }
}

// ---------------------------------------------------------------------------------------------
// Pressure projection, Game/environment.cu:851-987 and the kernels it calls.
// ---------------------------------------------------------------------------------------------
template <class T> struct Amat { std::vector<T> x, y, z, w; };

template <class T> inline T coef_of(T c, T n) {  // initAMatrix :1372
    return n == T(0) ? T(0) : -Fmax(T(1), T(1.225) / (T(2) / (T(1) / c + T(1) / n)));
}
template <class T> inline T char_trunc(T a) {  // (char) conversion of a float, Q3 (signed char)
    T t = a < T(0) ? Ceil(a) : std::floor(a);
    if (t < T(-128)) t = T(-128);
    if (t > T(127)) t = T(127);
    return t;
}

// The projection's linear system A p = r: resetVelPressProj on the winds, the matrix of
// initAMatrix and the divergence of calculateDivergenceGPU (r), as pressureProject sets them up.
template <class T>
void build_system(const Grid& g, const Config& cfg, State<T>& s, T dt, Amat<T>& A, std::vector<T>& r) {
    const bool ref = cfg.semantics == 0;
    const int64_t N = g.n();
    // resetVelPressProj :1648-1682 (REFERENCE: stop the column at the first ground z, Q8)
    for (int y = 0; y < g.Y; ++y)
        for (int x = 0; x < g.X; ++x)
            for (int z = 0; z < g.Z; ++z) {
                if (g.ground(x, y, z)) { if (ref) break; else continue; }
                const int64_t idx = g.id(x, y, z);
                if (y == g.Y - 1) s.v[idx] = 0;
                if (x == g.X - 1) s.u[idx] = s.defU[y];
                if (x + 1 < g.X && g.ground(x + 1, y, z)) s.u[idx] = 0;
                if (z == g.Z - 1) s.w[idx] = s.defW[y];
                if (z + 1 < g.Z && g.ground(x, y, z + 1)) s.w[idx] = 0;
            }
    // initAMatrix :1320-1393 with bounds {NEUMANN sides, DIRICHLET ground}
    const Bounds bA{NEUMANN, DIRICHLET};
    A.x.assign(N, 0); A.y.assign(N, 0); A.z.assign(N, 0); A.w.assign(N, 0);
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const T c = s.rho[idx];
                const T r = coef_of(c, ghost(g, s.rho, x + 1, y, z, bA, (const T*)nullptr));
                const T l = coef_of(c, ghost(g, s.rho, x - 1, y, z, bA, (const T*)nullptr));
                const T u = coef_of(c, ghost(g, s.rho, x, y + 1, z, bA, (const T*)nullptr));
                const T d = coef_of(c, ghost(g, s.rho, x, y - 1, z, bA, (const T*)nullptr));
                const T f = coef_of(c, ghost(g, s.rho, x, y, z + 1, bA, (const T*)nullptr));
                const T b = coef_of(c, ghost(g, s.rho, x, y, z - 1, bA, (const T*)nullptr));
                A.x[idx] = r; A.y[idx] = u; A.z[idx] = f;
                T w = 0; w -= r; w -= l; w -= u; w -= d; w -= f; w -= b;
                A.w[idx] = w;
            }
    // calculateDivergenceGPU :780-860; densities {NEUMANN sides, DIRICHLET ground}, velocities
    // m_boundsVelX = {CUSTOM sides, DIRICHLET ground}
    const Bounds bD{NEUMANN, DIRICHLET}, bV{CUSTOM, DIRICHLET};
    r.assign(N, 0);
    std::vector<T> oldrho(s.rho, s.rho + N);
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const T cur = s.rho[idx];
                const T ur = s.u[idx], ul = face_nb(g, s.u, x, y, z, -1, 0, 0, bV, s.defU[y]);
                const T uu = s.v[idx], ud = face_nb(g, s.v, x, y, z, 0, -1, 0, bV, T(0));
                const T uf = s.w[idx], ub = face_nb(g, s.w, x, y, z, 0, 0, -1, bV, s.defW[y]);
                auto hm = [&](T d) { return d == T(0) ? T(0) : T(2) / (T(1) / cur + T(1) / d); };
                const T dr = hm(ghost(g, s.rho, x + 1, y, z, bD, (const T*)nullptr));
                const T dl = hm(ghost(g, s.rho, x - 1, y, z, bD, (const T*)nullptr));
                const T du = hm(ghost(g, s.rho, x, y + 1, z, bD, (const T*)nullptr));
                const T dd = hm(ghost(g, s.rho, x, y - 1, z, bD, (const T*)nullptr));
                const T df = hm(ghost(g, s.rho, x, y, z + 1, bD, (const T*)nullptr));
                const T db = hm(ghost(g, s.rho, x, y, z - 1, bD, (const T*)nullptr));
                const T mfd = ((dr * ur - dl * ul) + (du * uu - dd * ud) + (df * uf - db * ub));
                const T dch = (cur - oldrho[idx]) / dt;
                r[idx] = mfd - dch;
            }
}

template <class T>
double project(const Grid& g, const Config& cfg, State<T>& s, T dt, Diag& dg) {
    const bool ref = cfg.semantics == 0;
    const int64_t N = g.n();
    Amat<T> A;
    std::vector<T> r;
    build_system(g, cfg, s, dt, A, r);
    std::vector<T> zv(N, 0), sv(N, 0), As(N, 0), pp(N, 0);
    // Jacobi preconditioner (initPrecon :1395) and the PCG loop (:898-987)
    auto precon = [&](int64_t i) { return A.w[i] == T(0) ? T(1) : T(1) / A.w[i]; };
    auto is_sky = [&](int64_t i, int& x, int& y, int& z) {
        x = int(i % g.X); y = int((i / g.X) % g.Y); z = int(i / (int64_t(g.X) * g.Y));
        return !g.ground(x, y, z);
    };
    // dot products over sky cells in double: kDotChunks fixed chunks summed in parallel, then the
    // chunk sums added in chunk order, so the result does not depend on the thread count
    constexpr int kDotChunks = 256;
    auto dot = [&](const std::vector<T>& a, const std::vector<T>& b) {
        double part[kDotChunks];
#pragma omp parallel for schedule(static)
        for (int ch = 0; ch < kDotChunks; ++ch) {
            const int64_t i0 = N * ch / kDotChunks, i1 = N * (ch + 1) / kDotChunks;
            double acc = 0;
            for (int64_t i = i0; i < i1; ++i) { int x, y, z; if (is_sky(i, x, y, z)) acc += double(a[i]) * double(b[i]); }
            part[ch] = acc;
        }
        double acc = 0;
        for (int ch = 0; ch < kDotChunks; ++ch) acc += part[ch];
        return acc;
    };
    auto applyA = [&](const std::vector<T>& in, std::vector<T>& out) {  // applyAGPU :719-778, ghost s = 0
#pragma omp parallel for collapse(2) schedule(static)
        for (int z = 0; z < g.Z; ++z)
            for (int y = 0; y < g.Y; ++y)
                for (int x = 0; x < g.X; ++x) {
                    const int64_t idx = g.id(x, y, z);
                    if (g.ground(x, y, z)) { out[idx] = 0; continue; }
                    auto S = [&](int dx, int dy, int dz) {
                        const int xn = x + dx, yn = y + dy, zn = z + dz;
                        if (!g.inside(xn, yn, zn) || g.ground(xn, yn, zn)) return T(0);
                        return in[g.id(xn, yn, zn)];
                    };
                    auto lower = [&](int dx, int dy, int dz, const std::vector<T>& arr) {
                        const int xn = x + dx, yn = y + dy, zn = z + dz;
                        if (!g.inside(xn, yn, zn) || g.ground(xn, yn, zn)) return T(0);
                        const T a = arr[g.id(xn, yn, zn)];
                        return ref ? char_trunc(a) : a;
                    };
                    const T l = S(-1, 0, 0), rr = S(1, 0, 0), d = S(0, -1, 0), u = S(0, 1, 0), f = S(0, 0, 1), b = S(0, 0, -1);
                    const T AL = lower(-1, 0, 0, A.x), AD = lower(0, -1, 0, A.y), AB = lower(0, 0, -1, A.z);
                    out[idx] = A.w[idx] * in[idx] + ((AL * l + AD * d + AB * b + A.x[idx] * rr + A.y[idx] * u + A.z[idx] * f));
                }
    };
    auto maxr = [&]() { return quirky_max(g, r.data(), ref); };
    double mr = maxr();
    dg.pcg_iters = 0;
    dg.converged = 1;
    double res = mr;
    if (mr != 0.0) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) { int x, y, z; zv[i] = is_sky(i, x, y, z) ? r[i] * precon(i) : T(0); }
        sv = zv;
        double sigma0 = dot(zv, r);
        double sigma1 = 0;
        dg.converged = 0;
        for (int it = 0; it < cfg.pcg_max_iter; ++it) {
            applyA(sv, As);
            const double sAs = dot(As, sv);
            sigma1 = ref ? sigma1 + sAs : sAs;  // Q1: the reference never clears sigma1 here
            const T alpha = T(sigma0 / sigma1);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; ++i) {
                int x, y, z;
                if (!is_sky(i, x, y, z)) continue;
                pp[i] += alpha * sv[i];
                r[i] -= alpha * As[i];
            }
            dg.pcg_iters = it + 1;
            mr = maxr();
            res = mr;
            if (mr <= double(T(cfg.pcg_tol))) { dg.converged = 1; break; }
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; ++i) { int x, y, z; zv[i] = is_sky(i, x, y, z) ? r[i] * precon(i) : T(0); }
            sigma1 = dot(zv, r);
            const T beta = T(sigma1 / sigma0);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; ++i) {
                int x, y, z;
                if (!is_sky(i, x, y, z)) continue;
                sv[i] = zv[i] + beta * sv[i];
            }
            sigma0 = sigma1;
        }
    }
    dg.pcg_residual = res;
    // updatePressure :1016, initDensity, applyPresProjGPU :862-908
    for (int64_t i = 0; i < N; ++i) { int x, y, z; if (is_sky(i, x, y, z)) s.p[i] -= pp[i] / T(100); }
    init_density(g, s);
    const Bounds bP{DIRICHLET, NEUMANN}, bD{NEUMANN, DIRICHLET};
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const T cp = pp[idx], cd = s.rho[idx];
                const T pr = face_nb(g, pp.data(), x, y, z, 1, 0, 0, bP, T(0));
                const T pu = face_nb(g, pp.data(), x, y, z, 0, 1, 0, bP, T(0));
                const T pf = face_nb(g, pp.data(), x, y, z, 0, 0, 1, bP, T(0));
                T dr = face_nb(g, s.rho, x, y, z, 1, 0, 0, bD, T(0));
                T du = face_nb(g, s.rho, x, y, z, 0, 1, 0, bD, T(0));
                T df = face_nb(g, s.rho, x, y, z, 0, 0, 1, bD, T(0));
                dr = dr == T(0) ? cd : T(2) / (T(1) / cd + T(1) / dr);
                du = du == T(0) ? cd : T(2) / (T(1) / cd + T(1) / du);
                df = df == T(0) ? cd : T(2) / (T(1) / cd + T(1) / df);
                s.u[idx] += (pr - cp) / dr;
                s.v[idx] += (pu - cp) / du;
                s.w[idx] += (pf - cp) / df;
            }
    return res;
}

// ---------------------------------------------------------------------------------------------
// Sky microphysics + latent heat: calculateEnvMicroPhysicsGPU Game/microPhysics.cu:1035-1354
// followed by addHeatGPU Game/kernelSky.cu:1249-1282 (both over sky cells).
// ---------------------------------------------------------------------------------------------
// Region-summed process amounts (Game/microPhysics.cu:1356-1413, the data graph): for the sky
// cells with lo <= (x, y, z) <= hi the 33 values of each cell after its update, PVCON and PVDEP
// split by sign into PVCON/PVVAP and PVDEP/PVSUB, PGWET times WTerm and PGDRY times (1 - WTerm),
// summed in double. Order: PVCON PVDEP PIMLT PIDW PIHOM PIACR PRACI PRAUT PRACW PREVP PRACS PSACW
// PSACR PSACI PSAUT PSFW PSFI PSDEP PSSUB PSMLT PGAUT PGFR PGACW PGACI PGACR PGDRY PGACS PGSUB PGMLT
// PGWET PGACR1 PVVAP PVSUB.
struct RateRegion {
    int lo[3], hi[3];
    double sums[33];
};

template <class T> void microphysics_sky(const Grid& g, State<T>& s, T dt, T speed, const Micro<T>& M, RateRegion* rr = nullptr) {
    const T kap = kappa<T>();
    double acc[33] = {0};
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : acc[:33])
    for (int z = 0; z < g.Z; ++z)
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                const int idxG = x + z * g.X;
                const T lo = T(1e-18);
                const T Qv = s.qv[idx] > lo ? s.qv[idx] : T(0), Qw = s.qw[idx] > lo ? s.qw[idx] : T(0);
                const T Qc = s.qc[idx] > lo ? s.qc[idx] : T(0), Qr = s.qr[idx] > lo ? s.qr[idx] : T(0);
                const T Qs = s.qs[idx] > lo ? s.qs[idx] : T(0), Qi = s.qi[idx] > lo ? s.qi[idx] : T(0);
                const T QwMin = T(0.001), QcMin = T(0.001), QiMin = T(0.0006);
                const T ps = s.p[idx];
                T UR = 0, US = 0, UI = 0;
                const T D = s.rho[idx];
                const T tK = s.th[idx] * Pow(ps / s.Pg[idxG], kap);
                const T t = tK - T(273.15);
                if (Qr > 0 || Qs > 0 || Qi > 0) fallingVelocity(Qr, Qs, Qi, D, 3, M.G.Qr, M.G.Qs, M.G.Qi, UR, US, UI);
                const T QWS = ws(t, ps), QWI = wi(t, ps);
                const T PT1 = (t < 0 && Qw + Qc > 0 + T(1e-6)) ? T(1) : T(0);
                const T PT2 = (t < 0 && Qr < T(1e-4) && Qs < T(1e-4)) ? T(1) : T(0);
                const T PT3 = (t < 0 && Qr < T(1e-4)) ? T(1) : T(0);
                const T sR = slopePrecip(D, Qr, 0), sS = slopePrecip(D, Qs, 1), sI = slopePrecip(D, Qi, 2);
                const T dtS = dt * speed;
                T PVCON = M.FPVCON(t, ps, Qv, QWS, dt, speed);
                T PVDEP = M.FPVDEP(t, ps, Qv, QWI, dt, speed);
                PVDEP = Fmin(PVDEP, T(0));
                T PIMLT = M.FPIMLT(t, Qc);
                T PIDW = M.FPIDW(dt, t, Qc, Qw, D, ps);
                T PIHOM = M.FPIHOM(t, Qw);
                T PIACR = M.FPIACR(Qr, Qc, D, sR);
                T PRACI = M.FPRACI(Qr, Qc, D, sR);
                T PRAUT = M.FPRAUT(Qw, QwMin, t);
                T PRACW = M.FPRACW(Qr, Qw, D, sR);
                T PREVP = M.FPREVP(t, Qr, Qv, QWS, D, ps, sR, PT1);
                T PRACS = M.FPRACS(Qr, Qs, PT2, UR, US, D, sS, sR);
                T PSACW = M.FPSACW(Qs, Qw, D, sS);
                T PSACR = M.FPSACR(Qr, Qs, UR, US, D, sR, sS);
                T PSACI = M.FPSACI(t, Qs, Qc, D, sS);
                T PSAUT = M.FPSAUT(t, Qc, QcMin);
                T PSFW = M.FPSFW(dt, t, ps, Qs, Qw, Qc, Qv, QWI, D);
                T PSFI = M.FPSFI(dt, t, ps, Qs, Qw, Qc, Qv, QWI, D);
                T PSDEP = M.FPSDEP(t, ps, Qv, QWI, D, sS);
                T PSSUB = M.FPSSUB(PSDEP);
                PSDEP = Fmax(T(0), PSDEP);
                T PSMLT = M.FPSMLT(t, ps, Qw, Qr, Qs, Qv, D, sS, PSACW, PSACR, dtS);
                T PGAUT = M.FPGAUT(t, Qs, QiMin);
                T PGFR = M.FPGFR(t, Qr, D, sR);
                T PGACW = M.FPGACW(Qi, Qw, sI, D);
                T PGACI = M.FPGACI(Qi, Qc, sI, D);
                T PGACR = M.FPGACR(Qi, Qr, D, UR, UI, sR, sI);
                T PGACS = M.FPGACS(t, Qs, Qi, D, US, UI, sS, sI, false);
                T PGSUB = M.FPGSUB(t, ps, Qv, QWI, Qi, D, sI);
                T PGMLT = M.FPGMLT(t, ps, Qw, Qr, Qi, Qv, D, sI, PGACW, PGACR, dtS);
                T PGDRY = M.FPGDRY(Qw, Qc, Qr, Qs, PGACW, PGACI, PGACR, PGACS, dtS);
                T PGWET = M.FPGWET(t, ps, Qc, Qs, Qi, Qv, US, UI, D, sS, sI, PGACI, PGACS, dtS);
                T PGACR1 = M.FPGACR1(t, Qw, Qc, Qs, Qi, D, US, UI, sS, sI, PGWET, PGACW, PGACI, PGACS, dtS);
                const T WT = PGDRY > PGWET ? T(1) : T(0);
                T condens = 0, depos = 0, freeze = 0;
                auto lim = [&](T cap, T rate) { return dt * Fmin(cap, speed * rate); };
                if (t < 0) {
                    if (PVCON >= 0) condens += PVCON = lim(Qv, PVCON);
                    else if (PVCON < 0) condens += PVCON = dt * Fmax(-Qw, speed * PVCON);
                    if (PVDEP >= 0) depos += PVDEP = lim(Qv, PVDEP);
                    else if (PVDEP < 0) depos += PVDEP = dt * Fmax(-Qc, speed * PVDEP);
                    depos += PIDW = lim(Qw, PIDW);
                    freeze += PIHOM = lim(Qw, PIHOM);
                    freeze += PIACR = lim(Qr, PIACR);
                    PRACI = lim(Qc, PRACI);
                    PRAUT = lim(Qw, PRAUT);
                    PRACW = lim(Qw, PRACW);
                    condens -= PREVP = lim(Qr, PREVP * (1 - PT1));
                    PRACS = lim(Qs, PRACS * (1 - PT2));
                    freeze += PSACR = lim(Qr, PSACR);
                    freeze += PSACW = lim(Qw, PSACW);
                    PSACI = lim(Qc, PSACI);
                    PSAUT = lim(Qc, PSAUT);
                    freeze += PSFW = lim(Qw, PSFW);
                    PSFI = lim(Qc, PSFI);
                    depos += PSDEP = lim(Qv, PSDEP * (PT1));
                    depos -= PSSUB = lim(Qs, PSSUB * (1 - PT1));
                    PGAUT = lim(Qs, PGAUT);
                    freeze += PGFR = lim(Qr, PGFR);
                    PGACI = lim(Qc, PGACI);
                    freeze += PGACR = lim(Qr, PGACR * (1 - WT));
                    PGACS = lim(Qs, PGACS);
                    depos -= PGSUB = lim(Qi, PGSUB * (1 - PT1));
                    if (WT == T(1)) {
                        if (PGACR1 >= 0) freeze += PGACR1 = lim(Qr, PGACR1);
                        else if (PGACR1 < 0) freeze += PGACR1 = dt * Fmax(-Qi, speed * PGACR1);
                    }
                } else {
                    if (PVCON >= 0) condens += PVCON = lim(Qv, PVCON);
                    else if (PVCON < 0) condens += PVCON = dt * Fmax(-Qw, speed * PVCON);
                    if (PVDEP >= 0) depos += PVDEP = lim(Qv, PVDEP);
                    else if (PVDEP < 0) depos += PVDEP = dt * Fmax(-Qc, speed * PVDEP);
                    freeze -= PIMLT = lim(Qc, PIMLT);
                    PIACR = 0;
                    PRAUT = lim(Qw, PRAUT);
                    PRACW = lim(Qw, PRACW);
                    condens -= PREVP = lim(Qr, PREVP * (1 - PT1));
                    PSACW = lim(Qw, PSACW);
                    freeze -= PSMLT = lim(Qs, PSMLT);
                    freeze += PGACW = lim(Qw, PGACW);
                    PGACS = lim(Qs, PGACS);
                    freeze -= PGMLT = lim(Qi, PGMLT);
                }
                if (t < 0) {
                    s.qv[idx] += PSSUB * (1 - PT1) + PGSUB * (1 - PT1) + PREVP * (1 - PT1) - PSDEP * (PT1) - PVCON - PVDEP;
                    s.qw[idx] += PVCON - PSACW - PSFW - PRAUT - PRACW - PIDW - PIHOM;
                    s.qc[idx] += PVDEP + PIDW + PIHOM - PSAUT - PSACI - PRACI - PSFI - PGACI;
                    s.qr[idx] += PRAUT + PRACW - PIACR - PSACR - PGACR * (1 - WT) - PGACR1 * (WT) - PGFR - PREVP * (1 - PT1);
                    s.qs[idx] += PSAUT + PSACI + PSACW + PSFW + PSFI + PRACI * (PT3) + PIACR * (PT3) - PGACS - PGAUT -
                                 PRACS * (1 - PT2) + PSACR * (PT2) - PSSUB * (1 - PT1) + PSDEP * (PT1);
                    s.qi[idx] += PGAUT + PGFR + PGDRY * (1 - WT) + PGWET * (WT) + PSACR * (1 - PT2) + PRACS * (1 - PT2) +
                                 PRACI * (1 - PT3) + PIACR * (1 - PT3) - PGSUB * (1 - PT1);
                } else {
                    s.qv[idx] += PREVP * (1 - PT1) - PVCON - PVDEP;
                    s.qw[idx] += PVCON + PIMLT - PRAUT - PRACW - PGACW - PSACW;
                    s.qc[idx] += PVDEP - PIMLT;
                    s.qr[idx] += PRAUT + PRACW + PSACW + PGACW + PGMLT + PSMLT - PREVP * (1 - PT1);
                    s.qs[idx] += -PSMLT - PGACS;
                    s.qi[idx] += -PGMLT + PGACS;
                }
                if (rr && x >= rr->lo[0] && x <= rr->hi[0] && y >= rr->lo[1] && y <= rr->hi[1] && z >= rr->lo[2] && z <= rr->hi[2]) {
                    const T PVVAP = PVCON < 0 ? -PVCON : T(0), PVSUB = PVDEP < 0 ? -PVDEP : T(0);
                    const T v[33] = {PVCON < 0 ? T(0) : PVCON, PVDEP < 0 ? T(0) : PVDEP, PIMLT, PIDW, PIHOM, PIACR, PRACI, PRAUT, PRACW,
                                     PREVP, PRACS, PSACW, PSACR, PSACI, PSAUT, PSFW, PSFI, PSDEP, PSSUB, PSMLT, PGAUT, PGFR, PGACW,
                                     PGACI, PGACR, PGDRY * (1 - WT), PGACS, PGSUB, PGMLT, PGWET * WT, PGACR1, PVVAP, PVSUB};
                    for (int k = 0; k < 33; ++k) acc[k] += double(v[k]);
                }
                // addHeatGPU with the updated Qv
                const T qv2 = s.qv[idx];
                const T Mair = T(0.02896), Mwat = T(0.01802);
                const T XV = (qv2 / Mwat) / ((qv2 / Mwat) + (1 - qv2) / Mair);
                const T Mth = XV * Mwat + (1 - XV) * Mair;
                const T Yair = T(1.4), yV = T(1.33);
                const T YV = XV * (Mwat / Mth);
                const T yth = YV * yV + (1 - YV) * Yair;
                const T cpth = yth * K<T>::R / (Mth * (yth - 1));
                T sum = 0;
                sum += Lwater(s.th[idx] - T(273.15)) / cpth * condens;
                sum += Lice(s.th[idx] - T(273.15)) / cpth * depos;
                sum += K<T>::Lf / cpth * freeze;
                s.th[idx] += sum;
            }
    if (rr)
        for (int k = 0; k < 33; ++k) rr->sums[k] = acc[k];
}

// ---------------------------------------------------------------------------------------------
// Ground / boundary kernels (2D, X*Z)
// ---------------------------------------------------------------------------------------------
// advectGroundWaterGPU Game/kernelSky.cu:120-253. The reference leaves the 16x16 tile halos
// unfilled between tiles (uninitialised shared memory); here every neighbour is the neighbouring
// column, and the domain edge repeats the cell itself as the reference does.
template <class T> void ground_water(const Grid& g, State<T>& s, T dt, T speed, T vox) {
    const int X = g.X, Z = g.Z;
    std::vector<T> rs(s.Qrs, s.Qrs + X * Z), gr(s.Qgr, s.Qgr + X * Z);
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int idx = x + z * X;
            const int iL = x == 0 ? idx : idx - 1, iR = x == X - 1 ? idx : idx + 1;
            const int iB = z == 0 ? idx : idx - X, iF = z == Z - 1 ? idx : idx + X;
            const T rsC = rs[idx], grC = gr[idx];
            T fGr = grC, fRs = rsC;
            auto flow = [&](T hFrom, T hTo, T grFrom, T grTo, T rsFrom, T rsTo) {
                const T n = T(1) / T(0.03);
                const T kk = T(5e-5);
                const T slope = hFrom - hTo / T(1);
                const bool fromPrev = slope > T(0);
                const T sRain = fromPrev ? grFrom : grTo;
                const T sWat = fromPrev ? rsFrom : rsTo;
                T changeRain = 0;
                if (sRain != T(0)) {
                    const T RH = sRain;
                    const T spd = n * Pow(RH, T(2) / T(3));
                    const T vel = spd * Pow(slope, T(0.5));
                    changeRain = vel * sRain;
                }
                const T changeWater = K<T>::g * kk * sWat * slope;
                const T DG = T(1.75e-3), DS = T(1.8e-5);
                const T dR = 1 / (vox * vox) * DG, dW = 1 / (vox * vox) * DS;
                const T lapR = (grFrom - grTo) * dR, lapSR = (rsFrom - rsTo) * dW;
                const bool pR = lapR > T(0), pSR = lapSR > T(0);
                const T fgR = dt * Fmin(Fabs(lapR) * speed, pR ? grFrom : grTo) * (lapR > T(0) ? T(1) : T(-1));
                const T fgW = dt * Fmin(Fabs(lapSR) * speed, pSR ? rsFrom : rsTo) * (lapSR > T(0) ? T(1) : T(-1));
                const T sfR = dt * Fmin(Fabs(changeRain) * speed, fromPrev ? grFrom : grTo) * (changeRain > T(0) ? T(1) : T(-1));
                const T sfW = dt * Fmin(Fabs(changeWater) * speed, fromPrev ? rsFrom : rsTo) * (changeWater > T(0) ? T(1) : T(-1));
                fGr += fgR + sfR;
                fRs += fgW + sfW;
            };
            const T hC = T(g.gh[idx]);
            flow(T(g.gh[iL]), hC, gr[iL], grC, rs[iL], rsC);
            flow(T(g.gh[iR]), hC, gr[iR], grC, rs[iR], rsC);
            flow(T(g.gh[iB]), hC, gr[iB], grC, rs[iB], rsC);
            flow(T(g.gh[iF]), hC, gr[iF], grC, rs[iF], rsC);
            s.Qgr[idx] = fGr;
            s.Qrs[idx] = fRs;
        }
}

// irridianceGPU Game/environment.cu:1021-1034 (host, float)
inline float irradiance(float time, int day, float longitude, float sun) {
    const float Gs = 1361.0f * sun;
    const float rd = 1 + 0.034f * cosf(2 * 3.14159265359f * day / 365);
    const float sd = 0.409f * sinf(2 * 3.14159265359f / 365 * (day - 81));
    const float th = time / 3600;
    const float lr = longitude * 0.01745329251994329576923690768489f;  // glm::radians
    const float sr = (th - (6.0f + 14.0f / 2.0f)) * (3.14159265359f / 12.0f);
    return std::max(0.0f, Gs * rd * (sinf(lr) * sinf(sd) + cosf(lr) * cosf(sd) * cosf(sr)));
}

template <class T> void ground_stage(const Grid& g, const Config& cfg, State<T>& s, T dt, T speed, T irr, const Micro<T>& M) {
    const int X = g.X, Z = g.Z;
    const T vox = T(cfg.voxel);
    const T kap = kappa<T>();
    ground_water(g, s, dt, speed, vox);
    // calculateCloudCoverGPU Game/kernelSky.cu:1034-1044
    std::vector<T> cc(X * Z);
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int idxG = x + z * X;
            T tot = 0;
            for (int y = g.gh[idxG] + 1; y < g.Y; ++y) tot += (s.qc[g.id(x, y, z)] + s.qw[g.id(x, y, z)]) * vox;
            cc[idxG] = Fmin(tot / T(1.2), T(1));
        }
    // calculateGroundTempGPU :1046-1059 (T^4 formed in the working precision, accumulated in double)
    for (int i = 0; i < X * Z; ++i) {
        const T gT = s.Tg[i];
        const double T4 = double(gT * gT * gT * gT);
        const T dtS = dt * speed;
        s.Tg[i] = T(double(s.Tg[i]) + double(dtS) * (double(1 - cc[i]) * ((double((1 - T(0.25)) * irr) - double(K<T>::ge * K<T>::oo) * T4) /
                                                                           double(T(1) * T(1500) * K<T>::Cpds))));
    }
    // calculatePrecipHittingGroundMicroPhysicsGPU Game/microPhysics.cu:1544-1636
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int idxG = x + z * X;
            const int64_t idx = g.id(x, g.gh[idxG] + 1, z);
            const T lo = T(1e-18);
            const T Qgr = s.Qgr[idxG] > lo ? s.Qgr[idxG] : T(0), Qgs = s.Qgs[idxG] > lo ? s.Qgs[idxG] : T(0), Qgi = s.Qgi[idxG] > lo ? s.Qgi[idxG] : T(0);
            const T Qv = s.qv[idx] > lo ? s.qv[idx] : T(0), Qr = s.qr[idx] > lo ? s.qr[idx] : T(0);
            const T Qs = s.qs[idx] > lo ? s.qs[idx] : T(0), Qi = s.qi[idx] > lo ? s.qi[idx] : T(0);
            T freeze = 0;
            const T tgC = s.Tg[idxG] - T(273.15);
            const T ps = s.p[idx], wind = s.u[idx], D = s.rho[idx];
            const T taK = s.th[idx] * Pow(ps / s.Pg[idxG], kap);
            T UR = 0, US = 0, UI = 0;
            if (Qgr > 0 || Qgs > 0 || Qgi > 0) fallingVelocity(Qgr, Qgs, Qgi, D, 3, M.G.Qr, M.G.Qs, M.G.Qi, UR, US, UI);
            T GR = dt * Fmin(Qr * speed, Qr), GS = dt * Fmin(Qs * speed, Qs), GI = dt * Fmin(Qi * speed, Qi);
            T PGRFR = M.FPGRFR(taK, tgC, ps, Qr, Qv, Qi, Qgr, Qgs, D, wind, UR);
            if (taK < T(273.15)) freeze += PGRFR = dt * Fmin(Qr, speed * PGRFR);
            s.qr[idx] += -GR;
            s.qs[idx] += -GS;
            s.qi[idx] += -GI;
            s.Qgr[idxG] += GR - PGRFR;
            s.Qgs[idxG] += GS;
            s.Qgi[idxG] += GI + PGRFR;
            const T Mair = T(0.02896), Mwat = T(0.01802);
            const T XV = (Qv / Mwat) / ((Qv / Mwat) + (1 - Qv) / Mair);
            const T Mth = XV * Mwat + (1 - XV) * Mair;
            const T YV = XV * (Mwat / Mth);
            const T yth = YV * T(1.33) + (1 - YV) * T(1.4);
            const T cpth = K<T>::R / (Mth * (yth - 1));
            T sum = 0;
            sum += K<T>::Lf / cpth * freeze;
            s.Tg[idxG] += sum;
        }
    // calculateGroundMicroPhysicsGPU Game/microPhysics.cu:1419-1541
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int idxG = x + z * X;
            const int64_t idx = g.id(x, g.gh[idxG] + 1, z);
            const T lo = T(1e-18);
            const T Qrs = s.Qrs[idxG] > lo ? s.Qrs[idxG] : T(0), Qgr = s.Qgr[idxG] > lo ? s.Qgr[idxG] : T(0);
            const T Qgs = s.Qgs[idxG] > lo ? s.Qgs[idxG] : T(0), Qgi = s.Qgi[idxG] > lo ? s.Qgi[idxG] : T(0);
            const T Qv = s.qv[idx] > lo ? s.qv[idx] : T(0);
            T condens = 0, freeze = 0, depos = 0;
            const T tgC = s.Tg[idxG] - T(273.15);
            const T ps = s.p[idx], wind = s.u[idx], cov = cc[idxG], D = s.rho[idx];
            T& tim = s.tg[idxG];
            const T taK = s.th[idx] * Pow(ps / s.Pg[idxG], kap);
            const T sS = slopePrecip(D, Qgs, 1), sI = slopePrecip(D, Qgi, 2);
            (void)sS;
            T PGREVP = M.FPGREVP(taK, tgC, ps, Qv, Qgr, irr, D, wind);
            T PGSMLT = M.FPGSMLT(taK, tgC, ps, Qgs, Qv, Qgr, irr, cov, D, wind, dt);
            T PGGMLT = M.FPGGMLT(tgC, Qgi, D, sI);
            T PGGFR = M.FPGGFR(taK, tgC, ps, Qgr, Qv, Qgi, D, irr, cov, wind, dt);
            T PGSFR = M.FPGSFR(taK, tgC, ps, Qv, Qgr, Qgs, D, wind, dt);
            T PGFLW = M.FPGFLW(Qgr);
            T PGDEVP = M.FPGDEVP(tim, Qgr, Qgs, Qgi, Qrs);
            condens -= PGREVP = dt * Fmin(Qgr, speed * PGREVP);
            freeze -= PGSMLT = dt * Fmin(Qgs, speed * PGSMLT);
            freeze -= PGGMLT = dt * Fmin(Qgi, speed * PGGMLT);
            freeze += PGGFR = dt * Fmin(Qgr, speed * PGGFR);
            freeze += PGSFR = dt * Fmin(Qgr, speed * PGSFR);
            PGFLW = dt * Fmin(Qgr, speed * PGFLW);
            condens -= PGDEVP = dt * Fmin(Qrs, speed * PGDEVP);
            s.Qrs[idxG] += PGFLW - PGDEVP;
            s.qv[idx] += PGREVP + PGDEVP;
            s.Qgr[idxG] += PGSMLT + PGGMLT - PGREVP - PGGFR - PGSFR - PGFLW;
            s.Qgs[idxG] += PGSFR - PGSMLT;
            s.Qgi[idxG] += PGGFR - PGGMLT;
            const T mass = T(1500) * T(0.1);
            T sum = 0;
            sum += Lwater(tgC) / (mass * T(1500)) * condens;
            sum += Lice(tgC) / (mass * T(1500)) * depos;
            sum += K<T>::Lf / (mass * T(1500)) * freeze;
            s.Tg[idxG] += sum;
        }
}

// setTempsAtGroundGPU Game/kernelSky.cu:255-268
template <class T> void set_temps_at_ground(const Grid& g, State<T>& s, T dtS) {
    for (int z = 0; z < g.Z; ++z)
        for (int x = 0; x < g.X; ++x) {
            const int Gi = x + z * g.X;
            const int y = g.gh[Gi] + 1;
            if (y >= g.Y - 1) continue;
            const int64_t idx = g.id(x, y, z);
            const T Tt = potentialTemp(s.Tg[Gi] - T(273.15), s.p[idx], s.Pg[Gi]) + T(273.15);
            const T dif2 = s.th[idx] - Tt;
            s.th[idx] -= dif2 * Fmin(T(1), dtS);
        }
}

// ---------------------------------------------------------------------------------------------
// One step, environmentGPU::updateGPU Game/environment.cu:391-555
// ---------------------------------------------------------------------------------------------
template <class T> int step(const Config& cfg, int X, int Y, int Z, State<T>& s, float dtf, float speedf, Diag& dg) {
    Grid g{X, Y, Z, s.gh};
    const T dt = T(dtf), speed = T(speedf);
    const T dtS = dt * speed;
    static const Micro<T> M;
    const T irr = T(irradiance(float(s.sim_time), s.day, s.longitude, s.sun));
    // ground
    ground_stage(g, cfg, s, dt, speed, irr, M);
    // sky 1: theta
    set_temps_at_ground(g, s, dtS);
    diffuse(g, cfg, s, s.th, 0, dtS);
    dg.nsub[0] = advect_field(g, cfg, s, s.th, s.isenT, Bounds{CUSTOM, CUSTOM}, dtS);
    // sky 2: momentum
    buoyancy(g, s, dtS);
    diffuse(g, cfg, s, s.u, 2, dtS);
    diffuse(g, cfg, s, s.v, 3, dtS);
    diffuse(g, cfg, s, s.w, 4, dtS);
    std::vector<T> zero(Y, T(0));
    dg.nsub[1] = advect_field(g, cfg, s, s.u, s.defU, Bounds{CUSTOM, DIRICHLET}, dtS);
    dg.nsub[2] = advect_field(g, cfg, s, s.v, (const T*)zero.data(), Bounds{DIRICHLET, DIRICHLET}, dtS);
    dg.nsub[3] = advect_field(g, cfg, s, s.w, s.defW, Bounds{CUSTOM, DIRICHLET}, dtS);
    init_density(g, s);
    project(g, cfg, s, dtS, dg);
    new_pressure(g, s);
    // sky 3: moisture
    diffuse(g, cfg, s, s.qv, 1, dtS);
    dg.nsub[4] = advect_field(g, cfg, s, s.qv, s.isenQv, Bounds{CUSTOM, CUSTOM}, dtS);
    const Bounds bm{DIRICHLET, DIRICHLET};
    static const Gammas<T> Gm;
    diffuse(g, cfg, s, s.qw, 5, dtS);
    dg.nsub[5] = advect_field(g, cfg, s, s.qw, (const T*)zero.data(), bm, dtS);
    diffuse(g, cfg, s, s.qc, 5, dtS);
    dg.nsub[6] = advect_field(g, cfg, s, s.qc, (const T*)zero.data(), bm, dtS);
    diffuse(g, cfg, s, s.qr, 5, dtS);
    advect_precip(g, cfg, s, s.qr, 0, dtS, Gm);
    dg.nsub[7] = advect_field(g, cfg, s, s.qr, (const T*)zero.data(), bm, dtS);
    diffuse(g, cfg, s, s.qs, 5, dtS);
    advect_precip(g, cfg, s, s.qs, 1, dtS, Gm);
    dg.nsub[8] = advect_field(g, cfg, s, s.qs, (const T*)zero.data(), bm, dtS);
    diffuse(g, cfg, s, s.qi, 5, dtS);
    advect_precip(g, cfg, s, s.qi, 2, dtS, Gm);
    dg.nsub[9] = advect_field(g, cfg, s, s.qi, (const T*)zero.data(), bm, dtS);
    // sky 4: microphysics + latent heat
    microphysics_sky(g, s, dt, speed, M);
    // clock (float, as m_time)
    float tm = float(s.sim_time);
    tm += speedf * dtf * float(!s.pause);
    if (tm > 86400.0f) tm = 0.0f;
    s.sim_time = tm;
    return 0;
}

// randomCuda, the PCG hash (Game/kernelMaths.cu:93-98)
inline uint32_t pcg_hash(uint32_t seed) {
    uint32_t st = seed * 747796405u + 2891336453u;
    uint32_t w = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
    return (w >> 22u) ^ w;
}

// environmentGPU::init Game/environment.cu:249-389 (host arrays already in SoA form)
template <class T> void init_state(int X, int Y, int Z, State<T>& s, int noise) {
    Grid g{X, Y, Z, s.gh};
    const int64_t N = g.n();
    init_density(g, s);
    for (int y = 0; y < Y; ++y) {  // default columns from (x=0, z=0), :299-303
        s.isenT[y] = s.th[g.id(0, y, 0)];
        s.isenQv[y] = s.qv[g.id(0, y, 0)];
        s.defU[y] = s.u[g.id(0, y, 0)];
        s.defW[y] = s.w[g.id(0, y, 0)];
    }
    if (noise) {  // randomArray :100-116 with the seed race resolved (every thread sees the seed)
        auto add = [&](T* a, float mn, float mx, uint32_t seed) {
            for (int64_t i = 0; i < N; ++i) {
                const float rnd = float(pcg_hash(uint32_t(seed + uint32_t(i))) % 1000u) / float(1000);
                a[i] += T(rnd * (mx - mn) + mn);
            }
        };
        add(s.th, -0.1f, 0.1f, 100);
        add(s.qv, 0.0f, 0.0001f, 101);
        add(s.u, 0.5f, 0.5f, 102);
        add(s.v, -0.2f, 0.2f, 103);
        add(s.w, 0.5f, 0.5f, 104);
    }
    // resetValueInGround on the 10 prognostic fields (kernelGround.cu:21-36)
    T* fl[10] = {s.th, s.qv, s.qw, s.qc, s.qr, s.qs, s.qi, s.u, s.v, s.w};
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x)
                if (g.ground(x, y, z))
                    for (T* f : fl) f[g.id(x, y, z)] = 0;
    // computeIsenTempGroundGPU kernelGround.cu:38-47
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int idx = x + z * X;
            const int GH = s.gh[idx] + 1 >= Y ? Y - 1 : s.gh[idx] + 1;
            const T Tt = potentialTemp(s.isenT[GH - 1] - T(273.15), s.Pg[idx], s.p[g.id(x, GH, z)]);
            s.Tg[idx] = Tt + T(273.15);
        }
}

// ---------------------------------------------------------------------------------------------
// Editing: prepareBrushGPU / prepareSelectionGPU / resetParameterGPU (Game/environment.cu:1127-1290)
// with applyBrushGPU, applySelectionGPU, setGround, compareAndResetValuesOutGround
// (Game/kernelSky.cu:1476-1642), editorDataGPU's ground block (Game/environment.cu:989-1011),
// setToDefault / setToValue (Game/kernelSky.cu:1714-1728, Game/kernelMaths.cu:12-23).
// Parameters: 0 theta, 1 Qv .. 6 Qi, 7 wind, 8 ground (Game/config.h:62-65).
// Two differences: the reference's bounds test lets z = Z through (`mZ > GRIDSIZESKYZ`) and writes
// one plane past the field, here that plane is skipped; a raise stops at row Y-2 so that every
// column keeps a sky cell.
// ---------------------------------------------------------------------------------------------
struct EditParams {
    int param;
    float value, dir[3];
    int erase;
};

template <class T> T* edit_field(State<T>& s, int param) {
    T* f[7] = {s.th, s.qv, s.qw, s.qc, s.qr, s.qs, s.qi};
    return param >= 0 && param < 7 ? f[param] : nullptr;
}

// one brushed/selected cell; amount = the value before the wind split. Returns true when the
// ground store changed (setGround, Game/kernelSky.cu:1597-1611).
template <class T>
bool edit_cell(const Grid& g, State<T>& s, std::vector<int32_t>& ghn, const EditParams& ep, int x, int y, int z, float amount, bool add) {
    const int ig = x + z * g.X;
    if (ep.param == 8) {
        if (ep.erase && y <= g.gh[ig]) { ghn[ig] = std::min(ghn[ig], y); return true; }
        if (!ep.erase && y > g.gh[ig]) { ghn[ig] = std::max(ghn[ig], std::min(y, g.Y - 2)); return true; }  // keep a sky cell
        return false;
    }
    const int64_t idx = g.id(x, y, z);
    float v1 = amount, v2 = 0, v3 = 0;
    if (ep.param == 7) {
        v3 = v1 * ep.dir[2];
        v2 = v1 * ep.dir[1];
        v1 *= ep.dir[0];
        if (add) { s.u[idx] += v1; s.v[idx] += v2; s.w[idx] += v3; }
        else { s.u[idx] = v1; s.v[idx] = v2; s.w[idx] = v3; }
    } else {
        T* f = edit_field(s, ep.param);
        if (add) f[idx] += v1;
        else f[idx] = v1;
    }
    return false;
}

// editorDataGPU's block (Game/environment.cu:992-1011), run after an edit and at the start of the
// next step while the ground has changed: ground cells of theta, Qv, Qw..Qi, u, v to 0; the ground
// temperature from the isentrope (computeIsenTempGroundGPU Game/kernelGround.cu:38-47)
template <class T> void editor_block(const Grid& g, State<T>& s) {
    const int X = g.X, Y = g.Y, Z = g.Z;
    T* fl[9] = {s.th, s.qv, s.qw, s.qc, s.qr, s.qs, s.qi, s.u, s.v};
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x)
                if (g.ground(x, y, z))
                    for (T* f : fl) f[g.id(x, y, z)] = 0;
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int idx = x + z * X;
            const int GH = s.gh[idx] + 1 >= Y ? Y - 1 : s.gh[idx] + 1;
            const T Tt = potentialTemp(s.isenT[GH - 1] - T(273.15), s.Pg[idx], s.p[g.id(x, GH, z)]);
            s.Tg[idx] = Tt + T(273.15);
        }
}

// after an edit whose ground store changed: reset the cells an erase freed, take the new heights
template <class T> void edit_finish(Grid& g, State<T>& s, std::vector<int32_t>& ghn, bool erase, const T* pcol) {
    const int X = g.X, Y = g.Y, Z = g.Z;
    if (erase)
        for (int z = 0; z < Z; ++z)
            for (int y = 0; y < Y; ++y)
                for (int x = 0; x < X; ++x) {
                    const int ig = x + z * X;
                    if (y > s.gh[ig] || y <= ghn[ig]) continue;
                    const int64_t idx = g.id(x, y, z);
                    s.qv[idx] = s.isenQv[y];
                    s.qw[idx] = s.qc[idx] = s.qr[idx] = s.qs[idx] = s.qi[idx] = 0;
                    s.th[idx] = s.isenT[y];
                    s.u[idx] = s.v[idx] = s.w[idx] = 0;
                    s.p[idx] = pcol[y];
                }
    std::copy(ghn.begin(), ghn.end(), s.gh);
}

// applyBrushGPU: the brush box is ceil(r) - floor(-r) cells wide in x and y, offset by ceil(r)
// (so x and y reach -ceil(r) .. ceil(r)-1), and runs over the whole column range in z
template <class T>
int brush(Grid& g, State<T>& s, const EditParams& ep, float size, const int pos[3], float smooth, float dt, float intensity, const T* pcol) {
    const int c = int(std::ceil(size));
    const int n = int(std::ceil(size)) - int(std::floor(-size));
    std::vector<int32_t> ghn(s.gh, s.gh + size_t(g.X) * g.Z);
    bool changed = false;
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x)
            for (int z = 0; z < g.Z; ++z) {
                const int lX = x - c, lY = y - c, lZ = z - c;
                const int mX = x + pos[0] - c, mY = y + pos[1] - c, mZ = z + pos[2] - c;
                if (mX >= g.X || mY >= g.Y || mZ >= g.Z || mX < 0 || mY < 0 || mZ < 0) continue;
                if (ep.param != 8 && mY <= g.gh[mX + mZ * g.X]) continue;
                const float d = float(lX) * float(lX) + float(lY) * float(lY) + float(lZ) * float(lZ);
                const float r = size * size;
                if (!(d <= r)) continue;
                float v = -(d / r - 1);
                v = std::pow(v, smooth);
                v *= dt * intensity * ep.value;
                changed |= edit_cell(g, s, ghn, ep, mX, mY, mZ, v, true);
            }
    if (changed) edit_finish(g, s, ghn, ep.erase != 0, pcol);
    return changed ? 1 : 0;
}

// applySelectionGPU: the box lo..hi (an empty x or y extent becomes one cell, as the host code does)
template <class T> int selection(Grid& g, State<T>& s, const EditParams& ep, const int lo[3], const int hi[3], const T* pcol) {
    int ny = hi[1] - lo[1] + 1, nx = hi[0] - lo[0] + 1;
    if (ny <= 0) ny = 1;
    if (nx <= 0) nx = 1;
    std::vector<int32_t> ghn(s.gh, s.gh + size_t(g.X) * g.Z);
    bool changed = false;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x)
            for (int z = lo[2]; z <= hi[2]; ++z) {
                const int mX = x + lo[0], mY = y + lo[1], mZ = z;
                if (mX >= g.X || mY >= g.Y || mZ >= g.Z || mX < 0 || mY < 0 || mZ < 0) continue;
                if (ep.param != 8 && mY <= g.gh[mX + mZ * g.X]) continue;
                changed |= edit_cell(g, s, ghn, ep, mX, mY, mZ, ep.value, false);
            }
    if (changed) edit_finish(g, s, ghn, ep.erase != 0, pcol);
    return changed ? 1 : 0;
}

// resetParameterGPU: setToDefault stops each (x, y) column at its first ground cell in z;
// setToValue covers every cell
template <class T> void reset_parameter(const Grid& g, State<T>& s, int param, const T* pcol) {
    auto to_default = [&](T* f, const T* def) {
        for (int y = 0; y < g.Y; ++y)
            for (int x = 0; x < g.X; ++x)
                for (int z = 0; z < g.Z; ++z) {
                    if (g.ground(x, y, z)) break;
                    f[g.id(x, y, z)] = def[y];
                }
    };
    auto to_value = [&](T* f, T v) { std::fill(f, f + g.n(), v); };
    switch (param) {
        case 0: to_default(s.th, s.isenT); break;
        case 7: to_default(s.u, s.defU); to_value(s.v, T(0)); to_default(s.w, s.defW); break;
        case 9: to_default(s.p, pcol); break;
        case 1: to_default(s.qv, s.isenQv); break;
        case 2: to_value(s.qw, T(0)); break;
        case 3: to_value(s.qc, T(0)); break;
        case 4: to_value(s.qr, T(0)); break;
        case 5: to_value(s.qs, T(0)); break;
        case 6: to_value(s.qi, T(0)); break;
        default: break;
    }
}

}  // namespace skt_oracle

// ------------------------------------- C ABI for the tests --------------------------------------
using namespace skt_oracle;

typedef struct {
    int semantics, diffuse_sweeps;
    float pcg_tol;
    int pcg_max_iter, max_substeps;
    float voxel;
} oc_config;

typedef struct {
    void *th, *qv, *qw, *qc, *qr, *qs, *qi, *u, *v, *w, *p, *rho;
    void *Qrs, *Qgr, *Qgs, *Qgi, *Pg, *tg, *Tg;
    void *isenT, *isenQv, *defU, *defW;
    int32_t* gh;
    double sim_time;
    int day;
    float longitude, sun;
    int pause;
} oc_state;

typedef struct {
    int pcg_iters;
    double pcg_residual;
    int nsub[10];
    int converged;
} oc_diag;

template <class T> static State<T> unpack(const oc_state* o) {
    State<T> s;
    s.th = (T*)o->th; s.qv = (T*)o->qv; s.qw = (T*)o->qw; s.qc = (T*)o->qc; s.qr = (T*)o->qr; s.qs = (T*)o->qs;
    s.qi = (T*)o->qi; s.u = (T*)o->u; s.v = (T*)o->v; s.w = (T*)o->w; s.p = (T*)o->p; s.rho = (T*)o->rho;
    s.Qrs = (T*)o->Qrs; s.Qgr = (T*)o->Qgr; s.Qgs = (T*)o->Qgs; s.Qgi = (T*)o->Qgi; s.Pg = (T*)o->Pg; s.tg = (T*)o->tg; s.Tg = (T*)o->Tg;
    s.isenT = (T*)o->isenT; s.isenQv = (T*)o->isenQv; s.defU = (T*)o->defU; s.defW = (T*)o->defW;
    s.gh = o->gh; s.sim_time = o->sim_time; s.day = o->day; s.longitude = o->longitude; s.sun = o->sun; s.pause = o->pause;
    return s;
}
static Config cfg_of(const oc_config* c) {
    return Config{c->semantics, c->diffuse_sweeps, c->pcg_tol, c->pcg_max_iter, c->max_substeps, c->voxel};
}

extern "C" {

#define OC_DEFINE(suffix, T)                                                                          \
    int oc_init_##suffix(int X, int Y, int Z, oc_state* st, int noise) {                             \
        State<T> s = unpack<T>(st);                                                                   \
        init_state<T>(X, Y, Z, s, noise);                                                             \
        return 0;                                                                                     \
    }                                                                                                 \
    int oc_step_##suffix(const oc_config* c, int X, int Y, int Z, oc_state* st, float dt, float sp, \
                         oc_diag* d) {                                                                \
        State<T> s = unpack<T>(st);                                                                   \
        Diag dg{};                                                                                    \
        int rc = step<T>(cfg_of(c), X, Y, Z, s, dt, sp, dg);                                          \
        st->sim_time = s.sim_time;                                                                    \
        if (d) {                                                                                      \
            d->pcg_iters = dg.pcg_iters; d->pcg_residual = dg.pcg_residual; d->converged = dg.converged; \
            for (int i = 0; i < 10; ++i) d->nsub[i] = dg.nsub[i];                                     \
        }                                                                                             \
        return rc;                                                                                    \
    }

OC_DEFINE(f32, float)
OC_DEFINE(f64, double)

float oc_irradiance(float time, int day, float longitude, float sun) { return irradiance(time, day, longitude, sun); }

int oc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // extern "C"

// Single-stage entry points used by the per-kernel parity tests.
template <class T> static int stage_impl(const oc_config* c, int X, int Y, int Z, oc_state* st, int stage, int arg, float dt, float speed, oc_diag* d) {
    State<T> s = unpack<T>(st);
    Grid g{X, Y, Z, s.gh};
    Config cf = cfg_of(c);
    static const Micro<T> M;
    static const Gammas<T> Gm;
    std::vector<T> zero(Y, T(0));
    Diag dg{};
    switch (stage) {
        case 0: diffuse(g, cf, s, arg == 0 ? s.th : arg == 1 ? s.qv : arg == 2 ? s.u : arg == 3 ? s.v : arg == 4 ? s.w : s.qw, arg, T(dt)); break;
        case 1: {  // advect field arg (0 th,1 u,2 v,3 w,4 qv,5 qw)
            T* f[6] = {s.th, s.u, s.v, s.w, s.qv, s.qw};
            const T* df[6] = {s.isenT, s.defU, zero.data(), s.defW, s.isenQv, zero.data()};
            Bounds bb[6] = {{CUSTOM, CUSTOM}, {CUSTOM, DIRICHLET}, {DIRICHLET, DIRICHLET}, {CUSTOM, DIRICHLET}, {CUSTOM, CUSTOM}, {DIRICHLET, DIRICHLET}};
            dg.nsub[0] = advect_field(g, cf, s, f[arg], df[arg], bb[arg], T(dt));
            break;
        }
        case 2: buoyancy(g, s, T(dt)); break;
        case 3: init_density(g, s); project(g, cf, s, T(dt), dg); break;
        case 4: microphysics_sky(g, s, T(dt), T(speed), M); break;
        case 5: advect_precip(g, cf, s, arg == 0 ? s.qr : arg == 1 ? s.qs : s.qi, arg, T(dt), Gm); break;
        case 6: {
            const T irr = T(irradiance(float(s.sim_time), s.day, s.longitude, s.sun));
            ground_stage(g, cf, s, T(dt), T(speed), irr, M);
            set_temps_at_ground(g, s, T(dt) * T(speed));  // the GPU fuses this into its ground stage
            break;
        }
        case 7: set_temps_at_ground(g, s, T(dt) * T(speed)); break;
        case 8: init_density(g, s); break;
        case 9: new_pressure(g, s); break;
        default: return -1;
    }
    if (d) { d->pcg_iters = dg.pcg_iters; d->pcg_residual = dg.pcg_residual; d->converged = dg.converged; d->nsub[0] = dg.nsub[0]; }
    return 0;
}


extern "C" {
int oc_stage_f32(const oc_config* c, int X, int Y, int Z, oc_state* st, int stage, int arg, float dt, float speed, oc_diag* d) {
    return stage_impl<float>(c, X, Y, Z, st, stage, arg, dt, speed, d);
}
int oc_stage_f64(const oc_config* c, int X, int Y, int Z, oc_state* st, int stage, int arg, float dt, float speed, oc_diag* d) {
    return stage_impl<double>(c, X, Y, Z, st, stage, arg, dt, speed, d);
}

// The residual r - A pp of the projection's linear system for a given pressure correction pp:
// A and r are built in float from the state as the projection stage (density, then
// pressureProject's set-up) builds them; the products and the residual are formed in double.
// The state is not modified. out: max |r - A pp| and its L2 norm over sky cells, then max |r| and
// its L2 norm (the divergence before the projection).
int oc_projection_residual_f32(const oc_config* c, int X, int Y, int Z, const oc_state* st, const float* pp, float dt, double* out) {
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    Config cf = cfg_of(c);
    const int64_t N = g.n();
    std::vector<float> u(s.u, s.u + N), v(s.v, s.v + N), w(s.w, s.w + N), rho(s.rho, s.rho + N);
    s.u = u.data(); s.v = v.data(); s.w = w.data(); s.rho = rho.data();
    init_density(g, s);
    Amat<float> A;
    std::vector<float> r;
    build_system(g, cf, s, dt, A, r);
    const bool ref = cf.semantics == 0;
    double mx = 0, l2 = 0, bmx = 0, bl2 = 0;
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x) {
                if (g.ground(x, y, z)) continue;
                const int64_t idx = g.id(x, y, z);
                auto S = [&](int dx, int dy, int dz) {
                    const int xn = x + dx, yn = y + dy, zn = z + dz;
                    if (!g.inside(xn, yn, zn) || g.ground(xn, yn, zn)) return 0.0;
                    return double(pp[g.id(xn, yn, zn)]);
                };
                auto lower = [&](int dx, int dy, int dz, const std::vector<float>& arr) {
                    const int xn = x + dx, yn = y + dy, zn = z + dz;
                    if (!g.inside(xn, yn, zn) || g.ground(xn, yn, zn)) return 0.0;
                    const float a = arr[g.id(xn, yn, zn)];
                    return double(ref ? char_trunc(a) : a);
                };
                const double Ap = double(A.w[idx]) * pp[idx] + lower(-1, 0, 0, A.x) * S(-1, 0, 0) + lower(0, -1, 0, A.y) * S(0, -1, 0) +
                                  lower(0, 0, -1, A.z) * S(0, 0, -1) + double(A.x[idx]) * S(1, 0, 0) + double(A.y[idx]) * S(0, 1, 0) +
                                  double(A.z[idx]) * S(0, 0, 1);
                const double res = double(r[idx]) - Ap;
                mx = std::max(mx, std::fabs(res));
                l2 += res * res;
                bmx = std::max(bmx, std::fabs(double(r[idx])));
                bl2 += double(r[idx]) * double(r[idx]);
            }
    out[0] = mx; out[1] = std::sqrt(l2); out[2] = bmx; out[3] = std::sqrt(bl2);
    return 0;
}

// the microphysics stage with the region-summed process amounts (region: lo x,y,z then hi x,y,z)
int oc_micro_rates_f32(int X, int Y, int Z, oc_state* st, float dt, float speed, const int* region, double* out) {
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    static const Micro<float> M;
    RateRegion rr{{region[0], region[1], region[2]}, {region[3], region[4], region[5]}, {0}};
    microphysics_sky(g, s, dt, speed, M, &rr);
    for (int k = 0; k < 33; ++k) out[k] = rr.sums[k];
    return 0;
}

// editing (f32 state): returns 1 when the ground changed, 0 otherwise, -1 for a bad parameter
int oc_brush_f32(int X, int Y, int Z, oc_state* st, int param, float size, const int* pos, float smooth, float dt, float intensity,
                 float value, const float* dir, int erase, const float* pcol) {
    if (param < 0 || param > 8) return -1;
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    EditParams ep{param, value, {dir[0], dir[1], dir[2]}, erase};
    return brush(g, s, ep, size, pos, smooth, dt, intensity, pcol);
}

int oc_selection_f32(int X, int Y, int Z, oc_state* st, int param, const int* lo, const int* hi, float value, const float* dir, int erase,
                     const float* pcol) {
    if (param < 0 || param > 8) return -1;
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    EditParams ep{param, value, {dir[0], dir[1], dir[2]}, erase};
    return selection(g, s, ep, lo, hi, pcol);
}

int oc_editor_block_f32(int X, int Y, int Z, oc_state* st) {
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    editor_block(g, s);
    return 0;
}

int oc_reset_parameter_f32(int X, int Y, int Z, oc_state* st, int param, const float* pcol) {
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    reset_parameter(g, s, param, pcol);
    return 0;
}

// the buoyancy stage with its per-cell velocity change in dbg
int oc_buoyancy_dbg_f32(int X, int Y, int Z, oc_state* st, float dt, float* dbg) {
    State<float> s = unpack<float>(st);
    Grid g{X, Y, Z, s.gh};
    buoyancy(g, s, dt, dbg);
    return 0;
}
}  // extern "C"
