// Mixed-precision pressure solve: FP64 iterative refinement around an FP32 conjugate gradient
// preconditioned by a geometric multigrid V-cycle.
//
// The reference's projection (calculatePressureProject, Game/environment.cu:898-987) runs a
// Jacobi-preconditioned CG for at most 200 iterations, which at 512x256x512 leaves the residual
// far above any tight tolerance. This solver uses the textbook (symmetric) operator A of the
// projection and solves it to a relative FP64 residual of refine_tol:
//
//   x64 = 0
//   repeat: r = b - A x64 (FP64 arithmetic, FP64 norm)    until |r|/|b| <= refine_tol
//           solve A e = r with MG-PCG in FP32 (FP64 reductions) to |r_inner| <= inner_rtol |r|
//           x64 += e
//
// Multigrid: cell-centred, the hierarchy of the full grid (ground cells inactive: diagonal 0).
// Coarse face coefficient = 1/2 x (sum of the four fine coefficients of that face), the
// boundary share of the diagonal coarsens the same way; a degree-2 Chebyshev smoother before
// and after the coarse correction, sum restriction, injection prolongation; the coarsest level
// (<= 4096 cells) is relaxed in one block in shared memory. Equal pre/post smoothing keeps the preconditioner
// symmetric, as CG needs. All levels keep A's sign convention: off-diagonal face coefficients
// <= 0, diagonal = -(sum of the cell's six face coefficients) > 0 (symmetric positive definite).
#include "skt_internal.cuh"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace skt {

namespace {

constexpr float kOmega = 0.8f;  // damped Jacobi weight of the coarsest-level relaxation
// Degree-2 Chebyshev smoother on D^-1 A over [lmax/8, 1.05 lmax], lmax = 2 (D^-1 A of this
// diagonally dominant M-matrix has its spectrum in (0, 2]):
//   step A: x1 = x0 + (b - A x0)/(theta D)
//   step B: x2 = x1 + c1 (x1 - x0) + c2 (b - A x1)/D
// From x0 = 0 step A is x1 = b/(theta D). Pre- and post-smoothing use the same polynomial, so
// the V-cycle stays symmetric.
constexpr float kChebTheta = 1.175f;                 // (2.1 + 0.25)/2
constexpr float kChebC1 = 0.44900f;                  // rho1 rho0
constexpr float kChebC2 = 1.23319f;                  // 2 rho1 / delta
constexpr int kCoarseMax = 4096;
constexpr int kCoarseSweeps = 60;
constexpr int MBX = 32, MBY = 8;

struct LvlView {
    int X, Y, Z;
    const float *ax, *ay, *az, *aw;
};

__device__ __forceinline__ int lidx(const LvlView& L, int x, int y, int z) { return x + L.X * (y + L.Y * z); }

// (A v)_c with zero values outside the grid; face coefficients of a cell's upper faces are
// stored at the cell, the lower ones at the neighbour.
__device__ __forceinline__ float apply_A(const LvlView& L, const float* __restrict__ v, int x, int y, int z, int c) {
    float s = L.aw[c] * v[c];
    if (x > 0) s += L.ax[c - 1] * v[c - 1];
    if (x + 1 < L.X) s += L.ax[c] * v[c + 1];
    if (y > 0) s += L.ay[c - L.X] * v[c - L.X];
    if (y + 1 < L.Y) s += L.ay[c] * v[c + L.X];
    const int XY = L.X * L.Y;
    if (z > 0) s += L.az[c - XY] * v[c - XY];
    if (z + 1 < L.Z) s += L.az[c] * v[c + XY];
    return s;
}

inline dim3 lgrid(int X, int Y, int Z) { return dim3((X + MBX - 1) / MBX, (Y + MBY - 1) / MBY, Z); }

// Coarse operator from the fine one. Interior faces only: a fine coefficient on a face leaving
// the grid (possible on the finest level, where it carries the boundary share) counts as
// boundary.
__global__ void k_mg_coarsen(LvlView F, int CX, int CY, int CZ, float* __restrict__ cax, float* __restrict__ cay, float* __restrict__ caz,
                             float* __restrict__ caw) {
    const int I = blockIdx.x * MBX + threadIdx.x, J = blockIdx.y * MBY + threadIdx.y, K = blockIdx.z;
    if (I >= CX || J >= CY) return;
    const int XY = F.X * F.Y;
    auto fax = [&](int x, int y, int z) { return (x >= 0 && x + 1 < F.X) ? F.ax[x + F.X * (y + F.Y * z)] : 0.0f; };
    auto fay = [&](int x, int y, int z) { return (y >= 0 && y + 1 < F.Y) ? F.ay[x + F.X * (y + F.Y * z)] : 0.0f; };
    auto faz = [&](int x, int y, int z) { return (z >= 0 && z + 1 < F.Z) ? F.az[x + F.X * (y + F.Y * z)] : 0.0f; };
    float px = 0, mx = 0, py = 0, my = 0, pz = 0, mz = 0, E = 0;
    for (int b = 0; b < 2; ++b)
        for (int d = 0; d < 2; ++d) {
            px += fax(2 * I + 1, 2 * J + b, 2 * K + d);
            mx += fax(2 * I - 1, 2 * J + b, 2 * K + d);
            py += fay(2 * I + b, 2 * J + 1, 2 * K + d);
            my += fay(2 * I + b, 2 * J - 1, 2 * K + d);
            pz += faz(2 * I + b, 2 * J + d, 2 * K + 1);
            mz += faz(2 * I + b, 2 * J + d, 2 * K - 1);
        }
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) {
                const int x = 2 * I + a, y = 2 * J + b, z = 2 * K + d;
                const int c = x + F.X * (y + F.Y * z);
                // diag = -(sum of the six face coefficients, boundary faces included), so the
                // boundary share is diag + (sum of the interior-face coefficients) >= 0
                const float interior = fax(x, y, z) + fax(x - 1, y, z) + fay(x, y, z) + fay(x, y - 1, z) + faz(x, y, z) + faz(x, y, z - 1);
                E += F.aw[c] + interior;
            }
    (void)XY;
    const int c = I + CX * (J + CY * K);
    const float ax_ = 0.5f * px, ay_ = 0.5f * py, az_ = 0.5f * pz;
    cax[c] = (I + 1 < CX) ? ax_ : 0.0f;
    cay[c] = (J + 1 < CY) ? ay_ : 0.0f;
    caz[c] = (K + 1 < CZ) ? az_ : 0.0f;
    caw[c] = 0.5f * E - (0.5f * px + 0.5f * mx + 0.5f * py + 0.5f * my + 0.5f * pz + 0.5f * mz);
}

// one smoother step: out = in + c1 (in - prev) + c2 (b - A in)/diag (prev may be null = 0);
// FIRST: out = b/(theta diag) (step A from zero). Inactive cells (diag 0) get 0.
template <bool FIRST>
__global__ void k_mg_jacobi(LvlView L, const float* __restrict__ in, const float* __restrict__ prev, float* __restrict__ out,
                            const float* __restrict__ b, float c1, float c2, const int* skip) {
    if (skip && *skip) return;
    const int x = blockIdx.x * MBX + threadIdx.x, y = blockIdx.y * MBY + threadIdx.y, z = blockIdx.z;
    if (x >= L.X || y >= L.Y) return;
    const int c = lidx(L, x, y, z);
    const float d = L.aw[c];
    if (d == 0.0f) { out[c] = 0.0f; return; }
    if (FIRST) { out[c] = __fdividef(b[c], kChebTheta * d); return; }
    const float v = in[c];
    const float pv = prev ? prev[c] : 0.0f;
    out[c] = v + c1 * (v - pv) + c2 * __fdividef(b[c] - apply_A(L, in, x, y, z, c), d);
}

// coarse right-hand side: the sum of the residuals of the eight children
__global__ void k_mg_restrict(LvlView F, const float* __restrict__ x, const float* __restrict__ b, int CX, int CY, int CZ,
                              float* __restrict__ cb, const int* skip) {
    if (skip && *skip) return;
    const int I = blockIdx.x * MBX + threadIdx.x, J = blockIdx.y * MBY + threadIdx.y, K = blockIdx.z;
    if (I >= CX || J >= CY) return;
    float s = 0.0f;
    for (int d = 0; d < 2; ++d)
        for (int bb = 0; bb < 2; ++bb)
            for (int a = 0; a < 2; ++a) {
                const int fx = 2 * I + a, fy = 2 * J + bb, fz = 2 * K + d;
                const int c = lidx(F, fx, fy, fz);
                if (F.aw[c] == 0.0f) continue;
                s += b[c] - apply_A(F, x, fx, fy, fz, c);
            }
    cb[I + CX * (J + CY * K)] = s;
}

// x += P e (injection of the parent's correction)
__global__ void k_mg_prolong(LvlView F, float* __restrict__ x, int CX, int CY, const float* __restrict__ ce, const int* skip) {
    if (skip && *skip) return;
    const int fx = blockIdx.x * MBX + threadIdx.x, fy = blockIdx.y * MBY + threadIdx.y, fz = blockIdx.z;
    if (fx >= F.X || fy >= F.Y) return;
    const int c = lidx(F, fx, fy, fz);
    if (F.aw[c] == 0.0f) return;
    x[c] += ce[(fx >> 1) + CX * ((fy >> 1) + CY * (fz >> 1))];
}

// the coarsest level: kCoarseSweeps damped Jacobi sweeps from zero, one block of kCoarseThreads;
// each thread keeps its (up to kCoarsePer) cells' seven coefficients in registers for all sweeps,
// the iterate lives in shared memory (a missing neighbour has coefficient 0; its index is only
// clamped into the level, the value read there is finite and multiplied by 0)
constexpr int kCoarseThreads = 1024, kCoarsePer = kCoarseMax / kCoarseThreads;
__global__ void __launch_bounds__(kCoarseThreads) k_mg_coarse(LvlView L, const float* __restrict__ b, float* __restrict__ x, const int* skip) {
    if (skip && *skip) return;
    extern __shared__ float sm[];
    const int n = L.X * L.Y * L.Z, XY = L.X * L.Y;
    float* xa = sm;
    float* xb = sm + n;
    float cw[kCoarsePer], cl[kCoarsePer], cr[kCoarsePer], cd[kCoarsePer], cu[kCoarsePer], cbk[kCoarsePer], cf[kCoarsePer], bv[kCoarsePer];
    int ci[kCoarsePer];
#pragma unroll
    for (int k = 0; k < kCoarsePer; ++k) {
        const int c = threadIdx.x + k * kCoarseThreads;
        const bool v = c < n;
        const int cc = v ? c : 0;
        const int xx = cc % L.X, yy = (cc / L.X) % L.Y, zz = cc / XY;
        ci[k] = cc;
        cw[k] = v ? L.aw[cc] : 0.0f;
        bv[k] = v ? b[cc] : 0.0f;
        cl[k] = (v && xx > 0) ? L.ax[cc - 1] : 0.0f;
        cr[k] = (v && xx + 1 < L.X) ? L.ax[cc] : 0.0f;
        cd[k] = (v && yy > 0) ? L.ay[cc - L.X] : 0.0f;
        cu[k] = (v && yy + 1 < L.Y) ? L.ay[cc] : 0.0f;
        cbk[k] = (v && zz > 0) ? L.az[cc - XY] : 0.0f;
        cf[k] = (v && zz + 1 < L.Z) ? L.az[cc] : 0.0f;
    }
    for (int i = threadIdx.x; i < n; i += kCoarseThreads) xa[i] = 0.0f;
    __syncthreads();
    for (int it = 0; it < kCoarseSweeps; ++it) {
#pragma unroll
        for (int k = 0; k < kCoarsePer; ++k) {
            if (threadIdx.x + k * kCoarseThreads >= n) break;
            const int c = ci[k];
            const float d = cw[k];
            const float xc = xa[c];
            const float ax_ = d * xc + cl[k] * xa[max(c - 1, 0)] + cr[k] * xa[min(c + 1, n - 1)] + cd[k] * xa[max(c - L.X, 0)] +
                              cu[k] * xa[min(c + L.X, n - 1)] + cbk[k] * xa[max(c - XY, 0)] + cf[k] * xa[min(c + XY, n - 1)];
            xb[c] = d == 0.0f ? 0.0f : xc + kOmega * __fdividef(bv[k] - ax_, d);
        }
        __syncthreads();
        float* t = xa; xa = xb; xb = t;
    }
    for (int i = threadIdx.x; i < n; i += kCoarseThreads) x[i] = xa[i];
}

// ---- refinement / CG helpers (1D over all cells) ---------------------------------------------

constexpr int RT = 256;

template <int NTH>
__device__ __forceinline__ double bsum(double v, double* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (NTH / 32) ? sm[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;
}
template <int NTH>
__device__ __forceinline__ float bmax(float v, float* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = 0.0f;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (NTH / 32) ? sm[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    }
    return t;
}
// last-block reduction of per-block (sum, max) partials; true in thread 0 of the last block
__device__ __forceinline__ bool finish(Scalars* sc, double* partials, double sum, float mx, double& tot, float& mall) {
    __shared__ bool last;
    __shared__ double sd[RT / 32];
    __shared__ float sf[RT / 32];
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = sum;
        partials[kMaxPartials + blockIdx.x] = double(mx);
        __threadfence();
        last = atomicAdd(&sc->done_blocks, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    float m = 0.0f;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) {
        s += __ldcg(partials + b);
        const float mb = float(__ldcg(partials + kMaxPartials + b));
        m = mb > m ? mb : m;
    }
    const double ts = bsum<RT>(s, sd);
    const float tm = bmax<RT>(m, sf);
    if (threadIdx.x == 0) {
        tot = ts;
        mall = tm;
        sc->done_blocks = 0;
        note_nonfinite(sc, ts);
    }
    return threadIdx.x == 0;
}

// ---- float-float refinement vector ----------------------------------------------------------
// The refinement's solution is kept as an unevaluated sum x = xh + xl of two floats (about 48
// significant bits) and its residual b - A x is formed with error-free transformations (Knuth's
// two-sum and the fma-based exact product), so the outer loop converges far below FP32 rounding
// on the FP32 pipes; the FP64 rate of this chip is a small fraction of its FP32 rate.

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}

struct FF {  // running float-float sum of products a * (xh + xl)
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void add_prod(float a, float xh, float xl) {
        const float p = a * xh;
        const float pe = fmaf(a, xh, -p);  // a*xh - p exactly
        float sh, se;
        two_sum(h, p, sh, se);
        h = sh;
        l += se + fmaf(a, xl, pe);
    }
};

// b - (h + l), rounded once to float
__device__ __forceinline__ float ff_resid(float b, const FF& acc) {
    float d, e;
    two_sum(b, -acc.h, d, e);
    return d + (e - acc.l);
}

// the refinement bookkeeping once |r|^2 and max|r| are known (first call: x = 0, r = b)
__device__ __forceinline__ void refine_record(Scalars* sc, double tot, float mall, float refine_tol, int first) {
    if (first) sc->rnorm0 = sqrt(tot);
    sc->rnorm = sqrt(tot);
    sc->residual = mall;
    const bool done = sc->rnorm0 == 0.0 || sc->rnorm <= double(refine_tol) * sc->rnorm0;
    sc->refine_done = done ? 1 : 0;
    sc->inner_tol = mall;  // the inner solves reduce the max residual relative to this
}

// r = b - A (xh + xl) in float-float, |r|^2 (compensated FP32 per thread, FP64 across threads)
// and max|r|; any grid
__global__ void __launch_bounds__(RT) k_resid_ff(Grid g, const float* __restrict__ ax, const float* __restrict__ ay, const float* __restrict__ az,
                                                 const float* __restrict__ aw, const float* __restrict__ xh, const float* __restrict__ xl,
                                                 const float* __restrict__ b, float* __restrict__ r, float refine_tol, int first, Scalars* sc,
                                                 double* partials) {
    __shared__ double smd[RT / 32];
    float acc = 0.0f, comp = 0.0f, mx = 0.0f;
    for (int c = blockIdx.x * RT + threadIdx.x; c < g.N; c += gridDim.x * RT) {
        float rv = 0.0f;
        if (aw[c] != 0.0f) {
            const int xx = c % g.X, yy = (c / g.X) % g.Y, zz = c / g.XY;
            FF s;
            s.add_prod(aw[c], xh[c], xl[c]);
            if (xx > 0) s.add_prod(ax[c - 1], xh[c - 1], xl[c - 1]);
            if (xx + 1 < g.X) s.add_prod(ax[c], xh[c + 1], xl[c + 1]);
            if (yy > 0) s.add_prod(ay[c - g.X], xh[c - g.X], xl[c - g.X]);
            if (yy + 1 < g.Y) s.add_prod(ay[c], xh[c + g.X], xl[c + g.X]);
            if (zz > 0) s.add_prod(az[c - g.XY], xh[c - g.XY], xl[c - g.XY]);
            if (zz + 1 < g.Z) s.add_prod(az[c], xh[c + g.XY], xl[c + g.XY]);
            rv = ff_resid(b[c], s);
        }
        r[c] = rv;
        const float yv = rv * rv - comp;
        const float tt = acc + yv;
        comp = (tt - acc) - yv;
        acc = tt;
        mx = fmaxf(mx, fabsf(rv));
    }
    const double bs = bsum<RT>(double(acc) - double(comp), smd);
    __shared__ float smf[RT / 32];
    const float bm = bmax<RT>(mx, smf);  // the block's max |r| (finish publishes thread 0's value)
    double tot;
    float mall;
    if (finish(sc, partials, bs, bm, tot, mall)) refine_record(sc, tot, mall, refine_tol, first);
}

// (xh, xl) += e and e = 0
__global__ void __launch_bounds__(RT) k_accum_ff(int n, float* __restrict__ xh, float* __restrict__ xl, float* __restrict__ e) {
    for (int c = blockIdx.x * RT + threadIdx.x; c < n; c += gridDim.x * RT) {
        float sh, se;
        two_sum(xh[c], e[c], sh, se);
        se += xl[c];
        const float h = sh + se;
        xh[c] = h;
        xl[c] = se - (h - sh);
        e[c] = 0.0f;
    }
}

__global__ void __launch_bounds__(RT) k_cast_ff(int n, const float* __restrict__ xh, const float* __restrict__ xl, float* __restrict__ p) {
    for (int c = blockIdx.x * RT + threadIdx.x; c < n; c += gridDim.x * RT) p[c] = xh[c] + xl[c];
}

// inner CG: rho = z.r (FP64) and s = z (start), or beta = rho_new/rho and s = z + beta s
template <bool START>
__global__ void __launch_bounds__(RT) k_zr_search(int n, const float* __restrict__ z, const float* __restrict__ r, float* __restrict__ s,
                                                  Scalars* sc, double* partials) {
    if (!START && sc->converged) return;
    // pass 1 of 2: the dot product; the search update runs in k_search_mg after beta is known
    __shared__ double smd[RT / 32];
    double acc = 0.0;
    for (int c = blockIdx.x * RT + threadIdx.x; c < n; c += gridDim.x * RT) {
        acc += double(z[c]) * double(r[c]);
        if (START) s[c] = z[c];
    }
    const double bs = bsum<RT>(acc, smd);
    double tot;
    float mall;
    if (finish(sc, partials, bs, 0.0f, tot, mall)) {
        if (START) {
            sc->sigma0 = tot;
            sc->converged = 0;
            sc->iters = 0;
        } else {
            sc->beta_f = float(tot / sc->sigma0);
            sc->sigma0 = tot;
        }
    }
}

__global__ void __launch_bounds__(RT) k_search_mg(int n, const float* __restrict__ z, float* __restrict__ s, const Scalars* sc) {
    if (sc->converged) return;
    const float beta = sc->beta_f;
    for (int c = blockIdx.x * RT + threadIdx.x; c < n; c += gridDim.x * RT) s[c] = z[c] + beta * s[c];
}

// As = A s and s.As -> alpha = rho / s.As
__global__ void __launch_bounds__(RT) k_matvec_mg(Grid g, const float* __restrict__ ax, const float* __restrict__ ay, const float* __restrict__ az,
                                                  const float* __restrict__ aw, const float* __restrict__ s, float* __restrict__ As,
                                                  Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[RT / 32];
    LvlView L{g.X, g.Y, g.Z, ax, ay, az, aw};
    double acc = 0.0;
    for (int c = blockIdx.x * RT + threadIdx.x; c < g.N; c += gridDim.x * RT) {
        float v = 0.0f;
        if (aw[c] != 0.0f) {
            const int xx = c % g.X, yy = (c / g.X) % g.Y, zz = c / g.XY;
            v = apply_A(L, s, xx, yy, zz, c);
        }
        As[c] = v;
        acc += double(v) * double(s[c]);
    }
    const double bs = bsum<RT>(acc, smd);
    double tot;
    float mall;
    if (finish(sc, partials, bs, 0.0f, tot, mall)) {
        sc->sigma1 = tot;
        sc->alpha = float(sc->sigma0 / tot);
    }
}

// e += alpha s; r -= alpha As; stop when max|r| <= inner_rtol * (max residual at entry)
__global__ void __launch_bounds__(RT) k_update_mg(int n, const float* __restrict__ s, const float* __restrict__ As, float* __restrict__ e,
                                                  float* __restrict__ r, float inner_rtol, int max_iter, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ float smf[RT / 32];
    const float alpha = sc->alpha;
    float mx = 0.0f;
    for (int c = blockIdx.x * RT + threadIdx.x; c < n; c += gridDim.x * RT) {
        e[c] += alpha * s[c];
        const float rv = r[c] - alpha * As[c];
        r[c] = rv;
        const float m = fabsf(rv);
        if (m > mx) mx = m;
    }
    const float bm = bmax<RT>(mx, smf);
    double tot;
    float mall;
    if (finish(sc, partials, 0.0, bm, tot, mall)) {
        sc->iters += 1;
        sc->outer_inner_total += 1;
        if (mall <= inner_rtol * sc->inner_tol) sc->converged = 1;
        else if (sc->iters >= max_iter) sc->converged = 2;
    }
}

// ---- vector levels (X % 4 == 0) -------------------------------------------------------------

constexpr int JVY = 8;  // rows per block: the rows above and below come mostly from L1

// The vector levels (X % 4 == 0) run every V-cycle step as one float4 z march: a thread owns
// four consecutive x cells of one (y) row and walks a run of z planes, keeping the input vector
// of planes z-1, z, z+1 and the back-face coefficients in registers. Neighbouring rows come from
// the block's other warps through L1, the x edges from the lanes beside it (warp shuffles).
// Coefficients are FP32 or, on the finest level, FP16 copies (4 halves = 8 bytes per 4 cells).

__device__ __forceinline__ float4 ld4(const float* p, int c) { return *reinterpret_cast<const float4*>(p + c); }
struct alignas(8) H4 { __half2 a, b; };
__device__ __forceinline__ float4 ld4(const __half* p, int c) {
    const H4 h = *reinterpret_cast<const H4*>(p + c);
    const float2 a = __half22float2(h.a), b = __half22float2(h.b);
    return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float ld1(const float* p, int c) { return p[c]; }
__device__ __forceinline__ float ld1(const __half* p, int c) { return __half2float(p[c]); }
__device__ __forceinline__ float comp4(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }
__device__ __forceinline__ void set4(float4& v, int k, float a) {
    if (k == 0) v.x = a; else if (k == 1) v.y = a; else if (k == 2) v.z = a; else v.w = a;
}

enum { SM_PRE = 0, SM_POSTA = 1, SM_POSTB = 2 };
enum { DOT_NONE = 0, DOT_START = 1, DOT_NEXT = 2 };

// Divisions by the diagonal use the fast divide: the preconditioner only has to be a fixed
// symmetric operator, and a deterministic approximate D^-1 keeps it one.
// The smoother's input vector u as seen by the stencil:
//   SM_PRE   u = b / (theta diag)       (step A of the Chebyshev smoother from zero, on the fly)
//   SM_POSTA u = x + P e_coarse         (the coarse correction, injected on the fly)
//   SM_POSTB u = x2                     (the output of step A)
// Values at inactive cells do not matter: every face coefficient that touches an inactive cell
// is 0 on every level (ground faces have coefficient 0 and coarsening sums them).
template <int MODE, class CT>
struct UIn {
    const float* v;
    const CT* aw;
    const float* ce;
    int CX, CY;
    __device__ __forceinline__ float4 row(int c, int x0, int y, int z) const {
        const float4 a = ld4(v, c);
        if (MODE == SM_PRE) {
            const float4 d = ld4(aw, c);
            return make_float4(d.x == 0.0f ? 0.0f : __fdividef(a.x, kChebTheta * d.x), d.y == 0.0f ? 0.0f : __fdividef(a.y, kChebTheta * d.y),
                               d.z == 0.0f ? 0.0f : __fdividef(a.z, kChebTheta * d.z), d.w == 0.0f ? 0.0f : __fdividef(a.w, kChebTheta * d.w));
        }
        if (MODE == SM_POSTA) {
            const float2 e = *reinterpret_cast<const float2*>(ce + (x0 >> 1) + CX * ((y >> 1) + CY * (z >> 1)));
            return make_float4(a.x + e.x, a.y + e.x, a.z + e.y, a.w + e.y);
        }
        return a;
    }
    __device__ __forceinline__ float one(int c, int xx, int y, int z) const {
        const float a = v[c];
        if (MODE == SM_PRE) {
            const float d = ld1(aw, c);
            return d == 0.0f ? 0.0f : __fdividef(a, kChebTheta * d);
        }
        if (MODE == SM_POSTA) return a + ce[(xx >> 1) + CX * ((y >> 1) + CY * (z >> 1))];
        return a;
    }
};

// block-wide sum over NTH threads with a linear thread id; the total is valid in tid 0
template <int NTH>
__device__ __forceinline__ double bsum_t(double v, double* sm, int tid) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) sm[tid >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (tid < 32) {
        t = tid < (NTH / 32) ? sm[tid] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;
}
// last-block reduction of one FP64 partial per block of a 3D grid; true in tid 0 of the last block
template <int NTH>
__device__ __forceinline__ bool finish_sum(Scalars* sc, double* partials, double sum, double& tot, int tid) {
    __shared__ bool last;
    __shared__ double sd[NTH / 32];
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int nblk = gridDim.x * gridDim.y * gridDim.z;
    if (tid == 0) {
        partials[bid] = sum;
        __threadfence();
        last = atomicAdd(&sc->done_blocks, 1u) == unsigned(nblk) - 1u;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    for (int b = tid; b < nblk; b += NTH) s += __ldcg(partials + b);
    const double ts = bsum_t<NTH>(s, sd, tid);
    if (tid == 0) {
        tot = ts;
        sc->done_blocks = 0;
        note_nonfinite(sc, ts);
    }
    return tid == 0;
}

// finish_sum with a max as well: mx is each thread's own max, reduced over the block here
// (partials[kMaxPartials + bid] holds the block maxima)
template <int NTH>
__device__ __forceinline__ bool finish_sum_max(Scalars* sc, double* partials, double sum, float mx, double& tot, float& mall, int tid) {
    __shared__ bool last;
    __shared__ double sd[NTH / 32];
    __shared__ float sf[NTH / 32];
    __shared__ float sb[NTH / 32];
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int nblk = gridDim.x * gridDim.y * gridDim.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) sb[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0)
        for (int w = 1; w < NTH / 32; ++w) mx = fmaxf(mx, sb[w]);
    if (tid == 0) {
        partials[bid] = sum;
        partials[kMaxPartials + bid] = double(mx);
        __threadfence();
        last = atomicAdd(&sc->done_blocks, 1u) == unsigned(nblk) - 1u;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    float m = 0.0f;
    for (int b = tid; b < nblk; b += NTH) {
        s += __ldcg(partials + b);
        m = fmaxf(m, float(__ldcg(partials + kMaxPartials + b)));
    }
    const double ts = bsum_t<NTH>(s, sd, tid);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __syncthreads();
    if ((tid & 31) == 0) sf[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int w = 0; w < NTH / 32; ++w) t = fmaxf(t, sf[w]);
        tot = ts;
        mall = t;
        sc->done_blocks = 0;
        note_nonfinite(sc, ts);
    }
    return tid == 0;
}

// (A u) at the four cells of a row from the z-march registers
struct Stencil4 {
    float4 a;
    __device__ __forceinline__ Stencil4(float4 cw, float4 cx, float4 cy, float4 ayd, float4 azb, float4 cz, float axl, float4 vc,
                                        float vl, float vr, float4 vd, float4 vu, float4 vb, float4 vf) {
        a.x = cw.x * vc.x + axl * vl + ayd.x * vd.x + azb.x * vb.x + cx.x * vc.y + cy.x * vu.x + cz.x * vf.x;
        a.y = cw.y * vc.y + cx.x * vc.x + ayd.y * vd.y + azb.y * vb.y + cx.y * vc.z + cy.y * vu.y + cz.y * vf.y;
        a.z = cw.z * vc.z + cx.y * vc.y + ayd.z * vd.z + azb.z * vb.z + cx.z * vc.w + cy.z * vu.z + cz.z * vf.z;
        a.w = cw.w * vc.w + cx.z * vc.z + ayd.w * vd.w + azb.w * vb.w + cx.w * vr + cy.w * vu.w + cz.w * vf.w;
    }
};

// One smoother step out = u + k1 (u - prev) + k2 (b - A u)/diag on a vector level (inactive
// cells get 0), u per MODE (see UIn); prev = 0 for SM_PRE (the step from zero), x + P e for
// SM_POSTB, unused for SM_POSTA (k1 = 0). SM_POSTB may write over x (prev is read at the cell
// being written only). DOT forms z.r (r = b) of the finest level's output for the CG:
// DOT_START sets sigma0 and restarts the iteration count, DOT_NEXT sets beta = rho_new/rho.
template <int MODE, int DOT, class CT>
__global__ void __launch_bounds__(32 * JVY, 32 / JVY) k_mg_smooth4(int X, int Y, int Z, int zlen, const CT* __restrict__ ax, const CT* __restrict__ ay,
                                                         const CT* __restrict__ az, const CT* __restrict__ aw, const float* __restrict__ b,
                                                         UIn<MODE, CT> U, UIn<SM_POSTA, CT> Pv, float* out, float k1, float k2,
                                                         const int* skip, Scalars* sc, double* partials) {
    if (skip && *skip) return;
    const int lane = threadIdx.x, tid = threadIdx.x + 32 * threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * JVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, Z);
    const bool act = x0 < X && y < Y;
    const int XY = X * Y;
    const int row = x0 + y * X;
    const float4 z4 = make_float4(0, 0, 0, 0);
    float4 vb = z4, vc = z4, azb = z4;
    if (act) {
        vc = U.row(row + zs * XY, x0, y, zs);
        if (zs > 0) { vb = U.row(row + (zs - 1) * XY, x0, y, zs - 1); azb = ld4(az, row + (zs - 1) * XY); }
    }
    float acc = 0.0f, comp = 0.0f;
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 vf = z4, vd = z4, vu = z4, ayd = z4, cx = z4, cy = z4, cz = z4, cw = z4, bb = z4;
        if (act) {
            if (z + 1 < Z) vf = U.row(c + XY, x0, y, z + 1);
            if (y > 0) { vd = U.row(c - X, x0, y - 1, z); ayd = ld4(ay, c - X); }
            if (y + 1 < Y) vu = U.row(c + X, x0, y + 1, z);
            cx = ld4(ax, c); cy = ld4(ay, c); cz = ld4(az, c); cw = ld4(aw, c); bb = ld4(b, c);
        }
        float vl = __shfl_up_sync(0xffffffffu, vc.w, 1);
        float axl = __shfl_up_sync(0xffffffffu, cx.w, 1);
        float vr = __shfl_down_sync(0xffffffffu, vc.x, 1);
        if (act && lane == 0) {
            if (x0 > 0) { vl = U.one(c - 1, x0 - 1, y, z); axl = ld1(ax, c - 1); } else { vl = 0.0f; axl = 0.0f; }
        }
        if (act && (lane == 31 || x0 + 4 >= X)) vr = (x0 + 4 < X) ? U.one(c + 4, x0 + 4, y, z) : 0.0f;
        if (act) {
            const float4 a = Stencil4(cw, cx, cy, ayd, azb, cz, axl, vc, vl, vr, vd, vu, vb, vf).a;
            const float4 pv = MODE == SM_POSTB ? Pv.row(c, x0, y, z) : z4;
            float4 o;
            o.x = cw.x == 0.0f ? 0.0f : vc.x + k1 * (vc.x - pv.x) + k2 * __fdividef(bb.x - a.x, cw.x);
            o.y = cw.y == 0.0f ? 0.0f : vc.y + k1 * (vc.y - pv.y) + k2 * __fdividef(bb.y - a.y, cw.y);
            o.z = cw.z == 0.0f ? 0.0f : vc.z + k1 * (vc.z - pv.z) + k2 * __fdividef(bb.z - a.z, cw.z);
            o.w = cw.w == 0.0f ? 0.0f : vc.w + k1 * (vc.w - pv.w) + k2 * __fdividef(bb.w - a.w, cw.w);
            *reinterpret_cast<float4*>(out + c) = o;
            if (DOT != DOT_NONE) {
                const float t = o.x * bb.x + o.y * bb.y + o.z * bb.z + o.w * bb.w;
                const float yv = t - comp;
                const float tt = acc + yv;
                comp = (tt - acc) - yv;
                acc = tt;
            }
        }
        vb = vc;
        vc = vf;
        azb = cz;
    }
    if (DOT != DOT_NONE) {
        __shared__ double smd[JVY];
        const double bs = bsum_t<32 * JVY>(double(acc) - double(comp), smd, tid);
        double tot;
        if (finish_sum<32 * JVY>(sc, partials, bs, tot, tid)) {
            if (DOT == DOT_START) {
                sc->sigma0 = tot;
                sc->beta_f = 0.0f;
                sc->converged = 0;
                sc->iters = 0;
            } else {
                sc->beta_f = float(tot / sc->sigma0);
                sc->sigma0 = tot;
            }
        }
    }
}

// Coarse right-hand side of a vector level: each coarse cell gets the sum of b - A x over its
// eight children. zlen, the z offset of every block, Y and JVY are even: a thread sums its row's
// x pairs over two planes, then the even row of each row pair adds its partner's sums.
template <class CT>
__global__ void __launch_bounds__(32 * JVY, 32 / JVY) k_mg_restrict4(int X, int Y, int Z, int zlen, const CT* __restrict__ ax, const CT* __restrict__ ay,
                                                           const CT* __restrict__ az, const CT* __restrict__ aw, const float* __restrict__ x,
                                                           const float* __restrict__ b, int CX, int CY, float* __restrict__ cb, const int* skip) {
    if (skip && *skip) return;
    __shared__ float2 part[JVY][32];
    const int lane = threadIdx.x;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * JVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, Z);
    const bool act = x0 < X && y < Y;
    const int XY = X * Y;
    const int row = x0 + y * X;
    const float4 z4 = make_float4(0, 0, 0, 0);
    float4 vb = z4, vc = z4, azb = z4;
    if (act) {
        vc = ld4(x, row + zs * XY);
        if (zs > 0) { vb = ld4(x, row + (zs - 1) * XY); azb = ld4(az, row + (zs - 1) * XY); }
    }
    float2 acc = make_float2(0.0f, 0.0f);
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 vf = z4, vd = z4, vu = z4, ayd = z4, cx = z4, cy = z4, cz = z4, cw = z4, bb = z4;
        if (act) {
            if (z + 1 < Z) vf = ld4(x, c + XY);
            if (y > 0) { vd = ld4(x, c - X); ayd = ld4(ay, c - X); }
            if (y + 1 < Y) vu = ld4(x, c + X);
            cx = ld4(ax, c); cy = ld4(ay, c); cz = ld4(az, c); cw = ld4(aw, c); bb = ld4(b, c);
        }
        float vl = __shfl_up_sync(0xffffffffu, vc.w, 1);
        float axl = __shfl_up_sync(0xffffffffu, cx.w, 1);
        float vr = __shfl_down_sync(0xffffffffu, vc.x, 1);
        if (act && lane == 0) {
            if (x0 > 0) { vl = x[c - 1]; axl = ld1(ax, c - 1); } else { vl = 0.0f; axl = 0.0f; }
        }
        if (act && (lane == 31 || x0 + 4 >= X)) vr = (x0 + 4 < X) ? x[c + 4] : 0.0f;
        if (act) {
            const float4 a = Stencil4(cw, cx, cy, ayd, azb, cz, axl, vc, vl, vr, vd, vu, vb, vf).a;
            acc.x += (cw.x == 0.0f ? 0.0f : bb.x - a.x) + (cw.y == 0.0f ? 0.0f : bb.y - a.y);
            acc.y += (cw.z == 0.0f ? 0.0f : bb.z - a.z) + (cw.w == 0.0f ? 0.0f : bb.w - a.w);
        }
        if (z & 1) {
            part[threadIdx.y][lane] = acc;
            __syncthreads();
            if (act && (threadIdx.y & 1) == 0) {
                const float2 o = part[threadIdx.y + 1][lane];
                *reinterpret_cast<float2*>(cb + (x0 >> 1) + CX * ((y >> 1) + CY * (z >> 1))) = make_float2(acc.x + o.x, acc.y + o.y);
            }
            __syncthreads();
            acc = make_float2(0.0f, 0.0f);
        }
        vb = vc;
        vc = vf;
        azb = cz;
    }
}

// CG search step fused with the operator: s_new = z + beta s_old (beta = 0: s_new = z, s_old
// is not read), As = A s_new with the FP32 finest coefficients, s_new.As -> alpha = rho/(s.As)
__global__ void __launch_bounds__(32 * JVY, 32 / JVY) k_mg_matvec_search4(int X, int Y, int Z, int zlen, const float* __restrict__ ax,
                                                                const float* __restrict__ ay, const float* __restrict__ az,
                                                                const float* __restrict__ aw, const float* __restrict__ zv,
                                                                const float* __restrict__ sold, float* __restrict__ snew,
                                                                float* __restrict__ As, Scalars* sc, double* partials) {
    if (sc->converged) return;
    const float beta = sc->beta_f;
    const bool old = beta != 0.0f;
    const int lane = threadIdx.x, tid = threadIdx.x + 32 * threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * JVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, Z);
    const bool act = x0 < X && y < Y;
    const int XY = X * Y;
    const int row = x0 + y * X;
    const float4 z4 = make_float4(0, 0, 0, 0);
    auto srow = [&](int c) {
        float4 v = ld4(zv, c);
        if (old) {
            const float4 s = ld4(sold, c);
            v.x += beta * s.x; v.y += beta * s.y; v.z += beta * s.z; v.w += beta * s.w;
        }
        return v;
    };
    auto sone = [&](int c) { return old ? zv[c] + beta * sold[c] : zv[c]; };
    float4 vb = z4, vc = z4, azb = z4;
    if (act) {
        vc = srow(row + zs * XY);
        if (zs > 0) { vb = srow(row + (zs - 1) * XY); azb = ld4(az, row + (zs - 1) * XY); }
    }
    float acc = 0.0f, comp = 0.0f;
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 vf = z4, vd = z4, vu = z4, ayd = z4, cx = z4, cy = z4, cz = z4, cw = z4;
        if (act) {
            if (z + 1 < Z) vf = srow(c + XY);
            if (y > 0) { vd = srow(c - X); ayd = ld4(ay, c - X); }
            if (y + 1 < Y) vu = srow(c + X);
            cx = ld4(ax, c); cy = ld4(ay, c); cz = ld4(az, c); cw = ld4(aw, c);
        }
        float vl = __shfl_up_sync(0xffffffffu, vc.w, 1);
        float axl = __shfl_up_sync(0xffffffffu, cx.w, 1);
        float vr = __shfl_down_sync(0xffffffffu, vc.x, 1);
        if (act && lane == 0) {
            if (x0 > 0) { vl = sone(c - 1); axl = ax[c - 1]; } else { vl = 0.0f; axl = 0.0f; }
        }
        if (act && (lane == 31 || x0 + 4 >= X)) vr = (x0 + 4 < X) ? sone(c + 4) : 0.0f;
        if (act) {
            float4 a = Stencil4(cw, cx, cy, ayd, azb, cz, axl, vc, vl, vr, vd, vu, vb, vf).a;
            if (cw.x == 0.0f) a.x = 0.0f;
            if (cw.y == 0.0f) a.y = 0.0f;
            if (cw.z == 0.0f) a.z = 0.0f;
            if (cw.w == 0.0f) a.w = 0.0f;
            *reinterpret_cast<float4*>(snew + c) = vc;
            *reinterpret_cast<float4*>(As + c) = a;
            const float t = a.x * vc.x + a.y * vc.y + a.z * vc.z + a.w * vc.w;
            const float yv = t - comp;
            const float tt = acc + yv;
            comp = (tt - acc) - yv;
            acc = tt;
        }
        vb = vc;
        vc = vf;
        azb = cz;
    }
    __shared__ double smd[JVY];
    const double bs = bsum_t<32 * JVY>(double(acc) - double(comp), smd, tid);
    double tot;
    if (finish_sum<32 * JVY>(sc, partials, bs, tot, tid)) {
        sc->sigma1 = tot;
        sc->alpha = float(sc->sigma0 / tot);
    }
}

// r = b - A (xh + xl) in float-float on a vector level: the z march of k_mg_matvec_search4 over
// the pair (xh, xl), |r|^2 and max|r| reduced as in k_resid_ff
__global__ void __launch_bounds__(32 * JVY) k_resid_ff4(int X, int Y, int Z, int zlen, const float* __restrict__ ax, const float* __restrict__ ay,
                                                        const float* __restrict__ az, const float* __restrict__ aw, const float* __restrict__ xh,
                                                        const float* __restrict__ xl, const float* __restrict__ b, float* __restrict__ r,
                                                        float refine_tol, int first, Scalars* sc, double* partials) {
    const int lane = threadIdx.x, tid = threadIdx.x + 32 * threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * JVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, Z);
    const bool act = x0 < X && y < Y;
    const int XY = X * Y;
    const int row = x0 + y * X;
    const float4 z4 = make_float4(0, 0, 0, 0);
    float4 hb = z4, hc = z4, lb = z4, lc = z4, azb = z4;
    if (act) {
        hc = ld4(xh, row + zs * XY);
        lc = ld4(xl, row + zs * XY);
        if (zs > 0) { hb = ld4(xh, row + (zs - 1) * XY); lb = ld4(xl, row + (zs - 1) * XY); azb = ld4(az, row + (zs - 1) * XY); }
    }
    float acc = 0.0f, comp = 0.0f, mx = 0.0f;
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 hf = z4, lf = z4, hd = z4, ld = z4, hu = z4, lu = z4, ayd = z4, cx = z4, cy = z4, cz = z4, cw = z4, bb = z4;
        if (act) {
            if (z + 1 < Z) { hf = ld4(xh, c + XY); lf = ld4(xl, c + XY); }
            if (y > 0) { hd = ld4(xh, c - X); ld = ld4(xl, c - X); ayd = ld4(ay, c - X); }
            if (y + 1 < Y) { hu = ld4(xh, c + X); lu = ld4(xl, c + X); }
            cx = ld4(ax, c); cy = ld4(ay, c); cz = ld4(az, c); cw = ld4(aw, c); bb = ld4(b, c);
        }
        float hl = __shfl_up_sync(0xffffffffu, hc.w, 1), ll = __shfl_up_sync(0xffffffffu, lc.w, 1);
        float axl = __shfl_up_sync(0xffffffffu, cx.w, 1);
        float hr = __shfl_down_sync(0xffffffffu, hc.x, 1), lr = __shfl_down_sync(0xffffffffu, lc.x, 1);
        if (act && lane == 0) {
            if (x0 > 0) { hl = xh[c - 1]; ll = xl[c - 1]; axl = ax[c - 1]; } else { hl = 0.0f; ll = 0.0f; axl = 0.0f; }
        }
        if (act && (lane == 31 || x0 + 4 >= X)) {
            if (x0 + 4 < X) { hr = xh[c + 4]; lr = xl[c + 4]; } else { hr = 0.0f; lr = 0.0f; }
        }
        if (act) {
            const float H[6] = {hl, hc.x, hc.y, hc.z, hc.w, hr}, L[6] = {ll, lc.x, lc.y, lc.z, lc.w, lr};
            const float AXm[4] = {axl, cx.x, cx.y, cx.z}, AXp[4] = {cx.x, cx.y, cx.z, cx.w};
            float4 o;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float d = comp4(cw, k);
                float rv = 0.0f;
                if (d != 0.0f) {
                    FF sacc;
                    sacc.add_prod(d, H[k + 1], L[k + 1]);
                    sacc.add_prod(AXm[k], H[k], L[k]);
                    sacc.add_prod(AXp[k], H[k + 2], L[k + 2]);
                    sacc.add_prod(comp4(ayd, k), comp4(hd, k), comp4(ld, k));
                    sacc.add_prod(comp4(cy, k), comp4(hu, k), comp4(lu, k));
                    sacc.add_prod(comp4(azb, k), comp4(hb, k), comp4(lb, k));
                    sacc.add_prod(comp4(cz, k), comp4(hf, k), comp4(lf, k));
                    rv = ff_resid(comp4(bb, k), sacc);
                }
                set4(o, k, rv);
                const float yv = rv * rv - comp;
                const float tt = acc + yv;
                comp = (tt - acc) - yv;
                acc = tt;
                mx = fmaxf(mx, fabsf(rv));
            }
            *reinterpret_cast<float4*>(r + c) = o;
        }
        hb = hc; lb = lc;
        hc = hf; lc = lf;
        azb = cz;
    }
    __shared__ double smd[JVY];
    const double bs = bsum_t<32 * JVY>(double(acc) - double(comp), smd, tid);
    double tot;
    float mall;
    if (finish_sum_max<32 * JVY>(sc, partials, bs, mx, tot, mall, tid)) refine_record(sc, tot, mall, refine_tol, first);
}

// FP16 copies of the finest level's coefficients for the V-cycle. Faces round toward zero; the
// diagonal is the sum of the cell's rounded interior faces plus its FP32 boundary share, rounded
// up, so every row keeps A's weak diagonal dominance and the smoothed operator stays symmetric
// positive definite. Inactive cells keep diagonal 0.
__global__ void __launch_bounds__(RT) k_mg_half(Grid g, const float* __restrict__ ax, const float* __restrict__ ay, const float* __restrict__ az,
                                                const float* __restrict__ aw, __half* __restrict__ hx, __half* __restrict__ hy,
                                                __half* __restrict__ hz, __half* __restrict__ hw) {
    for (int c = blockIdx.x * RT + threadIdx.x; c < g.N; c += gridDim.x * RT) {
        const __half fx = __float2half_ru(ax[c]), fy = __float2half_ru(ay[c]), fz = __float2half_ru(az[c]);
        hx[c] = fx;
        hy[c] = fy;
        hz[c] = fz;
        const float d = aw[c];
        if (d == 0.0f) { hw[c] = __float2half(0.0f); continue; }
        const int xx = c % g.X, yy = (c / g.X) % g.Y, zz = c / g.XY;
        float s = 0.0f, sh = 0.0f;
        auto face = [&](bool inner, float a, __half h) {
            if (inner) { s -= a; sh -= __half2float(h); }
        };
        face(xx + 1 < g.X, ax[c], fx);
        face(xx > 0, xx > 0 ? ax[c - 1] : 0.0f, __float2half_ru(xx > 0 ? ax[c - 1] : 0.0f));
        face(yy + 1 < g.Y, ay[c], fy);
        face(yy > 0, yy > 0 ? ay[c - g.X] : 0.0f, __float2half_ru(yy > 0 ? ay[c - g.X] : 0.0f));
        face(zz + 1 < g.Z, az[c], fz);
        face(zz > 0, zz > 0 ? az[c - g.XY] : 0.0f, __float2half_ru(zz > 0 ? az[c - g.XY] : 0.0f));
        const float share = fmaxf(d - s, 0.0f);
        hw[c] = __float2half_ru(sh + share);
    }
}

// e += alpha s; r -= alpha As; inner stop on max|r|, float4
__global__ void __launch_bounds__(RT) k_update_mg4(int n4, const float4* __restrict__ s, const float4* __restrict__ As, float4* __restrict__ e,
                                                   float4* __restrict__ r, float inner_rtol, int max_iter, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ float smf[RT / 32];
    const float alpha = sc->alpha;
    float mx = 0.0f;
    for (int i = blockIdx.x * RT + threadIdx.x; i < n4; i += gridDim.x * RT) {
        const float4 sv = s[i], av = As[i];
        float4 ev = e[i], rv = r[i];
        ev.x += alpha * sv.x; ev.y += alpha * sv.y; ev.z += alpha * sv.z; ev.w += alpha * sv.w;
        rv.x = rv.x - alpha * av.x; rv.y = rv.y - alpha * av.y; rv.z = rv.z - alpha * av.z; rv.w = rv.w - alpha * av.w;
        e[i] = ev;
        r[i] = rv;
        mx = fmaxf(mx, fmaxf(fmaxf(fabsf(rv.x), fabsf(rv.y)), fmaxf(fabsf(rv.z), fabsf(rv.w))));
    }
    const float bm = bmax<RT>(mx, smf);
    double tot;
    float mall;
    if (finish(sc, partials, 0.0, bm, tot, mall)) {
        sc->iters += 1;
        sc->outer_inner_total += 1;
        if (mall <= inner_rtol * sc->inner_tol) sc->converged = 1;
        else if (sc->iters >= max_iter) sc->converged = 2;
    }
}

// rho = z.r (FP64 across threads); START also sets s = z
template <bool START>
__global__ void __launch_bounds__(RT) k_zr4(int n4, const float4* __restrict__ z, const float4* __restrict__ r, float4* __restrict__ s,
                                            Scalars* sc, double* partials) {
    if (!START && sc->converged) return;
    __shared__ double smd[RT / 32];
    float acc = 0.0f, comp = 0.0f;
    for (int i = blockIdx.x * RT + threadIdx.x; i < n4; i += gridDim.x * RT) {
        const float4 zv = z[i], rv = r[i];
        const float t = zv.x * rv.x + zv.y * rv.y + zv.z * rv.z + zv.w * rv.w;
        const float yv = t - comp;
        const float tt = acc + yv;
        comp = (tt - acc) - yv;
        acc = tt;
        if (START) s[i] = zv;
    }
    const double bs = bsum<RT>(double(acc) - double(comp), smd);
    double tot;
    float mall;
    if (finish(sc, partials, bs, 0.0f, tot, mall)) {
        if (START) {
            sc->sigma0 = tot;
            sc->converged = 0;
            sc->iters = 0;
        } else {
            sc->beta_f = float(tot / sc->sigma0);
            sc->sigma0 = tot;
        }
    }
}

__global__ void __launch_bounds__(RT) k_search_mg4(int n4, const float4* __restrict__ z, float4* __restrict__ s, const Scalars* sc) {
    if (sc->converged) return;
    const float beta = sc->beta_f;
    for (int i = blockIdx.x * RT + threadIdx.x; i < n4; i += gridDim.x * RT) {
        const float4 zv = z[i];
        float4 sv = s[i];
        sv.x = zv.x + beta * sv.x; sv.y = zv.y + beta * sv.y; sv.z = zv.z + beta * sv.z; sv.w = zv.w + beta * sv.w;
        s[i] = sv;
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------

bool mg_allocate(Env& e) {
    const Grid& g = e.g;
    int X = g.X, Y = g.Y, Z = g.Z;
    e.mg_levels = 0;
    size_t bytes = 0;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    std::vector<int> dims;
    dims.insert(dims.end(), {X, Y, Z});
    while ((X % 2 == 0) && (Y % 2 == 0) && (Z % 2 == 0) && X * Y * Z > kCoarseMax && e.mg_levels + 1 < kMaxMgLevels) {
        X /= 2; Y /= 2; Z /= 2;
        dims.insert(dims.end(), {X, Y, Z});
        bytes += al(size_t(X) * Y * Z * 4) * 7;
        e.mg_levels++;
    }
    if (X * Y * Z > kCoarseMax) return false;  // no level small enough for the one-block solve
    const size_t hbytes = al(size_t(g.N) * 2) * 4;
    bytes += hbytes;
    if (cudaMalloc(&e.mg_pool, bytes) != cudaSuccess) { cudaGetLastError(); return false; }
    char* p = (char*)e.mg_pool;
    e.mg_h = p;
    p += hbytes;
    for (int l = 0; l <= e.mg_levels; ++l) {
        MgLevel& L = e.mg[l];
        L.X = dims[3 * l]; L.Y = dims[3 * l + 1]; L.Z = dims[3 * l + 2];
        if (l == 0) continue;
        const size_t n = size_t(L.X) * L.Y * L.Z;
        float** arr[7] = {&L.ax, &L.ay, &L.az, &L.aw, &L.x, &L.x2, &L.b};
        for (auto a : arr) { *a = (float*)p; p += al(n * 4); }
    }
    return true;
}

namespace {

LvlView view(Env& e, int l) {
    if (l == 0) return LvlView{e.g.X, e.g.Y, e.g.Z, e.ax, e.ay, e.az, e.aw};
    const MgLevel& L = e.mg[l];
    return LvlView{L.X, L.Y, L.Z, L.ax, L.ay, L.az, L.aw};
}

// the four FP16 coefficient arrays of the finest level (256-byte aligned, in mg_pool)
void half_arrays(const Env& e, __half* h[4]) {
    const size_t stride = (size_t(e.g.N) * 2 + 255) / 256 * 128;
    for (int k = 0; k < 4; ++k) h[k] = (__half*)e.mg_h + k * stride;
}

bool vec_level(const Env& e, int l);

void mg_setup(Env& e) {
    for (int l = 0; l < e.mg_levels; ++l) {
        const MgLevel& C = e.mg[l + 1];
        k_mg_coarsen<<<lgrid(C.X, C.Y, C.Z), dim3(MBX, MBY), 0, e.stream>>>(view(e, l), C.X, C.Y, C.Z, C.ax, C.ay, C.az, C.aw);
        e.launches += 1;
    }
    if (e.cfg.mg_half && vec_level(e, 0)) {
        __half* h[4];
        half_arrays(e, h);
        const int nb = std::min((e.g.N + RT - 1) / RT, stencil_sms(e) * 8);
        k_mg_half<<<nb, RT, 0, e.stream>>>(e.g, e.ax, e.ay, e.az, e.aw, h[0], h[1], h[2], h[3]);
        e.launches += 1;
    }
}

// z-march launch shape of a vector level: about 12 blocks of 32 x JVY threads per SM, at most
// kMaxPartials blocks (the fused dot products keep one partial per block), even plane runs. The
// kernels with a dot product are sized for all SMs (num_sms: their partials, and so their bits,
// follow the grid), the per-cell ones for stencil_sms.
struct March {
    dim3 grid;
    int zlen;
};
March march(const Env& e, int X, int Y, int Z, int sms) {
    const int gx = (X / 4 + 31) / 32, gy = (Y + JVY - 1) / JVY;
    int zc = std::max(1, std::min(Z, (sms * 12 + gx * gy - 1) / (gx * gy)));
    zc = std::max(1, std::min(zc, kMaxPartials / (gx * gy)));
    int zlen = (Z + zc - 1) / zc;
    zlen += zlen & 1;
    zc = (Z + zlen - 1) / zlen;
    return {dim3(gx, gy, zc), zlen};
}

// A level runs the float4 kernels when its x size is a multiple of 4; the finest level also
// needs its z-march grid to fit the partial slots of the fused dot product.
bool vec_level(const Env& e, int l) {
    const LvlView L = view(const_cast<Env&>(e), l);
    if (L.X % 4 != 0) return false;
    if (l > 0) return (L.Y % 2 == 0) && (L.Z % 2 == 0);
    const int gx = (L.X / 4 + 31) / 32, gy = (L.Y + JVY - 1) / JVY;
    return gx * gy <= kMaxPartials && (L.Y % 2 == 0) && (L.Z % 2 == 0);
}

template <class CT>
void vcycle_vec(Env& e, int l, const CT* ax, const CT* ay, const CT* az, const CT* aw, const float* b, float* x, float* x2,
                const int* skip, int dot);

// z = V(b) on level l (level 0: x = z0, x2 = z0b). skip: the kernels return at once while *skip
// is set (the CG has converged inside a chunk of queued iterations). On a vector finest level
// dot = DOT_START / DOT_NEXT also forms z.r in the last smoothing step (returns true).
bool vcycle(Env& e, int l, const float* b, float* x, float* x2, const int* skip, int dot) {
    const LvlView L = view(e, l);
    if (l == e.mg_levels) {
        const int n = L.X * L.Y * L.Z;
        k_mg_coarse<<<1, kCoarseThreads, 2 * n * sizeof(float), e.stream>>>(L, b, x, skip);
        e.launches += 1;
        return false;
    }
    if (vec_level(e, l)) {
        if (l == 0 && e.cfg.mg_half) {
            __half* h[4];
            half_arrays(e, h);
            vcycle_vec<__half>(e, 0, h[0], h[1], h[2], h[3], b, x, x2, skip, dot);
        } else {
            vcycle_vec<float>(e, l, L.ax, L.ay, L.az, L.aw, b, x, x2, skip, dot);
        }
        return l == 0 && dot != DOT_NONE;
    }
    const dim3 gr = lgrid(L.X, L.Y, L.Z), bl(MBX, MBY);
    MgLevel& C = e.mg[l + 1];
    const float c2a = 1.0f / kChebTheta;
    k_mg_jacobi<true><<<gr, bl, 0, e.stream>>>(L, nullptr, nullptr, x2, b, 0.0f, 0.0f, skip);
    k_mg_jacobi<false><<<gr, bl, 0, e.stream>>>(L, x2, nullptr, x, b, kChebC1, kChebC2, skip);
    k_mg_restrict<<<lgrid(C.X, C.Y, C.Z), bl, 0, e.stream>>>(L, x, b, C.X, C.Y, C.Z, C.b, skip);
    vcycle(e, l + 1, C.b, C.x, C.x2, skip, DOT_NONE);
    k_mg_prolong<<<gr, bl, 0, e.stream>>>(L, x, C.X, C.Y, C.x, skip);
    k_mg_jacobi<false><<<gr, bl, 0, e.stream>>>(L, x, nullptr, x2, b, 0.0f, c2a, skip);
    k_mg_jacobi<false><<<gr, bl, 0, e.stream>>>(L, x2, x, x, b, kChebC1, kChebC2, skip);
    e.launches += 6;
    return false;
}

template <class CT>
void vcycle_vec(Env& e, int l, const CT* ax, const CT* ay, const CT* az, const CT* aw, const float* b, float* x, float* x2,
                const int* skip, int dot) {
    const LvlView L = view(e, l);
    MgLevel& C = e.mg[l + 1];
    const March m = march(e, L.X, L.Y, L.Z, stencil_sms(e));
    const March md = march(e, L.X, L.Y, L.Z, e.num_sms);  // the smoothing step that forms z.r
    const dim3 jb(32, JVY);
    const float c2a = 1.0f / kChebTheta;
    UIn<SM_PRE, CT> upre{b, aw, nullptr, 0, 0};
    UIn<SM_POSTA, CT> upost{x, aw, C.x, C.X, C.Y};
    UIn<SM_POSTB, CT> ub{x2, aw, nullptr, 0, 0};
    // pre-smoothing from zero (steps A and B in one pass) -> x
    k_mg_smooth4<SM_PRE, DOT_NONE, CT><<<m.grid, jb, 0, e.stream>>>(L.X, L.Y, L.Z, m.zlen, ax, ay, az, aw, b, upre, upost, x,
                                                                   kChebC1, kChebC2, skip, e.sc, e.partials);
    k_mg_restrict4<CT><<<m.grid, jb, 0, e.stream>>>(L.X, L.Y, L.Z, m.zlen, ax, ay, az, aw, x, b, C.X, C.Y, C.b, skip);
    vcycle(e, l + 1, C.b, C.x, C.x2, skip, DOT_NONE);
    // post-smoothing: step A on x + P e -> x2, step B (prev = x + P e) -> x
    k_mg_smooth4<SM_POSTA, DOT_NONE, CT><<<m.grid, jb, 0, e.stream>>>(L.X, L.Y, L.Z, m.zlen, ax, ay, az, aw, b, upost, upost, x2,
                                                                     0.0f, c2a, skip, e.sc, e.partials);
    if (dot == DOT_START)
        k_mg_smooth4<SM_POSTB, DOT_START, CT><<<md.grid, jb, 0, e.stream>>>(L.X, L.Y, L.Z, md.zlen, ax, ay, az, aw, b, ub, upost, x,
                                                                          kChebC1, kChebC2, skip, e.sc, e.partials);
    else if (dot == DOT_NEXT)
        k_mg_smooth4<SM_POSTB, DOT_NEXT, CT><<<md.grid, jb, 0, e.stream>>>(L.X, L.Y, L.Z, md.zlen, ax, ay, az, aw, b, ub, upost, x,
                                                                         kChebC1, kChebC2, skip, e.sc, e.partials);
    else
        k_mg_smooth4<SM_POSTB, DOT_NONE, CT><<<m.grid, jb, 0, e.stream>>>(L.X, L.Y, L.Z, m.zlen, ax, ay, az, aw, b, ub, upost, x,
                                                                         kChebC1, kChebC2, skip, e.sc, e.partials);
    e.launches += 4;
}

}  // namespace

// graph mode, refinement loop: another refinement step while the relative residual is above the
// target, no NaN was met and the step cap is not reached (loop < 0: the loop's start)
__global__ void k_outer_cond(cudaGraphConditionalHandle h, Scalars* sc, int loop, int max_outer) {
    if (loop < 0) {
        sc->outer = 0;
    } else {
        note_trip(sc, loop);
        sc->outer += 1;
    }
    cudaGraphSetConditional(h, (sc->refine_done != 1 && sc->status == 0 && sc->outer < max_outer) ? 1u : 0u);
}
// graph mode, inner CG loop: another chunk of iterations while the inner solve has not stopped
__global__ void k_inner_cond(cudaGraphConditionalHandle h, Scalars* sc, int loop) {
    if (loop >= 0) note_trip(sc, loop);
    cudaGraphSetConditional(h, (sc->converged == 0 && sc->status == 0) ? 1u : 0u);
}

// The refinement as captured graph nodes: the first residual, then a WHILE loop of refinement steps
// (inner solve, correction, residual), each inner solve a WHILE loop of chunks of four CG
// iterations. The same kernels in the same order as mg_solve's stream-ordered loop; the stop tests
// run on the device instead of the host. sc->outer counts the refinement steps.
void mg_solve_graph(Env& e, bool fused, int max_outer, float* bvec, float* ecor, float* z0, float* z0b, float* xh, float* xl, int nb) {
    const Grid& g = e.g;
    const int n = g.N;
    auto resid = [&](int first) {
        ProfScope ps(e, "mg_refine");
        if (fused) {
            const March m = march(e, g.X, g.Y, g.Z, e.num_sms);
            k_resid_ff4<<<m.grid, dim3(32, JVY), 0, e.stream>>>(g.X, g.Y, g.Z, m.zlen, e.ax, e.ay, e.az, e.aw, xh, xl, bvec, e.r,
                                                              e.cfg.refine_tol, first, e.sc, e.partials);
        } else {
            k_resid_ff<<<nb, RT, 0, e.stream>>>(g, e.ax, e.ay, e.az, e.aw, xh, xl, bvec, e.r, e.cfg.refine_tol, first, e.sc, e.partials);
        }
        e.launches += 1;
    };
    const int* conv = &e.sc->converged;
    auto inner = [&]() {
        if (fused) {
            { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, nullptr, DOT_START); }
            const March m = march(e, g.X, g.Y, g.Z, e.num_sms);
            graph_while(
                e, [&](cudaGraphConditionalHandle h) {
                    k_inner_cond<<<1, 1, 0, e.stream>>>(h, e.sc, -1);
                    e.launches += 1;
                },
                [&](cudaGraphConditionalHandle h, int loop) {
                    float* s_old = e.s;
                    float* s_new = e.pp;
                    for (int k = 0; k < 4; ++k) {  // an even count: the buffers' roles repeat every trip
                        { ProfScope ps(e, "mg_matvec");
                          k_mg_matvec_search4<<<m.grid, dim3(32, JVY), 0, e.stream>>>(g.X, g.Y, g.Z, m.zlen, e.ax, e.ay, e.az, e.aw, z0,
                                                                                    s_old, s_new, e.As, e.sc, e.partials);
                          e.launches += 1; }
                        { ProfScope ps(e, "mg_update");
                          k_update_mg4<<<nb, RT, 0, e.stream>>>(n / 4, (const float4*)s_new, (const float4*)e.As, (float4*)ecor,
                                                               (float4*)e.r, e.cfg.inner_rtol, e.cfg.inner_max_iter, e.sc, e.partials);
                          e.launches += 1; }
                        { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, conv, DOT_NEXT); }
                        std::swap(s_old, s_new);
                    }
                    k_inner_cond<<<1, 1, 0, e.stream>>>(h, e.sc, loop);
                    e.launches += 1;
                });
            return;
        }
        { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, nullptr, DOT_NONE); }
        const bool vec = (g.X % 4) == 0;
        const int n4 = n / 4;
        if (vec) k_zr4<true><<<nb, RT, 0, e.stream>>>(n4, (const float4*)z0, (const float4*)e.r, (float4*)e.s, e.sc, e.partials);
        else k_zr_search<true><<<nb, RT, 0, e.stream>>>(n, z0, e.r, e.s, e.sc, e.partials);
        e.launches += 1;
        graph_while(
            e, [&](cudaGraphConditionalHandle h) {
                k_inner_cond<<<1, 1, 0, e.stream>>>(h, e.sc, -1);
                e.launches += 1;
            },
            [&](cudaGraphConditionalHandle h, int loop) {
                for (int k = 0; k < 4; ++k) {
                    if (vec) {
                        { ProfScope ps(e, "mg_matvec"); launch_matvec_textbook(e, e.s, e.As); }
                        { ProfScope ps(e, "mg_update");
                          k_update_mg4<<<nb, RT, 0, e.stream>>>(n4, (const float4*)e.s, (const float4*)e.As, (float4*)ecor, (float4*)e.r,
                                                               e.cfg.inner_rtol, e.cfg.inner_max_iter, e.sc, e.partials); }
                        { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, conv, DOT_NONE); }
                        { ProfScope ps(e, "mg_search");
                          k_zr4<false><<<nb, RT, 0, e.stream>>>(n4, (const float4*)z0, (const float4*)e.r, nullptr, e.sc, e.partials);
                          k_search_mg4<<<nb, RT, 0, e.stream>>>(n4, (const float4*)z0, (float4*)e.s, e.sc); }
                        e.launches += 3;
                        continue;
                    }
                    { ProfScope ps(e, "mg_matvec");
                      k_matvec_mg<<<nb, RT, 0, e.stream>>>(g, e.ax, e.ay, e.az, e.aw, e.s, e.As, e.sc, e.partials); }
                    { ProfScope ps(e, "mg_update");
                      k_update_mg<<<nb, RT, 0, e.stream>>>(n, e.s, e.As, ecor, e.r, e.cfg.inner_rtol, e.cfg.inner_max_iter, e.sc, e.partials); }
                    { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, conv, DOT_NONE); }
                    { ProfScope ps(e, "mg_search");
                      k_zr_search<false><<<nb, RT, 0, e.stream>>>(n, z0, e.r, e.s, e.sc, e.partials);
                      k_search_mg<<<nb, RT, 0, e.stream>>>(n, z0, e.s, e.sc); }
                    e.launches += 4;
                }
                k_inner_cond<<<1, 1, 0, e.stream>>>(h, e.sc, loop);
                e.launches += 1;
            });
    };
    resid(1);
    graph_while(
        e, [&](cudaGraphConditionalHandle h) {
            k_outer_cond<<<1, 1, 0, e.stream>>>(h, e.sc, -1, max_outer);
            e.launches += 1;
        },
        [&](cudaGraphConditionalHandle h, int loop) {
            inner();
            { ProfScope ps(e, "mg_refine");
              k_accum_ff<<<nb, RT, 0, e.stream>>>(n, xh, xl, ecor);
              e.launches += 1; }
            resid(0);
            k_outer_cond<<<1, 1, 0, e.stream>>>(h, e.sc, loop, max_outer);
            e.launches += 1;
        });
    k_cast_ff<<<nb, RT, 0, e.stream>>>(n, xh, xl, e.pp);
    e.launches += 1;
}

// Solves A p = b (b = the divergence in e.r on entry, A from k_build in textbook form) into
// e.pp. Uses e.tA (b), e.tB (inner correction), e.r/e.s/e.As (inner CG) and e.rd (V-cycle
// vectors). Returns after the refinement met refine_tol or the outer cap.
void mg_solve(Env& e) {
    const Grid& g = e.g;
    const int n = g.N;
    const int nb = std::min((n + RT - 1) / RT, std::min(e.num_sms * 16, kMaxPartials));
    float* bvec = e.tA;
    float* ecor = e.tB;
    float* z0 = (float*)e.rd;
    float* z0b = z0 + size_t(n);
    float* xh = (float*)e.xd;  // the float-float solution (xh, xl) in the FP64 field's storage
    float* xl = xh + size_t(n);
    {
        ProfScope ps(e, "mg_setup");
        mg_setup(e);
        cudaMemcpyAsync(bvec, e.r, sizeof(float) * size_t(n), cudaMemcpyDeviceToDevice, e.stream);
        cudaMemsetAsync(ecor, 0, sizeof(float) * size_t(n), e.stream);
        cudaMemsetAsync(xh, 0, sizeof(float) * 2 * size_t(n), e.stream);
        cudaMemsetAsync(&e.sc->outer_inner_total, 0, sizeof(int), e.stream);
    }
    const bool fused = e.mg_levels > 0 && vec_level(e, 0);
    int outer = 0;
    const int max_outer = 12;
    if (e.capturing) {
        mg_solve_graph(e, fused, max_outer, bvec, ecor, z0, z0b, xh, xl, nb);
        return;
    }
    for (; outer < max_outer; ++outer) {
        {
            ProfScope ps(e, "mg_refine");
            if (fused) {
                const March m = march(e, g.X, g.Y, g.Z, e.num_sms);
                k_resid_ff4<<<m.grid, dim3(32, JVY), 0, e.stream>>>(g.X, g.Y, g.Z, m.zlen, e.ax, e.ay, e.az, e.aw, xh, xl, bvec, e.r,
                                                                  e.cfg.refine_tol, outer == 0, e.sc, e.partials);
            } else {
                k_resid_ff<<<nb, RT, 0, e.stream>>>(g, e.ax, e.ay, e.az, e.aw, xh, xl, bvec, e.r, e.cfg.refine_tol, outer == 0, e.sc, e.partials);
            }
            e.launches += 1;
        }
        fetch_scalars(e);
        if (e.host_sc->refine_done == 1 || e.host_sc->status != 0) break;
        // inner MG-PCG on A e = r
        const int* conv = &e.sc->converged;
        if (fused) {
            // the V-cycle's last smoothing step forms z.r; the operator kernel forms the search
            // direction, written to the other buffer of the (s, pp) pair each iteration
            float* s_old = e.s;
            float* s_new = e.pp;
            { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, nullptr, DOT_START); }
            const March m = march(e, g.X, g.Y, g.Z, e.num_sms);
            const int chunk = 4;
            for (int it = 0; it < e.cfg.inner_max_iter; it += chunk) {
                for (int k = 0; k < chunk && it + k < e.cfg.inner_max_iter; ++k) {
                    { ProfScope ps(e, "mg_matvec");
                      k_mg_matvec_search4<<<m.grid, dim3(32, JVY), 0, e.stream>>>(g.X, g.Y, g.Z, m.zlen, e.ax, e.ay, e.az, e.aw, z0, s_old,
                                                                                s_new, e.As, e.sc, e.partials);
                      e.launches += 1; }
                    { ProfScope ps(e, "mg_update");
                      k_update_mg4<<<nb, RT, 0, e.stream>>>(n / 4, (const float4*)s_new, (const float4*)e.As, (float4*)ecor, (float4*)e.r,
                                                           e.cfg.inner_rtol, e.cfg.inner_max_iter, e.sc, e.partials);
                      e.launches += 1; }
                    { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, conv, DOT_NEXT); }
                    std::swap(s_old, s_new);
                }
                fetch_scalars(e);
                if (e.host_sc->converged || e.host_sc->status != 0) break;
            }
            { ProfScope ps(e, "mg_refine");
              k_accum_ff<<<nb, RT, 0, e.stream>>>(n, xh, xl, ecor);
              e.launches += 1; }
            continue;
        }
        {
            ProfScope ps(e, "mg_vcycle");
            vcycle(e, 0, e.r, z0, z0b, nullptr, DOT_NONE);
        }
        const bool vec = (g.X % 4) == 0;
        const int n4 = n / 4;
        if (vec) k_zr4<true><<<nb, RT, 0, e.stream>>>(n4, (const float4*)z0, (const float4*)e.r, (float4*)e.s, e.sc, e.partials);
        else k_zr_search<true><<<nb, RT, 0, e.stream>>>(n, z0, e.r, e.s, e.sc, e.partials);
        e.launches += 1;
        const int chunk = 4;
        for (int it = 0; it < e.cfg.inner_max_iter; it += chunk) {
            for (int k = 0; k < chunk && it + k < e.cfg.inner_max_iter; ++k) {
                if (vec) {
                    { ProfScope ps(e, "mg_matvec"); launch_matvec_textbook(e, e.s, e.As); }
                    { ProfScope ps(e, "mg_update");
                      k_update_mg4<<<nb, RT, 0, e.stream>>>(n4, (const float4*)e.s, (const float4*)e.As, (float4*)ecor, (float4*)e.r,
                                                           e.cfg.inner_rtol, e.cfg.inner_max_iter, e.sc, e.partials); }
                    { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, conv, DOT_NONE); }
                    { ProfScope ps(e, "mg_search");
                      k_zr4<false><<<nb, RT, 0, e.stream>>>(n4, (const float4*)z0, (const float4*)e.r, nullptr, e.sc, e.partials);
                      k_search_mg4<<<nb, RT, 0, e.stream>>>(n4, (const float4*)z0, (float4*)e.s, e.sc); }
                    e.launches += 3;
                    continue;
                }
                { ProfScope ps(e, "mg_matvec");
                  k_matvec_mg<<<nb, RT, 0, e.stream>>>(g, e.ax, e.ay, e.az, e.aw, e.s, e.As, e.sc, e.partials); }
                { ProfScope ps(e, "mg_update");
                  k_update_mg<<<nb, RT, 0, e.stream>>>(n, e.s, e.As, ecor, e.r, e.cfg.inner_rtol, e.cfg.inner_max_iter, e.sc, e.partials); }
                { ProfScope ps(e, "mg_vcycle"); vcycle(e, 0, e.r, z0, z0b, conv, DOT_NONE); }
                { ProfScope ps(e, "mg_search");
                  k_zr_search<false><<<nb, RT, 0, e.stream>>>(n, z0, e.r, e.s, e.sc, e.partials);
                  k_search_mg<<<nb, RT, 0, e.stream>>>(n, z0, e.s, e.sc); }
                e.launches += 4;
            }
            fetch_scalars(e);
            if (e.host_sc->converged || e.host_sc->status != 0) break;
        }
        { ProfScope ps(e, "mg_refine");
          k_accum_ff<<<nb, RT, 0, e.stream>>>(n, xh, xl, ecor);
          e.launches += 1; }
    }
    k_cast_ff<<<nb, RT, 0, e.stream>>>(n, xh, xl, e.pp);
    e.launches += 1;
    fetch_scalars(e);
    e.last_outer = outer;
    e.last_iters = e.host_sc->outer_inner_total;
    e.last_residual = float(e.host_sc->rnorm0 > 0 ? e.host_sc->rnorm / e.host_sc->rnorm0 : 0.0);
    e.last_converged = e.host_sc->refine_done == 1;
}

}  // namespace skt
