// Pressure projection: boundary reset, Poisson coefficients + divergence, Jacobi-preconditioned
// CG with FP64 reductions, pressure/density update and the velocity correction.
// Follows pressureProject / calculatePressureProject (Game/environment.cu:851-987).
#include "skt_internal.cuh"

namespace skt {

namespace {

constexpr int TX = 32, TY = 8, NT = TX * TY;

struct Tiles {
    int tx, ty, n;  // tiles along x, along y, total (including z)
};
inline Tiles tiles_of(const Grid& g) {
    Tiles t;
    t.tx = (g.X + TX - 1) / TX;
    t.ty = (g.Y + TY - 1) / TY;
    t.n = t.tx * t.ty * g.Z;
    return t;
}
__device__ __forceinline__ void tile_cell(const Grid& g, const Tiles& T, int t, int& x, int& y, int& z) {
    const int txy = T.tx * T.ty;
    z = t / txy;
    const int r = t - z * txy;
    const int ty = r / T.tx;
    const int tx = r - ty * T.tx;
    x = tx * TX + (threadIdx.x & (TX - 1));
    y = ty * TY + (threadIdx.x / TX);
}

// fixed-order block reductions
__device__ __forceinline__ double block_sum(double v, double* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sm[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (NT / 32) ? sm[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;  // valid in thread 0
}
__device__ __forceinline__ float block_max(float v, float* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sm[w] = v;
    __syncthreads();
    float t = 0.0f;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (NT / 32) ? sm[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    }
    return t;
}

// Publishes one block partial (sum, max) of a 1D NT-thread grid; thread 0 of the last block to
// finish gets the totals (see publish_n). Defined after the generic reductions below.
__device__ __forceinline__ bool publish(Scalars* sc, double* partials, double sum, float mx, double& tot, float& mxall);

__device__ __forceinline__ float char_trunc(float a) {  // (char) of a float: truncate, saturate (Q3)
    const float t = truncf(a);
    return fminf(fmaxf(t, -128.0f), 127.0f);
}
__device__ __forceinline__ float coef_of(float c, float n) {  // initAMatrix Game/kernelSky.cu:1372
    return n == 0.0f ? 0.0f : -fmaxf(1.0f, 1.225f / (2.0f / (1.0f / c + 1.0f / n)));
}
__device__ __forceinline__ float precon_of(float w) { return w == 0.0f ? 1.0f : 1.0f / w; }  // initPrecon :1409

// resetVelPressProj Game/kernelSky.cu:1648-1682; one thread per (x,y) marching z.
// reference=1 returns at the first ground cell of the column (Q8).
__global__ void k_reset_vel(Grid g, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, const float* __restrict__ defU,
                            const float* __restrict__ defW, int reference) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.XY) return;
    const int x = t % g.X, y = t / g.X;
    for (int z = 0; z < g.Z; ++z) {
        if (is_ground(g, x, y, z)) {
            if (reference) return;
            continue;
        }
        const int c = cidx(g, x, y, z);
        if (y == g.Y - 1) v[c] = 0.0f;
        if (x == g.X - 1) u[c] = defU[y];
        if (x + 1 < g.X && is_ground(g, x + 1, y, z)) u[c] = 0.0f;
        if (z == g.Z - 1) w[c] = defW[y];
        if (z + 1 < g.Z && is_ground(g, x, y, z + 1)) w[c] = 0.0f;
    }
}

// initAMatrix (Game/kernelSky.cu:1320-1393, density bounds NEUMANN sides / DIRICHLET ground)
// fused with calculateDivergenceGPU (:780-860, velocity bounds CUSTOM sides / DIRICHLET ground),
// the preconditioned start z = r/diag, s = z, sigma0 = z.r and the first max residual.
__global__ void __launch_bounds__(NT) k_build(Grid g, Tiles T, const float* __restrict__ rho, const float* __restrict__ u,
                                              const float* __restrict__ v, const float* __restrict__ w,
                                              const float* __restrict__ defU, const float* __restrict__ defW, float dt,
                                              float* __restrict__ ax, float* __restrict__ ay, float* __restrict__ az, float* __restrict__ aw,
                                              float* __restrict__ r, float* __restrict__ s, float* __restrict__ pp, float* __restrict__ As,
                                              int reference, Scalars* sc, double* partials) {
    __shared__ double smd[NT / 32];
    __shared__ float smf[NT / 32];
    double dsum = 0.0;
    float mx = 0.0f;
    for (int t = blockIdx.x; t < T.n; t += gridDim.x) {
        int x, y, z;
        tile_cell(g, T, t, x, y, z);
        if (x >= g.X || y >= g.Y) continue;
        const int c = cidx(g, x, y, z);
        pp[c] = 0.0f;
        As[c] = 0.0f;
        if (is_ground(g, x, y, z)) {
            ax[c] = ay[c] = az[c] = aw[c] = 0.0f;
            r[c] = 0.0f;
            s[c] = 0.0f;
            continue;
        }
        const float cur = rho[c];
        const float nr = ghost(g, rho, x + 1, y, z, NEUMANN, DIRICHLET, nullptr);
        const float nl = ghost(g, rho, x - 1, y, z, NEUMANN, DIRICHLET, nullptr);
        const float nu = ghost(g, rho, x, y + 1, z, NEUMANN, DIRICHLET, nullptr);
        const float nd = ghost(g, rho, x, y - 1, z, NEUMANN, DIRICHLET, nullptr);
        const float nf = ghost(g, rho, x, y, z + 1, NEUMANN, DIRICHLET, nullptr);
        const float nb = ghost(g, rho, x, y, z - 1, NEUMANN, DIRICHLET, nullptr);
        const float cr = coef_of(cur, nr), cl = coef_of(cur, nl), cu = coef_of(cur, nu);
        const float cd = coef_of(cur, nd), cf = coef_of(cur, nf), cb = coef_of(cur, nb);
        ax[c] = cr;
        ay[c] = cu;
        az[c] = cf;
        float wd = 0.0f;
        wd -= cr; wd -= cl; wd -= cu; wd -= cd; wd -= cf; wd -= cb;
        aw[c] = wd;
        // divergence
        const float ur = u[c], ul = face_nb(g, u, x, y, z, -1, 0, 0, CUSTOM, DIRICHLET, defU[y]);
        const float uu = v[c], ud = face_nb(g, v, x, y, z, 0, -1, 0, CUSTOM, DIRICHLET, 0.0f);
        const float uf = w[c], ub = face_nb(g, w, x, y, z, 0, 0, -1, CUSTOM, DIRICHLET, defW[y]);
        auto hm = [&](float d) { return d == 0.0f ? 0.0f : 2.0f / (1.0f / cur + 1.0f / d); };
        const float dr = hm(nr), dl = hm(nl), du = hm(nu), dd = hm(nd), df = hm(nf), db = hm(nb);
        const float mfd = ((dr * ur - dl * ul) + (du * uu - dd * ud) + (df * uf - db * ub));
        const float dch = (cur - rho[c]) / dt;  // the reference's old density is a copy of rho
        const float rv = mfd - dch;
        r[c] = rv;
        const float zv = rv * precon_of(wd);
        s[c] = zv;
        dsum += double(zv) * double(rv);
        const float m = (!reference || z == 0) ? fabsf(rv) : rv;
        if (m > mx) mx = m;
    }
    const double bs = block_sum(dsum, smd);
    const float bm = block_max(mx, smf);
    double tot;
    float mall;
    if (publish(sc, partials, bs, bm, tot, mall)) {
        sc->sigma0 = tot;
        sc->sigma1 = 0.0;
        sc->iters = 0;
        sc->residual = mall;
        sc->converged = (mall == 0.0f) ? 1 : 0;
    }
}

// As = A s and s.As (applyAGPU Game/kernelSky.cu:719-778 + dotProductGPU :675-717).
// reference=1: lower coefficients pass through a char (Q3) and the denominator keeps
// accumulating (Q1).
__global__ void __launch_bounds__(NT) k_matvec(Grid g, Tiles T, const float* __restrict__ ax, const float* __restrict__ ay,
                                               const float* __restrict__ az, const float* __restrict__ aw, const float* __restrict__ s,
                                               float* __restrict__ As, int reference, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[NT / 32];
    double dsum = 0.0;
    for (int t = blockIdx.x; t < T.n; t += gridDim.x) {
        int x, y, z;
        tile_cell(g, T, t, x, y, z);
        if (x >= g.X || y >= g.Y) continue;
        const int c = cidx(g, x, y, z);
        if (is_ground(g, x, y, z)) continue;  // As of ground cells stays 0
        const bool hl = x > 0 && !is_ground(g, x - 1, y, z);
        const bool hr = x + 1 < g.X && !is_ground(g, x + 1, y, z);
        const bool hd = y > 0 && !is_ground(g, x, y - 1, z);
        const bool hu = y + 1 < g.Y;
        const bool hb = z > 0 && !is_ground(g, x, y, z - 1);
        const bool hf = z + 1 < g.Z && !is_ground(g, x, y, z + 1);
        const float sl = hl ? s[c - 1] : 0.0f, sr = hr ? s[c + 1] : 0.0f;
        const float sd = hd ? s[c - g.X] : 0.0f, su = hu ? s[c + g.X] : 0.0f;
        const float sb = hb ? s[c - g.XY] : 0.0f, sf = hf ? s[c + g.XY] : 0.0f;
        float AL = hl ? ax[c - 1] : 0.0f, AD = hd ? ay[c - g.X] : 0.0f, AB = hb ? az[c - g.XY] : 0.0f;
        if (reference) { AL = char_trunc(AL); AD = char_trunc(AD); AB = char_trunc(AB); }
        const float sc0 = s[c];
        const float out = aw[c] * sc0 + ((AL * sl + AD * sd + AB * sb + ax[c] * sr + ay[c] * su + az[c] * sf));
        As[c] = out;
        dsum += double(out) * double(sc0);
    }
    const double bs = block_sum(dsum, smd);
    double tot;
    float mall;
    if (publish(sc, partials, bs, 0.0f, tot, mall)) {
        const double s1 = reference ? sc->sigma1 + tot : tot;
        sc->sigma1 = s1;
        sc->alpha = float(sc->sigma0 / s1);
    }
}

// p += alpha s; r -= alpha As (updatePandDiv :955-985), then the stop test on the max residual
// (getMaxDivergence, Q4 in reference mode), z = r/diag and z.r for the next search direction.
__global__ void __launch_bounds__(NT) k_update(Grid g, Tiles T, const float* __restrict__ aw, const float* __restrict__ s,
                                               const float* __restrict__ As, float* __restrict__ pp, float* __restrict__ r,
                                               int reference, float tol, int max_iter, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[NT / 32];
    __shared__ float smf[NT / 32];
    const float alpha = sc->alpha;
    double dsum = 0.0;
    float mx = 0.0f;
    for (int t = blockIdx.x; t < T.n; t += gridDim.x) {
        int x, y, z;
        tile_cell(g, T, t, x, y, z);
        if (x >= g.X || y >= g.Y) continue;
        if (is_ground(g, x, y, z)) continue;
        const int c = cidx(g, x, y, z);
        pp[c] += alpha * s[c];
        const float rv = r[c] - alpha * As[c];
        r[c] = rv;
        const float zv = rv * precon_of(aw[c]);
        dsum += double(zv) * double(rv);
        const float m = (!reference || z == 0) ? fabsf(rv) : rv;
        if (m > mx) mx = m;
    }
    const double bs = block_sum(dsum, smd);
    const float bm = block_max(mx, smf);
    double tot;
    float mall;
    if (publish(sc, partials, bs, bm, tot, mall)) {
        sc->iters += 1;
        sc->residual = mall;
        if (mall <= tol) {
            sc->converged = 1;
        } else if (sc->iters >= max_iter) {
            sc->converged = 2;  // stopped at the iteration cap (the reference falls through, :986)
        } else {
            sc->sigma1 = tot;
            sc->beta_f = float(tot / sc->sigma0);
            sc->sigma0 = tot;
        }
    }
}

// s = z + beta s (endIteration :987-1014), z recomputed from r and the diagonal
__global__ void __launch_bounds__(NT) k_search(Grid g, Tiles T, const float* __restrict__ aw, const float* __restrict__ r,
                                               float* __restrict__ s, const Scalars* sc) {
    if (sc->converged) return;
    const float beta = sc->beta_f;
    for (int t = blockIdx.x; t < T.n; t += gridDim.x) {
        int x, y, z;
        tile_cell(g, T, t, x, y, z);
        if (x >= g.X || y >= g.Y) continue;
        if (is_ground(g, x, y, z)) continue;
        const int c = cidx(g, x, y, z);
        const float zv = r[c] * precon_of(aw[c]);
        s[c] = zv + beta * s[c];
    }
}

// ---- vectorised PCG iteration (X % 4 == 0): float4 streams, FP32-compensated per-thread sums,
// FP64 across threads and blocks --------------------------------------------------------------

struct Kahan {  // compensated FP32 running sum
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

template <int NTH>
__device__ __forceinline__ double block_sum_n(double v, double* sm, int tid) {
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
template <int NTH>
__device__ __forceinline__ float block_max_n(float v, float* sm, int tid) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((tid & 31) == 0) sm[tid >> 5] = v;
    __syncthreads();
    float t = 0.0f;
    if (tid < 32) {
        t = tid < (NTH / 32) ? sm[tid] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    }
    return t;
}
// publish() for any grid shape: bid = linear block id, nb = number of blocks. The last block to
// finish reduces all partials with every thread (fixed assignment, fixed tree): deterministic.
// Returns true in thread 0 of that block, with tot/mxall set.
template <int NTH>
__device__ __forceinline__ bool publish_n(Scalars* sc, double* partials, int bid, int nb, int tid, double sum, float mx, double& tot,
                                          float& mxall) {
    __shared__ bool last;
    __shared__ double sms[NTH / 32];
    __shared__ float smm[NTH / 32];
    if (tid == 0) {
        partials[bid] = sum;
        partials[kMaxPartials + bid] = double(mx);
        __threadfence();
        const unsigned t = atomicAdd(&sc->done_blocks, 1u);
        last = (t == unsigned(nb) - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    float m = 0.0f;
    for (int b = tid; b < nb; b += NTH) {
        s += __ldcg(partials + b);
        const float mb = float(__ldcg(partials + kMaxPartials + b));
        m = mb > m ? mb : m;
    }
    const double ts = block_sum_n<NTH>(s, sms, tid);
    const float tm = block_max_n<NTH>(m, smm, tid);
    if (tid == 0) {
        tot = ts;
        mxall = tm;
        sc->done_blocks = 0;
        note_nonfinite(sc, ts);
    }
    return tid == 0;
}

__device__ __forceinline__ bool publish(Scalars* sc, double* partials, double sum, float mx, double& tot, float& mxall) {
    return publish_n<NT>(sc, partials, blockIdx.x, gridDim.x, threadIdx.x, sum, mx, tot, mxall);
}

constexpr int UT = 256;

// p += alpha s, r -= alpha As, z = r/diag, z.r and the max residual, over all cells as float4
// (ground cells hold s = As = r = 0 and diag 0, so they contribute nothing and stay zero).
__global__ void __launch_bounds__(UT) k_update4(int n4, int xy4, const float4* __restrict__ aw, const float4* __restrict__ s,
                                                const float4* __restrict__ As, float4* __restrict__ pp, float4* __restrict__ r,
                                                int reference, float tol, int max_iter, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[UT / 32];
    __shared__ float smf[UT / 32];
    const float alpha = sc->alpha;
    Kahan acc;
    float mx = 0.0f;
    for (int i = blockIdx.x * UT + threadIdx.x; i < n4; i += gridDim.x * UT) {
        const float4 a = aw[i], sv = s[i], av = As[i];
        float4 pv = pp[i], rv = r[i];
        pv.x += alpha * sv.x; pv.y += alpha * sv.y; pv.z += alpha * sv.z; pv.w += alpha * sv.w;
        rv.x = rv.x - alpha * av.x; rv.y = rv.y - alpha * av.y; rv.z = rv.z - alpha * av.z; rv.w = rv.w - alpha * av.w;
        pp[i] = pv;
        r[i] = rv;
        const float z0 = rv.x * precon_of(a.x), z1 = rv.y * precon_of(a.y), z2 = rv.z * precon_of(a.z), z3 = rv.w * precon_of(a.w);
        acc.add(z0 * rv.x);
        acc.add(z1 * rv.y);
        acc.add(z2 * rv.z);
        acc.add(z3 * rv.w);
        const bool absv = !reference || i < xy4;  // the reference takes |r| on the z = 0 plane only (Q4)
        const float m0 = absv ? fabsf(rv.x) : rv.x, m1 = absv ? fabsf(rv.y) : rv.y;
        const float m2 = absv ? fabsf(rv.z) : rv.z, m3 = absv ? fabsf(rv.w) : rv.w;
        if (m0 > mx) mx = m0;
        if (m1 > mx) mx = m1;
        if (m2 > mx) mx = m2;
        if (m3 > mx) mx = m3;
    }
    const double bs = block_sum_n<UT>(double(acc.s) - double(acc.c), smd, threadIdx.x);
    const float bm = block_max_n<UT>(mx, smf, threadIdx.x);
    double tot;
    float mall;
    if (publish_n<UT>(sc, partials, blockIdx.x, gridDim.x, threadIdx.x, bs, bm, tot, mall)) {
        sc->iters += 1;
        sc->residual = mall;
        if (mall <= tol) {
            sc->converged = 1;
        } else if (sc->iters >= max_iter) {
            sc->converged = 2;
        } else {
            sc->sigma1 = tot;
            sc->beta_f = float(tot / sc->sigma0);
            sc->sigma0 = tot;
        }
    }
}

// s = r/diag + beta s over all cells as float4
__global__ void __launch_bounds__(UT) k_search4(int n4, const float4* __restrict__ aw, const float4* __restrict__ r, float4* __restrict__ s,
                                                const Scalars* sc) {
    if (sc->converged) return;
    const float beta = sc->beta_f;
    for (int i = blockIdx.x * UT + threadIdx.x; i < n4; i += gridDim.x * UT) {
        const float4 a = aw[i], rv = r[i];
        float4 sv = s[i];
        sv.x = rv.x * precon_of(a.x) + beta * sv.x;
        sv.y = rv.y * precon_of(a.y) + beta * sv.y;
        sv.z = rv.z * precon_of(a.z) + beta * sv.z;
        sv.w = rv.w * precon_of(a.w) + beta * sv.w;
        s[i] = sv;
    }
}

constexpr int MVY = 32;           // y rows per block (neighbour rows of s mostly from L1)
constexpr int MVT = 32 * MVY;     // threads per block

__device__ __forceinline__ float4 ld4(const float* p, int c) { return *reinterpret_cast<const float4*>(p + c); }
__device__ __forceinline__ float4 f4zero() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }

// As = A s and s.As with 4 cells per thread along x and a march along z that keeps the planes
// z-1, z, z+1 of s and the previous plane's z-coefficient in registers. Neighbours outside the
// domain read as 0; ground neighbours need no test because their s and coefficients are 0.
// FLAT: the ground is the row y = 0 only (no heightfield reads).
template <bool FLAT>
__global__ void __launch_bounds__(MVT) k_matvec4(Grid g, int zlen, const float* __restrict__ ax, const float* __restrict__ ay,
                                                 const float* __restrict__ az, const float* __restrict__ aw, const float* __restrict__ s,
                                                 float* __restrict__ As, int reference, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[MVT / 32];
    const int lane = threadIdx.x, tid = threadIdx.x + 32 * threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * MVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const bool act = x0 < g.X && y < g.Y;
    const int X = g.X, XY = g.XY;
    const int row = x0 + y * X;
    Kahan acc;
    float4 sb = f4zero(), scur = f4zero(), azb = f4zero();
    if (act) {
        const int c = row + zs * XY;
        scur = ld4(s, c);
        if (zs > 0) { sb = ld4(s, c - XY); azb = ld4(az, c - XY); }
    }
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 sf = f4zero(), sd = f4zero(), su = f4zero(), ayd = f4zero(), cx = f4zero(), cy = f4zero(), cz = f4zero(), cw = f4zero();
        int4 gh4 = make_int4(0, 0, 0, 0);
        if (act) {
            if (z + 1 < g.Z) sf = ld4(s, c + XY);
            if (y > 0) { sd = ld4(s, c - X); ayd = ld4(ay, c - X); }
            if (y + 1 < g.Y) su = ld4(s, c + X);
            cx = ld4(ax, c); cy = ld4(ay, c); cz = ld4(az, c); cw = ld4(aw, c);
            if (!FLAT) gh4 = *reinterpret_cast<const int4*>(g.gh + x0 + z * X);
        }
        // x neighbours through the neighbouring lanes; the warp's edge lanes load them
        float sl = __shfl_up_sync(0xffffffffu, scur.w, 1);
        float axl = __shfl_up_sync(0xffffffffu, cx.w, 1);
        float sr = __shfl_down_sync(0xffffffffu, scur.x, 1);
        if (act && lane == 0) {
            if (x0 > 0) { sl = s[c - 1]; axl = ax[c - 1]; } else { sl = 0.0f; axl = 0.0f; }
        }
        if (act && (lane == 31 || x0 + 4 >= X)) sr = (x0 + 4 < X) ? s[c + 4] : 0.0f;
        if (act) {
            float AL0 = axl, AL1 = cx.x, AL2 = cx.y, AL3 = cx.z;
            float AD0 = ayd.x, AD1 = ayd.y, AD2 = ayd.z, AD3 = ayd.w;
            float AB0 = azb.x, AB1 = azb.y, AB2 = azb.z, AB3 = azb.w;
            if (reference) {
                AL0 = char_trunc(AL0); AL1 = char_trunc(AL1); AL2 = char_trunc(AL2); AL3 = char_trunc(AL3);
                AD0 = char_trunc(AD0); AD1 = char_trunc(AD1); AD2 = char_trunc(AD2); AD3 = char_trunc(AD3);
                AB0 = char_trunc(AB0); AB1 = char_trunc(AB1); AB2 = char_trunc(AB2); AB3 = char_trunc(AB3);
            }
            float4 o;
            o.x = cw.x * scur.x + ((AL0 * sl + AD0 * sd.x + AB0 * sb.x + cx.x * scur.y + cy.x * su.x + cz.x * sf.x));
            o.y = cw.y * scur.y + ((AL1 * scur.x + AD1 * sd.y + AB1 * sb.y + cx.y * scur.z + cy.y * su.y + cz.y * sf.y));
            o.z = cw.z * scur.z + ((AL2 * scur.y + AD2 * sd.z + AB2 * sb.z + cx.z * scur.w + cy.z * su.z + cz.z * sf.z));
            o.w = cw.w * scur.w + ((AL3 * scur.z + AD3 * sd.w + AB3 * sb.w + cx.w * sr + cy.w * su.w + cz.w * sf.w));
            if (FLAT) {
                if (y == 0) o = f4zero();
            } else {
                if (y <= gh4.x) o.x = 0.0f;
                if (y <= gh4.y) o.y = 0.0f;
                if (y <= gh4.z) o.z = 0.0f;
                if (y <= gh4.w) o.w = 0.0f;
            }
            *reinterpret_cast<float4*>(As + c) = o;
            acc.add(o.x * scur.x);
            acc.add(o.y * scur.y);
            acc.add(o.z * scur.z);
            acc.add(o.w * scur.w);
        }
        sb = scur;
        scur = sf;
        azb = cz;
    }
    const double bs = block_sum_n<MVT>(double(acc.s) - double(acc.c), smd, tid);
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    double tot;
    float mall;
    if (publish_n<MVT>(sc, partials, bid, nb, tid, bs, 0.0f, tot, mall)) {
        const double s1 = reference ? sc->sigma1 + tot : tot;
        sc->sigma1 = s1;
        sc->alpha = float(sc->sigma0 / s1);
    }
}

// ---- fused PCG iteration (X % 4 == 0): two launches per iteration instead of three --------
// The search step (endIteration :987-1014) and the next matrix product share one z march, and
// the pressure update of the previous iteration (updatePandDiv :955-985, p += alpha s) rides
// along where s_old is read anyway. The residual kernel stores z = r/diag (it forms z for z.r in
// any case), so the operator forms s_new = z + beta s_old from two arrays wherever it needs a
// neighbour's value. Every value is formed as in k_search4 / k_update4 (the search direction as
// fma(beta, s_old, z), the pressure as fma(alpha, s, p)); only the dot products' summation order
// differs.

// s_new = z + beta s_old, As = A s_new, s_new.As -> alpha, and p += alpha_pp s_old. The rows
// above and below and the next plane form their s_new from z and s_old (another warp's or
// block's rows, read through L1/L2); the x neighbours come from the neighbouring lanes. s_old
// and s_new are distinct buffers (a block's halo rows are another block's own rows, so s cannot
// be updated in place).
template <bool FLAT>
__global__ void __launch_bounds__(MVT) k_matvec_search4(Grid g, int zlen, const float* __restrict__ ax, const float* __restrict__ ay,
                                                        const float* __restrict__ az, const float* __restrict__ aw,
                                                        const float* __restrict__ zv, const float* __restrict__ sold,
                                                        float* __restrict__ snew, float* __restrict__ As, float* __restrict__ pp,
                                                        int reference, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[MVT / 32];
    const float beta = sc->beta_f, alpha_pp = sc->alpha_pp;
    const int lane = threadIdx.x, tid = threadIdx.x + 32 * threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * MVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const bool act = x0 < g.X && y < g.Y;
    const int X = g.X, XY = g.XY;
    const int row = x0 + y * X;
    auto srow = [&](int c) {
        const float4 z = ld4(zv, c), so = ld4(sold, c);
        return make_float4(__fmaf_rn(beta, so.x, z.x), __fmaf_rn(beta, so.y, z.y), __fmaf_rn(beta, so.z, z.z), __fmaf_rn(beta, so.w, z.w));
    };
    auto sone = [&](int c) { return __fmaf_rn(beta, sold[c], zv[c]); };
    Kahan acc;
    float4 vb = f4zero(), vc = f4zero(), azb = f4zero();
    if (act) {
        const int c = row + zs * XY;
        vc = srow(c);
        if (zs > 0) { vb = srow(c - XY); azb = ld4(az, c - XY); }
    }
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 vf = f4zero(), vd = f4zero(), vu = f4zero(), ayd = f4zero(), cx = f4zero(), cy = f4zero(), cz = f4zero(), cw = f4zero();
        int4 gh4 = make_int4(0, 0, 0, 0);
        if (act) {
            if (z + 1 < g.Z) vf = srow(c + XY);
            if (y > 0) { vd = srow(c - X); ayd = ld4(ay, c - X); }
            if (y + 1 < g.Y) vu = srow(c + X);
            cx = ld4(ax, c); cy = ld4(ay, c); cz = ld4(az, c); cw = ld4(aw, c);
            if (!FLAT) gh4 = *reinterpret_cast<const int4*>(g.gh + x0 + z * X);
            // the previous iteration's pressure update (s_old of this row was read for vc)
            const float4 so = ld4(sold, c);
            float4 pv = ld4(pp, c);
            pv.x = __fmaf_rn(alpha_pp, so.x, pv.x);
            pv.y = __fmaf_rn(alpha_pp, so.y, pv.y);
            pv.z = __fmaf_rn(alpha_pp, so.z, pv.z);
            pv.w = __fmaf_rn(alpha_pp, so.w, pv.w);
            *reinterpret_cast<float4*>(pp + c) = pv;
        }
        float sl = __shfl_up_sync(0xffffffffu, vc.w, 1);
        float axl = __shfl_up_sync(0xffffffffu, cx.w, 1);
        float sr = __shfl_down_sync(0xffffffffu, vc.x, 1);
        if (act && lane == 0) {
            if (x0 > 0) { sl = sone(c - 1); axl = ax[c - 1]; } else { sl = 0.0f; axl = 0.0f; }
        }
        if (act && (lane == 31 || x0 + 4 >= X)) sr = (x0 + 4 < X) ? sone(c + 4) : 0.0f;
        if (act) {
            float AL0 = axl, AL1 = cx.x, AL2 = cx.y, AL3 = cx.z;
            float AD0 = ayd.x, AD1 = ayd.y, AD2 = ayd.z, AD3 = ayd.w;
            float AB0 = azb.x, AB1 = azb.y, AB2 = azb.z, AB3 = azb.w;
            if (reference) {
                AL0 = char_trunc(AL0); AL1 = char_trunc(AL1); AL2 = char_trunc(AL2); AL3 = char_trunc(AL3);
                AD0 = char_trunc(AD0); AD1 = char_trunc(AD1); AD2 = char_trunc(AD2); AD3 = char_trunc(AD3);
                AB0 = char_trunc(AB0); AB1 = char_trunc(AB1); AB2 = char_trunc(AB2); AB3 = char_trunc(AB3);
            }
            float4 o;
            o.x = cw.x * vc.x + ((AL0 * sl + AD0 * vd.x + AB0 * vb.x + cx.x * vc.y + cy.x * vu.x + cz.x * vf.x));
            o.y = cw.y * vc.y + ((AL1 * vc.x + AD1 * vd.y + AB1 * vb.y + cx.y * vc.z + cy.y * vu.y + cz.y * vf.y));
            o.z = cw.z * vc.z + ((AL2 * vc.y + AD2 * vd.z + AB2 * vb.z + cx.z * vc.w + cy.z * vu.z + cz.z * vf.z));
            o.w = cw.w * vc.w + ((AL3 * vc.z + AD3 * vd.w + AB3 * vb.w + cx.w * sr + cy.w * vu.w + cz.w * vf.w));
            if (FLAT) {
                if (y == 0) o = f4zero();
            } else {
                if (y <= gh4.x) o.x = 0.0f;
                if (y <= gh4.y) o.y = 0.0f;
                if (y <= gh4.z) o.z = 0.0f;
                if (y <= gh4.w) o.w = 0.0f;
            }
            *reinterpret_cast<float4*>(snew + c) = vc;
            *reinterpret_cast<float4*>(As + c) = o;
            acc.add(o.x * vc.x);
            acc.add(o.y * vc.y);
            acc.add(o.z * vc.z);
            acc.add(o.w * vc.w);
        }
        vb = vc;
        vc = vf;
        azb = cz;
    }
    const double bs = block_sum_n<MVT>(double(acc.s) - double(acc.c), smd, tid);
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    double tot;
    float mall;
    if (publish_n<MVT>(sc, partials, bid, nb, tid, bs, 0.0f, tot, mall)) {
        const double s1 = reference ? sc->sigma1 + tot : tot;
        sc->sigma1 = s1;
        sc->alpha = float(sc->sigma0 / s1);
    }
}

// r -= alpha As, z = r/diag (stored), z.r and the max residual: k_update4 without the pressure
// update, which the next k_matvec_search4 or k_pressure_tail4 applies with alpha_pp = alpha
__global__ void __launch_bounds__(UT) k_residual4(int n4, int xy4, const float4* __restrict__ aw, const float4* __restrict__ As,
                                                  float4* __restrict__ r, float4* __restrict__ zout, int reference, float tol,
                                                  int max_iter, Scalars* sc, double* partials) {
    if (sc->converged) return;
    __shared__ double smd[UT / 32];
    __shared__ float smf[UT / 32];
    const float alpha = sc->alpha;
    Kahan acc;
    float mx = 0.0f;
    for (int i = blockIdx.x * UT + threadIdx.x; i < n4; i += gridDim.x * UT) {
        const float4 a = aw[i], av = As[i];
        float4 rv = r[i];
        rv.x = rv.x - alpha * av.x; rv.y = rv.y - alpha * av.y; rv.z = rv.z - alpha * av.z; rv.w = rv.w - alpha * av.w;
        r[i] = rv;
        const float z0 = rv.x * precon_of(a.x), z1 = rv.y * precon_of(a.y), z2 = rv.z * precon_of(a.z), z3 = rv.w * precon_of(a.w);
        zout[i] = make_float4(z0, z1, z2, z3);
        acc.add(z0 * rv.x);
        acc.add(z1 * rv.y);
        acc.add(z2 * rv.z);
        acc.add(z3 * rv.w);
        const bool absv = !reference || i < xy4;  // the reference takes |r| on the z = 0 plane only (Q4)
        const float m0 = absv ? fabsf(rv.x) : rv.x, m1 = absv ? fabsf(rv.y) : rv.y;
        const float m2 = absv ? fabsf(rv.z) : rv.z, m3 = absv ? fabsf(rv.w) : rv.w;
        if (m0 > mx) mx = m0;
        if (m1 > mx) mx = m1;
        if (m2 > mx) mx = m2;
        if (m3 > mx) mx = m3;
    }
    const double bs = block_sum_n<UT>(double(acc.s) - double(acc.c), smd, threadIdx.x);
    const float bm = block_max_n<UT>(mx, smf, threadIdx.x);
    double tot;
    float mall;
    if (publish_n<UT>(sc, partials, blockIdx.x, gridDim.x, threadIdx.x, bs, bm, tot, mall)) {
        sc->iters += 1;
        sc->residual = mall;
        sc->alpha_pp = alpha;
        if (mall <= tol) {
            sc->converged = 1;
        } else if (sc->iters >= max_iter) {
            sc->converged = 2;
        } else {
            sc->sigma1 = tot;
            sc->beta_f = float(tot / sc->sigma0);
            sc->sigma0 = tot;
        }
    }
}

// the last iteration's pressure update: p += alpha_pp s
__global__ void __launch_bounds__(UT) k_pressure_tail4(int n4, const float4* __restrict__ s, float4* __restrict__ pp, const Scalars* sc) {
    const float alpha = sc->alpha_pp;
    for (int i = blockIdx.x * UT + threadIdx.x; i < n4; i += gridDim.x * UT) {
        const float4 sv = s[i];
        float4 pv = pp[i];
        pv.x = __fmaf_rn(alpha, sv.x, pv.x);
        pv.y = __fmaf_rn(alpha, sv.y, pv.y);
        pv.z = __fmaf_rn(alpha, sv.z, pv.z);
        pv.w = __fmaf_rn(alpha, sv.w, pv.w);
        pp[i] = pv;
    }
}

// graph mode: the last iteration's pressure update from the direction buffer of its parity
__global__ void __launch_bounds__(UT) k_pressure_tail_sel(int n4, const float4* __restrict__ s0, const float4* __restrict__ s1,
                                                          float4* __restrict__ pp, const Scalars* sc) {
    const int it = sc->iters;
    if (it <= 0) return;
    const float4* __restrict__ s = ((it - 1) & 1) ? s1 : s0;
    const float alpha = sc->alpha_pp;
    for (int i = blockIdx.x * UT + threadIdx.x; i < n4; i += gridDim.x * UT) {
        const float4 sv = s[i];
        float4 pv = pp[i];
        pv.x = __fmaf_rn(alpha, sv.x, pv.x);
        pv.y = __fmaf_rn(alpha, sv.y, pv.y);
        pv.z = __fmaf_rn(alpha, sv.z, pv.z);
        pv.w = __fmaf_rn(alpha, sv.w, pv.w);
        pp[i] = pv;
    }
}

// graph mode, PCG loop: run (another) chunk of iterations while the solver has not stopped and no
// NaN was met; loop >= 0 counts a completed trip
__global__ void k_pcg_cond(cudaGraphConditionalHandle h, Scalars* sc, int loop) {
    if (loop >= 0) note_trip(sc, loop);
    cudaGraphSetConditional(h, (sc->converged == 0 && sc->status == 0) ? 1u : 0u);
}

// k_build for flat terrain and X % 4 == 0: four cells per thread, a march along z in blocks of
// MVY rows. Each cell's reciprocal density is formed once (the x neighbours' by shuffle, the next
// plane's carried), and each face once: a cell forms its right, up and front faces; the left face
// is the right face of the cell before (a shuffle across lanes), the back face the front face of
// the previous plane, the down face is formed again from the row below. coef_of and the harmonic
// mean are symmetric in their two densities (IEEE addition commutes), so every value equals
// k_build's; z.r is summed in FP64 in a different order.
__device__ __forceinline__ float fcomp(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }
__device__ __forceinline__ void fset(float4& v, int k, float a) {
    if (k == 0) v.x = a; else if (k == 1) v.y = a; else if (k == 2) v.z = a; else v.w = a;
}
__device__ __forceinline__ void face_of(float c, float rc, float n, float rn, float& h, float& coef) {
    // hm(n) = 2/(1/c + 1/n) and coef_of(c, n) = -max(1, 1.225/hm), both 0 across a zero density
    if (n == 0.0f) { h = 0.0f; coef = 0.0f; return; }
    h = 2.0f / (rc + rn);
    coef = -fmaxf(1.0f, 1.225f / h);
    (void)c;
}
__global__ void __launch_bounds__(MVT) k_build4(Grid g, int zlen, const float* __restrict__ rho, const float* __restrict__ u,
                                                const float* __restrict__ v, const float* __restrict__ w,
                                                const float* __restrict__ defU, const float* __restrict__ defW, float dt,
                                                float* __restrict__ ax, float* __restrict__ ay, float* __restrict__ az,
                                                float* __restrict__ aw, float* __restrict__ r, float* __restrict__ s,
                                                float* __restrict__ pp, float* __restrict__ As, int reference, Scalars* sc,
                                                double* partials) {
    __shared__ double smd[MVT / 32];
    __shared__ float smf[MVT / 32];
    const int lane = threadIdx.x, tid = threadIdx.x + 32 * threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * MVY + threadIdx.y;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const bool act = x0 < g.X && y < g.Y;
    const bool sky = act && y >= 1;
    const int X = g.X, XY = g.XY, Z = g.Z;
    const int row = x0 + y * X;
    const float4 z4 = make_float4(0, 0, 0, 0);
    double dsum = 0.0;
    float mx = 0.0f;
    const float du_ = sky ? defU[y] : 0.0f, dw_ = sky ? defW[y] : 0.0f;
    // own plane: density and reciprocal; the back face (front face of the plane before) and w there
    float4 pc = z4, rc = z4, hB = z4, cB = z4, wB = z4;
    if (sky) {
        pc = ld4(rho, row + zs * XY);
        rc = make_float4(1.0f / pc.x, 1.0f / pc.y, 1.0f / pc.z, 1.0f / pc.w);
        float4 pb = pc, rb = rc;  // outside at z = 0: the own density (NEUMANN)
        if (zs > 0) {
            pb = ld4(rho, row + (zs - 1) * XY);
            rb = make_float4(1.0f / pb.x, 1.0f / pb.y, 1.0f / pb.z, 1.0f / pb.w);
            wB = ld4(w, row + (zs - 1) * XY);
        } else {
            wB = make_float4(dw_, dw_, dw_, dw_);
        }
        face_of(pc.x, rc.x, pb.x, rb.x, hB.x, cB.x);
        face_of(pc.y, rc.y, pb.y, rb.y, hB.y, cB.y);
        face_of(pc.z, rc.z, pb.z, rb.z, hB.z, cB.z);
        face_of(pc.w, rc.w, pb.w, rb.w, hB.w, cB.w);
    }
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 pf = pc, rf = rc, pd = z4, rd = z4, pu = pc, ru = rc, uo = z4, vo = z4, wo = z4, vd = z4;
        if (sky) {
            if (z + 1 < Z) {
                pf = ld4(rho, c + XY);
                rf = make_float4(1.0f / pf.x, 1.0f / pf.y, 1.0f / pf.z, 1.0f / pf.w);
            }
            if (y > 1) {  // the row below (y = 1 has the ground below: density 0, v 0)
                pd = ld4(rho, c - X);
                rd = make_float4(1.0f / pd.x, 1.0f / pd.y, 1.0f / pd.z, 1.0f / pd.w);
                vd = ld4(v, c - X);
            }
            if (y + 1 < g.Y) {
                pu = ld4(rho, c + X);
                ru = make_float4(1.0f / pu.x, 1.0f / pu.y, 1.0f / pu.z, 1.0f / pu.w);
            }
            uo = ld4(u, c);
            vo = ld4(v, c);
            wo = ld4(w, c);
        }
        // the right neighbour of the last cell and the left neighbour of the first
        float pr = __shfl_down_sync(0xffffffffu, pc.x, 1), rr = __shfl_down_sync(0xffffffffu, rc.x, 1);
        float ul = __shfl_up_sync(0xffffffffu, uo.w, 1);
        if (sky && (lane == 31 || x0 + 4 >= X)) {
            if (x0 + 4 < X) { pr = rho[c + 4]; rr = 1.0f / pr; }
            else { pr = pc.w; rr = rc.w; }  // outside: the own density (NEUMANN)
        }
        float hR[4], cR[4];
        face_of(pc.x, rc.x, pc.y, rc.y, hR[0], cR[0]);
        face_of(pc.y, rc.y, pc.z, rc.z, hR[1], cR[1]);
        face_of(pc.z, rc.z, pc.w, rc.w, hR[2], cR[2]);
        face_of(pc.w, rc.w, pr, rr, hR[3], cR[3]);
        float hL0 = __shfl_up_sync(0xffffffffu, hR[3], 1), cL0 = __shfl_up_sync(0xffffffffu, cR[3], 1);
        if (sky && lane == 0) {
            float pl = pc.x, rl = rc.x;
            if (x0 > 0) { pl = rho[c - 1]; rl = 1.0f / pl; ul = u[c - 1]; }
            else ul = du_;
            face_of(pc.x, rc.x, pl, rl, hL0, cL0);
        }
        if (sky) {
            const float hL[4] = {hL0, hR[0], hR[1], hR[2]}, cL[4] = {cL0, cR[0], cR[1], cR[2]};
            const float uL[4] = {ul, uo.x, uo.y, uo.z};
            float4 oax, oay, oaz, oaw, orr, oss;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float cur = fcomp(pc, k);
                float hU, cU, hD, cD, hF, cF;
                face_of(cur, fcomp(rc, k), fcomp(pu, k), fcomp(ru, k), hU, cU);
                face_of(cur, fcomp(rc, k), fcomp(pd, k), fcomp(rd, k), hD, cD);
                face_of(cur, fcomp(rc, k), fcomp(pf, k), fcomp(rf, k), hF, cF);
                float wd = 0.0f;
                wd -= cR[k]; wd -= cL[k]; wd -= cU; wd -= cD; wd -= cF; wd -= fcomp(cB, k);
                const float mfd = ((hR[k] * fcomp(uo, k) - hL[k] * uL[k]) + (hU * fcomp(vo, k) - hD * fcomp(vd, k)) +
                                   (hF * fcomp(wo, k) - fcomp(hB, k) * fcomp(wB, k)));
                const float dch = (cur - cur) / dt;  // the reference's old density is a copy of rho
                const float rv = mfd - dch;
                const float zv = rv * precon_of(wd);
                fset(oax, k, cR[k]); fset(oay, k, cU); fset(oaz, k, cF); fset(oaw, k, wd);
                fset(orr, k, rv); fset(oss, k, zv);
                dsum += double(zv) * double(rv);
                const float m = (!reference || z == 0) ? fabsf(rv) : rv;
                if (m > mx) mx = m;
                fset(hB, k, hF); fset(cB, k, cF);
            }
            *reinterpret_cast<float4*>(ax + c) = oax;
            *reinterpret_cast<float4*>(ay + c) = oay;
            *reinterpret_cast<float4*>(az + c) = oaz;
            *reinterpret_cast<float4*>(aw + c) = oaw;
            *reinterpret_cast<float4*>(r + c) = orr;
            *reinterpret_cast<float4*>(s + c) = oss;
            *reinterpret_cast<float4*>(pp + c) = z4;
            *reinterpret_cast<float4*>(As + c) = z4;
        } else if (act) {  // the ground row
            *reinterpret_cast<float4*>(ax + c) = z4;
            *reinterpret_cast<float4*>(ay + c) = z4;
            *reinterpret_cast<float4*>(az + c) = z4;
            *reinterpret_cast<float4*>(aw + c) = z4;
            *reinterpret_cast<float4*>(r + c) = z4;
            *reinterpret_cast<float4*>(s + c) = z4;
            *reinterpret_cast<float4*>(pp + c) = z4;
            *reinterpret_cast<float4*>(As + c) = z4;
        }
        pc = pf;
        rc = rf;
        wB = wo;
    }
    const double bs = block_sum_n<MVT>(dsum, smd, tid);
    const float bm = block_max_n<MVT>(mx, smf, tid);
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    double tot;
    float mall;
    if (publish_n<MVT>(sc, partials, bid, nb, tid, bs, bm, tot, mall)) {
        sc->sigma0 = tot;
        sc->sigma1 = 0.0;
        sc->iters = 0;
        sc->residual = mall;
        sc->converged = (mall == 0.0f) ? 1 : 0;
    }
}

// updatePressure (:1016-1030) followed by initDensity (:1432-1452)
__global__ void __launch_bounds__(256) k_press_dens(Grid g, float* __restrict__ p, const float* __restrict__ pp, float* __restrict__ rho,
                                                    const float* __restrict__ th, const float* __restrict__ qv, const float* __restrict__ Pg) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    const float pn = p[c] - pp[c] / 100.0f;
    p[c] = pn;
    const float Tt = th[c] * powf(pn / Pg[x + z * g.X], KC::KAPPA);
    const float Tv = Tt * (0.608f * qv[c] + 1);
    rho[c] = pn * 100 / (KC::Rsd * Tv);
}

// applyPresProjGPU Game/kernelSky.cu:862-908 (pressure bounds DIRICHLET sides / NEUMANN ground,
// density bounds NEUMANN sides / DIRICHLET ground)
__global__ void __launch_bounds__(256) k_apply_proj(Grid g, const float* __restrict__ pp, const float* __restrict__ rho, float* __restrict__ u,
                                                    float* __restrict__ v, float* __restrict__ w) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    const float cp = pp[c], cd = rho[c];
    const float pr = face_nb(g, pp, x, y, z, 1, 0, 0, DIRICHLET, NEUMANN, 0.0f);
    const float pu = face_nb(g, pp, x, y, z, 0, 1, 0, DIRICHLET, NEUMANN, 0.0f);
    const float pf = face_nb(g, pp, x, y, z, 0, 0, 1, DIRICHLET, NEUMANN, 0.0f);
    float dr = face_nb(g, rho, x, y, z, 1, 0, 0, NEUMANN, DIRICHLET, 0.0f);
    float du = face_nb(g, rho, x, y, z, 0, 1, 0, NEUMANN, DIRICHLET, 0.0f);
    float df = face_nb(g, rho, x, y, z, 0, 0, 1, NEUMANN, DIRICHLET, 0.0f);
    dr = dr == 0.0f ? cd : 2.0f / (1.0f / cd + 1.0f / dr);
    du = du == 0.0f ? cd : 2.0f / (1.0f / cd + 1.0f / du);
    df = df == 0.0f ? cd : 2.0f / (1.0f / cd + 1.0f / df);
    u[c] += (pr - cp) / dr;
    v[c] += (pu - cp) / du;
    w[c] += (pf - cp) / df;
}

// k_apply_proj for flat terrain and X % 4 == 0: four cells per thread and a march along z over the
// sky rows (the next plane's pressure correction and density are the front neighbours and become
// the next step's own values); each cell's reciprocal density is formed once. Flat ground is
// the row y = 0, so the +x, +y and +z neighbours of a sky cell are never ground: outside the
// domain the correction is 0 (DIRICHLET) and the density the cell's own (NEUMANN). Same
// arithmetic as k_apply_proj.
__global__ void __launch_bounds__(256) k_apply_proj4(Grid g, int zlen, const float* __restrict__ pp, const float* __restrict__ rho,
                                                     float* __restrict__ u, float* __restrict__ v, float* __restrict__ w) {
    const int lane = threadIdx.x;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * 8 + threadIdx.y + 1;  // sky rows start at y = 1
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const bool act = x0 < g.X && y < g.Y;
    const int X = g.X, XY = g.XY;
    const int row = x0 + y * X;
    float4 pc = f4zero(), dc = f4zero();
    if (act) {
        pc = ld4(pp, row + zs * XY);
        dc = ld4(rho, row + zs * XY);
    }
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 pf = f4zero(), df = dc, pu = f4zero(), du = dc;
        if (act) {
            if (z + 1 < g.Z) { pf = ld4(pp, c + XY); df = ld4(rho, c + XY); }
            if (y + 1 < g.Y) { pu = ld4(pp, c + X); du = ld4(rho, c + X); }
        }
        float pr3 = __shfl_down_sync(0xffffffffu, pc.x, 1), dr3 = __shfl_down_sync(0xffffffffu, dc.x, 1);
        if (act && (lane == 31 || x0 + 4 >= X)) {
            if (x0 + 4 < X) { pr3 = pp[c + 4]; dr3 = rho[c + 4]; }
            else { pr3 = 0.0f; dr3 = dc.w; }
        }
        if (act) {
            const float prx[4] = {pc.y, pc.z, pc.w, pr3}, drx[4] = {dc.y, dc.z, dc.w, dr3};
            float4 uo = ld4(u, c), vo = ld4(v, c), wo = ld4(w, c);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float cp = fcomp(pc, k), cd = fcomp(dc, k), rc = 1.0f / cd;
                float dr = drx[k], dU = fcomp(du, k), dF = fcomp(df, k);
                dr = dr == 0.0f ? cd : 2.0f / (rc + 1.0f / dr);
                dU = dU == 0.0f ? cd : 2.0f / (rc + 1.0f / dU);
                dF = dF == 0.0f ? cd : 2.0f / (rc + 1.0f / dF);
                fset(uo, k, fcomp(uo, k) + (prx[k] - cp) / dr);
                fset(vo, k, fcomp(vo, k) + (fcomp(pu, k) - cp) / dU);
                fset(wo, k, fcomp(wo, k) + (fcomp(pf, k) - cp) / dF);
            }
            *reinterpret_cast<float4*>(u + c) = uo;
            *reinterpret_cast<float4*>(v + c) = vo;
            *reinterpret_cast<float4*>(w + c) = wo;
        }
        pc = pf;
        dc = df;
    }
}

}  // namespace

// As = A s and s.As -> alpha (textbook operator, vectorised; X % 4 == 0)
void launch_matvec_textbook(Env& e, const float* s, float* As) {
    const Grid& g = e.g;
    const dim3 mvb(32, MVY);
    const int gx = (g.X / 4 + 31) / 32, gy = (g.Y + MVY - 1) / MVY;
    int zc = std::max(1, std::min(g.Z, (e.num_sms * 8 + gx * gy - 1) / (gx * gy)));
    while (gx * gy * zc > kMaxPartials && zc > 1) --zc;
    const int zlen = (g.Z + zc - 1) / zc;
    zc = (g.Z + zlen - 1) / zlen;
    if (e.flat)
        k_matvec4<true><<<dim3(gx, gy, zc), mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, s, As, 0, e.sc, e.partials);
    else
        k_matvec4<false><<<dim3(gx, gy, zc), mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, s, As, 0, e.sc, e.partials);
    e.launches += 1;
}

void launch_project(Env& e, float dtS) {
    const Grid& g = e.g;
    const Tiles T = tiles_of(g);
    const int ref = e.cfg.semantics == 0;
    const int nblk = std::min(std::min(T.n, e.num_sms * 4), kMaxPartials);
    {
    ProfScope ps(e, "proj_setup");
    e.launches += 2;
    k_reset_vel<<<(g.XY + 127) / 128, 128, 0, e.stream>>>(g, e.u, e.v, e.w, e.defU, e.defW, ref);
    if (e.flat && (g.X % 4) == 0) {
        const int gx = (g.X / 4 + 31) / 32, gy = (g.Y + MVY - 1) / MVY;
        int zc = std::max(1, std::min(g.Z, (e.num_sms * 4 + gx * gy - 1) / (gx * gy)));
        while (gx * gy * zc > kMaxPartials && zc > 1) --zc;
        const int zlen = (g.Z + zc - 1) / zc;
        zc = (g.Z + zlen - 1) / zlen;
        k_build4<<<dim3(gx, gy, zc), dim3(32, MVY), 0, e.stream>>>(g, zlen, e.rho, e.u, e.v, e.w, e.defU, e.defW, dtS, e.ax, e.ay, e.az,
                                                                   e.aw, e.r, e.s, e.pp, e.As, ref, e.sc, e.partials);
    } else {
        k_build<<<nblk, NT, 0, e.stream>>>(g, T, e.rho, e.u, e.v, e.w, e.defU, e.defW, dtS, e.ax, e.ay, e.az, e.aw, e.r, e.s, e.pp, e.As,
                                          ref, e.sc, e.partials);
    }
    }
    if (e.cfg.precision == 1) {
        mg_solve(e);
    } else {
    const int chunk = 8;
    const bool vec = (g.X % 4) == 0;
    // vectorised launch shapes: streams at 16 blocks/SM (several waves of the grid-stride loop:
    // 8 per SM, 1.3 waves, left the second wave a third full), the matvec's z chunks sized to fill
    // the GPU
    const int n4 = g.N / 4;
    const int nstream = std::min(std::min((n4 + UT - 1) / UT, e.num_sms * 16), kMaxPartials);
    const dim3 mvb(32, MVY);
    const int gx = (g.X / 4 + 31) / 32, gy = (g.Y + MVY - 1) / MVY;
    // about 6 blocks of 1024 threads per SM in the operator's grid (one resident at a time): at
    // 512x512x256 the operator took 86.5 ms per step at 6, 87.0 at 8, 87.6 at 4, 89.1 at 12
    int zc = std::max(1, std::min(g.Z, (e.num_sms * 6 + gx * gy - 1) / (gx * gy)));
    while (gx * gy * zc > kMaxPartials && zc > 1) --zc;
    const int zlen = (g.Z + zc - 1) / zc;
    zc = (g.Z + zlen - 1) / zlen;
    const dim3 mvg(gx, gy, zc);
    // fused iterations: the search directions alternate between e.s and e.tB, z = r/diag lives in
    // e.tA (both free during the projection: the advection's scratch); iteration k's direction is
    // dirs[k % 2]
    float* dirs[2] = {e.s, e.tB};
    float* zbuf = e.tA;
    // iteration kk of the PCG (directions alternate between the two buffers in the fused form)
    auto iterate = [&](int kk) {
            if (vec && e.cfg.pcg_fused) {
                float* sd = dirs[kk & 1];
                { ProfScope ps(e, "pcg_matvec"); e.launches += 1;
                  if (kk == 0) {  // the first direction is z itself (set by the build)
                      if (e.flat) k_matvec4<true><<<mvg, mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, sd, e.As, ref, e.sc, e.partials);
                      else k_matvec4<false><<<mvg, mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, sd, e.As, ref, e.sc, e.partials);
                  } else {
                      const float* so = dirs[(kk - 1) & 1];
                      if (e.flat)
                          k_matvec_search4<true><<<mvg, mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, zbuf, so, sd, e.As, e.pp, ref,
                                                                            e.sc, e.partials);
                      else
                          k_matvec_search4<false><<<mvg, mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, zbuf, so, sd, e.As, e.pp, ref,
                                                                             e.sc, e.partials);
                  } }
                { ProfScope ps(e, "pcg_update"); e.launches += 1;
                  k_residual4<<<nstream, UT, 0, e.stream>>>(n4, g.XY / 4, (const float4*)e.aw, (const float4*)e.As, (float4*)e.r,
                                                            (float4*)zbuf, ref, e.cfg.pcg_tol, e.cfg.pcg_max_iter, e.sc, e.partials); }
            } else if (vec) {
                { ProfScope ps(e, "pcg_matvec"); e.launches += 1;
                  if (e.flat) k_matvec4<true><<<mvg, mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, e.s, e.As, ref, e.sc, e.partials);
                  else k_matvec4<false><<<mvg, mvb, 0, e.stream>>>(g, zlen, e.ax, e.ay, e.az, e.aw, e.s, e.As, ref, e.sc, e.partials); }
                { ProfScope ps(e, "pcg_update"); e.launches += 1;
                  k_update4<<<nstream, UT, 0, e.stream>>>(n4, g.XY / 4, (const float4*)e.aw, (const float4*)e.s, (const float4*)e.As,
                                                          (float4*)e.pp, (float4*)e.r, ref, e.cfg.pcg_tol, e.cfg.pcg_max_iter, e.sc, e.partials); }
                { ProfScope ps(e, "pcg_search"); e.launches += 1;
                  k_search4<<<nstream, UT, 0, e.stream>>>(n4, (const float4*)e.aw, (const float4*)e.r, (float4*)e.s, e.sc); }
            } else {
                { ProfScope ps(e, "pcg_matvec"); e.launches += 1; k_matvec<<<nblk, NT, 0, e.stream>>>(g, T, e.ax, e.ay, e.az, e.aw, e.s, e.As, ref, e.sc, e.partials); }
                { ProfScope ps(e, "pcg_update"); e.launches += 1; k_update<<<nblk, NT, 0, e.stream>>>(g, T, e.aw, e.s, e.As, e.pp, e.r, ref, e.cfg.pcg_tol, e.cfg.pcg_max_iter, e.sc, e.partials); }
                { ProfScope ps(e, "pcg_search"); e.launches += 1; k_search<<<nblk, NT, 0, e.stream>>>(g, T, e.aw, e.r, e.s, e.sc); }
            }
    };
    if (e.capturing) {
        // graph mode: iteration 0, then chunks of `chunk` iterations as a WHILE loop that runs while
        // the solver has not stopped (an even chunk keeps the direction buffers' parity); the
        // kernels of iterations past the stop return at once, as in the stream-ordered form
        if (e.cfg.pcg_max_iter > 0) {
            iterate(0);
            graph_while(
                e, [&](cudaGraphConditionalHandle h) {
                    k_pcg_cond<<<1, 1, 0, e.stream>>>(h, e.sc, -1);
                    e.launches += 1;
                },
                [&](cudaGraphConditionalHandle h, int loop) {
                    for (int kk = 1; kk <= chunk; ++kk) iterate(kk);
                    k_pcg_cond<<<1, 1, 0, e.stream>>>(h, e.sc, loop);
                    e.launches += 1;
                });
            if (vec && e.cfg.pcg_fused) {
                ProfScope ps(e, "pcg_update");
                e.launches += 1;
                k_pressure_tail_sel<<<nstream, UT, 0, e.stream>>>(n4, (const float4*)dirs[0], (const float4*)dirs[1], (float4*)e.pp, e.sc);
            }
        }
    } else {
    for (int it = 0; it < e.cfg.pcg_max_iter; it += chunk) {
        const int n = std::min(chunk, e.cfg.pcg_max_iter - it);
        for (int k = 0; k < n; ++k) iterate(it + k);
        fetch_scalars(e);
        if (e.host_sc->converged || e.host_sc->status != 0) break;
    }
    if (vec && e.cfg.pcg_fused && e.host_sc->iters > 0) {
        // the last iteration's pressure update (no later operator launch carried it)
        ProfScope ps(e, "pcg_update");
        e.launches += 1;
        k_pressure_tail4<<<nstream, UT, 0, e.stream>>>(n4, (const float4*)dirs[(e.host_sc->iters - 1) & 1], (float4*)e.pp, e.sc);
    }
    e.last_iters = e.host_sc->iters;
    e.last_residual = e.host_sc->residual;
    e.last_converged = e.host_sc->converged == 1;
    }
    }
    const dim3 grd((g.X + 31) / 32, (g.Y + 7) / 8, g.Z), blk(32, 8);
    ProfScope ps(e, "proj_apply");
    e.launches += 2;
    k_press_dens<<<grd, blk, 0, e.stream>>>(g, e.p, e.pp, e.rho, e.th, e.qv, e.Pg);
    if (e.flat && (g.X % 4) == 0) {
        const int ax = (g.X / 4 + 31) / 32, ay = (g.Y - 1 + 7) / 8;
        int az = std::max(1, std::min(g.Z, (stencil_sms(e) * 16 + ax * ay - 1) / (ax * ay)));
        const int alen = (g.Z + az - 1) / az;
        az = (g.Z + alen - 1) / alen;
        k_apply_proj4<<<dim3(ax, ay, az), dim3(32, 8), 0, e.stream>>>(g, alen, e.pp, e.rho, e.u, e.v, e.w);
    } else {
        k_apply_proj<<<grd, blk, 0, e.stream>>>(g, e.pp, e.rho, e.u, e.v, e.w);
    }
}

}  // namespace skt
