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

// Publishes one block partial (sum, max) and returns true in thread 0 of the last block to
// finish, which then sees every partial. Partials are summed in block order: deterministic.
__device__ __forceinline__ bool publish(Scalars* sc, double* partials, double sum, float mx, double& tot, float& mxall) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = sum;
        partials[kMaxPartials + blockIdx.x] = double(mx);
        __threadfence();
        const unsigned t = atomicAdd(&sc->done_blocks, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    if (threadIdx.x == 0) {
        __threadfence();
        double s = 0.0, m = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) {
            s += ((volatile double*)partials)[b];
            const double mb = ((volatile double*)partials)[kMaxPartials + b];
            m = mb > m ? mb : m;
        }
        tot = s;
        mxall = float(m);
        sc->done_blocks = 0;
    }
    return threadIdx.x == 0;
}

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

}  // namespace

void launch_project(Env& e, float dtS) {
    const Grid& g = e.g;
    const Tiles T = tiles_of(g);
    const int ref = e.cfg.semantics == 0;
    const int nblk = std::min(std::min(T.n, e.num_sms * 4), kMaxPartials);
    {
    ProfScope ps(e, "proj_setup");
    e.launches += 2;
    k_reset_vel<<<(g.XY + 127) / 128, 128, 0, e.stream>>>(g, e.u, e.v, e.w, e.defU, e.defW, ref);
    k_build<<<nblk, NT, 0, e.stream>>>(g, T, e.rho, e.u, e.v, e.w, e.defU, e.defW, dtS, e.ax, e.ay, e.az, e.aw, e.r, e.s, e.pp, e.As, ref,
                                      e.sc, e.partials);
    }
    const int chunk = 8;
    for (int it = 0; it < e.cfg.pcg_max_iter; it += chunk) {
        const int n = std::min(chunk, e.cfg.pcg_max_iter - it);
        for (int k = 0; k < n; ++k) {
            { ProfScope ps(e, "pcg_matvec"); e.launches += 1; k_matvec<<<nblk, NT, 0, e.stream>>>(g, T, e.ax, e.ay, e.az, e.aw, e.s, e.As, ref, e.sc, e.partials); }
            { ProfScope ps(e, "pcg_update"); e.launches += 1; k_update<<<nblk, NT, 0, e.stream>>>(g, T, e.aw, e.s, e.As, e.pp, e.r, ref, e.cfg.pcg_tol, e.cfg.pcg_max_iter, e.sc, e.partials); }
            { ProfScope ps(e, "pcg_search"); e.launches += 1; k_search<<<nblk, NT, 0, e.stream>>>(g, T, e.aw, e.r, e.s, e.sc); }
        }
        cudaMemcpyAsync(e.host_sc, e.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, e.stream);
        cudaStreamSynchronize(e.stream);
        if (e.host_sc->converged) break;
    }
    e.last_iters = e.host_sc->iters;
    e.last_residual = e.host_sc->residual;
    e.last_converged = e.host_sc->converged == 1;
    const dim3 grd((g.X + 31) / 32, (g.Y + 7) / 8, g.Z), blk(32, 8);
    ProfScope ps(e, "proj_apply");
    e.launches += 2;
    k_press_dens<<<grd, blk, 0, e.stream>>>(g, e.p, e.pp, e.rho, e.th, e.qv, e.Pg);
    k_apply_proj<<<grd, blk, 0, e.stream>>>(g, e.pp, e.rho, e.u, e.v, e.w);
}

}  // namespace skt
