// Stencil kernels of the atmosphere step: diffusion, PPM advection, Courant max, sedimentation,
// buoyancy and the equation of state.
#include "skt_internal.cuh"
#include "../../include/skewt.h"
#include <cuda.h>
#include <algorithm>
#include <mutex>
#include <string>
#include <type_traits>

namespace skt {

namespace {

constexpr int BX = 32, BY = 8;

inline dim3 cell_grid(const Grid& g) { return dim3((g.X + BX - 1) / BX, (g.Y + BY - 1) / BY, g.Z); }

// theta at a ground face seen from cell idx: potentialTempGPU(Tg-273.15, p_cell, Pg)+273.15
// (Game/kernelSky.cu:95-100)
__device__ __forceinline__ float theta_ground(const float* p, const float* Tg, const float* Pg, int idx, int idxg) {
    return potentialTemp(Tg[idxg] - 273.15f, p[idx], Pg[idxg]) + 273.15f;
}

// One cell of a Jacobi sweep, (c + k (l + r + u + d + f + b)) / (1 + 6k) with the division as a
// multiplication by rinv = 1 / (1 + 6k) (diffuseRedBlack Game/kernelSky.cu:110): the sum in this
// order and the fused multiply-add spelt out, so that every kernel that sweeps gives the same bits.
__device__ __forceinline__ float jacobi(float c, float l, float r, float u, float d, float f, float b, float k, float rinv) {
    const float s = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(l, r), u), d), f), b);
    return __fmul_rn(__fmaf_rn(k, s, c), rinv);
}

// One Jacobi sweep of the colour-split diffusion (diffuseRedBlack Game/kernelSky.cu:43-115; both
// colours read the same input array, Game/environment.cu:651-662).
template <bool THETA>
__global__ void __launch_bounds__(256) k_diffuse(Grid g, const float* __restrict__ in, float* __restrict__ out, int sides, int ground,
                                                 const float* __restrict__ def, float k, const float* __restrict__ p,
                                                 const float* __restrict__ Tg, const float* __restrict__ Pg) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    float l = ghost(g, in, x - 1, y, z, sides, ground, def);
    float r = ghost(g, in, x + 1, y, z, sides, ground, def);
    float d = ghost(g, in, x, y - 1, z, sides, ground, def);
    float u = ghost(g, in, x, y + 1, z, sides, ground, def);
    float f = ghost(g, in, x, y, z + 1, sides, ground, def);
    float b = ghost(g, in, x, y, z - 1, sides, ground, def);
    if (THETA) {
        const int idxG = x + z * g.X;
        if (y > 0 && is_ground(g, x, y - 1, z)) d = theta_ground(p, Tg, Pg, c, idxG);
        // lateral ground faces: only when isGroundLevel(z) holds for the reference's 16-wide tile
        // launch (Q5, Game/kernelSky.cu:1684-1694): blockIdx.x == GHeight[threadIdx.x + z*Z] + 1
        const bool gl = x > 0 && is_ground(g, x - 1, y, z), gr = x + 1 < g.X && is_ground(g, x + 1, y, z);
        const bool gf = z + 1 < g.Z && is_ground(g, x, y, z + 1), gb = z > 0 && is_ground(g, x, y, z - 1);
        if (gl | gr | gf | gb) {
            const int bw = min(16, g.X);
            int gi = (x % bw) + z * g.Z;
            if (gi >= g.X * g.Z) gi = g.X * g.Z - 1;
            const bool level = (x / bw) == g.gh[gi] + 1;
            if (level) {
                const int idxGL = x > 0 ? idxG - 1 : idxG, idxGR = x + 1 < g.X ? idxG + 1 : idxG;
                const int idxGF = z + g.X < g.Z ? idxG + g.X : idxG;  // the reference compares z + X < Z
                const int idxGB = z > 0 ? idxG - g.X : idxG;
                if (gl) l = theta_ground(p, Tg, Pg, c, idxGL);
                if (gr) r = theta_ground(p, Tg, Pg, c, idxGR);
                if (gf) f = theta_ground(p, Tg, Pg, c, idxGF);
                if (gb) b = theta_ground(p, Tg, Pg, c, idxGB);
            }
        }
    }
    out[c] = jacobi(in[c], l, r, u, d, f, b, k, 1.0f / (1 + 6 * k));
}

// Vectorised sweep for flat terrain (ground = the y = 0 layer) and X % 4 == 0: four cells per
// thread along x, a march along z holding the planes z-1, z, z+1 in registers, x neighbours from
// the neighbouring lanes. Same arithmetic and ghost values as k_diffuse.
constexpr int DVY = 16;  // rows per block: the rows above and below come mostly from L1
__device__ __forceinline__ float4 ld4f(const float* p, int c) { return *reinterpret_cast<const float4*>(p + c); }
__device__ __forceinline__ float side_val(int bc, float own, float d) { return bc == NEUMANN ? own : (bc == DIRICHLET ? 0.0f : d); }

// theta's ground-face values of the first sky row (theta_ground), once per diffusion call: they
// depend on p, Tg and Pg only, which the sweeps do not change
__global__ void __launch_bounds__(256) k_theta_face(Grid g, const float* __restrict__ p, const float* __restrict__ Tg,
                                                    const float* __restrict__ Pg, float* __restrict__ face) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.X * g.Z) return;
    face[col] = theta_ground(p, Tg, Pg, cidx(g, col % g.X, 1, col / g.X), col);
}

// face: theta's ground-face values per column (k_theta_face), read at the first sky row
template <bool THETA>
__global__ void __launch_bounds__(32 * DVY) k_diffuse4(Grid g, int zlen, const float* __restrict__ in, float* __restrict__ out, int sides,
                                                       int ground, const float* __restrict__ def, float k,
                                                       const float* __restrict__ face) {
    const int lane = threadIdx.x;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * DVY + threadIdx.y + 1;  // sky rows start at y = 1
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const bool act = x0 < g.X && y < g.Y;
    const int X = g.X, XY = g.XY;
    const int row = x0 + y * X;
    const float dy = act ? (def ? def[y] : 0.0f) : 0.0f;
    const float dy0 = def ? def[0] : 0.0f;
    const float rinv = 1.0f / (1 + 6 * k);
    float4 qb = make_float4(0, 0, 0, 0), qc = qb;
    if (act) {
        qc = ld4f(in, row + zs * XY);
        if (zs > 0) qb = ld4f(in, row + (zs - 1) * XY);
        else qb = make_float4(side_val(sides, qc.x, dy), side_val(sides, qc.y, dy), side_val(sides, qc.z, dy), side_val(sides, qc.w, dy));
    }
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        float4 qf = qb, qd = qb, qu = qb;
        if (act) {
            if (z + 1 < g.Z) qf = ld4f(in, c + XY);
            else qf = make_float4(side_val(sides, qc.x, dy), side_val(sides, qc.y, dy), side_val(sides, qc.z, dy), side_val(sides, qc.w, dy));
            if (y > 1) qd = ld4f(in, c - X);
            else {
                const float gv = ground == DIRICHLET ? 0.0f : dy0;
                qd = make_float4(gv, gv, gv, gv);
            }
            if (y + 1 < g.Y) qu = ld4f(in, c + X);
            else qu = make_float4(side_val(sides, qc.x, dy), side_val(sides, qc.y, dy), side_val(sides, qc.z, dy), side_val(sides, qc.w, dy));
        }
        float ql = __shfl_up_sync(0xffffffffu, qc.w, 1);
        float qr = __shfl_down_sync(0xffffffffu, qc.x, 1);
        if (act) {
            if (lane == 0) ql = x0 > 0 ? in[c - 1] : side_val(sides, qc.x, dy);
            if (lane == 31 || x0 + 4 >= X) qr = (x0 + 4 < X) ? in[c + 4] : side_val(sides, qc.w, dy);
            if (THETA && y == 1) qd = ld4f(face, x0 + z * X);  // theta's ground face (diffuseRedBlack :97)
            float4 o;
            o.x = jacobi(qc.x, ql, qc.y, qu.x, qd.x, qf.x, qb.x, k, rinv);
            o.y = jacobi(qc.y, qc.x, qc.z, qu.y, qd.y, qf.y, qb.y, k, rinv);
            o.z = jacobi(qc.z, qc.y, qc.w, qu.z, qd.z, qf.z, qb.z, k, rinv);
            o.w = jacobi(qc.w, qc.z, qr, qu.w, qd.w, qf.w, qb.w, k, rinv);
            *reinterpret_cast<float4*>(out + c) = o;
        }
        qb = qc;
        qc = qf;
    }
}

// Two Jacobi sweeps in one pass (temporal blocking of depth 2), flat terrain, X % 4 == 0.
//
// Tiles: a block of D2WARPS warps covers 28 x cells and D2WARPS*H rows and marches a run of z
// planes. The input planes stream through a ring of D2SLOTS shared-memory slots, each filled by one
// TMA copy (cp.async.bulk.tensor) of a 36 x (D2WARPS*H + 4) box: the tile with a halo of 2 cells on
// every side (4 on the left, so that the copy starts on a 16-byte boundary), issued D2SLOTS planes
// ahead by one thread and completed on an mbarrier. The copies in flight, not the registers, hide
// the memory latency. Each thread owns one x cell (lanes 2..29 write; lanes 0, 1, 30, 31 are the
// x halo of the intermediate sweep) and H rows: it keeps three planes of the input (rows y0-2 ..
// y0+H+1) and three planes of the intermediate sweep (rows y0-1 .. y0+H) in registers, recomputing
// the intermediate rows next to the neighbouring warps instead of exchanging them. Every cell of
// either sweep is computed with jacobi() from the same neighbour values as k_diffuse4, ghost values
// of each sweep included, so the pass equals two single sweeps bit for bit, while the field makes
// one trip through HBM per two sweeps instead of two.
constexpr int D2OUT = 28;   // cells a warp writes along x
constexpr int D2WARPS = 8;  // warps per block, stacked in y
constexpr int D2BW = D2OUT + 8;  // box width: 36 floats = 144 bytes
constexpr int D2SLOTS = 6;  // ring depth (planes in flight per block)
constexpr unsigned kMbarSpinLimit = 1u << 20;  // try_wait rounds before a wait is declared stuck

template <int H>
struct D2Rows {
    float v[H + 4];  // input rows y0-2 .. y0+H+1 (the intermediate sweep uses the first H+2)
};
template <int H>
constexpr int d2_box_rows() { return H * D2WARPS + 4; }
template <int H>
constexpr int d2_slot_bytes() { return ((D2BW * d2_box_rows<H>() * 4 + 127) / 128) * 128; }
template <int H>
constexpr int d2_smem_bytes() { return D2SLOTS * d2_slot_bytes<H>() + D2SLOTS * 8; }

__device__ __forceinline__ unsigned smem_u32(const void* p) { return unsigned(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// a bounded wait: false when the phase did not complete within kMbarSpinLimit rounds
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    for (unsigned i = 0; i < kMbarSpinLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <bool THETA, int H>
__global__ void __launch_bounds__(32 * D2WARPS) k_diffuse2(const __grid_constant__ CUtensorMap tin, Grid g, int zlen,
                                                          float* __restrict__ out, int sides, int ground, const float* __restrict__ def,
                                                          float k, const float* __restrict__ face, Scalars* __restrict__ sc) {
    extern __shared__ __align__(128) unsigned char d2_smem[];
    constexpr int BR = d2_box_rows<H>();
    constexpr int SLOT = d2_slot_bytes<H>();
    constexpr unsigned BOX_BYTES = D2BW * BR * 4;
    uint64_t* bar = reinterpret_cast<uint64_t*>(d2_smem + D2SLOTS * SLOT);
    const int lane = threadIdx.x, wy = threadIdx.y;
    const int tid = lane + 32 * wy;
    const int bx0 = int(blockIdx.x) * D2OUT - 4;  // box origin: a multiple of 4 cells (16 bytes)
    const int by0 = 1 + int(blockIdx.y) * H * D2WARPS - 2;
    const int x = bx0 + 2 + lane;
    const int y0 = 1 + (int(blockIdx.y) * D2WARPS + wy) * H;  // the warp's first written row
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const int X = g.X, Y = g.Y, Z = g.Z, XY = g.XY;
    const int zlo = max(zs - 2, 0), nplanes = min(ze + 1, Z - 1) - zlo + 1;
    const bool xin = x >= 0 && x < X;
    const int xc = min(max(x, 0), X - 1);
    const int srcl = lane - (x - xc);  // the lane holding the clamped (boundary) cell
    const bool xedge = blockIdx.x == 0 || bx0 + 2 + 31 >= X;  // block-uniform
    const bool top = y0 + H + 1 >= Y;                        // warp-uniform
    const float rinv = 1.0f / (1 + 6 * k);
    const float gv = ground == DIRICHLET ? 0.0f : (def ? def[0] : 0.0f);
    const float dtop = def ? def[Y - 1] : 0.0f;
    auto dval = [&](int y) { return def ? __ldg(def + y) : 0.0f; };
    // the value below the first sky row: the ground ghost, or theta's ground face of the plane
    auto down = [&](int z) { return THETA ? __ldg(face + xc + z * X) : gv; };

    if (tid == 0) {
        for (int s = 0; s < D2SLOTS; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int issued = 0;  // producer (thread 0): planes whose copy has been issued
    auto issue = [&](int q) {
        const int slot = q % D2SLOTS;
        mbar_expect_tx(&bar[slot], BOX_BYTES);
        tma_load_3d(d2_smem + slot * SLOT, &tin, &bar[slot], bx0, by0, zlo + q);
    };
    if (tid == 0) {
        for (; issued < min(D2SLOTS, nplanes); ++issued) issue(issued);
    }
    bool stuck = false;
    // Input plane z (planes are consumed in increasing order) into r: the slot's rows of this
    // thread, then the ghost rows and lanes. Rows <= 0 take the value below the first sky row,
    // rows >= Y the side ghost of row Y-1, lanes outside the grid the side ghost of the boundary lane.
    auto load_plane = [&](D2Rows<H>& r, int z) {
        const int q = z - zlo, slot = q % D2SLOTS;
        const bool ok = mbar_wait(&bar[slot], unsigned(q / D2SLOTS) & 1u);
        const float* sm = reinterpret_cast<const float*>(d2_smem + slot * SLOT) + wy * H * D2BW + lane + 2;
#pragma unroll
        for (int i = 0; i < H + 4; ++i) {
            const int y = y0 - 2 + i;
            r.v[i] = (ok && y >= 1 && y < Y && xin) ? sm[i * D2BW] : 0.0f;
        }
        // every thread has read the slot: it can be refilled (a stuck copy stops the whole block)
        if (__syncthreads_or(!ok)) {
            stuck = true;
            return;
        }
        if (tid == 0 && issued < nplanes) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(issued++);
        }
        if (y0 == 1) {
            const float dv = down(z);
            r.v[0] = dv;
            r.v[1] = dv;
        }
        if (top) {
            float t = 0.0f;  // row Y-1, picked with constant indices so that r stays in registers
#pragma unroll
            for (int i = 0; i < H + 4; ++i)
                if (y0 - 2 + i == Y - 1) t = r.v[i];
            const float gt = side_val(sides, t, dtop);
#pragma unroll
            for (int i = 0; i < H + 4; ++i)
                if (y0 - 2 + i >= Y) r.v[i] = gt;
        }
        if (xedge) {
#pragma unroll
            for (int i = 0; i < H + 4; ++i) {
                const float b = __shfl_sync(0xffffffffu, r.v[i], srcl);
                const int y = y0 - 2 + i;
                if (!xin && y >= 1 && y < Y) r.v[i] = side_val(sides, b, dval(y));
            }
        }
    };
    // the side ghost of a whole plane (z = -1 or z = Z) from the boundary plane b
    auto ghost_plane = [&](D2Rows<H>& r, const D2Rows<H>& b, int nrows, int ylo) {
#pragma unroll
        for (int i = 0; i < H + 4; ++i) {
            if (i >= nrows) break;
            const int y = ylo + i;
            r.v[i] = (y >= 1 && y < Y) ? side_val(sides, b.v[i], dval(y)) : b.v[i];
        }
    };
    // Intermediate sweep of plane z into m (rows y0-1 .. y0+H) from input planes a (z-1), b (z),
    // c (z+1); then its ghost rows and lanes.
    auto sweep1 = [&](D2Rows<H>& m, const D2Rows<H>& a, const D2Rows<H>& b, const D2Rows<H>& c, int z) {
#pragma unroll
        for (int j = 0; j < H + 2; ++j) {
            const float ctr = b.v[j + 1];
            const float l = __shfl_up_sync(0xffffffffu, ctr, 1), r = __shfl_down_sync(0xffffffffu, ctr, 1);
            m.v[j] = jacobi(ctr, l, r, b.v[j + 2], b.v[j], c.v[j + 1], a.v[j + 1], k, rinv);
        }
        if (y0 == 1) m.v[0] = down(z);  // row 0: ground, not swept
        if (top) {
            float t = 0.0f;
#pragma unroll
            for (int j = 0; j < H + 2; ++j)
                if (y0 - 1 + j == Y - 1) t = m.v[j];
            const float gt = side_val(sides, t, dtop);
#pragma unroll
            for (int j = 0; j < H + 2; ++j)
                if (y0 - 1 + j >= Y) m.v[j] = gt;
        }
        if (xedge) {
#pragma unroll
            for (int j = 0; j < H + 2; ++j) {
                const float bnd = __shfl_sync(0xffffffffu, m.v[j], srcl);
                const int y = y0 - 1 + j;
                if (!xin && y >= 1 && y < Y) m.v[j] = side_val(sides, bnd, dval(y));
            }
        }
    };
    // Second sweep of plane z from intermediate planes a (z-1), b (z), c (z+1): rows y0 .. y0+H-1.
    auto sweep2 = [&](const D2Rows<H>& a, const D2Rows<H>& b, const D2Rows<H>& c, int z) {
        const bool wr = xin && lane >= 2 && lane < 2 + D2OUT;
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float ctr = b.v[j + 1];
            const float l = __shfl_up_sync(0xffffffffu, ctr, 1), r = __shfl_down_sync(0xffffffffu, ctr, 1);
            const float o = jacobi(ctr, l, r, b.v[j + 2], b.v[j], c.v[j + 1], a.v[j + 1], k, rinv);
            const int y = y0 + j;
            if (wr && y < Y) out[x + y * X + z * XY] = o;
        }
    };

    // set-up, consuming the input planes in increasing order: zs-2, zs-1, zs, zs+1
    D2Rows<H> pm, p0, p1, p2, q0, q1, q2;
    if (zs >= 2) load_plane(pm, zs - 2);
    if (!stuck && zs >= 1) load_plane(p0, zs - 1);
    if (!stuck) load_plane(p1, zs);
    if (!stuck && zs + 1 < Z) load_plane(p2, zs + 1);
    if (!stuck) {
        if (zs < 1) ghost_plane(p0, p1, H + 4, y0 - 2);
        if (zs + 1 >= Z) ghost_plane(p2, p1, H + 4, y0 - 2);
        if (zs == 1) ghost_plane(pm, p0, H + 4, y0 - 2);
        sweep1(q1, p0, p1, p2, zs);
        if (zs >= 1) sweep1(q0, pm, p0, p1, zs - 1);
        else ghost_plane(q0, q1, H + 2, y0 - 1);
    }
    // one march step for plane z: input plane z+2 into F and intermediate plane z+1 into QF, then
    // the output plane z; the roles rotate through the three register sets (the loop is unrolled
    // three times so that no values are copied)
    auto step = [&](D2Rows<H>& A, D2Rows<H>& B, D2Rows<H>& F, D2Rows<H>& QA, D2Rows<H>& QB, D2Rows<H>& QF, int z) {
        if (z + 1 < Z) {
            if (z + 2 < Z) load_plane(F, z + 2); else ghost_plane(F, B, H + 4, y0 - 2);
            if (stuck) return;
            sweep1(QF, A, B, F, z + 1);
        } else {
            ghost_plane(QF, QB, H + 2, y0 - 1);
        }
        sweep2(QA, QB, QF, z);
    };
    int z = zs;
    for (; !stuck && z + 2 < ze; z += 3) {
        step(p1, p2, p0, q0, q1, q2, z);
        if (stuck) break;
        step(p2, p0, p1, q1, q2, q0, z + 1);
        if (stuck) break;
        step(p0, p1, p2, q2, q0, q1, z + 2);
    }
    if (!stuck && z < ze) {
        step(p1, p2, p0, q0, q1, q2, z);
        if (!stuck && z + 1 < ze) step(p2, p0, p1, q1, q2, q0, z + 1);
    }
    if (stuck && tid == 0) {
        // record the timeout, then let the copies already issued land before the block's shared
        // memory goes away (each wait again bounded)
        sc->status = SKT_TIMEOUT;
        for (int q = max(issued - D2SLOTS, 0); q < issued; ++q) (void)mbar_wait(&bar[q % D2SLOTS], unsigned(q / D2SLOTS) & 1u);
    }
}

// Two Jacobi sweeps in one pass with four cells per lane (temporal blocking of depth 2), flat
// terrain, X % 4 == 0.
//
// A block covers 128 x cells (one warp of float4 lanes) by R output rows and marches a run of z
// planes. Its R + 2 row warps compute the first sweep on rows yb-1 .. yb+R and the inner R of them
// the second sweep on rows yb .. yb+R-1; one more warp computes the first sweep's cells just left
// and right of the block (x = bx-1 and bx+128, one lane per row and side), the only cells outside
// the row warps' lanes that the second sweep reads. The input planes stream through a ring of
// P4SLOTS shared-memory slots, each filled by one TMA copy of a 136 x (R+4) box: the block's cells
// with 4 more on either side (the copy starts on a 16-byte boundary) and 2 rows above and below.
// A lane keeps its own row of two input planes and two first-sweep planes in registers and reads
// its neighbours (the rows above and below, the cells left and right) from the slot or from two
// shared planes of the first sweep. Per plane p the block passes one barrier: each warp stores its
// first-sweep row of plane p, then computes the second sweep of plane p-1 from the shared plane
// p-1 (complete since the previous barrier); after the barrier the slot of input plane p-1 is
// refilled. Every cell of either sweep is computed with jacobi() from the same neighbour and ghost
// values as k_diffuse4, so the pass equals two single sweeps bit for bit.
constexpr int P4W = 136;    // box width in cells: 4 + 128 + 4 (544 bytes)
constexpr int P4SLOTS = 8;  // ring depth: planes p-1, p, p+1 in use and five in flight
template <int R>
constexpr int p4_slot_bytes() { return ((P4W * (R + 4) * 4 + 127) / 128) * 128; }
template <int R>
constexpr int p4_mid_bytes() { return 2 * P4W * (R + 2) * 4; }
template <int R>
constexpr int p4_smem_bytes() { return P4SLOTS * p4_slot_bytes<R>() + p4_mid_bytes<R>() + P4SLOTS * 8; }
template <int R>
constexpr int p4_min_blocks() { return R >= 14 ? 2 : 4; }  // blocks per SM the registers are budgeted for

__device__ __forceinline__ float4 ld4s(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 zero4() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
__device__ __forceinline__ float4 side4(int bc, float4 c, float d) {
    return make_float4(side_val(bc, c.x, d), side_val(bc, c.y, d), side_val(bc, c.z, d), side_val(bc, c.w, d));
}
// four consecutive cells of a sweep: l and r the x neighbours of the first and the last cell
__device__ __forceinline__ float4 jacobi4(float4 c, float l, float r, float4 u, float4 d, float4 f, float4 b, float k, float rinv) {
    return make_float4(jacobi(c.x, l, c.y, u.x, d.x, f.x, b.x, k, rinv), jacobi(c.y, c.x, c.z, u.y, d.y, f.y, b.y, k, rinv),
                       jacobi(c.z, c.y, c.w, u.z, d.z, f.z, b.z, k, rinv), jacobi(c.w, c.z, r, u.w, d.w, f.w, b.w, k, rinv));
}

template <bool THETA, int R>
__global__ void __launch_bounds__(32 * (R + 3), p4_min_blocks<R>())
    k_diffuse_pair4(const __grid_constant__ CUtensorMap tin, Grid g, int zlen, float* __restrict__ out, int sides, int ground,
                    const float* __restrict__ def, float k, const float* __restrict__ face, Scalars* __restrict__ sc) {
    extern __shared__ __align__(128) unsigned char p4_smem[];
    constexpr int NR = R + 2;
    constexpr int SLOTF = p4_slot_bytes<R>() / 4;  // floats per slot
    constexpr unsigned BOX_BYTES = P4W * (R + 4) * 4;
    float* const ring = reinterpret_cast<float*>(p4_smem);
    float* const mid = ring + P4SLOTS * SLOTF;  // [plane & 1][NR rows][P4W]: the first sweep
    uint64_t* const bar = reinterpret_cast<uint64_t*>(mid + 2 * NR * P4W);
    const int tid = threadIdx.x, lane = tid & 31, wy = tid >> 5;  // a 1D block: the warp index is warp-uniform
    const int X = g.X, Y = g.Y, Z = g.Z, XY = g.XY;
    const int bx = int(blockIdx.x) * 128, yb = 1 + int(blockIdx.y) * R;
    const int zs = int(blockIdx.z) * zlen, ze = min(zs + zlen, Z);
    const int plo = max(zs - 1, 0), phi = min(ze, Z - 1);       // planes of the first sweep
    const int ilo = max(plo - 1, 0), ihi = min(phi + 1, Z - 1);  // input planes
    const float rinv = 1.0f / (1 + 6 * k);
    const float gv = ground == DIRICHLET ? 0.0f : (def ? def[0] : 0.0f);
    const float4 gv4 = make_float4(gv, gv, gv, gv);
    // row warps: row y, cells x0 .. x0+3 at column col of a slot row and of a shared plane row
    const bool edge = wy == NR;
    const int y = yb - 1 + wy, x0 = bx + 4 * lane, col = 4 + 4 * lane;
    const bool act = !edge && y >= 1 && y < Y;  // first sweep (warp-uniform; lanes past X compute unused values)
    const bool wr = act && wy >= 1 && wy <= R;   // second sweep (written out for x0 < X)
    const bool xin = x0 < X;
    const bool yin = y > 1 && y + 1 < Y;                   // no ghost row above or below (warp-uniform)
    const int own = (wy + 1) * P4W + col, mown = wy * P4W + col;
    const bool lfix = x0 == 0, rfix = x0 + 4 >= X;  // the x ghosts of the first and last cell
    // edge warp: lane 2 er + es holds row yb-1+er at x = bx-1 (es = 0) or bx+128 (es = 1)
    const int er = lane >> 1, es = lane & 1;
    const int ey = yb - 1 + er, ex = es ? bx + 128 : bx - 1, eown = (er + 1) * P4W + (es ? 132 : 3);
    const bool eact = edge && er < NR && ey >= 1 && ey < Y && ex >= 0 && ex < X;
    const int ry = edge ? ey : y;
    const float dy = (def && ry >= 0 && ry < Y) ? def[ry] : 0.0f;

    auto issue = [&](int q) {
        const int s = (q - ilo) % P4SLOTS;
        mbar_expect_tx(&bar[s], BOX_BYTES);
        tma_load_3d(ring + s * SLOTF, &tin, &bar[s], bx - 4, yb - 2, q);
    };
    if (tid == 0) {
        for (int s = 0; s < P4SLOTS; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int issued = ilo;  // thread 0: the next input plane to copy
    if (tid == 0)
        for (; issued <= min(ihi, ilo + P4SLOTS - 1); ++issued) issue(issued);
    // the input planes complete in order; wslot / wpar: slot and phase parity of the next one
    int waited = ilo, wslot = 0;
    unsigned wpar = 0;
    bool ok = true;
    auto wait_next = [&]() {  // waits for input plane `waited`
        if (!mbar_try_wait(&bar[wslot], wpar)) ok = mbar_wait(&bar[wslot], wpar) && ok;
        ++waited;
        if (++wslot == P4SLOTS) {
            wslot = 0;
            wpar ^= 1u;
        }
    };
    auto nxt = [](int s) { return s + 1 == P4SLOTS ? 0 : s + 1; };
    // x neighbours of a lane's four cells c from the shared row (at the warp's ends the edge warp's
    // cells), at the grid's ends the ghost. (Warp shuffles for the inner lanes measured slower: the
    // end lanes' loads become divergent branches.)
    auto xnb = [&](const float4& c, const float* row, float& l, float& r) {
        l = lfix ? side_val(sides, c.x, dy) : row[-1];
        r = rfix ? side_val(sides, c.w, dy) : row[4];
    };
    // first sweep of plane p for a row warp: ib, ic the input planes p-1, p; s0, s1 the slots of p,
    // p+1; f gets the input plane p+1; dg: the value below row 1 (theta's ground face of the plane,
    // else the ground ghost)
    auto sweep1 = [&](bool gen, int p, const float4& ib, const float4& ic, int s0, int s1, float4& f, const float4& dg) {
        const float* row = ring + s0 * SLOTF + own;
        f = ld4s(ring + s1 * SLOTF + own);
        float4 d = ld4s(row - P4W), u = ld4s(row + P4W);
        if (gen) {  // a ghost row or plane: rows 1 and Y-1, the last plane (warp-uniform)
            if (p + 1 >= Z) f = side4(sides, ic, dy);
            if (y == 1) d = dg;
            if (y + 1 >= Y) u = side4(sides, ic, dy);
        }
        float l, r;
        xnb(ic, row, l, r);
        return jacobi4(ic, l, r, u, d, f, ib, k, rinv);
    };
    // second sweep of plane zo from the first sweep's planes mb (zo-1), mc (zo), mf (zo+1)
    auto sweep2 = [&](bool gen, int zo, const float4& mb, const float4& mc, const float4& mf, bool store, const float4& dg) {
        const float* m2 = mid + (zo & 1) * (NR * P4W) + mown;
        float4 d = ld4s(m2 - P4W), u = ld4s(m2 + P4W);
        if (gen) {
            if (y == 1) d = dg;
            if (y + 1 >= Y) u = side4(sides, mc, dy);
        }
        float l, r;
        xnb(mc, m2, l, r);
        const float4 o = jacobi4(mc, l, r, u, d, mf, mb, k, rinv);
        if (xin && store) *reinterpret_cast<float4*>(out + x0 + y * X + zo * XY) = o;
    };

    // Every warp runs the plane steps p = plo .. phi with one barrier each; the row warps that
    // sweep and the other warps (the edge warp, rows outside the grid) run separate loops, so that
    // neither tests its role per step.
    auto refill = [&](int p) {  // thread 0, after the barrier of step p: slot p-1 takes plane p-1+P4SLOTS
        if (tid == 0 && p - 1 >= ilo && issued <= ihi) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(issued++);
        }
    };
    int s0 = (plo - ilo) % P4SLOTS;  // the slot of plane p
    bool stuck = false;
    wait_next();  // plane ilo
    if (plo > ilo) wait_next();
    // one plane step of a row warp: the first sweep of plane p, the second of plane p-1, the
    // barrier and the refill; false when a copy got stuck. G1 / G2: the first / second sweep may
    // meet a ghost row or plane (rows 1 and Y-1, the grid's last plane); WR: the warp writes the
    // second sweep; GEN: the grid's first or last plane (tests everything at run time).
    float4 ib = zero4(), ic = zero4(), mb = zero4(), mc = zero4();  // input planes p-1, p; first sweep p-2, p-1
    // row 1 of theta: the ground face of plane p (gc), loaded a step ahead; only the rows next to a
    // ghost row (G1) carry it
    const bool face_row = THETA && y == 1 && xin;
    auto face_at = [&](int z) { return face_row ? ld4f(face, x0 + z * X) : gv4; };
    auto row_step = [&](auto g1_c, auto g2_c, auto wr_c, auto gen_c, int p, float4& gc) {
        constexpr bool G1 = decltype(g1_c)::value, G2 = decltype(g2_c)::value, WR = decltype(wr_c)::value;
        constexpr bool GEN = decltype(gen_c)::value;
        if (!GEN || p + 1 <= ihi) wait_next();  // plane p+1
        const int s1 = nxt(s0);
        float4 f;
        const float4 g1 = gc;
        if (G1) gc = p + 1 < Z ? face_at(p + 1) : gv4;  // the next plane's face, loaded a step ahead
        const float4 mf = sweep1(G1, p, ib, ic, s0, s1, f, g1);
        *reinterpret_cast<float4*>(mid + (p & 1) * (NR * P4W) + mown) = mf;
        ib = ic;
        ic = f;
        // written from the run's first plane on; the face of plane p-1 was read a step ago (L1)
        if (WR) sweep2(G2, p - 1, mb, mc, mf, p - 1 >= zs, (G2 && p >= 1) ? face_at(p - 1) : gv4);
        mb = (GEN && p == 0) ? side4(sides, mf, dy) : mc;     // plane 0: the first sweep's ghost plane z = -1
        mc = mf;
        // the first sweep of plane p is complete and slot p-1 is read (a stuck copy stops the block)
        if (__syncthreads_or(!ok)) return false;
        refill(p);
        s0 = s1;
        return true;
    };
    auto rows = [&](auto ye_c, auto wr_c) {  // YE: the row has a ghost row above or below
        constexpr bool YE = decltype(ye_c)::value;
        using T = std::true_type;
        using F = std::false_type;
        ic = ld4s(ring + s0 * SLOTF + own);
        ib = plo >= 1 ? ld4s(ring + (plo - 1 - ilo) * SLOTF + own) : side4(sides, ic, dy);
        float4 gc = gv4;  // the face of plane p (rows next to a ghost row)
        if (YE) gc = face_at(plo);
        int p = plo;
        if (p == 0 && p <= phi && !row_step(T{}, T{}, wr_c, T{}, p++, gc)) return false;
        const int pend = phi == Z - 1 ? phi - 1 : phi;  // the grid's last plane runs the general step
        for (; p <= pend; ++p)
            if (!row_step(std::integral_constant<bool, YE>{}, std::integral_constant<bool, YE>{}, wr_c, F{}, p, gc)) return false;
        for (; p <= phi; ++p)
            if (!row_step(T{}, T{}, wr_c, T{}, p, gc)) return false;
        if (ze == Z && decltype(wr_c)::value) sweep2(true, Z - 1, mb, mc, side4(sides, mc, dy), Z - 1 >= zs, face_at(Z - 1));  // z+1 of Z-1: the ghost
        return true;
    };
    if (act) {
        using T = std::true_type;
        using F = std::false_type;
        bool fine;
        if (yin) fine = wr ? rows(F{}, T{}) : rows(F{}, F{});
        else fine = wr ? rows(T{}, T{}) : rows(T{}, F{});
        stuck = !fine;
    } else {
        for (int p = plo; p <= phi; ++p) {
            if (p + 1 <= ihi) wait_next();
            const int s1 = nxt(s0);
            if (eact) {  // the left cell's left neighbour is inside the grid (bx >= 128), as is the right cell's
                const float* row = ring + s0 * SLOTF + eown;
                const float c = row[0];
                const float r = ex + 1 < X ? row[1] : side_val(sides, c, dy);
                const float d = ey > 1 ? row[-P4W] : (THETA ? __ldg(face + ex + p * X) : gv);
                const float u = ey + 1 < Y ? row[P4W] : side_val(sides, c, dy);
                const float f = p + 1 < Z ? ring[s1 * SLOTF + eown] : side_val(sides, c, dy);
                const float b = p >= 1 ? ring[(s0 == 0 ? P4SLOTS - 1 : s0 - 1) * SLOTF + eown] : side_val(sides, c, dy);
                mid[(p & 1) * (NR * P4W) + er * P4W + (es ? 132 : 3)] = jacobi(c, row[-1], r, u, d, f, b, k, rinv);
            }
            if (__syncthreads_or(!ok)) {
                stuck = true;
                break;
            }
            refill(p);
            s0 = s1;
        }
    }
    if (stuck && tid == 0) {
        // record the timeout, then let the copies still in flight land before the block's shared
        // memory goes away (each wait again bounded)
        sc->status = SKT_TIMEOUT;
        for (int q = max(issued - P4SLOTS, ilo); q < issued; ++q) {
            const int rel = q - ilo;
            (void)mbar_wait(&bar[rel % P4SLOTS], unsigned(rel / P4SLOTS) & 1u);
        }
    }
}

// advectPPMFlux, Game/kernelSky.cu:270-366 (van Leer slope, Walcek limiter, Courant clamp),
// written without branches: the limiter ratios are formed unconditionally and selected, the
// parabola's sign case by a select. cdt = dt/vox: the Courant number is veli*cdt (the reference
// divides veli*dt by vox each call) and the limiter ratios use the fast divide; both change
// results by a few ulp at most.
__device__ __forceinline__ float ppm_flux(float veli, float vL, float vC, float vR, float cdt) {
    const float C = fminf(fmaxf(veli * cdt, -1.0f), 1.0f);
    const float qMin = fminf(vL, fminf(vC, vR));
    const float qMax = fmaxf(vL, fmaxf(vC, vR));
    const float dl = vC - vL, dr = vR - vC, db = vR - vL;
    const float lim = fminf(0.5f * fabsf(db), fminf(fabsf(dr), fabsf(dl)));
    const float s = dl * dr > 0.0f ? (db >= 0.0f ? lim : -lim) : 0.0f;
    const float qLS = vC - 0.5f * s, qRS = vC + 0.5f * s;
    const float denR = qRS - vC, denL = vC - qLS;
    const float bR = (qRS > qMax && denR > 1e-16f) ? __fdividef(qMax - vC, denR) : 1.0f;
    const float bL = (qLS < qMin && denL > 1e-16f) ? __fdividef(vC - qMin, denL) : 1.0f;
    const float B = fminf(1.0f, fminf(bR, bL));
    float qR = vC + B * (qRS - vC);
    float qL = vC + B * (qLS - vC);
    const bool flat = (qR - vC) * (vC - qL) <= 0.0f;
    qR = flat ? vC : qR;
    qL = flat ? vC : qL;
    const float lin = C > 0.0f ? (-qL - 2 * qR + 3 * vC) : (-2 * qL - qR + 3 * vC);
    const float qq = qR + C * lin + C * C * (qL + qR - 2 * vC);
    return veli * qq;
}

// The flux through the face between cells b (below) and c (above) with face velocity u, a below b
// and d above c: the reconstruction is taken on the upwind side (a, b, c for u >= 0, else d, c, b).
// A cell's upper-face flux (its velocity, window q-1..q+2) and the next cell's lower-face flux
// (the previous cell's velocity, window q-2..q+1 seen from it) are the same call, so each face is
// computed once and handed on. For a window of ones the flux is exactly u.
__device__ __forceinline__ float face_flux(float u, float a, float b, float c, float d, float cdt) {
    const bool up = u >= 0.0f;
    return ppm_flux(u, up ? a : d, up ? b : c, up ? c : b, cdt);
}

// the advected value over the advected density companion (divideValues Game/kernelMaths.cu:38)
__device__ __forceinline__ float ppm_update(float q, float fp, float fm, float fpo, float fmo, float cdt) {
    const float nq = q - cdt * (fp - fm);
    const float nr = 1.0f - cdt * (fpo - fmo);
    return nq / nr;
}

// ghost value of the density companion (a field of ones, custom value 1)
__device__ __forceinline__ float ghost_one(const Grid& g, int x, int y, int z, int sides, int ground) {
    if (!in_dom(g, x, y, z)) {
        const int xc = min(max(x, 0), g.X - 1), yc = min(max(y, 0), g.Y - 1), zc = min(max(z, 0), g.Z - 1);
        return bc_val(is_ground(g, xc, yc, zc) ? ground : sides, 1.0f, 1.0f);
    }
    if (is_ground(g, x, y, z)) return bc_val(ground, 1.0f, 1.0f);
    return 1.0f;
}

// One directional PPM pass (advectPPMX/Y/Z Game/kernelSky.cu:368-574) of q and of the density
// companion (advected ones), followed by q/rho* (divideValues Game/kernelMaths.cu:38).
// The velocity array is read as it stands when the pass starts.
template <int AXIS>
__global__ void __launch_bounds__(256) k_ppm(Grid g, const float* __restrict__ in, float* __restrict__ out, const float* __restrict__ vel,
                                             const float* __restrict__ def, int sides, int ground, const float* __restrict__ defU,
                                             const float* __restrict__ defW, float dtFull, int nsub_host, int half,
                                             const Scalars* __restrict__ sc, int slot) {
    int nsub = nsub_host;
    if (sc) {
        nsub = sc->nsub;
        if (slot >= nsub) return;
    }
    const float dtSub = dtFull / float(nsub);
    const float dt = half ? dtSub * 0.5f : dtSub;
    const float cdt = dt / g.vox;
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    constexpr int ax = AXIS == 0, ay = AXIS == 1, az = AXIS == 2;
    const int c = cidx(g, x, y, z);
    float q[5], o[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const int off = i - 2;
        if (off == 0) { q[i] = in[c]; o[i] = 1.0f; continue; }
        q[i] = ghost(g, in, x + off * ax, y + off * ay, z + off * az, sides, ground, def);
        o[i] = ghost_one(g, x + off * ax, y + off * ay, z + off * az, sides, ground);
    }
    const float custom = AXIS == 0 ? defU[y] : (AXIS == 1 ? 0.0f : defW[y]);
    const float vc = vel[c];
    const float vm = face_nb(g, vel, x, y, z, -ax, -ay, -az, sides, ground, custom);
    const float fp = face_flux(vc, q[1], q[2], q[3], q[4], cdt), fm = face_flux(vm, q[0], q[1], q[2], q[3], cdt);
    const float fpo = face_flux(vc, o[1], o[2], o[3], o[4], cdt), fmo = face_flux(vm, o[0], o[1], o[2], o[3], cdt);
    out[c] = ppm_update(q[2], fp, fm, fpo, fmo, cdt);
}

__device__ __forceinline__ float comp(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }
__device__ __forceinline__ void setc(float4& v, int k, float a) {
    if (k == 0) v.x = a; else if (k == 1) v.y = a; else if (k == 2) v.z = a; else v.w = a;
}

__device__ __forceinline__ float ppm_cdt(const Grid& g, float dtFull, int nsub, int half) {
    const float dtSub = dtFull / float(nsub);
    const float dt = half ? dtSub * 0.5f : dtSub;
    return dt / g.vox;
}

// Vectorised X pass (flat terrain, X % 4 == 0): a thread owns four cells of one row and marches
// z. Its four upper-face fluxes use the x window q(x0-1) .. q(x0+5); the lower face of its first
// cell is the upper face of the lane before it (a shuffle). For lane 0 that face lies in the
// previous warp's cells: its flux (and q(x0-1)) is computed for 32 planes at once, one plane per
// lane, and handed to lane 0 plane by plane, so the warp does not spend a whole flux evaluation
// per plane on one lane.
__global__ void __launch_bounds__(32 * DVY, 32 / DVY) k_ppm4x(Grid g, int zlen, const float* __restrict__ in, float* __restrict__ out,
                                                    const float* __restrict__ vel, const float* __restrict__ def, int sides,
                                                    const float* __restrict__ defU, float dtFull, int nsub_host, int half,
                                                    const Scalars* __restrict__ sc, int slot) {
    int nsub = nsub_host;
    if (sc) {
        nsub = sc->nsub;
        if (slot >= nsub) return;
    }
    const float cdt = ppm_cdt(g, dtFull, nsub, half);
    const int lane = threadIdx.x;
    const int xw = blockIdx.x * 128;  // the warp's first cell
    const int x0 = xw + lane * 4;
    const int y = blockIdx.y * DVY + threadIdx.y + 1;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    const bool wact = xw < g.X && y < g.Y;  // same for every lane of the warp
    const bool act = x0 < g.X && y < g.Y;
    const int X = g.X, XY = g.XY;
    const int row = x0 + y * X, roww = xw + y * X;
    const float dy = wact ? (def ? def[y] : 0.0f) : 0.0f;
    const float du = wact ? defU[y] : 0.0f;
    const float so = bc_val(sides, 1.0f, 1.0f);
    const bool xedge0 = xw < 4 || xw + 8 > X;
    auto ow0 = [&](int j) { return (xw - 2 + j >= 0 && xw - 2 + j < X) ? 1.0f : so; };
    // The density companion's window reaches outside the domain only for the cells x0 = 0 (lane 0
    // of the first warp of a row) and x0 = X - 4 (one lane of the last warp); elsewhere its flux
    // is the face velocity. Those lanes' four companion fluxes are formed in the 32-plane batch,
    // one plane per lane, and handed to the edge lane plane by plane (warp-uniform branches).
    const int xr = X - 4, lr = (xr - xw) >> 2;
    const bool has_l = wact && xw == 0, has_r = wact && xr >= xw && xr < xw + 128;
    auto owx = [&](int xe, int j) { return (xe - 2 + j >= 0 && xe - 2 + j < X) ? 1.0f : so; };
    for (int zb = zs; zb < ze; zb += 32) {
        // the warp's lower boundary face for planes zb .. zb+31: plane zb + lane on this lane
        float Bq = 0.0f, BF = 0.0f, BFo = 0.0f;
        if (wact && zb + lane < ze) {
            const int cw = roww + (zb + lane) * XY;
            const float a2 = in[cw], a3 = in[cw + 1];
            float a0, um;
            if (xw >= 4) { a0 = in[cw - 2]; Bq = in[cw - 1]; um = vel[cw - 1]; }
            else { a0 = Bq = bc_val(sides, a2, dy); um = bc_val(sides, vel[cw], du); }
            BF = face_flux(um, a0, Bq, a2, a3, cdt);
            BFo = xedge0 ? face_flux(um, ow0(0), ow0(1), ow0(2), ow0(3), cdt) : um;
        }
        float4 EL = make_float4(0, 0, 0, 0), ER = EL;  // the edge lanes' companion fluxes, plane zb + lane
        if ((has_l || has_r) && zb + lane < ze) {
            const int pz = y * X + (zb + lane) * XY;
            if (has_l) {
                const float4 ue = ld4f(vel, pz);
#pragma unroll
                for (int k = 0; k < 4; ++k) setc(EL, k, face_flux(comp(ue, k), owx(0, k + 1), owx(0, k + 2), owx(0, k + 3), owx(0, k + 4), cdt));
            }
            if (has_r) {
                const float4 ue = ld4f(vel, pz + xr);
#pragma unroll
                for (int k = 0; k < 4; ++k) setc(ER, k, face_flux(comp(ue, k), owx(xr, k + 1), owx(xr, k + 2), owx(xr, k + 3), owx(xr, k + 4), cdt));
            }
        }
        const int zend = min(zb + 32, ze);
        for (int z = zb; z < zend; ++z) {
            const int c = row + z * XY;
            float4 qc = make_float4(0, 0, 0, 0), uc = qc;
            if (act) { qc = ld4f(in, c); uc = ld4f(vel, c); }
            const int src = z - zb;
            const float bq = __shfl_sync(0xffffffffu, Bq, src);
            const float bf = __shfl_sync(0xffffffffu, BF, src);
            const float bfo = __shfl_sync(0xffffffffu, BFo, src);
            float qm1 = __shfl_up_sync(0xffffffffu, qc.w, 1);
            float qp4 = __shfl_down_sync(0xffffffffu, qc.x, 1), qp5 = __shfl_down_sync(0xffffffffu, qc.y, 1);
            if (lane == 0) qm1 = bq;
            if (act && (lane == 31 || x0 + 4 >= X)) {
                if (x0 + 4 < X) { qp4 = in[c + 4]; qp5 = in[c + 5]; }
                else { qp4 = qp5 = bc_val(sides, qc.w, dy); }
            }
            const float w[7] = {qm1, qc.x, qc.y, qc.z, qc.w, qp4, qp5};
            const float u[4] = {uc.x, uc.y, uc.z, uc.w};
            float F[4], Fo[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                F[k] = face_flux(u[k], w[k], w[k + 1], w[k + 2], w[k + 3], cdt);
                Fo[k] = u[k];
            }
            if (has_l) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float v = __shfl_sync(0xffffffffu, comp(EL, k), src);
                    if (lane == 0) Fo[k] = v;
                }
            }
            if (has_r) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float v = __shfl_sync(0xffffffffu, comp(ER, k), src);
                    if (lane == lr) Fo[k] = v;
                }
            }
            float Fm = __shfl_up_sync(0xffffffffu, F[3], 1);
            float Fmo = __shfl_up_sync(0xffffffffu, Fo[3], 1);
            if (lane == 0) { Fm = bf; Fmo = bfo; }
            if (act) {
                float4 o4;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float fm = k == 0 ? Fm : F[k - 1], fmo = k == 0 ? Fmo : Fo[k - 1];
                    setc(o4, k, ppm_update(w[k + 1], F[k], fm, Fo[k], fmo, cdt));
                }
                *reinterpret_cast<float4*>(out + c) = o4;
            }
        }
    }
}

// Vectorised Y pass: a thread owns four cells of one (x, z) column and marches a run of rows,
// keeping the window q(y-2) .. q(y+2) in registers and handing each upper-face flux on as the next
// row's lower-face flux. Rows <= 0 are the ground ghost, rows >= Y the side ghost of the top row.
constexpr int PY = 4;
__global__ void __launch_bounds__(32 * PY) k_ppm4y(Grid g, int ylen, const float* __restrict__ in, float* __restrict__ out,
                                                   const float* __restrict__ vel, const float* __restrict__ def, int sides, int ground,
                                                   float dtFull, int nsub_host, int half, const Scalars* __restrict__ sc, int slot) {
    int nsub = nsub_host;
    if (sc) {
        nsub = sc->nsub;
        if (slot >= nsub) return;
    }
    const float cdt = ppm_cdt(g, dtFull, nsub, half);
    const int lane = threadIdx.x;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int z = blockIdx.y * PY + threadIdx.y;
    const int ys = 1 + blockIdx.z * ylen, ye = min(ys + ylen, g.Y);
    if (x0 >= g.X || z >= g.Z || ys >= g.Y) return;
    const int X = g.X, Y = g.Y;
    const int base = x0 + z * g.XY;
    const float dyt = def ? def[Y - 1] : 0.0f;
    const float gq = bc_val(ground, 0.0f, def ? def[0] : 0.0f);
    const float go = bc_val(ground, 1.0f, 1.0f), so = bc_val(sides, 1.0f, 1.0f);
    auto qrow = [&](int r) -> float4 {
        if (r <= 0) return make_float4(gq, gq, gq, gq);
        if (r < Y) return ld4f(in, base + r * X);
        const float4 t = ld4f(in, base + (Y - 1) * X);
        return make_float4(bc_val(sides, t.x, dyt), bc_val(sides, t.y, dyt), bc_val(sides, t.z, dyt), bc_val(sides, t.w, dyt));
    };
    auto orow = [&](int r) { return r <= 0 ? go : (r < Y ? 1.0f : so); };
    float4 w0 = qrow(ys - 2), w1 = qrow(ys - 1), w2 = qrow(ys), w3 = qrow(ys + 1);
    float4 Fc, Fco;  // lower-face fluxes of the current row
    {
        const float4 vm = ys >= 2 ? ld4f(vel, base + (ys - 1) * X) : make_float4(0, 0, 0, 0);  // face below y = 1 is ground: 0
        const bool oin = ys >= 3 && ys + 1 < Y;
#pragma unroll
        for (int k = 0; k < 4; ++k) setc(Fc, k, face_flux(comp(vm, k), comp(w0, k), comp(w1, k), comp(w2, k), comp(w3, k), cdt));
        Fco = vm;  // the companion's flux is the face velocity where its window is all ones
        if (!oin) {  // warp-uniform: a branch, not a select, so the interior skips the evaluation
#pragma unroll
            for (int k = 0; k < 4; ++k) setc(Fco, k, face_flux(comp(vm, k), orow(ys - 2), orow(ys - 1), orow(ys), orow(ys + 1), cdt));
        }
    }
    for (int y = ys; y < ye; ++y) {
        const float4 w4 = qrow(y + 2);
        const float4 vc = ld4f(vel, base + y * X);
        const bool oin = y >= 2 && y + 2 < Y;
        float4 Fp, Fpo = vc, o4;
#pragma unroll
        for (int k = 0; k < 4; ++k) setc(Fp, k, face_flux(comp(vc, k), comp(w1, k), comp(w2, k), comp(w3, k), comp(w4, k), cdt));
        if (!oin) {
#pragma unroll
            for (int k = 0; k < 4; ++k) setc(Fpo, k, face_flux(comp(vc, k), orow(y - 1), orow(y), orow(y + 1), orow(y + 2), cdt));
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) setc(o4, k, ppm_update(comp(w2, k), comp(Fp, k), comp(Fc, k), comp(Fpo, k), comp(Fco, k), cdt));
        *reinterpret_cast<float4*>(out + base + y * X) = o4;
        Fc = Fp;
        Fco = Fpo;
        w0 = w1; w1 = w2; w2 = w3; w3 = w4;
    }
}

// Vectorised Z pass: the z march keeps the window q(z-2) .. q(z+2) and hands each upper-face
// flux on as the next plane's lower-face flux (computed directly at the first plane of a run; at
// z = 0 the face velocity is the boundary value).
__global__ void __launch_bounds__(32 * DVY) k_ppm4z(Grid g, int zlen, const float* __restrict__ in, float* __restrict__ out,
                                                    const float* __restrict__ vel, const float* __restrict__ def, int sides,
                                                    const float* __restrict__ defW, float dtFull, int nsub_host, int half,
                                                    const Scalars* __restrict__ sc, int slot) {
    int nsub = nsub_host;
    if (sc) {
        nsub = sc->nsub;
        if (slot >= nsub) return;
    }
    const float cdt = ppm_cdt(g, dtFull, nsub, half);
    const int lane = threadIdx.x;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * DVY + threadIdx.y + 1;
    const int zs = blockIdx.z * zlen, ze = min(zs + zlen, g.Z);
    if (x0 >= g.X || y >= g.Y) return;
    const int X = g.X, XY = g.XY, Z = g.Z;
    const int row = x0 + y * X;
    const float dy = def ? def[y] : 0.0f;
    const float so = bc_val(sides, 1.0f, 1.0f);
    auto side4 = [&](const float4& b) {
        return make_float4(bc_val(sides, b.x, dy), bc_val(sides, b.y, dy), bc_val(sides, b.z, dy), bc_val(sides, b.w, dy));
    };
    auto oz = [&](int zz) { return (zz >= 0 && zz < Z) ? 1.0f : so; };
    float4 w2 = ld4f(in, row + zs * XY);
    float4 w1 = zs >= 1 ? ld4f(in, row + (zs - 1) * XY) : side4(w2);
    float4 w0 = zs >= 2 ? ld4f(in, row + (zs - 2) * XY) : (zs == 1 ? side4(w1) : side4(w2));
    float4 w3 = zs + 1 < Z ? ld4f(in, row + (zs + 1) * XY) : side4(w2);
    float4 Fc, Fco;
    {
        float4 vm;
        if (zs == 0) {
            const float4 v0 = ld4f(vel, row);
            const float cu = defW[y];
            vm = make_float4(bc_val(sides, v0.x, cu), bc_val(sides, v0.y, cu), bc_val(sides, v0.z, cu), bc_val(sides, v0.w, cu));
        } else {
            vm = ld4f(vel, row + (zs - 1) * XY);
        }
        const bool oin = zs >= 2 && zs + 1 < Z;
#pragma unroll
        for (int k = 0; k < 4; ++k) setc(Fc, k, face_flux(comp(vm, k), comp(w0, k), comp(w1, k), comp(w2, k), comp(w3, k), cdt));
        Fco = vm;  // the companion's flux is the face velocity where its window is all ones
        if (!oin) {  // warp-uniform: a branch, not a select, so the interior skips the evaluation
#pragma unroll
            for (int k = 0; k < 4; ++k) setc(Fco, k, face_flux(comp(vm, k), oz(zs - 2), oz(zs - 1), oz(zs), oz(zs + 1), cdt));
        }
    }
    for (int z = zs; z < ze; ++z) {
        const int c = row + z * XY;
        const float4 w4 = z + 2 < Z ? ld4f(in, c + 2 * XY) : (z + 1 < Z ? side4(w3) : side4(w2));
        const float4 vc = ld4f(vel, c);
        const bool oin = z >= 1 && z + 2 < Z;
        float4 Fp, Fpo = vc, o4;
#pragma unroll
        for (int k = 0; k < 4; ++k) setc(Fp, k, face_flux(comp(vc, k), comp(w1, k), comp(w2, k), comp(w3, k), comp(w4, k), cdt));
        if (!oin) {
#pragma unroll
            for (int k = 0; k < 4; ++k) setc(Fpo, k, face_flux(comp(vc, k), oz(z - 1), oz(z), oz(z + 1), oz(z + 2), cdt));
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) setc(o4, k, ppm_update(comp(w2, k), comp(Fp, k), comp(Fc, k), comp(Fpo, k), comp(Fco, k), cdt));
        *reinterpret_cast<float4*>(out + c) = o4;
        Fc = Fp;
        Fco = Fpo;
        w0 = w1; w1 = w2; w2 = w3; w3 = w4;
    }
}

// copy the sky cells of src into dst (the end-of-substep copy, Game/environment.cu:805)
__global__ void __launch_bounds__(256) k_copy_sky(Grid g, const float* __restrict__ src, float* __restrict__ dst, const Scalars* __restrict__ sc, int slot) {
    if (sc && slot >= sc->nsub) return;
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    dst[c] = src[c];
}

// flat terrain: copy rows y >= 1 of every plane as float4
__global__ void __launch_bounds__(256) k_copy_sky4(int n4, int X4, int Y, const float4* __restrict__ src, float4* __restrict__ dst,
                                                   const Scalars* __restrict__ sc, int slot) {
    if (sc && slot >= sc->nsub) return;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < n4; i += gridDim.x * 256) {
        if ((i / X4) % Y == 0) continue;  // the ground layer
        dst[i] = src[i];
    }
}

// Max over sky cells of three fields (getMaxDivergence Game/kernelSky.cu:910-953 applied to
// u, v and w into one slot). reference=1: |a| at z=0, signed a for z>=1, floored at 0.
__global__ void __launch_bounds__(256) k_maxvel(Grid g, const float* __restrict__ a0, const float* __restrict__ a1, const float* __restrict__ a2,
                                                int reference, Scalars* __restrict__ sc) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    float m = 0.0f;
    bool bad = false;
    if (x < g.X && y < g.Y && !is_ground(g, x, y, z)) {
        const int c = cidx(g, x, y, z);
        const bool absv = !reference || z == 0;
        float v0 = a0[c], v1 = a1[c], v2 = a2[c];
        bad = nonfinite(v0) | nonfinite(v1) | nonfinite(v2);
        if (absv) { v0 = fabsf(v0); v1 = fabsf(v1); v2 = fabsf(v2); }
        if (v0 > m) m = v0;
        if (v1 > m) m = v1;
        if (v2 > m) m = v2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float t = __shfl_xor_sync(0xffffffffu, m, o);
        if (t > m) m = t;
    }
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(&sc->maxbits, __float_as_uint(m));
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) sc->status = SKT_NAN_DETECTED;  // a NaN or Inf wind
}

// flat terrain: the same max over rows y >= 1, as float4 streams with one atomic per block
__global__ void __launch_bounds__(256) k_maxvel4(int n4, int X4, int Y, int XY4, const float4* __restrict__ a0, const float4* __restrict__ a1,
                                                 const float4* __restrict__ a2, int reference, Scalars* __restrict__ sc) {
    __shared__ float sm[8];
    float m = 0.0f;
    bool bad = false;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < n4; i += gridDim.x * 256) {
        if ((i / X4) % Y == 0) continue;  // the ground layer
        const bool absv = !reference || i < XY4;
        const float4 v[3] = {a0[i], a1[i], a2[i]};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float e0 = v[j].x, e1 = v[j].y, e2 = v[j].z, e3 = v[j].w;
            bad |= nonfinite(e0) | nonfinite(e1) | nonfinite(e2) | nonfinite(e3);
            if (absv) { e0 = fabsf(e0); e1 = fabsf(e1); e2 = fabsf(e2); e3 = fabsf(e3); }
            if (e0 > m) m = e0;
            if (e1 > m) m = e1;
            if (e2 > m) m = e2;
            if (e3 > m) m = e3;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float t = __shfl_xor_sync(0xffffffffu, m, o);
        if (t > m) m = t;
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) sc->status = SKT_NAN_DETECTED;  // a NaN or Inf wind
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.0f;
        for (int w = 0; w < 8; ++w) b = sm[w] > b ? sm[w] : b;
        if (b > 0.0f) atomicMax(&sc->maxbits, __float_as_uint(b));
    }
}

// Courant substeps from the max velocity, on the device (Game/environment.cu:726-730)
__global__ void k_nsub(Scalars* sc, float dt, float vox, float maxsub) {
    const float maxVel = __uint_as_float(sc->maxbits);
    const float C = maxVel * dt / vox;
    sc->nsub = int(fminf(ceilf(fabsf(C)), maxsub));
}

// Sedimentation of one precipitation species (advectPrecipGPU Game/kernelSky.cu:576-657), one
// thread per (x,z) column marching up; each cell loses its outflow and gains the outflow of the
// cell above, both from the values at the start of the substep.
__global__ void __launch_bounds__(128) k_precip(Grid g, float* __restrict__ q, const float* __restrict__ th, const float* __restrict__ qv,
                                                const float* __restrict__ p, const float* __restrict__ Pg, int type, float dt, Gammas G) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.X * g.Z) return;
    const int x = col % g.X, z = col / g.X;
    const int gh = g.gh[col];
    const float vox = g.vox;
    const float pgc = Pg[col];
    auto fall = [&](float Q, int i) {
        const float T = th[i] * powf(p[i] / pgc, KC::KAPPA);
        const float Tv = T * (0.608f * qv[i] + 1);
        const float dens = p[i] * 100 / (KC::Rsd * Tv);
        float UR, US, UI;
        fallingVelocity(Q, Q, Q, dens, type, G.Qr, G.Qs, G.Qi, UR, US, UI);
        return type == 0 ? UR : (type == 1 ? US : UI);
    };
    int y = max(gh + 1, 0);
    if (y >= g.Y) return;
    int c = cidx(g, x, y, z);
    float QC = q[c];
    float fv = fall(QC, c);
    for (; y < g.Y; ++y) {
        const bool up = y < g.Y - 1;
        float QU = 0.0f, fvu = 0.0f;
        if (up) { QU = q[c + g.X]; fvu = fall(QU, c + g.X); }
        float val = QC;
        val -= dt * fminf((fv / vox) * QC, QC);
        if (up) val += dt * fminf((fvu / vox) * QU, QU);
        q[c] = val;
        QC = QU;
        fv = fvu;
        c += g.X;
    }
}

// The three falling species in one column march: precipGPU for rain, snow and ice
// (Game/kernelSky.cu:576-657, one launch per species in the reference). A species touches only its
// own mixing ratio and every species of a cell uses the same temperature, virtual temperature and
// density, so the three marches are one here, with each species' arithmetic unchanged. mask selects
// the species of this march (a species with more Courant substeps gets further marches). The
// loads of the row two above are issued one iteration ahead.
__device__ __forceinline__ float precip_dens(float thv, float qvv, float pv, float pgc) {
    const float T = thv * powf(pv / pgc, KC::KAPPA);
    const float Tv = T * (0.608f * qvv + 1);
    return pv * 100 / (KC::Rsd * Tv);
}
__device__ __forceinline__ float precip_speed(float Q, float dens, int type, const Gammas& G) {
    float UR, US, UI;
    fallingVelocity(Q, Q, Q, dens, type, G.Qr, G.Qs, G.Qi, UR, US, UI);
    return type == 0 ? UR : (type == 1 ? US : UI);
}
__global__ void __launch_bounds__(128) k_precip3(Grid g, float* __restrict__ qr, float* __restrict__ qs, float* __restrict__ qi,
                                                 const float* __restrict__ th, const float* __restrict__ qv,
                                                 const float* __restrict__ p, const float* __restrict__ Pg, int mask, float dtr,
                                                 float dts, float dti, Gammas G) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.X * g.Z) return;
    const int x = col % g.X, z = col / g.X;
    int y = max(g.gh[col] + 1, 0);
    if (y >= g.Y) return;
    float* const qs3[3] = {qr, qs, qi};
    const float dt3[3] = {dtr, dts, dti};
    const float vox = g.vox, pgc = Pg[col];
    const int X = g.X;
    int c = cidx(g, x, y, z);
    float QC[3] = {0.0f, 0.0f, 0.0f}, fv[3] = {0.0f, 0.0f, 0.0f};
    {
        const float d = precip_dens(th[c], qv[c], p[c], pgc);
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (mask & (1 << t)) { QC[t] = qs3[t][c]; fv[t] = precip_speed(QC[t], d, t, G); }
    }
    // the row above, loaded ahead
    float thN = 0.0f, qvN = 0.0f, pN = 0.0f, QN[3] = {0.0f, 0.0f, 0.0f};
    if (y + 1 < g.Y) {
        thN = th[c + X]; qvN = qv[c + X]; pN = p[c + X];
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (mask & (1 << t)) QN[t] = qs3[t][c + X];
    }
    for (; y < g.Y; ++y) {
        const bool up = y < g.Y - 1;
        float QU[3] = {0.0f, 0.0f, 0.0f}, fvu[3] = {0.0f, 0.0f, 0.0f};
        if (up) {
            const float d = precip_dens(thN, qvN, pN, pgc);
#pragma unroll
            for (int t = 0; t < 3; ++t)
                if (mask & (1 << t)) { QU[t] = QN[t]; fvu[t] = precip_speed(QU[t], d, t, G); }
        }
        if (y + 2 < g.Y) {
            const int c2 = c + 2 * X;
            thN = th[c2]; qvN = qv[c2]; pN = p[c2];
#pragma unroll
            for (int t = 0; t < 3; ++t)
                if (mask & (1 << t)) QN[t] = qs3[t][c2];
        }
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            if (!(mask & (1 << t))) continue;
            float val = QC[t];
            val -= dt3[t] * fminf((fv[t] / vox) * QC[t], QC[t]);
            if (up) val += dt3[t] * fminf((fvu[t] / vox) * QU[t], QU[t]);
            qs3[t][c] = val;
            QC[t] = QU[t];
            fv[t] = fvu[t];
        }
        c += X;
    }
}

// buoyancyGPU Game/kernelSky.cu:1061-1247 (bounds DIRICHLET everywhere)
__global__ void __launch_bounds__(256) k_buoyancy(Grid g, float* __restrict__ v, const float* __restrict__ th, const float* __restrict__ qv,
                                                  const float* __restrict__ qr, const float* __restrict__ qs, const float* __restrict__ qi,
                                                  const float* __restrict__ isenT, const float* __restrict__ isenQv,
                                                  const float* __restrict__ p, const float* __restrict__ Pg, float dt, float* __restrict__ dbg) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    const float vel = v[c];
    const bool up = y < g.Y - 1;
    const bool down = y > 0 && !is_ground(g, x, y - 1, z);
    auto valid = [&](int dx, int dz) { return in_dom(g, x + dx, y, z + dz) && !is_ground(g, x + dx, y, z + dz); };
    const int nv = int(valid(-1, 0)) + int(valid(1, 0)) + int(valid(0, -1)) + int(valid(0, 1));
    if (nv == 0) {
        if (dbg) dbg[c] = 0.0f;
        return;
    }
    const float Pgs = Pg[x + z * g.X];
    const float psC = p[c];
    const float psU = up ? p[c + g.X] : psC;
    const float psD = down ? p[c - g.X] : psC;
    auto Q = [&](int dx, int dy, int dz) { return ghost(g, qv, x + dx, y + dy, z + dz, DIRICHLET, DIRICHLET, isenQv); };
    auto TH = [&](int dx, int dy, int dz) { return ghost(g, th, x + dx, y + dy, z + dz, DIRICHLET, DIRICHLET, isenT); };
    const float QP = qv[c];
    const float Qenv = (Q(1, 0, 0) + Q(-1, 0, 0) + Q(0, 0, 1) + Q(0, 0, -1)) / nv;
    const float QenvUp = Q(0, 1, 0), QenvDown = Q(0, -1, 0);
    const float thc = th[c];
    const float thU = TH(0, 1, 0), thD = TH(0, -1, 0);
    const float TDown = thD * powf(psD / Pgs, KC::KAPPA);
    const float Tc = thc * powf(psC / Pgs, KC::KAPPA);
    const float TUp = thU * powf(psU / Pgs, KC::KAPPA);
    float Tad = thc, TadUp = thc, TadDown = thc;
    const float Tenv = (TH(1, 0, 0) + TH(-1, 0, 0) + TH(0, 0, 1) + TH(0, 0, -1)) / nv;
    const float TenvUp = thU, TenvDown = thD;
    if (down) {
        if ((Tc < 0.0f && QP >= wi(TDown - 273.15f, psD)) || QP >= ws(TDown - 273.15f, psD)) {
            TadDown = Tc - MLR(Tc - 273.15f, psC) * (psC - psD);
            TadDown = TadDown * powf(Pgs / psD, KC::KAPPA);
        }
    }
    if (up) {
        if ((Tc < 0.0f && QP >= wi(TUp - 273.15f, psU)) || QP >= ws(TUp - 273.15f, psU)) {
            TadUp = MLR(Tc - 273.15f, psC) * (psU - psC) + Tc;
            TadUp = TadUp * powf(Pgs / psU, KC::KAPPA);
        }
    }
    float B = 0.0f, BUp = 0.0f, BDown = 0.0f;
    const float totalQ = qr[c] + qs[c] + qi[c];
    if (down) {
        const float VTP = TadDown * (1.0f + 0.608f * QP), VTE = TenvDown * (1.0f + 0.608f * QenvDown);
        BDown = KC::g * ((VTP - VTE) / VTE) - totalQ * KC::g;
    }
    {
        const float VTP = Tad * (1.0f + 0.608f * QP), VTE = Tenv * (1.0f + 0.608f * Qenv);
        B = KC::g * ((VTP - VTE) / VTE) - totalQ * KC::g;
    }
    if (up) {
        const float VTP = TadUp * (1.0f + 0.608f * QP), VTE = TenvUp * (1.0f + 0.608f * QenvUp);
        BUp = KC::g * ((VTP - VTE) / VTE) - totalQ * KC::g;
    }
    float fin = B;
    if (vel > 0.0f) fin = BUp;
    else if (vel < 0.0f) fin = BDown;
    float change = fin * dt;
    if ((up && vel > 0.0f && -change > vel) || (down && vel < 0.0f && -change < vel)) change = -vel;
    if (dbg) dbg[c] = change;  // buoyancyStor, the reference's second debug field
    v[c] = vel + change;
}

// k_buoyancy for flat terrain and X % 4 == 0: four cells per thread and a march up the rows. A
// cell's temperature th (p/Pg)^kappa and its ws(T - 273.15, p) are the "down" values of the cell
// above and the "up" values of the cell below (the same calls on the same inputs), so each is
// formed once per cell and handed along the march instead of three times. The horizontal means
// take x neighbours from the neighbouring lanes and z neighbours from the rows of the block's
// other warps. Arithmetic and the order of every sum as in k_buoyancy.
constexpr int BZ4 = 8;
__device__ __forceinline__ float buoy_change(float vel, bool up, bool down, float Pgs, float psC, float psU, float psD, float QP,
                                             float Qenv, float QenvUp, float QenvDown, float thc, float thU, float thD, float Tc,
                                             float TUp, float TDown, float WUp, float WDown, float Tenv, float totalQ, float dt) {
    float Tad = thc, TadUp = thc, TadDown = thc;
    const float TenvUp = thU, TenvDown = thD;
    if (down) {
        if ((Tc < 0.0f && QP >= wi(TDown - 273.15f, psD)) || QP >= WDown) {
            TadDown = Tc - MLR(Tc - 273.15f, psC) * (psC - psD);
            TadDown = TadDown * powf(Pgs / psD, KC::KAPPA);
        }
    }
    if (up) {
        if ((Tc < 0.0f && QP >= wi(TUp - 273.15f, psU)) || QP >= WUp) {
            TadUp = MLR(Tc - 273.15f, psC) * (psU - psC) + Tc;
            TadUp = TadUp * powf(Pgs / psU, KC::KAPPA);
        }
    }
    float B = 0.0f, BUp = 0.0f, BDown = 0.0f;
    if (down) {
        const float VTP = TadDown * (1.0f + 0.608f * QP), VTE = TenvDown * (1.0f + 0.608f * QenvDown);
        BDown = KC::g * ((VTP - VTE) / VTE) - totalQ * KC::g;
    }
    {
        const float VTP = Tad * (1.0f + 0.608f * QP), VTE = Tenv * (1.0f + 0.608f * Qenv);
        B = KC::g * ((VTP - VTE) / VTE) - totalQ * KC::g;
    }
    if (up) {
        const float VTP = TadUp * (1.0f + 0.608f * QP), VTE = TenvUp * (1.0f + 0.608f * QenvUp);
        BUp = KC::g * ((VTP - VTE) / VTE) - totalQ * KC::g;
    }
    float fin = B;
    if (vel > 0.0f) fin = BUp;
    else if (vel < 0.0f) fin = BDown;
    float change = fin * dt;
    if ((up && vel > 0.0f && -change > vel) || (down && vel < 0.0f && -change < vel)) change = -vel;
    return change;
}

__global__ void __launch_bounds__(32 * BZ4) k_buoyancy4(Grid g, int ylen, float* __restrict__ v, const float* __restrict__ th,
                                                        const float* __restrict__ qv, const float* __restrict__ qr,
                                                        const float* __restrict__ qs, const float* __restrict__ qi,
                                                        const float* __restrict__ p, const float* __restrict__ Pg, float dt,
                                                        float* __restrict__ dbg) {
    const int lane = threadIdx.x;
    const int xw = blockIdx.x * 128, x0 = xw + lane * 4;
    const int z = blockIdx.y * BZ4 + threadIdx.y;
    const int ys = 1 + blockIdx.z * ylen, ye = min(ys + ylen, g.Y);
    if (xw >= g.X || z >= g.Z || ys >= g.Y) return;  // the whole warp
    const bool act = x0 < g.X;
    const int X = g.X, XY = g.XY, Y = g.Y, Z = g.Z;
    const int col = x0 + z * XY;  // + y*X
    const float4 z4 = make_float4(0, 0, 0, 0);
    const float4 pg = act ? ld4f(Pg, x0 + z * X) : make_float4(1, 1, 1, 1);
    // valid horizontal neighbours per cell (flat terrain: the in-domain ones)
    float nv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = x0 + k;
        nv[k] = float(int(x + 1 < X) + int(x > 0) + int(z + 1 < Z) + int(z > 0));
    }
    auto temps = [&](const float4& thv, const float4& pv, float4& T, float4& W) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float t = comp(thv, k) * powf(comp(pv, k) / comp(pg, k), KC::KAPPA);
            setc(T, k, t);
            setc(W, k, ws(t - 273.15f, comp(pv, k)));
        }
    };
    // rows y-1 (d), y (c), y+1 (u): theta, qv, p, T, W
    float4 thd = z4, qvd = z4, pd = z4, Td = z4, Wd = z4;
    float4 thc = z4, qvc = z4, pc = z4, Tc = z4, Wc = z4;
    if (act) {
        if (ys >= 2) {
            const int c = col + (ys - 1) * X;
            thd = ld4f(th, c); qvd = ld4f(qv, c); pd = ld4f(p, c);
            temps(thd, pd, Td, Wd);
        }
        const int c = col + ys * X;
        thc = ld4f(th, c); qvc = ld4f(qv, c); pc = ld4f(p, c);
        temps(thc, pc, Tc, Wc);
    }
    for (int y = ys; y < ye; ++y) {
        const int c = col + y * X;
        const bool up = y < Y - 1, down = y >= 2;
        float4 thu = z4, qvu = z4, pu = pc, Tu = z4, Wu = z4;
        float4 vel = z4, tq = z4, thb = z4, thf = z4, qb = z4, qf = z4;
        if (act) {
            if (up) {
                thu = ld4f(th, c + X); qvu = ld4f(qv, c + X); pu = ld4f(p, c + X);
                temps(thu, pu, Tu, Wu);
            }
            vel = ld4f(v, c);
            const float4 a = ld4f(qr, c), b = ld4f(qs, c), d = ld4f(qi, c);
            tq = make_float4(a.x + b.x + d.x, a.y + b.y + d.y, a.z + b.z + d.z, a.w + b.w + d.w);
            if (z > 0) { thb = ld4f(th, c - XY); qb = ld4f(qv, c - XY); }
            if (z + 1 < Z) { thf = ld4f(th, c + XY); qf = ld4f(qv, c + XY); }
        }
        // x neighbours of the row's ends (outside the domain: DIRICHLET, 0)
        float thl = __shfl_up_sync(0xffffffffu, thc.w, 1), ql = __shfl_up_sync(0xffffffffu, qvc.w, 1);
        float thr = __shfl_down_sync(0xffffffffu, thc.x, 1), qr_ = __shfl_down_sync(0xffffffffu, qvc.x, 1);
        if (act) {
            if (lane == 0) { thl = x0 > 0 ? th[c - 1] : 0.0f; ql = x0 > 0 ? qv[c - 1] : 0.0f; }
            if (lane == 31 || x0 + 4 >= X) {
                thr = x0 + 4 < X ? th[c + 4] : 0.0f;
                qr_ = x0 + 4 < X ? qv[c + 4] : 0.0f;
            }
            const float thxp[4] = {thc.y, thc.z, thc.w, thr}, thxm[4] = {thl, thc.x, thc.y, thc.z};
            const float qxp[4] = {qvc.y, qvc.z, qvc.w, qr_}, qxm[4] = {ql, qvc.x, qvc.y, qvc.z};
            float4 nvel, ch;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float Qenv = (qxp[k] + qxm[k] + comp(qf, k) + comp(qb, k)) / nv[k];
                const float Tenv = (thxp[k] + thxm[k] + comp(thf, k) + comp(thb, k)) / nv[k];
                const float psC = comp(pc, k);
                const float psU = up ? comp(pu, k) : psC, psD = down ? comp(pd, k) : psC;
                const float thU = up ? comp(thu, k) : 0.0f, thD = down ? comp(thd, k) : 0.0f;
                const float QU = up ? comp(qvu, k) : 0.0f, QD = down ? comp(qvd, k) : 0.0f;
                const float change = buoy_change(comp(vel, k), up, down, comp(pg, k), psC, psU, psD, comp(qvc, k), Qenv, QU, QD,
                                                 comp(thc, k), thU, thD, comp(Tc, k), comp(Tu, k), comp(Td, k), comp(Wu, k),
                                                 comp(Wd, k), Tenv, comp(tq, k), dt);
                setc(ch, k, change);
                setc(nvel, k, comp(vel, k) + change);
            }
            *reinterpret_cast<float4*>(v + c) = nvel;
            if (dbg) *reinterpret_cast<float4*>(dbg + c) = ch;
        }
        thd = thc; qvd = qvc; pd = pc; Td = Tc; Wd = Wc;
        thc = thu; qvc = qvu; pc = pu; Tc = Tu; Wc = Wu;
    }
}

// initDensity Game/kernelSky.cu:1432-1452
__global__ void __launch_bounds__(256) k_init_density(Grid g, float* __restrict__ rho, const float* __restrict__ th, const float* __restrict__ p,
                                                      const float* __restrict__ qv, const float* __restrict__ Pg) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    const float T = th[c] * powf(p[c] / Pg[x + z * g.X], KC::KAPPA);
    const float Tv = T * (0.608f * qv[c] + 1);
    rho[c] = p[c] * 100 / (KC::Rsd * Tv);
}

// calculateNewPressure Game/kernelSky.cu:1454-1474
__global__ void __launch_bounds__(256) k_new_pressure(Grid g, float* __restrict__ p, const float* __restrict__ rho, const float* __restrict__ th,
                                                      const float* __restrict__ qv, const float* __restrict__ Pg) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    const float T = th[c] * powf(p[c] / Pg[x + z * g.X], KC::KAPPA);
    const float Tv = T * (0.608f * qv[c] + 1);
    p[c] = rho[c] * KC::Rsd * Tv / 100.0f;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------------

namespace {

// Flat terrain, X % 4 == 0: the sweeps alternate between the scratch fields and the last one
// writes f itself, so no copy is needed (no sweep reads the array it writes, and the ground rows
// of the scratch fields are never read). A single sweep goes through a scratch field.
// z chunking of a march over gx x gy columns of blocks: about bps blocks per SM in the grid
inline int z_runs(const Env& e, int gx, int gy, int bps, int& zlen) {
    int zc = std::max(1, std::min(e.g.Z, (stencil_sms(e) * bps + gx * gy - 1) / (gx * gy)));
    zlen = (e.g.Z + zc - 1) / zc;
    return (e.g.Z + zlen - 1) / zlen;
}

// cuTensorMapEncodeTiled through the runtime's driver entry points (no link against libcuda)
typedef CUresult (*TensorMapEncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                      const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                      CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
TensorMapEncodeFn tensor_map_encoder() {
    static TensorMapEncodeFn fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<TensorMapEncodeFn>(p);
    }
    return fn;
}

// A field as a 3D tensor (x fastest) read in boxes of width x rows x 1 cells; false if it cannot be encoded.
bool field_tensor_map(const Grid& g, const float* base, int width, int rows, CUtensorMap* map) {
    TensorMapEncodeFn enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {cuuint64_t(g.X), cuuint64_t(g.Y), cuuint64_t(g.Z)};
    const cuuint64_t strides[2] = {cuuint64_t(g.X) * 4, cuuint64_t(g.XY) * 4};
    const cuuint32_t box[3] = {cuuint32_t(width), cuuint32_t(rows), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool THETA, int H>
bool launch_diffuse2(Env& e, int bps, const float* src, float* dst, int sides, int ground, const float* def, float k,
                     const float* face) {
    const Grid& g = e.g;
    CUtensorMap map;
    if (!field_tensor_map(g, src, D2BW, d2_box_rows<H>(), &map)) return false;
    const int gx = (g.X + D2OUT - 1) / D2OUT, gy = (g.Y - 1 + H * D2WARPS - 1) / (H * D2WARPS);
    int zlen;
    const int zc = z_runs(e, gx, gy, bps, zlen);
    constexpr int smem = d2_smem_bytes<H>();
    static bool attr = false;  // per template instance
    if (!attr) {
        cudaFuncSetAttribute(k_diffuse2<THETA, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    k_diffuse2<THETA, H><<<dim3(gx, gy, zc), dim3(32, D2WARPS), smem, e.stream>>>(map, g, zlen, dst, sides, ground, def, k, face, e.sc);
    return true;
}

template <bool THETA, int R>
bool launch_diffuse_pair4(Env& e, int bps, const float* src, float* dst, int sides, int ground, const float* def, float k,
                          const float* face) {
    const Grid& g = e.g;
    CUtensorMap map;
    if (!field_tensor_map(g, src, P4W, R + 4, &map)) return false;
    const int gx = (g.X + 127) / 128, gy = (g.Y - 1 + R - 1) / R;
    int zlen;
    const int zc = z_runs(e, gx, gy, bps, zlen);
    constexpr int smem = p4_smem_bytes<R>();
    static bool attr = false;  // per template instance
    if (!attr) {
        cudaFuncSetAttribute(k_diffuse_pair4<THETA, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    k_diffuse_pair4<THETA, R><<<dim3(gx, gy, zc), 32 * (R + 3), smem, e.stream>>>(map, g, zlen, dst, sides, ground, def, k, face,
                                                                                    e.sc);
    return true;
}

// one pass of two sweeps with the tuned kernel: k_diffuse_pair4 (float4 lanes, rows 6 or 14 per
// block) or k_diffuse2 (one cell per lane, rows 4 or 8 per warp); false without a tensor map
template <bool THETA>
bool launch_pair(Env& e, const float* src, float* dst, int sides, int ground, const float* def, float k, const float* face) {
    const int h = e.tune.diffuse_h, bps = e.tune.diffuse2_bps;
    switch (h) {
        case 14: return launch_diffuse_pair4<THETA, 14>(e, bps, src, dst, sides, ground, def, k, face);
        case 6: return launch_diffuse_pair4<THETA, 6>(e, bps, src, dst, sides, ground, def, k, face);
        case 8: return launch_diffuse2<THETA, 8>(e, bps, src, dst, sides, ground, def, k, face);
        default: return launch_diffuse2<THETA, 4>(e, bps, src, dst, sides, ground, def, k, face);
    }
}

void diffuse_vec(Env& e, float* f, int type, int sides, int ground, const float* def, float k, int sweeps) {
    const Grid& g = e.g;
    const int vx = (g.X / 4 + 31) / 32, vy = (g.Y - 1 + DVY - 1) / DVY;
    int vlen;
    const int vz = z_runs(e, vx, vy, e.tune.diffuse_bps, vlen);
    float* buf[3] = {e.tA, e.tB, e.As};  // As: the middle sweep of a pair when no tensor map can be made
    const float* src = f;
    float* face = e.g2a;  // ground scratch: free until the ground stage refills it
    if (type == 0) {
        k_theta_face<<<(g.X * g.Z + 255) / 256, 256, 0, e.stream>>>(g, e.p, e.Tg, e.Pg, face);
        e.launches += 1;
    }
    // passes of one sweep, or (temporal blocking of depth 2) of two sweeps: an odd count starts
    // with a single sweep
    const bool pairs = e.tune.diffuse_depth == 2;
    const int npass = pairs ? sweeps / 2 + sweeps % 2 : sweeps;
    for (int q = 0; q < npass; ++q) {
        float* dst = (q == npass - 1 && q > 0) ? f : buf[q % 2];
        const bool two = pairs && !(q == 0 && sweeps % 2 == 1);
        if (two) {
            const bool ok = type == 0 ? launch_pair<true>(e, src, dst, sides, ground, def, k, face)
                                      : launch_pair<false>(e, src, dst, sides, ground, def, k, nullptr);
            if (!ok) {  // no tensor-map encoder: the two sweeps as two passes
                if (type == 0) {
                    k_diffuse4<true><<<dim3(vx, vy, vz), dim3(32, DVY), 0, e.stream>>>(g, vlen, src, buf[2], sides, ground, def, k, face);
                    k_diffuse4<true><<<dim3(vx, vy, vz), dim3(32, DVY), 0, e.stream>>>(g, vlen, buf[2], dst, sides, ground, def, k, face);
                } else {
                    k_diffuse4<false><<<dim3(vx, vy, vz), dim3(32, DVY), 0, e.stream>>>(g, vlen, src, buf[2], sides, ground, def, k, nullptr);
                    k_diffuse4<false><<<dim3(vx, vy, vz), dim3(32, DVY), 0, e.stream>>>(g, vlen, buf[2], dst, sides, ground, def, k, nullptr);
                }
                e.launches += 1;
            }
        } else if (type == 0) {
            k_diffuse4<true><<<dim3(vx, vy, vz), dim3(32, DVY), 0, e.stream>>>(g, vlen, src, dst, sides, ground, def, k, face);
        } else {
            k_diffuse4<false><<<dim3(vx, vy, vz), dim3(32, DVY), 0, e.stream>>>(g, vlen, src, dst, sides, ground, def, k, nullptr);
        }
        e.launches += 1;
        src = dst;
    }
    if (npass == 1) {
        const int n4 = g.N / 4;
        k_copy_sky4<<<std::min((n4 + 255) / 256, stencil_sms(e) * 8), 256, 0, e.stream>>>(n4, g.X / 4, g.Y, (const float4*)src, (float4*)f,
                                                                                     nullptr, 0);
        e.launches += 1;
    }
}

}  // namespace

// diffuseGPU Game/environment.cu:597-673: per-type boundary table :603-638, k = 0.005*dt/vox^2
void launch_diffuse(Env& e, float* f, int type, float dtS) {
    const Grid& g = e.g;
    const float* def = nullptr;
    int sides = NEUMANN, ground = DIRICHLET;
    switch (type) {
        case 0: def = e.isenT; sides = CUSTOM; ground = CUSTOM; break;
        case 1: def = e.isenQv; sides = CUSTOM; ground = DIRICHLET; break;
        case 2: def = e.defU; sides = CUSTOM; break;
        case 3: def = nullptr; sides = NEUMANN; break;
        case 4: def = e.defW; sides = CUSTOM; break;
        default: def = e.zeroY; break;
    }
    const float k = 0.005f * dtS / (g.vox * g.vox);
    const int sweeps = e.cfg.diffuse_sweeps;
    ProfScope ps(e, "diffuse");
    if (e.flat && (g.X % 4) == 0 && sweeps > 0) {
        diffuse_vec(e, f, type, sides, ground, def, k, sweeps);
        return;
    }
    e.launches += sweeps + 1;
    cudaMemcpyAsync(e.tA, f, sizeof(float) * size_t(g.N), cudaMemcpyDeviceToDevice, e.stream);
    cudaMemcpyAsync(e.tB, f, sizeof(float) * size_t(g.N), cudaMemcpyDeviceToDevice, e.stream);
    float* a = e.tA;
    float* o = e.tB;
    // general heightfield or X % 4 != 0 (or no sweeps): the scalar sweep
    const bool vec = e.flat && (g.X % 4) == 0;
    for (int s = 0; s < sweeps; ++s) {
        const float* in = (s % 2 == 0) ? a : o;
        float* out = (s % 2 == 0) ? o : a;
        if (type == 0)
            k_diffuse<true><<<cell_grid(g), dim3(BX, BY), 0, e.stream>>>(g, in, out, sides, ground, def, k, e.p, e.Tg, e.Pg);
        else
            k_diffuse<false><<<cell_grid(g), dim3(BX, BY), 0, e.stream>>>(g, in, out, sides, ground, def, k, e.p, e.Tg, e.Pg);
    }
    const float* res = (sweeps % 2 == 0) ? a : o;
    if (vec) {
        const int n4 = g.N / 4;
        k_copy_sky4<<<std::min((n4 + 255) / 256, stencil_sms(e) * 8), 256, 0, e.stream>>>(n4, g.X / 4, g.Y, (const float4*)res, (float4*)f,
                                                                                     nullptr, 0);
    } else {
        k_copy_sky<<<cell_grid(g), dim3(BX, BY), 0, e.stream>>>(g, res, f, nullptr, 0);
    }
}

// Graph mode, advection loop: the first trip runs when the field has any substep; each trip counts
// a substep and runs again while substeps remain. The field's count is kept for the step's stats.
__global__ void k_adv_begin(cudaGraphConditionalHandle h, Scalars* sc, int field) {
    sc->slot = 0;
    if (field >= 0 && field < 10) sc->nsub_f[field] = sc->nsub;
    cudaGraphSetConditional(h, sc->nsub > 0 ? 1u : 0u);
}
__global__ void k_adv_next(cudaGraphConditionalHandle h, Scalars* sc, int loop) {
    note_trip(sc, loop);
    sc->slot += 1;
    cudaGraphSetConditional(h, sc->slot < sc->nsub ? 1u : 0u);
}

// advectPPMWGPU Game/environment.cu:692-824. With host_sync the substep count is read back as
// the reference does; otherwise max_substeps slots are launched and the ones beyond the device
// count exit at once (graph capture). Returns the substep count (or -1 when not read back).
int launch_advect(Env& e, float* f, const float* def, int sides, int ground, float dtS, int slot_id, bool host_sync,
                  bool same_wind) {
    const Grid& g = e.g;
    ProfScope ps(e, "advect");
    // same_wind: the wind has not changed since the last advection (the moisture fields after the
    // projection), so its Courant substep count (sc->nsub, and the host copy) stands
    if (!same_wind || e.adv_nsub < 0) {
        e.launches += 2;
        cudaMemsetAsync(&e.sc->maxbits, 0, sizeof(unsigned int), e.stream);
        if (e.flat && (g.X % 4) == 0) {
            const int n4 = g.N / 4;
            k_maxvel4<<<std::min((n4 + 255) / 256, stencil_sms(e) * 8), 256, 0, e.stream>>>(n4, g.X / 4, g.Y, g.XY / 4, (const float4*)e.u,
                                                                                      (const float4*)e.v, (const float4*)e.w,
                                                                                      e.cfg.semantics == 0, e.sc);
        } else {
            k_maxvel<<<cell_grid(g), dim3(BX, BY), 0, e.stream>>>(g, e.u, e.v, e.w, e.cfg.semantics == 0, e.sc);
        }
        k_nsub<<<1, 1, 0, e.stream>>>(e.sc, dtS, g.vox, float(e.cfg.max_substeps));
        e.adv_nsub = -1;
        if (host_sync && !e.capturing) {
            fetch_scalars(e);
            e.adv_nsub = e.host_sc->nsub;
        } else {
            e.adv_nsub = 0;  // on the device only (sc->nsub)
        }
    }
    int nsub = -1;
    int slots;
    const Scalars* chk = nullptr;
    if (host_sync) {
        nsub = e.adv_nsub;
        slots = nsub;
    } else {
        slots = e.cfg.max_substeps;
        chk = e.sc;
    }
    const dim3 grd = cell_grid(g), blk(BX, BY);
    float* A = f;
    float* O = e.tA;
    const bool vec = e.flat && (g.X % 4) == 0;
    const int gx = (g.X / 4 + 31) / 32, gy = (g.Y - 1 + DVY - 1) / DVY;
    int zc = std::max(1, std::min(g.Z, (stencil_sms(e) * e.tune.ppm_bps + gx * gy - 1) / (gx * gy)));
    const int zlen = (g.Z + zc - 1) / zc;
    zc = (g.Z + zlen - 1) / zlen;
    const dim3 vg(gx, gy, zc), vb(32, DVY);
    // the Z pass marches: fewer, longer z chunks
    int zc2 = std::max(1, std::min(g.Z, (stencil_sms(e) * e.tune.ppmz_bps + gx * gy - 1) / (gx * gy)));
    const int zlen2 = (g.Z + zc2 - 1) / zc2;
    zc2 = (g.Z + zlen2 - 1) / zlen2;
    const dim3 vg2(gx, gy, zc2);
    // the Y pass marches rows in runs
    const int ygz = (g.Z + PY - 1) / PY;
    int yc = std::max(1, std::min(g.Y - 1, (stencil_sms(e) * e.tune.ppmy_bps + gx * ygz - 1) / (gx * ygz)));
    const int ylen = (g.Y - 1 + yc - 1) / yc;
    yc = (g.Y - 1 + ylen - 1) / ylen;
    const dim3 yg(gx, ygz, yc), yb(32, PY);
    const int n4 = g.N / 4;
    const int ncopy = std::min((n4 + 255) / 256, stencil_sms(e) * 8);
    // one substep (slot i; with chk set, the kernels read the substep count from the device and
    // slots at or beyond it return at once)
    auto substep = [&](int i, const Scalars* chk) {
        if (vec && f != e.v) {
            // A -> O -> B -> O -> B -> A through the second scratch field: the last pass writes the
            // field's sky cells itself (no copy). A pass reads the wind as it stands: for u (x
            // passes) and w (z pass) that is the chain's current buffer.
            float* B = e.tB;
            k_ppm4x<<<vg, vb, 0, e.stream>>>(g, zlen, A, O, e.u, def, sides, e.defU, dtS, nsub, 1, chk, i);
            k_ppm4y<<<yg, yb, 0, e.stream>>>(g, ylen, O, B, e.v, def, sides, ground, dtS, nsub, 1, chk, i);
            k_ppm4z<<<vg2, vb, 0, e.stream>>>(g, zlen2, B, O, f == e.w ? B : e.w, def, sides, e.defW, dtS, nsub, 0, chk, i);
            k_ppm4y<<<yg, yb, 0, e.stream>>>(g, ylen, O, B, e.v, def, sides, ground, dtS, nsub, 1, chk, i);
            k_ppm4x<<<vg, vb, 0, e.stream>>>(g, zlen, B, A, f == e.u ? B : e.u, def, sides, e.defU, dtS, nsub, 1, chk, i);
            return;
        }
        if (vec) {
            k_ppm4x<<<vg, vb, 0, e.stream>>>(g, zlen, A, O, e.u, def, sides, e.defU, dtS, nsub, 1, chk, i);
            const float* vy = e.v;
            if (f == e.v) {
                cudaMemcpyAsync(e.tB, e.v, sizeof(float) * size_t(g.N), cudaMemcpyDeviceToDevice, e.stream);
                vy = e.tB;
            }
            k_ppm4y<<<yg, yb, 0, e.stream>>>(g, ylen, O, A, vy, def, sides, ground, dtS, nsub, 1, chk, i);
            k_ppm4z<<<vg2, vb, 0, e.stream>>>(g, zlen2, A, O, e.w, def, sides, e.defW, dtS, nsub, 0, chk, i);
            vy = e.v;
            if (f == e.v) {
                cudaMemcpyAsync(e.tB, e.v, sizeof(float) * size_t(g.N), cudaMemcpyDeviceToDevice, e.stream);
                vy = e.tB;
            }
            k_ppm4y<<<yg, yb, 0, e.stream>>>(g, ylen, O, A, vy, def, sides, ground, dtS, nsub, 1, chk, i);
            k_ppm4x<<<vg, vb, 0, e.stream>>>(g, zlen, A, O, e.u, def, sides, e.defU, dtS, nsub, 1, chk, i);
            k_copy_sky4<<<ncopy, 256, 0, e.stream>>>(n4, g.X / 4, g.Y, (const float4*)O, (float4*)A, chk, i);
            return;
        }
        // pass 1: X half, A -> O (velocity u as it stands: for f == u this is A)
        k_ppm<0><<<grd, blk, 0, e.stream>>>(g, A, O, e.u, def, sides, ground, e.defU, e.defW, dtS, nsub, 1, chk, i);
        // pass 2: Y half, O -> A; the velocity is v as it stands before the pass (for f == v: q0)
        const float* vy = e.v;
        if (f == e.v) {
            cudaMemcpyAsync(e.tB, e.v, sizeof(float) * size_t(g.N), cudaMemcpyDeviceToDevice, e.stream);
            vy = e.tB;
        }
        k_ppm<1><<<grd, blk, 0, e.stream>>>(g, O, A, vy, def, sides, ground, e.defU, e.defW, dtS, nsub, 1, chk, i);
        // pass 3: Z full, A -> O
        k_ppm<2><<<grd, blk, 0, e.stream>>>(g, A, O, e.w, def, sides, ground, e.defU, e.defW, dtS, nsub, 0, chk, i);
        // pass 4: Y half, O -> A
        vy = e.v;
        if (f == e.v) {
            cudaMemcpyAsync(e.tB, e.v, sizeof(float) * size_t(g.N), cudaMemcpyDeviceToDevice, e.stream);
            vy = e.tB;
        }
        k_ppm<1><<<grd, blk, 0, e.stream>>>(g, O, A, vy, def, sides, ground, e.defU, e.defW, dtS, nsub, 1, chk, i);
        // pass 5: X half, A -> O, then A = O on sky cells
        k_ppm<0><<<grd, blk, 0, e.stream>>>(g, A, O, e.u, def, sides, ground, e.defU, e.defW, dtS, nsub, 1, chk, i);
        k_copy_sky<<<grd, blk, 0, e.stream>>>(g, O, A, chk, i);
    };
    if (e.capturing) {
        // graph mode: the substep count stays on the device and the substeps run as a WHILE loop
        e.adv_nsub = 0;
        graph_while(
            e, [&](cudaGraphConditionalHandle h) {
                k_adv_begin<<<1, 1, 0, e.stream>>>(h, e.sc, slot_id);
                e.launches += 1;
            },
            [&](cudaGraphConditionalHandle h, int loop) {
                e.launches += 6;
                substep(0, e.sc);
                k_adv_next<<<1, 1, 0, e.stream>>>(h, e.sc, loop);
                e.launches += 1;
            });
        return -1;
    }
    e.launches += 6LL * slots;
    for (int i = 0; i < slots; ++i) substep(i, chk);
    (void)slot_id;
    return nsub;
}

// advectPrecip Game/environment.cu:826-849: substeps from the guessed fall speeds 5/1/8 m/s
void launch_precip(Env& e, float* q, int type, float dtS) {
    const Grid& g = e.g;
    const float maxVel = type == 0 ? 5.0f : (type == 1 ? 1.0f : 8.0f);
    const float C = maxVel * dtS / g.vox;
    const int sub = int(fminf(ceilf(fabsf(C)), float(e.cfg.max_substeps)));
    const float dts = dtS / float(sub);
    const int cols = g.X * g.Z;
    ProfScope ps(e, "precip");
    e.launches += sub;
    for (int i = 0; i < sub; ++i)
        k_precip<<<(cols + 127) / 128, 128, 0, e.stream>>>(g, q, e.th, e.qv, e.p, e.Pg, type, dts, e.gam);
}

// rain, snow and ice with their own Courant substeps (maximum fall speeds 5, 1, 8 m/s as in
// launch_precip); march s updates the species that need more than s substeps
void launch_precip3(Env& e, float dtS) {
    const Grid& g = e.g;
    const float maxVel[3] = {5.0f, 1.0f, 8.0f};
    int sub[3], passes = 0;
    float dts[3];
    for (int t = 0; t < 3; ++t) {
        const float C = maxVel[t] * dtS / g.vox;
        sub[t] = int(fminf(ceilf(fabsf(C)), float(e.cfg.max_substeps)));
        dts[t] = dtS / float(sub[t]);
        passes = std::max(passes, sub[t]);
    }
    const int cols = g.X * g.Z;
    ProfScope ps(e, "precip");
    for (int s = 0; s < passes; ++s) {
        const int mask = (sub[0] > s ? 1 : 0) | (sub[1] > s ? 2 : 0) | (sub[2] > s ? 4 : 0);
        e.launches += 1;
        k_precip3<<<(cols + 127) / 128, 128, 0, e.stream>>>(g, e.qr, e.qs, e.qi, e.th, e.qv, e.p, e.Pg, mask, dts[0], dts[1],
                                                            dts[2], e.gam);
    }
}

void launch_buoyancy(Env& e, float dtS) {
    ProfScope ps(e, "buoyancy");
    e.launches += 1;
    float* dbg = (e.diag_flags & SKT_DIAG_BUOYANCY) ? e.dbg_buoy : nullptr;
    const Grid& g = e.g;
    if (e.flat && (g.X % 4) == 0) {
        const int gx = (g.X / 4 + 31) / 32, gz = (g.Z + BZ4 - 1) / BZ4;
        int yc = std::max(1, std::min(g.Y - 1, (stencil_sms(e) * 8 + gx * gz - 1) / (gx * gz)));
        const int ylen = (g.Y - 1 + yc - 1) / yc;
        yc = (g.Y - 1 + ylen - 1) / ylen;
        k_buoyancy4<<<dim3(gx, gz, yc), dim3(32, BZ4), 0, e.stream>>>(g, ylen, e.v, e.th, e.qv, e.qr, e.qs, e.qi, e.p, e.Pg, dtS, dbg);
        return;
    }
    k_buoyancy<<<cell_grid(g), dim3(BX, BY), 0, e.stream>>>(g, e.v, e.th, e.qv, e.qr, e.qs, e.qi, e.isenT, e.isenQv, e.p, e.Pg, dtS, dbg);
}
void launch_init_density(Env& e) {
    ProfScope ps(e, "eos");
    e.launches += 1;
    k_init_density<<<cell_grid(e.g), dim3(BX, BY), 0, e.stream>>>(e.g, e.rho, e.th, e.p, e.qv, e.Pg);
}
void launch_new_pressure(Env& e) {
    ProfScope ps(e, "eos");
    e.launches += 1;
    k_new_pressure<<<cell_grid(e.g), dim3(BX, BY), 0, e.stream>>>(e.g, e.p, e.rho, e.th, e.qv, e.Pg);
}

// ---------------------------------------------------------------------------------------------
// Allocation-free diffusion of one caller-owned field.
//
// For callers that must not allocate device memory themselves: code running inside a host
// framework that owns a fixed device memory pool and forbids outside allocations, or code on a
// path where a cudaMalloc would synchronise the device or fail (for instance while a real-time
// loop is running). Such callers pass their own input and output buffers; the one intermediate
// buffer the sweeps need lives in the file-scope array below, reserved when the library loads
// and held on every GPU that loads it until the process exits.
// ---------------------------------------------------------------------------------------------

namespace {

constexpr unsigned kNoAllocMaxCells = 1u << 21;  // 2,097,152 cells: 8 MiB of scratch

// Shared by every call on a device: it keeps the last call's contents. Nothing in it needs to
// start at zero, because each sweep writes every sky cell before the next sweep reads it and
// ground cells are never read. Calls whose work overlaps on the GPU race on it.
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocMaxCells];

// The array's device address, looked up once per CUDA context. A context, not a device number,
// is the key: a host framework may make its own driver-API context current on a device, and after
// cudaDeviceReset the device's next primary context is a new one. Contexts are told apart by
// cuCtxGetId (unique for the life of the process), reached through the runtime's driver entry
// points so that the library needs no link against libcuda.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
struct NoAllocSlot {
    unsigned long long ctx_id;
    float* ptr;
};
constexpr int kNoAllocMaxContexts = 64;
std::mutex g_noalloc_mu;
NoAllocSlot g_noalloc_slots[kNoAllocMaxContexts];
int g_noalloc_nslots = 0;

bool current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return false;
        get_current = (CtxGetCurrentFn)f1;
        get_id = (CtxGetIdFn)f2;
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

// The scratch array's address in the current context (looked up on the first call there).
// Returns nullptr with the error text set when no context can be made current.
float* noalloc_scratch_address(std::string& err) {
    unsigned long long id = 0;
    if (!current_context_id(&id)) {
        // no context is current yet: the runtime makes the current device's primary context
        // current on its first call that needs one, which the lookup below is
        float* probe = nullptr;
        const cudaError_t e0 = cudaGetSymbolAddress((void**)&probe, g_noalloc_scratch);
        if (e0 != cudaSuccess || !current_context_id(&id)) {
            err = e0 != cudaSuccess ? cudaGetErrorString(e0) : "no current CUDA context";
            return nullptr;
        }
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    for (int i = 0; i < g_noalloc_nslots; ++i)
        if (g_noalloc_slots[i].ctx_id == id) return g_noalloc_slots[i].ptr;
    float* ptr = nullptr;
    const cudaError_t e1 = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e1 != cudaSuccess || !ptr) {
        err = e1 != cudaSuccess ? cudaGetErrorString(e1) : "null symbol address";
        return nullptr;
    }
    // the table keeps the most recent contexts: a full table drops its oldest entry
    if (g_noalloc_nslots == kNoAllocMaxContexts) {
        for (int i = 1; i < kNoAllocMaxContexts; ++i) g_noalloc_slots[i - 1] = g_noalloc_slots[i];
        --g_noalloc_nslots;
    }
    g_noalloc_slots[g_noalloc_nslots++] = NoAllocSlot{id, ptr};
    return ptr;
}

__global__ void k_copy_all(const float* __restrict__ src, float* __restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

}  // namespace

void set_global_error(const char* msg);  // skt_last_error(NULL) text, defined in skt_api.cu

extern "C" skt_status skt_diffuse_noalloc(int nx, int ny, int nz, float voxel, int field_type, float dt_speed, int sweeps,
                                          const float* in_dev, float* out_dev, const int32_t* ground_height_dev,
                                          const float* default_column_dev, const float* p_dev, const float* ground_T_dev,
                                          const float* ground_p_dev, void* stream) {
    const long long n = (long long)nx * ny * nz;
    if (nx < 1 || ny < 2 || nz < 1 || !(voxel > 0.0f) || sweeps < 0 || field_type < 0 || field_type > 5) {
        set_global_error("skt_diffuse_noalloc: invalid grid, sweep count or field type");
        return SKT_INVALID_ARG;
    }
    if (n > (long long)kNoAllocMaxCells) {
        set_global_error("skt_diffuse_noalloc: nx*ny*nz exceeds SKT_NOALLOC_MAX_CELLS (2097152 cells); "
                         "diffuse larger grids through skt_create/skt_step");
        return SKT_INVALID_ARG;
    }
    if (nz > 65535 || (ny + BY - 1) / BY > 65535) {  // the launch grid's y and z limits
        set_global_error("skt_diffuse_noalloc: nz must be <= 65535 and ny <= 524280 (CUDA grid limits)");
        return SKT_INVALID_ARG;
    }
    if (!in_dev || !out_dev || !ground_height_dev || in_dev == out_dev) {
        set_global_error("skt_diffuse_noalloc: null or aliased input/output buffer");
        return SKT_INVALID_ARG;
    }
    if ((field_type == 0 && (!default_column_dev || !p_dev || !ground_T_dev || !ground_p_dev)) ||
        ((field_type == 1 || field_type == 2 || field_type == 4) && !default_column_dev)) {
        set_global_error("skt_diffuse_noalloc: this field type needs its default column (and, for theta, p/ground T/ground p)");
        return SKT_INVALID_ARG;
    }
    // Set-up, once per CUDA context and with it current: the address of the array. In host code
    // its name only stands in for the device symbol, so the kernels get this pointer.
    std::string err_text;
    float* scratch = noalloc_scratch_address(err_text);
    if (!scratch) {
        set_global_error(("skt_diffuse_noalloc: " + err_text).c_str());
        return SKT_CUDA_ERROR;
    }
    Grid g;
    g.X = nx; g.Y = ny; g.Z = nz; g.XY = nx * ny; g.N = int(n); g.gh = ground_height_dev; g.vox = voxel;
    int sides = NEUMANN, ground = DIRICHLET;
    const float* def = default_column_dev;
    switch (field_type) {  // diffuseGPU's boundary table, Game/environment.cu:603-638
        case 0: sides = CUSTOM; ground = CUSTOM; break;
        case 1: sides = CUSTOM; ground = DIRICHLET; break;
        case 2: sides = CUSTOM; break;
        case 3: def = nullptr; break;
        case 4: sides = CUSTOM; break;
        default: break;  // NEUMANN sides, DIRICHLET ground, custom column unused
    }
    cudaStream_t st = (cudaStream_t)stream;
    const float k = 0.005f * dt_speed / (voxel * voxel);
    // out takes the input first so its ground cells keep their values; the sweeps then alternate
    // between out and the scratch array so that the last one lands in out.
    k_copy_all<<<(int(n) + 255) / 256, 256, 0, st>>>(in_dev, out_dev, int(n));
    const float* src = in_dev;
    for (int s = 0; s < sweeps; ++s) {
        float* dst = ((sweeps - 1 - s) % 2 == 0) ? out_dev : scratch;
        if (field_type == 0)
            k_diffuse<true><<<cell_grid(g), dim3(BX, BY), 0, st>>>(g, src, dst, sides, ground, def, k, p_dev, ground_T_dev, ground_p_dev);
        else
            k_diffuse<false><<<cell_grid(g), dim3(BX, BY), 0, st>>>(g, src, dst, sides, ground, def, k, p_dev, ground_T_dev, ground_p_dev);
        src = dst;
    }
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_global_error(cudaGetErrorString(err));
        return SKT_CUDA_ERROR;
    }
    return SKT_OK;
}

}  // namespace skt
