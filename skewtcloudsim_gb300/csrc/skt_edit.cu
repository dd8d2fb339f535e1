// Editing the atmosphere between steps: the brush, the box selection and the parameter reset of
// environmentGPU (prepareBrushGPU / prepareSelectionGPU / resetParameterGPU,
// Game/environment.cu:1127-1290) with their kernels (applyBrushGPU, applySelectionGPU, setGround,
// compareAndResetValuesOutGround, Game/kernelSky.cu:1476-1642; setToDefault :1714-1728;
// setToValue Game/kernelMaths.cu:12-23) and editorDataGPU's ground block
// (Game/environment.cu:989-1011).
//
// Parameters as the reference's enum (Game/config.h:62-65): 0 theta, 1 Qv .. 6 Qi, 7 wind (u, v, w
// by a direction vector), 8 ground (the heightfield), 9 pressure (reset only: the reference's
// getParamArray has no pressure array for the brush and selection, Game/environment.cu:1076-1125).
// The reference's bounds test lets z = Z through (`mZ > GRIDSIZESKYZ`) and writes one plane past
// the field; here that plane is skipped. A raise stops at row ny-2 so that every column keeps a sky
// cell (the ground kernels read the first sky cell above the ground).
#include "skt_internal.cuh"
#include "../../include/skewt.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace skt {

namespace {

struct EditArgs {
    int param;
    float value, dx, dy, dz;
    int erase;
};

struct EditFields {
    float *f, *u, *v, *w;  // f: the scalar field (param 0..6)
};

// one brushed/selected cell; amount = the value before the wind split (setGround
// Game/kernelSky.cu:1597-1611 for the ground: the new heights go to ghn)
__device__ __forceinline__ void edit_cell(const Grid& g, const EditArgs& a, const EditFields& F, int* ghn, int* changed, int x, int y, int z,
                                          float amount, bool add) {
    const int ig = x + z * g.X;
    if (a.param == 8) {
        if (a.erase && y <= g.gh[ig]) {
            atomicMin(ghn + ig, y);
            *changed = 1;
        } else if (!a.erase && y > g.gh[ig]) {
            atomicMax(ghn + ig, min(y, g.Y - 2));  // every column keeps a sky cell above its ground
            *changed = 1;
        }
        return;
    }
    const int c = cidx(g, x, y, z);
    float v1 = amount;
    if (a.param == 7) {
        const float v3 = v1 * a.dz, v2 = v1 * a.dy;
        v1 *= a.dx;
        if (add) { F.u[c] += v1; F.v[c] += v2; F.w[c] += v3; }
        else { F.u[c] = v1; F.v[c] = v2; F.w[c] = v3; }
    } else if (add) {
        F.f[c] += v1;
    } else {
        F.f[c] = v1;
    }
}

// applyBrushGPU: an n x n box in x and y (n = ceil(r) - floor(-r), offset ceil(r)) over the whole
// column range in z, value (1 - d^2/r^2)^smooth * dt * intensity * value inside the sphere
__global__ void k_brush(Grid g, EditArgs a, EditFields F, int* ghn, int* changed, float size, int px, int py, int pz, float smooth, float dt,
                        float intensity, int c, int n) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= n || y >= n) return;
    const int lX = x - c, lY = y - c, lZ = z - c;
    const int mX = x + px - c, mY = y + py - c, mZ = z + pz - c;
    if (mX >= g.X || mY >= g.Y || mZ >= g.Z || mX < 0 || mY < 0 || mZ < 0) return;
    if (a.param != 8 && mY <= g.gh[mX + mZ * g.X]) return;  // the ground is not brushed
    const float d = float(lX) * float(lX) + float(lY) * float(lY) + float(lZ) * float(lZ);
    const float r = size * size;
    if (!(d <= r)) return;
    float v = -(d / r - 1);
    v = powf(v, smooth);
    v *= dt * intensity * a.value;
    edit_cell(g, a, F, ghn, changed, mX, mY, mZ, v, true);
}

// applySelectionGPU: every cell of the box lo .. hi (nx x ny columns, z from zlo to zhi) set
__global__ void k_select(Grid g, EditArgs a, EditFields F, int* ghn, int* changed, int lx, int ly, int nx, int ny, int zlo) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = zlo + int(blockIdx.z);
    if (x >= nx || y >= ny) return;
    const int mX = x + lx, mY = y + ly, mZ = z;
    if (mX >= g.X || mY >= g.Y || mZ >= g.Z || mX < 0 || mY < 0 || mZ < 0) return;
    if (a.param != 8 && mY <= g.gh[mX + mZ * g.X]) return;
    edit_cell(g, a, F, ghn, changed, mX, mY, mZ, a.value, false);
}

// compareAndResetValuesOutGround: cells the erase freed (new height < y <= old height) take the
// default columns
__global__ void k_compare_reset(Grid g, const int* __restrict__ ghOld, const int* __restrict__ ghNew, const float* __restrict__ isenT,
                                const float* __restrict__ isenQv, const float* __restrict__ pcol, float* qv, float* qw, float* qc, float* qr,
                                float* qs, float* qi, float* th, float* u, float* v, float* w, float* p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    const int ig = x + z * g.X;
    if (y > ghOld[ig] || y <= ghNew[ig]) return;
    const int c = cidx(g, x, y, z);
    qv[c] = isenQv[y];
    qw[c] = 0.0f; qc[c] = 0.0f; qr[c] = 0.0f; qs[c] = 0.0f; qi[c] = 0.0f;
    th[c] = isenT[y];
    u[c] = 0.0f; v[c] = 0.0f; w[c] = 0.0f;
    p[c] = pcol[y];
}

// editorDataGPU's resetValueInGround calls (Game/kernelGround.cu:21-36): ground cells of theta,
// Qv, Qw, Qc, Qr, Qs, Qi, u and v to 0
__global__ void k_reset_in_ground(Grid g, float* th, float* qv, float* qw, float* qc, float* qr, float* qs, float* qi, float* u, float* v) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    if (!is_ground(g, x, y, z)) return;
    const int c = cidx(g, x, y, z);
    th[c] = 0.0f; qv[c] = 0.0f; qw[c] = 0.0f; qc[c] = 0.0f; qr[c] = 0.0f; qs[c] = 0.0f; qi[c] = 0.0f; u[c] = 0.0f; v[c] = 0.0f;
}

// setToDefault: one thread per (x, y) column marching z; it stops at the column's first ground
// cell (the reference returns there)
__global__ void k_set_default(Grid g, float* f, const float* __restrict__ def) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.XY) return;
    const int x = t % g.X, y = t / g.X;
    const float d = def[y];
    for (int z = 0; z < g.Z; ++z) {
        if (is_ground(g, x, y, z)) return;
        f[cidx(g, x, y, z)] = d;
    }
}

__global__ void k_set_value(int n, float* f, float value) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) f[i] = value;
}

float* edit_field(Env& e, int param) {
    float* f[7] = {e.th, e.qv, e.qw, e.qc, e.qr, e.qs, e.qi};
    return param >= 0 && param < 7 ? f[param] : nullptr;
}

// after the edit kernels: when the ground store changed, reset what an erase freed and take the new
// heights; then, while the ground has changed since the last step, editorDataGPU's block
int edit_finish(Env& e, int* ghn, int erase) {
    const Grid& g = e.g;
    const size_t NG = size_t(g.X) * g.Z;
    int changed = 0;
    cudaMemcpyAsync(&changed, &e.sc->edit_changed, sizeof(int), cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    const dim3 blk(32, 8), grd((g.X + 31) / 32, (g.Y + 7) / 8, g.Z);
    if (changed) {
        if (erase) {
            k_compare_reset<<<grd, blk, 0, e.stream>>>(g, e.gh, ghn, e.isenT, e.isenQv, e.pcol, e.qv, e.qw, e.qc, e.qr, e.qs, e.qi, e.th, e.u, e.v,
                                                       e.w, e.p);
            e.launches += 1;
        }
        cudaMemcpyAsync(e.gh, ghn, NG * sizeof(int), cudaMemcpyDeviceToDevice, e.stream);
        std::vector<int> h(NG);
        cudaMemcpyAsync(h.data(), e.gh, NG * sizeof(int), cudaMemcpyDeviceToHost, e.stream);
        cudaStreamSynchronize(e.stream);
        e.flat = std::all_of(h.begin(), h.end(), [](int v) { return v == 0; }) ? 1 : 0;
        e.ground_changed = 1;
    }
    if (e.ground_changed) launch_editor_block(e);
    return changed;
}

skt_status check_edit_param(Env& e, int param) {
    if (param < 0 || param > 8)
        return report(&e, SKT_INVALID_ARG, "brush/selection parameter must be 0..8 (theta, Qv..Qi, wind, ground)");
    return SKT_OK;
}

}  // namespace

// editorDataGPU's ground block (Game/environment.cu:992-1011): ground cells of theta, Qv, Qw..Qi,
// u and v to 0, the ground temperature from the isentrope
void launch_editor_block(Env& e) {
    const Grid& g = e.g;
    const dim3 blk(32, 8), grd((g.X + 31) / 32, (g.Y + 7) / 8, g.Z);
    k_reset_in_ground<<<grd, blk, 0, e.stream>>>(g, e.th, e.qv, e.qw, e.qc, e.qr, e.qs, e.qi, e.u, e.v);
    e.launches += 1;
    launch_isen_ground(e);
}

}  // namespace skt

using namespace skt;

skt_status skt_apply_brush(skt_env* env, int param, float brush_size, const int pos[3], float smoothness, float dt, float intensity,
                           float value, const float dir[3], int ground_erase, int* ground_changed) {
    if (!env || !pos) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (!e.initialized) return report(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    if (check_edit_param(e, param) != SKT_OK) return SKT_INVALID_ARG;
    if (!(brush_size >= 0.0f) || brush_size > 4096.0f) return report(&e, SKT_INVALID_ARG, "brush size must be in [0, 4096]");
    const Grid& g = e.g;
    const int c = int(std::ceil(brush_size));
    const int n = int(std::ceil(brush_size)) - int(std::floor(-brush_size));
    EditArgs a{param, value, dir ? dir[0] : 1.0f, dir ? dir[1] : 0.0f, dir ? dir[2] : 0.0f, ground_erase ? 1 : 0};
    EditFields F{edit_field(e, param), e.u, e.v, e.w};
    int* ghn = reinterpret_cast<int*>(e.g2b);  // the ground scratch holds the new heights during the edit
    cudaMemcpyAsync(ghn, e.gh, sizeof(int) * size_t(g.X) * g.Z, cudaMemcpyDeviceToDevice, e.stream);
    cudaMemsetAsync(&e.sc->edit_changed, 0, sizeof(int), e.stream);
    if (n > 0) {
        const dim3 blk(16, 16), grd((n + 15) / 16, (n + 15) / 16, g.Z);
        k_brush<<<grd, blk, 0, e.stream>>>(g, a, F, ghn, &e.sc->edit_changed, brush_size, pos[0], pos[1], pos[2], smoothness, dt, intensity,
                                           c, n);
        e.launches += 1;
    }
    const int changed = edit_finish(e, ghn, a.erase);
    if (ground_changed) *ground_changed = changed;
    return check_cuda(e, "apply_brush");
}

skt_status skt_apply_selection(skt_env* env, int param, const int lo[3], const int hi[3], float value, const float dir[3], int ground_erase,
                               int* ground_changed) {
    if (!env || !lo || !hi) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (!e.initialized) return report(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    if (check_edit_param(e, param) != SKT_OK) return SKT_INVALID_ARG;
    const Grid& g = e.g;
    // the host code turns an empty x or y extent into one cell (Game/environment.cu:1202-1207)
    const int ny = std::max(hi[1] - lo[1] + 1, 1), nx = std::max(hi[0] - lo[0] + 1, 1);
    EditArgs a{param, value, dir ? dir[0] : 1.0f, dir ? dir[1] : 0.0f, dir ? dir[2] : 0.0f, ground_erase ? 1 : 0};
    EditFields F{edit_field(e, param), e.u, e.v, e.w};
    int* ghn = reinterpret_cast<int*>(e.g2b);
    cudaMemcpyAsync(ghn, e.gh, sizeof(int) * size_t(g.X) * g.Z, cudaMemcpyDeviceToDevice, e.stream);
    cudaMemsetAsync(&e.sc->edit_changed, 0, sizeof(int), e.stream);
    // the box clipped to the grid (cells outside it are skipped by the reference's bounds test)
    const int x0 = std::max(lo[0], 0), x1 = std::min(lo[0] + nx - 1, g.X - 1);
    const int y0 = std::max(lo[1], 0), y1 = std::min(lo[1] + ny - 1, g.Y - 1);
    const int z0 = std::max(lo[2], 0), z1 = std::min(hi[2], g.Z - 1);
    if (x1 >= x0 && y1 >= y0 && z1 >= z0) {
        const int cx = x1 - x0 + 1, cy = y1 - y0 + 1;
        const dim3 blk(32, 8), grd(unsigned((cx + 31) / 32), unsigned((cy + 7) / 8), unsigned(z1 - z0 + 1));
        k_select<<<grd, blk, 0, e.stream>>>(g, a, F, ghn, &e.sc->edit_changed, x0, y0, cx, cy, z0);
        e.launches += 1;
    }
    const int changed = edit_finish(e, ghn, a.erase);
    if (ground_changed) *ground_changed = changed;
    return check_cuda(e, "apply_selection");
}

skt_status skt_reset_parameter(skt_env* env, int param) {
    if (!env) return report(nullptr, SKT_INVALID_ARG, "null env");
    Env& e = env->e;
    if (!e.initialized) return report(&e, SKT_NOT_INITIALIZED, "skt_init has not run");
    const Grid& g = e.g;
    const int nb = (g.XY + 255) / 256;
    const int nv = std::min((g.N + 255) / 256, e.num_sms * 8);
    auto to_default = [&](float* f, const float* def) { k_set_default<<<nb, 256, 0, e.stream>>>(g, f, def); ++e.launches; };
    auto to_value = [&](float* f) { k_set_value<<<nv, 256, 0, e.stream>>>(g.N, f, 0.0f); ++e.launches; };
    switch (param) {
        case SKT_POTTEMP: to_default(e.th, e.isenT); break;
        case SKT_WIND: to_default(e.u, e.defU); to_value(e.v); to_default(e.w, e.defW); break;
        case SKT_PRESSURE: to_default(e.p, e.pcol); break;
        case SKT_QV: to_default(e.qv, e.isenQv); break;
        case SKT_QW: to_value(e.qw); break;
        case SKT_QC: to_value(e.qc); break;
        case SKT_QR: to_value(e.qr); break;
        case SKT_QS: to_value(e.qs); break;
        case SKT_QI: to_value(e.qi); break;
        case SKT_PGROUND: break;  // nothing to reset (as in the reference)
        default: return report(&e, SKT_INVALID_ARG, "unknown parameter");
    }
    cudaStreamSynchronize(e.stream);
    return check_cuda(e, "reset_parameter");
}

namespace skt {
// The boundary class of each neighbour one cell away, by the rule ghost() applies: a neighbour
// outside the domain takes the class of the cell itself (ground or sky), one inside is ground
// when y <= gh. Written as the reference's Neigh record (computeNeighbourGPU,
// Game/kernelSky.cu:1284-1316; Game/config.h:24-38): left, right, up, down, forward, backward,
// each {outside, type} with type 0 = SKY, 1 = GROUND.
__global__ void k_neigh_classes(Grid g, uchar2* __restrict__ out) {
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= size_t(g.N)) return;
    const int x = int(i % g.X), y = int((i / g.X) % g.Y), z = int(i / g.XY);
    const int dx[6] = {-1, 1, 0, 0, 0, 0}, dy[6] = {0, 0, 1, -1, 0, 0}, dz[6] = {0, 0, 0, 0, 1, -1};
    const bool self_ground = is_ground(g, x, y, z);
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        const int xn = x + dx[d], yn = y + dy[d], zn = z + dz[d];
        const bool outside = !in_dom(g, xn, yn, zn);
        const bool ground = outside ? self_ground : is_ground(g, xn, yn, zn);
        out[i * 6 + d] = make_uchar2(outside ? 1 : 0, ground ? 1 : 0);
    }
}
}  // namespace skt

skt_status skt_read_neighbours(skt_env* env, uint8_t* dst, size_t n) {
    if (!env || !dst) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (n != size_t(e.g.N)) return report(&e, SKT_INVALID_ARG, "size mismatch (n is the cell count)");
    uchar2* tmp = nullptr;
    if (cudaMalloc(&tmp, n * 12) != cudaSuccess) {
        cudaGetLastError();
        return report(&e, SKT_OUT_OF_MEMORY, "neighbour record allocation failed");
    }
    k_neigh_classes<<<unsigned((n + 255) / 256), 256, 0, e.stream>>>(e.g, tmp);
    e.launches += 1;
    cudaMemcpyAsync(dst, tmp, n * 12, cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    cudaFree(tmp);
    return check_cuda(e, "read_neighbours");
}

skt_status skt_read_ground_height(skt_env* env, int32_t* dst, size_t n) {
    if (!env || !dst) return report(env ? &env->e : nullptr, SKT_INVALID_ARG, "null argument");
    Env& e = env->e;
    if (n != size_t(e.g.X) * e.g.Z) return report(&e, SKT_INVALID_ARG, "size mismatch");
    cudaMemcpyAsync(dst, e.gh, n * sizeof(int32_t), cudaMemcpyDeviceToHost, e.stream);
    cudaStreamSynchronize(e.stream);
    return check_cuda(e, "read_ground_height");
}
