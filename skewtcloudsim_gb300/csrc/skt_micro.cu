// Bulk six-species microphysics fused with its latent heating, the ground/surface column
// kernels, and the state initialisation kernels.
#include "skt_internal.cuh"

namespace skt {

namespace {

constexpr int BX = 32, BY = 8;

// the selection box of the region-summed process amounts (inclusive, reference layout x, y, z)
struct RateBox {
    int lo[3], hi[3];
};
constexpr int kRates = 33;

// Region sums of the data graph (Game/microPhysics.cu:1356-1413): each block adds its cells'
// 33 values (registers -> warp shuffles -> shared memory) and one thread per value adds the block
// total to an FP64 accumulator; only blocks that meet the box take part.
__device__ __forceinline__ void add_rates(const float (&v)[kRates], bool inside, bool block_meets, double* rates) {
    if (!block_meets) return;
    __shared__ float part[BX * BY / 32][kRates];
    const int tid = threadIdx.x + BX * threadIdx.y, warp = tid >> 5, lane = tid & 31;
#pragma unroll
    for (int k = 0; k < kRates; ++k) {
        float a = inside ? v[k] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) part[warp][k] = a;
    }
    __syncthreads();
    if (tid < kRates) {
        double t = 0.0;
        for (int w = 0; w < BX * BY / 32; ++w) t += double(part[w][tid]);
        atomicAdd(rates + tid, t);
    }
}

// calculateEnvMicroPhysicsGPU (Game/microPhysics.cu:1035-1354) + addHeatGPU
// (Game/kernelSky.cu:1249-1282) in one pass: the condensation/deposition/freezing sums stay in
// registers instead of three global arrays. RATES: also the region-summed process amounts.
template <bool RATES>
__global__ void __launch_bounds__(256) k_micro(Grid g, float* __restrict__ qv_, float* __restrict__ qw_, float* __restrict__ qc_,
                                               float* __restrict__ qr_, float* __restrict__ qs_, float* __restrict__ qi_,
                                               float* __restrict__ th, const float* __restrict__ rho, const float* __restrict__ p,
                                               const float* __restrict__ Pg, float dt, float speed, Micro M, RateBox rb, double* rates) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    bool live = x < g.X && y < g.Y && !is_ground(g, x, y, z);
    if (!RATES && !live) return;
    bool block_meets = false;
    if (RATES) {
        const int bx0 = blockIdx.x * BX, by0 = blockIdx.y * BY;
        block_meets = bx0 <= rb.hi[0] && bx0 + BX - 1 >= rb.lo[0] && by0 <= rb.hi[1] && by0 + BY - 1 >= rb.lo[1] && z >= rb.lo[2] && z <= rb.hi[2];
        if (!live) {
            float zero[kRates] = {0};
            add_rates(zero, false, block_meets, rates);
            return;
        }
    }
    const int c = cidx(g, x, y, z);
    const float lo = 1e-18f;
    const float Qv = qv_[c] > lo ? qv_[c] : 0.0f, Qw = qw_[c] > lo ? qw_[c] : 0.0f;
    const float Qc = qc_[c] > lo ? qc_[c] : 0.0f, Qr = qr_[c] > lo ? qr_[c] : 0.0f;
    const float Qs = qs_[c] > lo ? qs_[c] : 0.0f, Qi = qi_[c] > lo ? qi_[c] : 0.0f;
    const float QwMin = 0.001f, QcMin = 0.001f, QiMin = 0.0006f;
    const float ps = p[c];
    float UR = 0.0f, US = 0.0f, UI = 0.0f;
    const float D = rho[c];
    const float thc = th[c];
    const float tK = thc * powf(ps / Pg[x + z * g.X], KC::KAPPA);
    const float t = tK - 273.15f;
    if (Qr > 0.0f || Qs > 0.0f || Qi > 0.0f) fallingVelocity(Qr, Qs, Qi, D, 3, M.G.Qr, M.G.Qs, M.G.Qi, UR, US, UI);
    const float QWS = ws(t, ps), QWI = wi(t, ps);
    const float PT1 = (t < 0.0f && Qw + Qc > 0 + 1e-6f) ? 1.0f : 0.0f;
    const float PT2 = (t < 0.0f && Qr < 1e-4f && Qs < 1e-4f) ? 1.0f : 0.0f;
    const float PT3 = (t < 0.0f && Qr < 1e-4f) ? 1.0f : 0.0f;
    const float sR = slopePrecip(D, Qr, 0), sS = slopePrecip(D, Qs, 1), sI = slopePrecip(D, Qi, 2);
    const float dtS = dt * speed;
    float PVCON = M.FPVCON(t, ps, Qv, QWS, dt, speed);
    float PVDEP = M.FPVDEP(t, ps, Qv, QWI, dt, speed);
    PVDEP = fminf(PVDEP, 0.0f);
    float PIMLT = M.FPIMLT(t, Qc);
    float PIDW = M.FPIDW(dt, t, Qc, Qw, D, ps);
    float PIHOM = M.FPIHOM(t, Qw);
    float PIACR = M.FPIACR(Qr, Qc, D, sR);
    float PRACI = M.FPRACI(Qr, Qc, D, sR);
    float PRAUT = M.FPRAUT(Qw, QwMin, t);
    float PRACW = M.FPRACW(Qr, Qw, D, sR);
    float PREVP = M.FPREVP(t, Qr, Qv, QWS, D, ps, sR, PT1);
    float PRACS = M.FPRACS(Qr, Qs, PT2, UR, US, D, sS, sR);
    float PSACW = M.FPSACW(Qs, Qw, D, sS);
    float PSACR = M.FPSACR(Qr, Qs, UR, US, D, sR, sS);
    float PSACI = M.FPSACI(t, Qs, Qc, D, sS);
    float PSAUT = M.FPSAUT(t, Qc, QcMin);
    float PSFW = M.FPSFW(dt, t, ps, Qs, Qw, Qc, Qv, QWI, D);
    float PSFI = M.FPSFI(dt, t, ps, Qs, Qw, Qc, Qv, QWI, D);
    float PSDEP = M.FPSDEP(t, ps, Qv, QWI, D, sS);
    float PSSUB = M.FPSSUB(PSDEP);
    PSDEP = fmaxf(0.0f, PSDEP);
    float PSMLT = M.FPSMLT(t, ps, Qw, Qr, Qs, Qv, D, sS, PSACW, PSACR, dtS);
    float PGAUT = M.FPGAUT(t, Qs, QiMin);
    float PGFR = M.FPGFR(t, Qr, D, sR);
    float PGACW = M.FPGACW(Qi, Qw, sI, D);
    float PGACI = M.FPGACI(Qi, Qc, sI, D);
    float PGACR = M.FPGACR(Qi, Qr, D, UR, UI, sR, sI);
    float PGACS = M.FPGACS(t, Qs, Qi, D, US, UI, sS, sI, false);
    float PGSUB = M.FPGSUB(t, ps, Qv, QWI, Qi, D, sI);
    float PGMLT = M.FPGMLT(t, ps, Qw, Qr, Qi, Qv, D, sI, PGACW, PGACR, dtS);
    float PGDRY = M.FPGDRY(Qw, Qc, Qr, Qs, PGACW, PGACI, PGACR, PGACS, dtS);
    float PGWET = M.FPGWET(t, ps, Qc, Qs, Qi, Qv, US, UI, D, sS, sI, PGACI, PGACS, dtS);
    float PGACR1 = M.FPGACR1(t, Qw, Qc, Qs, Qi, D, US, UI, sS, sI, PGWET, PGACW, PGACI, PGACS, dtS);
    const float WT = PGDRY > PGWET ? 1.0f : 0.0f;
    float condens = 0.0f, depos = 0.0f, freeze = 0.0f;
    auto lim = [&](float cap, float rate) { return dt * fminf(cap, speed * rate); };
    if (t < 0.0f) {
        if (PVCON >= 0) condens += PVCON = lim(Qv, PVCON);
        else if (PVCON < 0) condens += PVCON = dt * fmaxf(-Qw, speed * PVCON);
        if (PVDEP >= 0) depos += PVDEP = lim(Qv, PVDEP);
        else if (PVDEP < 0) depos += PVDEP = dt * fmaxf(-Qc, speed * PVDEP);
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
        if (WT == 1.0f) {
            if (PGACR1 >= 0) freeze += PGACR1 = lim(Qr, PGACR1);
            else if (PGACR1 < 0) freeze += PGACR1 = dt * fmaxf(-Qi, speed * PGACR1);
        }
    } else {
        if (PVCON >= 0) condens += PVCON = lim(Qv, PVCON);
        else if (PVCON < 0) condens += PVCON = dt * fmaxf(-Qw, speed * PVCON);
        if (PVDEP >= 0) depos += PVDEP = lim(Qv, PVDEP);
        else if (PVDEP < 0) depos += PVDEP = dt * fmaxf(-Qc, speed * PVDEP);
        freeze -= PIMLT = lim(Qc, PIMLT);
        PIACR = 0.0f;
        PRAUT = lim(Qw, PRAUT);
        PRACW = lim(Qw, PRACW);
        condens -= PREVP = lim(Qr, PREVP * (1 - PT1));
        PSACW = lim(Qw, PSACW);
        freeze -= PSMLT = lim(Qs, PSMLT);
        freeze += PGACW = lim(Qw, PGACW);
        PGACS = lim(Qs, PGACS);
        freeze -= PGMLT = lim(Qi, PGMLT);
    }
    float nqv;
    if (t < 0.0f) {
        nqv = qv_[c] + (PSSUB * (1 - PT1) + PGSUB * (1 - PT1) + PREVP * (1 - PT1) - PSDEP * (PT1) - PVCON - PVDEP);
        qw_[c] += PVCON - PSACW - PSFW - PRAUT - PRACW - PIDW - PIHOM;
        qc_[c] += PVDEP + PIDW + PIHOM - PSAUT - PSACI - PRACI - PSFI - PGACI;
        qr_[c] += PRAUT + PRACW - PIACR - PSACR - PGACR * (1 - WT) - PGACR1 * (WT) - PGFR - PREVP * (1 - PT1);
        qs_[c] += PSAUT + PSACI + PSACW + PSFW + PSFI + PRACI * (PT3) + PIACR * (PT3) - PGACS - PGAUT - PRACS * (1 - PT2) +
                  PSACR * (PT2) - PSSUB * (1 - PT1) + PSDEP * (PT1);
        qi_[c] += PGAUT + PGFR + PGDRY * (1 - WT) + PGWET * (WT) + PSACR * (1 - PT2) + PRACS * (1 - PT2) + PRACI * (1 - PT3) +
                  PIACR * (1 - PT3) - PGSUB * (1 - PT1);
    } else {
        nqv = qv_[c] + (PREVP * (1 - PT1) - PVCON - PVDEP);
        qw_[c] += PVCON + PIMLT - PRAUT - PRACW - PGACW - PSACW;
        qc_[c] += PVDEP - PIMLT;
        qr_[c] += PRAUT + PRACW + PSACW + PGACW + PGMLT + PSMLT - PREVP * (1 - PT1);
        qs_[c] += -PSMLT - PGACS;
        qi_[c] += -PGMLT + PGACS;
    }
    qv_[c] = nqv;
    if (RATES) {
        const bool inside = x >= rb.lo[0] && x <= rb.hi[0] && y >= rb.lo[1] && y <= rb.hi[1] && z >= rb.lo[2] && z <= rb.hi[2];
        const float v[kRates] = {PVCON < 0.0f ? 0.0f : PVCON, PVDEP < 0.0f ? 0.0f : PVDEP, PIMLT, PIDW, PIHOM, PIACR, PRACI, PRAUT, PRACW,
                                 PREVP, PRACS, PSACW, PSACR, PSACI, PSAUT, PSFW, PSFI, PSDEP, PSSUB, PSMLT, PGAUT, PGFR, PGACW, PGACI,
                                 PGACR, PGDRY * (1 - WT), PGACS, PGSUB, PGMLT, PGWET * WT, PGACR1, PVCON < 0.0f ? -PVCON : 0.0f,
                                 PVDEP < 0.0f ? -PVDEP : 0.0f};
        add_rates(v, inside, block_meets, rates);
    }
    // latent heat with the updated vapour (addHeatGPU)
    const float Mair = 0.02896f, Mwat = 0.01802f;
    const float XV = (nqv / Mwat) / ((nqv / Mwat) + (1 - nqv) / Mair);
    const float Mth = XV * Mwat + (1 - XV) * Mair;
    const float YV = XV * (Mwat / Mth);
    const float yth = YV * 1.33f + (1 - YV) * 1.4f;
    const float cpth = yth * KC::R / (Mth * (yth - 1));
    float sum = 0.0f;
    sum += Lwater(thc - 273.15f) / cpth * condens;
    sum += Lice(thc - 273.15f) / cpth * depos;
    sum += KC::Lf / cpth * freeze;
    th[c] = thc + sum;
}

// advectGroundWaterGPU Game/kernelSky.cu:120-253 on the X*Z ground grid (old values in rs/gr).
// Neighbours are the neighbouring columns; the reference's unfilled tile halos are not copied.
__global__ void k_ground_water(Grid g, const float* __restrict__ rs, const float* __restrict__ gr, float* __restrict__ Qrs, float* __restrict__ Qgr,
                               float dt, float speed) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.X * g.Z) return;
    const int x = idx % g.X, z = idx / g.X;
    const int iL = x == 0 ? idx : idx - 1, iR = x == g.X - 1 ? idx : idx + 1;
    const int iB = z == 0 ? idx : idx - g.X, iF = z == g.Z - 1 ? idx : idx + g.X;
    const float rsC = rs[idx], grC = gr[idx];
    float fGr = grC, fRs = rsC;
    const float vox = g.vox;
    auto flow = [&](float hFrom, float hTo, float grFrom, float grTo, float rsFrom, float rsTo) {
        const float n = 1 / 0.03f;
        const float kk = 5e-5f;
        const float slope = hFrom - hTo / 1.0f;
        const bool fromPrev = slope > 0.0f;
        const float sRain = fromPrev ? grFrom : grTo;
        const float sWat = fromPrev ? rsFrom : rsTo;
        float changeRain = 0.0f;
        if (sRain != 0.0f) {
            const float spd = n * powf(sRain, 2.0f / 3.0f);
            const float vel = spd * powf(slope, 0.5f);
            changeRain = vel * sRain;
        }
        const float changeWater = KC::g * kk * sWat * slope;
        const float dR = 1 / (vox * vox) * 1.75e-3f, dW = 1 / (vox * vox) * 1.8e-5f;
        const float lapR = (grFrom - grTo) * dR, lapSR = (rsFrom - rsTo) * dW;
        const bool pR = lapR > 0.0f, pSR = lapSR > 0.0f;
        const float fgR = dt * fminf(fabsf(lapR) * speed, pR ? grFrom : grTo) * (lapR > 0.0f ? 1.0f : -1.0f);
        const float fgW = dt * fminf(fabsf(lapSR) * speed, pSR ? rsFrom : rsTo) * (lapSR > 0.0f ? 1.0f : -1.0f);
        const float sfR = dt * fminf(fabsf(changeRain) * speed, fromPrev ? grFrom : grTo) * (changeRain > 0.0f ? 1.0f : -1.0f);
        const float sfW = dt * fminf(fabsf(changeWater) * speed, fromPrev ? rsFrom : rsTo) * (changeWater > 0.0f ? 1.0f : -1.0f);
        fGr += fgR + sfR;
        fRs += fgW + sfW;
    };
    const float hC = float(g.gh[idx]);
    flow(float(g.gh[iL]), hC, gr[iL], grC, rs[iL], rsC);
    flow(float(g.gh[iR]), hC, gr[iR], grC, rs[iR], rsC);
    flow(float(g.gh[iB]), hC, gr[iB], grC, rs[iB], rsC);
    flow(float(g.gh[iF]), hC, gr[iF], grC, rs[iF], rsC);
    Qgr[idx] = fGr;
    Qrs[idx] = fRs;
}

struct GroundPtrs {
    float *qv, *qw, *qc, *qr, *qs, *qi, *th, *rho, *p, *u;
    float *Qrs, *Qgr, *Qgs, *Qgi, *Pg, *tg, *Tg, *cover;
};

// One thread per ground column: cloud cover (calculateCloudCoverGPU :1034), ground temperature
// (calculateGroundTempGPU :1046), precipitation reaching the ground
// (calculatePrecipHittingGroundMicroPhysicsGPU Game/microPhysics.cu:1544), ground
// microphysics (calculateGroundMicroPhysicsGPU :1419) and the relaxation of the first sky cell
// towards the ground potential temperature (setTempsAtGroundGPU Game/kernelSky.cu:255).
// irr_dev: in graph mode the irradiance is read from device memory (the graph's first node writes
// it); otherwise irr is used
__global__ void k_ground_column(Grid g, GroundPtrs P, float dt, float speed, float irr_arg, const float* __restrict__ irr_dev, Micro M) {
    const int idxG = blockIdx.x * blockDim.x + threadIdx.x;
    if (idxG >= g.X * g.Z) return;
    const float irr = irr_dev ? *irr_dev : irr_arg;
    const int x = idxG % g.X, z = idxG / g.X;
    const int gh = g.gh[idxG];
    const float vox = g.vox;
    const float lo = 1e-18f;
    // cloud cover
    float tot = 0.0f;
    for (int y = gh + 1; y < g.Y; ++y) {
        const int c = cidx(g, x, y, z);
        tot += (P.qc[c] + P.qw[c]) * vox;
    }
    const float cov = fminf(tot / 1.2f, 1.0f);
    P.cover[idxG] = cov;
    // ground temperature, T^4 in FP32 then the balance in FP64 as the reference's double T4
    {
        const float gT = P.Tg[idxG];
        const double T4 = double(gT * gT * gT * gT);
        const float dtS = dt * speed;
        P.Tg[idxG] = float(double(gT) + double(dtS) * (double(1 - cov) * ((double((1 - 0.25f) * irr) - double(KC::ge * KC::oo) * T4) /
                                                                         double(1.0f * 1500.0f * KC::Cpds))));
    }
    if (gh + 1 >= g.Y) return;
    const int c = cidx(g, x, gh + 1, z);
    const float Pgc = P.Pg[idxG];
    // precipitation hitting the ground
    {
        const float Qgr = P.Qgr[idxG] > lo ? P.Qgr[idxG] : 0.0f, Qgs = P.Qgs[idxG] > lo ? P.Qgs[idxG] : 0.0f;
        const float Qgi = P.Qgi[idxG] > lo ? P.Qgi[idxG] : 0.0f;
        const float Qv = P.qv[c] > lo ? P.qv[c] : 0.0f, Qr = P.qr[c] > lo ? P.qr[c] : 0.0f;
        const float Qs = P.qs[c] > lo ? P.qs[c] : 0.0f, Qi = P.qi[c] > lo ? P.qi[c] : 0.0f;
        float freeze = 0.0f;
        const float tgC = P.Tg[idxG] - 273.15f;
        const float ps = P.p[c], wind = P.u[c], D = P.rho[c];
        const float taK = P.th[c] * powf(ps / Pgc, KC::KAPPA);
        float UR = 0.0f, US = 0.0f, UI = 0.0f;
        if (Qgr > 0.0f || Qgs > 0.0f || Qgi > 0.0f) fallingVelocity(Qgr, Qgs, Qgi, D, 3, M.G.Qr, M.G.Qs, M.G.Qi, UR, US, UI);
        const float GR = dt * fminf(Qr * speed, Qr), GS = dt * fminf(Qs * speed, Qs), GI = dt * fminf(Qi * speed, Qi);
        float PGRFR = M.FPGRFR(taK, tgC, ps, Qr, Qv, Qi, Qgr, Qgs, D, wind, UR);
        if (taK < 273.15f) freeze += PGRFR = dt * fminf(Qr, speed * PGRFR);
        P.qr[c] += -GR;
        P.qs[c] += -GS;
        P.qi[c] += -GI;
        P.Qgr[idxG] += GR - PGRFR;
        P.Qgs[idxG] += GS;
        P.Qgi[idxG] += GI + PGRFR;
        const float Mair = 0.02896f, Mwat = 0.01802f;
        const float XV = (Qv / Mwat) / ((Qv / Mwat) + (1 - Qv) / Mair);
        const float Mth = XV * Mwat + (1 - XV) * Mair;
        const float YV = XV * (Mwat / Mth);
        const float yth = YV * 1.33f + (1 - YV) * 1.4f;
        const float cpth = KC::R / (Mth * (yth - 1));
        float sum = 0.0f;
        sum += KC::Lf / cpth * freeze;
        P.Tg[idxG] += sum;
    }
    // ground microphysics
    {
        const float Qrs = P.Qrs[idxG] > lo ? P.Qrs[idxG] : 0.0f, Qgr = P.Qgr[idxG] > lo ? P.Qgr[idxG] : 0.0f;
        const float Qgs = P.Qgs[idxG] > lo ? P.Qgs[idxG] : 0.0f, Qgi = P.Qgi[idxG] > lo ? P.Qgi[idxG] : 0.0f;
        const float Qv = P.qv[c] > lo ? P.qv[c] : 0.0f;
        float condens = 0.0f, freeze = 0.0f, depos = 0.0f;
        const float tgC = P.Tg[idxG] - 273.15f;
        const float ps = P.p[c], wind = P.u[c], D = P.rho[c];
        float tim = P.tg[idxG];
        const float taK = P.th[c] * powf(ps / Pgc, KC::KAPPA);
        const float sI = slopePrecip(D, Qgi, 2);
        float PGREVP = M.FPGREVP(taK, tgC, ps, Qv, Qgr, irr, D, wind);
        float PGSMLT = M.FPGSMLT(taK, tgC, ps, Qgs, Qv, Qgr, irr, cov, D, wind, dt);
        float PGGMLT = M.FPGGMLT(tgC, Qgi, D, sI);
        float PGGFR = M.FPGGFR(taK, tgC, ps, Qgr, Qv, Qgi, D, irr, cov, wind, dt);
        float PGSFR = M.FPGSFR(taK, tgC, ps, Qv, Qgr, Qgs, D, wind, dt);
        float PGFLW = M.FPGFLW(Qgr);
        float PGDEVP = M.FPGDEVP(tim, Qgr, Qgs, Qgi, Qrs);
        condens -= PGREVP = dt * fminf(Qgr, speed * PGREVP);
        freeze -= PGSMLT = dt * fminf(Qgs, speed * PGSMLT);
        freeze -= PGGMLT = dt * fminf(Qgi, speed * PGGMLT);
        freeze += PGGFR = dt * fminf(Qgr, speed * PGGFR);
        freeze += PGSFR = dt * fminf(Qgr, speed * PGSFR);
        PGFLW = dt * fminf(Qgr, speed * PGFLW);
        condens -= PGDEVP = dt * fminf(Qrs, speed * PGDEVP);
        P.tg[idxG] = tim;
        P.Qrs[idxG] += PGFLW - PGDEVP;
        P.qv[c] += PGREVP + PGDEVP;
        P.Qgr[idxG] += PGSMLT + PGGMLT - PGREVP - PGGFR - PGSFR - PGFLW;
        P.Qgs[idxG] += PGSFR - PGSMLT;
        P.Qgi[idxG] += PGGFR - PGGMLT;
        const float mass = 1500.0f * 0.1f;
        float sum = 0.0f;
        sum += Lwater(tgC) / (mass * 1500.0f) * condens;
        sum += Lice(tgC) / (mass * 1500.0f) * depos;
        sum += KC::Lf / (mass * 1500.0f) * freeze;
        P.Tg[idxG] += sum;
    }
    // setTempsAtGroundGPU (skipped for columns whose first sky cell is the top level)
    if (gh + 1 >= g.Y - 1) return;
    {
        const float Tt = potentialTemp(P.Tg[idxG] - 273.15f, P.p[c], Pgc) + 273.15f;
        const float dif2 = P.th[c] - Tt;
        P.th[c] -= dif2 * fminf(1.0f, dt * speed);
    }
}

// ---- initialisation (environmentGPU::init Game/environment.cu:249-389) ----------------------
__global__ void k_columns(Grid g, const float* th, const float* qv, const float* u, const float* w, float* isenT, float* isenQv, float* defU,
                          float* defW, float* zeroY) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= g.Y) return;
    const int c = y * g.X;  // column x = 0, z = 0 (:299-303)
    isenT[y] = th[c];
    isenQv[y] = qv[c];
    defU[y] = u[c];
    defW[y] = w[c];
    zeroY[y] = 0.0f;
}

__device__ __forceinline__ unsigned pcg_hash(unsigned seed) {  // randomCuda Game/kernelMaths.cu:93
    const unsigned st = seed * 747796405u + 2891336453u;
    const unsigned w = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
    return (w >> 22u) ^ w;
}

// randomArray (Game/kernelMaths.cu:100-116) with every thread seeing the new seed, then
// resetValueInGround of the ten prognostic fields (Game/kernelGround.cu:21-36)
__global__ void k_noise_ground(Grid g, float* th, float* qv, float* qw, float* qc, float* qr, float* qs, float* qi, float* u, float* v, float* w,
                               int noise, unsigned seed_base) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= g.X || y >= g.Y) return;
    const int c = cidx(g, x, y, z);
    if (noise) {
        auto add = [&](float* a, float mn, float mx, unsigned seed) {
            const float rnd = float(pcg_hash(seed + unsigned(c)) % 1000u) / float(1000);
            a[c] += rnd * (mx - mn) + mn;
        };
        add(th, -0.1f, 0.1f, seed_base + 0);
        add(qv, 0.0f, 0.0001f, seed_base + 1);
        add(u, 0.5f, 0.5f, seed_base + 2);
        add(v, -0.2f, 0.2f, seed_base + 3);
        add(w, 0.5f, 0.5f, seed_base + 4);
    }
    if (is_ground(g, x, y, z)) {
        th[c] = qv[c] = qw[c] = qc[c] = qr[c] = qs[c] = qi[c] = u[c] = v[c] = w[c] = 0.0f;
    }
}

// computeIsenTempGroundGPU Game/kernelGround.cu:38-47
__global__ void k_isen_ground(Grid g, float* Tg, const float* isenT, const float* Pg, const float* p) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.X * g.Z) return;
    const int x = idx % g.X, z = idx / g.X;
    const int GH = g.gh[idx] + 1 >= g.Y ? g.Y - 1 : g.gh[idx] + 1;
    const float T = potentialTemp(isenT[GH - 1] - 273.15f, Pg[idx], p[cidx(g, x, GH, z)]);
    Tg[idx] = T + 273.15f;
}

}  // namespace

void launch_micro(Env& e, float dt, float speed) {
    const Grid& g = e.g;
    Micro M;
    M.G = e.gam;
    ProfScope ps(e, "micro");
    e.launches += 1;
    const dim3 grid((g.X + BX - 1) / BX, (g.Y + BY - 1) / BY, g.Z), blk(BX, BY);
    if (e.rates_on) {
        RateBox rb{{e.rate_lo[0], e.rate_lo[1], e.rate_lo[2]}, {e.rate_hi[0], e.rate_hi[1], e.rate_hi[2]}};
        cudaMemsetAsync(e.rates_dev, 0, sizeof(double) * kRates, e.stream);
        k_micro<true><<<grid, blk, 0, e.stream>>>(g, e.qv, e.qw, e.qc, e.qr, e.qs, e.qi, e.th, e.rho, e.p, e.Pg, dt, speed, M, rb, e.rates_dev);
    } else {
        k_micro<false><<<grid, blk, 0, e.stream>>>(g, e.qv, e.qw, e.qc, e.qr, e.qs, e.qi, e.th, e.rho, e.p, e.Pg, dt, speed, M, RateBox{},
                                                   nullptr);
    }
}

void launch_ground(Env& e, float dt, float speed, float irr) {
    const Grid& g = e.g;
    const int n2 = g.X * g.Z;
    ProfScope ps(e, "ground");
    e.launches += 2;
    cudaMemcpyAsync(e.g2a, e.Qrs, sizeof(float) * n2, cudaMemcpyDeviceToDevice, e.stream);
    cudaMemcpyAsync(e.g2b, e.Qgr, sizeof(float) * n2, cudaMemcpyDeviceToDevice, e.stream);
    k_ground_water<<<(n2 + 127) / 128, 128, 0, e.stream>>>(g, e.g2a, e.g2b, e.Qrs, e.Qgr, dt, speed);
    GroundPtrs P{e.qv, e.qw, e.qc, e.qr, e.qs, e.qi, e.th, e.rho, e.p, e.u, e.Qrs, e.Qgr, e.Qgs, e.Qgi, e.Pg, e.tg, e.Tg, e.cover};
    Micro M;
    M.G = e.gam;
    k_ground_column<<<(n2 + 127) / 128, 128, 0, e.stream>>>(g, P, dt, speed, irr, e.capturing ? e.irr_dev : nullptr, M);
}

void launch_isen_ground(Env& e) {
    const Grid& g = e.g;
    k_isen_ground<<<(g.X * g.Z + 127) / 128, 128, 0, e.stream>>>(g, e.Tg, e.isenT, e.Pg, e.p);
    e.launches += 1;
}

void launch_init_state(Env& e, int noise, uint32_t seed) {
    const Grid& g = e.g;
    launch_init_density(e);
    k_columns<<<(g.Y + 127) / 128, 128, 0, e.stream>>>(g, e.th, e.qv, e.u, e.w, e.isenT, e.isenQv, e.defU, e.defW, e.zeroY);
    k_noise_ground<<<dim3((g.X + BX - 1) / BX, (g.Y + BY - 1) / BY, g.Z), dim3(BX, BY), 0, e.stream>>>(
        g, e.th, e.qv, e.qw, e.qc, e.qr, e.qs, e.qi, e.u, e.v, e.w, noise, seed);
    k_isen_ground<<<(g.X * g.Z + 127) / 128, 128, 0, e.stream>>>(g, e.Tg, e.isenT, e.Pg, e.p);
}

}  // namespace skt
