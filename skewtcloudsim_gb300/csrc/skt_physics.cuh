// Device thermodynamics and bulk microphysics of the atmosphere step (FP32).
//
// Restates Game/meteoformulas.cuh (saturation, latent heats, diffusivity, fall speeds, moist
// lapse rate) and the process rates of Game/microPhysics.cu:67-1032 with CUDA's powf/expf/logf,
// exactly the functions the reference calls, so the per-cell arithmetic is the reference's.
// Physical constants: Game/environment.cu:28-60.
#pragma once
#include <cuda_runtime.h>

namespace skt {

namespace KC {
constexpr float g = 9.8076f, Hv = 2501000.0f, R = 8.3145f, Rsd = 287.0528f, Rsw = 461.5f;
constexpr float Cpd = 1003.5f, Cvl = 4119.0f, Cpi = 2093.0f, Cpds = 800.0f, Mw = 18.02f;
constexpr float E0v = 2.374e+6f, Lf = 3.3355e+5f, Ls = 2.834e+6f, Ka = 2.40e-2f;
constexpr float PI = 3.14159265359f, oo = 5.67e-8f, ge = 0.95f;
constexpr float E = 287.0528f / 461.5f;      // Rsd / Rsw
constexpr float KAPPA = 287.0528f / 1003.5f; // Rsd / Cpd
}  // namespace KC

// ---- Game/meteoformulas.cuh ---------------------------------------------------------------
__device__ __forceinline__ float es(float t) { return 0.61078f * expf((17.27f * t) / (t + 237.3f)); }        // :16
__device__ __forceinline__ float ei(float t) { return 0.61078f * expf((21.875f * t) / (t + 265.5f)); }       // :27
__device__ __forceinline__ float ws(float t, float p) { float e = es(t) * 10.0f; return (KC::E * e) / (p - e); }          // :41
__device__ __forceinline__ float wi(float t, float p) { float e = ei(t) * 10.0f; return (KC::E * e) / (p - e); }          // :52
__device__ __forceinline__ float qs(float t, float p) { float e = ei(t) * 10.0f; return (KC::E * e) / (p - (1 - KC::E) * e); }  // :62
__device__ __forceinline__ float Ni(float t) {                                                                       // :83
    const float EI = ei(t) * 1000, ES = es(t) * 1000;
    return 10000 * expf((12.96f * (ES - EI)) / (EI - 0.639f));
}
__device__ __forceinline__ float pwater(float t) {                                                                   // :92
    return 999.83311f + (0.0752f * t) - (0.0089f * t * t) + (7.36413e-5f * t * t * t) -
           (4.74639e-7f * t * t * t * t) + (1.34888e-9f * t * t * t * t * t);
}
__device__ __forceinline__ float Lwater(float t) { return (2500.8f - 2.36f * t + 0.0016f * t * t - 0.00006f * t * t * t) * 1e3f; }  // :108
__device__ __forceinline__ float Lice(float t) { return (2834.1f - 0.29f * t - 0.004f * t * t) * 1e3f; }  // :117
__device__ __forceinline__ float DQVair(float t, float p) { return 2.26e-5f * powf((t + 273.15f) / 273.15f, 1.94f) * (1013.25f / p); }  // :146
__device__ __forceinline__ float ViscAir(float t) {                                                                  // :155
    return powf((t + 273.15f) / 273.15f, 3.0f / 2.0f) * ((273.15f + 111.0f) / (t + 111.0f)) * 1.716e-5f;
}
__device__ __forceinline__ float slopePrecip(float D, float Q, int type) {                                              // :167
    float num;
    if (type == 0) num = KC::PI * 0.99f * 8e-2f;
    else if (type == 1) num = KC::PI * 0.11f * 3e-2f;
    else if (type == 2) num = KC::PI * 0.91f * 4e-4f;
    else return 0.0f;
    const float den = fmaxf(D * Q * 0.001f, 1e-14f);
    return powf(num / den, 0.25f);
}
// Game/meteoformulas.cuh:219-260.  The else-if chain means type 3 ("all") computes rain only.
__device__ __forceinline__ void fallingVelocity(float Qr, float Qs, float Qi, float dens, int type, float gR, float gS, float gI, float& UR, float& US, float& UI) {
    const bool all = type == 3;
    UR = US = UI = 0.0f;
    if (gR == 0.0f) { UR = US = UI = -1.0f; return; }
    if (type == 0 || all) {
        float sR = slopePrecip(dens, Qr, 0);
        UR = 2115.0f * (gR / (6 * powf(sR, 0.8f))) * sqrtf(1.225f / dens);
        UR *= 0.01f;
    } else if (type == 1 || all) {
        float sS = slopePrecip(dens, Qs, 1);
        US = 152.93f * (gS / (6 * powf(sS, 0.25f))) * sqrtf(1.225f / dens);
        US *= 0.01f;
    } else if (type == 2 || all) {
        float sI = slopePrecip(dens, Qi, 2);
        UI = (gI / (6 * powf(sI, 0.5f))) * powf(4 * KC::g * 100 * 0.91f / (3 * 0.6f * dens * 0.001f), 0.5f);
        UI *= 0.01f;
    }
}
__device__ __forceinline__ float cvd(float t, float p, float dens) {                                                         // :276
    const float EI = ei(t) * 1000, ES = es(t) * 1000;
    const float A = (KC::Ls / (KC::Ka * (t + 273.15f))) * (KC::Ls / (KC::Rsw * (t + 273.15f)) - 1);
    const float B = (KC::Rsw * (t + 273.15f) * p) / (2.21f * EI);
    const float N = 10000 * expf((12.96f * (ES - EI)) / (EI - 0.639f));
    return 65.2f * ((powf(N, 0.5f) * (ES - EI)) / (powf(dens, 0.5f) * (A + B) * EI));
}
__device__ __forceinline__ float potentialTemp(float t, float pk, float pt) { return (t + 273.15f) * powf(pt / pk, KC::KAPPA) - 273.15f; }  // :299
__device__ __forceinline__ float MLR(float t, float p) {                                                                 // :309
    const float Tk = t + 273.15f;
    const float W = ws(t, p);
    const float Tw = ((KC::Rsd * Tk + KC::Hv * W) /
                  (KC::Cpd + (KC::Hv * KC::Hv * W * KC::E / (KC::Rsd * Tk * Tk))));
    return Tw / p;
}

// ---- Gammas, Game/microPhysics.cu:31-61 and Game/kernelSky.cu:30-37 -------------------------
struct Gammas {
    float R, ER, S, RC, SS, I, RI, Qr, Qs, Qi;
};

// ---- Process rates, Game/microPhysics.cu:67-685 -----------------------------------------------
struct Micro {
    Gammas G;
    __device__ float FPVCON(float t, float ps, float Qv, float QWS, float dt, float sp) const {  // :67
        const float e = es(t) * 10.0f;
        const float der = ((KC::E * ps) / ((ps - e) * (ps - e))) * (e * (17.27f * 237.3f / ((t + 237.3f) * (t + 237.3f))));
        return 1 / (dt * sp) * (Qv - QWS) / (1 + KC::E0v / KC::Cpd * der);
    }
    __device__ float FPVDEP(float t, float ps, float Qv, float QWI, float dt, float sp) const {  // :77
        const float e = ei(t) * 10.0f;
        const float der = ((KC::E * ps) / ((ps - e) * (ps - e))) * (e * (21.875f * 265.5f / ((t + 265.5f) * (t + 265.5f))));
        return 1 / (dt * sp) * (Qv - QWI) / (1 + KC::Ls / KC::Cpd * der);
    }
    __device__ float FPIMLT(float t, float Qc) const { return t >= 0 ? Qc : 0.0f; }  // :88
    __device__ float FPIDW(float dt, float t, float Qc, float Qw, float D, float ps) const {  // :99
        if (t < 0 && Qw > 0) {
            const float a = 0.5f;
            const float quu = fmaxf(1e-12f * Ni(t) / (D * 0.001f), Qc);
            return powf((1 - a) * cvd(t, ps, D * 0.001f) * dt + powf(quu, 1 - a), 1 / (1 - a)) - Qc;
        }
        return 0;
    }
    __device__ float FPIHOM(float t, float Qw) const { return (t < -40 && Qw > 0) ? Qw : 0.0f; }  // :115
    __device__ float FPIACR(float Qr, float Qc, float D, float sR) const {  // :124
        if (Qr > 0 && Qc > 0) {
            const float dens = powf(1.225f / D, 0.5f);
            return (KC::PI * KC::PI * 0.3f * 8e-2f * 2115.0f * Qc * 0.99f * G.RC) / (24 * 4.19e-10f * powf(sR, 6 + 0.8f)) * dens;
        }
        return 0;
    }
    __device__ float FPRACI(float Qr, float Qc, float D, float sR) const {  // :147
        if (Qr > 0 && Qc > 0) {
            const float dens = powf(1.225f / D, 0.5f);
            return (KC::PI * 0.3f * 8e-2f * 2115.0f * Qc * G.R) / (4 * powf(sR, 3 + 0.8f)) * dens;
        }
        return 0;
    }
    __device__ float FPRAUT(float Qw, float QwMin, float t) const {  // :167 (note 4 / 3 is integer division in the reference)
        if (Qw >= QwMin) {
            const float rc = 10e-6f;
            float Nc = (Qw / (float(4 / 3) * KC::PI * pwater(t) * rc * rc * rc)) * 1.225f;
            Nc /= 1e6f;
            const float disE = 0.5f * 0.5f;
            const float disp = ((1 + 3 * disE) * (1 + 4 * disE) * (1 + 5 * disE)) / ((1 + disE) * (1 + 2 * disE));
            const float L = Qw * 1.225f * 1e-3f;
            return 1e3f * 1.1e10f * disp * (L * L * L) * powf(Nc, -1.0f) *
                   float(1 - expf(-powf(1.03e16f * powf(Nc, -2.0f / 3.0f) * (L * L), 1.0f)));
        }
        return 0;
    }
    __device__ float FPRACW(float Qr, float Qw, float D, float sR) const {  // :189
        if (Qr > 0 && Qw > 0) {
            const float dens = powf(1.225f / D, 0.5f);
            return (KC::PI * 1.0f * 8e-2f * 2115.0f * Qw * G.R) / (4 * powf(sR, 3 + 0.8f)) * dens;
        }
        return 0;
    }
    __device__ float FPREVP(float t, float Qr, float Qv, float QWS, float D, float ps, float sR, float PT1) const {  // :210
        if (Qr > 0 && Qv / QWS < 1 && (1 - PT1) != 0) {
            const float tK = t + 273.15f, S = Qv / QWS, b = 0.8f, a = 2115.0f;
            const float dQv = DQVair(t, ps), kv = ViscAir(t);
            float Sc = kv / dQv;
            const float dens = powf(1.225f / (D * 0.001f), 0.25f);
            return fmaxf(0.0f, -1 * 2 * KC::PI * (S - 1) * 8e-2f *
                                   (0.78f * powf(sR, -2.0f) + 0.31f * powf(Sc, 1.0f / 3.0f) * G.ER * powf(a, 0.5f) *
                                                                   powf(kv, -0.5f) * dens * powf(sR, -((b + 5) / 2))) *
                                   1 / (D * 0.001f) *
                                   powf(KC::E0v * KC::E0v / (KC::Ka * KC::Rsw * tK * tK) + (1 / (D * 0.001f * QWS * dQv)), -1.0f));
        }
        return 0;
    }
    __device__ float FPRACS(float Qr, float Qs, float PT2, float UR, float US, float D, float sS, float sR) const {  // :238
        if (Qr > 0 && Qs > 0 && PT2 == 0) {
            const float size = KC::PI * KC::PI * 1.0f * 8e-2f * 3e-2f;
            return size * fabsf(UR - US) * (0.11f / (D * 0.001f)) *
                   (5 / (powf(sS, 6.0f) * sR) + (2 / (powf(sS, 5.0f) * powf(sR, 2.0f))) + (0.5f / (powf(sS, 4.0f) * powf(sR, 3.0f))));
        }
        return 0;
    }
    __device__ float FPSACW(float Qs, float Qw, float D, float sS) const {  // :263
        if (Qs > 0 && Qw > 0) {
            const float dens = powf(1.225f / D, 0.5f);
            return (KC::PI * 1.0f * 3e-2f * 152.93f * Qw * G.S) / (4 * powf(sS, 3 + 0.25f)) * dens;
        }
        return 0;
    }
    __device__ float FPSACR(float Qr, float Qs, float UR, float US, float D, float sR, float sS) const {  // :283
        if (Qr > 0 && Qs > 0) {
            const float size = KC::PI * KC::PI * 1.0f * 8e-2f * 3e-2f;
            return size * fabsf(US - UR) * (0.99f / (D * 0.001f)) *
                   (5 / (powf(sR, 6.0f) * sS) + (2 / (powf(sR, 5.0f) * powf(sS, 2.0f))) + (0.5f / (powf(sR, 4.0f) * powf(sS, 3.0f))));
        }
        return 0;
    }
    __device__ float FPSACI(float t, float Qs, float Qc, float D, float sS) const {  // :307
        if (Qs > 0 && Qc > 0) {
            const float ESI = expf(0.025f * t);
            const float dens = powf(1.225f / D, 0.5f);
            return (KC::PI * ESI * 3e-2f * 152.93f * Qc * G.S) / (4 * powf(sS, 3 + 0.25f)) * dens;
        }
        return 0;
    }
    __device__ float FPSAUT(float t, float Qc, float QcMin) const {  // :327
        if (Qc - QcMin > 0 && t < 0) return 1e-3f * expf(0.025f * t) * (Qc - QcMin);
        return 0;
    }
    __device__ float FPSFW(float dt, float t, float ps, float Qs, float Qw, float Qc, float Qv, float QWI, float D) const {  // :336
        if (Qs > 0 && Qw > 0) {
            const float tK = t + 273.15f;
            const float RI50 = 5e-3f, mI50 = 4.8e-7f, mI40 = 2.46e-7f, UI50 = 100.0f;
            float Si = Qv / QWI;
            const float X = DQVair(t, ps);
            const float A = KC::E0v / (KC::Ka * tK) * (KC::Ls * KC::Mw * 0.001f / (KC::R * tK) - 1);
            const float B = KC::R * tK * X * KC::Mw * 0.001f * ei(t) * 1000;
            const float a1g = 206.2f * (Si - 1) / (A + B);
            const float a2g = expf(0.09f * t);
            const float dt1 = 1 / (a1g * (1 - a2g)) * (powf(mI50, 1 - a2g) - powf(mI40, 1 - a2g));
            const float Qc50 = Qc * (dt / dt1) / 100;
            const float NI50 = Qc50 / mI50;
            return NI50 * (a1g * powf(mI50, a2g) + KC::PI * 1.0f * (D * 0.001f) * Qw * RI50 * RI50 * UI50);
        }
        return 0;
    }
    __device__ float FPSFI(float dt, float t, float ps, float Qs, float Qw, float Qc, float Qv, float QWI, float D) const {  // :371
        (void)dt; (void)Qw; (void)D;
        if (Qs > 0 && Qc > 0) {
            const float tK = t + 273.15f;
            const float mI50 = 4.8e-7f, mI40 = 2.46e-7f;
            float Si = Qv / QWI;
            const float X = DQVair(t, ps);
            const float A = KC::E0v / (KC::Ka * tK) * (KC::Ls * KC::Mw * 0.001f / (KC::R * tK) - 1);
            const float B = KC::R * tK * X * KC::Mw * 0.001f * ei(t) * 1000;
            const float a1g = 206.2f * (Si - 1) / (A + B);
            const float a2g = expf(0.09f * t);
            if (a1g > 0) return a2g * a1g * Qc / (powf(mI50, 0.5f) - powf(mI40, 0.5f));
        }
        return 0;
    }
    __device__ float FPSDEP(float t, float ps, float Qv, float QWI, float D, float sS) const {  // :397
        if (t < 0) {
            const float tK = t + 273.15f, c = 152.93f, d = 0.25f;
            const float dQv = DQVair(t, ps), kv = ViscAir(t);
            float Sc = kv / dQv, Si = Qv / QWI;
            const float A = KC::Ls * KC::Ls / (KC::Ka * KC::Rsw * tK * tK);
            const float B = 1 / (D * 0.001f * wi(t, ps) * dQv);
            const float dens = powf(1.225f / D, 0.25f);
            return KC::PI * KC::PI * (Si - 1) / (D * 0.001f * (A + B)) * 3e-2f *
                   (0.78f * powf(sS, -2.0f) + 0.31f * powf(Sc, 1.0f / 3.0f) * G.SS * powf(c, 0.5f) * dens * powf(kv, -0.5f) * powf(sS, -(d + 5) / 2));
        }
        return 0;
    }
    __device__ float FPSSUB(float PSDEP) const { return fmaxf(0.0f, -1 * PSDEP); }  // :424
    __device__ float FPSMLT(float t, float ps, float Qw, float Qr, float Qs, float Qv, float D, float sS, float PSACW, float PSACR, float dtS) const {  // :429
        (void)Qw; (void)Qr; (void)D; (void)dtS;
        if (t >= 0 && Qs > 0) {
            const float c = 152.93f, d = 0.25f;
            const float dQv = DQVair(t, ps), kv = ViscAir(t);
            float Sc = kv / dQv;
            const float Drs = ws(0.0f, ps) - Qv;
            const float dens = powf(1.225f / D, 0.25f);
            return fmaxf(0.0f, -1 * (-(2 * KC::PI / (dens * 0.001f * KC::Lf)) * (KC::Ka * t - KC::E0v * dQv * dens * 0.001f * Drs) * 3e-2f *
                                        (0.78f * powf(sS, -2.0f) + 0.31f * powf(Sc, 1.0f / 3.0f) * G.SS * powf(c, 0.5f) * dens * powf(kv, -0.5f) * powf(sS, -(d + 5) / 2)) -
                                    (KC::Cvl * t / KC::Lf) * (PSACW + PSACR)));
        }
        return 0;
    }
    __device__ float FPGAUT(float t, float Qs, float QiMin) const {  // :462
        const float sur = Qs - QiMin;
        if (sur > 0 && t < 0) return (1e-3f * expf(0.09f * t)) * sur;
        return 0;
    }
    __device__ float FPGFR(float t, float Qr, float D, float sR) const {  // :472
        if (Qr > 0 && t < 0)
            return 20 * KC::PI * KC::PI * 100.0f * 8e-2f * (0.99f / (D * 0.001f)) * (expf(0.66f * (-t)) - 1) * powf(sR, -7.0f);
        return 0;
    }
    __device__ float gfact(float D) const { return powf(4 * KC::g * 100 * 0.91f / (3 * 0.6f * D * 0.001f), 0.5f); }
    __device__ float FPGACW(float Qi, float Qw, float sI, float D) const {  // :489
        if (Qi > 0 && Qw > 0) return KC::PI * 1.0f * 4e-4f * Qw * G.I / (4 * powf(sI, 3.5f)) * gfact(D);
        return 0;
    }
    __device__ float FPGACI(float Qi, float Qc, float sI, float D) const {  // :506
        if (Qi > 0 && Qc > 0) return KC::PI * 1.0f * 4e-4f * Qc * G.I / (4 * powf(sI, 3.5f)) * gfact(D);
        return 0;
    }
    __device__ float FPGACR(float Qi, float Qr, float D, float UR, float UI, float sR, float sI) const {  // :523
        if (Qi > 0 && Qr > 0)
            return KC::PI * KC::PI * 0.1f * 8e-2f * 4e-4f * fabsf(UI - UR) * (0.99f / (D * 0.001f)) *
                   (5 / (powf(sR, 6.0f) * sI) + (2 / (powf(sR, 5.0f) * powf(sI, 2.0f))) + (0.5f / (powf(sR, 4.0f) * powf(sI, 3.0f))));
        return 0;
    }
    __device__ float FPGACS(float t, float Qs, float Qi, float D, float US, float UI, float sS, float sI, bool EGS1) const {  // :541
        if (Qs > 0 && Qi > 0) {
            const float EGS = (t >= 0 || EGS1) ? 1.0f : expf(0.09f * t);
            return KC::PI * KC::PI * EGS * 3e-2f * 4e-4f * fabsf(UI - US) * (0.11f / (D * 0.001f)) *
                   (5 / (powf(sS, 6.0f) * sI) + (2 / (powf(sS, 5.0f) * powf(sI, 2.0f))) + (0.5f / (powf(sS, 4.0f) * powf(sI, 3.0f))));
        }
        return 0;
    }
    __device__ float FPGDRY(float Qw, float Qc, float Qr, float Qs, float PGACW, float PGACI, float PGACR, float PGACS, float dtS) const {  // :560
        return fminf(Qw, PGACW * dtS) + fminf(Qc, PGACI * dtS) + fminf(Qr, PGACR * dtS) + fminf(Qs, PGACS * dtS);
    }
    __device__ float FPGSUB(float t, float ps, float Qv, float QWI, float Qi, float D, float sI) const {  // :572
        float Si = Qv / QWI;
        if (Qi > 0 && Si < 1) {
            const float tK = t + 273.15f;
            const float dQv = DQVair(t, ps), kv = ViscAir(t);
            float Sc = kv / dQv;
            const float A = KC::Ls * KC::Ls / (KC::Ka * KC::Rsw * tK * tK);
            const float B = 1 / (D * 0.001f * wi(t, ps) * dQv);
            const float dens = powf(4 * KC::g * 100 * 0.91f / (3 * 0.6f * D * 0.001f), 0.25f);
            return fmaxf(0.0f, -1 * KC::PI * KC::PI * (Si - 1) / (D * 0.001f * (A + B)) * 4e-4f *
                                  (0.78f * powf(sI, -2.0f) + 0.31f * powf(Sc, 1.0f / 3.0f) * G.RI * dens * powf(kv, -0.5f) * powf(sI, -2.75f)));
        }
        return 0;
    }
    __device__ float FPGMLT(float t, float ps, float Qw, float Qr, float Qi, float Qv, float D, float sI, float PGACW, float PGACR, float dtS) const {  // :602
        if (Qi > 0) {
            const float L1 = fminf(Qw, PGACW * dtS), L2 = fminf(Qr, PGACR * dtS);
            const float dQv = DQVair(t, ps), kv = ViscAir(t);
            float Sc = kv / dQv;
            const float Drs = ws(0.0f, ps) - Qv;
            const float dens = powf(4 * KC::g * 100 * 0.91f / (3 * 0.6f), 0.25f);
            return fmaxf(0.0f, -1 * (-2 * KC::PI / (D * 0.001f * KC::Lf) * (KC::Ka * t - KC::E0v * dQv * D * 0.001f * Drs) * 4e-4f *
                                        (0.78f * powf(sI, -2.0f) + 0.31f * powf(Sc, 1.0f / 3.0f) * G.RI * dens * powf(kv, -0.5f) * powf(sI, -2.75f)) -
                                    KC::Cvl * t / KC::Lf * (L1 + L2)));
        }
        return 0;
    }
    __device__ float FPGWET(float t, float ps, float Qc, float Qs, float Qi, float Qv, float US, float UI, float D, float sS, float sI, float PGACI, float PGACS, float dtS) const {  // :632
        if (Qi > 0) {
            const float PGACI1 = PGACI * 10.0f;
            const float PGACS1 = t >= 0 ? PGACS : FPGACS(t, Qs, Qi, D, US, UI, sS, sI, true);
            const float L1 = fminf(Qc, PGACI1 * dtS), L2 = fminf(Qs, PGACS1 * dtS);
            const float dQv = DQVair(t, ps), kv = ViscAir(t);
            float Sc = kv / dQv;
            const float Drs = ws(0.0f, ps) - Qv;
            const float dens = powf(4 * KC::g * 100.0f * 0.91f / (3 * 0.6f), 0.25f);
            return 2 * KC::PI * 4e-4f * (D * 0.001f * KC::E0v * dQv * Drs - KC::Ka * t) / (D * 0.001f * (KC::Lf + KC::Cvl * t)) *
                       (0.78f * powf(sI, -2.0f) + 0.31f * powf(Sc, 1.0f / 3.0f) * G.RI * dens * powf(kv, -0.5f) * powf(sI, -2.75f)) +
                   (L1 + L2) * (1 - KC::Cpi * t / (KC::Lf + KC::Cvl * t));
        }
        return 0;
    }
    __device__ float FPGACR1(float t, float Qw, float Qc, float Qs, float Qi, float D, float US, float UI, float sS, float sI, float PGWET, float PGACW, float PGACI, float PGACS, float dtS) const {  // :667
        if (Qi > 0) {
            const float PGACI1 = PGACI * 10.0f;
            const float PGACS1 = t >= 0 ? PGACS : FPGACS(t, Qs, Qi, D, US, UI, sS, sI, true);
            return PGWET - fminf(Qw, PGACW * dtS) - fminf(Qc, PGACI1 * dtS) - fminf(Qs, PGACS1 * dtS);
        }
        return 0;
    }

    // ---- ground processes, Game/microPhysics.cu:687-1032 ----
    __device__ float FPGFLW(float Qr) const { return Qr > 0 ? 100.0f * 5e-5f * Qr : 0.0f; }  // :687
    __device__ float FPGGMLT(float tgC, float Qi, float D, float sI) const {  // :698
        if (Qi > 0) {
            const float k4 = 0.955f * 1.0e-2f;
            const float cd = Qi * D * 0.001f;
            const float amount = cd / 0.91f;
            const float h = amount * 100.0f;
            const float af = 0.45f;
            const float QG = af * k4 * tgC / h;
            const float melt = fmaxf(0.0f, QG / KC::Lf);
            return melt * 4e-4f * powf(sI, -2.0f) * af / (D * 0.001f);
        }
        return 0;
    }
    __device__ float FPGSMLT(float taK, float tgC, float ps, float Qs_, float Qv, float Qr, float irr, float cc, float D, float wind, float dt) const {  // :731
        if (Qs_ > 0) {
            float Qsw = 0, Ql = 0, Qh = 0, Qe = 0, Qg = 0, Qp = 0;
            const float Tac = taK - 273.15f;
            const float Ts = 0, Tsk = Ts + 273.15f;
            Qsw = (1 - 0.9f) * irr;
            const float eac = 9.2e-6f * taK * taK;
            const float ea = (1 - 0.84f * cc) * eac + 0.84f * cc;
            Ql = ea * KC::oo * Tsk * Tsk * Tsk * Tsk - 310.0f;
            const float k = 0.41f;
            const float Ch = k * k / (logf(1.0f / 0.001f) * logf(2.0f / 0.0002f));
            Qh = D * KC::Cpd * Ch * wind * (Tac - Ts);
            const float Qvs = Qv / (1 + Qv);
            Qe = D * KC::E0v * Ch * wind * (Qvs - qs(Ts, ps));
            const float Td = tgC - Ts;
            if (Td > 0) {
                const float cd = Qsw * D * 0.001f;  // the reference shadows Qs here: the shortwave term
                const float amount = cd / 0.11f;
                Qg = 0.3f * (tgC - Ts) / amount;
            }
            Qp = KC::Cvl * 0.001f * Qr * D * taK;
            const float Q = Qsw + Ql + Qh + Qe + Qg + Qp;
            const float Qss = Qsw * D;
            const float QE = (Q * dt) / Qss;
            const float mf = QE / KC::Lf;
            return fmaxf(0.0f, mf * Qsw);
        }
        return 0;
    }
    __device__ float FPGREVP(float taK, float tgC, float ps, float Qv, float Qr, float irr, float D, float wind) const {  // :797
        if (Qr != 0) {
            const float tgK = tgC + 273.15f;
            const float VPD = es(tgC) * 1000.0f * (1 - Qv / ws(tgC, ps));
            const float k = 0.41f, z0m = 0.0001f, z0h = z0m * 0.1f;
            const float ga = wind * k * k / (logf(1.0f / z0m) * logf(2.0f / z0h));
            const float y = KC::Cpd * ps * 100.0f / (0.622f * KC::E0v);
            const float aP = es(taK - 273.15f) * 10.0f * (Qv / ws(taK - 273.15f, ps));
            const float ea = 1.24f * powf((aP / taK), 1.0f / 7.0f);
            const float Rn = irr * (1 - 0.08f) + KC::oo * 0.96f * (ea * (taK * taK * taK * taK) - (tgK * tgK * tgK * tgK));
            const float RnG = Rn - 0.2f * Rn;
            const float m = es(tgC) * 1000.0f * KC::E0v / (KC::Rsw * tgK * tgK);
            const float Em = (m * RnG + D * KC::Cpd * VPD * ga) / (KC::E0v * (m + y));
            const float EmD = fmaxf(0.0f, Em / D);
            const float areaW = fminf(1.0f, 0.01f * sqrtf(Qr));
            return EmD * areaW;
        }
        return 0;
    }
    __device__ float FPGDEVP(float& time, float Qr, float Qs_, float Qi, float Qrs) const {  // :847
        if (Qrs != 0) {
            if (Qr == 0 && Qs_ == 0 && Qi == 0) {
                const float secsInDay = float(60 * 60 * 24);
                const float O_ = 0.21f * secsInDay;
                return 200.0f * 1e-6f * Qrs * expf(-time / O_);
            }
            time = 0;
        }
        return 0;
    }
    __device__ float FPGGFR(float taK, float tgC, float ps, float Qr, float Qv, float Qi, float D, float irr, float cc, float wind, float dt) const {  // :873
        const float Tac = taK - 273.15f;
        if (Qr != 0 && Tac < 0) {
            float Qw = 0, Qc = 0, Qe = 0, Ql = 0, Qsw = 0, Qg = 0, Qf = 0;
            Qf = KC::Lf * Qr * D / dt;
            Qw = KC::Cvl * (273.15f - taK) * Qr * D / dt;
            const float k = 0.41f, z0m = 0.0001f, z0h = z0m * 0.1f;
            const float ga = wind * k * k / (logf(1.0f / z0m) * logf(1.0f / z0h));
            Qc = D * KC::Cpd * ga * (tgC - Tac);
            const float Ce = k * k;
            const float Qvs = Qv / (1 + Qv);
            Qe = D * KC::E0v * Ce * wind * fmaxf(0.0f, Qvs - qs(0.0f, ps));
            Qsw = -(1 - 0.06f) * irr;
            const float eac = 9.2e-6f * taK * taK;
            const float ea = (1 - 0.84f * cc) * eac + 0.84f * cc;
            Ql = ea * KC::oo * 273.15f * 273.15f * 273.15f * 273.15f - 310.0f;
            if (Qi > 0) {
                const float cd = Qi * D * 0.001f;
                const float h = cd / 0.91f;
                Qg = 0.3f * (tgC - 0) / h;
                Qg *= -1;
            }
            const float f = fminf(fmaxf((Qw + Qe + Qc + Qsw + Ql + Qg) / Qf, 0.0f), 1.0f);
            return f * Qr;
        }
        return 0;
    }
    __device__ float FPGSFR(float taK, float tgC, float ps, float Qv, float Qr, float Qs_, float D, float wind, float dt) const {  // :936
        if (Qr != 0 && Qs_ != 0) {
            float Qw = 0, Qe = 0, Qg = 0, Qf = 0;
            Qf = KC::Lf * Qr * D / dt;
            Qw = KC::Cvl * (273.15f - taK) * Qr * D / dt;
            const float k = 0.41f, Ce = k * k;
            const float Qvs = Qv / (1 + Qv);
            Qe = D * KC::E0v * Ce * wind * fmaxf(0.0f, Qvs - qs(0.0f, ps));
            const float cd = Qs_ * D * 0.001f;
            const float h = cd / 0.11f;
            Qg = 0.3f * (tgC - 0) / h;
            Qg *= -1;
            const float f = fminf(fmaxf((Qw + Qe + Qg) / Qf, 0.0f), 1.0f);
            return f * Qr;
        }
        return 0;
    }
    __device__ float FPGRFR(float taK, float tgC, float ps, float Qr, float Qv, float Qi, float Qgr, float Qgs, float D, float wind, float UR) const {  // :982
        const float Tac = taK - 273.15f;
        if (Qgr == 0 && Qgs == 0 && Qr != 0 && Tac < 0) {
            float Qw = 0, Qc = 0, Qe = 0, Ql = 0, Qsw = 0, Qg = 0, Qf = 0;
            const float densW = 0.99f;
            const float Rr = Qr * D * UR;
            const float P = Rr * 3600.0f / (densW * 1000.0f) * 1000;
            const float FFW = sqrtf(powf(P * densW / 3.6f, 2.0f) + powf(0.067f * powf(P, 0.846f) * wind, 2.0f));
            Qf = KC::Lf * 0.001f * FFW;
            Qw = KC::Cvl * 0.001f * (0 - Tac) * FFW;
            const float k = 0.41f, z0m = 0.1f, z0h = z0m * 0.1f;
            const float ga = wind * k * k / (logf(1.0f / z0m) * logf(1.0f / z0h));
            Qc = D * KC::Cpd * ga * (tgC - Tac);
            const float Ce = k * k;
            const float Qvs = Qv / (1 + Qv);
            Qe = D * KC::E0v * Ce * wind * fmaxf(0.0f, Qvs - qs(0.0f, ps));
            const float Td = tgC - 0;
            if (Td > 0) {
                const float cd = Qi * D * 0.001f;
                const float h = cd / 0.91f;
                Qg = 0.3f * (tgC - 0) / h;
                Qg *= -1;
            }
            const float f = fminf(fmaxf((Qw + Qc + Qe + Ql + Qsw + Qg) / Qf, 0.0f), 1.0f);
            return f * Qr;
        }
        return 0;
    }
};


}  // namespace skt
