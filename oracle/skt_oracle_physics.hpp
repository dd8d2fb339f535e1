// ORACLE — test infrastructure only. Nothing in the product library includes this file.
//
// CPU restatement of the per-cell thermodynamics and bulk microphysics of skewTCloudSim
// (Game/meteoformulas.cuh, Game/microPhysics.cu, constants Game/environment.cu:28-60).
// Templated on the floating type: float reproduces the reference's FP32 arithmetic (libm
// powf/expf/logf), double gives the FP64 oracle of the same method.
#pragma once
#include <cmath>
#include <algorithm>
#include <type_traits>

namespace skt_oracle {

// Physical constants, Game/environment.cu:28-60.  Values are spelled once; the float
// instantiation uses the float literal, the double one the decimal value.
#define SKT_ORACLE_CONSTANTS(X)                                                             \
    X(g, 9.8076) X(Hv, 2501000.0) X(R, 8.3145) X(Rsd, 287.0528) X(Rsw, 461.5)             \
    X(Cpd, 1003.5) X(Cvl, 4119.0) X(Cpi, 2093.0) X(Cpds, 800.0) X(Mw, 18.02)              \
    X(E0v, 2.374e+6) X(Lf, 3.3355e+5) X(Ls, 2.834e+6) X(Ka, 2.40e-2) X(PI, 3.14159265359) \
    X(oo, 5.67e-8) X(ge, 0.95)

template <class T> struct K;
template <> struct K<float> {
#define SKT_XF(n, v) static constexpr float n = v##f;
    SKT_ORACLE_CONSTANTS(SKT_XF)
#undef SKT_XF
    static constexpr float E = 287.0528f / 461.5f;  // Game/environment.cu:36
};
template <> struct K<double> {
#define SKT_XD(n, v) static constexpr double n = v;
    SKT_ORACLE_CONSTANTS(SKT_XD)
#undef SKT_XD
    static constexpr double E = 287.0528 / 461.5;
};

// libm dispatch: float -> powf/expf/..., double -> pow/exp/...
inline float Pow(float a, float b) { return powf(a, b); }
inline double Pow(double a, double b) { return pow(a, b); }
inline float Exp(float a) { return expf(a); }
inline double Exp(double a) { return exp(a); }
inline float Log(float a) { return logf(a); }
inline double Log(double a) { return log(a); }
inline float Sqrt(float a) { return sqrtf(a); }
inline double Sqrt(double a) { return sqrt(a); }
inline float Fmin(float a, float b) { return fminf(a, b); }
inline double Fmin(double a, double b) { return fmin(a, b); }
inline float Fmax(float a, float b) { return fmaxf(a, b); }
inline double Fmax(double a, double b) { return fmax(a, b); }
inline float Fabs(float a) { return fabsf(a); }
inline double Fabs(double a) { return fabs(a); }
inline float Ceil(float a) { return ceilf(a); }
inline double Ceil(double a) { return ceil(a); }
inline float Tgamma(float a) { return tgammaf(a); }
inline double Tgamma(double a) { return tgamma(a); }

template <class T> inline T kappa() { return K<T>::Rsd / K<T>::Cpd; }

// ---- Game/meteoformulas.cuh ---------------------------------------------------------------
template <class T> inline T es(T t) { return T(0.61078) * Exp((T(17.27) * t) / (t + T(237.3))); }        // :16
template <class T> inline T ei(T t) { return T(0.61078) * Exp((T(21.875) * t) / (t + T(265.5))); }       // :27
template <class T> inline T ws(T t, T p) { T e = es(t) * T(10); return (K<T>::E * e) / (p - e); }          // :41
template <class T> inline T wi(T t, T p) { T e = ei(t) * T(10); return (K<T>::E * e) / (p - e); }          // :52
template <class T> inline T qs(T t, T p) { T e = ei(t) * T(10); return (K<T>::E * e) / (p - (1 - K<T>::E) * e); }  // :62
template <class T> inline T Ni(T t) {                                                                       // :83
    const T EI = ei(t) * 1000, ES = es(t) * 1000;
    return 10000 * Exp((T(12.96) * (ES - EI)) / (EI - T(0.639)));
}
template <class T> inline T pwater(T t) {                                                                   // :92
    return T(999.83311) + (T(0.0752) * t) - (T(0.0089) * t * t) + (T(7.36413e-5) * t * t * t) -
           (T(4.74639e-7) * t * t * t * t) + (T(1.34888e-9) * t * t * t * t * t);
}
template <class T> inline T Lwater(T t) { return (T(2500.8) - T(2.36) * t + T(0.0016) * t * t - T(0.00006) * t * t * t) * T(1e3); }  // :108
template <class T> inline T Lice(T t) { return (T(2834.1) - T(0.29) * t - T(0.004) * t * t) * T(1e3); }  // :117
template <class T> inline T DQVair(T t, T p) { return T(2.26e-5) * Pow((t + T(273.15)) / T(273.15), T(1.94)) * (T(1013.25) / p); }  // :146
template <class T> inline T ViscAir(T t) {                                                                  // :155
    return Pow((t + T(273.15)) / T(273.15), T(3) / T(2)) * ((T(273.15) + T(111)) / (t + T(111))) * T(1.716e-5);
}
template <class T> inline T slopePrecip(T D, T Q, int type) {                                              // :167
    T num;
    if (type == 0) num = K<T>::PI * T(0.99) * T(8e-2);
    else if (type == 1) num = K<T>::PI * T(0.11) * T(3e-2);
    else if (type == 2) num = K<T>::PI * T(0.91) * T(4e-4);
    else return T(0);
    const T den = Fmax(D * Q * T(0.001), T(1e-14));
    return Pow(num / den, T(0.25));
}
struct Fall3 { double x, y, z; };
// Game/meteoformulas.cuh:219-260.  The else-if chain means type 3 ("all") computes rain only.
template <class T> inline void fallingVelocity(T Qr, T Qs, T Qi, T dens, int type, T gR, T gS, T gI, T& UR, T& US, T& UI) {
    const bool all = type == 3;
    UR = US = UI = T(0);
    if (gR == T(0)) { UR = US = UI = T(-1); return; }
    if (type == 0 || all) {
        T sR = slopePrecip(dens, Qr, 0);
        UR = T(2115) * (gR / (6 * Pow(sR, T(0.8)))) * Sqrt(T(1.225) / dens);
        UR *= T(0.01);
    } else if (type == 1 || all) {
        T sS = slopePrecip(dens, Qs, 1);
        US = T(152.93) * (gS / (6 * Pow(sS, T(0.25)))) * Sqrt(T(1.225) / dens);
        US *= T(0.01);
    } else if (type == 2 || all) {
        T sI = slopePrecip(dens, Qi, 2);
        UI = (gI / (6 * Pow(sI, T(0.5)))) * Pow(4 * K<T>::g * 100 * T(0.91) / (3 * T(0.6) * dens * T(0.001)), T(0.5));
        UI *= T(0.01);
    }
}
template <class T> inline T cvd(T t, T p, T dens) {                                                         // :276
    const T EI = ei(t) * 1000, ES = es(t) * 1000;
    const T A = (K<T>::Ls / (K<T>::Ka * (t + T(273.15)))) * (K<T>::Ls / (K<T>::Rsw * (t + T(273.15))) - 1);
    const T B = (K<T>::Rsw * (t + T(273.15)) * p) / (T(2.21) * EI);
    const T N = 10000 * Exp((T(12.96) * (ES - EI)) / (EI - T(0.639)));
    return T(65.2) * ((Pow(N, T(0.5)) * (ES - EI)) / (Pow(dens, T(0.5)) * (A + B) * EI));
}
template <class T> inline T potentialTemp(T t, T pk, T pt) { return (t + T(273.15)) * Pow(pt / pk, kappa<T>()) - T(273.15); }  // :299
template <class T> inline T MLR(T t, T p) {                                                                 // :309
    const T Tk = t + T(273.15);
    const T W = ws(t, p);
    const T Tw = ((K<T>::Rsd * Tk + K<T>::Hv * W) /
                  (K<T>::Cpd + (K<T>::Hv * K<T>::Hv * W * K<T>::E / (K<T>::Rsd * Tk * Tk))));
    return Tw / p;
}

// ---- Gammas, Game/microPhysics.cu:31-61 and Game/kernelSky.cu:30-37 -------------------------
template <class T> struct Gammas {
    T R, ER, S, RC, SS, I, RI, Qr, Qs, Qi;
    Gammas() {
        const T b = T(0.8), d = T(0.25);
        R = Tgamma(3 + b); ER = Tgamma((b + T(5)) / T(2)); S = Tgamma(3 + d); RC = Tgamma(6 + b);
        SS = Tgamma((d + T(5)) / T(2)); I = Tgamma(T(3.5)); RI = Tgamma(T(2.75));
        Qr = Tgamma(T(4) + b); Qs = Tgamma(T(4) + d); Qi = Qs;
    }
};

// ---- Process rates, Game/microPhysics.cu:67-685 -----------------------------------------------
template <class T> struct Micro {
    using C = K<T>;
    Gammas<T> G;
    T FPVCON(T t, T ps, T Qv, T QWS, T dt, T sp) const {  // :67
        const T e = es(t) * T(10);
        const T der = ((C::E * ps) / ((ps - e) * (ps - e))) * (e * (T(17.27) * T(237.3) / ((t + T(237.3)) * (t + T(237.3)))));
        return 1 / (dt * sp) * (Qv - QWS) / (1 + C::E0v / C::Cpd * der);
    }
    T FPVDEP(T t, T ps, T Qv, T QWI, T dt, T sp) const {  // :77
        const T e = ei(t) * T(10);
        const T der = ((C::E * ps) / ((ps - e) * (ps - e))) * (e * (T(21.875) * T(265.5) / ((t + T(265.5)) * (t + T(265.5)))));
        return 1 / (dt * sp) * (Qv - QWI) / (1 + C::Ls / C::Cpd * der);
    }
    T FPIMLT(T t, T Qc) const { return t >= 0 ? Qc : T(0); }  // :88
    T FPIDW(T dt, T t, T Qc, T Qw, T D, T ps) const {  // :99
        if (t < 0 && Qw > 0) {
            const T a = T(0.5);
            const T quu = Fmax(T(1e-12) * Ni(t) / (D * T(0.001)), Qc);
            return Pow((1 - a) * cvd(t, ps, D * T(0.001)) * dt + Pow(quu, 1 - a), 1 / (1 - a)) - Qc;
        }
        return 0;
    }
    T FPIHOM(T t, T Qw) const { return (t < -40 && Qw > 0) ? Qw : T(0); }  // :115
    T FPIACR(T Qr, T Qc, T D, T sR) const {  // :124
        if (Qr > 0 && Qc > 0) {
            const T dens = Pow(T(1.225) / D, T(0.5));
            return (C::PI * C::PI * T(0.3) * T(8e-2) * T(2115) * Qc * T(0.99) * G.RC) / (24 * T(4.19e-10) * Pow(sR, 6 + T(0.8))) * dens;
        }
        return 0;
    }
    T FPRACI(T Qr, T Qc, T D, T sR) const {  // :147
        if (Qr > 0 && Qc > 0) {
            const T dens = Pow(T(1.225) / D, T(0.5));
            return (C::PI * T(0.3) * T(8e-2) * T(2115) * Qc * G.R) / (4 * Pow(sR, 3 + T(0.8))) * dens;
        }
        return 0;
    }
    T FPRAUT(T Qw, T QwMin, T t) const {  // :167 (note 4 / 3 is integer division in the reference)
        if (Qw >= QwMin) {
            const T rc = T(10e-6);
            T Nc = (Qw / (T(4 / 3) * C::PI * pwater(t) * rc * rc * rc)) * T(1.225);
            Nc /= T(1e6);
            const T disE = T(0.5) * T(0.5);
            const T disp = ((1 + 3 * disE) * (1 + 4 * disE) * (1 + 5 * disE)) / ((1 + disE) * (1 + 2 * disE));
            const T L = Qw * T(1.225) * T(1e-3);
            return T(1e3) * T(1.1e10) * disp * (L * L * L) * Pow(Nc, T(-1)) *
                   T(1 - Exp(-Pow(T(1.03e16) * Pow(Nc, T(-2) / T(3)) * (L * L), T(1))));
        }
        return 0;
    }
    T FPRACW(T Qr, T Qw, T D, T sR) const {  // :189
        if (Qr > 0 && Qw > 0) {
            const T dens = Pow(T(1.225) / D, T(0.5));
            return (C::PI * T(1) * T(8e-2) * T(2115) * Qw * G.R) / (4 * Pow(sR, 3 + T(0.8))) * dens;
        }
        return 0;
    }
    T FPREVP(T t, T Qr, T Qv, T QWS, T D, T ps, T sR, T PT1) const {  // :210
        if (Qr > 0 && Qv / QWS < 1 && (1 - PT1) != 0) {
            const T tK = t + T(273.15), S = Qv / QWS, b = T(0.8), a = T(2115);
            const T dQv = DQVair(t, ps), kv = ViscAir(t);
            T Sc = kv / dQv;
            const T dens = Pow(T(1.225) / (D * T(0.001)), T(0.25));
            return Fmax(T(0), -1 * 2 * C::PI * (S - 1) * T(8e-2) *
                                   (T(0.78) * Pow(sR, T(-2)) + T(0.31) * Pow(Sc, T(1) / T(3)) * G.ER * Pow(a, T(0.5)) *
                                                                   Pow(kv, T(-0.5)) * dens * Pow(sR, -((b + 5) / 2))) *
                                   1 / (D * T(0.001)) *
                                   Pow(C::E0v * C::E0v / (C::Ka * C::Rsw * tK * tK) + (1 / (D * T(0.001) * QWS * dQv)), T(-1)));
        }
        return 0;
    }
    T FPRACS(T Qr, T Qs, T PT2, T UR, T US, T D, T sS, T sR) const {  // :238
        if (Qr > 0 && Qs > 0 && PT2 == 0) {
            const T size = C::PI * C::PI * T(1) * T(8e-2) * T(3e-2);
            return size * Fabs(UR - US) * (T(0.11) / (D * T(0.001))) *
                   (5 / (Pow(sS, T(6)) * sR) + (2 / (Pow(sS, T(5)) * Pow(sR, T(2)))) + (T(0.5) / (Pow(sS, T(4)) * Pow(sR, T(3)))));
        }
        return 0;
    }
    T FPSACW(T Qs, T Qw, T D, T sS) const {  // :263
        if (Qs > 0 && Qw > 0) {
            const T dens = Pow(T(1.225) / D, T(0.5));
            return (C::PI * T(1) * T(3e-2) * T(152.93) * Qw * G.S) / (4 * Pow(sS, 3 + T(0.25))) * dens;
        }
        return 0;
    }
    T FPSACR(T Qr, T Qs, T UR, T US, T D, T sR, T sS) const {  // :283
        if (Qr > 0 && Qs > 0) {
            const T size = C::PI * C::PI * T(1) * T(8e-2) * T(3e-2);
            return size * Fabs(US - UR) * (T(0.99) / (D * T(0.001))) *
                   (5 / (Pow(sR, T(6)) * sS) + (2 / (Pow(sR, T(5)) * Pow(sS, T(2)))) + (T(0.5) / (Pow(sR, T(4)) * Pow(sS, T(3)))));
        }
        return 0;
    }
    T FPSACI(T t, T Qs, T Qc, T D, T sS) const {  // :307
        if (Qs > 0 && Qc > 0) {
            const T ESI = Exp(T(0.025) * t);
            const T dens = Pow(T(1.225) / D, T(0.5));
            return (C::PI * ESI * T(3e-2) * T(152.93) * Qc * G.S) / (4 * Pow(sS, 3 + T(0.25))) * dens;
        }
        return 0;
    }
    T FPSAUT(T t, T Qc, T QcMin) const {  // :327
        if (Qc - QcMin > 0 && t < 0) return T(1e-3) * Exp(T(0.025) * t) * (Qc - QcMin);
        return 0;
    }
    T FPSFW(T dt, T t, T ps, T Qs, T Qw, T Qc, T Qv, T QWI, T D) const {  // :336
        if (Qs > 0 && Qw > 0) {
            const T tK = t + T(273.15);
            const T RI50 = T(5e-3), mI50 = T(4.8e-7), mI40 = T(2.46e-7), UI50 = T(100);
            T Si = Qv / QWI;
            const T X = DQVair(t, ps);
            const T A = C::E0v / (C::Ka * tK) * (C::Ls * C::Mw * T(0.001) / (C::R * tK) - 1);
            const T B = C::R * tK * X * C::Mw * T(0.001) * ei(t) * 1000;
            const T a1g = T(206.2) * (Si - 1) / (A + B);
            const T a2g = Exp(T(0.09) * t);
            const T dt1 = 1 / (a1g * (1 - a2g)) * (Pow(mI50, 1 - a2g) - Pow(mI40, 1 - a2g));
            const T Qc50 = Qc * (dt / dt1) / 100;
            const T NI50 = Qc50 / mI50;
            return NI50 * (a1g * Pow(mI50, a2g) + C::PI * T(1) * (D * T(0.001)) * Qw * RI50 * RI50 * UI50);
        }
        return 0;
    }
    T FPSFI(T dt, T t, T ps, T Qs, T Qw, T Qc, T Qv, T QWI, T D) const {  // :371
        (void)dt; (void)Qw; (void)D;
        if (Qs > 0 && Qc > 0) {
            const T tK = t + T(273.15);
            const T mI50 = T(4.8e-7), mI40 = T(2.46e-7);
            T Si = Qv / QWI;
            const T X = DQVair(t, ps);
            const T A = C::E0v / (C::Ka * tK) * (C::Ls * C::Mw * T(0.001) / (C::R * tK) - 1);
            const T B = C::R * tK * X * C::Mw * T(0.001) * ei(t) * 1000;
            const T a1g = T(206.2) * (Si - 1) / (A + B);
            const T a2g = Exp(T(0.09) * t);
            if (a1g > 0) return a2g * a1g * Qc / (Pow(mI50, T(0.5)) - Pow(mI40, T(0.5)));
        }
        return 0;
    }
    T FPSDEP(T t, T ps, T Qv, T QWI, T D, T sS) const {  // :397
        if (t < 0) {
            const T tK = t + T(273.15), c = T(152.93), d = T(0.25);
            const T dQv = DQVair(t, ps), kv = ViscAir(t);
            T Sc = kv / dQv, Si = Qv / QWI;
            const T A = C::Ls * C::Ls / (C::Ka * C::Rsw * tK * tK);
            const T B = 1 / (D * T(0.001) * wi(t, ps) * dQv);
            const T dens = Pow(T(1.225) / D, T(0.25));
            return C::PI * C::PI * (Si - 1) / (D * T(0.001) * (A + B)) * T(3e-2) *
                   (T(0.78) * Pow(sS, T(-2)) + T(0.31) * Pow(Sc, T(1) / T(3)) * G.SS * Pow(c, T(0.5)) * dens * Pow(kv, T(-0.5)) * Pow(sS, -(d + 5) / 2));
        }
        return 0;
    }
    T FPSSUB(T PSDEP) const { return Fmax(T(0), -1 * PSDEP); }  // :424
    T FPSMLT(T t, T ps, T Qw, T Qr, T Qs, T Qv, T D, T sS, T PSACW, T PSACR, T dtS) const {  // :429
        (void)Qw; (void)Qr; (void)D; (void)dtS;
        if (t >= 0 && Qs > 0) {
            const T c = T(152.93), d = T(0.25);
            const T dQv = DQVair(t, ps), kv = ViscAir(t);
            T Sc = kv / dQv;
            const T Drs = ws(T(0), ps) - Qv;
            const T dens = Pow(T(1.225) / D, T(0.25));
            return Fmax(T(0), -1 * (-(2 * C::PI / (dens * T(0.001) * C::Lf)) * (C::Ka * t - C::E0v * dQv * dens * T(0.001) * Drs) * T(3e-2) *
                                        (T(0.78) * Pow(sS, T(-2)) + T(0.31) * Pow(Sc, T(1) / T(3)) * G.SS * Pow(c, T(0.5)) * dens * Pow(kv, T(-0.5)) * Pow(sS, -(d + 5) / 2)) -
                                    (C::Cvl * t / C::Lf) * (PSACW + PSACR)));
        }
        return 0;
    }
    T FPGAUT(T t, T Qs, T QiMin) const {  // :462
        const T sur = Qs - QiMin;
        if (sur > 0 && t < 0) return (T(1e-3) * Exp(T(0.09) * t)) * sur;
        return 0;
    }
    T FPGFR(T t, T Qr, T D, T sR) const {  // :472
        if (Qr > 0 && t < 0)
            return 20 * C::PI * C::PI * T(100) * T(8e-2) * (T(0.99) / (D * T(0.001))) * (Exp(T(0.66) * (-t)) - 1) * Pow(sR, T(-7));
        return 0;
    }
    T gfact(T D) const { return Pow(4 * C::g * 100 * T(0.91) / (3 * T(0.6) * D * T(0.001)), T(0.5)); }
    T FPGACW(T Qi, T Qw, T sI, T D) const {  // :489
        if (Qi > 0 && Qw > 0) return C::PI * T(1) * T(4e-4) * Qw * G.I / (4 * Pow(sI, T(3.5))) * gfact(D);
        return 0;
    }
    T FPGACI(T Qi, T Qc, T sI, T D) const {  // :506
        if (Qi > 0 && Qc > 0) return C::PI * T(1) * T(4e-4) * Qc * G.I / (4 * Pow(sI, T(3.5))) * gfact(D);
        return 0;
    }
    T FPGACR(T Qi, T Qr, T D, T UR, T UI, T sR, T sI) const {  // :523
        if (Qi > 0 && Qr > 0)
            return C::PI * C::PI * T(0.1) * T(8e-2) * T(4e-4) * Fabs(UI - UR) * (T(0.99) / (D * T(0.001))) *
                   (5 / (Pow(sR, T(6)) * sI) + (2 / (Pow(sR, T(5)) * Pow(sI, T(2)))) + (T(0.5) / (Pow(sR, T(4)) * Pow(sI, T(3)))));
        return 0;
    }
    T FPGACS(T t, T Qs, T Qi, T D, T US, T UI, T sS, T sI, bool EGS1) const {  // :541
        if (Qs > 0 && Qi > 0) {
            const T EGS = (t >= 0 || EGS1) ? T(1) : Exp(T(0.09) * t);
            return C::PI * C::PI * EGS * T(3e-2) * T(4e-4) * Fabs(UI - US) * (T(0.11) / (D * T(0.001))) *
                   (5 / (Pow(sS, T(6)) * sI) + (2 / (Pow(sS, T(5)) * Pow(sI, T(2)))) + (T(0.5) / (Pow(sS, T(4)) * Pow(sI, T(3)))));
        }
        return 0;
    }
    T FPGDRY(T Qw, T Qc, T Qr, T Qs, T PGACW, T PGACI, T PGACR, T PGACS, T dtS) const {  // :560
        return Fmin(Qw, PGACW * dtS) + Fmin(Qc, PGACI * dtS) + Fmin(Qr, PGACR * dtS) + Fmin(Qs, PGACS * dtS);
    }
    T FPGSUB(T t, T ps, T Qv, T QWI, T Qi, T D, T sI) const {  // :572
        T Si = Qv / QWI;
        if (Qi > 0 && Si < 1) {
            const T tK = t + T(273.15);
            const T dQv = DQVair(t, ps), kv = ViscAir(t);
            T Sc = kv / dQv;
            const T A = C::Ls * C::Ls / (C::Ka * C::Rsw * tK * tK);
            const T B = 1 / (D * T(0.001) * wi(t, ps) * dQv);
            const T dens = Pow(4 * C::g * 100 * T(0.91) / (3 * T(0.6) * D * T(0.001)), T(0.25));
            return Fmax(T(0), -1 * C::PI * C::PI * (Si - 1) / (D * T(0.001) * (A + B)) * T(4e-4) *
                                  (T(0.78) * Pow(sI, T(-2)) + T(0.31) * Pow(Sc, T(1) / T(3)) * G.RI * dens * Pow(kv, T(-0.5)) * Pow(sI, T(-2.75))));
        }
        return 0;
    }
    T FPGMLT(T t, T ps, T Qw, T Qr, T Qi, T Qv, T D, T sI, T PGACW, T PGACR, T dtS) const {  // :602
        if (Qi > 0) {
            const T L1 = Fmin(Qw, PGACW * dtS), L2 = Fmin(Qr, PGACR * dtS);
            const T dQv = DQVair(t, ps), kv = ViscAir(t);
            T Sc = kv / dQv;
            const T Drs = ws(T(0), ps) - Qv;
            const T dens = Pow(4 * C::g * 100 * T(0.91) / (3 * T(0.6)), T(0.25));
            return Fmax(T(0), -1 * (-2 * C::PI / (D * T(0.001) * C::Lf) * (C::Ka * t - C::E0v * dQv * D * T(0.001) * Drs) * T(4e-4) *
                                        (T(0.78) * Pow(sI, T(-2)) + T(0.31) * Pow(Sc, T(1) / T(3)) * G.RI * dens * Pow(kv, T(-0.5)) * Pow(sI, T(-2.75))) -
                                    C::Cvl * t / C::Lf * (L1 + L2)));
        }
        return 0;
    }
    T FPGWET(T t, T ps, T Qc, T Qs, T Qi, T Qv, T US, T UI, T D, T sS, T sI, T PGACI, T PGACS, T dtS) const {  // :632
        if (Qi > 0) {
            const T PGACI1 = PGACI * T(10);
            const T PGACS1 = t >= 0 ? PGACS : FPGACS(t, Qs, Qi, D, US, UI, sS, sI, true);
            const T L1 = Fmin(Qc, PGACI1 * dtS), L2 = Fmin(Qs, PGACS1 * dtS);
            const T dQv = DQVair(t, ps), kv = ViscAir(t);
            T Sc = kv / dQv;
            const T Drs = ws(T(0), ps) - Qv;
            const T dens = Pow(4 * C::g * T(100) * T(0.91) / (3 * T(0.6)), T(0.25));
            return 2 * C::PI * T(4e-4) * (D * T(0.001) * C::E0v * dQv * Drs - C::Ka * t) / (D * T(0.001) * (C::Lf + C::Cvl * t)) *
                       (T(0.78) * Pow(sI, T(-2)) + T(0.31) * Pow(Sc, T(1) / T(3)) * G.RI * dens * Pow(kv, T(-0.5)) * Pow(sI, T(-2.75))) +
                   (L1 + L2) * (1 - C::Cpi * t / (C::Lf + C::Cvl * t));
        }
        return 0;
    }
    T FPGACR1(T t, T Qw, T Qc, T Qs, T Qi, T D, T US, T UI, T sS, T sI, T PGWET, T PGACW, T PGACI, T PGACS, T dtS) const {  // :667
        if (Qi > 0) {
            const T PGACI1 = PGACI * T(10);
            const T PGACS1 = t >= 0 ? PGACS : FPGACS(t, Qs, Qi, D, US, UI, sS, sI, true);
            return PGWET - Fmin(Qw, PGACW * dtS) - Fmin(Qc, PGACI1 * dtS) - Fmin(Qs, PGACS1 * dtS);
        }
        return 0;
    }

    // ---- ground processes, Game/microPhysics.cu:687-1032 ----
    T FPGFLW(T Qr) const { return Qr > 0 ? T(100) * T(5e-5) * Qr : T(0); }  // :687
    T FPGGMLT(T tgC, T Qi, T D, T sI) const {  // :698
        if (Qi > 0) {
            const T k4 = T(0.955) * T(1.0e-2);
            const T cd = Qi * D * T(0.001);
            const T amount = cd / T(0.91);
            const T h = amount * T(100);
            const T af = T(0.45);
            const T QG = af * k4 * tgC / h;
            const T melt = Fmax(T(0), QG / C::Lf);
            return melt * T(4e-4) * Pow(sI, T(-2)) * af / (D * T(0.001));
        }
        return 0;
    }
    T FPGSMLT(T taK, T tgC, T ps, T Qs_, T Qv, T Qr, T irr, T cc, T D, T wind, T dt) const {  // :731
        if (Qs_ > 0) {
            T Qsw = 0, Ql = 0, Qh = 0, Qe = 0, Qg = 0, Qp = 0;
            const T Tac = taK - T(273.15);
            const T Ts = 0, Tsk = Ts + T(273.15);
            Qsw = (1 - T(0.9)) * irr;
            const T eac = T(9.2e-6) * taK * taK;
            const T ea = (1 - T(0.84) * cc) * eac + T(0.84) * cc;
            Ql = ea * C::oo * Tsk * Tsk * Tsk * Tsk - T(310);
            const T k = T(0.41);
            const T Ch = k * k / (Log(T(1) / T(0.001)) * Log(T(2) / T(0.0002)));
            Qh = D * C::Cpd * Ch * wind * (Tac - Ts);
            const T Qvs = Qv / (1 + Qv);
            Qe = D * C::E0v * Ch * wind * (Qvs - qs(Ts, ps));
            const T Td = tgC - Ts;
            if (Td > 0) {
                const T cd = Qsw * D * T(0.001);  // the reference shadows Qs here: the shortwave term
                const T amount = cd / T(0.11);
                Qg = T(0.3) * (tgC - Ts) / amount;
            }
            Qp = C::Cvl * T(0.001) * Qr * D * taK;
            const T Q = Qsw + Ql + Qh + Qe + Qg + Qp;
            const T Qss = Qsw * D;
            const T QE = (Q * dt) / Qss;
            const T mf = QE / C::Lf;
            return Fmax(T(0), mf * Qsw);
        }
        return 0;
    }
    T FPGREVP(T taK, T tgC, T ps, T Qv, T Qr, T irr, T D, T wind) const {  // :797
        if (Qr != 0) {
            const T tgK = tgC + T(273.15);
            const T VPD = es(tgC) * T(1000) * (1 - Qv / ws(tgC, ps));
            const T k = T(0.41), z0m = T(0.0001), z0h = z0m * T(0.1);
            const T ga = wind * k * k / (Log(T(1) / z0m) * Log(T(2) / z0h));
            const T y = C::Cpd * ps * T(100) / (T(0.622) * C::E0v);
            const T aP = es(taK - T(273.15)) * T(10) * (Qv / ws(taK - T(273.15), ps));
            const T ea = T(1.24) * Pow((aP / taK), T(1) / T(7));
            const T Rn = irr * (1 - T(0.08)) + C::oo * T(0.96) * (ea * (taK * taK * taK * taK) - (tgK * tgK * tgK * tgK));
            const T RnG = Rn - T(0.2) * Rn;
            const T m = es(tgC) * T(1000) * C::E0v / (C::Rsw * tgK * tgK);
            const T Em = (m * RnG + D * C::Cpd * VPD * ga) / (C::E0v * (m + y));
            const T EmD = Fmax(T(0), Em / D);
            const T areaW = Fmin(T(1), T(0.01) * Sqrt(Qr));
            return EmD * areaW;
        }
        return 0;
    }
    T FPGDEVP(T& time, T Qr, T Qs_, T Qi, T Qrs) const {  // :847
        if (Qrs != 0) {
            if (Qr == 0 && Qs_ == 0 && Qi == 0) {
                const T secsInDay = T(60 * 60 * 24);
                const T O_ = T(0.21) * secsInDay;
                return T(200) * T(1e-6) * Qrs * Exp(-time / O_);
            }
            time = 0;
        }
        return 0;
    }
    T FPGGFR(T taK, T tgC, T ps, T Qr, T Qv, T Qi, T D, T irr, T cc, T wind, T dt) const {  // :873
        const T Tac = taK - T(273.15);
        if (Qr != 0 && Tac < 0) {
            T Qw = 0, Qc = 0, Qe = 0, Ql = 0, Qsw = 0, Qg = 0, Qf = 0;
            Qf = C::Lf * Qr * D / dt;
            Qw = C::Cvl * (T(273.15) - taK) * Qr * D / dt;
            const T k = T(0.41), z0m = T(0.0001), z0h = z0m * T(0.1);
            const T ga = wind * k * k / (Log(T(1) / z0m) * Log(T(1) / z0h));
            Qc = D * C::Cpd * ga * (tgC - Tac);
            const T Ce = k * k;
            const T Qvs = Qv / (1 + Qv);
            Qe = D * C::E0v * Ce * wind * Fmax(T(0), Qvs - qs(T(0), ps));
            Qsw = -(1 - T(0.06)) * irr;
            const T eac = T(9.2e-6) * taK * taK;
            const T ea = (1 - T(0.84) * cc) * eac + T(0.84) * cc;
            Ql = ea * C::oo * T(273.15) * T(273.15) * T(273.15) * T(273.15) - T(310);
            if (Qi > 0) {
                const T cd = Qi * D * T(0.001);
                const T h = cd / T(0.91);
                Qg = T(0.3) * (tgC - 0) / h;
                Qg *= -1;
            }
            const T f = Fmin(Fmax((Qw + Qe + Qc + Qsw + Ql + Qg) / Qf, T(0)), T(1));
            return f * Qr;
        }
        return 0;
    }
    T FPGSFR(T taK, T tgC, T ps, T Qv, T Qr, T Qs_, T D, T wind, T dt) const {  // :936
        if (Qr != 0 && Qs_ != 0) {
            T Qw = 0, Qe = 0, Qg = 0, Qf = 0;
            Qf = C::Lf * Qr * D / dt;
            Qw = C::Cvl * (T(273.15) - taK) * Qr * D / dt;
            const T k = T(0.41), Ce = k * k;
            const T Qvs = Qv / (1 + Qv);
            Qe = D * C::E0v * Ce * wind * Fmax(T(0), Qvs - qs(T(0), ps));
            const T cd = Qs_ * D * T(0.001);
            const T h = cd / T(0.11);
            Qg = T(0.3) * (tgC - 0) / h;
            Qg *= -1;
            const T f = Fmin(Fmax((Qw + Qe + Qg) / Qf, T(0)), T(1));
            return f * Qr;
        }
        return 0;
    }
    T FPGRFR(T taK, T tgC, T ps, T Qr, T Qv, T Qi, T Qgr, T Qgs, T D, T wind, T UR) const {  // :982
        const T Tac = taK - T(273.15);
        if (Qgr == 0 && Qgs == 0 && Qr != 0 && Tac < 0) {
            T Qw = 0, Qc = 0, Qe = 0, Ql = 0, Qsw = 0, Qg = 0, Qf = 0;
            const T densW = T(0.99);
            const T Rr = Qr * D * UR;
            const T P = Rr * T(3600) / (densW * T(1000)) * 1000;
            const T FFW = Sqrt(Pow(P * densW / T(3.6), T(2)) + Pow(T(0.067) * Pow(P, T(0.846)) * wind, T(2)));
            Qf = C::Lf * T(0.001) * FFW;
            Qw = C::Cvl * T(0.001) * (0 - Tac) * FFW;
            const T k = T(0.41), z0m = T(0.1), z0h = z0m * T(0.1);
            const T ga = wind * k * k / (Log(T(1) / z0m) * Log(T(1) / z0h));
            Qc = D * C::Cpd * ga * (tgC - Tac);
            const T Ce = k * k;
            const T Qvs = Qv / (1 + Qv);
            Qe = D * C::E0v * Ce * wind * Fmax(T(0), Qvs - qs(T(0), ps));
            const T Td = tgC - 0;
            if (Td > 0) {
                const T cd = Qi * D * T(0.001);
                const T h = cd / T(0.91);
                Qg = T(0.3) * (tgC - 0) / h;
                Qg *= -1;
            }
            const T f = Fmin(Fmax((Qw + Qc + Qe + Ql + Qsw + Qg) / Qf, T(0)), T(1));
            return f * Qr;
        }
        return 0;
    }
};

}  // namespace skt_oracle
