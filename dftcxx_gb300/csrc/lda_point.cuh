// lda_point.cuh -- closed-shell Slater (alpha = 2/3) + VWN point functions
// (functionals.cpp:24-158), shared by the build and its derivative.
#pragma once
#include "dftg_internal.cuh"

namespace dftg {

template <typename T> struct LdaMath;
template <> struct LdaMath<double> {
    static __device__ double pw(double x, double y) { return pow(x, y); }
    static __device__ double lg(double x) { return log(x); }
    static __device__ double at(double x) { return atan(x); }
    static __device__ double sq(double x) { return sqrt(x); }
};
template <> struct LdaMath<float> {
    static __device__ float pw(float x, float y) { return powf(x, y); }
    static __device__ float lg(float x) { return logf(x); }
    static __device__ float at(float x) { return atanf(x); }
    static __device__ float sq(float x) { return sqrtf(x); }
};

template <typename T>
__device__ __forceinline__ T vwn_xx(T x, T b, T c) { return x * x + b * x + c; }

template <typename T>
__device__ T vwn_eps(T x, T a, T x0, T b, T c)
{
    using M = LdaMath<T>;
    const T q = M::sq(T(4) * c - b * b);
    return a * (M::lg(x * x / vwn_xx(x, b, c))
                - b * (x0 / vwn_xx(x0, b, c)) * M::lg((x - x0) * (x - x0) / vwn_xx(x, b, c))
                + (T(2) * b / q) * (T(1) - (x0 * (T(2) * x0 + b) / vwn_xx(x0, b, c))) * M::at(q / (T(2) * x + b)));
}

template <typename T>
__device__ T vwn_deps(T x, T a, T x0, T b, T c)
{
    using M = LdaMath<T>;
    const T q = M::sq(T(4) * c - b * b);
    const T t = (T(2) * x + b) * (T(2) * x + b) + q * q;
    return a * (T(2) / x - (T(2) * x + b) / vwn_xx(x, b, c) - T(4) * b / t
                - (b * x0 / vwn_xx(x0, b, c)) * (T(2) / (x - x0) - (T(2) * x + b) / vwn_xx(x, b, c)
                                                 - T(4) * (T(2) * x0 + b) / t));
}

// closed-shell point kernel: e_x + e_c and 0.5 * (vxa + vxb + vca + vcb)
template <typename T>
__device__ void lda_point(double rho_d, T &e, T &v)
{
    using M = LdaMath<T>;
    const T tol = T(1e-10);
    const T fac = T(-2.25 * (2.0 / 3.0)) * M::pw(T(3.0 / 4.0 / kPi), T(1.0 / 3.0));
    const T da = T(rho_d * 0.5);
    T ex = 0, vxa = 0;
    if (!(da < tol)) {
        const T r3 = M::pw(da, T(1.0 / 3.0));
        ex = fac * da * r3;
        vxa = T(4.0 / 3.0) * fac * r3;
    }
    // rho_b == rho_a: identical second spin channel
    ex = ex + ex;
    const T vx = vxa;   // (vxa + vxb) / 2
    T ec = 0, vc = 0;
    const T dens = da + da;
    if (!(dens < tol)) {
        const T x = M::pw(T(3.0 / 4.0 / kPi) / dens, T(1.0 / 6.0));
        const T epsp = vwn_eps<T>(x, T(0.0310907), T(-0.10498), T(3.72744), T(12.9352));
        const T depsp = vwn_deps<T>(x, T(0.0310907), T(-0.10498), T(3.72744), T(12.9352));
        // zeta = 0 gives g = 0 < tol: paramagnetic branch (functionals.cpp:94-99)
        ec = epsp * dens;
        vc = epsp - (x / T(6)) * depsp;
    }
    e = ex + ec;
    v = vx + vc;
}

// Mixed point kernel with the energy density as a double-float (no FP64 work):
// the transcendental parts in FP32, every constant shared by all points and
// every product that carries the energy in double-float (TwoProd), so no
// rounding is common to all points.
__device__ inline void lda_point_df(dfl rho, dfl &e, float &v)
{
    constexpr double FAC = -0.93052573634910019, K34PI = 0.238732414637843;
    constexpr double A = 0.0310907, K1 = -0.031167608678943783, K2 = 1.2474243062431216;
    constexpr float Af = 0.0310907f, X0f = -0.10498f, Bf = 3.72744f, Cf = 12.9352f, Qf = 6.1519908197590798f,
                    Q2f = 37.846991046399992f, K1f = -0.031167608678943783f, VXf = -1.2407009817988002f;
    const dfl FACd = {(float)FAC, (float)(FAC - (double)(float)FAC)};
    const dfl Ad = {(float)A, (float)(A - (double)(float)A)};
    const dfl K1d = {(float)K1, (float)(K1 - (double)(float)K1)};
    const dfl K2d = {(float)K2, (float)(K2 - (double)(float)K2)};
    constexpr float K34PIh = (float)K34PI, K34PIl = (float)(K34PI - (double)(float)K34PI);
    const float rf = rho.h + rho.l;
    const dfl da = {0.5f * rho.h, 0.5f * rho.l};             // exact
    e = dfl{0.f, 0.f};
    v = 0.f;
    if (!(rf * 0.5f < 1e-10f)) {
        const float r3 = cbrtf(da.h);
        const dfl ex = df_mul(df_mul(FACd, da), dfl{2.f * r3, 0.f});   // 2 FAC da^(4/3)
        e = ex;
        v = VXf * r3;
    }
    if (!(rf < 1e-10f)) {
        // x^6 = (3 / 4 pi) / rho in FP32 (no division in FP64): K split hi + lo
        const float rinv = 1.f / rf;
        const float x = sqrtf(cbrtf(fmaf(K34PIh, rinv, K34PIl * rinv)));
        const float X = fmaf(x, x + Bf, Cf);
        const float L1 = logf(x * x / X);
        const float L2 = logf((x - X0f) * (x - X0f) / X);
        const float tb = 2.f * x + Bf;
        const float T = atanf(Qf / tb);
        // eps = A (L1 - K1 L2 + K2 T), ec = eps rho
        const dfl inner = df_add(df_sub(dfl{L1, 0.f}, df_mul(K1d, dfl{L2, 0.f})), df_mul(K2d, dfl{T, 0.f}));
        const dfl eps = df_mul(Ad, inner);
        e = df_add(e, df_mul(eps, rho));
        const float den = tb * tb + Q2f;
        const float deps = Af * (2.f / x - tb / X - 4.f * Bf / den -
                                 K1f * (2.f / (x - X0f) - tb / X - 4.f * (2.f * X0f + Bf) / den));
        v += (eps.h + eps.l) - (x / 6.f) * deps;
    }
}

}  // namespace dftg
