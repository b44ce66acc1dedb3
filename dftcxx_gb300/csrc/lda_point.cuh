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

}  // namespace dftg
