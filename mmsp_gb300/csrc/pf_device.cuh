// pf_device.cuh -- device arithmetic shared by the step and reduction kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "MMSP.gpu.h"
#include "pf_internal.h"

namespace pf {

// Arithmetic of the two forms.  The FP64 (plain) form rounds every operation
// separately with the _rn intrinsics, so nothing is fused into a
// multiply-add: that is how the reference's serial x86-64 build evaluates
// the same expressions, and it keeps the device result bit-identical to it.
// The FP32 (precision) form uses ordinary operators and lets the compiler
// contract them.
template <typename T> struct Ar;
template <> struct Ar<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
};
template <> struct Ar<float> {
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
};

// x^3 for the shipped examples' pow(x,3).  The exact cube is
// q + f + e*x with x*x = p + e and p*x = q + f split by the fused
// multiply-add error-free product (Dekker 1971; Ogita, Rump and Oishi 2005);
// rounding q + (f + e*x) once more gives the correctly rounded cube except
// in rare ties, within the 1-ulp bound of the C library's pow.
static __device__ __forceinline__ double cube(double x)
{
    double p = __dmul_rn(x, x);
    double e = __fma_rn(x, x, -p);
    double q = __dmul_rn(p, x);
    double f = __fma_rn(p, x, -q);
    return __dadd_rn(q, __fma_rn(e, x, f));
}
static __device__ __forceinline__ float cube(float x) { return x * x * x; }

// Model constants in the state type.
template <typename T> struct P {
    T wx, wy, wz;      // Laplacian weights of padded axes X, Y, Z
    T kappa, dtm, gamma2, neg_r, u;
    double noise;               // thermal noise standard deviation (0: none)
    unsigned long long seed;    // noise stream
    long long step;             // step index within the stream, when stepp is null
    const long long* stepp;     // device word holding the step index (a handle's step counter)
};

// The step index of the noise stream: the handle's device counter, so that
// graph replays of noisy steps draw each step's own deviates.
template <typename T>
static __device__ __forceinline__ long long step_of(const P<T>& p)
{
    return p.stepp ? *p.stepp : p.step;
}

// Value j of the SplitMix64 stream `seed` (Steele, Lea and Flood, OOPSLA
// 2014): the same function as mmsp_gb300/inputs.py and the oracle use.
static __device__ __forceinline__ unsigned long long splitmix64_at(unsigned long long seed, unsigned long long j)
{
    unsigned long long z = seed + (j + 1ULL) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Standard normal deviate k of stream `seed` by the Box-Muller transform of
// uniforms 2k and 2k+1 (top 53 bits): sqrt(-2 log(1 - u1)) cos(2 pi u2).
// Counter-based, so a cell's noise is the same wherever it is recomputed.
static __device__ __forceinline__ double gauss_at(unsigned long long seed, unsigned long long k)
{
    const double u1 = (double)(splitmix64_at(seed, 2ULL * k) >> 11) * 0x1.0p-53;
    const double u2 = (double)(splitmix64_at(seed, 2ULL * k + 1ULL) >> 11) * 0x1.0p-53;
    return sqrt(-2.0 * log(1.0 - u1)) * cos(6.283185307179586 * u2);
}

// The same deviate in single precision for the FP32 form, without FP64
// arithmetic: 1 - u1 is formed exactly in the integers from the 53-bit u1
// before it is rounded to float, so the logarithm keeps its accuracy as u1
// approaches 1; u2 keeps its top 24 bits.  Within a few 1e-7 of gauss_at.
static __device__ __forceinline__ float gauss_at_f(unsigned long long seed, unsigned long long k)
{
    const unsigned long long m1 = splitmix64_at(seed, 2ULL * k) >> 11;            // u1 = m1 * 2^-53
    const float t = (float)((1ULL << 53) - m1) * 0x1.0p-53f;                        // 1 - u1, in (0, 1]
    const float u2 = (float)(splitmix64_at(seed, 2ULL * k + 1ULL) >> 40) * 0x1.0p-24f;
    return sqrtf(-2.0f * logf(t)) * cosf(6.28318530717958648f * u2);
}

// The noise term of cell `cell` in the current step, std * N(0,1), as the
// examples' gaussian(0.0, std) returns it (model_A.cpp:13-40: ave + u*std),
// in the state type.
static __device__ __forceinline__ double noise_at(const P<double>& p, long long cells, long long cell)
{
    const unsigned long long k = (unsigned long long)step_of(p) * (unsigned long long)cells + (unsigned long long)cell;
    return 0.0 + gauss_at(p.seed, k) * p.noise;
}
static __device__ __forceinline__ float noise_at(const P<float>& p, long long cells, long long cell)
{
    const unsigned long long k = (unsigned long long)step_of(p) * (unsigned long long)cells + (unsigned long long)cell;
    return gauss_at_f(p.seed, k) * (float)p.noise;
}

// 2.0*y, which is exact.  For FP64 a normal y whose double stays finite is
// doubled by adding 1 to its exponent on the integer pipe; zeros,
// subnormals, values near overflow, infinities and NaNs take the multiply.
// Either way the bits are those of __dmul_rn(2.0, y).
static __device__ __forceinline__ double twice(double y)
{
    const long long b = __double_as_longlong(y);
    const unsigned e = (unsigned)((b >> 52) & 0x7ff);
    if (e - 1u < 2045u) return __longlong_as_double(b + (1LL << 52));
    return __dmul_rn(2.0, y);
}
static __device__ __forceinline__ float twice(float y) { return 2.0f * y; }

// 0.0 + t, which is t except that -0.0 becomes +0.0: a select on the bits
// instead of an FP64 add.
static __device__ __forceinline__ double plus_zero(double t)
{
    const long long b = __double_as_longlong(t);
    return b == (long long)0x8000000000000000ULL ? 0.0 : t;
}
static __device__ __forceinline__ float plus_zero(float t) { return t + 0.0f; }

// One axis of MMSP::laplacian (grid.cpp:2055-2064):
//   acc + weight * (yh - 2.0*y + yl), with y2 = 2.0*y precomputed (exact).
// FIRST marks the first axis, where acc is the initial 0.0.
template <typename T, bool UNIT_W, bool FIRST = false>
static __device__ __forceinline__ T lap_axis(T acc, T yh, T y2, T yl, T w)
{
    using A = Ar<T>;
    T t = A::add(A::sub(yh, y2), yl);
    if (!UNIT_W) t = A::mul(w, t);
    if (FIRST) return plus_zero(t);
    return A::add(acc, t);
}

// The whole Laplacian of a DIM-dimensional grid in the reference's axis
// order (axis 0 first): padded axes X (DIM 3), Y (DIM >= 2), Z.
template <typename T, bool UNIT_W, int DIM>
static __device__ __forceinline__ T lap_ref(T y2, T xh, T xl, T yh, T yl, T zh, T zl, T wx, T wy, T wz)
{
    T lap = T(0);
    if (DIM == 3) lap = lap_axis<T, UNIT_W, true>(lap, xh, y2, xl, wx);
    if (DIM == 3) lap = lap_axis<T, UNIT_W, false>(lap, yh, y2, yl, wy);
    if (DIM == 2) lap = lap_axis<T, UNIT_W, true>(lap, yh, y2, yl, wy);
    if (DIM >= 2) lap = lap_axis<T, UNIT_W, false>(lap, zh, y2, zl, wz);
    else lap = lap_axis<T, UNIT_W, true>(lap, zh, y2, zl, wz);
    return lap;
}

// kappa*lap, skipping the multiply when kappa is exactly 1 (1.0*x == x).
template <typename T>
static __device__ __forceinline__ T kappa_times(T kappa, T lap)
{
    return kappa == T(1) ? lap : Ar<T>::mul(kappa, lap);
}

// Chemical potential of the Cahn-Hilliard models.
template <typename T, int MODEL>
static __device__ __forceinline__ T ch_mu(T phi, T lap, const P<T>& p)
{
    using A = Ar<T>;
    if (MODEL == MMSP_GPU_CH) {
        // 2.0*phi*(1.0-phi)*(1.0-2.0*phi) - K*lap
        T t2 = twice(phi);
        T fp = A::mul(A::mul(t2, A::sub(T(1), phi)), A::sub(T(1), t2));
        return A::sub(fp, kappa_times(p.kappa, lap));
    } else {
        // -r*phi + u*pow(phi,3) - K*lap   (cahn-hilliard.cpp:71)
        T a = A::add(A::mul(p.neg_r, phi), A::mul(p.u, cube(phi)));
        return A::sub(a, kappa_times(p.kappa, lap));
    }
}

// New value of one order parameter of the Allen-Cahn models.
template <typename T, int MODEL>
static __device__ __forceinline__ T ac_new(T phi, T sum, T lap, const P<T>& p)
{
    using A = Ar<T>;
    if (MODEL == MMSP_GPU_AC) {
        // phi - dt*L*(-phi + phi*phi*phi + 2.0*gamma*phi*(sum - phi*phi) - kappa*lap)
        T p2 = A::mul(phi, phi);
        T p3 = A::mul(p2, phi);
        T a = A::add(-phi, p3);
        T g = A::mul(A::mul(p.gamma2, phi), A::sub(sum, p2));
        T c = A::sub(A::add(a, g), kappa_times(p.kappa, lap));
        return A::sub(phi, A::mul(p.dtm, c));
    } else if (MODEL == MMSP_GPU_GG || MODEL == MMSP_GPU_ZENER) {
        // phi - dt*(-phi - pow(phi,3) + 2.0*(phi*sum - lap))   (graingrowth.cpp:105, zener.cpp:135)
        T e = A::add(A::sub(-phi, cube(phi)), twice(A::sub(A::mul(phi, sum), lap)));
        return A::sub(phi, A::mul(p.dtm, e));
    } else {
        // phi - dt*M*(-r*phi + u*pow(phi,3) - K*lap)   (allen-cahn.cpp:70)
        T e = A::sub(A::add(A::mul(p.neg_r, phi), A::mul(p.u, cube(phi))), kappa_times(p.kappa, lap));
        return A::sub(phi, A::mul(p.dtm, e));
    }
}

// Periodic index: any integer onto [0, n), as repeated application of
// check_boundary's wrap (utility.cpp:47,51) would place it.
static __device__ __forceinline__ int wrapi(int v, int n)
{
    int r = v % n;
    return r < 0 ? r + n : r;
}

// v mod n for v in [-n, 2n): one compare and add instead of a division.
static __device__ __forceinline__ int wrap_near(int v, int n)
{
    return v < 0 ? v + n : (v >= n ? v - n : v);
}

// Model constants narrowed to the state type; padded axes X, Y, Z take the
// last `dim` real-axis weights.
template <typename T>
static inline P<T> narrow(const Coeffs& c, int dim)
{
    P<T> p;
    double w[3] = {1.0, 1.0, 1.0};
    for (int a = 0; a < dim; a++) w[3 - dim + a] = c.w[a];
    p.wx = (T)w[0];
    p.wy = (T)w[1];
    p.wz = (T)w[2];
    p.kappa = (T)c.kappa;
    p.dtm = (T)c.dtm;
    p.gamma2 = (T)c.gamma2;
    p.neg_r = (T)c.neg_r;
    p.u = (T)c.u;
    p.noise = c.noise;
    p.seed = c.seed;
    p.step = c.step;
    p.stepp = nullptr;
    return p;
}

}  // namespace pf
