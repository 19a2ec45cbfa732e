// Interval push kernels: Parker (16-component table) and focused transport
// (21 components), plain FP64 or mixed precision.
//
// The per-substep physics restates reference src/main.cpp:1131-1306 (Parker)
// and :1384-1733 (focused) once, templated on the arithmetic type.
//
// GB300 notes.  FP64 issues at a small fraction of the FP32 rate on this
// part, so the two paths differ in how they carry particle state:
//  * plain FP64: every operation in double, position wrap and cell search as
//    the reference computes them (parity within 1e-10 of the oracle);
//  * mixed: table, interpolation, coefficients and noise in FP32; the
//    position lives in a 64-bit fixed-point phase over the periodic width
//    (2^-64 of the domain, finer than FP64 near the domain edge), so the
//    periodic wrap is modular integer addition and the cell search (uniform
//    axis: a 64x64->128-bit multiply; stretched axis: exact integer compares
//    against fixed-point cell centres) runs on the integer pipes; time and
//    momentum accumulate in FP64.
//
// Scheduling: a persistent grid of warps pulls particles from a device
// cursor; a lane whose particle reached the interval end refills from the
// cursor, so warps stay full although particles need very different substep
// counts.  An optional permutation (a cell sort of particle indices) orders
// the work for cache locality without moving particle storage.  Noise is the
// keyed Philox stream (seed, particle index, frame), so results do not depend
// on the lane, launch shape or work order.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <type_traits>

#include "kpt_device.cuh"
#include "kpt_internal.h"
#include "kpt_pow.h"

// What this translation unit emits.  0 (the default): everything but the
// strict FP64 push and the FP64 table sampling, with FMA contraction and
// CUDA's pow in the FP64 push it does contain (the contracted mode); 1: only
// the strict FP64 push and FP64 sampling, compiled apart with FMA contraction
// off (kpt_push_f64.cu, nvcc -fmad=false) and the project pow, so their
// double arithmetic rounds exactly as written, as the host oracle's does (the
// oracle and the reference build use -ffp-contract=off).
#ifndef KPT_PUSH_PART
#define KPT_PUSH_PART 0
#endif

namespace kpt {
namespace {

constexpr double kSqrt3 = 1.7320508075688772935;

// FP32 square roots of the mixed path through sqrt.approx.f32 (a couple of
// ulp, like the path's other fast intrinsics): +2.3 % on the learned-closure
// push, no change on the plain-closure one.
#ifndef KPT_FAST_SQRT
#define KPT_FAST_SQRT 1
#endif

template <typename T>
struct Num;

template <>
struct Num<double> {
#if KPT_PUSH_PART == 1
    // the project pow (kpt_pow.h): rounds exactly as the host oracle does
    static __device__ __forceinline__ double pow(double a, double b) { return kpt_pow(a, b); }
#else
    // the contracted FP64 push: CUDA's pow
    static __device__ __forceinline__ double pow(double a, double b) { return ::pow(a, b); }
#endif
    static __device__ __forceinline__ double sqrt(double a) { return ::sqrt(a); }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
    static __device__ __forceinline__ bool finite(double a) { return isfinite(a); }
    static __device__ __forceinline__ double abs(double a) { return fabs(a); }
    // uniform_sqrt3 (RandomManager.hpp:111-114) on draw (lo, hi).
    static __device__ __forceinline__ double noise(uint32_t lo, uint32_t hi) {
        return __dadd_rn(-kSqrt3, __dmul_rn(kSqrt3 + kSqrt3, u01_f64(lo, hi)));
    }
};

template <>
struct Num<float> {
    // x^y for x >= 0 through the hardware exp2/log2 approximations.
    static __device__ __forceinline__ float pow(float a, float b) {
        return exp2f(b * __log2f(a));
    }
#if KPT_FAST_SQRT
    // sqrt.approx.f32: one MUFU-based instruction (sqrt(+0) = +0,
    // negative -> NaN, +inf -> +inf)
    static __device__ __forceinline__ float sqrt(float a) {
        float r;
        asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
        return r;
    }
#else
    static __device__ __forceinline__ float sqrt(float a) { return sqrtf(a); }
#endif
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ bool finite(float a) { return isfinite(a); }
    static __device__ __forceinline__ float abs(float a) { return fabsf(a); }
    static __device__ __forceinline__ float noise(uint32_t, uint32_t hi) {
        return -static_cast<float>(kSqrt3) + static_cast<float>(2.0 * kSqrt3) * u01_f32(hi);
    }
};

template <typename T>
__device__ __forceinline__ T square(T v) {
    return v * v;
}

template <typename T>
__device__ __forceinline__ T min_positive(T a, T b) {
    return a < b ? a : b;
}

template <typename T>
__device__ __forceinline__ T clamp_mu(T v, T m) {
    if (v > m) return m;
    if (v < -m) return -m;
    return v;
}

// The settings the substep physics reads, in the arithmetic type of the
// path (built once per launch on the host, so the FP32 path never converts
// a double inside the loop).
template <typename T>
struct Consts {
    T p0, gamma_turb, pindex, kpara0, kperp_over_kpara, drift_param1, drift_param2, charge;
    T particle_v0, duu0, h0, mu_max, dx, dy;
    T qlt_gk, qlt_h0, qlt_lc, qlt_sigma2, qlt_norm, qlt_omega0;
    int magnetic_dependency, momentum_dependency, closure;
};

template <typename T>
Consts<T> make_consts(const DeviceSettings& s) {
    Consts<T> k;
    k.p0 = s.p0;
    k.gamma_turb = s.gamma_turb;
    k.pindex = s.pindex;
    k.kpara0 = s.kpara0;
    k.kperp_over_kpara = s.kperp_over_kpara;
    k.drift_param1 = s.drift_param1;
    k.drift_param2 = s.drift_param2;
    k.charge = s.charge;
    k.particle_v0 = s.particle_v0;
    k.duu0 = s.duu0;
    k.h0 = s.h0;
    k.mu_max = s.mu_max;
    k.dx = s.dx;
    k.dy = s.dy;
    k.qlt_gk = s.qlt_gk;
    k.qlt_h0 = s.qlt_h0;
    k.qlt_lc = s.qlt_lc;
    k.qlt_sigma2 = s.qlt_sigma2;
    k.qlt_norm = s.qlt_norm;
    k.qlt_omega0 = s.qlt_omega0;
    k.magnetic_dependency = s.magnetic_dependency;
    k.momentum_dependency = s.momentum_dependency;
    k.closure = s.closure;
    return k;
}

// ------------------------------------------------------------ sampling
template <typename T>
struct Vec;
template <>
struct Vec<double> {
    using type = double2;
    static constexpr int width = 2;
};
template <>
struct Vec<float> {
    using type = float4;
    static constexpr int width = 4;
};

template <typename T>
__device__ __forceinline__ T vec_get(const typename Vec<T>::type& v, int k);
template <>
__device__ __forceinline__ double vec_get<double>(const double2& v, int k) {
    return k == 0 ? v.x : v.y;
}
template <>
__device__ __forceinline__ float vec_get<float>(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// 256-bit read-only loads (sm_100+): 8 floats or 4 doubles per lane and
// instruction, half the L1 wavefronts of 128-bit loads for the scattered
// table gathers.  Table rows are 32-byte aligned (64 B / 96 B FP32 rows,
// 128 B FP64 Parker rows; the focused FP64 row of 176 B keeps 128-bit loads).
__device__ __forceinline__ void load8(const float* p, float v[8]) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
          "=f"(v[7])
        : "l"(p));
}

__device__ __forceinline__ void load8(const double* p, double v[4]) {
    asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
        : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
        : "l"(p));
}

template <typename T, int STRIDE>
struct Wide {
    // elements per 256-bit load, and whether rows allow it
    static constexpr int width = sizeof(T) == 4 ? 8 : 4;
    static constexpr bool ok = (STRIDE * sizeof(T)) % 32 == 0;
};

// Bilinear sample of one frame (LinearPositionInterpolator::sample,
// FieldInterpolator.hpp:346-380): sum over corners (00, 10, 01, 11) of
// weight * value.  FP64 tables are point-major rows of STRIDE doubles; FP32
// tables are laid out in planes over `points` (table_f32_offset).
template <typename T, int C, int STRIDE>
__device__ __forceinline__ void sample_frame(const T* __restrict__ table, uint64_t points,
                                             const size_t pt[4], const T wc[4], T out[C]) {
    if constexpr (Wide<T, STRIDE>::ok) {
        constexpr int W = Wide<T, STRIDE>::width;
#pragma unroll
        for (int corner = 0; corner < 4; ++corner) {
#pragma unroll
            for (int chunk = 0; chunk < (C + W - 1) / W; ++chunk) {
                T v[W];
                if constexpr (sizeof(T) == 4) {
                    load8(table + table_f32_offset(C == 21, points, pt[corner], chunk * W), v);
                } else {
                    load8(table + pt[corner] * STRIDE + chunk * W, v);
                }
#pragma unroll
                for (int k = 0; k < W; ++k) {
                    const int comp = chunk * W + k;
                    if (comp < C) {
                        out[comp] = corner == 0 ? wc[0] * v[k] : out[comp] + wc[corner] * v[k];
                    }
                }
            }
        }
    } else {
        static_assert(sizeof(T) == 8, "FP32 tables are read in whole 256-bit chunks");
        using V = typename Vec<T>::type;
        constexpr int W = Vec<T>::width;
#pragma unroll
        for (int corner = 0; corner < 4; ++corner) {
            const V* src = reinterpret_cast<const V*>(table + pt[corner] * STRIDE);
#pragma unroll
            for (int chunk = 0; chunk < (C + W - 1) / W; ++chunk) {
                const V v = __ldg(src + chunk);
#pragma unroll
                for (int k = 0; k < W; ++k) {
                    const int comp = chunk * W + k;
                    if (comp < C) {
                        const T val = vec_get<T>(v, k);
                        out[comp] = corner == 0 ? wc[0] * val : out[comp] + wc[corner] * val;
                    }
                }
            }
        }
    }
}

// Time interpolation (src/main.cpp:1055-1077) of the two frames sampled at
// the same stencil.
template <typename T, int C, int STRIDE>
__device__ __forceinline__ void sample_stencil(const T* __restrict__ lower,
                                               const T* __restrict__ upper, uint64_t points,
                                               const size_t pt[4], const T wc[4], T uw,
                                               int use_time, T c[C]) {
    sample_frame<T, C, STRIDE>(lower, points, pt, wc, c);
    if (use_time == 0) {
        return;
    }
    T u[C];
    sample_frame<T, C, STRIDE>(upper, points, pt, wc, u);
    const T lw = T(1) - uw;
#pragma unroll
    for (int k = 0; k < C; ++k) {
        c[k] = lw * c[k] + uw * u[k];
    }
}

// Packed FP32 pairs (sm_100+ f32x2 arithmetic): two table components per
// instruction, carried in a 64-bit register.
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ unsigned long long f2_splat(float v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1,%1};" : "=l"(r) : "f"(v));
    return r;
}

__device__ __forceinline__ void f2_split(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0,%1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// 256-bit read-only load as four component pairs.
__device__ __forceinline__ void load4_pairs(const float* p, unsigned long long v[4]) {
    asm("ld.global.nc.v4.u64 {%0,%1,%2,%3}, [%4];"
        : "=l"(v[0]), "=l"(v[1]), "=l"(v[2]), "=l"(v[3])
        : "l"(p));
}

// Mixed path: the bilinear and the time interpolation in one pass over the
// eight corner points, on component pairs: c = sum over corners of
// (w (1 - uw)) lower + (w uw) upper (lower alone without time
// interpolation).  The 8 floats of chunk k of point p sit at
// table_f32_offset(p, 8 k) (Parker: chunk-major planes; focused: whole
// rows).  A point holds STRIDE floats (whole chunks, the components
// padded); the pair of the last odd component carries a padding value that
// is dropped.
template <int C, int STRIDE>
__device__ __forceinline__ void sample_stencil_pairs(const float* __restrict__ lower,
                                                     const float* __restrict__ upper,
                                                     uint64_t points, const size_t pt[4],
                                                     const float wc[4], float uw, int use_time,
                                                     float c[C]) {
    static_assert(STRIDE % 8 == 0, "points must hold whole 256-bit chunks");
    constexpr int kPairs = (C + 1) / 2;
    constexpr int kChunks = (C + 7) / 8;
    unsigned long long acc[kPairs];
    const float lw = use_time != 0 ? 1.0f - uw : 1.0f;
#pragma unroll
    for (int frame = 0; frame < 2; ++frame) {
        if (frame == 1 && use_time == 0) break;
        const float* table = frame == 0 ? lower : upper;
        const float tw = frame == 0 ? lw : uw;
#pragma unroll
        for (int corner = 0; corner < 4; ++corner) {
            const unsigned long long w2 = f2_splat(wc[corner] * tw);
#pragma unroll
            for (int chunk = 0; chunk < kChunks; ++chunk) {
                unsigned long long v[4];
                load4_pairs(table + table_f32_offset(C == 21, points, pt[corner], 8 * chunk), v);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int pair = chunk * 4 + k;
                    if (pair < kPairs) {
                        acc[pair] = frame == 0 && corner == 0 ? f2_mul(w2, v[k])
                                                              : f2_fma(w2, v[k], acc[pair]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int pair = 0; pair < kPairs; ++pair) {
        float lo, hi;
        f2_split(acc[pair], lo, hi);
        c[2 * pair] = lo;
        if (2 * pair + 1 < C) c[2 * pair + 1] = hi;
    }
}

__device__ __forceinline__ void corner_points(int lo0, int hi0, int lo1, int hi1, int ex,
                                              size_t pt[4]) {
    const size_t e = static_cast<size_t>(ex);
    pt[0] = static_cast<size_t>(lo0 + 2) + static_cast<size_t>(lo1 + 2) * e;
    pt[1] = static_cast<size_t>(hi0 + 2) + static_cast<size_t>(lo1 + 2) * e;
    pt[2] = static_cast<size_t>(lo0 + 2) + static_cast<size_t>(hi1 + 2) * e;
    pt[3] = static_cast<size_t>(hi0 + 2) + static_cast<size_t>(hi1 + 2) * e;
}

// FP64 path: the driver's own sampling arithmetic (src/main.cpp:1142-1148).
template <typename T, int C, int STRIDE>
__device__ __forceinline__ void sample_coefficients(const Grid& g, const T* __restrict__ lower,
                                                    const T* __restrict__ upper, double q0,
                                                    double q1, double rt, int use_time,
                                                    T c[C]) {
    const double c0 = grid_wrap(g.axis[0], q0);
    const double c1 = grid_wrap(g.axis[1], q1);
    int lo0, hi0, lo1, hi1;
    double w0, w1;
    axis_stencil(g.axis[0], c0, lo0, hi0, w0);
    axis_stencil(g.axis[1], c1, lo1, hi1, w1);
    const double a0 = 1.0 - w0;
    const double a1 = 1.0 - w1;
    const T wc[4] = {static_cast<T>(a0 * a1), static_cast<T>(w0 * a1), static_cast<T>(a0 * w1),
                     static_cast<T>(w0 * w1)};
    size_t pt[4];
    corner_points(lo0, hi0, lo1, hi1, g.ex, pt);
    const double uwd = rt < 0.0 ? 0.0 : (rt > 1.0 ? 1.0 : rt);
    const uint64_t points = static_cast<uint64_t>(g.ex) * static_cast<uint64_t>(g.axis[1].n + 4);
    sample_stencil<T, C, STRIDE>(lower, upper, points, pt, wc, static_cast<T>(uwd), use_time, c);
}

// ------------------------------------------------------------- physics
// Slab quasi-linear pitch-angle scattering (LegencyModel.hpp:557-645):
// D_mumu and dD_mumu/dmu at one (mu, Omega, v).
template <typename T>
__device__ __forceinline__ void qlt_scattering(T mu, T omega, T speed, const Consts<T>& s,
                                               T& dmumu, T& dmumu_dmu) {
    using N = Num<T>;
    dmumu = T(0);
    dmumu_dmu = T(0);
    const T one_minus_mu2 = T(1) - mu * mu;
    if (one_minus_mu2 <= T(0)) {
        return;
    }
    const T gk = s.qlt_gk;
    const T reg = N::abs(mu) + s.qlt_h0;
    const T xi = N::div(omega * s.qlt_lc, speed);
    const T reg_gk1 = N::pow(reg, gk - T(1));
    const T denominator = N::pow(reg, gk) + N::pow(xi, gk);
    const T prefactor = static_cast<T>(0.25 * 3.141592653589793238462643383279502884) * omega *
                        s.qlt_sigma2 * s.qlt_norm;
    dmumu = N::div(prefactor * one_minus_mu2 * xi * reg_gk1, denominator);
    if (dmumu == T(0) || mu == T(0)) {
        return;
    }
    const T sign_mu = mu > T(0) ? T(1) : T(-1);
    const T shape = sign_mu * (N::div(gk - T(1), reg) - N::div(gk * reg_gk1, denominator));
    const T endpoint = N::div(T(-2) * mu, one_minus_mu2);
    dmumu_dmu = dmumu * (endpoint + shape);
}

// Closure values served by the learned surrogate (mixed focused push).
struct Served {
    bool use;
    float kpara, duu, duu_du;
};

template <typename T>
struct Rates {
    T dx_dt, dy_dt, dp_dt, dmu_dt, duu;
    T skperp, skpara_perp, ib, bx, by, bz;
    T pitch_mu;
    T dt;        // limiter result (valid when !fixed_dt)
    bool fixed_dt;
};

// Coefficients, drift, dp/dt, dmu/dt and the step-size limiters of one
// substep (src/main.cpp:1167-1257 Parker, :1421-1630 focused).  Returns
// false where the reference sets status 2.
template <typename T, bool FOCUSED, bool SURR = false>
__device__ __forceinline__ bool physics(const T* c, T p, T pitch_mu, const Consts<T>& s,
                                        Rates<T>& r, const Served* served = nullptr) {
    using N = Num<T>;
    T vx, vy, bx, by, bz, b, dvx_dx, dvy_dy, dbx_dx, dbx_dy, dby_dx, dby_dy, dbz_dx, dbz_dy,
        db_dx, db_dy;
    T dvx_dy = 0, dvy_dx = 0, dvz_dx = 0, dvz_dy = 0;
    if (FOCUSED) {
        vx = c[0]; vy = c[1]; bx = c[3]; by = c[4]; bz = c[5]; b = c[6];
        dvx_dx = c[7]; dvx_dy = c[8]; dvy_dx = c[9]; dvy_dy = c[10]; dvz_dx = c[11];
        dvz_dy = c[12]; dbx_dx = c[13]; dbx_dy = c[14]; dby_dx = c[15]; dby_dy = c[16];
        dbz_dx = c[17]; dbz_dy = c[18]; db_dx = c[19]; db_dy = c[20];
    } else {
        vx = c[0]; vy = c[1]; bx = c[2]; by = c[3]; bz = c[4]; b = c[5]; dvx_dx = c[6];
        dvy_dy = c[7]; dbx_dx = c[8]; dbx_dy = c[9]; dby_dx = c[10]; dby_dy = c[11];
        dbz_dx = c[12]; dbz_dy = c[13]; db_dx = c[14]; db_dy = c[15];
    }
    if (!N::finite(p) || p <= T(0) || !N::finite(b) || b <= T(0)) {
        return false;
    }
    const T p0 = s.p0;
    const T gamma = s.gamma_turb;
    const T ib = N::div(T(1), b);
    const T ib2 = ib * ib;
    const T ib3 = ib2 * ib;

    T kpara;
    if (SURR && served->use) {
        kpara = served->kpara;
    } else {
        T knorm_para = T(1);
        if (s.magnetic_dependency == 1) {
            knorm_para *= N::pow(b, gamma - T(2));
        }
        T knorm = knorm_para;
        if (s.momentum_dependency == 1) {
            knorm *= N::pow(N::div(p, p0), s.pindex);
        }
        kpara = s.kpara0 * knorm;
    }
    const T kperp = kpara * s.kperp_over_kpara;
    if (!N::finite(kpara) || kpara <= T(0) || !N::finite(kperp) || kperp < T(0)) {
        return false;
    }
    const T skpara = N::sqrt(T(2) * kpara);
    const T skperp = N::sqrt(T(2) * kperp);
    T skpara_perp;
    if (FOCUSED) {
        skpara_perp = kpara > kperp ? N::sqrt(T(2) * (kpara - kperp)) : T(0);
    } else {
        skpara_perp = N::sqrt(T(2) * (kpara - kperp));
    }
    const T kpp = FOCUSED ? -kperp : kpara - kperp;

    T dkdx = T(0);
    T dkdy = T(0);
    if (s.magnetic_dependency == 1) {
        const T magnetic_exponent = gamma - T(2);
        dkdx = db_dx * ib * magnetic_exponent;
        dkdy = db_dy * ib * magnetic_exponent;
    }
    const T dkxx_dx = kperp * dkdx + kpp * dkdx * bx * bx * ib2 +
                      T(2) * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3;
    const T dkyy_dy = kperp * dkdy + kpp * dkdy * by * by * ib2 +
                      T(2) * kpp * by * (dby_dy * b - by * db_dy) * ib3;
    const T dkxy_dx = kpp * dkdx * bx * by * ib2 +
                      kpp * ((dbx_dx * by + bx * dby_dx) * ib2 - T(2) * bx * by * db_dx * ib3);
    const T dkxy_dy = kpp * dkdy * bx * by * ib2 +
                      kpp * ((dbx_dy * by + bx * dby_dy) * ib2 - T(2) * bx * by * db_dy * ib3);

    const T d1 = s.drift_param1;
    const T d2 = s.drift_param2;
    const T drift_denominator =
        N::sqrt(square(N::div(d1 * p0, p)) + square(N::div(d2 * p0 * p0, p * p)));

    T dx_dt, dy_dt, dp_dt;
    T dmu_dt = T(0), duu = T(0);
    if (FOCUSED) {
        pitch_mu = clamp_mu(pitch_mu, s.mu_max);
        const T mu2 = pitch_mu * pitch_mu;
        const T muf1 = T(0.5) * (T(1) - mu2);
        const T muf2 = T(0.5) * (T(3) * mu2 - T(1));
        const T kx = bx * dbx_dx + by * dbx_dy;
        const T ky = bx * dby_dx + by * dby_dy;
        const T kz = bx * dbz_dx + by * dbz_dy;
        const T bdot_curvb = bx * dbz_dy - by * dbz_dx + bz * (dby_dx - dbx_dy);
        const T vdp = N::div(N::div(T(1), s.charge), drift_denominator);
        const T vdx = vdp * (muf1 * (-bz * db_dy) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                             muf1 * bx * bdot_curvb * ib3);
        const T vdy = vdp * (muf1 * (bz * db_dx) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                             muf1 * by * bdot_curvb * ib3);
        const T speed = N::div(s.particle_v0 * p, p0);
        if (!N::finite(speed) || speed <= T(0)) {
            return false;
        }
        const T v_parallel_over_b = speed * pitch_mu * ib;
        dx_dt = vx + vdx + v_parallel_over_b * bx + dkxx_dx + dkxy_dy;
        dy_dt = vy + vdy + v_parallel_over_b * by + dkxy_dx + dkyy_dy;

        const T divv = dvx_dx + dvy_dy;
        const T bb_gradv = (bx * (bx * dvx_dx + by * dvx_dy) + by * (bx * dvy_dx + by * dvy_dy) +
                            bz * (bx * dvz_dx + by * dvz_dy)) *
                           ib2;
        const T bv_gradv = (bx * (vx * dvx_dx + vy * dvx_dy) + by * (vx * dvy_dx + vy * dvy_dy) +
                            bz * (vx * dvz_dx + vy * dvz_dy)) *
                           ib;
        const T acc_rate = -(muf1 * divv + muf2 * bb_gradv + N::div(pitch_mu * bv_gradv, speed));
        dp_dt = p * acc_rate;

        const T div_bnorm = -(bx * db_dx + by * db_dy) * ib2;
        dmu_dt = speed * div_bnorm + pitch_mu * divv - T(3) * pitch_mu * bb_gradv -
                 N::div(T(2) * bv_gradv, speed);
        dmu_dt *= T(0.5) * (T(1) - mu2);
        T duu_du = T(0);
        if (SURR && served->use) {
            duu = served->duu;
            duu_du = served->duu_du;
        } else if (s.closure != 0) {
            // slab QLT closure (extension): Omega = Omega_0 |B| / gamma
            const T omega = N::div(s.qlt_omega0 * b, N::sqrt(T(1) + p * p));
            qlt_scattering<T>(pitch_mu, omega, speed, s, duu, duu_du);
        } else {
            // the driver's reduced closure (src/main.cpp:1551-1589)
            const T abs_mu = N::abs(pitch_mu);
            const T dtmp = N::pow(abs_mu, gamma - T(1)) + s.h0;
            const T duu0 = s.duu0;
            duu = duu0 * (T(1) - mu2) * dtmp;
            if (pitch_mu > T(0)) {
                duu_du = duu0 * (T(-2) * pitch_mu * dtmp +
                                 (T(1) - mu2) * N::pow(abs_mu, gamma - T(2)));
            } else if (pitch_mu < T(0)) {
                duu_du = duu0 * (T(-2) * pitch_mu * dtmp -
                                 (T(1) - mu2) * N::pow(abs_mu, gamma - T(2)));
            }
            T duu_norm = T(1);
            if (s.magnetic_dependency == 1) {
                duu_norm *= N::pow(b, T(2) - gamma);
            }
            if (s.momentum_dependency == 1) {
                duu_norm *= N::pow(N::div(p, p0), gamma - T(1));
            }
            duu *= duu_norm;
            duu_du *= duu_norm;
        }
        dmu_dt += duu_du;
        if (!N::finite(dmu_dt) || !N::finite(duu) || duu < T(0)) {
            return false;
        }
    } else {
        const T vdp = N::div(N::div(T(1), T(3) * s.charge), drift_denominator);
        const T vdx = vdp * (dbz_dy * ib2 - T(2) * bz * db_dy * ib3);
        const T vdy = vdp * (-dbz_dx * ib2 + T(2) * bz * db_dx * ib3);
        dx_dt = vx + vdx + dkxx_dx + dkxy_dy;
        dy_dt = vy + vdy + dkxy_dx + dkyy_dy;
        const T divv = dvx_dx + dvy_dy;
        dp_dt = N::div(-p * divv, T(3));
    }

    // Step-size limiters (src/main.cpp:1243-1257, :1596-1650).
    const T dxs = s.dx;
    const T dys = s.dy;
    r.fixed_dt = false;
    r.dt = T(0);
    if (FOCUSED) {
        const T diffusion_scale = skperp > T(0) ? skperp : skpara;
        if (dx_dt != T(0) && dy_dt != T(0) && dp_dt != T(0) && dmu_dt != T(0) &&
            diffusion_scale > T(0)) {
            T dt = min_positive(square(N::div(T(0.5) * dxs, diffusion_scale)),
                                square(N::div(T(0.5) * dys, diffusion_scale)));
            dt = min_positive(dt, square(N::div(diffusion_scale, dx_dt)));
            dt = min_positive(dt, square(N::div(diffusion_scale, dy_dt)));
            dt = min_positive(dt, N::div(T(0.1) * p, N::abs(dp_dt)));
            dt = min_positive(dt, N::div(T(0.1), N::abs(dmu_dt)));
            dt = min_positive(dt, N::div(T(2) * duu, square(dmu_dt)));
            r.dt = dt;
        } else {
            r.fixed_dt = true;
        }
    } else if (dx_dt != T(0) && dy_dt != T(0) && dp_dt != T(0)) {
        const T advection_scale = skperp > T(0) ? skperp : skpara;
        T dt = min_positive(square(N::div(T(0.5) * dxs, skpara)),
                            square(N::div(T(0.5) * dys, skpara)));
        dt = min_positive(dt, square(N::div(advection_scale, dx_dt)));
        dt = min_positive(dt, square(N::div(advection_scale, dy_dt)));
        dt = min_positive(dt, N::div(T(0.1) * p, N::abs(dp_dt)));
        r.dt = dt;
    } else {
        r.fixed_dt = true;
    }
    r.dx_dt = dx_dt;
    r.dy_dt = dy_dt;
    r.dp_dt = dp_dt;
    r.dmu_dt = dmu_dt;
    r.duu = duu;
    r.skperp = skperp;
    r.skpara_perp = skpara_perp;
    r.ib = ib;
    r.bx = bx;
    r.by = by;
    r.bz = bz;
    r.pitch_mu = pitch_mu;
    return true;
}

// Displacements and the new pitch cosine from the four draws of a substep
// (src/main.cpp:1280-1291 Parker, :1660-1702 focused).
template <typename T, bool FOCUSED>
__device__ __forceinline__ void increments(const Rates<T>& r, T dt, const uint4& r0,
                                           const uint4& r1, const Consts<T>& s, T& delta_x,
                                           T& delta_y, T& new_mu) {
    using N = Num<T>;
    const T sdt = N::sqrt(dt);
    if (FOCUSED) {
        const T ran1 = N::noise(r0.x, r0.y);
        const T ran2 = N::noise(r0.z, r0.w);
        const T pitch_random = N::noise(r1.z, r1.w);
        const T bxn = r.bx * r.ib;
        const T byn = r.by * r.ib;
        const T bzn = r.bz * r.ib;
        const T bxy_norm = N::sqrt(bxn * bxn + byn * byn);
        T stochastic_x = T(0);
        T stochastic_y = T(0);
        if (bxy_norm > T(0)) {
            const T ibxy_norm = N::div(T(1), bxy_norm);
            // (-by, +bx) on ran2 as written in src/main.cpp:1682-1687.
            stochastic_x = r.skperp * ibxy_norm * sdt * (-bxn * bzn * ran1 - r.by * ran2);
            stochastic_y = r.skperp * ibxy_norm * sdt * (-byn * bzn * ran1 + r.bx * ran2);
        }
        delta_x = r.dx_dt * dt + stochastic_x;
        delta_y = r.dy_dt * dt + stochastic_y;
        new_mu = clamp_mu(r.pitch_mu + r.dmu_dt * dt + pitch_random * N::sqrt(T(2) * r.duu) * sdt,
                          s.mu_max);
    } else {
        const T ran1 = N::noise(r0.x, r0.y);
        const T ran2 = N::noise(r0.z, r0.w);
        const T ran3 = N::noise(r1.x, r1.y);
        delta_x = r.dx_dt * dt + ran1 * r.skperp * sdt + ran3 * r.skpara_perp * sdt * r.bx * r.ib;
        delta_y = r.dy_dt * dt + ran2 * r.skperp * sdt + ran3 * r.skpara_perp * sdt * r.by * r.ib;
        new_mu = r.pitch_mu;
    }
}

struct PushParams {
    Grid grid;
    FixedGrid fixed;
    Consts<double> kd;
    Consts<float> kf;
    const void* lower;
    const void* upper;
    uint64_t table_points;  // ghosted points of a table (chunk plane of FP32 tables)
    ParticleArrays parts;
    const uint32_t* order;  // optional work order (permutation of [0, count))
    uint64_t count;
    DeviceSettings s;
    double interval_start;
    double interval_end;
    float inv_mhd_dt;
    uint32_t frame;
    uint2 key;
    PushCounters* counters;
    SurrogateDevice sg;  // used by the surrogate instantiation only
    const float* records;  // cell records of (lower, upper); nullptr: point-major sampling
};

// ------------------------------------------------------------- FP64 path
struct StateF64 {
    double x, y, p, t, diag_dt, mu;
    int steps;
    int status;
    uint32_t index;
};

// The first part of an FP64 substep: count it, wrap the position and sample
// the time-interpolated table at the shifted position.
template <bool FOCUSED>
__device__ __forceinline__ void sample_f64(StateF64& st, const PushParams& P,
                                           double c[FOCUSED ? 21 : 16]) {
    constexpr int C = FOCUSED ? 21 : 16;
    constexpr int STRIDE = FOCUSED ? 22 : 16;
    const DeviceSettings& s = P.s;
    ++st.steps;
    st.x = wrap_driver(st.x, s.x_lower, s.x_upper, s.x_width);
    st.y = wrap_driver(st.y, s.y_lower, s.y_upper, s.y_width);
    const double rt = __ddiv_rn(__dsub_rn(st.t, P.interval_start), s.mhd_dt);
    sample_coefficients<double, C, STRIDE>(P.grid, static_cast<const double*>(P.lower),
                                           static_cast<const double*>(P.upper),
                                           __dadd_rn(st.x, s.shift_x), __dadd_rn(st.y, s.shift_y),
                                           rt, s.time_interpolation, c);
}

// The rest of an FP64 substep from the sampled table values: physics (with
// the served closure when SURR), step size, noise and the update.
template <bool FOCUSED, bool SURR = false>
__device__ __forceinline__ bool advance_f64(StateF64& st, const PushParams& P, const double* c,
                                            const Served* served = nullptr) {
    const DeviceSettings& s = P.s;
    Rates<double> r;
    if (!physics<double, FOCUSED, SURR>(c, st.p, st.mu, P.kd, r, served)) {
        st.status = 2;
        return false;
    }
    double dt = r.fixed_dt ? s.dt_min : r.dt;
    if (dt < s.dt_min) dt = s.dt_min;
    if (dt > s.dt_max) dt = s.dt_max;
    st.diag_dt = dt;
    const double remaining = __dsub_rn(P.interval_end, st.t);
    if (dt > remaining) dt = remaining;
    if (!isfinite(dt) || dt <= 0.0) {
        st.status = 2;
        return false;
    }
    const uint32_t block = 2u * static_cast<uint32_t>(st.steps - 1);
    const uint4 r0 = philox4x32_10(make_uint4(block, st.index, P.frame, kTagPush), P.key);
    const uint4 r1 = philox4x32_10(make_uint4(block + 1u, st.index, P.frame, kTagPush), P.key);
    double dx, dy, mu;
    increments<double, FOCUSED>(r, dt, r0, r1, P.kd, dx, dy, mu);
    st.mu = mu;
    st.x = __dadd_rn(st.x, dx);
    st.y = __dadd_rn(st.y, dy);
    st.p = __dadd_rn(st.p, r.dp_dt * dt);
    st.t = __dadd_rn(st.t, dt);
    const double pfloor = 0.25 * s.p0;
    if (st.p < pfloor) st.p = pfloor;
    if (!isfinite(st.x) || !isfinite(st.y) || !isfinite(st.p) || !isfinite(st.t)) {
        st.status = 2;
        return false;
    }
    return st.t < P.interval_end && st.steps < s.max_steps;
}

template <bool FOCUSED>
__device__ __forceinline__ bool substep(StateF64& st, const PushParams& P) {
    double c[FOCUSED ? 21 : 16];
    sample_f64<FOCUSED>(st, P, c);
    return advance_f64<FOCUSED>(st, P, c);
}

template <bool FOCUSED>
__device__ __forceinline__ void load(StateF64& st, const PushParams& P, uint32_t index) {
    const ParticleArrays& a = P.parts;
    st.index = index;
    st.x = a.x[index];
    st.y = a.y[index];
    st.p = a.p[index];
    st.t = a.t[index];
    st.diag_dt = a.step_dt[index];
    st.mu = FOCUSED ? clamp_mu(a.mu[index], P.s.mu_max) : 0.0;
    st.steps = 0;
    st.status = 0;
}

template <bool FOCUSED>
__device__ __forceinline__ void store(StateF64& st, const PushParams& P) {
    const ParticleArrays& a = P.parts;
    const DeviceSettings& s = P.s;
    if (st.steps >= s.max_steps && st.t < P.interval_end) st.status = 2;
    const uint32_t i = st.index;
    a.x[i] = wrap_driver(st.x, s.x_lower, s.x_upper, s.x_width);
    a.y[i] = wrap_driver(st.y, s.y_lower, s.y_upper, s.y_width);
    a.p[i] = st.p;
    a.t[i] = st.t;
    a.step_dt[i] = st.diag_dt;
    if (FOCUSED) a.mu[i] = st.mu;
    a.status[i] = st.status;
}

__device__ __forceinline__ bool live(const StateF64& st, const PushParams& P) {
    return st.t < P.interval_end && st.steps < P.s.max_steps;
}

// ------------------------------------------------------------ mixed path
// No FP64 instruction runs inside the mixed substep loop:
//  * position: 64-bit fixed-point phase over each periodic width;
//  * time: 64-bit fixed-point fraction of the interval (2^62 = interval
//    end), so the last step lands exactly on the interval end;
//  * momentum: an unevaluated pair of floats (hi + lo, ~48-bit significand)
//    updated with an error-free sum.
// FP64 is used once per particle and push, to convert state in and out.
struct StateMixed {
    uint64_t px, py;   // phase over the periodic widths
    long long tau;     // (t - interval_start) / mhd_dt * 2^62
    float p_hi, p_lo;  // momentum = p_hi + p_lo
    float mu, diag_dt;
    int steps;
    int status;
    uint32_t index;
};

constexpr long long kTauEnd = 1ll << 62;

// Exact float -> int64 (truncation) with integer operations only.
__device__ __forceinline__ long long float_to_s64(float f) {
    const int bits = __float_as_int(f);
    const int e = ((bits >> 23) & 0xff) - 150;
    const long long m = static_cast<long long>((bits & 0x7fffff) | 0x800000);
    long long v;
    if (e >= 0) {
        v = e < 40 ? (m << e) : 0x7fffffffffffffffll;
    } else {
        v = e > -24 ? (m >> (-e)) : 0;
    }
    return bits < 0 ? -v : v;
}

// Non-negative int64 below 2^63 -> float from its top bits (integer pipe
// plus one 32-bit conversion).
__device__ __forceinline__ float s64_to_float_scaled(long long v, float scale_2_32) {
    return static_cast<float>(static_cast<uint32_t>(static_cast<unsigned long long>(v) >> 32)) *
               scale_2_32 +
           static_cast<float>(static_cast<uint32_t>(v)) * (scale_2_32 * (1.0f / 4294967296.0f));
}

// Cell index and upper weight of the driver's stencil for a fixed-point
// position q (already shifted by half a mean cell), uniform axis:
// logical = q*n/2^64 - 1/2 from one 64x64->128-bit product.
__device__ __forceinline__ void fixed_stencil_uniform(uint64_t q, int n, int& lo, float& w) {
    const uint64_t hi = __umul64hi(q, static_cast<uint64_t>(n));
    const uint64_t frac = q * static_cast<uint64_t>(n);
    const uint64_t shifted = frac - (1ull << 63);
    const int borrow = frac < (1ull << 63) ? 1 : 0;
    lo = static_cast<int>(hi) - borrow;
    w = static_cast<float>(static_cast<uint32_t>(shifted >> 40)) * (1.0f / 16777216.0f);
}

// Stretched axis: find k with C[k] <= q < C[k+1] among the fixed-point
// ghosted cell centres (exact integer compares), seeded by a bucket table.
__device__ __forceinline__ void fixed_stencil_stored(const FixedAxis& a, uint64_t q, int& lo,
                                                     float& w) {
    const long long qy = static_cast<long long>(q >> 2);  // 2^62 scale
    int k = __ldg(a.buckets + static_cast<int>(q >> a.bucket_shift));
    while (k < a.n && __ldg(a.centers + k + 3) <= qy) {
        ++k;
    }
    while (k > -2 && __ldg(a.centers + k + 2) > qy) {
        --k;
    }
    lo = k;
    const unsigned long long d = static_cast<unsigned long long>(qy - __ldg(a.centers + k + 2));
    w = static_cast<float>(static_cast<uint32_t>(d >> a.spacing_shift)) *
        __ldg(a.inv_spacing + k + 2);
}

// hi + lo += d (error-free sum, then renormalise).
__device__ __forceinline__ void add_pair(float& hi, float& lo, float d) {
    const float s = hi + d;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (d - bb);
    const float l = lo + err;
    hi = s + l;
    lo = l - (hi - s);
}

// The fixed-point stencil of a mixed particle: the cell's lower-left ghosted
// point, the axis weights and the clamped time weight.
__device__ __forceinline__ void mixed_stencil(const StateMixed& st, const PushParams& P,
                                              size_t& cell, float& w0, float& w1, float& rt) {
    const FixedGrid& F = P.fixed;
    const uint64_t qx = st.px + F.axis[0].half_cell;
    const uint64_t qy = st.py + F.axis[1].half_cell;
    int lo0, lo1;
    if (F.axis[0].stored) {
        fixed_stencil_stored(F.axis[0], qx, lo0, w0);
    } else {
        fixed_stencil_uniform(qx, F.axis[0].n, lo0, w0);
    }
    if (F.axis[1].stored) {
        fixed_stencil_stored(F.axis[1], qy, lo1, w1);
    } else {
        fixed_stencil_uniform(qy, F.axis[1].n, lo1, w1);
    }
    cell = static_cast<size_t>(lo0 + 2) +
           static_cast<size_t>(lo1 + 2) * static_cast<size_t>(P.grid.ex);
    rt = st.tau <= 0 ? 0.0f : s64_to_float_scaled(st.tau, 1.0f / 1073741824.0f);
    rt = rt > 1.0f ? 1.0f : rt;
}

// Table values at the particle (fixed-point stencil, time interpolation),
// from the point-major tables.
template <bool FOCUSED>
__device__ __forceinline__ void sample_mixed(const StateMixed& st, const PushParams& P,
                                             float (&c)[FOCUSED ? 21 : 16]) {
    constexpr int C = FOCUSED ? 21 : 16;
    constexpr int STRIDE = FOCUSED ? 24 : 16;
    size_t cell;
    float w0, w1, rt;
    mixed_stencil(st, P, cell, w0, w1, rt);
    const float a0 = 1.0f - w0;
    const float a1 = 1.0f - w1;
    const float wc[4] = {a0 * a1, w0 * a1, a0 * w1, w0 * w1};
    const size_t ex = static_cast<size_t>(P.grid.ex);
    const size_t pt[4] = {cell, cell + 1, cell + ex, cell + ex + 1};
    sample_stencil_pairs<C, STRIDE>(static_cast<const float*>(P.lower),
                                    static_cast<const float*>(P.upper), P.table_points, pt, wc,
                                    rt, P.s.time_interpolation, c);
}

// Per-warp shared memory of the record sampler: 32 rows of the components
// rounded up to whole pairs (row strides of 22 and 18 floats keep its 64-bit
// stores and loads free of bank conflicts).
__host__ __device__ constexpr int record_xpose_stride(bool focused) {
    return focused ? 22 : 18;
}
__host__ __device__ constexpr size_t record_xpose_bytes(bool focused, int warps) {
    return static_cast<size_t>(warps) * 32u * record_xpose_stride(focused) * sizeof(float);
}

// Warp-collective sampling from the cell records (every lane calls it,
// converged; rec = the lane's cell record, any valid record for a lane
// without a particle).  Lanes 4g..4g+3 form a group: for each of the
// group's four particles in turn, lane 4g+s reads the sectors of component
// pairs s, s+4, s+8 of that particle's record -- one 128-byte line per
// request for the group -- and interpolates each pair from its own sectors
// with the eight corner weights, in the operations and the order of
// sample_stencil_pairs, so the values equal the point-major sampler's bit
// for bit.  The pairs then reach their particle's lane through the warp's
// rows of shared memory.
// Particles of a group whose requests the sampler unrolls together (4: all
// of the group's loads may be in flight at once, register pressure allowing).
#ifndef KPT_RECORD_Q_UNROLL
#define KPT_RECORD_Q_UNROLL 4
#endif
constexpr int kRecordQUnroll = KPT_RECORD_Q_UNROLL;
template <bool FOCUSED, bool USE_TIME>
__device__ __forceinline__ void sample_records(const float* rec, float w0, float w1, float rt,
                                               float (&c)[FOCUSED ? 21 : 16], float* xpose) {
    constexpr int C = FOCUSED ? 21 : 16;
    constexpr int GROUPS = record_sectors(FOCUSED) / 8;  // line pairs (frames 0 and 1)
    constexpr int XS = record_xpose_stride(FOCUSED);
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned group = lane & ~3u;
    const int s = static_cast<int>(lane & 3u);
    const unsigned long long my_rec = reinterpret_cast<unsigned long long>(rec);
#pragma unroll kRecordQUnroll
    for (int q = 0; q < 4; ++q) {
        const int src = static_cast<int>(group) + q;
        const unsigned long long qrec = __shfl_sync(full, my_rec, src);
        const float qw0 = __shfl_sync(full, w0, src);
        const float qw1 = __shfl_sync(full, w1, src);
        const float qrt = USE_TIME ? __shfl_sync(full, rt, src) : 0.0f;
        const float a0 = 1.0f - qw0;
        const float a1 = 1.0f - qw1;
        const float wc[4] = {a0 * a1, qw0 * a1, a0 * qw1, qw0 * qw1};
        const float lw = USE_TIME ? 1.0f - qrt : 1.0f;
        unsigned long long w_lo[4], w_hi[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            w_lo[k] = f2_splat(wc[k] * lw);
            if (USE_TIME) w_hi[k] = f2_splat(wc[k] * qrt);
        }
        const float* sector = reinterpret_cast<const float*>(qrec) + 8 * s;
        float* row = xpose + (group + q) * XS;
#pragma unroll
        for (int m = 0; m < GROUPS; ++m) {
            unsigned long long v[4];
            load4_pairs(sector + 64 * m, v);
            unsigned long long acc = f2_mul(w_lo[0], v[0]);
#pragma unroll
            for (int k = 1; k < 4; ++k) acc = f2_fma(w_lo[k], v[k], acc);
            if (USE_TIME) {
                load4_pairs(sector + 64 * m + 32, v);
#pragma unroll
                for (int k = 0; k < 4; ++k) acc = f2_fma(w_hi[k], v[k], acc);
            }
            const int first = 2 * (4 * m + s);
            if (8 * m + 7 < C || first < C) {
                *reinterpret_cast<unsigned long long*>(row + first) = acc;
            }
        }
    }
    __syncwarp();
    const unsigned long long* mine = reinterpret_cast<const unsigned long long*>(xpose + lane * XS);
#pragma unroll
    for (int k = 0; k < (C + 1) / 2; ++k) {
        float lo, hi;
        f2_split(mine[k], lo, hi);
        c[2 * k] = lo;
        if (2 * k + 1 < C) c[2 * k + 1] = hi;
    }
    __syncwarp();
}

// Warp-collective mixed sampling: the record sampler when the push has cell
// records (xpose = the warp's shared rows), else the point-major sampler on
// the lanes that hold a particle.
template <bool FOCUSED>
__device__ __forceinline__ void sample_mixed_warp(const StateMixed& st, const PushParams& P,
                                                  bool have, float (&c)[FOCUSED ? 21 : 16],
                                                  float* xpose) {
    if (xpose != nullptr) {
        size_t cell = 0;
        float w0 = 0.0f, w1 = 0.0f, rt = 0.0f;
        if (have) mixed_stencil(st, P, cell, w0, w1, rt);
        const float* rec = P.records + cell * record_floats(FOCUSED);
        if (P.s.time_interpolation != 0) {
            sample_records<FOCUSED, true>(rec, w0, w1, rt, c, xpose);
        } else {
            sample_records<FOCUSED, false>(rec, w0, w1, rt, c, xpose);
        }
    } else if (have) {
        sample_mixed<FOCUSED>(st, P, c);
    }
}

// Physics, step size, noise and the state update of one substep.
template <bool FOCUSED, bool SURR = false>
__device__ __forceinline__ bool advance_mixed(StateMixed& st, const PushParams& P,
                                              const float (&c)[FOCUSED ? 21 : 16],
                                              const Served* served = nullptr) {
    const DeviceSettings& s = P.s;
    const FixedGrid& F = P.fixed;
    Rates<float> r;
    if (!physics<float, FOCUSED, SURR>(c, st.p_hi, st.mu, P.kf, r, served)) {
        st.status = 2;
        return false;
    }
    float dtf = r.fixed_dt ? F.dt_min : r.dt;
    if (dtf < F.dt_min) dtf = F.dt_min;
    if (dtf > F.dt_max) dtf = F.dt_max;
    st.diag_dt = dtf;
    long long dtau = float_to_s64(dtf * F.tau_per_time);
    const long long remaining = kTauEnd - st.tau;
    if (dtau >= remaining) {
        dtau = remaining;
        dtf = s64_to_float_scaled(remaining, F.time_per_tau_2_32);
    }
    if (!(dtf > 0.0f) || !isfinite(dtf) || dtau <= 0) {
        st.status = 2;
        return false;
    }
    const uint32_t block = 2u * static_cast<uint32_t>(st.steps - 1);
    const uint4 r0 = philox4x32_10(make_uint4(block, st.index, P.frame, kTagPush), P.key);
    const uint4 r1 = philox4x32_10(make_uint4(block + 1u, st.index, P.frame, kTagPush), P.key);
    float dx, dy, mu;
    increments<float, FOCUSED>(r, dtf, r0, r1, P.kf, dx, dy, mu);
    const float dp = r.dp_dt * dtf;
    if (!isfinite(dx) || !isfinite(dy) || !isfinite(dp)) {
        st.status = 2;
        return false;
    }
    st.mu = mu;
    st.px += static_cast<uint64_t>(float_to_s64(dx * F.axis[0].to_fixed));
    st.py += static_cast<uint64_t>(float_to_s64(dy * F.axis[1].to_fixed));
    add_pair(st.p_hi, st.p_lo, dp);
    st.tau += dtau;
    if (st.p_hi < F.pfloor_hi) {
        st.p_hi = F.pfloor_hi;
        st.p_lo = F.pfloor_lo;
    }
    return st.tau < kTauEnd && st.steps < s.max_steps;
}

template <bool FOCUSED>
__device__ __forceinline__ bool substep(StateMixed& st, const PushParams& P) {
    ++st.steps;
    float c[FOCUSED ? 21 : 16];
    sample_mixed<FOCUSED>(st, P, c);
    return advance_mixed<FOCUSED>(st, P, c);
}

// The same substep, warp-collective over the cell records (every lane calls
// it; lanes without a particle only help sample).
template <bool FOCUSED>
__device__ __forceinline__ bool substep_records(StateMixed& st, const PushParams& P, bool have,
                                                float* xpose) {
    if (have) ++st.steps;
    float c[FOCUSED ? 21 : 16];
    sample_mixed_warp<FOCUSED>(st, P, have, c, xpose);
    return have && advance_mixed<FOCUSED>(st, P, c);
}

// Per-lane tallies of the surrogate judge.
struct JudgeTally {
    unsigned long long evaluations, judged, fallbacks;
    float max_error;
};

// The closure values of one lane, in FP32: the network's normalised outputs
// y mapped back to D_mumu, dD_mumu/dmu and kappa_parallel (use = inside the
// training box), with the plain slab-QLT closure evaluated beside them in
// FP32 to judge one substep in judge_period, to blend over [mu_cut,
// 2 mu_cut] and to serve the lanes outside the box.  All of a warp's lanes
// that need the plain closure take it in this one branch, so a warp
// evaluates it at most once per substep.  A lane whose plain values are not
// finite and positive returns use = false: the physics then evaluates the
// plain closure in its own precision.
__device__ __forceinline__ Served serve_closure(const PushParams& P, bool use, float mu,
                                                float b, float p, int steps,
                                                const float (&y)[kMlpOut], JudgeTally& tally) {
    const SurrogateBox& box = P.sg.box;
    Served served;
    served.use = use;
    const float amu = fabsf(mu);
    const float sign = mu > 0.0f ? 1.0f : -1.0f;
    if (use) {
        const float y0 = y[0] * box.out_scale[0] + box.out_offset[0];
        const float y1 = y[1] * box.out_scale[1] + box.out_offset[1];
        const float y2 = y[2] * box.out_scale[2] + box.out_offset[2];
        const float one_minus_mu2 = 1.0f - mu * mu;
        served.duu = one_minus_mu2 * __expf(y0);
        served.duu_du = served.duu * (__fdividef(sign * y1, amu + P.kf.qlt_h0) -
                                      __fdividef(2.0f * mu, one_minus_mu2));
        served.kpara = __expf(y2);
        ++tally.evaluations;
    } else {
        ++tally.fallbacks;
    }
    const bool blend = use && amu < 2.0f * box.mu_cut;
    const bool judge = use && (steps & (P.sg.judge_period - 1)) == 0;
    if (blend || judge || !use) {
        const Consts<float>& k = P.kf;
        const float speed = __fdividef(k.particle_v0 * p, k.p0);
        const float omega = __fdividef(k.qlt_omega0 * b, Num<float>::sqrt(1.0f + p * p));
        float duu, duu_du;
        qlt_scattering<float>(mu, omega, speed, k, duu, duu_du);
        // kappa_parallel in the order the physics forms it
        float knorm = 1.0f;
        if (k.magnetic_dependency == 1) knorm *= Num<float>::pow(b, k.gamma_turb - 2.0f);
        if (k.momentum_dependency == 1) knorm *= Num<float>::pow(__fdividef(p, k.p0), k.pindex);
        const float kpara = k.kpara0 * knorm;
        if (judge) {
            const float e_d = fabsf(served.duu - duu) / duu;
            const float e_k = fabsf(served.kpara - kpara) / kpara;
            const float e = fmaxf(e_d, e_k);
            tally.max_error = isfinite(e) ? fmaxf(tally.max_error, e) : INFINITY;
            ++tally.judged;
        }
        if (blend) {
            // continuous hand-over to the plain closure below mu_cut: a
            // linear blend over [mu_cut, 2 mu_cut], with the weight's
            // derivative in dD/dmu so the Ito drift stays consistent
            const float w = __fdividef(amu - box.mu_cut, box.mu_cut);
            const float dw = __fdividef(sign, box.mu_cut);
            const float dd = served.duu - duu;
            served.duu_du = duu_du + w * (served.duu_du - duu_du) + dw * dd;
            served.duu = duu + w * dd;
            served.kpara = kpara + w * (served.kpara - kpara);
        }
        if (!use) {
            served.duu = duu;
            served.duu_du = duu_du;
            served.kpara = kpara;
            served.use = isfinite(duu) && duu >= 0.0f && isfinite(duu_du) && isfinite(kpara) &&
                         kpara > 0.0f;
        }
    }
    return served;
}

// Warp-collective focused substep with the learned closure.  Every lane of
// the warp calls it (converged); lanes without a particle (have = false)
// feed zero rows to the network and return false.  Lanes whose inputs leave
// the training box, or with |mu| < mu_cut, use the plain closure; one
// substep in judge_period of each particle also evaluates the plain closure
// and records the larger relative error of D_mumu and kappa_parallel.
// TC = true serves the network on the tensor cores, block-collective (every
// thread of the block calls it); *stop is then set, uniformly over the
// block, when a completion wait timed out (the substep is abandoned).
template <bool FP16, int H, bool TC = false>
__device__ __forceinline__ bool substep_surrogate(StateMixed& st, const PushParams& P, bool have,
                                                  const uint2* smem, JudgeTally& tally,
                                                  float* xpose, TcNet* net = nullptr,
                                                  bool* fail = nullptr, bool* stop = nullptr) {
    const SurrogateDevice& sg = P.sg;
    const SurrogateBox& box = sg.box;
    float c[21];
    float f[kMlpIn] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool use = false;
    float mu = 0.0f;
    if (have) ++st.steps;
    sample_mixed_warp<true>(st, P, have, c, xpose);
    if (have) {
        mu = clamp_mu(st.mu, P.kf.mu_max);
        const float b = c[6];
        const float p = st.p_hi;
        const float amu = fabsf(mu);
        if (sg.constants_in_box && amu >= box.mu_cut && b > 0.0f && p > 0.0f) {
            const float lm = __logf(amu);
            const float lp = __logf(p);
            const float lb = __logf(b);
            use = lm <= box.in_hi[0] && lp >= box.in_lo[1] && lp <= box.in_hi[1] &&
                  lb >= box.in_lo[2] && lb <= box.in_hi[2];
            if (use) {
                f[0] = lm * box.in_scale[0] + box.in_offset[0];
                f[1] = lp * box.in_scale[1] + box.in_offset[1];
                f[2] = lb * box.in_scale[2] + box.in_offset[2];
                f[3] = sg.f3;
                f[4] = sg.f4;
            }
        }
    }
    float y[kMlpOut];
    if constexpr (TC) {
        __syncwarp();
        *stop = mlp_cta<FP16, H>(*net, f, y, *fail);
        if (*stop) {
            return false;
        }
    } else {
        __syncwarp();
        mlp_warp<FP16, H>(smem, f, y);
    }
    if (!have) {
        return false;
    }
    const Served served = serve_closure(P, use, mu, c[6], st.p_hi, st.steps, y, tally);
    return advance_mixed<true, true>(st, P, c, &served);
}

// The FP64 focused substep with the learned closure, warp-collective on the
// mma.sync engine (as the mixed one above): the table is sampled and the
// physics evaluated in FP64, the network serves D_mumu, dD_mumu/dmu and
// kappa_parallel in place of the plain closure's powers.  The plain closure
// answers outside the training box and below mu_cut, blends in over
// [mu_cut, 2 mu_cut] and judges one substep in judge_period, in FP64.
template <bool FP16, int H>
__device__ __forceinline__ bool substep_surrogate(StateF64& st, const PushParams& P, bool have,
                                                  const uint2* smem, JudgeTally& tally,
                                                  float* /*xpose: FP64 tables have no records*/) {
    const SurrogateDevice& sg = P.sg;
    const SurrogateBox& box = sg.box;
    double c[21];
    float f[kMlpIn] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool use = false;
    double mu = 0.0;
    if (have) {
        sample_f64<true>(st, P, c);
        mu = clamp_mu(st.mu, P.kd.mu_max);
        const float b = static_cast<float>(c[6]);
        const float p = static_cast<float>(st.p);
        const float amu = fabsf(static_cast<float>(mu));
        if (sg.constants_in_box && amu >= box.mu_cut && b > 0.0f && p > 0.0f) {
            const float lm = __logf(amu);
            const float lp = __logf(p);
            const float lb = __logf(b);
            use = lm <= box.in_hi[0] && lp >= box.in_lo[1] && lp <= box.in_hi[1] &&
                  lb >= box.in_lo[2] && lb <= box.in_hi[2];
            if (use) {
                f[0] = lm * box.in_scale[0] + box.in_offset[0];
                f[1] = lp * box.in_scale[1] + box.in_offset[1];
                f[2] = lb * box.in_scale[2] + box.in_offset[2];
                f[3] = sg.f3;
                f[4] = sg.f4;
            }
        }
    }
    float y[kMlpOut];
    __syncwarp();
    mlp_warp<FP16, H>(smem, f, y);
    if (!have) {
        return false;
    }
    // The served values are FP32 whichever closure gives them, so the lanes
    // outside the training box (and the judged and blended ones) take the
    // plain closure in FP32 too: a warp then never runs the FP64 closure's
    // five powers for a few of its lanes.
    const Served served = serve_closure(P, use, static_cast<float>(mu), static_cast<float>(c[6]),
                                        static_cast<float>(st.p), st.steps, y, tally);
    return advance_f64<true, true>(st, P, c, &served);
}

// Position <-> fixed-point phase (once per particle and push).
__device__ __forceinline__ uint64_t to_phase(double x, double lower, double inv_width) {
    double f = (x - lower) * inv_width;
    f = f - floor(f);
    const double scaled = f * 18446744073709551616.0;
    return scaled >= 18446744073709551615.0 ? 0ull : __double2ull_rn(scaled);
}

__device__ __forceinline__ double from_phase(uint64_t phase, double lower, double width) {
    return lower + static_cast<double>(phase) * (width * (1.0 / 18446744073709551616.0));
}

template <bool FOCUSED>
__device__ __forceinline__ void load(StateMixed& st, const PushParams& P, uint32_t index) {
    const ParticleArrays& a = P.parts;
    const DeviceSettings& s = P.s;
    st.index = index;
    const double x = wrap_driver(a.x[index], s.x_lower, s.x_upper, s.x_width);
    const double y = wrap_driver(a.y[index], s.y_lower, s.y_upper, s.y_width);
    st.px = to_phase(x, s.x_lower, P.grid.axis[0].inv_width);
    st.py = to_phase(y, s.y_lower, P.grid.axis[1].inv_width);
    const double p = a.p[index];
    st.p_hi = static_cast<float>(p);
    st.p_lo = static_cast<float>(p - static_cast<double>(st.p_hi));
    const double t = a.t[index];
    const double f = (t - P.interval_start) / s.mhd_dt;
    st.tau = t >= P.interval_end ? kTauEnd
                                 : (f <= -1.0 ? -kTauEnd : __double2ll_rn(f * 4611686018427387904.0));
    st.diag_dt = static_cast<float>(a.step_dt[index]);
    st.mu = FOCUSED ? clamp_mu(static_cast<float>(a.mu[index]), static_cast<float>(s.mu_max))
                    : 0.0f;
    st.steps = 0;
    st.status = 0;
    if (!isfinite(a.x[index]) || !isfinite(a.y[index]) || !isfinite(p) || !isfinite(t)) {
        st.status = 2;
    }
}

template <bool FOCUSED>
__device__ __forceinline__ void store(StateMixed& st, const PushParams& P) {
    const ParticleArrays& a = P.parts;
    const DeviceSettings& s = P.s;
    if (st.steps >= s.max_steps && st.tau < kTauEnd) st.status = 2;
    const uint32_t i = st.index;
    if (st.steps > 0) {
        a.x[i] = wrap_driver(from_phase(st.px, s.x_lower, s.x_width), s.x_lower, s.x_upper,
                             s.x_width);
        a.y[i] = wrap_driver(from_phase(st.py, s.y_lower, s.y_width), s.y_lower, s.y_upper,
                             s.y_width);
        a.p[i] = static_cast<double>(st.p_hi) + static_cast<double>(st.p_lo);
        a.t[i] = st.tau >= kTauEnd
                     ? P.interval_end
                     : P.interval_start + static_cast<double>(st.tau) *
                                              (s.mhd_dt * (1.0 / 4611686018427387904.0));
        a.step_dt[i] = static_cast<double>(st.diag_dt);
        if (FOCUSED) a.mu[i] = static_cast<double>(st.mu);
    } else {
        a.x[i] = wrap_driver(a.x[i], s.x_lower, s.x_upper, s.x_width);
        a.y[i] = wrap_driver(a.y[i], s.y_lower, s.y_upper, s.y_width);
    }
    a.status[i] = st.status;
}

__device__ __forceinline__ bool live(const StateMixed& st, const PushParams& P) {
    return st.status == 0 && st.tau < kTauEnd && st.steps < P.s.max_steps;
}

// ---------------------------------------------------------------- drivers
__device__ __forceinline__ void flush_counters(PushCounters* counters, unsigned long long steps,
                                               unsigned long long pushed,
                                               unsigned long long failed, unsigned int max_steps) {
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) {
        steps += __shfl_down_sync(full, steps, offset);
        pushed += __shfl_down_sync(full, pushed, offset);
        failed += __shfl_down_sync(full, failed, offset);
        max_steps = max(max_steps, __shfl_down_sync(full, max_steps, offset));
    }
    if ((threadIdx.x & 31u) == 0u) {
        if (steps) atomicAdd(&counters->particle_steps, steps);
        if (pushed) atomicAdd(&counters->pushed, pushed);
        if (failed) atomicAdd(&counters->failed, failed);
        if (max_steps) atomicMax(&counters->max_steps, max_steps);
    }
}

__device__ __forceinline__ void flush_judge(unsigned long long* judge, JudgeTally t) {
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) {
        t.evaluations += __shfl_down_sync(full, t.evaluations, offset);
        t.judged += __shfl_down_sync(full, t.judged, offset);
        t.fallbacks += __shfl_down_sync(full, t.fallbacks, offset);
        t.max_error = fmaxf(t.max_error, __shfl_down_sync(full, t.max_error, offset));
    }
    if ((threadIdx.x & 31u) == 0u) {
        if (t.evaluations) atomicAdd(judge + 0, t.evaluations);
        if (t.judged) atomicAdd(judge + 1, t.judged);
        if (t.fallbacks) atomicAdd(judge + 2, t.fallbacks);
        // non-negative floats order like their bit patterns
        atomicMax(judge + 3, static_cast<unsigned long long>(__float_as_uint(t.max_error)));
    }
}

// Persistent warps with lane refill.  A warp claims particles from the
// cursor in batches of (idle lanes); each trip advances every busy lane by
// one substep.  Every trip either advances a particle (bounded by the step
// guard) or moves the cursor, so the loop always terminates.
// Resident blocks of 128 threads per SM the register budget targets: the
// mixed kernels are latency-bound gathers and want more warps in flight.
#ifndef KPT_MIXED_MIN_BLOCKS
#define KPT_MIXED_MIN_BLOCKS 5
#endif
template <typename State, bool FOCUSED>
struct MinBlocks {
    static constexpr int value = FOCUSED ? 2 : 4;
};
template <>
struct MinBlocks<StateMixed, false> {
    static constexpr int value = KPT_MIXED_MIN_BLOCKS;
};
// Focused mixed push with the plain closure: 5 blocks (96 registers, a few
// spilled bytes) measured 2.9 % faster than 4 blocks at 128 registers.
#ifndef KPT_MIXED_FOCUSED_MIN_BLOCKS
#define KPT_MIXED_FOCUSED_MIN_BLOCKS 5
#endif
template <>
struct MinBlocks<StateMixed, true> {
    static constexpr int value = KPT_MIXED_FOCUSED_MIN_BLOCKS;
};

// The surrogate instantiations keep the MLP fragments live beside the
// particle state and the sampled coefficients.  SURR: 1 BF16 and 2 FP16
// networks of hidden width 64, 3 BF16 and 4 FP16 networks of width 32.
#ifndef KPT_SURROGATE_MIN_BLOCKS
#define KPT_SURROGATE_MIN_BLOCKS 4
#endif
#ifndef KPT_SURROGATE32_MIN_BLOCKS
#define KPT_SURROGATE32_MIN_BLOCKS 4
#endif
__host__ __device__ constexpr bool surr_fp16(int surr) { return surr == 2 || surr == 4; }
__host__ __device__ constexpr int surr_hidden(int surr) { return surr <= 2 ? 64 : 32; }
template <typename State, bool FOCUSED, int SURR = 0>
__global__ void __launch_bounds__(128, !std::is_same<State, StateMixed>::value
                                           ? MinBlocks<State, FOCUSED>::value
                                       : SURR >= 3 ? KPT_SURROGATE32_MIN_BLOCKS
                                       : SURR      ? KPT_SURROGATE_MIN_BLOCKS
                                                   : MinBlocks<State, FOCUSED>::value)
    push_refill_kernel(const PushParams P) {
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    extern __shared__ uint2 surrogate_smem[];
    JudgeTally tally{0ull, 0ull, 0ull, 0.0f};
    if (SURR) {
        load_surrogate_block<surr_hidden(SURR)>(P.sg.block, surrogate_smem);
    }
    // the warp's rows for the record sampler, after the network's block
    float* xpose = nullptr;
    if (std::is_same<State, StateMixed>::value && P.records != nullptr) {
        xpose = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(surrogate_smem) +
                                         (SURR ? mlp_smem_bytes(surr_hidden(SURR)) : 0)) +
                (threadIdx.x >> 5) * 32 * record_xpose_stride(FOCUSED);
    }
    State st;
    bool have = false;
    bool exhausted = false;
    unsigned long long my_steps = 0, my_pushed = 0, my_failed = 0;
    unsigned int my_max = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(full, !have);
        if (idle != 0u && !exhausted) {
            const unsigned n_idle = __popc(idle);
            const int leader = __ffs(idle) - 1;
            unsigned base = 0;
            if (static_cast<int>(lane) == leader) {
                base = atomicAdd(&P.counters->next_particle, n_idle);
            }
            base = __shfl_sync(full, base, leader);
            if (static_cast<uint64_t>(base) + n_idle >= P.count) {
                exhausted = true;
            }
            if (!have) {
                const uint64_t slot = static_cast<uint64_t>(base) + __popc(idle & lanes_below);
                if (slot < P.count) {
                    const uint32_t idx = P.order != nullptr ? __ldg(P.order + slot)
                                                            : static_cast<uint32_t>(slot);
                    if (P.parts.status[idx] == 0) {
                        load<FOCUSED>(st, P, idx);
                        ++my_pushed;
                        have = true;
                        if (!live(st, P)) {
                            store<FOCUSED>(st, P);
                            my_failed += st.status != 0 ? 1 : 0;
                            have = false;
                        }
                    }
                }
            }
        }
        if (!__any_sync(full, have)) {
            if (exhausted) {
                break;
            }
            continue;
        }
        bool more;
        if constexpr (SURR) {
            more = substep_surrogate<surr_fp16(SURR), surr_hidden(SURR)>(
                st, P, have, surrogate_smem, tally, xpose);
        } else if constexpr (std::is_same<State, StateMixed>::value) {
            more = xpose != nullptr ? substep_records<FOCUSED>(st, P, have, xpose)
                                    : have && substep<FOCUSED>(st, P);
        } else {
            more = have && substep<FOCUSED>(st, P);
        }
        if (have && !more) {
            store<FOCUSED>(st, P);
            my_steps += static_cast<unsigned long long>(st.steps);
            my_max = max(my_max, static_cast<unsigned int>(st.steps));
            my_failed += st.status != 0 ? 1 : 0;
            have = false;
        }
    }
    flush_counters(P.counters, my_steps, my_pushed, my_failed, my_max);
    if (SURR) {
        flush_judge(P.sg.judge, tally);
    }
}

// The learned-closure push with the network on the tcgen05 tensor cores.
// Warps refill their lanes from the cursor as in push_refill_kernel, but the
// network is block-collective (M = 128 rows = the block's lanes), so the
// block advances in lockstep: a trip runs while any lane of the block holds
// a particle, idle lanes feed zero rows, and the loop ends once every warp
// has found the cursor exhausted.  A completion wait that times out stops
// the block (counted in PushCounters::network_timeouts); the block frees its
// TMEM before it returns.
#ifndef KPT_SURROGATE_TC_MIN_BLOCKS
#define KPT_SURROGATE_TC_MIN_BLOCKS 4
#endif
#ifndef KPT_SURROGATE_TC32_MIN_BLOCKS
#define KPT_SURROGATE_TC32_MIN_BLOCKS 4
#endif
template <bool FP16, int H>
__global__ void __launch_bounds__(128, H == 32 ? KPT_SURROGATE_TC32_MIN_BLOCKS
                                               : KPT_SURROGATE_TC_MIN_BLOCKS)
    push_tc_kernel(const PushParams P) {
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    extern __shared__ __align__(128) unsigned char tc_smem[];
    TcNet net = tc_setup<H>(P.sg.tc_block, tc_smem);
    tc_constants<FP16, H>(net);
    float* xpose = P.records == nullptr
                       ? nullptr
                       : reinterpret_cast<float*>(tc_smem + tc_xpose_offset<H>()) +
                             (threadIdx.x >> 5) * 32 * record_xpose_stride(true);
    JudgeTally tally{0ull, 0ull, 0ull, 0.0f};
    StateMixed st;
    bool have = false;
    bool exhausted = false;
    bool fail = false;
    unsigned long long my_steps = 0, my_pushed = 0, my_failed = 0;
    unsigned int my_max = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(full, !have);
        if (idle != 0u && !exhausted) {
            const unsigned n_idle = __popc(idle);
            const int leader = __ffs(idle) - 1;
            unsigned base = 0;
            if (static_cast<int>(lane) == leader) {
                base = atomicAdd(&P.counters->next_particle, n_idle);
            }
            base = __shfl_sync(full, base, leader);
            if (static_cast<uint64_t>(base) + n_idle >= P.count) {
                exhausted = true;
            }
            if (!have) {
                const uint64_t slot = static_cast<uint64_t>(base) + __popc(idle & lanes_below);
                if (slot < P.count) {
                    const uint32_t idx = P.order != nullptr ? __ldg(P.order + slot)
                                                            : static_cast<uint32_t>(slot);
                    if (P.parts.status[idx] == 0) {
                        load<true>(st, P, idx);
                        ++my_pushed;
                        have = true;
                        if (!live(st, P)) {
                            store<true>(st, P);
                            my_failed += st.status != 0 ? 1 : 0;
                            have = false;
                        }
                    }
                }
            }
        }
        if (!__syncthreads_or(have ? 1 : 0)) {
            if (__syncthreads_and(exhausted ? 1 : 0)) {
                break;
            }
            continue;
        }
        bool stop = false;
        const bool more = substep_surrogate<FP16, H, true>(st, P, have, nullptr, tally, xpose,
                                                           &net, &fail, &stop);
        if (stop) {
            break;
        }
        if (have && !more) {
            store<true>(st, P);
            my_steps += static_cast<unsigned long long>(st.steps);
            my_max = max(my_max, static_cast<unsigned int>(st.steps));
            my_failed += st.status != 0 ? 1 : 0;
            have = false;
        }
    }
    fail = __syncthreads_or(fail ? 1 : 0) != 0;
    if (fail && threadIdx.x == 0) {
        atomicAdd(&P.counters->network_timeouts, 1u);
    }
    if (!tc_teardown<H>(net, fail) && threadIdx.x == 0) {
        atomicAdd(&P.counters->teardown_incomplete, 1u);
    }
    flush_counters(P.counters, my_steps, my_pushed, my_failed, my_max);
    flush_judge(P.sg.judge, tally);
}

// One particle per thread, no refill (schedule alternative for the tuner).
template <typename State, bool FOCUSED>
__global__ void __launch_bounds__(128) push_simple_kernel(const PushParams P) {
    unsigned long long my_steps = 0, my_pushed = 0, my_failed = 0;
    unsigned int my_max = 0;
    for (uint64_t slot = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
         slot < P.count; slot += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t idx =
            P.order != nullptr ? __ldg(P.order + slot) : static_cast<uint32_t>(slot);
        if (P.parts.status[idx] != 0) {
            continue;
        }
        State st;
        load<FOCUSED>(st, P, idx);
        ++my_pushed;
        if (live(st, P)) {
            while (substep<FOCUSED>(st, P)) {
            }
        }
        store<FOCUSED>(st, P);
        my_steps += static_cast<unsigned long long>(st.steps);
        my_max = max(my_max, static_cast<unsigned int>(st.steps));
        my_failed += st.status != 0 ? 1 : 0;
    }
    flush_counters(P.counters, my_steps, my_pushed, my_failed, my_max);
}

PushParams make_push_params(const PushLaunch& L) {
    PushParams P;
    P.grid = L.grid;
    P.fixed = L.fixed;
    P.lower = L.lower;
    P.upper = L.upper;
    P.table_points = static_cast<uint64_t>(L.grid.ex) *
                     static_cast<uint64_t>(L.grid.axis[1].n + 4);
    P.parts = L.parts;
    P.order = L.order;
    P.count = L.count;
    P.s = L.settings;
    P.kd = make_consts<double>(L.settings);
    P.kf = make_consts<float>(L.settings);
    P.interval_start = L.interval_start;
    P.interval_end = L.interval_end;
    P.inv_mhd_dt = static_cast<float>(1.0 / L.settings.mhd_dt);
    P.frame = L.frame;
    P.key = make_uint2(static_cast<uint32_t>(L.seed), static_cast<uint32_t>(L.seed >> 32));
    P.counters = L.counters;
    if (L.surrogate != nullptr) {
        P.sg = *L.surrogate;
    }
    P.records = L.precision == kPrecisionMixed ? L.records : nullptr;
    return P;
}

// Persistent grid of the tcgen05 push: as many blocks per SM as both the
// TMEM (TcMlp<H>::Cols of the SM's 512 columns each) and the registers
// admit.  The occupancy query reports 1 block per SM for this kernel, so
// the register bound is computed from the kernel's attributes (registers
// per thread rounded to the allocation unit of 8); should the registers
// admit more blocks than the TMEM, the dynamic shared memory is padded
// until they do not (a further block would only wait in tcgen05.alloc).
template <bool FP16, int H>
cudaError_t launch_push_tc(const PushParams& P, const PushLaunch& L, cudaStream_t stream) {
    const int threads = 128;
    constexpr int kTmemBlocks = 512 / static_cast<int>(TcMlp<H>::Cols);
    size_t smem = P.records != nullptr ? tc_xpose_offset<H>() + record_xpose_bytes(true, 4)
                                       : tc_smem_bytes<H>();
    cudaFuncAttributes attr{};
    cudaError_t err = cudaFuncGetAttributes(&attr, push_tc_kernel<FP16, H>);
    if (err != cudaSuccess) return err;
    const int regs = attr.numRegs > 0 ? (attr.numRegs + 7) / 8 * 8 : 8;
    const int reg_blocks = 65536 / (regs * threads);
    if (reg_blocks > kTmemBlocks) {
        int device = 0, per_sm_smem = 0;
        err = cudaGetDevice(&device);
        if (err != cudaSuccess) return err;
        err = cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                     device);
        if (err != cudaSuccess) return err;
        const size_t padded = static_cast<size_t>(per_sm_smem) / (kTmemBlocks + 1) + 1;
        if (padded > smem) {
            smem = padded;
            err = cudaFuncSetAttribute(push_tc_kernel<FP16, H>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
            if (err != cudaSuccess) return err;
        }
    }
    const int resident = reg_blocks < kTmemBlocks ? (reg_blocks > 0 ? reg_blocks : 1)
                                                  : kTmemBlocks;
    const int per_sm =
        L.blocks_per_sm > 0 && L.blocks_per_sm < resident ? L.blocks_per_sm : resident;
    push_tc_kernel<FP16, H><<<L.sm_count * per_sm, threads, smem, stream>>>(P);
    return cudaGetLastError();
}

template <typename State, bool FOCUSED, int SURR = 0>
cudaError_t launch_push(const PushLaunch& L, cudaStream_t stream) {
    const PushParams P = make_push_params(L);
    const int threads = 128;
    if constexpr (SURR != 0 && std::is_same<State, StateMixed>::value) {
        if (L.surrogate->engine == kEngineTcgen05) {
            return launch_push_tc<surr_fp16(SURR), surr_hidden(SURR)>(P, L, stream);
        }
    }
    const size_t smem = (SURR ? mlp_smem_bytes(surr_hidden(SURR)) : 0) +
                        (P.records != nullptr ? record_xpose_bytes(FOCUSED, threads / 32) : 0);
    if (L.schedule == kScheduleSimple && !SURR) {
        const uint64_t want = (L.count + threads - 1) / threads;
        const int blocks =
            static_cast<int>(want < 1 ? 1 : (want > 65535u * 8u ? 65535u * 8u : want));
        push_simple_kernel<State, FOCUSED><<<blocks, threads, 0, stream>>>(P);
    } else {
        // Persistent grid: as many resident blocks per SM as the kernel's
        // registers allow (or fewer on request).
        int resident = 0;
        cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &resident, push_refill_kernel<State, FOCUSED, SURR>, threads, smem);
        if (err != cudaSuccess) return err;
        resident = resident < 1 ? 1 : resident;
        const int per_sm = L.blocks_per_sm > 0 && L.blocks_per_sm < resident ? L.blocks_per_sm
                                                                            : resident;
        push_refill_kernel<State, FOCUSED, SURR>
            <<<L.sm_count * per_sm, threads, smem, stream>>>(P);
    }
    return cudaGetLastError();
}

#if KPT_PUSH_PART == 0
// ---------------------------------------------------------------- batches
// Many independent runs (own fields, settings, particles, seeds and frames)
// in one persistent launch.  The work cursor walks the concatenation of the
// runs' particle ranges; a lane finds its run by binary search over the run
// offsets (kept in shared memory) and reads that run's parameter block from
// global memory.  Lanes of one warp may belong to different runs.  Each
// finished particle adds its counters to its run's counters.
constexpr int kBatchMaxRuns = 1024;

__device__ __forceinline__ int batch_run_of(const uint64_t* offsets, int runs, uint64_t slot) {
    int lo = 0;
    int hi = runs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= slot) {
            lo = mid;
        } else {
            hi = mid - 1;
        }
    }
    return lo;
}

__device__ __forceinline__ void batch_finish(const PushParams& P, const StateMixed& st) {
    atomicAdd(&P.counters->particle_steps, static_cast<unsigned long long>(st.steps));
    atomicAdd(&P.counters->pushed, 1ull);
    if (st.status != 0) atomicAdd(&P.counters->failed, 1ull);
    atomicMax(&P.counters->max_steps, static_cast<unsigned int>(st.steps));
}

// A batched substep over the cell records, warp-collective: every lane
// calls it; lanes of one warp may belong to different runs (each samples
// its run's records) and lanes without a particle help sample.  A warp
// whose particles' runs disagree on time interpolation samples the point
// tables instead (the same values).
template <bool FOCUSED>
__device__ __forceinline__ bool substep_batch_records(StateMixed& st, const PushParams* runs,
                                                      int run, bool have, float* xpose) {
    const unsigned full = 0xffffffffu;
    const PushParams& P = runs[run];
    float c[FOCUSED ? 21 : 16];
    size_t cell = 0;
    float w0 = 0.0f, w1 = 0.0f, rt = 0.0f;
    int time_on = 0;
    if (have) {
        ++st.steps;
        mixed_stencil(st, P, cell, w0, w1, rt);
        time_on = P.s.time_interpolation != 0 ? 1 : 0;
    }
    const float* rec = P.records + cell * record_floats(FOCUSED);
    if (__all_sync(full, !have || time_on != 0)) {
        sample_records<FOCUSED, true>(rec, w0, w1, rt, c, xpose);
    } else if (__all_sync(full, !have || time_on == 0)) {
        sample_records<FOCUSED, false>(rec, w0, w1, rt, c, xpose);
    } else if (have) {
        sample_mixed<FOCUSED>(st, P, c);
    }
    return have && advance_mixed<FOCUSED>(st, P, c);
}

// Register budget of the batched push per launch shape: the resident
// threads per SM of the single-run mixed push (MinBlocks x 128), divided by
// the particles a lane carries (each carries its own state).
template <bool FOCUSED, int THREADS, int PPL>
struct BatchMinBlocks {
    static constexpr int threads_per_sm = MinBlocks<StateMixed, FOCUSED>::value * 128 / PPL;
    static constexpr int value = threads_per_sm / THREADS > 0 ? threads_per_sm / THREADS : 1;
};

// PPL particles per lane: each lane keeps PPL particle states and advances
// every one it holds by one substep per trip, so the table gathers of
// independent particles are in flight together; each slot refills from the
// cursor on its own.
template <bool FOCUSED, int THREADS, int PPL>
__global__ void __launch_bounds__(THREADS, (BatchMinBlocks<FOCUSED, THREADS, PPL>::value))
    push_batch_kernel(const BatchLaunch B) {
    __shared__ uint64_t offsets[kBatchMaxRuns + 1];
    extern __shared__ float batch_xpose[];
    for (int k = threadIdx.x; k <= B.runs; k += blockDim.x) offsets[k] = B.offsets[k];
    __syncthreads();
    const PushParams* runs = static_cast<const PushParams*>(B.params);
    float* xpose = B.records != 0
                       ? batch_xpose + (threadIdx.x >> 5) * 32 * record_xpose_stride(FOCUSED)
                       : nullptr;
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    const uint64_t total = offsets[B.runs];
    StateMixed st[PPL];
    int run[PPL];
    bool have[PPL];
#pragma unroll
    for (int s = 0; s < PPL; ++s) {
        run[s] = 0;
        have[s] = false;
    }
    bool exhausted = false;
    for (;;) {
#pragma unroll
        for (int s = 0; s < PPL; ++s) {
            const unsigned idle = __ballot_sync(full, !have[s]);
            if (idle != 0u && !exhausted) {
                const unsigned n_idle = __popc(idle);
                const int leader = __ffs(idle) - 1;
                unsigned long long base = 0;
                if (static_cast<int>(lane) == leader) {
                    base = atomicAdd(B.cursor, static_cast<unsigned long long>(n_idle));
                }
                base = __shfl_sync(full, base, leader);
                if (base + n_idle >= total) {
                    exhausted = true;
                }
                if (!have[s]) {
                    const uint64_t slot = base + __popc(idle & lanes_below);
                    if (slot < total) {
                        run[s] = batch_run_of(offsets, B.runs, slot);
                        const PushParams& P = runs[run[s]];
                        const uint64_t local = slot - offsets[run[s]];
                        const uint32_t idx = P.order != nullptr ? __ldg(P.order + local)
                                                                : static_cast<uint32_t>(local);
                        if (P.parts.status[idx] == 0) {
                            load<FOCUSED>(st[s], P, idx);
                            have[s] = true;
                            if (!live(st[s], P)) {
                                store<FOCUSED>(st[s], P);
                                batch_finish(P, st[s]);
                                have[s] = false;
                            }
                        }
                    }
                }
            }
        }
        bool any = false;
#pragma unroll
        for (int s = 0; s < PPL; ++s) any = any || have[s];
        if (!__any_sync(full, any)) {
            if (exhausted) {
                break;
            }
            continue;
        }
#pragma unroll
        for (int s = 0; s < PPL; ++s) {
            const bool more = xpose != nullptr
                                  ? substep_batch_records<FOCUSED>(st[s], runs, run[s], have[s],
                                                                   xpose)
                                  : have[s] && substep<FOCUSED>(st[s], runs[run[s]]);
            if (have[s] && !more) {
                const PushParams& P = runs[run[s]];
                store<FOCUSED>(st[s], P);
                batch_finish(P, st[s]);
                have[s] = false;
            }
        }
    }
}

// Next interval of every run: frame + 1, interval bounds recomputed as the
// host computes them (frame x mhd_dt), counters cleared.
__global__ void batch_next_frame_kernel(void* params, int runs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= runs) return;
    PushParams& P = static_cast<PushParams*>(params)[r];
    P.frame += 1u;
    P.interval_start = static_cast<double>(P.frame) * P.s.mhd_dt;
    P.interval_end = P.interval_start + P.s.mhd_dt;
}

__global__ void batch_clear_counters_kernel(void* params, int runs, unsigned long long* cursor) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) *cursor = 0ull;
    if (r >= runs) return;
    PushCounters* c = static_cast<PushParams*>(params)[r].counters;
    c->particle_steps = 0;
    c->pushed = 0;
    c->failed = 0;
    c->max_steps = 0;
}

#endif  // KPT_PUSH_PART == 0

// Table values at given positions through the FP64 sampling path (driver
// wrap, half-cell shift, grid wrap, stencil, time interpolation).
template <typename T, bool FOCUSED>
__global__ void sample_kernel(const SampleLaunch L) {
    constexpr int C = FOCUSED ? 21 : 16;
    constexpr int STRIDE = FOCUSED ? (sizeof(T) == 8 ? 22 : 24) : 16;
    const Axis& ax = L.grid.axis[0];
    const Axis& ay = L.grid.axis[1];
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < L.n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const double x = wrap_driver(L.x[i], ax.lower, ax.upper, __dsub_rn(ax.upper, ax.lower));
        const double y = wrap_driver(L.y[i], ay.lower, ay.upper, __dsub_rn(ay.upper, ay.lower));
        T c[C];
        sample_coefficients<T, C, STRIDE>(L.grid, static_cast<const T*>(L.lower),
                                          static_cast<const T*>(L.upper),
                                          __dadd_rn(x, L.shift_x), __dadd_rn(y, L.shift_y),
                                          L.rt[i], L.time_interpolation, c);
#pragma unroll
        for (int k = 0; k < C; ++k) {
            L.out[i * C + k] = static_cast<double>(c[k]);
        }
    }
}

}  // namespace

#if KPT_PUSH_PART == 1

cudaError_t launch_push_interval_f64(const PushLaunch& launch, cudaStream_t stream) {
    return launch.focused ? launch_push<StateF64, true>(launch, stream)
                          : launch_push<StateF64, false>(launch, stream);
}

cudaError_t launch_sample_f64(const SampleLaunch& L, int blocks, cudaStream_t stream) {
    if (L.focused) {
        sample_kernel<double, true><<<blocks, 128, 0, stream>>>(L);
    } else {
        sample_kernel<double, false><<<blocks, 128, 0, stream>>>(L);
    }
    return cudaGetLastError();
}

#else  // KPT_PUSH_PART == 0

cudaError_t launch_sample(const SampleLaunch& L, cudaStream_t stream) {
    if (L.n == 0) {
        return cudaSuccess;
    }
    const int threads = 128;
    const uint64_t want = (L.n + threads - 1) / threads;
    const int blocks = static_cast<int>(want > 152u * 16u ? 152u * 16u : want);
    if (L.precision == kPrecisionF64) {
        return launch_sample_f64(L, blocks, stream);
    }
    if (L.focused) {
        sample_kernel<float, true><<<blocks, threads, 0, stream>>>(L);
    } else {
        sample_kernel<float, false><<<blocks, threads, 0, stream>>>(L);
    }
    return cudaGetLastError();
}

size_t push_params_size() { return sizeof(PushParams); }

void build_push_params(const PushLaunch& launch, void* out) {
    const PushParams P = make_push_params(launch);
    std::memcpy(out, &P, sizeof(P));
}

namespace {

template <bool FOCUSED, int THREADS, int PPL>
cudaError_t launch_batch_shape(const BatchLaunch& B, cudaStream_t stream) {
    const size_t smem = B.records != 0 ? record_xpose_bytes(FOCUSED, THREADS / 32) : 0;
    int resident = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &resident, push_batch_kernel<FOCUSED, THREADS, PPL>, THREADS, smem);
    if (err != cudaSuccess) return err;
    resident = resident < 1 ? 1 : resident;
    const int per_sm = B.blocks_per_sm > 0 && B.blocks_per_sm < resident ? B.blocks_per_sm
                                                                        : resident;
    push_batch_kernel<FOCUSED, THREADS, PPL><<<B.sm_count * per_sm, THREADS, smem, stream>>>(B);
    return cudaGetLastError();
}

template <bool FOCUSED>
cudaError_t launch_batch_focused(const BatchLaunch& B, cudaStream_t stream) {
    switch (B.threads * 4 + B.particles_per_lane) {
        case 64 * 4 + 1: return launch_batch_shape<FOCUSED, 64, 1>(B, stream);
        case 64 * 4 + 2: return launch_batch_shape<FOCUSED, 64, 2>(B, stream);
        case 128 * 4 + 1: return launch_batch_shape<FOCUSED, 128, 1>(B, stream);
        case 128 * 4 + 2: return launch_batch_shape<FOCUSED, 128, 2>(B, stream);
        case 256 * 4 + 1: return launch_batch_shape<FOCUSED, 256, 1>(B, stream);
        case 256 * 4 + 2: return launch_batch_shape<FOCUSED, 256, 2>(B, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_push_interval_f64_contracted(const PushLaunch& launch, cudaStream_t stream) {
    return launch.focused ? launch_push<StateF64, true>(launch, stream)
                          : launch_push<StateF64, false>(launch, stream);
}

bool batch_shape_supported(int threads, int particles_per_lane) {
    return (threads == 64 || threads == 128 || threads == 256) &&
           (particles_per_lane == 1 || particles_per_lane == 2);
}

cudaError_t launch_push_batch(const BatchLaunch& B, cudaStream_t stream) {
    if (B.runs <= 0 || B.runs > kBatchMaxRuns) return cudaErrorInvalidValue;
    if (!batch_shape_supported(B.threads, B.particles_per_lane)) return cudaErrorInvalidValue;
    batch_clear_counters_kernel<<<(B.runs + 127) / 128, 128, 0, stream>>>(B.params, B.runs,
                                                                          B.cursor);
    return B.focused ? launch_batch_focused<true>(B, stream)
                     : launch_batch_focused<false>(B, stream);
}

cudaError_t launch_batch_next_frame(const BatchLaunch& B, cudaStream_t stream) {
    batch_next_frame_kernel<<<(B.runs + 127) / 128, 128, 0, stream>>>(B.params, B.runs);
    return cudaGetLastError();
}

int batch_max_runs() { return kBatchMaxRuns; }

cudaError_t launch_push_interval(const PushLaunch& launch, cudaStream_t stream) {
    if (launch.precision == kPrecisionF64) {
        if (launch.surrogate != nullptr) {
            // the FP64 push with the learned closure (mma.sync engine), built
            // with the contracted FP64 arithmetic
            const SurrogateBox& box = launch.surrogate->box;
            if (box.hidden == 64) {
                return box.fp16 ? launch_push<StateF64, true, 2>(launch, stream)
                                : launch_push<StateF64, true, 1>(launch, stream);
            }
            return box.fp16 ? launch_push<StateF64, true, 4>(launch, stream)
                            : launch_push<StateF64, true, 3>(launch, stream);
        }
        return launch.fp64_contracted ? launch_push_interval_f64_contracted(launch, stream)
                                      : launch_push_interval_f64(launch, stream);
    }
    if (launch.surrogate != nullptr) {
        const SurrogateBox& box = launch.surrogate->box;
        if (box.hidden == 64) {
            return box.fp16 ? launch_push<StateMixed, true, 2>(launch, stream)
                            : launch_push<StateMixed, true, 1>(launch, stream);
        }
        return box.fp16 ? launch_push<StateMixed, true, 4>(launch, stream)
                        : launch_push<StateMixed, true, 3>(launch, stream);
    }
    return launch.focused ? launch_push<StateMixed, true>(launch, stream)
                          : launch_push<StateMixed, false>(launch, stream);
}

#endif  // KPT_PUSH_PART

}  // namespace kpt
