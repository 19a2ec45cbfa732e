// Interval push kernels: Parker (16-component table) and focused transport
// (21 components), plain FP64 or mixed precision (FP32 table, interpolation,
// coefficients and noise; FP64 position, time, momentum and cell search).
//
// The per-substep physics restates reference src/main.cpp:1131-1306 (Parker)
// and :1384-1733 (focused).  Scheduling is GB300-first: a persistent grid of
// warps pulls particles from a device cursor, and a lane whose particle has
// reached the interval end refills from the cursor, so warps stay full while
// particles need very different substep counts (random injection times).
// Noise is the keyed Philox stream, so results do not depend on which lane
// or launch shape pushed a particle.
#include <cuda_runtime.h>

#include <cstdint>

#include "kpt_device.cuh"
#include "kpt_internal.h"

namespace kpt {
namespace {

constexpr double kSqrt3 = 1.7320508075688772935;

template <typename T>
struct Num;

template <>
struct Num<double> {
    static __device__ __forceinline__ double pow(double a, double b) { return ::pow(a, b); }
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
    static __device__ __forceinline__ float sqrt(float a) { return sqrtf(a); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ bool finite(float a) { return isfinite(a); }
    static __device__ __forceinline__ float abs(float a) { return fabsf(a); }
    static __device__ __forceinline__ float noise(uint32_t, uint32_t hi) {
        return -static_cast<float>(kSqrt3) +
               static_cast<float>(2.0 * kSqrt3) * u01_f32(hi);
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

// Vector width used to stream one table point.
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

// Bilinear sample of one frame at precomputed corner points and weights
// (LinearPositionInterpolator::sample, FieldInterpolator.hpp:346-380):
// out = sum over corners in order (00, 10, 01, 11) of weight * value.
template <typename T, int C, int STRIDE>
__device__ __forceinline__ void sample_frame(const T* __restrict__ table, const size_t pt[4],
                                             const T wc[4], T out[C]) {
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

// sample_time_interpolated_coefficients (src/main.cpp:1055-1077) at the
// driver's shifted position (src/main.cpp:1142-1148).
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
    const size_t ex = static_cast<size_t>(g.ex);
    const size_t pt[4] = {static_cast<size_t>(lo0 + 2) + static_cast<size_t>(lo1 + 2) * ex,
                          static_cast<size_t>(hi0 + 2) + static_cast<size_t>(lo1 + 2) * ex,
                          static_cast<size_t>(lo0 + 2) + static_cast<size_t>(hi1 + 2) * ex,
                          static_cast<size_t>(hi0 + 2) + static_cast<size_t>(hi1 + 2) * ex};
    sample_frame<T, C, STRIDE>(lower, pt, wc, c);
    if (use_time == 0) {
        return;
    }
    T u[C];
    sample_frame<T, C, STRIDE>(upper, pt, wc, u);
    const double uwd = rt < 0.0 ? 0.0 : (rt > 1.0 ? 1.0 : rt);
    const T uw = static_cast<T>(uwd);
    const T lw = static_cast<T>(1.0 - uwd);
#pragma unroll
    for (int k = 0; k < C; ++k) {
        c[k] = lw * c[k] + uw * u[k];
    }
}

template <typename T>
struct State {
    double x, y, p, t, dt, diag_dt;
    T mu;
    int steps;
    int status;
    uint32_t index;
};

struct PushParams {
    Grid grid;
    const void* lower;
    const void* upper;
    ParticleArrays parts;
    uint64_t count;
    DeviceSettings s;
    double interval_start;
    double interval_end;
    uint32_t frame;
    uint2 key;
    PushCounters* counters;
};

// One substep of the driver loop body.  Returns false once the particle
// leaves the loop (interval end, step guard or failure).
template <typename T, bool FOCUSED>
__device__ __forceinline__ bool substep(State<T>& st, const PushParams& P) {
    using N = Num<T>;
    constexpr int C = FOCUSED ? 21 : 16;
    constexpr int STRIDE = FOCUSED ? (sizeof(T) == 8 ? 22 : 24) : 16;
    const DeviceSettings& s = P.s;

    ++st.steps;
    st.x = wrap_driver(st.x, s.x_lower, s.x_upper, s.x_width);
    st.y = wrap_driver(st.y, s.y_lower, s.y_upper, s.y_width);
    const double q0 = __dadd_rn(st.x, s.shift_x);
    const double q1 = __dadd_rn(st.y, s.shift_y);
    const double rt = __ddiv_rn(__dsub_rn(st.t, P.interval_start), s.mhd_dt);
    T c[C];
    sample_coefficients<T, C, STRIDE>(P.grid, static_cast<const T*>(P.lower),
                                      static_cast<const T*>(P.upper), q0, q1, rt,
                                      s.time_interpolation, c);

    T vx, vy, bx, by, bz, b, dvx_dx, dvy_dy, dbx_dx, dbx_dy, dby_dx, dby_dy, dbz_dx, dbz_dy,
        db_dx, db_dy;
    T vz = 0, dvx_dy = 0, dvy_dx = 0, dvz_dx = 0, dvz_dy = 0;
    if (FOCUSED) {
        vx = c[0]; vy = c[1]; vz = c[2]; bx = c[3]; by = c[4]; bz = c[5]; b = c[6];
        dvx_dx = c[7]; dvx_dy = c[8]; dvy_dx = c[9]; dvy_dy = c[10]; dvz_dx = c[11];
        dvz_dy = c[12]; dbx_dx = c[13]; dbx_dy = c[14]; dby_dx = c[15]; dby_dy = c[16];
        dbz_dx = c[17]; dbz_dy = c[18]; db_dx = c[19]; db_dy = c[20];
    } else {
        vx = c[0]; vy = c[1]; bx = c[2]; by = c[3]; bz = c[4]; b = c[5]; dvx_dx = c[6];
        dvy_dy = c[7]; dbx_dx = c[8]; dbx_dy = c[9]; dby_dx = c[10]; dby_dy = c[11];
        dbz_dx = c[12]; dbz_dy = c[13]; db_dx = c[14]; db_dy = c[15];
    }
    (void)vz;

    const T p = static_cast<T>(st.p);
    if (!isfinite(st.p) || st.p <= 0.0 || !N::finite(b) || b <= T(0)) {
        st.status = 2;
        return false;
    }
    const T p0 = static_cast<T>(s.p0);
    const T gamma = static_cast<T>(s.gamma_turb);
    const T ib = N::div(T(1), b);
    const T ib2 = ib * ib;
    const T ib3 = ib2 * ib;

    T knorm_para = T(1);
    if (s.magnetic_dependency == 1) {
        knorm_para *= N::pow(b, gamma - T(2));
    }
    T knorm = knorm_para;
    if (s.momentum_dependency == 1) {
        knorm *= N::pow(N::div(p, p0), static_cast<T>(s.pindex));
    }
    const T kpara = static_cast<T>(s.kpara0) * knorm;
    const T kperp = kpara * static_cast<T>(s.kperp_over_kpara);
    if (!N::finite(kpara) || kpara <= T(0) || !N::finite(kperp) || kperp < T(0)) {
        st.status = 2;
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
    (void)skpara_perp;
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

    const T d1 = static_cast<T>(s.drift_param1);
    const T d2 = static_cast<T>(s.drift_param2);
    const T drift_denominator =
        N::sqrt(square(N::div(d1 * p0, p)) + square(N::div(d2 * p0 * p0, p * p)));

    T dx_dt, dy_dt, dp_dt;
    T dmu_dt = T(0), duu = T(0);
    T pitch_mu = st.mu;
    if (FOCUSED) {
        const T mu_max = static_cast<T>(s.mu_max);
        pitch_mu = clamp_mu(pitch_mu, mu_max);
        const T mu2 = pitch_mu * pitch_mu;
        const T muf1 = T(0.5) * (T(1) - mu2);
        const T muf2 = T(0.5) * (T(3) * mu2 - T(1));
        const T kx = bx * dbx_dx + by * dbx_dy;
        const T ky = bx * dby_dx + by * dby_dy;
        const T kz = bx * dbz_dx + by * dbz_dy;
        const T bdot_curvb = bx * dbz_dy - by * dbz_dx + bz * (dby_dx - dbx_dy);
        const T vdp = N::div(N::div(T(1), static_cast<T>(s.charge)), drift_denominator);
        const T vdx = vdp * (muf1 * (-bz * db_dy) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                             muf1 * bx * bdot_curvb * ib3);
        const T vdy = vdp * (muf1 * (bz * db_dx) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                             muf1 * by * bdot_curvb * ib3);
        const T speed = N::div(static_cast<T>(s.particle_v0) * p, p0);
        if (!N::finite(speed) || speed <= T(0)) {
            st.status = 2;
            return false;
        }
        const T v_parallel_over_b = speed * pitch_mu * ib;
        const T vbx = v_parallel_over_b * bx;
        const T vby = v_parallel_over_b * by;
        dx_dt = vx + vdx + vbx + dkxx_dx + dkxy_dy;
        dy_dt = vy + vdy + vby + dkxy_dx + dkyy_dy;

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
        const T abs_mu = N::abs(pitch_mu);
        const T dtmp = N::pow(abs_mu, gamma - T(1)) + static_cast<T>(s.h0);
        const T duu0 = static_cast<T>(s.duu0);
        duu = duu0 * (T(1) - mu2) * dtmp;
        T duu_du = T(0);
        if (pitch_mu > T(0)) {
            duu_du = duu0 * (T(-2) * pitch_mu * dtmp + (T(1) - mu2) * N::pow(abs_mu, gamma - T(2)));
        } else if (pitch_mu < T(0)) {
            duu_du = duu0 * (T(-2) * pitch_mu * dtmp - (T(1) - mu2) * N::pow(abs_mu, gamma - T(2)));
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
        dmu_dt += duu_du;
        if (!N::finite(dmu_dt) || !N::finite(duu) || duu < T(0)) {
            st.status = 2;
            return false;
        }
    } else {
        const T vdp = N::div(N::div(T(1), T(3) * static_cast<T>(s.charge)), drift_denominator);
        const T vdx = vdp * (dbz_dy * ib2 - T(2) * bz * db_dy * ib3);
        const T vdy = vdp * (-dbz_dx * ib2 + T(2) * bz * db_dx * ib3);
        dx_dt = vx + vdx + dkxx_dx + dkxy_dy;
        dy_dt = vy + vdy + dkxy_dx + dkyy_dy;
        const T divv = dvx_dx + dvy_dy;
        dp_dt = N::div(-p * divv, T(3));
    }

    // Step-size control (src/main.cpp:1243-1277, :1596-1657).
    const T dxs = static_cast<T>(s.dx);
    const T dys = static_cast<T>(s.dy);
    T dtt;
    bool fixed = false;
    if (FOCUSED) {
        const T diffusion_scale = skperp > T(0) ? skperp : skpara;
        if (dx_dt != T(0) && dy_dt != T(0) && dp_dt != T(0) && dmu_dt != T(0) &&
            diffusion_scale > T(0)) {
            const T diffusion_dt_x = square(N::div(T(0.5) * dxs, diffusion_scale));
            const T diffusion_dt_y = square(N::div(T(0.5) * dys, diffusion_scale));
            const T advection_dt_x = square(N::div(diffusion_scale, dx_dt));
            const T advection_dt_y = square(N::div(diffusion_scale, dy_dt));
            const T momentum_dt = N::div(T(0.1) * p, N::abs(dp_dt));
            const T pitch_advection_dt = N::div(T(0.1), N::abs(dmu_dt));
            const T pitch_balance_dt = N::div(T(2) * duu, square(dmu_dt));
            dtt = min_positive(diffusion_dt_x, diffusion_dt_y);
            dtt = min_positive(dtt, advection_dt_x);
            dtt = min_positive(dtt, advection_dt_y);
            dtt = min_positive(dtt, momentum_dt);
            dtt = min_positive(dtt, pitch_advection_dt);
            dtt = min_positive(dtt, pitch_balance_dt);
        } else {
            fixed = true;
        }
    } else if (dx_dt != T(0) && dy_dt != T(0) && dp_dt != T(0)) {
        const T diffusion_dt_x = square(N::div(T(0.5) * dxs, skpara));
        const T diffusion_dt_y = square(N::div(T(0.5) * dys, skpara));
        const T advection_scale = skperp > T(0) ? skperp : skpara;
        const T advection_dt_x = square(N::div(advection_scale, dx_dt));
        const T advection_dt_y = square(N::div(advection_scale, dy_dt));
        const T momentum_dt = N::div(T(0.1) * p, N::abs(dp_dt));
        dtt = min_positive(diffusion_dt_x, diffusion_dt_y);
        dtt = min_positive(dtt, advection_dt_x);
        dtt = min_positive(dtt, advection_dt_y);
        dtt = min_positive(dtt, momentum_dt);
    } else {
        fixed = true;
    }
    double dt = fixed ? s.dt_min : static_cast<double>(dtt);
    if (dt < s.dt_min) {
        dt = s.dt_min;
    }
    if (dt > s.dt_max) {
        dt = s.dt_max;
    }
    st.diag_dt = dt;
    const double remaining = __dsub_rn(P.interval_end, st.t);
    if (dt > remaining) {
        dt = remaining;
    }
    if (!isfinite(dt) || dt <= 0.0) {
        st.status = 2;
        return false;
    }

    // Noise: four uniform_sqrt3 draws per substep, blocks 2(s-1), 2(s-1)+1.
    const uint32_t block = 2u * static_cast<uint32_t>(st.steps - 1);
    const uint4 r0 = philox4x32_10(make_uint4(block, st.index, P.frame, kTagPush), P.key);
    const uint4 r1 = philox4x32_10(make_uint4(block + 1u, st.index, P.frame, kTagPush), P.key);
    const T dtT = static_cast<T>(dt);
    const T sdt = N::sqrt(dtT);
    double delta_x, delta_y;
    if (FOCUSED) {
        const T ran1 = N::noise(r0.x, r0.y);
        const T ran2 = N::noise(r0.z, r0.w);
        const T pitch_random = N::noise(r1.z, r1.w);
        const T bxn = bx * ib;
        const T byn = by * ib;
        const T bzn = bz * ib;
        const T bxy_norm = N::sqrt(bxn * bxn + byn * byn);
        T stochastic_x = T(0);
        T stochastic_y = T(0);
        if (bxy_norm > T(0)) {
            const T ibxy_norm = N::div(T(1), bxy_norm);
            // (-by, +bx) on ran2 as written in src/main.cpp:1682-1687.
            stochastic_x = skperp * ibxy_norm * sdt * (-bxn * bzn * ran1 - by * ran2);
            stochastic_y = skperp * ibxy_norm * sdt * (-byn * bzn * ran1 + bx * ran2);
        }
        delta_x = static_cast<double>(dx_dt * dtT + stochastic_x);
        delta_y = static_cast<double>(dy_dt * dtT + stochastic_y);
        st.mu = clamp_mu(pitch_mu + dmu_dt * dtT + pitch_random * N::sqrt(T(2) * duu) * sdt,
                         static_cast<T>(s.mu_max));
    } else {
        const T ran1 = N::noise(r0.x, r0.y);
        const T ran2 = N::noise(r0.z, r0.w);
        const T ran3 = N::noise(r1.x, r1.y);
        delta_x = static_cast<double>(dx_dt * dtT + ran1 * skperp * sdt +
                                      ran3 * skpara_perp * sdt * bx * ib);
        delta_y = static_cast<double>(dy_dt * dtT + ran2 * skperp * sdt +
                                      ran3 * skpara_perp * sdt * by * ib);
    }
    const double delta_p = static_cast<double>(dp_dt * dtT);

    st.x = __dadd_rn(st.x, delta_x);
    st.y = __dadd_rn(st.y, delta_y);
    st.p = __dadd_rn(st.p, delta_p);
    st.t = __dadd_rn(st.t, dt);
    const double pfloor = 0.25 * s.p0;
    if (st.p < pfloor) {
        st.p = pfloor;
    }
    if (!isfinite(st.x) || !isfinite(st.y) || !isfinite(st.p) || !isfinite(st.t)) {
        st.status = 2;
        return false;
    }
    return st.t < P.interval_end && st.steps < s.max_steps;
}

template <typename T, bool FOCUSED>
__device__ __forceinline__ void load_state(State<T>& st, const PushParams& P, uint32_t index) {
    const ParticleArrays& a = P.parts;
    st.index = index;
    st.x = a.x[index];
    st.y = a.y[index];
    st.p = a.p[index];
    st.t = a.t[index];
    st.dt = a.step_dt[index];
    st.diag_dt = st.dt;
    st.mu = FOCUSED ? clamp_mu(static_cast<T>(a.mu[index]), static_cast<T>(P.s.mu_max)) : T(0);
    st.steps = 0;
    st.status = 0;
}

template <typename T, bool FOCUSED>
__device__ __forceinline__ void store_state(State<T>& st, const PushParams& P) {
    const ParticleArrays& a = P.parts;
    const DeviceSettings& s = P.s;
    if (st.steps >= s.max_steps && st.t < P.interval_end) {
        st.status = 2;
    }
    const uint32_t i = st.index;
    a.x[i] = wrap_driver(st.x, s.x_lower, s.x_upper, s.x_width);
    a.y[i] = wrap_driver(st.y, s.y_lower, s.y_upper, s.y_width);
    a.p[i] = st.p;
    a.t[i] = st.t;
    a.step_dt[i] = st.diag_dt;
    if (FOCUSED) {
        a.mu[i] = static_cast<double>(st.mu);
    }
    a.status[i] = st.status;
}

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

// Persistent warps with lane refill.  Each warp claims particles from the
// cursor in batches of (number of idle lanes); a lane advances its particle
// by one substep per loop trip and refills when the particle is done.  The
// loop ends when the cursor is past `count` and no lane holds a particle;
// every trip either advances a particle or moves the cursor, so it always
// terminates.
template <typename T, bool FOCUSED>
__global__ void __launch_bounds__(128) push_refill_kernel(const PushParams P) {
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    State<T> st;
    bool have = false;
    bool exhausted = false;
    unsigned long long my_steps = 0, my_pushed = 0, my_failed = 0;
    unsigned int my_max = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(full, !have);
        if (idle != 0u && !exhausted) {
            const unsigned n_idle = __popc(idle);
            unsigned base = 0;
            const int leader = __ffs(idle) - 1;
            if (static_cast<int>(lane) == leader) {
                base = atomicAdd(&P.counters->next_particle, n_idle);
            }
            base = __shfl_sync(full, base, leader);
            if (static_cast<uint64_t>(base) + n_idle >= P.count) {
                exhausted = true;
            }
            if (!have) {
                const uint64_t idx = static_cast<uint64_t>(base) + __popc(idle & lanes_below);
                if (idx < P.count && P.parts.status[idx] == 0) {
                    load_state<T, FOCUSED>(st, P, static_cast<uint32_t>(idx));
                    ++my_pushed;
                    have = true;
                    if (!(st.t < P.interval_end && st.steps < P.s.max_steps)) {
                        store_state<T, FOCUSED>(st, P);
                        have = false;
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
        if (have) {
            if (!substep<T, FOCUSED>(st, P)) {
                store_state<T, FOCUSED>(st, P);
                my_steps += static_cast<unsigned long long>(st.steps);
                my_max = max(my_max, static_cast<unsigned int>(st.steps));
                if (st.status != 0) {
                    ++my_failed;
                }
                have = false;
            }
        }
    }
    flush_counters(P.counters, my_steps, my_pushed, my_failed, my_max);
}

// One particle per thread, no refill (kept for the schedule tuner).
template <typename T, bool FOCUSED>
__global__ void __launch_bounds__(128) push_simple_kernel(const PushParams P) {
    unsigned long long my_steps = 0, my_pushed = 0, my_failed = 0;
    unsigned int my_max = 0;
    for (uint64_t idx = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
         idx < P.count; idx += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        if (P.parts.status[idx] != 0) {
            continue;
        }
        State<T> st;
        load_state<T, FOCUSED>(st, P, static_cast<uint32_t>(idx));
        ++my_pushed;
        if (st.t < P.interval_end && st.steps < P.s.max_steps) {
            while (substep<T, FOCUSED>(st, P)) {
            }
        }
        store_state<T, FOCUSED>(st, P);
        my_steps += static_cast<unsigned long long>(st.steps);
        my_max = max(my_max, static_cast<unsigned int>(st.steps));
        if (st.status != 0) {
            ++my_failed;
        }
    }
    flush_counters(P.counters, my_steps, my_pushed, my_failed, my_max);
}

template <typename T, bool FOCUSED>
cudaError_t launch_push(const PushLaunch& L, cudaStream_t stream) {
    PushParams P;
    P.grid = L.grid;
    P.lower = L.lower;
    P.upper = L.upper;
    P.parts = L.parts;
    P.count = L.count;
    P.s = L.settings;
    P.interval_start = L.interval_start;
    P.interval_end = L.interval_end;
    P.frame = L.frame;
    P.key = make_uint2(static_cast<uint32_t>(L.seed), static_cast<uint32_t>(L.seed >> 32));
    P.counters = L.counters;
    const int threads = 128;
    if (L.schedule == kScheduleSimple) {
        const uint64_t want = (L.count + threads - 1) / threads;
        const int blocks = static_cast<int>(want < 1 ? 1 : (want > 65535u * 8u ? 65535u * 8u : want));
        push_simple_kernel<T, FOCUSED><<<blocks, threads, 0, stream>>>(P);
    } else {
        const int blocks = L.sm_count * L.blocks_per_sm;
        push_refill_kernel<T, FOCUSED><<<blocks, threads, 0, stream>>>(P);
    }
    return cudaGetLastError();
}

// Table values at given positions, through the push's own sampling path
// (driver wrap, half-cell shift, grid wrap, stencil, time interpolation).
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

cudaError_t launch_sample(const SampleLaunch& L, cudaStream_t stream) {
    if (L.n == 0) {
        return cudaSuccess;
    }
    const int threads = 128;
    const uint64_t want = (L.n + threads - 1) / threads;
    const int blocks = static_cast<int>(want > 152u * 16u ? 152u * 16u : want);
    if (L.precision == kPrecisionF64) {
        if (L.focused) {
            sample_kernel<double, true><<<blocks, threads, 0, stream>>>(L);
        } else {
            sample_kernel<double, false><<<blocks, threads, 0, stream>>>(L);
        }
    } else {
        if (L.focused) {
            sample_kernel<float, true><<<blocks, threads, 0, stream>>>(L);
        } else {
            sample_kernel<float, false><<<blocks, threads, 0, stream>>>(L);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_push_interval(const PushLaunch& launch, cudaStream_t stream) {
    if (launch.precision == kPrecisionF64) {
        return launch.focused ? launch_push<double, true>(launch, stream)
                              : launch_push<double, false>(launch, stream);
    }
    return launch.focused ? launch_push<float, true>(launch, stream)
                          : launch_push<float, false>(launch, stream);
}

}  // namespace kpt
