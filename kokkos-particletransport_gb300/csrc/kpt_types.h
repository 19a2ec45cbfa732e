// Plain structs shared by the host library and the kernels.
#pragma once

#include <cstdint>

namespace kpt {

// One periodic axis with two ghost layers.  Uniform axes use the analytic map
// (start + i*step); non-uniform axes keep their ghosted cell centres in
// device memory plus a bucket index that seeds the interval search.
struct Axis {
    int n;
    int stored;
    double start;
    double step;
    double lower;      // physical face bounds
    double upper;
    double width;
    double inv_width;
    const double* centers;   // stored: n+4 centres, logical -2..n+1
    const int* buckets;      // stored: first interval index per bucket
    int bucket_count;
    double bucket_origin;
    double bucket_scale;
};

struct Grid {
    Axis axis[2];
    int ex;  // nx + 4: point stride of one ghosted row
};

// The same axis as seen by the mixed-precision push, whose positions are
// 64-bit fixed-point phases over the periodic width: x = lower + width *
// phase / 2^64.
struct FixedAxis {
    int n;
    int stored;
    uint64_t half_cell;            // phase of half a mean cell, 2^63 / n
    float to_fixed;                // 2^64 / width
    const long long* centers;      // stored: n+4 ghosted centres, (c - lower) / width * 2^62
    const float* inv_spacing;      // stored: n+3 entries, 2^spacing_shift / (C[k+1] - C[k])
    const int* buckets;            // stored: first interval index per phase bucket
    int bucket_shift;              // phase >> bucket_shift = bucket
    int spacing_shift;
};

struct FixedGrid {
    FixedAxis axis[2];
    float dt_min;
    float dt_max;
    float tau_per_time;        // 2^62 / mhd_dt (fixed-point time units per time unit)
    float time_per_tau_2_32;   // mhd_dt / 2^30 (time per 2^32 fixed-point units)
    float pfloor_hi;           // 0.25 p0 as a float pair
    float pfloor_lo;
};

// Device copy of the driver's settings after make_device_settings
// (reference src/main.cpp:596-636).
struct DeviceSettings {
    double x_lower, x_upper, y_lower, y_upper, x_width, y_width, dx, dy;
    double shift_x, shift_y;
    double mhd_dt, p0, pmax, gamma_turb, pindex, kpara0, kperp_over_kpara;
    double dt_min, dt_max, drift_param1, drift_param2, charge, particle_v0, duu0;
    double h0, split_ratio, pmin_split, mu_max;
    int max_steps, momentum_dependency, magnetic_dependency, time_interpolation;
    int split_particles, focused;
    // focused scattering closure (kpt_closure) and its slab-QLT parameters;
    // qlt_norm = gamma_k sin(pi / gamma_k) / pi, computed on the host
    int closure;
    double qlt_sigma2, qlt_gk, qlt_h0, qlt_omega0, qlt_lc, qlt_norm;
};

struct ParticleArrays {
    double* x;
    double* y;
    double* p;
    double* t;
    double* step_dt;
    double* weight;
    double* mu;
    int32_t* status;
    int32_t* split_level;
};

// Device-side counters written by the push.
struct PushCounters {
    unsigned long long particle_steps;
    unsigned long long pushed;
    unsigned long long failed;
    unsigned int max_steps;
    unsigned int next_particle;  // work-queue cursor
    unsigned int network_timeouts;  // blocks stopped by a tensor-core completion timeout
    unsigned int teardown_incomplete;  // of those, blocks whose MMAs were still in flight
                                       // when their tensor memory was freed
};

}  // namespace kpt
