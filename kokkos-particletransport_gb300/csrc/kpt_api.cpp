// C-ABI layer of libkpt: handles, validation, host-side file reading and the
// launches of the device kernels.  Every entry point returns a kpt_status and
// records a message for kpt_last_error() on failure; there is no CPU path.
#include "kpt.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "kpt_internal.h"
#include "kpt_pow.h"

// One substep in KPT_JUDGE_PERIOD (a power of two) of every particle also
// evaluates the plain closure to judge the learned one.
#ifndef KPT_JUDGE_PERIOD
#define KPT_JUDGE_PERIOD 64
#endif

namespace {

thread_local std::string g_last_error;

int set_error(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

#define KPT_CUDA(expr)                                                                  \
    do {                                                                                \
        const cudaError_t kpt_err_ = (expr);                                            \
        if (kpt_err_ != cudaSuccess) {                                                  \
            return set_error(kpt_err_ == cudaErrorMemoryAllocation ? KPT_ERROR_OUT_OF_MEMORY \
                                                                   : KPT_ERROR_CUDA,    \
                             std::string(#expr) + ": " + cudaGetErrorString(kpt_err_)); \
        }                                                                               \
    } while (0)

#define KPT_REQUIRE(cond, message)                                   \
    do {                                                             \
        if (!(cond)) {                                               \
            return set_error(KPT_ERROR_INVALID_ARGUMENT, (message)); \
        }                                                            \
    } while (0)

// Growable device buffer owned by a context.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t want) {
        if (want <= bytes) {
            return cudaSuccess;
        }
        if (ptr != nullptr) {
            cudaFree(ptr);
            ptr = nullptr;
            bytes = 0;
        }
        const cudaError_t err = cudaMalloc(&ptr, want);
        if (err == cudaSuccess) {
            bytes = want;
        }
        return err;
    }
    void release() {
        if (ptr != nullptr) {
            cudaFree(ptr);
        }
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(ptr);
    }
};

// A DeviceBuffer freed when it goes out of scope (scratch of one call; the
// call synchronises its stream before returning).
struct ScopedBuffer : DeviceBuffer {
    ScopedBuffer() = default;
    ScopedBuffer(const ScopedBuffer&) = delete;
    ScopedBuffer& operator=(const ScopedBuffer&) = delete;
    ~ScopedBuffer() { release(); }
};

}  // namespace

struct kpt_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    DeviceBuffer counters;
    DeviceBuffer split_counts, split_offsets, split_totals, split_levels;
    double split_key[3] = {0.0, 0.0, 0.0};
    int split_level_count = 0;
    DeviceBuffer hist_bins, hist_edge_count, hist_edge_index;
    DeviceBuffer summary_partials, summary_result;
    DeviceBuffer sample_io;
    kpt_surrogate* surrogate = nullptr;
    DeviceBuffer judge;
    int push_schedule = kpt::kScheduleRefill;
    int fp64_arithmetic = KPT_FP64_STRICT;
    int push_blocks_per_sm = 0;  // 0: as many as fit (occupancy)
    // cell records of the last table pair a mixed push used (by field serial),
    // the stream they were built on and an event marking the build's end
    DeviceBuffer records;
    uint64_t records_lower = 0, records_upper = 0;
    int records_mode = KPT_RECORDS_AUTO;
    cudaStream_t records_stream = nullptr;
    cudaEvent_t records_ready = nullptr;
};

struct kpt_surrogate {
    kpt_context* ctx = nullptr;
    int device = 0;
    kpt::SurrogateBox box{};
    std::vector<float> params;  // FP32 trained parameters
    float* d_params = nullptr;  // FP32 copy (SIMT evaluation)
    uint2* d_block = nullptr;   // BF16 mma.sync B fragments + FP32 biases
    uint4* d_tc_block = nullptr;  // tcgen05 B operands, biases folded in (canonical layout)
    int engine = kpt::kEngineTcgen05;
    double final_loss = 0.0;
    // settings the targets were generated with (checked at push time)
    double kperp_over_kpara = 0.0;
};

struct kpt_field {
    kpt_context* ctx = nullptr;
    int device = 0;
    int nx = 0, ny = 0;
    int kind = 0, precision = 0, stride = 0;
    uint64_t points = 0;
    void* table = nullptr;
    double* centers[2] = {nullptr, nullptr};
    int* buckets[2] = {nullptr, nullptr};
    long long* fixed_centers[2] = {nullptr, nullptr};
    float* fixed_spacing[2] = {nullptr, nullptr};
    int* fixed_buckets[2] = {nullptr, nullptr};
    kpt::Grid grid{};
    kpt::FixedAxis fixed[2]{};
    uint64_t serial = 0;  // unique per field of the process (record cache key)
};

struct kpt_field_data {
    int nx = 0, ny = 0;
    std::vector<double> x_edges, y_edges;
    double* cells = nullptr;  // Bx By Bz Vx Vy Vz (ny x nx each), page-locked
};

struct kpt_particles {
    kpt_context* ctx = nullptr;
    int device = 0;
    uint64_t capacity = 0;
    uint64_t count = 0;
    void* block = nullptr;  // owned storage; NULL for wrapped external arrays
    kpt::ParticleArrays arrays{};
    // Work order from the last cell sort; valid while count is unchanged.
    DeviceBuffer order, keys, tile_counts;
    bool order_valid = false;
};

namespace {

bool edges_uniform(const double* e, int n, double* step_out) {
    const double span = e[n] - e[0];
    const double step = span / static_cast<double>(n);
    if (!std::isfinite(step) || step <= 0.0) {
        return false;
    }
    for (int i = 1; i <= n; ++i) {
        const double current = e[i] - e[i - 1];
        const double magnitude =
            std::max({std::fabs(span), std::fabs(step), std::fabs(current), 1.0});
        const double tolerance = 1024.0 * std::numeric_limits<double>::epsilon() * magnitude;
        if (std::fabs(current - step) > tolerance) {
            return false;
        }
    }
    *step_out = step;
    return true;
}

// Axis map for one dimension (analytic if the edges are uniform by the
// reference reader's test, AthenaFieldReader.hpp:167-193; stored otherwise).
int build_axis(int n, const double* e, kpt::Axis& axis, std::vector<double>& centers,
               std::vector<int>& buckets) {
    for (int i = 0; i <= n; ++i) {
        if (!std::isfinite(e[i])) {
            return set_error(KPT_ERROR_FORMAT, "field: non-finite face coordinate");
        }
        if (i > 0 && !(e[i] > e[i - 1])) {
            return set_error(KPT_ERROR_FORMAT,
                             "field: face coordinates must be strictly ascending");
        }
    }
    axis = kpt::Axis{};
    axis.n = n;
    double step = 0.0;
    if (edges_uniform(e, n, &step)) {
        const double x0 = e[0];
        axis.stored = 0;
        axis.start = x0;
        axis.step = step;
        axis.lower = x0 + 0.0 * step;
        axis.upper = x0 + static_cast<double>(n) * step;
    } else {
        const double w = e[n] - e[0];
        std::vector<double> faces(static_cast<size_t>(n) + 5);
        for (int k = -2; k <= n + 2; ++k) {
            faces[k + 2] = k < 0 ? e[n + k] - w : (k > n ? e[k - n] + w : e[k]);
        }
        centers.resize(static_cast<size_t>(n) + 4);
        for (int s = 0; s < n + 4; ++s) {
            centers[s] = 0.5 * (faces[s] + faces[s + 1]);
        }
        axis.stored = 1;
        axis.lower = faces[2];
        axis.upper = faces[n + 2];
        // Bucket index: for each of 4(n+4) equal buckets over the centre
        // range, the interval whose left centre is the last <= bucket start.
        const int m = 4 * (n + 4);
        const double origin = centers.front();
        const double span = centers.back() - origin;
        buckets.resize(static_cast<size_t>(m));
        int k = -2;
        for (int b = 0; b < m; ++b) {
            const double x = origin + span * (static_cast<double>(b) / m);
            while (k < n && centers[k + 3] <= x) {
                ++k;
            }
            buckets[b] = k;
        }
        axis.bucket_count = m;
        axis.bucket_origin = origin;
        axis.bucket_scale = static_cast<double>(m) / span;
    }
    axis.width = axis.upper - axis.lower;
    axis.inv_width = axis.width != 0.0 ? 1.0 / axis.width : 0.0;
    return KPT_OK;
}

// Fixed-point description of an axis for the mixed-precision push (phase =
// (x - lower) / width * 2^64).  Stretched axes get their ghosted cell
// centres at a 2^62 scale, the per-interval inverse spacing and a bucket
// table that seeds the interval search.
struct FixedAxisHost {
    kpt::FixedAxis axis{};
    std::vector<long long> centers;
    std::vector<float> inv_spacing;
    std::vector<int> buckets;
};

FixedAxisHost build_fixed_axis(const kpt::Axis& a, const std::vector<double>& centers) {
    FixedAxisHost h;
    h.axis.n = a.n;
    h.axis.stored = a.stored;
    h.axis.half_cell = 9223372036854775808ull / static_cast<unsigned long long>(a.n);
    h.axis.to_fixed = static_cast<float>(18446744073709551616.0 / a.width);
    if (!a.stored) {
        return h;
    }
    const long double scale = 4611686018427387904.0L / static_cast<long double>(a.width);
    h.centers.resize(centers.size());
    for (size_t k = 0; k < centers.size(); ++k) {
        h.centers[k] = static_cast<long long>(
            std::llround(static_cast<long double>(centers[k] - a.lower) * scale));
    }
    long long max_spacing = 1;
    for (size_t k = 0; k + 1 < h.centers.size(); ++k) {
        max_spacing = std::max(max_spacing, h.centers[k + 1] - h.centers[k]);
    }
    int bits = 0;
    while (bits < 63 && (max_spacing >> bits) != 0) {
        ++bits;
    }
    const int shift = std::max(0, bits - 31);
    h.axis.spacing_shift = shift;
    h.inv_spacing.resize(h.centers.size() - 1);
    for (size_t k = 0; k + 1 < h.centers.size(); ++k) {
        h.inv_spacing[k] = static_cast<float>(std::ldexp(1.0, shift) /
                                              static_cast<double>(h.centers[k + 1] - h.centers[k]));
    }
    int log2b = 0;
    while ((1 << log2b) < 4 * (a.n + 4) && log2b < 20) {
        ++log2b;
    }
    h.axis.bucket_shift = 64 - log2b;
    h.buckets.resize(static_cast<size_t>(1) << log2b);
    int k = -2;
    for (size_t b = 0; b < h.buckets.size(); ++b) {
        const long long start = static_cast<long long>(
            (static_cast<unsigned long long>(b) << h.axis.bucket_shift) >> 2);
        while (k < a.n && h.centers[k + 3] <= start) {
            ++k;
        }
        h.buckets[b] = k;
    }
    return h;
}

// Reconnection2DSettings::validate, physics block (src/main.cpp:222-239).
int validate_settings(const kpt_settings* s) {
    if (s == nullptr) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT, "settings is NULL");
    }
    const bool ok = std::isfinite(s->mhd_dt) && s->mhd_dt > 0.0 && std::isfinite(s->p0) &&
                    s->p0 > 0.0 && std::isfinite(s->pmin) && s->pmin > 0.0 &&
                    std::isfinite(s->pmax) && s->pmax > s->pmin &&
                    std::isfinite(s->gamma_turb) && std::isfinite(s->kpara0) &&
                    s->kpara0 > 0.0 && std::isfinite(s->kperp_over_kpara) &&
                    s->kperp_over_kpara >= 0.0 && std::isfinite(s->dt_min_rel) &&
                    s->dt_min_rel > 0.0 && std::isfinite(s->dt_max_rel) &&
                    s->dt_max_rel >= s->dt_min_rel && std::isfinite(s->drift_param1) &&
                    std::isfinite(s->drift_param2) && std::isfinite(s->charge) &&
                    s->charge != 0.0 && std::isfinite(s->particle_v0) &&
                    s->particle_v0 > 0.0 && std::isfinite(s->duu0) && s->duu0 >= 0.0 &&
                    std::isfinite(s->split_ratio) && s->split_ratio > 1.0 &&
                    std::isfinite(s->pmin_split_over_p0) && s->pmin_split_over_p0 > 0.0 &&
                    std::isfinite(s->mu_max) && s->mu_max > 0.0;
    if (!ok) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "Reconnection2DSettings: invalid physical parameters.");
    }
    if (s->max_steps <= 0) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "Reconnection2DSettings: step guard must be positive.");
    }
    if (s->closure != KPT_CLOSURE_DRIVER) {
        // PitchAngleScatteringParameters::validate (LegencyModel.hpp:205-221)
        // plus positive Omega_0, L_c and sigma^2 (LegencyModel.hpp:566-570)
        const bool qlt_ok = (s->closure == KPT_CLOSURE_QLT || s->closure == KPT_CLOSURE_SURROGATE) &&
                            std::isfinite(s->qlt_spectral_index) && s->qlt_spectral_index > 1.0 &&
                            std::isfinite(s->qlt_h0) && s->qlt_h0 > 0.0 &&
                            std::isfinite(s->qlt_sigma2) && s->qlt_sigma2 > 0.0 &&
                            std::isfinite(s->qlt_omega0) && s->qlt_omega0 > 0.0 &&
                            std::isfinite(s->qlt_lc) && s->qlt_lc > 0.0;
        if (!qlt_ok) {
            return set_error(KPT_ERROR_INVALID_ARGUMENT,
                             "kpt_settings: invalid scattering closure parameters.");
        }
    }
    return KPT_OK;
}

// make_device_settings (src/main.cpp:596-636).
kpt::DeviceSettings device_settings(const kpt_settings* s, const kpt::Grid& g) {
    kpt::DeviceSettings d{};
    d.x_lower = g.axis[0].lower;
    d.x_upper = g.axis[0].upper;
    d.y_lower = g.axis[1].lower;
    d.y_upper = g.axis[1].upper;
    d.x_width = d.x_upper - d.x_lower;
    d.y_width = d.y_upper - d.y_lower;
    d.dx = d.x_width / static_cast<double>(g.axis[0].n);
    d.dy = d.y_width / static_cast<double>(g.axis[1].n);
    d.shift_x = 0.5 * d.dx;
    d.shift_y = 0.5 * d.dy;
    d.mhd_dt = s->mhd_dt;
    d.p0 = s->p0;
    d.pmax = s->pmax;
    d.gamma_turb = s->gamma_turb;
    d.pindex = 3.0 - s->gamma_turb;
    d.kpara0 = s->kpara0;
    d.kperp_over_kpara = s->kperp_over_kpara;
    d.dt_min = s->dt_min_rel * s->mhd_dt;
    d.dt_max = s->dt_max_rel * s->mhd_dt;
    d.drift_param1 = s->drift_param1;
    d.drift_param2 = s->drift_param2;
    d.charge = s->charge;
    d.particle_v0 = s->particle_v0;
    d.duu0 = s->duu0;
    d.h0 = 0.2;  // Reconnection2DDeviceSettings::pitch_angle_scattering_h0
    d.split_ratio = s->split_ratio;
    d.pmin_split = s->pmin_split_over_p0 * s->p0;
    d.mu_max = s->mu_max;
    d.max_steps = s->max_steps;
    d.momentum_dependency = s->momentum_dependency;
    d.magnetic_dependency = s->magnetic_dependency;
    d.time_interpolation = s->time_interpolation;
    d.split_particles = s->split_particles;
    d.focused = s->focused;
    d.closure = s->closure;
    d.qlt_sigma2 = s->qlt_sigma2;
    d.qlt_gk = s->qlt_spectral_index;
    d.qlt_h0 = s->qlt_h0;
    d.qlt_omega0 = s->qlt_omega0;
    d.qlt_lc = s->qlt_lc;
    // pitch_angle_spectrum_normalization (LegencyModel.hpp:539-552)
    const double pi = 3.141592653589793238462643383279502884;
    d.qlt_norm = s->qlt_spectral_index * std::sin(pi / s->qlt_spectral_index) / pi;
    return d;
}

int activate(kpt_context* ctx) {
    KPT_CUDA(cudaSetDevice(ctx->device));
    return KPT_OK;
}

}  // namespace

extern "C" {

int kpt_abi_version(void) { return KPT_ABI_VERSION; }

const char* kpt_last_error(void) { return g_last_error.c_str(); }

void kpt_default_settings(kpt_settings* s) {
    if (s == nullptr) {
        return;
    }
    std::memset(s, 0, sizeof(*s));
    s->mhd_dt = 0.1;
    s->p0 = 0.1;
    s->pmin = 1.0e-2;
    s->pmax = 1.0e1;
    s->gamma_turb = 1.6666667;
    s->kpara0 = 0.00743592;
    s->kperp_over_kpara = 0.01;
    s->dt_min_rel = 1.0e-7;
    s->dt_max_rel = 1.0e-2;
    s->drift_param1 = 850964.408;
    s->drift_param2 = 13575468.975;
    s->charge = -1.0;
    s->particle_v0 = 17.20195;
    s->duu0 = 5578.445;
    s->split_ratio = 2.0;
    s->pmin_split_over_p0 = 2.0;
    s->mu_max = 0.99;
    s->max_steps = 200000;
    s->momentum_dependency = 1;
    s->magnetic_dependency = 1;
    s->time_interpolation = 1;
    s->split_particles = 1;
    s->focused = 0;
    s->closure = KPT_CLOSURE_DRIVER;
    s->qlt_sigma2 = 0.1;
    s->qlt_spectral_index = 5.0 / 3.0;
    s->qlt_h0 = 1.0e-6;
    s->qlt_omega0 = 1000.0;
    s->qlt_lc = 0.05;
}

int kpt_context_create(int device, kpt_context** out) {
    KPT_REQUIRE(out != nullptr, "kpt_context_create: out is NULL");
    *out = nullptr;
    int count = 0;
    const cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess || count == 0) {
        return set_error(KPT_ERROR_NO_DEVICE,
                         std::string("kpt_context_create: no CUDA device (") +
                             cudaGetErrorString(err) + ")");
    }
    KPT_REQUIRE(device >= 0 && device < count, "kpt_context_create: device out of range");
    std::unique_ptr<kpt_context> ctx(new (std::nothrow) kpt_context());
    if (!ctx) {
        return set_error(KPT_ERROR_OUT_OF_MEMORY, "kpt_context_create: host allocation");
    }
    ctx->device = device;
    KPT_CUDA(cudaSetDevice(device));
    int major = 0;
    KPT_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
    KPT_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
    KPT_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
    ctx->stream = ctx->own_stream;
    KPT_CUDA(ctx->counters.reserve(sizeof(kpt::PushCounters)));
    *out = ctx.release();
    return KPT_OK;
}

int kpt_context_destroy(kpt_context* ctx) {
    if (ctx == nullptr) {
        return KPT_OK;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (DeviceBuffer* b : {&ctx->counters, &ctx->split_counts, &ctx->split_offsets,
                            &ctx->split_totals, &ctx->split_levels, &ctx->hist_bins,
                            &ctx->hist_edge_count, &ctx->hist_edge_index,
                            &ctx->summary_partials, &ctx->summary_result, &ctx->sample_io,
                            &ctx->judge, &ctx->records}) {
        b->release();
    }
    if (ctx->records_ready != nullptr) {
        cudaEventDestroy(ctx->records_ready);
    }
    if (ctx->own_stream != nullptr) {
        cudaStreamDestroy(ctx->own_stream);
    }
    delete ctx;
    return KPT_OK;
}

int kpt_context_set_stream(kpt_context* ctx, void* cuda_stream) {
    KPT_REQUIRE(ctx != nullptr, "kpt_context_set_stream: ctx is NULL");
    ctx->stream = cuda_stream != nullptr ? static_cast<cudaStream_t>(cuda_stream)
                                         : ctx->own_stream;
    return KPT_OK;
}

int kpt_context_set_push_schedule(kpt_context* ctx, int schedule, int blocks_per_sm) {
    KPT_REQUIRE(ctx != nullptr, "kpt_context_set_push_schedule: ctx is NULL");
    KPT_REQUIRE(schedule == KPT_SCHEDULE_REFILL || schedule == KPT_SCHEDULE_SIMPLE,
                "kpt_context_set_push_schedule: unknown schedule");
    KPT_REQUIRE(blocks_per_sm >= 0 && blocks_per_sm <= 32,
                "kpt_context_set_push_schedule: blocks_per_sm must be in [0, 32]");
    ctx->push_schedule = schedule == KPT_SCHEDULE_SIMPLE ? kpt::kScheduleSimple
                                                         : kpt::kScheduleRefill;
    ctx->push_blocks_per_sm = blocks_per_sm;
    return KPT_OK;
}

int kpt_context_set_fp64_arithmetic(kpt_context* ctx, int mode) {
    KPT_REQUIRE(ctx != nullptr, "kpt_context_set_fp64_arithmetic: ctx is NULL");
    KPT_REQUIRE(mode == KPT_FP64_STRICT || mode == KPT_FP64_CONTRACTED,
                "kpt_context_set_fp64_arithmetic: mode must be KPT_FP64_STRICT or "
                "KPT_FP64_CONTRACTED");
    ctx->fp64_arithmetic = mode;
    return KPT_OK;
}

int kpt_context_set_cell_records(kpt_context* ctx, int mode) {
    KPT_REQUIRE(ctx != nullptr, "kpt_context_set_cell_records: ctx is NULL");
    KPT_REQUIRE(mode == KPT_RECORDS_AUTO || mode == KPT_RECORDS_OFF || mode == KPT_RECORDS_ON,
                "kpt_context_set_cell_records: mode must be KPT_RECORDS_AUTO, KPT_RECORDS_OFF "
                "or KPT_RECORDS_ON");
    ctx->records_mode = mode;
    return KPT_OK;
}

int kpt_context_synchronize(kpt_context* ctx) {
    KPT_REQUIRE(ctx != nullptr, "kpt_context_synchronize: ctx is NULL");
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_context_fp64_fma_rate(kpt_context* ctx, double* tflops) {
    KPT_REQUIRE(ctx != nullptr && tflops != nullptr, "kpt_context_fp64_fma_rate: NULL argument");
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(kpt::fp64_fma_rate(ctx->sm_count, ctx->stream, tflops));
    return KPT_OK;
}

int kpt_math_pow(kpt_context* ctx, uint64_t n, const double* x, const double* y, double* out) {
    KPT_REQUIRE(ctx != nullptr && (n == 0 || (x && y && out)), "kpt_math_pow: NULL argument");
    if (n == 0) return KPT_OK;
    if (int rc = activate(ctx)) return rc;
    ScopedBuffer buf;
    KPT_CUDA(buf.reserve(3 * n * sizeof(double)));
    double* dx = buf.as<double>();
    double* dy = dx + n;
    double* dout = dy + n;
    KPT_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(dy, y, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(kpt::launch_pow(n, dx, dy, dout, ctx->sm_count, ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

namespace {
int field_create(kpt_context* ctx, int nx, int ny, const double* x_edges, const double* y_edges,
                 const double* b_cells, const double* v_cells, int table_kind, int precision,
                 const double* b_device, const double* v_device, kpt_field** out);
}  // namespace

int kpt_field_create(kpt_context* ctx, int nx, int ny, const double* x_edges,
                     const double* y_edges, const double* b_cells, const double* v_cells,
                     int table_kind, int precision, kpt_field** out) {
    return field_create(ctx, nx, ny, x_edges, y_edges, b_cells, v_cells, table_kind, precision,
                        nullptr, nullptr, out);
}

}  // extern "C"

namespace {

// b_device / v_device (optional): device addresses of mapped page-locked
// cells the kernels read in place (NVLink-C2C / PCIe reads), so no staging
// copy is made; b_cells / v_cells stay the host view used for validation.
int field_create(kpt_context* ctx, int nx, int ny, const double* x_edges, const double* y_edges,
                 const double* b_cells, const double* v_cells, int table_kind, int precision,
                 const double* b_device, const double* v_device, kpt_field** out) {
    const bool device_readable = b_device != nullptr && v_device != nullptr;
    KPT_REQUIRE(ctx != nullptr && out != nullptr, "kpt_field_create: NULL handle");
    *out = nullptr;
    KPT_REQUIRE(nx > 0 && ny > 0, "AthenaFieldReader: Athena binary dimensions must be positive.");
    KPT_REQUIRE(x_edges && y_edges && b_cells && v_cells, "kpt_field_create: NULL array");
    KPT_REQUIRE(table_kind == KPT_TABLE_PARKER16 || table_kind == KPT_TABLE_FOCUSED21,
                "kpt_field_create: unknown table kind");
    KPT_REQUIRE(precision == KPT_PRECISION_F64 || precision == KPT_PRECISION_MIXED,
                "kpt_field_create: unknown precision");
    const size_t cells = static_cast<size_t>(nx) * static_cast<size_t>(ny);
    // data read by kpt_field_data_read was checked on the reading thread
    for (size_t k = 0; !device_readable && k < 3 * cells; ++k) {
        if (!std::isfinite(b_cells[k]) || !std::isfinite(v_cells[k])) {
            return set_error(KPT_ERROR_FORMAT, "AthenaFieldReader: non-finite field value.");
        }
    }
    if (int rc = activate(ctx)) return rc;
    struct FieldDeleter {
        void operator()(kpt_field* doomed) const { kpt_field_destroy(doomed); }
    };
    std::unique_ptr<kpt_field, FieldDeleter> f(new kpt_field());
    static std::atomic<uint64_t> next_serial{1};
    f->serial = next_serial.fetch_add(1);
    f->ctx = ctx;
    f->device = ctx->device;
    f->nx = nx;
    f->ny = ny;
    f->kind = table_kind;
    f->precision = precision;
    f->stride = kpt::table_stride(table_kind == KPT_TABLE_FOCUSED21, precision);
    f->points = static_cast<uint64_t>(nx + 4) * static_cast<uint64_t>(ny + 4);
    f->grid.ex = nx + 4;
    const double* edges[2] = {x_edges, y_edges};
    const int counts[2] = {nx, ny};
    for (int d = 0; d < 2; ++d) {
        std::vector<double> centers;
        std::vector<int> buckets;
        if (int rc = build_axis(counts[d], edges[d], f->grid.axis[d], centers, buckets)) {
            return rc;
        }
        FixedAxisHost fixed = build_fixed_axis(f->grid.axis[d], centers);
        f->fixed[d] = fixed.axis;
        if (!centers.empty()) {
            KPT_CUDA(cudaMalloc(&f->fixed_centers[d], fixed.centers.size() * sizeof(long long)));
            KPT_CUDA(cudaMemcpy(f->fixed_centers[d], fixed.centers.data(),
                                fixed.centers.size() * sizeof(long long), cudaMemcpyHostToDevice));
            KPT_CUDA(cudaMalloc(&f->fixed_spacing[d], fixed.inv_spacing.size() * sizeof(float)));
            KPT_CUDA(cudaMemcpy(f->fixed_spacing[d], fixed.inv_spacing.data(),
                                fixed.inv_spacing.size() * sizeof(float), cudaMemcpyHostToDevice));
            KPT_CUDA(cudaMalloc(&f->fixed_buckets[d], fixed.buckets.size() * sizeof(int)));
            KPT_CUDA(cudaMemcpy(f->fixed_buckets[d], fixed.buckets.data(),
                                fixed.buckets.size() * sizeof(int), cudaMemcpyHostToDevice));
            f->fixed[d].centers = f->fixed_centers[d];
            f->fixed[d].inv_spacing = f->fixed_spacing[d];
            f->fixed[d].buckets = f->fixed_buckets[d];
            KPT_CUDA(cudaMalloc(&f->centers[d], centers.size() * sizeof(double)));
            KPT_CUDA(cudaMemcpy(f->centers[d], centers.data(), centers.size() * sizeof(double),
                                cudaMemcpyHostToDevice));
            KPT_CUDA(cudaMalloc(&f->buckets[d], buckets.size() * sizeof(int)));
            KPT_CUDA(cudaMemcpy(f->buckets[d], buckets.data(), buckets.size() * sizeof(int),
                                cudaMemcpyHostToDevice));
            f->grid.axis[d].centers = f->centers[d];
            f->grid.axis[d].buckets = f->buckets[d];
        }
    }
    const size_t elem = precision == KPT_PRECISION_F64 ? sizeof(double) : sizeof(float);
    KPT_CUDA(cudaMalloc(&f->table, f->points * f->stride * elem));
    double* staging = nullptr;
    cudaError_t err = cudaSuccess;
    if (!device_readable) {
        KPT_CUDA(cudaMalloc(&staging, 6 * cells * sizeof(double)));
        err = cudaMemcpyAsync(staging, b_cells, 3 * cells * sizeof(double),
                              cudaMemcpyHostToDevice, ctx->stream);
        if (err == cudaSuccess) {
            err = cudaMemcpyAsync(staging + 3 * cells, v_cells, 3 * cells * sizeof(double),
                                  cudaMemcpyHostToDevice, ctx->stream);
        }
    }
    if (err == cudaSuccess) {
        kpt::TableLaunch launch{};
        launch.grid = f->grid;
        launch.b_cells = device_readable ? b_device : staging;
        launch.v_cells = device_readable ? v_device : staging + 3 * cells;
        launch.table = f->table;
        launch.focused = table_kind == KPT_TABLE_FOCUSED21;
        launch.precision = precision;
        err = kpt::launch_build_table(launch, ctx->stream);
    }
    if (err == cudaSuccess) {
        err = cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(staging);
    if (err != cudaSuccess) {
        return set_error(KPT_ERROR_CUDA,
                         std::string("kpt_field_create: ") + cudaGetErrorString(err));
    }
    *out = f.release();
    return KPT_OK;
}

}  // namespace

extern "C" {

// Compact field reader: layout and checks of AthenaFieldReader.hpp:290-360
// (non-uniform edges accepted as an extension).
int kpt_field_data_read(const kpt_context* ctx, const char* path, kpt_field_data** out) {
    KPT_REQUIRE(ctx != nullptr && path != nullptr && out != nullptr,
                "kpt_field_data_read: NULL argument");
    *out = nullptr;
    // the calling thread may be a helper thread: bind it to the context's device
    KPT_CUDA(cudaSetDevice(ctx->device));
    std::ifstream stream(path, std::ios::binary);
    if (!stream) {
        return set_error(KPT_ERROR_IO, "AthenaFieldReader: failed to open Athena binary file.");
    }
    int32_t dims[2] = {0, 0};
    stream.read(reinterpret_cast<char*>(dims), sizeof(dims));
    if (!stream) {
        return set_error(KPT_ERROR_FORMAT, "AthenaFieldReader: failed to read nx.");
    }
    const int nx = dims[0], ny = dims[1];
    if (nx <= 0 || ny <= 0) {
        return set_error(KPT_ERROR_FORMAT,
                         "AthenaFieldReader: Athena binary dimensions must be positive.");
    }
    std::unique_ptr<kpt_field_data, int (*)(kpt_field_data*)> d(new kpt_field_data(),
                                                                kpt_field_data_free);
    d->nx = nx;
    d->ny = ny;
    const size_t cells = static_cast<size_t>(nx) * static_cast<size_t>(ny);
    d->x_edges.resize(static_cast<size_t>(nx) + 1);
    d->y_edges.resize(static_cast<size_t>(ny) + 1);
    // cell data in page-locked memory (portable across devices) so the
    // upload runs at full host-device bandwidth
    KPT_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&d->cells), 6 * cells * sizeof(double),
                           cudaHostAllocPortable | cudaHostAllocMapped));
    auto read = [&](double* dst, size_t n, const char* name) -> int {
        stream.read(reinterpret_cast<char*>(dst), static_cast<std::streamsize>(n * sizeof(double)));
        if (!stream) {
            return set_error(KPT_ERROR_FORMAT,
                             std::string("AthenaFieldReader: failed to read ") + name + ".");
        }
        return KPT_OK;
    };
    if (int rc = read(d->x_edges.data(), d->x_edges.size(), "x_edges")) return rc;
    if (int rc = read(d->y_edges.data(), d->y_edges.size(), "y_edges")) return rc;
    const char* names[6] = {"Bx", "By", "Bz", "Vx", "Vy", "Vz"};
    for (int c = 0; c < 6; ++c) {
        if (int rc = read(d->cells + c * cells, cells, names[c])) return rc;
    }
    if (stream.peek() != std::char_traits<char>::eof()) {
        return set_error(KPT_ERROR_FORMAT,
                         "AthenaFieldReader: Athena binary file has trailing payload.");
    }
    for (size_t k = 0; k < 6 * cells; ++k) {
        if (!std::isfinite(d->cells[k])) {
            return set_error(KPT_ERROR_FORMAT, "AthenaFieldReader: non-finite field value.");
        }
    }
    *out = d.release();
    return KPT_OK;
}

int kpt_field_data_free(kpt_field_data* data) {
    if (data == nullptr) return KPT_OK;
    if (data->cells != nullptr) cudaFreeHost(data->cells);
    delete data;
    return KPT_OK;
}

int kpt_field_data_shape(const kpt_field_data* data, int* nx, int* ny) {
    KPT_REQUIRE(data != nullptr, "kpt_field_data_shape: NULL handle");
    if (nx) *nx = data->nx;
    if (ny) *ny = data->ny;
    return KPT_OK;
}

int kpt_field_create_from_data(kpt_context* ctx, const kpt_field_data* data, int table_kind,
                               int precision, kpt_field** out) {
    KPT_REQUIRE(ctx && data && out, "kpt_field_create_from_data: NULL argument");
    const size_t cells = static_cast<size_t>(data->nx) * static_cast<size_t>(data->ny);
    if (int rc = activate(ctx)) return rc;
    // the device's address of the mapped page-locked cells
    void* mapped = nullptr;
    KPT_CUDA(cudaHostGetDevicePointer(&mapped, data->cells, 0));
    const double* cells_dev = static_cast<const double*>(mapped);
    return field_create(ctx, data->nx, data->ny, data->x_edges.data(), data->y_edges.data(),
                        data->cells, data->cells + 3 * cells, table_kind, precision, cells_dev,
                        cells_dev + 3 * cells, out);
}

int kpt_field_load(kpt_context* ctx, const char* path, int table_kind, int precision,
                   kpt_field** out) {
    KPT_REQUIRE(ctx != nullptr, "kpt_field_load: ctx is NULL");
    kpt_field_data* data = nullptr;
    if (int rc = kpt_field_data_read(ctx, path, &data)) return rc;
    const int rc = kpt_field_create_from_data(ctx, data, table_kind, precision, out);
    kpt_field_data_free(data);
    return rc;
}

int kpt_field_destroy(kpt_field* field) {
    if (field == nullptr) {
        return KPT_OK;
    }
    // cudaFree waits for outstanding work on the memory; the context (which
    // may already be gone) is not touched.
    cudaSetDevice(field->device);
    cudaFree(field->table);
    for (int d = 0; d < 2; ++d) {
        cudaFree(field->centers[d]);
        cudaFree(field->buckets[d]);
        cudaFree(field->fixed_centers[d]);
        cudaFree(field->fixed_spacing[d]);
        cudaFree(field->fixed_buckets[d]);
    }
    delete field;
    return KPT_OK;
}

int kpt_field_shape(const kpt_field* field, int* nx, int* ny, uint64_t* points,
                    int* components) {
    KPT_REQUIRE(field != nullptr, "kpt_field_shape: field is NULL");
    if (nx) *nx = field->nx;
    if (ny) *ny = field->ny;
    if (points) *points = field->points;
    if (components) *components = field->kind == KPT_TABLE_FOCUSED21 ? 21 : 16;
    return KPT_OK;
}

int kpt_field_download_table(const kpt_field* field, double* out, uint64_t out_len) {
    KPT_REQUIRE(field != nullptr && out != nullptr, "kpt_field_download_table: NULL");
    const int ncomp = field->kind == KPT_TABLE_FOCUSED21 ? 21 : 16;
    KPT_REQUIRE(out_len >= field->points * ncomp, "kpt_field_download_table: out too small");
    if (int rc = activate(field->ctx)) return rc;
    const size_t n = field->points * field->stride;
    if (field->precision == KPT_PRECISION_F64) {
        std::vector<double> host(n);
        KPT_CUDA(cudaMemcpyAsync(host.data(), field->table, n * sizeof(double),
                                 cudaMemcpyDeviceToHost, field->ctx->stream));
        KPT_CUDA(cudaStreamSynchronize(field->ctx->stream));
        for (uint64_t p = 0; p < field->points; ++p) {
            for (int c = 0; c < ncomp; ++c) {
                out[p * ncomp + c] = host[p * field->stride + c];
            }
        }
    } else {
        std::vector<float> host(n);
        KPT_CUDA(cudaMemcpyAsync(host.data(), field->table, n * sizeof(float),
                                 cudaMemcpyDeviceToHost, field->ctx->stream));
        KPT_CUDA(cudaStreamSynchronize(field->ctx->stream));
        for (uint64_t p = 0; p < field->points; ++p) {
            for (int c = 0; c < ncomp; ++c) {
                out[p * ncomp + c] =
                    static_cast<double>(host[kpt::table_f32_offset(
                        field->kind == KPT_TABLE_FOCUSED21, field->points, p, c)]);
            }
        }
    }
    return KPT_OK;
}

int kpt_particles_create(kpt_context* ctx, uint64_t capacity, kpt_particles** out) {
    KPT_REQUIRE(ctx != nullptr && out != nullptr, "kpt_particles_create: NULL handle");
    *out = nullptr;
    KPT_REQUIRE(capacity > 0,
                "Reconnection2DSettings: particle counts and capacity must be positive.");
    KPT_REQUIRE(capacity < (1ull << 32), "kpt_particles_create: capacity must be < 2^32");
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_particles> parts(new kpt_particles());
    parts->ctx = ctx;
    parts->device = ctx->device;
    parts->capacity = capacity;
    // One allocation: 7 double arrays then 2 int32 arrays, each 256-byte aligned.
    auto round_up = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
    const size_t dbytes = round_up(capacity * sizeof(double));
    const size_t ibytes = round_up(capacity * sizeof(int32_t));
    KPT_CUDA(cudaMalloc(&parts->block, 7 * dbytes + 2 * ibytes));
    char* base = static_cast<char*>(parts->block);
    double** dptrs[7] = {&parts->arrays.x, &parts->arrays.y, &parts->arrays.p,
                         &parts->arrays.t, &parts->arrays.step_dt, &parts->arrays.weight,
                         &parts->arrays.mu};
    for (int k = 0; k < 7; ++k) {
        *dptrs[k] = reinterpret_cast<double*>(base + k * dbytes);
    }
    parts->arrays.status = reinterpret_cast<int32_t*>(base + 7 * dbytes);
    parts->arrays.split_level = reinterpret_cast<int32_t*>(base + 7 * dbytes + ibytes);
    // Storage starts zeroed with status 2 (src/main.cpp:326-331).
    KPT_CUDA(cudaMemsetAsync(parts->block, 0, 7 * dbytes + 2 * ibytes, ctx->stream));
    std::vector<int32_t> twos(capacity, 2);
    KPT_CUDA(cudaMemcpyAsync(parts->arrays.status, twos.data(), capacity * sizeof(int32_t),
                             cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = parts.release();
    return KPT_OK;
}

int kpt_particles_wrap(kpt_context* ctx, uint64_t capacity, uint64_t count,
                       const kpt_particle_arrays* arrays, kpt_particles** out) {
    KPT_REQUIRE(ctx != nullptr && arrays != nullptr && out != nullptr,
                "kpt_particles_wrap: NULL argument");
    *out = nullptr;
    KPT_REQUIRE(capacity > 0 && capacity < (1ull << 32) && count <= capacity,
                "kpt_particles_wrap: need 0 < capacity < 2^32 and count <= capacity");
    const void* ptrs[9] = {arrays->x, arrays->y, arrays->p, arrays->t, arrays->step_dt,
                           arrays->weight, arrays->mu, arrays->status, arrays->split_level};
    for (const void* ptr : ptrs) {
        KPT_REQUIRE(ptr != nullptr, "kpt_particles_wrap: NULL array");
        cudaPointerAttributes attr{};
        KPT_CUDA(cudaPointerGetAttributes(&attr, ptr));
        KPT_REQUIRE(attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged,
                    "kpt_particles_wrap: arrays must be device (or managed) memory");
    }
    std::unique_ptr<kpt_particles> parts(new kpt_particles());
    parts->ctx = ctx;
    parts->device = ctx->device;
    parts->capacity = capacity;
    parts->count = count;
    parts->arrays.x = arrays->x;
    parts->arrays.y = arrays->y;
    parts->arrays.p = arrays->p;
    parts->arrays.t = arrays->t;
    parts->arrays.step_dt = arrays->step_dt;
    parts->arrays.weight = arrays->weight;
    parts->arrays.mu = arrays->mu;
    parts->arrays.status = arrays->status;
    parts->arrays.split_level = arrays->split_level;
    *out = parts.release();
    return KPT_OK;
}

int kpt_particles_destroy(kpt_particles* parts) {
    if (parts == nullptr) {
        return KPT_OK;
    }
    cudaSetDevice(parts->device);
    cudaFree(parts->block);
    parts->order.release();
    parts->keys.release();
    parts->tile_counts.release();
    delete parts;
    return KPT_OK;
}

int kpt_particles_count(const kpt_particles* parts, uint64_t* count, uint64_t* capacity) {
    KPT_REQUIRE(parts != nullptr, "kpt_particles_count: NULL handle");
    if (count) *count = parts->count;
    if (capacity) *capacity = parts->capacity;
    return KPT_OK;
}

int kpt_particles_set_count(kpt_particles* parts, uint64_t count) {
    KPT_REQUIRE(parts != nullptr, "kpt_particles_set_count: NULL handle");
    KPT_REQUIRE(count <= parts->capacity, "kpt_particles_set_count: count exceeds capacity");
    parts->count = count;
    parts->order_valid = false;
    return KPT_OK;
}

int kpt_particles_upload(kpt_particles* parts, uint64_t count, const double* x,
                         const double* y, const double* p, const double* t,
                         const double* step_dt, const double* weight, const double* mu,
                         const int32_t* status, const int32_t* split_level) {
    KPT_REQUIRE(parts != nullptr, "kpt_particles_upload: NULL handle");
    KPT_REQUIRE(count <= parts->capacity, "kpt_particles_upload: count exceeds capacity");
    if (int rc = activate(parts->ctx)) return rc;
    cudaStream_t s = parts->ctx->stream;
    const kpt::ParticleArrays& a = parts->arrays;
    const void* src[9] = {x, y, p, t, step_dt, weight, mu, status, split_level};
    void* dst[9] = {a.x, a.y, a.p, a.t, a.step_dt, a.weight, a.mu, a.status, a.split_level};
    for (int k = 0; k < 9; ++k) {
        if (src[k] != nullptr && count > 0) {
            const size_t elem = k < 7 ? sizeof(double) : sizeof(int32_t);
            KPT_CUDA(cudaMemcpyAsync(dst[k], src[k], count * elem, cudaMemcpyHostToDevice, s));
        }
    }
    KPT_CUDA(cudaStreamSynchronize(s));
    parts->count = count;
    parts->order_valid = false;
    return KPT_OK;
}

int kpt_particles_download(const kpt_particles* parts, uint64_t count, double* x, double* y,
                           double* p, double* t, double* step_dt, double* weight, double* mu,
                           int32_t* status, int32_t* split_level) {
    KPT_REQUIRE(parts != nullptr, "kpt_particles_download: NULL handle");
    KPT_REQUIRE(count <= parts->capacity, "kpt_particles_download: count exceeds capacity");
    if (int rc = activate(parts->ctx)) return rc;
    cudaStream_t s = parts->ctx->stream;
    const kpt::ParticleArrays& a = parts->arrays;
    void* dst[9] = {x, y, p, t, step_dt, weight, mu, status, split_level};
    const void* src[9] = {a.x, a.y, a.p, a.t, a.step_dt, a.weight, a.mu, a.status,
                          a.split_level};
    for (int k = 0; k < 9; ++k) {
        if (dst[k] != nullptr && count > 0) {
            const size_t elem = k < 7 ? sizeof(double) : sizeof(int32_t);
            KPT_CUDA(cudaMemcpyAsync(dst[k], src[k], count * elem, cudaMemcpyDeviceToHost, s));
        }
    }
    KPT_CUDA(cudaStreamSynchronize(s));
    return KPT_OK;
}

int kpt_particles_device_arrays(const kpt_particles* parts, kpt_particle_arrays* out) {
    KPT_REQUIRE(parts != nullptr && out != nullptr, "kpt_particles_device_arrays: NULL");
    const kpt::ParticleArrays& a = parts->arrays;
    out->x = a.x;
    out->y = a.y;
    out->p = a.p;
    out->t = a.t;
    out->step_dt = a.step_dt;
    out->weight = a.weight;
    out->mu = a.mu;
    out->status = a.status;
    out->split_level = a.split_level;
    return KPT_OK;
}

int kpt_inject_uniform(kpt_context* ctx, kpt_particles* parts, const kpt_field* grid,
                       const kpt_settings* settings, uint64_t requested, uint32_t frame,
                       uint64_t seed, double band_lo, double band_hi, uint64_t* injected) {
    KPT_REQUIRE(ctx && parts && grid, "kpt_inject_uniform: NULL handle");
    if (int rc = validate_settings(settings)) return rc;
    if (injected) *injected = 0;
    if (parts->count >= parts->capacity) {
        return KPT_OK;
    }
    if (int rc = activate(ctx)) return rc;
    const uint64_t n = std::min(requested, parts->capacity - parts->count);
    const kpt::DeviceSettings d = device_settings(settings, grid->grid);
    kpt::InjectLaunch launch{};
    launch.parts = parts->arrays;
    launch.first = parts->count;
    launch.n = n;
    launch.x_lower = d.x_lower;
    launch.x_upper = d.x_upper;
    launch.y_lower = band_lo < band_hi ? band_lo : d.y_lower;
    launch.y_upper = band_lo < band_hi ? band_hi : d.y_upper;
    launch.p0 = settings->p0;
    launch.interval_start = static_cast<double>(frame) * settings->mhd_dt;
    launch.mhd_dt = settings->mhd_dt;
    launch.dt_min = d.dt_min;
    launch.mu_max = settings->mu_max;
    launch.frame = frame;
    launch.seed = seed;
    KPT_CUDA(kpt::launch_inject(launch, ctx->stream));
    parts->count += n;
    if (n > 0) parts->order_valid = false;
    if (injected) *injected = n;
    return KPT_OK;
}

}  // extern "C"

namespace {

// The push launch of one interval of one particle store (shared by
// kpt_push_interval and the batched runs).
void fill_push_launch(const kpt_context* ctx, const kpt_particles* parts, const kpt_field* lower,
                      const kpt_field* upper, const kpt_settings* settings, uint32_t frame,
                      uint64_t seed, kpt::PushCounters* counters, kpt::PushLaunch& launch) {
    launch = kpt::PushLaunch{};
    launch.grid = lower->grid;
    launch.lower = lower->table;
    launch.upper = upper->table;
    launch.parts = parts->arrays;
    launch.count = parts->count;
    launch.settings = device_settings(settings, lower->grid);
    launch.interval_start = static_cast<double>(frame) * settings->mhd_dt;
    launch.interval_end = launch.interval_start + settings->mhd_dt;
    launch.frame = frame;
    launch.seed = seed;
    launch.counters = counters;
    launch.fixed.axis[0] = lower->fixed[0];
    launch.fixed.axis[1] = lower->fixed[1];
    launch.fixed.dt_min = static_cast<float>(launch.settings.dt_min);
    launch.fixed.dt_max = static_cast<float>(launch.settings.dt_max);
    launch.fixed.tau_per_time = static_cast<float>(4611686018427387904.0 / settings->mhd_dt);
    launch.fixed.time_per_tau_2_32 = static_cast<float>(settings->mhd_dt / 1073741824.0);
    const double pfloor = 0.25 * settings->p0;
    launch.fixed.pfloor_hi = static_cast<float>(pfloor);
    launch.fixed.pfloor_lo =
        static_cast<float>(pfloor - static_cast<double>(launch.fixed.pfloor_hi));
    launch.order = parts->order_valid ? parts->order.as<uint32_t>() : nullptr;
    launch.precision = lower->precision;
    launch.focused = settings->focused != 0;
    launch.schedule = ctx->push_schedule;
    launch.fp64_contracted = ctx->fp64_arithmetic == KPT_FP64_CONTRACTED ? 1 : 0;
    launch.sm_count = ctx->sm_count;
    launch.blocks_per_sm = ctx->push_blocks_per_sm;
    launch.surrogate = nullptr;
}

// The cell records a mixed push samples (*out = nullptr: the point-major
// tables), built on the context's stream when the table pair differs from
// the one they hold.  Should the records not fit in device memory the push
// samples the point tables, which gives the same values.
int push_records(kpt_context* ctx, const kpt_particles* parts, const kpt_field* lower,
                 const kpt_field* upper, const float** out) {
    *out = nullptr;
    if (lower->precision != KPT_PRECISION_MIXED || ctx->push_schedule != kpt::kScheduleRefill ||
        parts->count == 0 || ctx->records_mode == KPT_RECORDS_OFF ||
        lower->points >= (1ull << 32)) {
        return KPT_OK;
    }
    if (ctx->records_mode == KPT_RECORDS_AUTO && parts->count * 4 < lower->points) {
        return KPT_OK;
    }
    if (ctx->records_lower != lower->serial || ctx->records_upper != upper->serial ||
        ctx->records.ptr == nullptr) {
        const bool focused = lower->kind == KPT_TABLE_FOCUSED21;
        const size_t bytes = lower->points * kpt::record_floats(focused) * sizeof(float);
        ctx->records_lower = ctx->records_upper = 0;
        if (ctx->records.reserve(bytes) != cudaSuccess) {
            cudaGetLastError();  // out of memory: sample the point tables
            ctx->records.release();
            return KPT_OK;
        }
        kpt::RecordLaunch rl{};
        rl.lower = static_cast<const float*>(lower->table);
        rl.upper = static_cast<const float*>(upper->table);
        rl.records = ctx->records.as<float>();
        rl.points = lower->points;
        rl.ex = lower->nx + 4;
        rl.ey = lower->ny + 4;
        rl.focused = focused ? 1 : 0;
        KPT_CUDA(kpt::launch_build_records(rl, ctx->stream));
        if (ctx->records_ready == nullptr) {
            KPT_CUDA(cudaEventCreateWithFlags(&ctx->records_ready, cudaEventDisableTiming));
        }
        KPT_CUDA(cudaEventRecord(ctx->records_ready, ctx->stream));
        ctx->records_stream = ctx->stream;
        ctx->records_lower = lower->serial;
        ctx->records_upper = upper->serial;
    } else if (ctx->stream != ctx->records_stream) {
        // built on another stream (the caller switched streams): order this
        // push after the build
        KPT_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->records_ready, 0));
    }
    *out = ctx->records.as<float>();
    return KPT_OK;
}

}  // namespace

extern "C" {

int kpt_push_interval(kpt_context* ctx, kpt_particles* parts, const kpt_field* lower,
                      const kpt_field* upper, const kpt_settings* settings, uint32_t frame,
                      uint64_t seed, kpt_push_stats* stats) {
    KPT_REQUIRE(ctx && parts && lower && upper, "kpt_push_interval: NULL handle");
    if (int rc = validate_settings(settings)) return rc;
    KPT_REQUIRE(lower->kind == upper->kind && lower->precision == upper->precision &&
                    lower->nx == upper->nx && lower->ny == upper->ny,
                "kpt_push_interval: lower and upper tables differ in kind, precision or shape");
    KPT_REQUIRE((lower->kind == KPT_TABLE_FOCUSED21) == (settings->focused != 0),
                "kpt_push_interval: table kind does not match settings.focused");
    if (int rc = activate(ctx)) return rc;
    kpt::PushLaunch launch{};
    fill_push_launch(ctx, parts, lower, upper, settings, frame, seed,
                     ctx->counters.as<kpt::PushCounters>(), launch);
    launch.surrogate = nullptr;
    kpt::SurrogateDevice served{};
    if (settings->closure == KPT_CLOSURE_SURROGATE) {
        const kpt_surrogate* sg = ctx->surrogate;
        KPT_REQUIRE(sg != nullptr,
                    "kpt_push_interval: closure SURROGATE needs kpt_context_set_surrogate");
        KPT_REQUIRE(settings->focused != 0,
                    "kpt_push_interval: the surrogate closure runs in the focused push");
        const kpt::SurrogateBox& box = sg->box;
        KPT_REQUIRE(box.p0 == settings->p0 && box.particle_v0 == settings->particle_v0 &&
                        box.kpara0 == settings->kpara0 &&
                        box.gamma_turb == settings->gamma_turb &&
                        box.qlt_omega0 == settings->qlt_omega0 &&
                        box.qlt_lc == settings->qlt_lc && box.qlt_h0 == settings->qlt_h0 &&
                        box.magnetic_dependency == settings->magnetic_dependency &&
                        box.momentum_dependency == settings->momentum_dependency,
                    "kpt_push_interval: settings differ from those the surrogate was trained with");
        served.block = sg->d_block;
        served.tc_block = sg->d_tc_block;
        // the FP64 push serves the network on the warp-collective engine
        served.engine = lower->precision == KPT_PRECISION_F64 ? kpt::kEngineMmaSync : sg->engine;
        served.box = box;
        const double f3 = std::log(settings->qlt_sigma2);
        const double f4 = settings->qlt_spectral_index;
        served.constants_in_box = f3 >= box.in_lo[3] && f3 <= box.in_hi[3] && f4 >= box.in_lo[4] &&
                                  f4 <= box.in_hi[4];
        served.f3 = static_cast<float>(f3) * box.in_scale[3] + box.in_offset[3];
        served.f4 = static_cast<float>(f4) * box.in_scale[4] + box.in_offset[4];
        served.judge_period = KPT_JUDGE_PERIOD;
        served.judge = ctx->judge.as<unsigned long long>();  // zeroed by set_surrogate
        launch.surrogate = &served;
    }
    if (int rc = push_records(ctx, parts, lower, upper, &launch.records)) return rc;
    KPT_CUDA(cudaMemsetAsync(launch.counters, 0, sizeof(kpt::PushCounters), ctx->stream));
    if (parts->count > 0) {
        KPT_CUDA(kpt::launch_push_interval(launch, ctx->stream));
    }
    // The tcgen05 engine's completion waits are bounded; a block that gives
    // up stops early, so its particles are not stored back.  Its counters are
    // therefore always read back and checked, with or without `stats`.
    const bool bounded_waits =
        launch.surrogate != nullptr && served.engine == KPT_ENGINE_TCGEN05 && parts->count > 0;
    if (stats != nullptr || bounded_waits) {
        kpt::PushCounters host{};
        KPT_CUDA(cudaMemcpyAsync(&host, launch.counters, sizeof(host), cudaMemcpyDeviceToHost,
                                 ctx->stream));
        KPT_CUDA(cudaStreamSynchronize(ctx->stream));
        if (stats != nullptr) {
            stats->particle_steps = host.particle_steps;
            stats->pushed = host.pushed;
            stats->failed = host.failed;
            stats->max_steps = host.max_steps;
            stats->pad = 0;
        }
        if (host.teardown_incomplete != 0) {
            return set_error(KPT_ERROR_CUDA,
                             "kpt_push_interval: a tensor-core completion wait timed out and "
                             "tensor memory was freed with MMAs in flight (results of this "
                             "push are invalid for every particle)");
        }
        if (host.network_timeouts != 0) {
            return set_error(KPT_ERROR_CUDA,
                             "kpt_push_interval: a tensor-core completion wait timed out "
                             "(results of this push are invalid)");
        }
    }
    return KPT_OK;
}

int kpt_split(kpt_context* ctx, kpt_particles* parts, const kpt_settings* settings,
              uint64_t* split, uint64_t* skipped) {
    KPT_REQUIRE(ctx && parts, "kpt_split: NULL handle");
    if (int rc = validate_settings(settings)) return rc;
    if (split) *split = 0;
    if (skipped) *skipped = 0;
    if (parts->count >= parts->capacity || settings->split_particles == 0) {
        return KPT_OK;
    }
    if (int rc = activate(ctx)) return rc;
    // Per-level thresholds pmin_split * ratio^level (the project pow) up to the first
    // level whose threshold exceeds pmax; later levels can never split.
    const double pmin_split = settings->pmin_split_over_p0 * settings->p0;
    if (ctx->split_level_count == 0 || ctx->split_key[0] != pmin_split ||
        ctx->split_key[1] != settings->split_ratio || ctx->split_key[2] != settings->pmax) {
        std::vector<double> thresholds;
        for (int level = 0; level < 65536; ++level) {
            const double thr = pmin_split * kpt_pow(settings->split_ratio,
                                                     static_cast<double>(level));
            thresholds.push_back(thr);
            if (!(thr < settings->pmax)) {
                break;
            }
        }
        if (thresholds.back() < settings->pmax) {
            return set_error(KPT_ERROR_INVALID_ARGUMENT,
                             "kpt_split: split ratio too close to 1 for the level table");
        }
        const int levels = static_cast<int>(thresholds.size());
        std::vector<double> table(2 * static_cast<size_t>(levels));
        for (int level = 0; level < levels; ++level) {
            table[level] = thresholds[level];
            table[levels + level] = kpt_pow(0.5, static_cast<double>(level + 1));
        }
        KPT_CUDA(ctx->split_levels.reserve(table.size() * sizeof(double)));
        KPT_CUDA(cudaMemcpyAsync(ctx->split_levels.ptr, table.data(),
                                 table.size() * sizeof(double), cudaMemcpyHostToDevice,
                                 ctx->stream));
        ctx->split_level_count = levels;
        ctx->split_key[0] = pmin_split;
        ctx->split_key[1] = settings->split_ratio;
        ctx->split_key[2] = settings->pmax;
    }
    const size_t nblocks = kpt::split_scratch_blocks(parts->count);
    KPT_CUDA(ctx->split_counts.reserve(std::max<size_t>(nblocks, 1) * sizeof(unsigned int)));
    KPT_CUDA(ctx->split_offsets.reserve(std::max<size_t>(nblocks, 1) *
                                        sizeof(unsigned long long)));
    KPT_CUDA(ctx->split_totals.reserve(2 * sizeof(unsigned long long)));
    kpt::SplitLaunch launch{};
    launch.parts = parts->arrays;
    launch.count = parts->count;
    launch.capacity = parts->capacity;
    launch.thresholds = ctx->split_levels.as<double>();
    launch.weights = ctx->split_levels.as<double>() + ctx->split_level_count;
    launch.level_count = ctx->split_level_count;
    launch.pmax = settings->pmax;
    launch.block_counts = ctx->split_counts.as<unsigned int>();
    launch.block_offsets = ctx->split_offsets.as<unsigned long long>();
    launch.totals = ctx->split_totals.as<unsigned long long>();
    KPT_CUDA(kpt::launch_split(launch, ctx->stream));
    unsigned long long wanted = 0;
    KPT_CUDA(cudaMemcpyAsync(&wanted, launch.totals, sizeof(wanted), cudaMemcpyDeviceToHost,
                             ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint64_t room = parts->capacity - parts->count;
    const uint64_t written = std::min<uint64_t>(wanted, room);
    parts->count += written;
    if (written > 0) parts->order_valid = false;
    if (split) *split = written;
    if (skipped) *skipped = wanted - written;
    return KPT_OK;
}

int kpt_histogram(kpt_context* ctx, const kpt_particles* parts, double pmin, double pmax,
                  int nbins, double* bins) {
    KPT_REQUIRE(ctx && parts && bins, "kpt_histogram: NULL argument");
    KPT_REQUIRE(nbins > 0 && nbins <= 4096, "kpt_histogram: nbins must be in [1, 4096]");
    KPT_REQUIRE(std::isfinite(pmin) && std::isfinite(pmax) && pmin > 0.0 && pmax > pmin,
                "kpt_histogram: need 0 < pmin < pmax");
    if (int rc = activate(ctx)) return rc;
    const uint64_t count = parts->count;
    KPT_CUDA(ctx->hist_bins.reserve(sizeof(double) * nbins));
    KPT_CUDA(ctx->hist_edge_count.reserve(sizeof(unsigned long long)));
    KPT_CUDA(ctx->hist_edge_index.reserve(sizeof(unsigned int) * std::max<uint64_t>(count, 1)));
    const double log_pmin = std::log(pmin);
    const double inv_dlogp = static_cast<double>(nbins) / (std::log(pmax) - log_pmin);
    kpt::HistogramLaunch launch{};
    launch.p = parts->arrays.p;
    launch.weight = parts->arrays.weight;
    launch.status = parts->arrays.status;
    launch.count = count;
    launch.pmin = pmin;
    launch.pmax = pmax;
    launch.log_pmin = log_pmin;
    launch.inv_dlogp = inv_dlogp;
    launch.nbins = nbins;
    launch.bins = ctx->hist_bins.as<double>();
    launch.edge_count = ctx->hist_edge_count.as<unsigned long long>();
    launch.edge_index = ctx->hist_edge_index.as<unsigned int>();
    KPT_CUDA(kpt::launch_histogram(launch, ctx->stream));
    unsigned long long edges = 0;
    KPT_CUDA(cudaMemcpyAsync(bins, launch.bins, sizeof(double) * nbins, cudaMemcpyDeviceToHost,
                             ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(&edges, launch.edge_count, sizeof(edges), cudaMemcpyDeviceToHost,
                             ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (edges > 0) {
        // Host re-binning of particles whose bin coordinate sits within 1e-7
        // of an edge, with the host log the reference uses.
        std::vector<unsigned int> index(edges);
        KPT_CUDA(cudaMemcpy(index.data(), launch.edge_index, edges * sizeof(unsigned int),
                            cudaMemcpyDeviceToHost));
        for (unsigned long long k = 0; k < edges; ++k) {
            double p = 0.0, w = 0.0;
            KPT_CUDA(cudaMemcpy(&p, parts->arrays.p + index[k], sizeof(double),
                                cudaMemcpyDeviceToHost));
            KPT_CUDA(cudaMemcpy(&w, parts->arrays.weight + index[k], sizeof(double),
                                cudaMemcpyDeviceToHost));
            int bin = static_cast<int>((std::log(p) - log_pmin) * inv_dlogp);
            bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
            bins[bin] += w;
        }
    }
    return KPT_OK;
}

int kpt_summarize(kpt_context* ctx, const kpt_particles* parts, kpt_summary* out) {
    KPT_REQUIRE(ctx && parts && out, "kpt_summarize: NULL argument");
    std::memset(out, 0, sizeof(*out));
    out->stored = parts->count;
    if (parts->count == 0) {
        return KPT_OK;
    }
    if (int rc = activate(ctx)) return rc;
    const int nblocks = kpt::summary_blocks(parts->count);
    KPT_CUDA(ctx->summary_partials.reserve(sizeof(kpt::SummaryPartial) * nblocks));
    KPT_CUDA(ctx->summary_result.reserve(sizeof(kpt::SummaryPartial)));
    kpt::SummaryLaunch launch{};
    launch.p = parts->arrays.p;
    launch.dt = parts->arrays.step_dt;
    launch.weight = parts->arrays.weight;
    launch.status = parts->arrays.status;
    launch.level = parts->arrays.split_level;
    launch.count = parts->count;
    launch.partials = ctx->summary_partials.as<kpt::SummaryPartial>();
    launch.result = ctx->summary_result.as<kpt::SummaryPartial>();
    KPT_CUDA(kpt::launch_summary(launch, ctx->stream));
    kpt::SummaryPartial r{};
    KPT_CUDA(cudaMemcpyAsync(&r, launch.result, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    out->active = r.active;
    out->inactive = r.inactive;
    out->weight_sum = r.weight_sum;
    out->max_split_level = r.max_level;
    if (r.active > 0) {
        out->p_min = r.p_min;
        out->p_max = r.p_max;
        out->dt_min = r.dt_min;
        out->dt_max = r.dt_max;
        out->p_avg = r.p_sum / static_cast<double>(r.active);
        out->dt_avg = r.dt_sum / static_cast<double>(r.active);
    }
    return KPT_OK;
}

// ---------------------------------------------------------------- surrogate

namespace {

// float -> bfloat16, round to nearest even (upper 16 bits of the float).
uint32_t to_bf16(float f) {
    uint32_t bits;
    std::memcpy(&bits, &f, sizeof(bits));
    const uint32_t rounding = 0x7fffu + ((bits >> 16) & 1u);
    return (bits + rounding) >> 16;
}

// float -> IEEE binary16, round to nearest even, subnormals kept, overflow to
// infinity (finite weights only reach it beyond 65504).
uint32_t to_fp16(float f) {
    uint32_t bits;
    std::memcpy(&bits, &f, sizeof(bits));
    const uint32_t sign = (bits >> 16) & 0x8000u;
    const uint32_t abs = bits & 0x7fffffffu;
    if (abs >= 0x7f800000u) {  // inf / nan
        return sign | 0x7c00u | (abs > 0x7f800000u ? 0x200u : 0u);
    }
    const int exp = static_cast<int>(abs >> 23) - 127;
    if (exp > 15) return sign | 0x7c00u;
    uint32_t mant = (abs & 0x7fffffu) | 0x800000u;  // 24-bit significand
    int shift;                                        // bits dropped from it
    uint32_t base;
    if (exp >= -14) {
        shift = 13;
        base = static_cast<uint32_t>(exp + 15) << 10;
        mant &= 0x7fffffu;  // implicit bit carried by the exponent field
    } else {
        if (exp < -25) return sign;  // rounds to zero
        shift = 13 + (-14 - exp);    // subnormal: value = mant * 2^(exp-23)
        base = 0u;
    }
    const uint32_t kept = mant >> shift;
    const uint32_t rest = mant & ((1u << shift) - 1u);
    const uint32_t half = 1u << (shift - 1);
    uint32_t out = base + kept;  // a mantissa carry rolls into the exponent
    if (rest > half || (rest == half && (kept & 1u))) ++out;
    return sign | out;
}

// 16-bit pattern (bfloat16 or IEEE binary16) -> float, exactly.
float from_16(uint32_t h, bool fp16) {
    if (!fp16) {
        const uint32_t bits = h << 16;
        float f;
        std::memcpy(&f, &bits, sizeof(f));
        return f;
    }
    const float sign = (h & 0x8000u) ? -1.0f : 1.0f;
    const int exp = static_cast<int>((h >> 10) & 0x1fu);
    const int mant = static_cast<int>(h & 0x3ffu);
    if (exp == 0) return sign * std::ldexp(static_cast<float>(mant), -24);
    if (exp == 31) return mant ? std::nanf("") : sign * INFINITY;
    return sign * std::ldexp(static_cast<float>(mant + 1024), exp - 25);
}

uint32_t pack_pair(float lo, float hi, bool fp16) {
    return fp16 ? (to_fp16(lo) | (to_fp16(hi) << 16)) : (to_bf16(lo) | (to_bf16(hi) << 16));
}

// B fragments of mma.m16n8k16 (bf16, "col" operand) for out = in * W^T with
// W[n][k] (n outputs, k inputs), zero-padded to ktiles x 16 by ntiles x 8:
// lane l of tile (kt, nt) holds {W[n][k0], W[n][k0+1]} and
// {W[n][k0+8], W[n][k0+9]}, n = 8 nt + l/4, k0 = 16 kt + 2 (l%4).
void pack_fragments(const float* w, int n_out, int k_in, int ktiles, int ntiles, bool fp16,
                    std::vector<uint32_t>& out) {
    auto at = [&](int n, int k) { return (n < n_out && k < k_in) ? w[n * k_in + k] : 0.0f; };
    for (int kt = 0; kt < ktiles; ++kt) {
        for (int nt = 0; nt < ntiles; ++nt) {
            for (int lane = 0; lane < 32; ++lane) {
                const int n = 8 * nt + lane / 4;
                const int k0 = 16 * kt + 2 * (lane % 4);
                out.push_back(pack_pair(at(n, k0), at(n, k0 + 1), fp16));
                out.push_back(pack_pair(at(n, k0 + 8), at(n, k0 + 9), fp16));
            }
        }
    }
}

// B operand of a tcgen05 MMA in the canonical K-major, no-swizzle layout:
// W[n][k] (n outputs, k inputs) zero padded to n_rows x k_cols, element
// (n, k) at byte (n/8) (k_cols/8) 128 + (k/8) 128 + (n%8) 16 + (k%8) 2.
void pack_canonical(const float* w, int n_out, int k_in, int n_rows, int k_cols, bool fp16,
                    std::vector<uint16_t>& out) {
    const size_t base = out.size();
    out.resize(base + static_cast<size_t>(n_rows) * k_cols, 0);
    for (int n = 0; n < n_rows; ++n) {
        for (int k = 0; k < k_cols; ++k) {
            const float v = (n < n_out && k < k_in) ? w[n * k_in + k] : 0.0f;
            const size_t byte = static_cast<size_t>(n / 8) * (k_cols / 8) * 128 +
                                static_cast<size_t>(k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2;
            out[base + byte / 2] = static_cast<uint16_t>(fp16 ? to_fp16(v) : to_bf16(v));
        }
    }
}

// The tcgen05 engine's B operands from the FP32 parameter block (W1[H][5]
// b1[H] W2[H][H] b2[H] W3[3][H] b3[3]): each layer's bias becomes two extra
// input columns, its 16-bit head and the 16-bit rounding of the remainder,
// fed by constant ones; layer 1 is H x 16, layer 2 H x (H + 16), layer 3
// 16 x (H + 16), each in the canonical layout.
void pack_tc_block(const float* p, int hidden, bool fp16, std::vector<uint16_t>& tc) {
    const int pw1 = 0;
    const int pw2 = pw1 + hidden * kpt::kMlpIn + hidden;
    const int pw3 = pw2 + hidden * hidden + hidden;
    const int k2 = hidden + 16;
    std::vector<float> w1(static_cast<size_t>(hidden) * 16, 0.0f);
    std::vector<float> w2(static_cast<size_t>(hidden) * k2, 0.0f);
    std::vector<float> w3(static_cast<size_t>(16) * k2, 0.0f);
    auto split = [&](float b, float* row) {
        const float hi = from_16(fp16 ? to_fp16(b) : to_bf16(b), fp16);
        row[0] = hi;
        row[1] = b - hi;
    };
    for (int n = 0; n < hidden; ++n) {
        for (int k = 0; k < kpt::kMlpIn; ++k) w1[n * 16 + k] = p[pw1 + n * kpt::kMlpIn + k];
        split(p[pw1 + hidden * kpt::kMlpIn + n], &w1[n * 16 + kpt::kMlpIn]);
        for (int k = 0; k < hidden; ++k) w2[n * k2 + k] = p[pw2 + n * hidden + k];
        split(p[pw2 + hidden * hidden + n], &w2[n * k2 + hidden]);
    }
    for (int n = 0; n < kpt::kMlpOut; ++n) {
        for (int k = 0; k < hidden; ++k) w3[n * k2 + k] = p[pw3 + n * hidden + k];
        split(p[pw3 + kpt::kMlpOut * hidden + n], &w3[n * k2 + hidden]);
    }
    pack_canonical(w1.data(), hidden, 16, hidden, 16, fp16, tc);
    pack_canonical(w2.data(), hidden, k2, hidden, k2, fp16, tc);
    pack_canonical(w3.data(), 16, k2, 16, k2, fp16, tc);
}

}  // namespace

int kpt_surrogate_pack_tc(const float* params, int32_t hidden_width, int32_t fp16,
                          uint16_t* out, uint64_t out_len) {
    KPT_REQUIRE(params && out, "kpt_surrogate_pack_tc: NULL argument");
    KPT_REQUIRE(hidden_width == 32 || hidden_width == 64,
                "kpt_surrogate_pack_tc: hidden_width must be 32 or 64");
    std::vector<uint16_t> tc;
    pack_tc_block(params, hidden_width, fp16 != 0, tc);
    KPT_REQUIRE(out_len >= tc.size(), "kpt_surrogate_pack_tc: output too short");
    std::copy(tc.begin(), tc.end(), out);
    return KPT_OK;
}

void kpt_surrogate_default_config(kpt_surrogate_config* c) {
    if (c == nullptr) return;
    std::memset(c, 0, sizeof(*c));
    c->samples = 2000000;
    c->steps = 16000;
    c->batch = 8192;
    c->element_type = KPT_SURROGATE_BF16;
    c->quantization_aware = 0;
    c->hidden_width = kpt::kMlpHiddenDefault;
    c->learning_rate = 1e-2;
    c->mu_cut = 0.02;
    c->mu_max = 0.999;
    c->p_lo_over_p0 = 0.1;
    c->p_hi_over_p0 = 1000.0;
    c->sigma2_lo = 0.01;
    c->sigma2_hi = 1.0;
    c->gk_lo = 1.5;
    c->gk_hi = 2.0;
    c->b_lo = 0.05;
    c->b_hi = 5.0;
    c->seed = 2024;
}

int kpt_surrogate_train(kpt_context* ctx, const kpt_settings* settings,
                        const kpt_surrogate_config* config, kpt_surrogate** out,
                        double* final_loss) {
    KPT_REQUIRE(ctx && settings && config && out, "kpt_surrogate_train: NULL argument");
    *out = nullptr;
    if (int rc = validate_settings(settings)) return rc;
    const kpt_surrogate_config& c = *config;
    KPT_REQUIRE(c.samples > 0 && c.steps > 0 && c.batch > 0 && c.batch <= (1 << 20),
                "kpt_surrogate_train: samples, steps and batch must be positive");
    KPT_REQUIRE(c.element_type == KPT_SURROGATE_BF16 || c.element_type == KPT_SURROGATE_FP16,
                "kpt_surrogate_train: element_type must be KPT_SURROGATE_BF16 or _FP16");
    const int hidden = c.hidden_width == 0 ? kpt::kMlpHiddenDefault : c.hidden_width;
    KPT_REQUIRE(hidden == 32 || hidden == 64, "kpt_surrogate_train: hidden_width must be 32 or 64");
    KPT_REQUIRE(c.mu_cut > 0.0 && c.mu_cut < c.mu_max && c.mu_max < 1.0 &&
                    c.p_lo_over_p0 > 0.0 && c.p_hi_over_p0 > c.p_lo_over_p0 &&
                    c.sigma2_lo > 0.0 && c.sigma2_hi > c.sigma2_lo && c.gk_lo > 1.0 &&
                    c.gk_hi > c.gk_lo && c.b_lo > 0.0 && c.b_hi > c.b_lo &&
                    c.learning_rate > 0.0,
                "kpt_surrogate_train: invalid training box");
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_surrogate> sg(new kpt_surrogate());
    sg->ctx = ctx;
    sg->device = ctx->device;
    kpt::SurrogateBox& box = sg->box;
    const double lo[5] = {std::log(c.mu_cut), std::log(c.p_lo_over_p0 * settings->p0),
                          std::log(c.b_lo), std::log(c.sigma2_lo), c.gk_lo};
    const double hi[5] = {std::log(c.mu_max), std::log(c.p_hi_over_p0 * settings->p0),
                          std::log(c.b_hi), std::log(c.sigma2_hi), c.gk_hi};
    for (int k = 0; k < 5; ++k) {
        box.in_lo[k] = static_cast<float>(lo[k]);
        box.in_hi[k] = static_cast<float>(hi[k]);
        box.in_scale[k] = static_cast<float>(2.0 / (hi[k] - lo[k]));
        box.in_offset[k] = static_cast<float>(-(hi[k] + lo[k]) / (hi[k] - lo[k]));
    }
    box.mu_cut = static_cast<float>(c.mu_cut);
    box.fp16 = c.element_type == KPT_SURROGATE_FP16 ? 1 : 0;
    box.hidden = hidden;
    // the engine measured faster on GB300 for the width: at width 32 the
    // block-collective GEMMs' barriers and tensor-memory round trips cost
    // more than the warp-level MMAs they replace (273 vs 314 ms per
    // 1000-step interval of the 4 Mi-particle workload), at width 64 less
    sg->engine = hidden == 32 ? kpt::kEngineMmaSync : kpt::kEngineTcgen05;
    box.magnetic_dependency = settings->magnetic_dependency;
    box.momentum_dependency = settings->momentum_dependency;
    box.p0 = settings->p0;
    box.particle_v0 = settings->particle_v0;
    box.kpara0 = settings->kpara0;
    box.gamma_turb = settings->gamma_turb;
    box.qlt_omega0 = settings->qlt_omega0;
    box.qlt_lc = settings->qlt_lc;
    box.qlt_h0 = settings->qlt_h0;
    cudaStream_t st = ctx->stream;
    const size_t n = static_cast<size_t>(c.samples);
    ScopedBuffer data, work;
    KPT_CUDA(data.reserve(n * (kpt::kMlpIn + kpt::kMlpOut) * sizeof(float)));
    float* x = data.as<float>();
    float* t = x + n * kpt::kMlpIn;
    KPT_CUDA(kpt::surrogate_make_samples(c.seed, c.samples, box, x, t, st));
    std::vector<float> host_t(n * kpt::kMlpOut);
    KPT_CUDA(cudaMemcpyAsync(host_t.data(), t, host_t.size() * sizeof(float),
                             cudaMemcpyDeviceToHost, st));
    KPT_CUDA(cudaStreamSynchronize(st));
    for (int o = 0; o < kpt::kMlpOut; ++o) {
        double sum = 0.0, sum2 = 0.0;
        for (size_t i = 0; i < n; ++i) {
            const double v = host_t[i * kpt::kMlpOut + o];
            sum += v;
            sum2 += v * v;
        }
        const double mean = sum / static_cast<double>(n);
        const double var = std::max(sum2 / static_cast<double>(n) - mean * mean, 1e-12);
        if (!std::isfinite(mean) || !std::isfinite(var)) {
            return set_error(KPT_ERROR_INVALID_ARGUMENT,
                             "kpt_surrogate_train: non-finite training targets");
        }
        box.out_offset[o] = static_cast<float>(mean);
        box.out_scale[o] = static_cast<float>(std::sqrt(var));
    }
    // Xavier-uniform initial weights, zero biases.
    const int pw1 = 0, pw2 = pw1 + hidden * kpt::kMlpIn + hidden;
    const int pw3 = pw2 + hidden * hidden + hidden;
    sg->params.assign(kpt::mlp_params(hidden), 0.0f);
    std::mt19937_64 rng(c.seed ^ 0x5851f42d4c957f2dull);
    auto init = [&](int base, int rows, int cols) {
        const float a = std::sqrt(6.0f / static_cast<float>(rows + cols));
        std::uniform_real_distribution<float> u(-a, a);
        for (int k = 0; k < rows * cols; ++k) sg->params[base + k] = u(rng);
    };
    init(pw1, hidden, kpt::kMlpIn);
    init(pw2, hidden, hidden);
    init(pw3, kpt::kMlpOut, hidden);
    const size_t b = static_cast<size_t>(c.batch);
    const size_t pcount = static_cast<size_t>(kpt::mlp_params(hidden));
    const size_t chunks = (b + kpt::kGradChunk - 1) / kpt::kGradChunk;
    const size_t floats = 4 * pcount + b * (kpt::kMlpIn + 4 * hidden + kpt::kMlpOut) +
                          static_cast<size_t>(c.steps) + chunks * pcount;
    KPT_CUDA(work.reserve(floats * sizeof(float)));
    KPT_CUDA(cudaMemsetAsync(work.ptr, 0, floats * sizeof(float), st));
    kpt::SurrogateTrainLaunch L{};
    float* w = work.as<float>();
    L.x = x;
    L.t = t;
    L.n = c.samples;
    L.seed = c.seed;
    L.batch = c.batch;
    L.box = box;
    L.params = w;
    L.grad = w + pcount;
    L.m = w + 2 * pcount;
    L.v = w + 3 * pcount;
    L.xb = w + 4 * pcount;
    L.h1 = L.xb + b * kpt::kMlpIn;
    L.h2 = L.h1 + b * hidden;
    L.g1 = L.h2 + b * hidden;
    L.g2 = L.g1 + b * hidden;
    L.gy = L.g2 + b * hidden;
    L.loss = L.gy + b * kpt::kMlpOut;
    L.partial = L.loss + c.steps;
    L.beta1 = 0.9f;
    L.beta2 = 0.999f;
    // quantization-aware fine-tuning: the last quarter of the steps sees the
    // served element type's rounding
    L.quant = c.quantization_aware ? (box.fp16 ? 2 : 1) : 0;
    L.quant_from = c.steps - c.steps / 4;
    KPT_CUDA(cudaMemcpyAsync(L.params, sg->params.data(), pcount * sizeof(float),
                             cudaMemcpyHostToDevice, st));
    const double pi = 3.141592653589793238462643383279502884;
    for (int step = 0; step < c.steps; ++step) {
        const double phase = static_cast<double>(step) / static_cast<double>(c.steps);
        L.lr = static_cast<float>(c.learning_rate * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(pi * phase))));
        KPT_CUDA(kpt::surrogate_train_step(L, step, st));
    }
    std::vector<float> losses(static_cast<size_t>(c.steps));
    KPT_CUDA(cudaMemcpyAsync(losses.data(), L.loss, losses.size() * sizeof(float),
                             cudaMemcpyDeviceToHost, st));
    KPT_CUDA(cudaMemcpyAsync(sg->params.data(), L.params, pcount * sizeof(float),
                             cudaMemcpyDeviceToHost, st));
    KPT_CUDA(cudaStreamSynchronize(st));
    const int tail = std::min(c.steps, 50);
    double acc = 0.0;
    for (int k = c.steps - tail; k < c.steps; ++k) acc += losses[static_cast<size_t>(k)];
    sg->final_loss = acc / tail;
    if (final_loss) *final_loss = sg->final_loss;
    // inference copies: FP32 parameters and the BF16 fragment + bias block
    std::vector<uint32_t> words;
    const bool fp16 = box.fp16 != 0;
    const int nt = hidden / 8, kt = hidden / 16;
    pack_fragments(sg->params.data() + pw1, hidden, kpt::kMlpIn, 1, nt, fp16, words);
    pack_fragments(sg->params.data() + pw2, hidden, hidden, kt, nt, fp16, words);
    pack_fragments(sg->params.data() + pw3, kpt::kMlpOut, hidden, kt, 1, fp16, words);
    std::vector<float> bias(2 * hidden + 8, 0.0f);
    for (int k = 0; k < hidden; ++k) {
        bias[k] = sg->params[pw1 + hidden * kpt::kMlpIn + k];
        bias[hidden + k] = sg->params[pw2 + hidden * hidden + k];
    }
    for (int k = 0; k < kpt::kMlpOut; ++k) {
        bias[2 * hidden + k] = sg->params[pw3 + kpt::kMlpOut * hidden + k];
    }
    for (float b : bias) {
        uint32_t bits;
        std::memcpy(&bits, &b, sizeof(bits));
        words.push_back(bits);
    }
    KPT_CUDA(cudaMalloc(&sg->d_params, pcount * sizeof(float)));
    const size_t block_bytes = kpt::mlp_smem_bytes(hidden);
    KPT_REQUIRE(words.size() * sizeof(uint32_t) == block_bytes,
                "kpt_surrogate_train: fragment block size mismatch");
    KPT_CUDA(cudaMalloc(&sg->d_block, block_bytes));
    KPT_CUDA(cudaMemcpy(sg->d_params, sg->params.data(), pcount * sizeof(float),
                        cudaMemcpyHostToDevice));
    KPT_CUDA(cudaMemcpy(sg->d_block, words.data(), block_bytes, cudaMemcpyHostToDevice));
    // the tcgen05 engine's operand block
    std::vector<uint16_t> tc;
    pack_tc_block(sg->params.data(), hidden, fp16, tc);
    const size_t tc_bytes = kpt::tc_block_bytes(hidden);
    KPT_REQUIRE(tc.size() * sizeof(uint16_t) == tc_bytes,
                "kpt_surrogate_train: tensor-core block size mismatch");
    KPT_CUDA(cudaMalloc(&sg->d_tc_block, tc_bytes));
    KPT_CUDA(cudaMemcpy(sg->d_tc_block, tc.data(), tc_bytes, cudaMemcpyHostToDevice));
    *out = sg.release();
    return KPT_OK;
}

int kpt_surrogate_destroy(kpt_surrogate* sg) {
    if (sg == nullptr) return KPT_OK;
    cudaSetDevice(sg->device);
    cudaFree(sg->d_params);
    cudaFree(sg->d_block);
    cudaFree(sg->d_tc_block);
    delete sg;
    return KPT_OK;
}

int kpt_surrogate_parameters(const kpt_surrogate* sg, float* params, int len, float* norm,
                             int norm_len) {
    KPT_REQUIRE(sg != nullptr, "kpt_surrogate_parameters: NULL handle");
    if (params != nullptr) {
        KPT_REQUIRE(len >= static_cast<int>(sg->params.size()),
                    "kpt_surrogate_parameters: params too short");
        std::copy(sg->params.begin(), sg->params.end(), params);
    }
    if (norm != nullptr) {
        KPT_REQUIRE(norm_len >= 17, "kpt_surrogate_parameters: normalisation too short");
        for (int k = 0; k < 5; ++k) {
            norm[k] = sg->box.in_lo[k];
            norm[5 + k] = sg->box.in_hi[k];
        }
        for (int k = 0; k < 3; ++k) {
            norm[10 + k] = sg->box.out_offset[k];
            norm[13 + k] = sg->box.out_scale[k];
        }
        norm[16] = sg->box.mu_cut;
    }
    return KPT_OK;
}

int kpt_surrogate_shape(const kpt_surrogate* sg, int32_t* hidden_width, int32_t* parameters) {
    KPT_REQUIRE(sg != nullptr, "kpt_surrogate_shape: NULL handle");
    if (hidden_width) *hidden_width = sg->box.hidden;
    if (parameters) *parameters = static_cast<int32_t>(sg->params.size());
    return KPT_OK;
}

int kpt_surrogate_evaluate(kpt_surrogate* sg, uint64_t n, const double* inputs, int tensor_cores,
                           double* outputs, int32_t* served) {
    KPT_REQUIRE(sg && inputs && outputs, "kpt_surrogate_evaluate: NULL argument");
    KPT_REQUIRE(n < (1ull << 30), "kpt_surrogate_evaluate: too many inputs");
    if (n == 0) return KPT_OK;
    KPT_CUDA(cudaSetDevice(sg->device));
    ScopedBuffer buf;
    KPT_CUDA(buf.reserve(n * 8 * sizeof(double) + n * sizeof(int) + sizeof(unsigned int)));
    double* din = buf.as<double>();
    double* dout = din + n * 5;
    int* dserved = reinterpret_cast<int*>(dout + n * 3);
    cudaStream_t st = sg->ctx->stream;
    KPT_CUDA(cudaMemcpyAsync(din, inputs, n * 5 * sizeof(double), cudaMemcpyHostToDevice, st));
    unsigned int* dtimeouts = reinterpret_cast<unsigned int*>(dserved + n);
    KPT_CUDA(cudaMemsetAsync(dtimeouts, 0, sizeof(unsigned int), st));
    kpt::SurrogateServe serve{sg->d_params, sg->d_block, sg->d_tc_block,
                              tensor_cores == 0 ? -1 : sg->engine, dtimeouts};
    KPT_CUDA(kpt::surrogate_eval(static_cast<int>(n), din, sg->box, serve, dout, dserved, st));
    unsigned int timeouts = 0;
    KPT_CUDA(cudaMemcpyAsync(&timeouts, dtimeouts, sizeof(timeouts), cudaMemcpyDeviceToHost, st));
    KPT_CUDA(cudaMemcpyAsync(outputs, dout, n * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (served) {
        KPT_CUDA(cudaMemcpyAsync(served, dserved, n * sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    KPT_CUDA(cudaStreamSynchronize(st));
    if (timeouts != 0) {
        return set_error(KPT_ERROR_CUDA,
                         "kpt_surrogate_evaluate: a tensor-core completion wait timed out");
    }
    return KPT_OK;
}

int kpt_surrogate_set_engine(kpt_surrogate* sg, int engine) {
    KPT_REQUIRE(sg != nullptr, "kpt_surrogate_set_engine: NULL handle");
    KPT_REQUIRE(engine == KPT_ENGINE_TCGEN05 || engine == KPT_ENGINE_MMA_SYNC,
                "kpt_surrogate_set_engine: unknown engine");
    sg->engine = engine;
    return KPT_OK;
}

int kpt_surrogate_check_timeout(kpt_surrogate* sg, uint32_t blocks, uint32_t polls,
                                uint32_t* timed_out, uint32_t* finished) {
    KPT_REQUIRE(sg != nullptr, "kpt_surrogate_check_timeout: NULL handle");
    KPT_REQUIRE(sg->box.hidden == 64, "kpt_surrogate_check_timeout: needs a width-64 network");
    KPT_REQUIRE(blocks >= 1 && blocks <= 4096, "kpt_surrogate_check_timeout: 1 <= blocks <= 4096");
    KPT_REQUIRE(polls >= 1 && polls <= (1u << 20), "kpt_surrogate_check_timeout: 1 <= polls <= 2^20");
    KPT_CUDA(cudaSetDevice(sg->device));
    cudaStream_t st = sg->ctx->stream;
    ScopedBuffer buf;
    KPT_CUDA(buf.reserve(2 * sizeof(unsigned int)));
    KPT_CUDA(cudaMemsetAsync(buf.ptr, 0, 2 * sizeof(unsigned int), st));
    KPT_CUDA(kpt::surrogate_tc_timeout_check(sg->d_tc_block, static_cast<int>(blocks), polls,
                                             buf.as<unsigned int>(), st));
    unsigned int host[2] = {0, 0};
    KPT_CUDA(cudaMemcpyAsync(host, buf.ptr, sizeof(host), cudaMemcpyDeviceToHost, st));
    KPT_CUDA(cudaStreamSynchronize(st));
    if (timed_out) *timed_out = host[0];
    if (finished) *finished = host[1];
    return KPT_OK;
}

int kpt_surrogate_get_engine(const kpt_surrogate* sg, int32_t* engine) {
    KPT_REQUIRE(sg && engine, "kpt_surrogate_get_engine: NULL argument");
    *engine = sg->engine;
    return KPT_OK;
}

int kpt_surrogate_gradient(kpt_context* ctx, int32_t hidden_width, const float* params,
                           uint64_t n, const float* inputs, const float* targets, float* grad,
                           float* loss) {
    KPT_REQUIRE(ctx && params && inputs && targets && grad, "kpt_surrogate_gradient: NULL");
    KPT_REQUIRE(n > 0 && n <= (1u << 20), "kpt_surrogate_gradient: 0 < n <= 2^20");
    const int hidden = hidden_width == 0 ? kpt::kMlpHiddenDefault : hidden_width;
    KPT_REQUIRE(hidden == 32 || hidden == 64,
                "kpt_surrogate_gradient: hidden_width must be 32 or 64");
    if (int rc = activate(ctx)) return rc;
    const size_t pcount = static_cast<size_t>(kpt::mlp_params(hidden));
    const size_t chunks = (n + kpt::kGradChunk - 1) / kpt::kGradChunk;
    const size_t floats =
        n * (5 + 3) + 2 * pcount + n * (5 + 4 * hidden + 3) + 1 + chunks * pcount;
    ScopedBuffer buf;
    KPT_CUDA(buf.reserve(floats * sizeof(float)));
    KPT_CUDA(cudaMemsetAsync(buf.ptr, 0, floats * sizeof(float), ctx->stream));
    float* w = buf.as<float>();
    kpt::SurrogateTrainLaunch L{};
    float* x = w;
    float* t = x + n * 5;
    L.x = x;
    L.t = t;
    L.n = static_cast<int>(n);
    L.batch = static_cast<int>(n);
    for (int k = 0; k < 5; ++k) {
        L.box.in_lo[k] = -1.0f;
        L.box.in_hi[k] = 1.0f;
        L.box.in_scale[k] = 1.0f;
        L.box.in_offset[k] = 0.0f;
    }
    for (int k = 0; k < 3; ++k) {
        L.box.out_offset[k] = 0.0f;
        L.box.out_scale[k] = 1.0f;
    }
    L.params = t + n * 3;
    L.grad = L.params + pcount;
    L.xb = L.grad + pcount;
    L.box.hidden = hidden;
    L.h1 = L.xb + n * 5;
    L.h2 = L.h1 + n * hidden;
    L.g1 = L.h2 + n * hidden;
    L.g2 = L.g1 + n * hidden;
    L.gy = L.g2 + n * hidden;
    L.loss = L.gy + n * 3;
    L.partial = L.loss + 1;
    cudaStream_t st = ctx->stream;
    KPT_CUDA(cudaMemcpyAsync(x, inputs, n * 5 * sizeof(float), cudaMemcpyHostToDevice, st));
    KPT_CUDA(cudaMemcpyAsync(t, targets, n * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
    KPT_CUDA(cudaMemcpyAsync(L.params, params, pcount * sizeof(float), cudaMemcpyHostToDevice, st));
    KPT_CUDA(kpt::surrogate_gradient(L, st));
    KPT_CUDA(cudaMemcpyAsync(grad, L.grad, pcount * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (loss) KPT_CUDA(cudaMemcpyAsync(loss, L.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    KPT_CUDA(cudaStreamSynchronize(st));
    return KPT_OK;
}

int kpt_context_set_surrogate(kpt_context* ctx, kpt_surrogate* sg) {
    KPT_REQUIRE(ctx != nullptr, "kpt_context_set_surrogate: ctx is NULL");
    ctx->surrogate = sg;
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(ctx->judge.reserve(4 * sizeof(unsigned long long)));
    KPT_CUDA(cudaMemsetAsync(ctx->judge.ptr, 0, 4 * sizeof(unsigned long long), ctx->stream));
    return KPT_OK;
}

int kpt_surrogate_judge(kpt_context* ctx, uint64_t* evaluations, uint64_t* judged,
                        uint64_t* fallbacks, double* max_rel_error) {
    KPT_REQUIRE(ctx != nullptr, "kpt_surrogate_judge: ctx is NULL");
    unsigned long long host[4] = {0, 0, 0, 0};
    if (ctx->judge.ptr != nullptr) {
        if (int rc = activate(ctx)) return rc;
        KPT_CUDA(cudaMemcpyAsync(host, ctx->judge.ptr, sizeof(host), cudaMemcpyDeviceToHost,
                                 ctx->stream));
        KPT_CUDA(cudaMemsetAsync(ctx->judge.ptr, 0, sizeof(host), ctx->stream));
        KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    if (evaluations) *evaluations = host[0];
    if (judged) *judged = host[1];
    if (fallbacks) *fallbacks = host[2];
    if (max_rel_error) {
        float f;
        const uint32_t bits = static_cast<uint32_t>(host[3]);
        std::memcpy(&f, &bits, sizeof(f));
        *max_rel_error = static_cast<double>(f);
    }
    return KPT_OK;
}

int kpt_particles_sort(kpt_context* ctx, kpt_particles* parts, const kpt_field* grid,
                       int tile_x, int tile_y) {
    KPT_REQUIRE(ctx && parts && grid, "kpt_particles_sort: NULL handle");
    KPT_REQUIRE(tile_x > 0 && tile_y > 0, "kpt_particles_sort: tile sizes must be positive");
    if (int rc = activate(ctx)) return rc;
    const int tiles_x = (grid->nx + tile_x - 1) / tile_x;
    const int tiles_y = (grid->ny + tile_y - 1) / tile_y;
    KPT_REQUIRE(static_cast<long long>(tiles_x) * tiles_y < (1ll << 30),
                "kpt_particles_sort: too many tiles");
    const uint64_t n = std::max<uint64_t>(parts->count, 1);
    KPT_CUDA(parts->order.reserve(n * sizeof(uint32_t)));
    KPT_CUDA(parts->keys.reserve(n * sizeof(uint32_t)));
    KPT_CUDA(parts->tile_counts.reserve((static_cast<size_t>(tiles_x) * tiles_y + 1) *
                                        sizeof(uint32_t)));
    kpt::SortLaunch launch{};
    launch.grid = grid->grid;
    launch.parts = parts->arrays;
    launch.count = parts->count;
    launch.tile_x = tile_x;
    launch.tile_y = tile_y;
    launch.tiles_x = tiles_x;
    launch.tiles_y = tiles_y;
    launch.keys = parts->keys.as<unsigned int>();
    launch.counts = parts->tile_counts.as<unsigned int>();
    launch.order = parts->order.as<unsigned int>();
    KPT_CUDA(kpt::launch_sort(launch, ctx->stream));
    parts->order_valid = true;
    return KPT_OK;
}

int kpt_particles_pack_records(kpt_context* ctx, const kpt_particles* parts,
                               double initial_kinetic_energy, void* out, uint64_t out_len) {
    KPT_REQUIRE(ctx && parts && out, "kpt_particles_pack_records: NULL argument");
    const uint64_t bytes = parts->count * 100;
    KPT_REQUIRE(out_len >= bytes, "kpt_particles_pack_records: output shorter than count x 100");
    if (parts->count == 0) return KPT_OK;
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(ctx->sample_io.reserve(bytes));
    KPT_CUDA(kpt::launch_pack_records(parts->arrays, parts->count, initial_kinetic_energy,
                                      ctx->sample_io.as<uint32_t>(), ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(out, ctx->sample_io.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_host_alloc(uint64_t bytes, void** out) {
    KPT_REQUIRE(out != nullptr, "kpt_host_alloc: NULL argument");
    *out = nullptr;
    if (bytes == 0) return KPT_OK;
    KPT_CUDA(cudaHostAlloc(out, bytes, cudaHostAllocPortable));
    return KPT_OK;
}

int kpt_host_free(void* ptr) {
    if (ptr != nullptr) cudaFreeHost(ptr);
    return KPT_OK;
}

int kpt_particles_clear_order(kpt_particles* parts) {
    KPT_REQUIRE(parts != nullptr, "kpt_particles_clear_order: NULL handle");
    parts->order_valid = false;
    return KPT_OK;
}

int kpt_summarize_noalloc(const kpt_particle_arrays* arrays, uint64_t count, void* cuda_stream,
                          kpt_summary* out) {
    KPT_REQUIRE(arrays != nullptr && out != nullptr, "kpt_summarize_noalloc: NULL argument");
    std::memset(out, 0, sizeof(*out));
    out->stored = count;
    if (count == 0) {
        return KPT_OK;
    }
    if (count > kpt::noalloc_summary_max_particles()) {
        return set_error(KPT_ERROR_CAPACITY,
                         "kpt_summarize_noalloc: count " + std::to_string(count) +
                             " exceeds the fixed scratch limit of " +
                             std::to_string(kpt::noalloc_summary_max_particles()) +
                             " particles; use kpt_summarize");
    }
    KPT_REQUIRE(arrays->p && arrays->step_dt && arrays->weight && arrays->status &&
                    arrays->split_level,
                "kpt_summarize_noalloc: NULL device array");
    kpt::SummaryLaunch launch{};
    launch.p = arrays->p;
    launch.dt = arrays->step_dt;
    launch.weight = arrays->weight;
    launch.status = arrays->status;
    launch.level = arrays->split_level;
    launch.count = count;
    kpt::SummaryPartial r{};
    KPT_CUDA(kpt::noalloc_summary(launch, static_cast<cudaStream_t>(cuda_stream), &r));
    out->active = r.active;
    out->inactive = r.inactive;
    out->weight_sum = r.weight_sum;
    out->max_split_level = r.max_level;
    if (r.active > 0) {
        out->p_min = r.p_min;
        out->p_max = r.p_max;
        out->dt_min = r.dt_min;
        out->dt_max = r.dt_max;
        out->p_avg = r.p_sum / static_cast<double>(r.active);
        out->dt_avg = r.dt_sum / static_cast<double>(r.active);
    }
    return KPT_OK;
}

int kpt_sample_table(kpt_context* ctx, const kpt_field* lower, const kpt_field* upper,
                     uint64_t n, const double* x, const double* y, const double* rt,
                     int time_interpolation, double* out) {
    KPT_REQUIRE(ctx && lower && upper && out && x && y && rt, "kpt_sample_table: NULL argument");
    KPT_REQUIRE(lower->kind == upper->kind && lower->precision == upper->precision &&
                    lower->nx == upper->nx && lower->ny == upper->ny,
                "kpt_sample_table: tables differ");
    if (n == 0) {
        return KPT_OK;
    }
    if (int rc = activate(ctx)) return rc;
    const int ncomp = lower->kind == KPT_TABLE_FOCUSED21 ? 21 : 16;
    const size_t bytes = n * sizeof(double) * (3 + ncomp);
    KPT_CUDA(ctx->sample_io.reserve(bytes));
    double* dx = ctx->sample_io.as<double>();
    double* dy = dx + n;
    double* drt = dy + n;
    double* dout = drt + n;
    KPT_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(dy, y, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(drt, rt, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    kpt::SampleLaunch launch{};
    launch.grid = lower->grid;
    launch.lower = lower->table;
    launch.upper = upper->table;
    launch.x = dx;
    launch.y = dy;
    launch.rt = drt;
    launch.n = n;
    const kpt::Axis& ax = lower->grid.axis[0];
    const kpt::Axis& ay = lower->grid.axis[1];
    launch.shift_x = 0.5 * ((ax.upper - ax.lower) / static_cast<double>(ax.n));
    launch.shift_y = 0.5 * ((ay.upper - ay.lower) / static_cast<double>(ay.n));
    launch.time_interpolation = time_interpolation;
    launch.focused = lower->kind == KPT_TABLE_FOCUSED21;
    launch.precision = lower->precision;
    launch.out = dout;
    KPT_CUDA(kpt::launch_sample(launch, ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(out, dout, n * ncomp * sizeof(double), cudaMemcpyDeviceToHost,
                             ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

}  // extern "C"

// ====================================================================
// Header-library step API: ParkerSolver / ParticleSystem (2D Cartesian)
// ====================================================================

struct kpt_grid {
    kpt_context* ctx = nullptr;
    int device = 0;
    int nx = 0, ny = 0;
    kpt::LibGrid g{};
    DeviceBuffer coordinates;  // stored axes: faces then cell centres of each axis
    ~kpt_grid() {
        if (coordinates.ptr != nullptr) {
            cudaSetDevice(device);
            coordinates.release();
        }
    }
};

struct kpt_system {
    kpt_context* ctx = nullptr;
    int device = 0;
    uint64_t count = 0;
    uint64_t capacity = 0;
    kpt_particle_properties props{};
    kpt_split_policy policy{};
    void* block = nullptr;
    kpt::SystemArrays a{};
    DeviceBuffer flags, block_counts, tallies;
    DeviceBuffer keys_a, keys_b, idx_a, idx_b, hist, staging, scalars;
};

struct kpt_focus_solver {
    kpt_context* ctx = nullptr;
    int device = 0;
    kpt::LibGrid grid{};
    uint64_t points = 0;
    double* basis = nullptr;
    int constant_ratio = 0;
    double courant = 0.3;
    double max_mu = 1.0;
    kpt_scattering_parameters scattering{};
    DeviceBuffer terms, scalars, dt_history;
    int precision = KPT_PRECISION_F64;
    DeviceBuffer basis_f32;        // the mixed step's FP32 copy of the basis
    bool basis_f32_valid = false;  // cleared whenever the FP64 basis changes
};

struct kpt_parker_solver {
    kpt_context* ctx = nullptr;
    int device = 0;
    kpt::LibGrid grid{};
    uint64_t points = 0;
    double* basis = nullptr;
    int constant_ratio = 0;
    double courant = 0.3;
    int precision = KPT_PRECISION_F64;
    DeviceBuffer basis_f32;        // the mixed step's FP32 copy of the basis
    bool basis_f32_valid = false;  // cleared whenever the FP64 basis changes
    DeviceBuffer terms;
    // min bits (u64), dt (f64), error (i32 + pad), error index (u64)
    DeviceBuffer scalars;
    DeviceBuffer dt_history;
};

namespace {

const char* lib_error_message(int code) {
    switch (code) {
        case 1: return "FieldInterpolator: position lies outside the interpolation domain.";
        case 2: return "ParkerSolver: stochastic diffusion requires |B| > 0.";
        case 3: return "ParkerSolver: diffusion coefficients must be finite and non-negative.";
        case 4: return "ParkerSolver: projected diffusion coefficient is invalid.";
        case 5: return "ParkerSolver: local physical cell width must be positive.";
        case 7: return "ParkerSolver: adaptive deterministic time step is not positive and finite.";
        case 8: return "FocusTransportSolver: pitch-angle cosine is not finite.";
        case 9: return "FocusTransportSolver: focused transport requires |B| > 0.";
        case 10: return "FocusTransportSolver: interpolated magnetic direction is invalid.";
        case 11: return "FocusTransportSolver: diffusion coefficients must be finite and non-negative.";
        case 12: return "FocusTransportSolver: pitch-angle stepping requires positive particle speed.";
        case 13: return "LegencyModel: pitch-angle scattering requires positive local inputs.";
        case 14: return "LegencyModel: D_mumu requires positive omega, speed, sigma2, and Lc.";
        case 15: return "LegencyModel: D_mumu denominator must be positive.";
        case 16: return "FocusTransportSolver: adaptive stochastic time step is not positive and finite.";
        case 17: return "FocusTransportSolver: adaptive deterministic time step is not positive and finite.";
        default: return "ParkerSolver: adaptive stochastic time step is not positive and finite.";
    }
}

int validate_properties(const kpt_particle_properties* p) {
    // ParticleProperties::validate (ParticleSystem.hpp:152-164)
    KPT_REQUIRE(p != nullptr, "ParticleProperties: NULL");
    if (!std::isfinite(p->rest_mass) || p->rest_mass <= 0.0 || !std::isfinite(p->charge) ||
        !std::isfinite(p->speed_of_light) || p->speed_of_light <= 0.0 ||
        !std::isfinite(p->energy_scale_erg) || p->energy_scale_erg <= 0.0) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "ParticleProperties: rest mass and speed of light must be positive "
                         "finite dimensionless values, charge must be finite, and the energy "
                         "scale must be positive and finite.");
    }
    return KPT_OK;
}

}  // namespace

extern "C" {

int kpt_grid_create(kpt_context* ctx, int nx, int ny, const double* x_edges,
                    const double* y_edges, const int32_t* periodic, kpt_grid** out) {
    KPT_REQUIRE(ctx && x_edges && y_edges && periodic && out, "kpt_grid_create: NULL argument");
    *out = nullptr;
    KPT_REQUIRE(nx > 0 && ny > 0, "kpt_grid_create: nx and ny must be positive");
    std::unique_ptr<kpt_grid> g(new kpt_grid());
    g->ctx = ctx;
    g->device = ctx->device;
    g->nx = nx;
    g->ny = ny;
    const double* edges[2] = {x_edges, y_edges};
    const int counts[2] = {nx, ny};
    for (int dim = 0; dim < 2; ++dim) {
        const double* e = edges[dim];
        const int n = counts[dim];
        for (int i = 0; i <= n; ++i) {
            KPT_REQUIRE(std::isfinite(e[i]) && (i == 0 || e[i] > e[i - 1]),
                        "kpt_grid_create: face coordinates must be finite and strictly ascending");
        }
        double step = 0.0;
        KPT_REQUIRE(edges_uniform(e, n, &step),
                    "kpt_grid_create: the library grid needs uniform edges");
        kpt::LibAxis& a = g->g.axis[dim];
        a.n = n;
        a.periodic = periodic[dim] != 0 ? 1 : 0;
        a.x0 = e[0];
        a.dx = step;
        a.inv_dx = 1.0 / step;
        // AnalyticCoordinateMapping face coordinates x0 + i dx
        // (MappedCoordinateGrid.hpp:118-147)
        a.lower = a.x0 + 0.0 * a.dx;
        a.upper = a.x0 + static_cast<double>(n) * a.dx;
        a.ghost_lower = a.x0 + (-2.0) * a.dx;
        a.ghost_upper = a.x0 + static_cast<double>(n + 2) * a.dx;
        a.width = a.upper - a.lower;
        a.inv_width = a.width != 0.0 ? 1.0 / a.width : 0.0;
    }
    g->g.ex = nx + 4;
    *out = g.release();
    return KPT_OK;
}

// StoredCoordinateGrid from face coordinates (StoredCoordinateGrid.hpp:53-66,
// GridValidation.hpp:123-170, :773-784): n + 5 faces per axis including the
// two ghost faces on each side, checked as the reference's validation does;
// cell centres are the midpoints of adjacent faces (:423-436) and the cached
// bounds faces 0, n (physical) and -2, n + 2 (ghosted) (:79-103).
int kpt_grid_create_stored(kpt_context* ctx, int nx, int ny, const double* x_faces,
                           const double* y_faces, const int32_t* periodic, kpt_grid** out) {
    KPT_REQUIRE(ctx && x_faces && y_faces && periodic && out,
                "kpt_grid_create_stored: NULL argument");
    *out = nullptr;
    KPT_REQUIRE(nx > 0 && ny > 0, "kpt_grid_create_stored: nx and ny must be positive");
    const double* faces[2] = {x_faces, y_faces};
    const int counts[2] = {nx, ny};
    for (int dim = 0; dim < 2; ++dim) {
        const double* f = faces[dim];
        const int count = counts[dim] + 5;
        const std::string label = "dim " + std::to_string(dim);
        for (int i = 0; i < count; ++i) {
            KPT_REQUIRE(std::isfinite(f[i]),
                        "GridValidation: non-finite face-centered coordinate in " + label + ".");
        }
        const double first_dx = f[1] - f[0];
        KPT_REQUIRE(first_dx != 0.0,
                    "GridValidation: duplicate adjacent face-centered coordinates in " + label +
                        ".");
        KPT_REQUIRE(first_dx > 0.0,
                    "GridValidation: descending face-centered coordinates are not supported in " +
                        label + ".");
        for (int i = 1; i < count - 1; ++i) {
            const double dx = f[i + 1] - f[i];
            KPT_REQUIRE(dx != 0.0,
                        "GridValidation: duplicate adjacent face-centered coordinates in " +
                            label + ".");
            KPT_REQUIRE(dx > 0.0,
                        "GridValidation: non-monotonic face-centered coordinates in " + label +
                            ".");
        }
    }
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_grid> g(new kpt_grid());
    g->ctx = ctx;
    g->device = ctx->device;
    g->nx = nx;
    g->ny = ny;
    // per axis: n + 5 faces, then n + 4 cell centres
    std::vector<double> host;
    size_t offsets[2][2];
    for (int dim = 0; dim < 2; ++dim) {
        const int n = counts[dim];
        const double* f = faces[dim];
        offsets[dim][0] = host.size();
        host.insert(host.end(), f, f + n + 5);
        offsets[dim][1] = host.size();
        for (int k = 0; k < n + 4; ++k) {
            host.push_back(0.5 * (f[k] + f[k + 1]));
        }
    }
    KPT_CUDA(g->coordinates.reserve(host.size() * sizeof(double)));
    KPT_CUDA(cudaMemcpy(g->coordinates.ptr, host.data(), host.size() * sizeof(double),
                        cudaMemcpyHostToDevice));
    for (int dim = 0; dim < 2; ++dim) {
        const int n = counts[dim];
        const double* f = faces[dim];
        kpt::LibAxis& a = g->g.axis[dim];
        a.n = n;
        a.periodic = periodic[dim] != 0 ? 1 : 0;
        a.stored = 1;
        a.faces = g->coordinates.as<double>() + offsets[dim][0];
        a.cells = g->coordinates.as<double>() + offsets[dim][1];
        a.x0 = f[2];
        a.dx = 0.0;
        a.inv_dx = 0.0;
        a.lower = f[2];
        a.upper = f[n + 2];
        a.ghost_lower = f[0];
        a.ghost_upper = f[n + 4];
        a.width = a.upper - a.lower;
        a.inv_width = a.width != 0.0 ? 1.0 / a.width : 0.0;
    }
    g->g.ex = nx + 4;
    *out = g.release();
    return KPT_OK;
}

int kpt_grid_destroy(kpt_grid* grid) {
    delete grid;
    return KPT_OK;
}

int kpt_system_create(kpt_context* ctx, uint64_t count, uint64_t capacity,
                      const kpt_particle_properties* properties, const kpt_split_policy* policy,
                      kpt_system** out) {
    KPT_REQUIRE(ctx && out, "kpt_system_create: NULL argument");
    *out = nullptr;
    if (int rc = validate_properties(properties)) return rc;
    kpt_split_policy pol{2.0, 0.0};
    if (policy != nullptr) pol = *policy;
    // ParticleSplittingPolicy::validate (ParticleSystem.hpp:287-294)
    KPT_REQUIRE(std::isfinite(pol.energy_split_ratio) && pol.energy_split_ratio > 1.0 &&
                    std::isfinite(pol.minimum_child_weight) && pol.minimum_child_weight >= 0.0,
                "ParticleSplittingPolicy: energy split ratio must be greater than one and "
                "minimum child weight must be finite and non-negative.");
    KPT_REQUIRE(capacity >= count,
                "ParticleSystem: capacity must be greater than or equal to count.");
    KPT_REQUIRE(capacity < (1ull << 31), "kpt_system_create: capacity must be below 2^31");
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_system> sys(new kpt_system());
    sys->ctx = ctx;
    sys->device = ctx->device;
    sys->count = count;
    sys->capacity = capacity;
    sys->props = *properties;
    sys->policy = pol;
    const size_t cap = capacity > 0 ? capacity : 1;
    const size_t dbytes = (cap * sizeof(double) + 255) & ~size_t(255);
    const size_t ibytes = (cap * sizeof(int32_t) + 255) & ~size_t(255);
    const size_t total = 12 * dbytes + 3 * ibytes;  // id (8 B) + 11 doubles
    KPT_CUDA(cudaMalloc(&sys->block, total));
    char* base = static_cast<char*>(sys->block);
    kpt::SystemArrays& a = sys->a;
    a.id = reinterpret_cast<uint64_t*>(base);
    double** dptrs[11] = {&a.x, &a.y, &a.prev_x, &a.prev_y, &a.prevstep_x, &a.prevstep_y,
                          &a.p, &a.mu, &a.weight, &a.e0, nullptr};
    for (int k = 0; k < 10; ++k) *dptrs[k] = reinterpret_cast<double*>(base + (k + 1) * dbytes);
    a.status = reinterpret_cast<int*>(base + 12 * dbytes);
    a.split_level = reinterpret_cast<int*>(base + 12 * dbytes + ibytes);
    a.sort_key = reinterpret_cast<int*>(base + 12 * dbytes + 2 * ibytes);
    KPT_CUDA(kpt::system_default_state(a, count, capacity, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = sys.release();
    return KPT_OK;
}

int kpt_system_destroy(kpt_system* sys) {
    if (sys == nullptr) return KPT_OK;
    cudaSetDevice(sys->device);
    cudaFree(sys->block);
    for (DeviceBuffer* b : {&sys->flags, &sys->block_counts, &sys->tallies, &sys->keys_a,
                            &sys->keys_b, &sys->idx_a, &sys->idx_b, &sys->hist, &sys->staging,
                            &sys->scalars}) {
        b->release();
    }
    delete sys;
    return KPT_OK;
}

int kpt_system_count(const kpt_system* sys, uint64_t* count, uint64_t* capacity) {
    KPT_REQUIRE(sys != nullptr, "kpt_system_count: NULL handle");
    if (count) *count = sys->count;
    if (capacity) *capacity = sys->capacity;
    return KPT_OK;
}

int kpt_system_set_count(kpt_system* sys, uint64_t count) {
    KPT_REQUIRE(sys != nullptr, "kpt_system_set_count: NULL handle");
    KPT_REQUIRE(count <= sys->capacity, "kpt_system_set_count: count exceeds capacity");
    sys->count = count;
    return KPT_OK;
}

namespace {

int system_copy(const kpt_system* sys, uint64_t n, const kpt_system_arrays* h, bool upload) {
    KPT_REQUIRE(sys && h, "kpt_system copy: NULL argument");
    KPT_REQUIRE(n <= sys->capacity, "kpt_system copy: n exceeds capacity");
    KPT_CUDA(cudaSetDevice(sys->device));
    const kpt::SystemArrays& a = sys->a;
    cudaStream_t st = sys->ctx->stream;
    struct Pair {
        void* dev;
        void* host;
        size_t size;
    } pairs[14] = {{a.id, h->id, 8},         {a.x, h->x, 8},
                   {a.y, h->y, 8},           {a.prev_x, h->prev_x, 8},
                   {a.prev_y, h->prev_y, 8}, {a.prevstep_x, h->prevstep_x, 8},
                   {a.prevstep_y, h->prevstep_y, 8}, {a.p, h->p, 8},
                   {a.mu, h->mu, 8},         {a.weight, h->weight, 8},
                   {a.e0, h->e0, 8},         {a.status, h->status, 4},
                   {a.split_level, h->split_level, 4}, {a.sort_key, h->sort_key, 4}};
    for (const Pair& pr : pairs) {
        if (pr.host == nullptr || n == 0) continue;
        if (upload) {
            KPT_CUDA(cudaMemcpyAsync(pr.dev, pr.host, n * pr.size, cudaMemcpyHostToDevice, st));
        } else {
            KPT_CUDA(cudaMemcpyAsync(pr.host, pr.dev, n * pr.size, cudaMemcpyDeviceToHost, st));
        }
    }
    KPT_CUDA(cudaStreamSynchronize(st));
    return KPT_OK;
}

}  // namespace

int kpt_system_upload(kpt_system* sys, uint64_t n, const kpt_system_arrays* host) {
    return system_copy(sys, n, host, true);
}

int kpt_system_download(const kpt_system* sys, uint64_t n, const kpt_system_arrays* host) {
    return system_copy(sys, n, host, false);
}

int kpt_system_capture_previous_positions(kpt_context* ctx, kpt_system* sys) {
    KPT_REQUIRE(ctx && sys, "kpt_system_capture_previous_positions: NULL handle");
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(kpt::system_capture(sys->a, sys->capacity, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_system_apply_boundary(kpt_context* ctx, kpt_system* sys, const kpt_grid* grid) {
    KPT_REQUIRE(ctx && sys && grid, "kpt_system_apply_boundary: NULL handle");
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(kpt::system_boundary(grid->g, sys->a, sys->count, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_system_sort_by_key(kpt_context* ctx, kpt_system* sys, int32_t minimum_key,
                           int32_t maximum_key) {
    KPT_REQUIRE(ctx && sys, "kpt_system_sort_by_key: NULL handle");
    if (sys->count <= 1 || minimum_key == maximum_key) return KPT_OK;
    KPT_REQUIRE(maximum_key >= minimum_key, "ParticleSystem: invalid sort key range.");
    if (int rc = activate(ctx)) return rc;
    const uint64_t n = sys->count;
    const uint64_t blocks = (n + 255) / 256;
    KPT_CUDA(sys->keys_a.reserve(n * 4));
    KPT_CUDA(sys->keys_b.reserve(n * 4));
    KPT_CUDA(sys->idx_a.reserve(n * 4));
    KPT_CUDA(sys->idx_b.reserve(n * 4));
    KPT_CUDA(sys->hist.reserve(256 * blocks * 4));
    KPT_CUDA(sys->staging.reserve(n * 8));
    KPT_CUDA(sys->scalars.reserve(64));
    kpt::LibSortLaunch L{};
    L.sys = sys->a;
    L.count = n;
    L.lo = minimum_key;
    L.hi = maximum_key;
    L.keys_a = sys->keys_a.as<unsigned int>();
    L.keys_b = sys->keys_b.as<unsigned int>();
    L.idx_a = sys->idx_a.as<unsigned int>();
    L.idx_b = sys->idx_b.as<unsigned int>();
    L.hist = sys->hist.as<unsigned int>();
    L.scratch_total = sys->scalars.as<unsigned long long>();
    L.staging = sys->staging.ptr;
    KPT_CUDA(kpt::system_sort(L, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_system_compact(kpt_context* ctx, kpt_system* sys, uint64_t* active_count) {
    KPT_REQUIRE(ctx && sys, "kpt_system_compact: NULL handle");
    if (active_count) *active_count = 0;
    if (sys->count == 0) return KPT_OK;
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(sys->scalars.reserve(64));
    unsigned long long* active = sys->scalars.as<unsigned long long>() + 1;
    KPT_CUDA(kpt::system_compact_keys(sys->a, sys->count, active, ctx->stream));
    unsigned long long host = 0;
    KPT_CUDA(cudaMemcpyAsync(&host, active, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (int rc = kpt_system_sort_by_key(ctx, sys, 0, 1)) return rc;
    sys->count = host;
    if (active_count) *active_count = host;
    return KPT_OK;
}

int kpt_system_split_energy(kpt_context* ctx, kpt_system* sys, kpt_split_statistics* out) {
    KPT_REQUIRE(ctx && sys, "kpt_system_split_energy: NULL handle");
    kpt_split_statistics stats{};
    if (out) *out = stats;
    if (sys->count == 0 || sys->count >= sys->capacity) return KPT_OK;
    if (int rc = activate(ctx)) return rc;
    const uint64_t n = sys->count;
    const uint64_t blocks = (n + 255) / 256;
    KPT_REQUIRE(blocks <= 1024ull * 1024ull, "kpt_system_split_energy: too many particles");
    KPT_CUDA(sys->flags.reserve(n * sizeof(int)));
    KPT_CUDA(sys->block_counts.reserve(blocks * sizeof(unsigned int)));
    KPT_CUDA(sys->tallies.reserve(8 * sizeof(unsigned long long)));
    KPT_CUDA(cudaMemsetAsync(sys->tallies.ptr, 0, 8 * sizeof(unsigned long long), ctx->stream));
    kpt::LibSplitLaunch L{};
    L.sys = sys->a;
    L.count = n;
    L.capacity = sys->capacity;
    L.rest_mass = sys->props.rest_mass;
    L.speed_of_light = sys->props.speed_of_light;
    L.mc = sys->props.rest_mass * sys->props.speed_of_light;
    L.split_ratio = sys->policy.energy_split_ratio;
    L.log_split_ratio = std::log(sys->policy.energy_split_ratio);
    L.min_child_weight = sys->policy.minimum_child_weight;
    L.flags = sys->flags.as<int>();
    L.block_counts = sys->block_counts.as<unsigned int>();
    L.tallies = sys->tallies.as<unsigned long long>();
    KPT_CUDA(kpt::system_split(L, ctx->stream));
    unsigned long long host[8] = {};
    KPT_CUDA(cudaMemcpyAsync(host, L.tallies, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    // tallies: 0 active, 1 skipped capacity, 2 invalid baseline, 3 min weight, 4 wanted
    const uint64_t available = sys->capacity - n;
    const uint64_t appended = std::min<uint64_t>(host[4], available);
    sys->count = n + appended;
    stats.active_count = host[0];
    stats.split_count = appended;
    stats.skipped_capacity_count = host[1];
    stats.skipped_invalid_baseline_count = host[2];
    stats.skipped_minimum_weight_count = host[3];
    if (out) *out = stats;
    return KPT_OK;
}

int kpt_system_reset_split_baselines(kpt_context* ctx, kpt_system* sys) {
    KPT_REQUIRE(ctx && sys, "kpt_system_reset_split_baselines: NULL handle");
    if (int rc = activate(ctx)) return rc;
    kpt::LibSplitLaunch L{};
    L.sys = sys->a;
    L.count = sys->count;
    L.capacity = sys->capacity;
    L.rest_mass = sys->props.rest_mass;
    L.speed_of_light = sys->props.speed_of_light;
    L.mc = sys->props.rest_mass * sys->props.speed_of_light;
    KPT_CUDA(kpt::system_reset_baselines(L, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_parker_solver_create(kpt_context* ctx, const kpt_grid* grid, const double* basis,
                             int constant_ratio, double courant, kpt_parker_solver** out) {
    KPT_REQUIRE(ctx && grid && basis && out, "kpt_parker_solver_create: NULL argument");
    *out = nullptr;
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_parker_solver> s(new kpt_parker_solver());
    s->ctx = ctx;
    s->device = ctx->device;
    s->grid = grid->g;
    s->points = static_cast<uint64_t>(grid->nx + 4) * static_cast<uint64_t>(grid->ny + 4);
    s->courant = courant;
    KPT_CUDA(cudaMalloc(&s->basis, s->points * kpt::kLibBasisStride * sizeof(double)));
    KPT_CUDA(s->scalars.reserve(64));
    kpt_parker_solver* raw = s.release();
    if (int rc = kpt_parker_solver_set_basis(raw, basis, constant_ratio)) {
        kpt_parker_solver_destroy(raw);
        return rc;
    }
    *out = raw;
    return KPT_OK;
}

int kpt_parker_solver_destroy(kpt_parker_solver* s) {
    if (s == nullptr) return KPT_OK;
    cudaSetDevice(s->device);
    cudaFree(s->basis);
    s->basis_f32.release();
    s->terms.release();
    s->scalars.release();
    s->dt_history.release();
    delete s;
    return KPT_OK;
}

int kpt_parker_solver_set_basis(kpt_parker_solver* s, const double* basis, int constant_ratio) {
    KPT_REQUIRE(s && basis, "kpt_parker_solver_set_basis: NULL argument");
    KPT_CUDA(cudaSetDevice(s->device));
    KPT_CUDA(cudaMemcpy(s->basis, basis, s->points * kpt::kLibBasis * sizeof(double),
                        cudaMemcpyHostToDevice));
    s->constant_ratio = constant_ratio != 0 ? 1 : 0;
    s->basis_f32_valid = false;
    return KPT_OK;
}

int kpt_parker_solver_set_precision(kpt_parker_solver* s, int precision) {
    KPT_REQUIRE(s != nullptr, "kpt_parker_solver_set_precision: NULL handle");
    KPT_REQUIRE(precision == KPT_PRECISION_F64 || precision == KPT_PRECISION_MIXED,
                "kpt_parker_solver_set_precision: precision must be KPT_PRECISION_F64 or "
                "KPT_PRECISION_MIXED");
    s->precision = precision;
    return KPT_OK;
}

int kpt_parker_solver_set_courant(kpt_parker_solver* s, double courant) {
    KPT_REQUIRE(s != nullptr, "kpt_parker_solver_set_courant: NULL handle");
    s->courant = courant;
    return KPT_OK;
}

namespace {

// validate_for_deterministic_step (ParkerSolver.hpp:311-340).
int parker_validate(const kpt_parker_solver* s, const kpt_system* sys) {
    if (!std::isfinite(s->courant) || s->courant <= 0.0) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "ParkerSolver: Courant scale must be positive and finite.");
    }
    if (!std::isfinite(sys->props.charge) || sys->props.charge == 0.0) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "ParkerSolver: Parker drift requires a finite nonzero particle charge.");
    }
    return KPT_OK;
}

int parker_launch(kpt_context* ctx, kpt_parker_solver* s, kpt_system* sys, int advance,
                  int stochastic, uint64_t seed, uint32_t step, double* dt_history,
                  kpt::LibParkerLaunch* out) {
    KPT_CUDA(s->terms.reserve(std::max<uint64_t>(sys->count, 1) * kpt::kLibTermCount *
                              sizeof(double)));
    kpt::LibParkerLaunch& L = *out;
    L = kpt::LibParkerLaunch{};
    L.grid = s->grid;
    L.basis = s->basis;
    if (s->precision == KPT_PRECISION_MIXED) {
        if (!s->basis_f32_valid) {
            KPT_CUDA(s->basis_f32.reserve(s->points * kpt::kLibBasisStrideF32 * sizeof(float)));
            KPT_CUDA(kpt::lib_basis_to_f32(s->basis, kpt::kLibBasisStride,
                                           s->basis_f32.as<float>(), kpt::kLibBasisStrideF32,
                                           kpt::kLibBasis, s->points, ctx->stream));
            s->basis_f32_valid = true;
        }
        L.basis_f32 = s->basis_f32.as<float>();
        L.mixed = 1;
    }
    L.constant_ratio = s->constant_ratio;
    L.sys = sys->a;
    L.count = sys->count;
    L.capacity = sys->capacity;
    L.rest_mass = sys->props.rest_mass;
    L.charge = sys->props.charge;
    L.speed_of_light = sys->props.speed_of_light;
    L.mc = sys->props.rest_mass * sys->props.speed_of_light;
    L.courant = s->courant;
    L.terms = s->terms.as<double>();
    char* sc = static_cast<char*>(s->scalars.ptr);
    L.min_bits = reinterpret_cast<unsigned long long*>(sc);
    L.dt_device_out = reinterpret_cast<double*>(sc + 8);
    L.error = reinterpret_cast<int*>(sc + 16);
    L.error_index = reinterpret_cast<unsigned long long*>(sc + 24);
    L.dt_history = dt_history;
    L.apply_boundary = advance;
    L.advance = advance;
    L.stochastic = stochastic;
    L.capture = 1;
    L.key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    L.frame = step;
    return KPT_OK;
}

int step_finish(kpt_context* ctx, void* scalars, double* dt_out, bool stochastic, bool focus) {
    char host[32];
    KPT_CUDA(cudaMemcpyAsync(host, scalars, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    double dt;
    int error;
    unsigned long long index;
    std::memcpy(&dt, host + 8, sizeof(dt));
    std::memcpy(&error, host + 16, sizeof(error));
    std::memcpy(&index, host + 24, sizeof(index));
    if (dt_out) *dt_out = dt;
    if (error != 0) {
        int code = error;
        if (error == 6) code = focus ? (stochastic ? 16 : 17) : (stochastic ? 6 : 7);
        std::string msg = lib_error_message(code);
        if (error != 6) msg += " (particle " + std::to_string(index) + ")";
        return set_error(KPT_ERROR_INVALID_ARGUMENT, msg);
    }
    return KPT_OK;
}

// Caller normals [4][count] (host) copied to the device for one step.
int upload_noise(kpt_context* ctx, const double* normals, uint64_t count, ScopedBuffer& buf,
                 const double** device) {
    *device = nullptr;
    if (normals == nullptr || count == 0) return KPT_OK;
    KPT_CUDA(buf.reserve(4 * count * sizeof(double)));
    KPT_CUDA(cudaMemcpyAsync(buf.ptr, normals, 4 * count * sizeof(double),
                             cudaMemcpyHostToDevice, ctx->stream));
    *device = buf.as<double>();
    return KPT_OK;
}

int parker_step(kpt_context* ctx, kpt_parker_solver* s, kpt_system* sys, int advance,
                int stochastic, uint64_t seed, uint32_t step, double* dt_out,
                const double* normals = nullptr) {
    KPT_REQUIRE(ctx && s && sys, "ParkerSolver: NULL handle");
    if (int rc = parker_validate(s, sys)) return rc;
    if (int rc = activate(ctx)) return rc;
    kpt::LibParkerLaunch L;
    if (int rc = parker_launch(ctx, s, sys, advance, stochastic, seed, step, nullptr, &L)) {
        return rc;
    }
    ScopedBuffer noise;
    if (int rc = upload_noise(ctx, normals, sys->count, noise, &L.noise)) return rc;
    KPT_CUDA(cudaMemsetAsync(s->scalars.ptr, 0, 32, ctx->stream));
    KPT_CUDA(kpt::lib_parker_step(L, ctx->stream));
    return step_finish(ctx, s->scalars.ptr, dt_out, stochastic != 0, false);
}

}  // namespace

int kpt_parker_compute_time_step(kpt_context* ctx, kpt_parker_solver* s, kpt_system* sys,
                                 double* dt) {
    return parker_step(ctx, s, sys, 0, 0, 0, 0, dt);
}

int kpt_parker_advance_stochastic(kpt_context* ctx, kpt_parker_solver* s, kpt_system* sys,
                                  uint64_t seed, uint32_t step, double* dt_used) {
    return parker_step(ctx, s, sys, 1, 1, seed, step, dt_used);
}

int kpt_parker_advance_deterministic(kpt_context* ctx, kpt_parker_solver* s, kpt_system* sys,
                                     double* dt_used) {
    return parker_step(ctx, s, sys, 1, 0, 0, 0, dt_used);
}

int kpt_parker_advance_with_noise(kpt_context* ctx, kpt_parker_solver* s, kpt_system* sys,
                                  const double* normals, double* dt_used) {
    KPT_REQUIRE(normals != nullptr, "kpt_parker_advance_with_noise: normals is NULL");
    return parker_step(ctx, s, sys, 1, 1, 0, 0, dt_used, normals);
}

int kpt_parker_advance_stochastic_steps(kpt_context* ctx, kpt_parker_solver* s,
                                        kpt_system* sys, uint64_t seed, uint32_t first_step,
                                        uint32_t steps, double* dts) {
    KPT_REQUIRE(ctx && s && sys, "ParkerSolver: NULL handle");
    if (steps == 0) return KPT_OK;
    if (int rc = parker_validate(s, sys)) return rc;
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(s->dt_history.reserve(static_cast<size_t>(steps) * sizeof(double)));
    KPT_CUDA(cudaMemsetAsync(s->scalars.ptr, 0, 32, ctx->stream));
    std::vector<kpt::LibParkerLaunch> launches(steps);
    for (uint32_t k = 0; k < steps; ++k) {
        if (int rc = parker_launch(ctx, s, sys, 1, 1, seed, first_step + k,
                                   s->dt_history.as<double>() + k, &launches[k])) {
            return rc;
        }
    }
    // Record the step sequence once and replay it; a stream that cannot be
    // captured (the legacy default stream) runs the same launches directly.
    cudaGraph_t graph = nullptr;
    bool captured = false;
    if (ctx->stream != nullptr &&
        cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        cudaError_t err = cudaSuccess;
        for (uint32_t k = 0; k < steps && err == cudaSuccess; ++k) {
            err = kpt::lib_parker_step(launches[k], ctx->stream);
        }
        const cudaError_t end = cudaStreamEndCapture(ctx->stream, &graph);
        if ((err != cudaSuccess || end != cudaSuccess) && graph != nullptr) {
            cudaGraphDestroy(graph);  // a capture that failed part-way still returns a graph
        }
        KPT_CUDA(err);
        KPT_CUDA(end);
        captured = true;
    }
    if (captured) {
        cudaGraphExec_t exec = nullptr;
        const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
        if (inst != cudaSuccess) {
            cudaGraphDestroy(graph);
            KPT_CUDA(inst);
        }
        const cudaError_t run = cudaGraphLaunch(exec, ctx->stream);
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        KPT_CUDA(run);
    } else {
        for (uint32_t k = 0; k < steps; ++k) {
            KPT_CUDA(kpt::lib_parker_step(launches[k], ctx->stream));
        }
    }
    if (dts) {
        KPT_CUDA(cudaMemcpyAsync(dts, s->dt_history.ptr, steps * sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    }
    return step_finish(ctx, s->scalars.ptr, nullptr, true, false);
}

}  // extern "C"

// ---- FocusTransportSolver ----------------------------------------------------

namespace {

int focus_validate(const kpt_focus_solver* s, const kpt_system* sys) {
    if (!std::isfinite(s->courant) || s->courant <= 0.0) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "FocusTransportSolver: Courant scale must be positive and finite.");
    }
    if (!std::isfinite(sys->props.charge) || sys->props.charge == 0.0) {
        return set_error(KPT_ERROR_INVALID_ARGUMENT,
                         "FocusTransportSolver: focused drift requires nonzero charge.");
    }
    return KPT_OK;
}

int focus_launch(kpt_focus_solver* s, kpt_system* sys, int advance, int stochastic,
                 uint64_t seed, uint32_t step, double* dt_history, kpt::LibFocusLaunch* out) {
    KPT_CUDA(s->terms.reserve(std::max<uint64_t>(sys->count, 1) * kpt::kFocusTermCount *
                              sizeof(double)));
    kpt::LibFocusLaunch& L = *out;
    L = kpt::LibFocusLaunch{};
    L.grid = s->grid;
    L.basis = s->basis;
    if (s->precision == KPT_PRECISION_MIXED) {
        if (!s->basis_f32_valid) {
            KPT_CUDA(s->basis_f32.reserve(s->points * kpt::kFocusBasisStrideF32 *
                                          sizeof(float)));
            KPT_CUDA(kpt::lib_basis_to_f32(s->basis, kpt::kFocusBasisStride,
                                           s->basis_f32.as<float>(), kpt::kFocusBasisStrideF32,
                                           kpt::kFocusBasis, s->points, s->ctx->stream));
            s->basis_f32_valid = true;
        }
        L.basis_f32 = s->basis_f32.as<float>();
        L.mixed = 1;
    }
    L.constant_ratio = s->constant_ratio;
    L.sys = sys->a;
    L.count = sys->count;
    L.capacity = sys->capacity;
    L.rest_mass = sys->props.rest_mass;
    L.charge = sys->props.charge;
    L.abs_charge = std::fabs(sys->props.charge);
    L.speed_of_light = sys->props.speed_of_light;
    L.mc = sys->props.rest_mass * sys->props.speed_of_light;
    const kpt_scattering_parameters& sc = s->scattering;
    L.gk = sc.spectral_index;
    L.h0 = sc.h0;
    // pitch_angle_spectrum_normalization (LegencyModel.hpp:539-552)
    L.qlt_norm = sc.spectral_index * std::sin(3.141592653589793238462643383279502884 /
                                              sc.spectral_index) /
                 3.141592653589793238462643383279502884;
    L.min_b = sc.minimum_magnetic_field_magnitude;
    L.min_sigma2 = sc.minimum_sigma2;
    L.min_lc = sc.minimum_correlation_length;
    L.min_speed = sc.minimum_speed;
    L.max_mu = s->max_mu;
    L.courant = s->courant;
    L.terms = s->terms.as<double>();
    char* scp = static_cast<char*>(s->scalars.ptr);
    L.min_bits = reinterpret_cast<unsigned long long*>(scp);
    L.dt_device_out = reinterpret_cast<double*>(scp + 8);
    L.error = reinterpret_cast<int*>(scp + 16);
    L.error_index = reinterpret_cast<unsigned long long*>(scp + 24);
    L.dt_history = dt_history;
    L.apply_boundary = advance;
    L.advance = advance;
    L.stochastic = stochastic;
    L.capture = 1;
    L.key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    L.frame = step;
    return KPT_OK;
}

int focus_step(kpt_context* ctx, kpt_focus_solver* s, kpt_system* sys, int advance,
               int stochastic, uint64_t seed, uint32_t step, double* dt_out,
               const double* normals = nullptr) {
    KPT_REQUIRE(ctx && s && sys, "FocusTransportSolver: NULL handle");
    if (int rc = focus_validate(s, sys)) return rc;
    if (int rc = activate(ctx)) return rc;
    kpt::LibFocusLaunch L;
    if (int rc = focus_launch(s, sys, advance, stochastic, seed, step, nullptr, &L)) return rc;
    ScopedBuffer noise;
    if (int rc = upload_noise(ctx, normals, sys->count, noise, &L.noise)) return rc;
    KPT_CUDA(cudaMemsetAsync(s->scalars.ptr, 0, 32, ctx->stream));
    KPT_CUDA(kpt::lib_focus_step(L, ctx->stream));
    return step_finish(ctx, s->scalars.ptr, dt_out, stochastic != 0, true);
}

}  // namespace

// The solver without its basis: validated scattering parameters, the
// device basis allocated.
static int focus_solver_allocate(kpt_context* ctx, const kpt_grid* grid, double courant,
                                 const kpt_scattering_parameters* scattering,
                                 kpt_focus_solver** out) {
    kpt_scattering_parameters sc{5.0 / 3.0, 1.0e-6, 0.0, 0.0, 0.0, 0.0};
    if (scattering != nullptr) sc = *scattering;
    // PitchAngleScatteringParameters::validate (LegencyModel.hpp:205-221)
    KPT_REQUIRE(std::isfinite(sc.spectral_index) && sc.spectral_index > 1.0 &&
                    std::isfinite(sc.h0) && sc.h0 > 0.0 &&
                    std::isfinite(sc.minimum_magnetic_field_magnitude) &&
                    sc.minimum_magnetic_field_magnitude >= 0.0 &&
                    std::isfinite(sc.minimum_sigma2) && sc.minimum_sigma2 >= 0.0 &&
                    std::isfinite(sc.minimum_correlation_length) &&
                    sc.minimum_correlation_length >= 0.0 && std::isfinite(sc.minimum_speed) &&
                    sc.minimum_speed >= 0.0,
                "LegencyModel::PitchAngleScatteringParameters: coefficients and floors must be "
                "finite, with spectral_index > 1 and resonance_regularization_h0 > 0.");
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_focus_solver> s(new kpt_focus_solver());
    s->ctx = ctx;
    s->device = ctx->device;
    s->grid = grid->g;
    s->points = static_cast<uint64_t>(grid->nx + 4) * static_cast<uint64_t>(grid->ny + 4);
    s->courant = courant;
    s->scattering = sc;
    KPT_CUDA(cudaMalloc(&s->basis, s->points * kpt::kFocusBasisStride * sizeof(double)));
    KPT_CUDA(cudaMemset(s->basis, 0, s->points * kpt::kFocusBasisStride * sizeof(double)));
    KPT_CUDA(s->scalars.reserve(64));
    *out = s.release();
    return KPT_OK;
}

extern "C" {

int kpt_focus_solver_create(kpt_context* ctx, const kpt_grid* grid, const double* basis,
                            int constant_ratio, double courant,
                            const kpt_scattering_parameters* scattering,
                            kpt_focus_solver** out) {
    KPT_REQUIRE(ctx && grid && basis && out, "kpt_focus_solver_create: NULL argument");
    *out = nullptr;
    kpt_focus_solver* raw = nullptr;
    if (int rc = focus_solver_allocate(ctx, grid, courant, scattering, &raw)) return rc;
    if (int rc = kpt_focus_solver_set_basis(raw, basis, constant_ratio)) {
        kpt_focus_solver_destroy(raw);
        return rc;
    }
    *out = raw;
    return KPT_OK;
}

int kpt_focus_solver_destroy(kpt_focus_solver* s) {
    if (s == nullptr) return KPT_OK;
    cudaSetDevice(s->device);
    cudaFree(s->basis);
    s->basis_f32.release();
    s->terms.release();
    s->scalars.release();
    s->dt_history.release();
    delete s;
    return KPT_OK;
}

int kpt_focus_solver_set_basis(kpt_focus_solver* s, const double* basis, int constant_ratio) {
    KPT_REQUIRE(s && basis, "kpt_focus_solver_set_basis: NULL argument");
    KPT_CUDA(cudaSetDevice(s->device));
    // rows of 27 values to the 28-value stride
    KPT_CUDA(cudaMemcpy2D(s->basis, kpt::kFocusBasisStride * sizeof(double), basis,
                          kpt::kFocusBasis * sizeof(double), kpt::kFocusBasis * sizeof(double),
                          s->points, cudaMemcpyHostToDevice));
    s->constant_ratio = constant_ratio != 0 ? 1 : 0;
    s->basis_f32_valid = false;
    return KPT_OK;
}

int kpt_focus_solver_set_precision(kpt_focus_solver* s, int precision) {
    KPT_REQUIRE(s != nullptr, "kpt_focus_solver_set_precision: NULL handle");
    KPT_REQUIRE(precision == KPT_PRECISION_F64 || precision == KPT_PRECISION_MIXED,
                "kpt_focus_solver_set_precision: precision must be KPT_PRECISION_F64 or "
                "KPT_PRECISION_MIXED");
    s->precision = precision;
    return KPT_OK;
}

int kpt_focus_solver_set_courant(kpt_focus_solver* s, double courant) {
    KPT_REQUIRE(s != nullptr, "kpt_focus_solver_set_courant: NULL handle");
    s->courant = courant;
    return KPT_OK;
}

int kpt_focus_solver_set_maximum_mu(kpt_focus_solver* s, double maximum_mu) {
    KPT_REQUIRE(s != nullptr, "kpt_focus_solver_set_maximum_mu: NULL handle");
    KPT_REQUIRE(std::isfinite(maximum_mu) && maximum_mu > 0.0 && maximum_mu <= 1.0,
                "FocusTransportSolver: maximum |mu| must satisfy 0 < value <= 1.");
    s->max_mu = maximum_mu;
    return KPT_OK;
}

int kpt_focus_compute_time_step(kpt_context* ctx, kpt_focus_solver* s, kpt_system* sys,
                                double* dt) {
    return focus_step(ctx, s, sys, 0, 0, 0, 0, dt);
}

int kpt_focus_advance_stochastic(kpt_context* ctx, kpt_focus_solver* s, kpt_system* sys,
                                 uint64_t seed, uint32_t step, double* dt_used) {
    return focus_step(ctx, s, sys, 1, 1, seed, step, dt_used);
}

int kpt_focus_advance_deterministic(kpt_context* ctx, kpt_focus_solver* s, kpt_system* sys,
                                    double* dt_used) {
    return focus_step(ctx, s, sys, 1, 0, 0, 0, dt_used);
}

int kpt_focus_advance_with_noise(kpt_context* ctx, kpt_focus_solver* s, kpt_system* sys,
                                 const double* normals, double* dt_used) {
    KPT_REQUIRE(normals != nullptr, "kpt_focus_advance_with_noise: normals is NULL");
    return focus_step(ctx, s, sys, 1, 1, 0, 0, dt_used, normals);
}

int kpt_focus_advance_stochastic_steps(kpt_context* ctx, kpt_focus_solver* s, kpt_system* sys,
                                       uint64_t seed, uint32_t first_step, uint32_t steps,
                                       double* dts) {
    KPT_REQUIRE(ctx && s && sys, "FocusTransportSolver: NULL handle");
    if (steps == 0) return KPT_OK;
    if (int rc = focus_validate(s, sys)) return rc;
    if (int rc = activate(ctx)) return rc;
    KPT_CUDA(s->dt_history.reserve(static_cast<size_t>(steps) * sizeof(double)));
    KPT_CUDA(cudaMemsetAsync(s->scalars.ptr, 0, 32, ctx->stream));
    std::vector<kpt::LibFocusLaunch> launches(steps);
    for (uint32_t k = 0; k < steps; ++k) {
        if (int rc = focus_launch(s, sys, 1, 1, seed, first_step + k,
                                  s->dt_history.as<double>() + k, &launches[k])) {
            return rc;
        }
    }
    cudaGraph_t graph = nullptr;
    bool captured = false;
    if (ctx->stream != nullptr &&
        cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        cudaError_t err = cudaSuccess;
        for (uint32_t k = 0; k < steps && err == cudaSuccess; ++k) {
            err = kpt::lib_focus_step(launches[k], ctx->stream);
        }
        const cudaError_t end = cudaStreamEndCapture(ctx->stream, &graph);
        if ((err != cudaSuccess || end != cudaSuccess) && graph != nullptr) {
            cudaGraphDestroy(graph);  // a capture that failed part-way still returns a graph
        }
        KPT_CUDA(err);
        KPT_CUDA(end);
        captured = true;
    }
    if (captured) {
        cudaGraphExec_t exec = nullptr;
        const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
        if (inst != cudaSuccess) {
            cudaGraphDestroy(graph);
            KPT_CUDA(inst);
        }
        const cudaError_t run = cudaGraphLaunch(exec, ctx->stream);
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        KPT_CUDA(run);
    } else {
        for (uint32_t k = 0; k < steps; ++k) {
            KPT_CUDA(kpt::lib_focus_step(launches[k], ctx->stream));
        }
    }
    if (dts) {
        KPT_CUDA(cudaMemcpyAsync(dts, s->dt_history.ptr, steps * sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    }
    return step_finish(ctx, s->scalars.ptr, nullptr, true, true);
}

}  // extern "C"

// ====================================================================
// Parker coefficient precompute on the library grid
// ====================================================================

namespace {

// DiffusionModelParameters::validate (LegencyModel.hpp:95-116),
// ParticleProperties::validate (ParticleSystem.hpp:155-165) and the
// floors' checks of the curl and divergence builders.
int validate_coefficient_inputs(const kpt_turbulence* t, const kpt_particle_properties* pr,
                                const kpt_diffusion_parameters* p) {
    KPT_REQUIRE(std::isfinite(p->parallel_prefactor) && p->parallel_prefactor > 0.0 &&
                    std::isfinite(p->perpendicular_prefactor) &&
                    p->perpendicular_prefactor > 0.0 &&
                    std::isfinite(p->perpendicular_parallel_ratio) &&
                    p->perpendicular_parallel_ratio >= 0.0 &&
                    std::isfinite(p->minimum_magnetic_field_magnitude) &&
                    p->minimum_magnetic_field_magnitude >= 0.0 &&
                    std::isfinite(p->minimum_solar_wind_speed) &&
                    p->minimum_solar_wind_speed >= 0.0 && std::isfinite(p->minimum_sigma2) &&
                    p->minimum_sigma2 >= 0.0,
                "LegencyModel::DiffusionModelParameters: coefficients and floors must be "
                "finite positive or non-negative values.");
    KPT_REQUIRE(p->perpendicular_model == 0 || p->perpendicular_model == 1,
                "kpt_diffusion_parameters: unknown perpendicular model");
    KPT_REQUIRE(p->perpendicular_model == 0 || p->perpendicular_parallel_ratio > 0.0,
                "LegencyModel::DiffusionModelParameters: constant perpendicular ratio must be "
                "positive when selected.");
    KPT_REQUIRE(p->ghost_fill_mode == 0 || p->ghost_fill_mode == 1,
                "kpt_diffusion_parameters: unknown ghost fill mode");
    KPT_REQUIRE(std::isfinite(pr->rest_mass) && pr->rest_mass > 0.0 &&
                    std::isfinite(pr->charge) && std::isfinite(pr->speed_of_light) &&
                    pr->speed_of_light > 0.0 && std::isfinite(pr->energy_scale_erg) &&
                    pr->energy_scale_erg > 0.0,
                "ParticleProperties: rest mass and speed of light must be positive finite "
                "dimensionless values, charge must be finite, and the energy scale must be "
                "positive and finite.");
    KPT_REQUIRE(std::isfinite(p->minimum_magnetic_field_squared_for_drift) &&
                    p->minimum_magnetic_field_squared_for_drift >= 0.0,
                "ParkerCoefficient: magnetic field floor must be finite and non-negative.");
    KPT_REQUIRE(t->storage == 0 || t->storage == 1, "kpt_turbulence: unknown storage");
    if (t->storage == 0) {
        const double lc = t->lc > 0.0 ? t->lc : t->lslab;
        KPT_REQUIRE(std::isfinite(t->sigma2) && t->sigma2 > 0.0 && std::isfinite(t->l2d) &&
                        t->l2d > 0.0 && std::isfinite(t->lslab) && t->lslab > 0.0 &&
                        std::isfinite(lc) && lc > 0.0,
                    "TurbulencePropertyModel: coefficients must be positive finite values.");
    } else {
        KPT_REQUIRE(t->sigma2_field && t->l2d_field && t->lc_field,
                    "kpt_turbulence: field storage needs sigma2, l2d and lc fields");
    }
    return KPT_OK;
}

const char* coefficient_error_message(int code) {
    switch (code) {
        case 10: return "FieldOperator: direction is undefined at zero magnitude.";
        case 11: return "FocusCoefficient: ln |B| requires a positive magnetic field.";
        case 12: return "FocusCoefficient: focused drift requires |B| > 0.";
        case 20: return "ParkerCoefficient: curl(B/B^2) is undefined where B^2 <= 0.";
        case 21: return "LegencyModel: gyrofrequency requires |B| > 0.";
        case 22: return "LegencyModel: kappa_parallel requires positive Vsw, Lc, omega, and sigma2.";
        case 23:
            return "LegencyModel: kappa_perpendicular requires positive Vsw, L2D, sigma2_2D, "
                   "and kappa_parallel.";
        case 24:
            return "LegencyModel: constant-ratio kappa_perpendicular requires positive "
                   "kappa_parallel and ratio.";
        case 26:
            return "ParkerCoefficient: diffusion tensor direction is undefined where |B| <= 0.";
    }
    return "ParkerCoefficient: coefficient precompute failed";
}

// Builds the packed basis into `packed` (device): the Parker basis
// (kLibBasisStride per point) or, with focused set, the focused basis
// (kFocusBasisStride per point) from B, V and dV/dt (NULL = zero).
int build_coefficients(kpt_context* ctx, const kpt_grid* grid, const double* b, const double* v,
                       const double* dvdt, const kpt_turbulence* t,
                       const kpt_particle_properties* pr, const kpt_diffusion_parameters* p,
                       bool focused, double builder_floor, double* packed) {
    if (int rc = validate_coefficient_inputs(t, pr, p)) return rc;
    if (focused) {
        KPT_REQUIRE(std::isfinite(builder_floor) && builder_floor >= 0.0,
                    "FocusCoefficient: magnetic-field magnitude floor must be finite and "
                    "non-negative.");
    }
    const uint64_t points = static_cast<uint64_t>(grid->nx + 4) * (grid->ny + 4);
    const int fields = t->storage == 1 ? 3 : 0;
    const int vectors = focused && dvdt != nullptr ? 3 : 2;
    ScopedBuffer inputs;
    const size_t vec_bytes = points * 3 * sizeof(double);
    const size_t scratch_bytes = focused ? points * 8 * sizeof(double) : 0;
    KPT_CUDA(inputs.reserve(vectors * vec_bytes + fields * points * sizeof(double) +
                            scratch_bytes + 64));
    char* base = static_cast<char*>(inputs.ptr);
    double* db = reinterpret_cast<double*>(base);
    double* dv = reinterpret_cast<double*>(base + vec_bytes);
    double* ddvdt = vectors == 3 ? reinterpret_cast<double*>(base + 2 * vec_bytes) : nullptr;
    double* dt = reinterpret_cast<double*>(base + vectors * vec_bytes);
    double* dscratch = reinterpret_cast<double*>(base + vectors * vec_bytes +
                                                 fields * points * sizeof(double));
    int* err = reinterpret_cast<int*>(base + vectors * vec_bytes +
                                      fields * points * sizeof(double) + scratch_bytes);
    KPT_CUDA(cudaMemcpyAsync(db, b, vec_bytes, cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(dv, v, vec_bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (ddvdt != nullptr) {
        KPT_CUDA(cudaMemcpyAsync(ddvdt, dvdt, vec_bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    if (fields) {
        const double* src[3] = {t->sigma2_field, t->l2d_field, t->lc_field};
        for (int k = 0; k < 3; ++k) {
            KPT_CUDA(cudaMemcpyAsync(dt + k * points, src[k], points * sizeof(double),
                                     cudaMemcpyHostToDevice, ctx->stream));
        }
    }
    const int no_error = kpt::parker_coefficients_no_error();
    KPT_CUDA(cudaMemcpyAsync(err, &no_error, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    kpt::CoefLaunch L{};
    L.grid = grid->g;
    L.b = db;
    L.v = dv;
    L.turbulence_fields = fields ? 1 : 0;
    L.sigma2 = t->sigma2;
    L.l2d = t->l2d;
    L.lc = t->lc > 0.0 ? t->lc : t->lslab;
    L.sigma2_field = fields ? dt : nullptr;
    L.l2d_field = fields ? dt + points : nullptr;
    L.lc_field = fields ? dt + 2 * points : nullptr;
    L.abs_charge = std::fabs(pr->charge);
    L.rest_mass = pr->rest_mass;
    L.speed_of_light = pr->speed_of_light;
    L.constant_ratio = p->perpendicular_model == 1 ? 1 : 0;
    L.parallel_prefactor = p->parallel_prefactor;
    L.perpendicular_prefactor = p->perpendicular_prefactor;
    L.ratio = p->perpendicular_parallel_ratio;
    L.min_b = p->minimum_magnetic_field_magnitude;
    L.min_vsw = p->minimum_solar_wind_speed;
    L.min_sigma2 = p->minimum_sigma2;
    L.drift_floor = p->minimum_magnetic_field_squared_for_drift;
    L.ghost_mode = p->ghost_fill_mode;
    L.packed = packed;
    L.error = err;
    if (focused) {
        L.stride = kpt::kFocusBasisStride;
        L.kpar_slot = 19;
        L.kperp_slot = 20;
        L.dvdt = ddvdt;
        L.direction_floor = builder_floor;
        L.scratch = dscratch;
        KPT_CUDA(kpt::focus_coefficients(L, ctx->stream));
    } else {
        L.stride = kpt::kLibBasisStride;
        L.kpar_slot = 15;
        L.kperp_slot = 16;
        KPT_CUDA(kpt::parker_coefficients(L, ctx->stream));
    }
    int code = no_error;
    KPT_CUDA(cudaMemcpyAsync(&code, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    KPT_REQUIRE(code == no_error, coefficient_error_message(code));
    return KPT_OK;
}

}  // namespace

extern "C" {

void kpt_default_diffusion_parameters(kpt_diffusion_parameters* out) {
    if (out == nullptr) return;
    *out = kpt_diffusion_parameters{};
    out->perpendicular_model = 0;
    out->ghost_fill_mode = 0;
    out->parallel_prefactor = 1.622;
    out->perpendicular_prefactor = 0.198;
}

int kpt_parker_coefficients(kpt_context* ctx, const kpt_grid* grid, const double* b,
                            const double* v, const kpt_turbulence* turbulence,
                            const kpt_particle_properties* properties,
                            const kpt_diffusion_parameters* parameters, double* packed) {
    KPT_REQUIRE(ctx && grid && b && v && turbulence && properties && parameters && packed,
                "kpt_parker_coefficients: NULL argument");
    if (int rc = activate(ctx)) return rc;
    const uint64_t points = static_cast<uint64_t>(grid->nx + 4) * (grid->ny + 4);
    ScopedBuffer out;
    KPT_CUDA(out.reserve(points * kpt::kLibBasisStride * sizeof(double)));
    if (int rc = build_coefficients(ctx, grid, b, v, nullptr, turbulence, properties, parameters,
                                    false, 0.0, out.as<double>())) {
        return rc;
    }
    KPT_CUDA(cudaMemcpy(packed, out.ptr, points * kpt::kLibBasisStride * sizeof(double),
                        cudaMemcpyDeviceToHost));
    return KPT_OK;
}

int kpt_focus_coefficients(kpt_context* ctx, const kpt_grid* grid, const double* b,
                           const double* v, const double* dvdt, const kpt_turbulence* turbulence,
                           const kpt_particle_properties* properties,
                           const kpt_diffusion_parameters* parameters,
                           double minimum_magnetic_field_magnitude, double* packed) {
    KPT_REQUIRE(ctx && grid && b && v && turbulence && properties && parameters && packed,
                "kpt_focus_coefficients: NULL argument");
    if (int rc = activate(ctx)) return rc;
    const uint64_t points = static_cast<uint64_t>(grid->nx + 4) * (grid->ny + 4);
    ScopedBuffer out;
    KPT_CUDA(out.reserve(points * kpt::kFocusBasisStride * sizeof(double)));
    if (int rc = build_coefficients(ctx, grid, b, v, dvdt, turbulence, properties, parameters,
                                    true, minimum_magnetic_field_magnitude, out.as<double>())) {
        return rc;
    }
    // device rows of kFocusBasisStride -> host rows of kFocusBasis
    KPT_CUDA(cudaMemcpy2D(packed, kpt::kFocusBasis * sizeof(double), out.ptr,
                          kpt::kFocusBasisStride * sizeof(double),
                          kpt::kFocusBasis * sizeof(double), points, cudaMemcpyDeviceToHost));
    return KPT_OK;
}

int kpt_focus_solver_create_from_fields(kpt_context* ctx, const kpt_grid* grid, const double* b,
                                        const double* v, const double* dvdt,
                                        const kpt_turbulence* turbulence,
                                        const kpt_particle_properties* properties,
                                        const kpt_diffusion_parameters* parameters,
                                        double minimum_magnetic_field_magnitude, double courant,
                                        const kpt_scattering_parameters* scattering,
                                        kpt_focus_solver** out) {
    KPT_REQUIRE(ctx && grid && b && v && turbulence && properties && parameters && out,
                "kpt_focus_solver_create_from_fields: NULL argument");
    *out = nullptr;
    kpt_focus_solver* raw = nullptr;
    if (int rc = focus_solver_allocate(ctx, grid, courant, scattering, &raw)) return rc;
    raw->constant_ratio = parameters->perpendicular_model == 1 ? 1 : 0;
    if (int rc = build_coefficients(ctx, grid, b, v, dvdt, turbulence, properties, parameters,
                                    true, minimum_magnetic_field_magnitude, raw->basis)) {
        kpt_focus_solver_destroy(raw);
        return rc;
    }
    *out = raw;
    return KPT_OK;
}

int kpt_parker_solver_create_from_fields(kpt_context* ctx, const kpt_grid* grid, const double* b,
                                         const double* v, const kpt_turbulence* turbulence,
                                         const kpt_particle_properties* properties,
                                         const kpt_diffusion_parameters* parameters,
                                         double courant, kpt_parker_solver** out) {
    KPT_REQUIRE(ctx && grid && b && v && turbulence && properties && parameters && out,
                "kpt_parker_solver_create_from_fields: NULL argument");
    *out = nullptr;
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_parker_solver> s(new kpt_parker_solver());
    s->ctx = ctx;
    s->device = ctx->device;
    s->grid = grid->g;
    s->points = static_cast<uint64_t>(grid->nx + 4) * static_cast<uint64_t>(grid->ny + 4);
    s->courant = courant;
    s->constant_ratio = parameters->perpendicular_model == 1 ? 1 : 0;
    KPT_CUDA(cudaMalloc(&s->basis, s->points * kpt::kLibBasisStride * sizeof(double)));
    KPT_CUDA(s->scalars.reserve(64));
    kpt_parker_solver* raw = s.release();
    if (int rc = build_coefficients(ctx, grid, b, v, nullptr, turbulence, properties, parameters,
                                    false, 0.0, raw->basis)) {
        kpt_parker_solver_destroy(raw);
        return rc;
    }
    *out = raw;
    return KPT_OK;
}

}  // extern "C"

// ====================================================================
// ParticleGenerator: injection and recycling on the library grid
// ====================================================================

struct kpt_lib_field {
    kpt_context* ctx = nullptr;
    int device = 0;
    kpt::LibGrid grid{};
    int components = 0;
    int centering[2] = {0, 0};
    int ext[2] = {0, 0};
    uint64_t points = 0;
    double* values = nullptr;
    ~kpt_lib_field() {
        if (values) cudaFree(values);
    }
};

struct kpt_candidates {
    kpt_context* ctx = nullptr;
    int device = 0;
    kpt::LibGrid grid{};
    kpt::GenCandidates view{};
    ScopedBuffer indices, cumulative;
};

namespace {

kpt::GenField gen_field_view(const kpt_lib_field* f) {
    kpt::GenField v{};
    v.values = f->values;
    v.components = f->components;
    for (int dim = 0; dim < 2; ++dim) {
        v.centering[dim] = f->centering[dim];
        v.ext[dim] = f->ext[dim];
    }
    return v;
}

// AxisAlignedParticleRegion::validate (ParticleGenerator.hpp:27-36).
int validate_region(const kpt_region* r) {
    for (int dim = 0; dim < 2; ++dim) {
        KPT_REQUIRE(std::isfinite(r->lower[dim]) && std::isfinite(r->upper[dim]) &&
                        r->upper[dim] > r->lower[dim],
                    "AxisAlignedParticleRegion: bounds must be finite and ascending.");
    }
    return KPT_OK;
}

// validate_particle_injection_kinematics (ParticleGenerator.hpp:89-103).
int validate_kinematics(const kpt_injection_kinematics* k) {
    KPT_REQUIRE(std::isfinite(k->mu) && std::isfinite(k->weight) && k->weight > 0.0,
                "ParticleInjectionKinematics: mu must be finite and weight must be positive.");
    KPT_REQUIRE(std::isfinite(k->momentum_magnitude) && k->momentum_magnitude >= 0.0,
                "ParticleInjectionKinematics: momentum magnitude must be finite and "
                "non-negative.");
    KPT_REQUIRE(k->status >= 0 && k->status <= 2,
                "ParticleInjectionKinematics: status must be a ParticleStatus value");
    return KPT_OK;
}

// validate_particle_injection_plan (ParticleGenerator.hpp:860-881).
int validate_plan(const kpt_system* sys, const kpt_injection_plan* plan) {
    KPT_REQUIRE(plan->max_attempts > 0, "ParticleInjectionPlan: max_attempts must be positive.");
    KPT_REQUIRE(plan->first_particle_index <= sys->count,
                "ParticleInjectionPlan: first index is out of range.");
    KPT_REQUIRE(plan->first_particle_index <= sys->capacity,
                "ParticleInjectionPlan: first index exceeds capacity.");
    KPT_REQUIRE(plan->particle_count <= sys->capacity - plan->first_particle_index,
                "ParticleInjectionPlan: requested range exceeds capacity.");
    return KPT_OK;
}

int gen_common(kpt_context* ctx, kpt_system* sys, kpt::GenLaunch& L, uint64_t seed,
               uint32_t frame, const kpt_injection_kinematics* k) {
    L.sys = sys->a;
    L.momentum = k->momentum_magnitude;
    L.mu = k->mu;
    L.weight = k->weight;
    L.status = k->status;
    L.rest_mass = sys->props.rest_mass;
    L.speed_of_light = sys->props.speed_of_light;
    L.mc = sys->props.rest_mass * sys->props.speed_of_light;
    L.key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    L.frame = frame;
    (void)ctx;
    return KPT_OK;
}

int gen_predicate(const kpt_field_predicate* p, const kpt_grid* grid_or_null,
                  kpt::GenPredicate* out) {
    *out = kpt::GenPredicate{};
    if (p == nullptr) return KPT_OK;
    KPT_REQUIRE(p->field != nullptr, "kpt_field_predicate: field is NULL");
    KPT_REQUIRE(p->component >= 0 && p->component < p->field->components,
                "FieldThresholdParticlePredicate: component index is out of range.");
    KPT_REQUIRE(p->comparison >= 0 && p->comparison <= 5,
                "kpt_field_predicate: unknown comparison");
    KPT_REQUIRE(p->domain == 0 || p->domain == 1, "kpt_field_predicate: unknown domain");
    (void)grid_or_null;
    out->enabled = 1;
    out->field = gen_field_view(p->field);
    out->threshold = p->threshold;
    out->comparison = p->comparison;
    out->component = p->component;
    out->domain = p->domain;
    return KPT_OK;
}

int gen_finish(kpt_context* ctx, kpt_system* sys, kpt::GenLaunch& L, uint64_t* recycled) {
    DeviceBuffer& counter = sys->scalars;
    if (L.recycle) {
        KPT_CUDA(counter.reserve(64));
        L.recycled = counter.as<unsigned long long>();
    }
    KPT_CUDA(kpt::generator_run(L, ctx->stream));
    if (L.recycle) {
        unsigned long long n = 0;
        KPT_CUDA(cudaMemcpyAsync(&n, L.recycled, sizeof(n), cudaMemcpyDeviceToHost,
                                 ctx->stream));
        KPT_CUDA(cudaStreamSynchronize(ctx->stream));
        if (recycled) *recycled = n;
    } else {
        // commit_particle_range (ParticleSystem.hpp:474-491)
        const uint64_t end = L.first_index + L.count;
        if (L.count > 0 && end > sys->count) sys->count = end;
    }
    return KPT_OK;
}

}  // namespace

extern "C" {

int kpt_lib_field_create(kpt_context* ctx, const kpt_grid* grid, int32_t components,
                         const int32_t centering[2], const double* values,
                         kpt_lib_field** out) {
    KPT_REQUIRE(ctx && grid && centering && values && out, "kpt_lib_field_create: NULL argument");
    *out = nullptr;
    KPT_REQUIRE(components > 0 && components <= 64,
                "kpt_lib_field_create: components must be in [1, 64]");
    KPT_REQUIRE((centering[0] == 0 || centering[0] == 1) &&
                    (centering[1] == 0 || centering[1] == 1),
                "kpt_lib_field_create: centering must be 0 (cell) or 1 (face)");
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_lib_field> f(new kpt_lib_field());
    f->ctx = ctx;
    f->device = ctx->device;
    f->grid = grid->g;
    f->components = components;
    const int n[2] = {grid->nx, grid->ny};
    f->points = 1;
    for (int dim = 0; dim < 2; ++dim) {
        f->centering[dim] = centering[dim];
        // Field::compute_extents: ghosted cells n+4, faces n+5
        f->ext[dim] = n[dim] + 4 + (centering[dim] != 0 ? 1 : 0);
        f->points *= static_cast<uint64_t>(f->ext[dim]);
    }
    const size_t bytes = f->points * static_cast<size_t>(components) * sizeof(double);
    KPT_CUDA(cudaMalloc(&f->values, bytes));
    KPT_CUDA(cudaMemcpyAsync(f->values, values, bytes, cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = f.release();
    return KPT_OK;
}

int kpt_lib_field_destroy(kpt_lib_field* field) {
    delete field;
    return KPT_OK;
}

int kpt_lib_field_points(const kpt_lib_field* field, uint64_t* points) {
    KPT_REQUIRE(field && points, "kpt_lib_field_points: NULL argument");
    *points = field->points;
    return KPT_OK;
}

int kpt_region_from_grid(const kpt_grid* grid, int32_t domain, kpt_region* out) {
    KPT_REQUIRE(grid && out, "kpt_region_from_grid: NULL argument");
    KPT_REQUIRE(domain == 0 || domain == 1, "kpt_region_from_grid: unknown domain");
    for (int dim = 0; dim < 2; ++dim) {
        const kpt::LibAxis& a = grid->g.axis[dim];
        out->lower[dim] = domain != 0 ? a.ghost_lower : a.lower;
        out->upper[dim] = domain != 0 ? a.ghost_upper : a.upper;
    }
    return validate_region(out);
}

int kpt_candidates_from_field(kpt_context* ctx, const kpt_lib_field* field,
                              const kpt_region* region, double threshold, int32_t comparison,
                              int32_t component, int32_t domain, kpt_candidates** out) {
    KPT_REQUIRE(ctx && field && out, "kpt_candidates_from_field: NULL argument");
    *out = nullptr;
    KPT_REQUIRE(component >= 0 && component < field->components,
                "Field particle injection: component index is out of range.");
    KPT_REQUIRE(comparison >= 0 && comparison <= 5,
                "kpt_candidates_from_field: unknown comparison");
    KPT_REQUIRE(domain == 0 || domain == 1, "kpt_candidates_from_field: unknown domain");
    kpt_region whole{};
    if (region == nullptr) {
        for (int dim = 0; dim < 2; ++dim) {
            const kpt::LibAxis& a = field->grid.axis[dim];
            whole.lower[dim] = domain != 0 ? a.ghost_lower : a.lower;
            whole.upper[dim] = domain != 0 ? a.ghost_upper : a.upper;
        }
        region = &whole;
    }
    if (int rc = validate_region(region)) return rc;
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_candidates> c(new kpt_candidates());
    c->ctx = ctx;
    c->device = ctx->device;
    c->grid = field->grid;
    const uint64_t points = field->points;
    KPT_CUDA(c->indices.reserve(points * sizeof(uint64_t)));
    ScopedBuffer block_counts, scratch;
    const uint64_t blocks = (points + 255) / 256;
    KPT_CUDA(block_counts.reserve(blocks * sizeof(unsigned int) + sizeof(unsigned long long) * 2));
    kpt::GenCandidateBuild B{};
    B.grid = field->grid;
    B.field = gen_field_view(field);
    for (int dim = 0; dim < 2; ++dim) {
        B.region_lo[dim] = region->lower[dim];
        B.region_hi[dim] = region->upper[dim];
    }
    B.threshold = threshold;
    B.comparison = comparison;
    B.component = component;
    B.domain = domain;
    B.points = points;
    B.indices = c->indices.as<uint64_t>();
    B.block_counts = block_counts.as<unsigned int>();
    B.count_out = reinterpret_cast<unsigned long long*>(
        static_cast<char*>(block_counts.ptr) +
        ((blocks * sizeof(unsigned int) + 7) / 8) * 8);
    KPT_CUDA(kpt::generator_field_candidates(B, ctx->stream));
    unsigned long long count = 0;
    KPT_CUDA(cudaMemcpyAsync(&count, B.count_out, sizeof(count), cudaMemcpyDeviceToHost,
                             ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    double total = 0.0;
    if (count > 0) {
        KPT_CUDA(c->cumulative.reserve(count * sizeof(double)));
        KPT_CUDA(scratch.reserve(kpt::generator_scan_scratch(count) * sizeof(double)));
        B.cumulative = c->cumulative.as<double>();
        B.block_sums = scratch.as<double>();
        KPT_CUDA(kpt::generator_field_weights(B, count, ctx->stream));
        KPT_CUDA(cudaMemcpyAsync(&total, B.cumulative + (count - 1), sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
        KPT_CUDA(cudaStreamSynchronize(ctx->stream));
        KPT_REQUIRE(std::isfinite(total) && total > 0.0,
                    "Field particle candidate set: total physical volume must be positive.");
    }
    kpt::GenCandidates& v = c->view;
    v.kind = 0;
    v.indices = c->indices.as<uint64_t>();
    v.cumulative = count > 0 ? c->cumulative.as<double>() : nullptr;
    v.count = count;
    v.total = total;
    v.field = B.field;
    v.field.values = nullptr;  // the candidate set needs the layout, not the values
    *out = c.release();
    return KPT_OK;
}

int kpt_candidates_from_grid(kpt_context* ctx, const kpt_grid* grid, int32_t domain,
                             kpt_candidates** out) {
    KPT_REQUIRE(ctx && grid && out, "kpt_candidates_from_grid: NULL argument");
    *out = nullptr;
    KPT_REQUIRE(domain == 0 || domain == 1, "kpt_candidates_from_grid: unknown domain");
    if (int rc = activate(ctx)) return rc;
    std::unique_ptr<kpt_candidates> c(new kpt_candidates());
    c->ctx = ctx;
    c->device = ctx->device;
    c->grid = grid->g;
    kpt::GenCandidates& v = c->view;
    v.kind = 1;
    uint64_t count = 1;
    const int n[2] = {grid->nx, grid->ny};
    for (int dim = 0; dim < 2; ++dim) {
        v.lower[dim] = domain != 0 ? -2 : 0;
        const int upper = domain != 0 ? n[dim] + 1 : n[dim] - 1;
        v.extents[dim] = upper - v.lower[dim] + 1;
        KPT_REQUIRE(v.extents[dim] > 0, "Grid particle candidate set: grid domain has no cells.");
        count *= static_cast<uint64_t>(v.extents[dim]);
    }
    KPT_CUDA(c->cumulative.reserve(count * sizeof(double)));
    ScopedBuffer scratch;
    KPT_CUDA(scratch.reserve(kpt::generator_scan_scratch(count) * sizeof(double)));
    KPT_CUDA(kpt::generator_grid_weights(grid->g, v.lower, v.extents, count,
                                         c->cumulative.as<double>(), scratch.as<double>(),
                                         ctx->stream));
    double total = 0.0;
    KPT_CUDA(cudaMemcpyAsync(&total, c->cumulative.as<double>() + (count - 1), sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    KPT_REQUIRE(std::isfinite(total) && total > 0.0,
                "Grid particle candidate set: total physical volume must be positive.");
    v.cumulative = c->cumulative.as<double>();
    v.count = count;
    v.total = total;
    *out = c.release();
    return KPT_OK;
}

int kpt_candidates_info(const kpt_candidates* c, uint64_t* count, double* total_weight) {
    KPT_REQUIRE(c, "kpt_candidates_info: NULL handle");
    if (count) *count = c->view.count;
    if (total_weight) *total_weight = c->view.total;
    return KPT_OK;
}

int kpt_candidates_download(kpt_context* ctx, const kpt_candidates* c, uint64_t* indices,
                            double* cumulative_weights) {
    KPT_REQUIRE(ctx && c, "kpt_candidates_download: NULL handle");
    if (int rc = activate(ctx)) return rc;
    const uint64_t n = c->view.count;
    if (n == 0) return KPT_OK;
    if (indices) {
        if (c->view.kind == 0) {
            KPT_CUDA(cudaMemcpyAsync(indices, c->view.indices, n * sizeof(uint64_t),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            for (uint64_t k = 0; k < n; ++k) indices[k] = k;
        }
    }
    if (cumulative_weights) {
        KPT_CUDA(cudaMemcpyAsync(cumulative_weights, c->view.cumulative, n * sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    }
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

int kpt_candidates_destroy(kpt_candidates* candidates) {
    delete candidates;
    return KPT_OK;
}

int kpt_generator_inject_uniform(kpt_context* ctx, kpt_system* sys, uint64_t seed,
                                 uint32_t frame, const kpt_region* region,
                                 const kpt_injection_plan* plan,
                                 const kpt_injection_kinematics* kinematics,
                                 const kpt_field_predicate* predicate) {
    KPT_REQUIRE(ctx && sys && region && plan && kinematics,
                "kpt_generator_inject_uniform: NULL argument");
    if (int rc = validate_region(region)) return rc;
    if (int rc = validate_kinematics(kinematics)) return rc;
    if (int rc = validate_plan(sys, plan)) return rc;
    kpt::GenLaunch L{};
    if (int rc = gen_predicate(predicate, nullptr, &L.predicate)) return rc;
    if (int rc = activate(ctx)) return rc;
    gen_common(ctx, sys, L, seed, frame, kinematics);
    if (predicate) L.grid = predicate->field->grid;
    L.recycle = 0;
    L.source = 0;
    for (int dim = 0; dim < 2; ++dim) {
        L.region_lo[dim] = region->lower[dim];
        L.region_hi[dim] = region->upper[dim];
    }
    L.first_index = plan->first_particle_index;
    L.count = plan->particle_count;
    L.first_id = plan->first_particle_id;
    L.max_attempts = plan->max_attempts;
    return gen_finish(ctx, sys, L, nullptr);
}

int kpt_generator_inject_candidates(kpt_context* ctx, kpt_system* sys, uint64_t seed,
                                    uint32_t frame, const kpt_candidates* candidates,
                                    const kpt_injection_plan* plan,
                                    const kpt_injection_kinematics* kinematics) {
    KPT_REQUIRE(ctx && sys && candidates && plan && kinematics,
                "kpt_generator_inject_candidates: NULL argument");
    if (int rc = validate_kinematics(kinematics)) return rc;
    if (int rc = validate_plan(sys, plan)) return rc;
    KPT_REQUIRE(candidates->view.count > 0,
                candidates->view.kind == 0
                    ? "ParticleGenerator: field-conditioned injection has no candidate grid "
                      "points."
                    : "ParticleGenerator: grid injection has no candidate cells.");
    if (int rc = activate(ctx)) return rc;
    kpt::GenLaunch L{};
    gen_common(ctx, sys, L, seed, frame, kinematics);
    L.grid = candidates->grid;
    L.recycle = 0;
    L.source = 1;
    L.candidates = candidates->view;
    L.first_index = plan->first_particle_index;
    L.count = plan->particle_count;
    L.first_id = plan->first_particle_id;
    L.max_attempts = plan->max_attempts;
    return gen_finish(ctx, sys, L, nullptr);
}

int kpt_generator_recycle_uniform(kpt_context* ctx, kpt_system* sys, uint64_t seed,
                                  uint32_t frame, const kpt_region* region,
                                  const kpt_injection_kinematics* kinematics,
                                  const kpt_field_predicate* predicate, int32_t selection,
                                  int32_t max_attempts, uint64_t* recycled) {
    KPT_REQUIRE(ctx && sys && region && kinematics,
                "kpt_generator_recycle_uniform: NULL argument");
    if (recycled) *recycled = 0;
    if (int rc = validate_region(region)) return rc;
    if (int rc = validate_kinematics(kinematics)) return rc;
    KPT_REQUIRE(max_attempts > 0, "ParticleGenerator: recycle max_attempts must be positive.");
    KPT_REQUIRE(selection >= 0 && selection <= 2, "kpt_generator_recycle_uniform: unknown selection");
    kpt::GenLaunch L{};
    if (int rc = gen_predicate(predicate, nullptr, &L.predicate)) return rc;
    if (int rc = activate(ctx)) return rc;
    gen_common(ctx, sys, L, seed, frame, kinematics);
    if (predicate) L.grid = predicate->field->grid;
    L.recycle = 1;
    L.source = 0;
    for (int dim = 0; dim < 2; ++dim) {
        L.region_lo[dim] = region->lower[dim];
        L.region_hi[dim] = region->upper[dim];
    }
    L.count = sys->count;
    L.selection = selection;
    L.max_attempts = max_attempts;
    return gen_finish(ctx, sys, L, recycled);
}

int kpt_generator_recycle_candidates(kpt_context* ctx, kpt_system* sys, uint64_t seed,
                                     uint32_t frame, const kpt_candidates* candidates,
                                     const kpt_injection_kinematics* kinematics,
                                     int32_t selection, uint64_t* recycled) {
    KPT_REQUIRE(ctx && sys && candidates && kinematics,
                "kpt_generator_recycle_candidates: NULL argument");
    if (recycled) *recycled = 0;
    if (int rc = validate_kinematics(kinematics)) return rc;
    KPT_REQUIRE(candidates->view.count > 0,
                candidates->view.kind == 0
                    ? "ParticleGenerator: field-conditioned recycling has no candidate grid "
                      "points."
                    : "ParticleGenerator: grid recycling has no candidate cells.");
    KPT_REQUIRE(selection >= 0 && selection <= 2, "kpt_generator_recycle_candidates: unknown selection");
    if (int rc = activate(ctx)) return rc;
    kpt::GenLaunch L{};
    gen_common(ctx, sys, L, seed, frame, kinematics);
    L.grid = candidates->grid;
    L.recycle = 1;
    L.source = 1;
    L.candidates = candidates->view;
    L.count = sys->count;
    L.selection = selection;
    return gen_finish(ctx, sys, L, recycled);
}

}  // extern "C"

// ====================================================================
// Batched runs: many independent driver runs pushed by one launch
// ====================================================================

struct kpt_batch {
    kpt_context* ctx = nullptr;
    int device = 0;
    struct Run {
        kpt_particles* parts;
        const kpt_field* lower;
        const kpt_field* upper;
        kpt_settings settings;
        uint64_t seed;
        uint32_t frame;
    };
    std::vector<Run> runs;
    int focused = -1;
    int sort_tile = 16;
    int blocks_per_sm = 0;
    int sort_every = 1;
    int threads = 128;            // threads per block of the batched push
    int particles_per_lane = 1;   // particles a lane advances side by side
    DeviceBuffer params, offsets, cursor, counters, saved;
    // cell records of every run's table pair (all runs or none), with the
    // field serials they were built from
    std::vector<DeviceBuffer> records;
    std::vector<std::pair<uint64_t, uint64_t>> record_serials;
    bool use_records = false;
    // cached graph of the last interval loop
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace {

// Cell records for the batched push: every run's table pair gets its
// records (built on the context's stream, kept while the pair is the same)
// when the context's mode asks for them -- KPT_RECORDS_AUTO: the runs
// together hold at least a quarter as many particles as their tables have
// points.  Out of device memory the batch samples the point tables.
int batch_records(kpt_batch* b) {
    kpt_context* ctx = b->ctx;
    const size_t runs = b->runs.size();
    uint64_t particles = 0, points = 0;
    for (const kpt_batch::Run& run : b->runs) {
        particles += run.parts->count;
        points += run.lower->points;
    }
    b->use_records = ctx->records_mode == KPT_RECORDS_ON ||
                     (ctx->records_mode == KPT_RECORDS_AUTO && particles * 4 >= points);
    if (!b->use_records) return KPT_OK;
    b->records.resize(runs);
    b->record_serials.resize(runs, {0, 0});
    for (size_t r = 0; r < runs; ++r) {
        const kpt_batch::Run& run = b->runs[r];
        const std::pair<uint64_t, uint64_t> key{run.lower->serial, run.upper->serial};
        if (b->record_serials[r] == key && b->records[r].ptr != nullptr) continue;
        const bool focused = run.lower->kind == KPT_TABLE_FOCUSED21;
        b->record_serials[r] = {0, 0};
        if (run.lower->points >= (1ull << 32) ||
            b->records[r].reserve(run.lower->points * kpt::record_floats(focused) *
                                  sizeof(float)) != cudaSuccess) {
            cudaGetLastError();  // out of memory: the point tables for every run
            for (DeviceBuffer& d : b->records) d.release();
            b->use_records = false;
            return KPT_OK;
        }
        kpt::RecordLaunch rl{};
        rl.lower = static_cast<const float*>(run.lower->table);
        rl.upper = static_cast<const float*>(run.upper->table);
        rl.records = b->records[r].as<float>();
        rl.points = run.lower->points;
        rl.ex = run.lower->nx + 4;
        rl.ey = run.lower->ny + 4;
        rl.focused = focused ? 1 : 0;
        KPT_CUDA(kpt::launch_build_records(rl, ctx->stream));
        b->record_serials[r] = key;
    }
    return KPT_OK;
}

int batch_prepare(kpt_batch* b) {
    kpt_context* ctx = b->ctx;
    const size_t runs = b->runs.size();
    const size_t psize = kpt::push_params_size();
    KPT_CUDA(b->params.reserve(runs * psize));
    KPT_CUDA(b->offsets.reserve((runs + 1) * sizeof(uint64_t)));
    KPT_CUDA(b->cursor.reserve(sizeof(unsigned long long)));
    KPT_CUDA(b->counters.reserve(runs * sizeof(kpt::PushCounters)));
    std::vector<char> host(runs * psize);
    std::vector<uint64_t> offsets(runs + 1, 0);
    if (int rc = batch_records(b)) return rc;
    for (size_t r = 0; r < runs; ++r) {
        kpt_batch::Run& run = b->runs[r];
        kpt_particles* parts = run.parts;
        if (b->sort_tile > 0) {
            // reserve the sort buffers outside any capture
            const int tx = (run.lower->nx + b->sort_tile - 1) / b->sort_tile;
            const int ty = (run.lower->ny + b->sort_tile - 1) / b->sort_tile;
            const uint64_t n = std::max<uint64_t>(parts->count, 1);
            KPT_CUDA(parts->order.reserve(n * sizeof(uint32_t)));
            KPT_CUDA(parts->keys.reserve(n * sizeof(uint32_t)));
            KPT_CUDA(parts->tile_counts.reserve((static_cast<size_t>(tx) * ty + 1) *
                                                sizeof(uint32_t)));
            parts->order_valid = true;
        } else {
            parts->order_valid = false;
        }
        kpt::PushLaunch launch;
        fill_push_launch(ctx, parts, run.lower, run.upper, &run.settings, run.frame, run.seed,
                         b->counters.as<kpt::PushCounters>() + r, launch);
        launch.records = b->use_records ? b->records[r].as<float>() : nullptr;
        kpt::build_push_params(launch, host.data() + r * psize);
        offsets[r + 1] = offsets[r] + parts->count;
    }
    KPT_CUDA(cudaMemcpyAsync(b->params.ptr, host.data(), host.size(), cudaMemcpyHostToDevice,
                             ctx->stream));
    KPT_CUDA(cudaMemcpyAsync(b->offsets.ptr, offsets.data(), offsets.size() * sizeof(uint64_t),
                             cudaMemcpyHostToDevice, ctx->stream));
    KPT_CUDA(cudaStreamSynchronize(ctx->stream));
    return KPT_OK;
}

kpt::BatchLaunch batch_launch(const kpt_batch* b) {
    kpt::BatchLaunch B{};
    B.params = b->params.ptr;
    B.offsets = b->offsets.as<uint64_t>();
    B.runs = static_cast<int>(b->runs.size());
    B.focused = b->focused;
    B.cursor = b->cursor.as<unsigned long long>();
    B.sm_count = b->ctx->sm_count;
    B.blocks_per_sm = b->blocks_per_sm;
    B.threads = b->threads;
    B.particles_per_lane = b->particles_per_lane;
    B.records = b->use_records ? 1 : 0;
    return B;
}

cudaError_t batch_sort_all(const kpt_batch* b, cudaStream_t stream) {
    for (const kpt_batch::Run& run : b->runs) {
        kpt_particles* parts = run.parts;
        if (parts->count == 0) continue;
        kpt::SortLaunch s{};
        s.grid = run.lower->grid;
        s.parts = parts->arrays;
        s.count = parts->count;
        s.tile_x = b->sort_tile;
        s.tile_y = b->sort_tile;
        s.tiles_x = (run.lower->nx + b->sort_tile - 1) / b->sort_tile;
        s.tiles_y = (run.lower->ny + b->sort_tile - 1) / b->sort_tile;
        s.keys = parts->keys.as<unsigned int>();
        s.counts = parts->tile_counts.as<unsigned int>();
        s.order = parts->order.as<unsigned int>();
        const cudaError_t err = kpt::launch_sort(s, stream);
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

// intervals x (cell sort every sort_every intervals, batched push, next frame)
cudaError_t batch_enqueue(const kpt_batch* b, uint32_t intervals, cudaStream_t stream) {
    const kpt::BatchLaunch B = batch_launch(b);
    for (uint32_t k = 0; k < intervals; ++k) {
        if (b->sort_tile > 0 && (k % static_cast<uint32_t>(b->sort_every)) == 0) {
            cudaError_t err = batch_sort_all(b, stream);
            if (err != cudaSuccess) return err;
        }
        cudaError_t err = kpt::launch_push_batch(B, stream);
        if (err != cudaSuccess) return err;
        err = kpt::launch_batch_next_frame(B, stream);
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

void batch_drop_graph(kpt_batch* b) {
    if (b->graph != nullptr) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
}

}  // namespace

extern "C" {

int kpt_batch_create(kpt_context* ctx, kpt_batch** out) {
    KPT_REQUIRE(ctx && out, "kpt_batch_create: NULL argument");
    *out = nullptr;
    std::unique_ptr<kpt_batch> b(new kpt_batch());
    b->ctx = ctx;
    b->device = ctx->device;
    *out = b.release();
    return KPT_OK;
}

int kpt_batch_destroy(kpt_batch* b) {
    if (b == nullptr) return KPT_OK;
    cudaSetDevice(b->device);
    batch_drop_graph(b);
    for (DeviceBuffer* d : {&b->params, &b->offsets, &b->cursor, &b->counters, &b->saved}) {
        d->release();
    }
    for (DeviceBuffer& d : b->records) d.release();
    delete b;
    return KPT_OK;
}

int kpt_batch_add_run(kpt_batch* b, kpt_particles* parts, const kpt_field* lower,
                      const kpt_field* upper, const kpt_settings* settings, uint64_t seed,
                      uint32_t first_frame, int* run_index) {
    KPT_REQUIRE(b && parts && lower && upper, "kpt_batch_add_run: NULL handle");
    if (int rc = validate_settings(settings)) return rc;
    KPT_REQUIRE(static_cast<int>(b->runs.size()) < kpt::batch_max_runs(),
                "kpt_batch_add_run: too many runs in one batch");
    KPT_REQUIRE(lower->precision == KPT_PRECISION_MIXED && upper->precision == KPT_PRECISION_MIXED,
                "kpt_batch_add_run: batched runs use mixed-precision tables");
    KPT_REQUIRE(lower->kind == upper->kind && lower->nx == upper->nx && lower->ny == upper->ny,
                "kpt_batch_add_run: lower and upper tables differ in kind or shape");
    KPT_REQUIRE((lower->kind == KPT_TABLE_FOCUSED21) == (settings->focused != 0),
                "kpt_batch_add_run: table kind does not match settings.focused");
    KPT_REQUIRE(settings->closure != KPT_CLOSURE_SURROGATE,
                "kpt_batch_add_run: the learned closure is not batched");
    KPT_REQUIRE(b->focused < 0 || b->focused == (settings->focused != 0 ? 1 : 0),
                "kpt_batch_add_run: all runs of a batch share the transport model");
    for (const kpt_batch::Run& run : b->runs) {
        KPT_REQUIRE(run.parts != parts, "kpt_batch_add_run: a particle store is in the batch twice");
    }
    b->focused = settings->focused != 0 ? 1 : 0;
    b->runs.push_back(kpt_batch::Run{parts, lower, upper, *settings, seed, first_frame});
    batch_drop_graph(b);
    if (run_index) *run_index = static_cast<int>(b->runs.size()) - 1;
    return KPT_OK;
}

int kpt_batch_set_schedule(kpt_batch* b, int sort_tile, int blocks_per_sm, int sort_every) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_set_schedule: NULL handle");
    KPT_REQUIRE(sort_tile >= 0 && blocks_per_sm >= 0 && sort_every >= 1,
                "kpt_batch_set_schedule: sort_tile >= 0, blocks_per_sm >= 0, sort_every >= 1");
    b->sort_tile = sort_tile;
    b->blocks_per_sm = blocks_per_sm;
    b->sort_every = sort_every;
    batch_drop_graph(b);
    return KPT_OK;
}

int kpt_batch_set_launch_shape(kpt_batch* b, int threads_per_block, int particles_per_lane) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_set_launch_shape: NULL handle");
    KPT_REQUIRE(kpt::batch_shape_supported(threads_per_block, particles_per_lane),
                "kpt_batch_set_launch_shape: threads_per_block 64, 128 or 256 and "
                "particles_per_lane 1 or 2");
    b->threads = threads_per_block;
    b->particles_per_lane = particles_per_lane;
    batch_drop_graph(b);
    return KPT_OK;
}

int kpt_batch_get_launch_shape(const kpt_batch* b, int* threads_per_block,
                               int* particles_per_lane) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_get_launch_shape: NULL handle");
    if (threads_per_block) *threads_per_block = b->threads;
    if (particles_per_lane) *particles_per_lane = b->particles_per_lane;
    return KPT_OK;
}

int kpt_batch_get_schedule(const kpt_batch* b, int* sort_tile, int* blocks_per_sm,
                           int* sort_every) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_get_schedule: NULL handle");
    if (sort_tile) *sort_tile = b->sort_tile;
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    if (sort_every) *sort_every = b->sort_every;
    return KPT_OK;
}

int kpt_batch_run(kpt_batch* b, uint32_t intervals, int use_graph) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_run: NULL handle");
    KPT_REQUIRE(!b->runs.empty(), "kpt_batch_run: no runs");
    if (intervals == 0) return KPT_OK;
    kpt_context* ctx = b->ctx;
    if (int rc = activate(ctx)) return rc;
    if (int rc = batch_prepare(b)) return rc;
    cudaStream_t st = ctx->stream;
    const uint32_t key[8] = {intervals, static_cast<uint32_t>(b->sort_tile),
                             static_cast<uint32_t>(b->blocks_per_sm),
                             static_cast<uint32_t>(b->sort_every),
                             static_cast<uint32_t>(b->runs.size()),
                             static_cast<uint32_t>(b->threads),
                             static_cast<uint32_t>(b->particles_per_lane),
                             b->use_records ? 1u : 0u};
    if (use_graph && st != nullptr) {
        if (b->graph == nullptr || std::memcmp(key, b->graph_key, sizeof(key)) != 0) {
            batch_drop_graph(b);
            cudaGraph_t graph = nullptr;
            KPT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const cudaError_t err = batch_enqueue(b, intervals, st);
            const cudaError_t end = cudaStreamEndCapture(st, &graph);
            if ((err != cudaSuccess || end != cudaSuccess) && graph != nullptr) {
                cudaGraphDestroy(graph);
            }
            KPT_CUDA(err);
            KPT_CUDA(end);
            const cudaError_t inst = cudaGraphInstantiate(&b->graph, graph, 0);
            cudaGraphDestroy(graph);
            KPT_CUDA(inst);
            std::memcpy(b->graph_key, key, sizeof(key));
        }
        KPT_CUDA(cudaGraphLaunch(b->graph, st));
    } else {
        KPT_CUDA(batch_enqueue(b, intervals, st));
    }
    KPT_CUDA(cudaStreamSynchronize(st));
    for (kpt_batch::Run& run : b->runs) run.frame += intervals;
    return KPT_OK;
}

int kpt_batch_stats(const kpt_batch* b, int run, kpt_push_stats* out) {
    KPT_REQUIRE(b && out, "kpt_batch_stats: NULL argument");
    KPT_REQUIRE(run >= 0 && run < static_cast<int>(b->runs.size()),
                "kpt_batch_stats: run index out of range");
    KPT_REQUIRE(b->counters.ptr != nullptr, "kpt_batch_stats: the batch has not run");
    KPT_CUDA(cudaSetDevice(b->device));
    kpt::PushCounters host{};
    KPT_CUDA(cudaMemcpy(&host, b->counters.as<kpt::PushCounters>() + run, sizeof(host),
                        cudaMemcpyDeviceToHost));
    out->particle_steps = host.particle_steps;
    out->pushed = host.pushed;
    out->failed = host.failed;
    out->max_steps = host.max_steps;
    out->pad = 0;
    return KPT_OK;
}

int kpt_batch_frame(const kpt_batch* b, int run, uint32_t* frame) {
    KPT_REQUIRE(b && frame, "kpt_batch_frame: NULL argument");
    KPT_REQUIRE(run >= 0 && run < static_cast<int>(b->runs.size()),
                "kpt_batch_frame: run index out of range");
    *frame = b->runs[static_cast<size_t>(run)].frame;
    return KPT_OK;
}

int kpt_batch_set_frame(kpt_batch* b, int run, uint32_t frame) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_set_frame: NULL handle");
    KPT_REQUIRE(run >= 0 && run < static_cast<int>(b->runs.size()),
                "kpt_batch_set_frame: run index out of range");
    b->runs[static_cast<size_t>(run)].frame = frame;
    return KPT_OK;
}

int kpt_batch_autotune(kpt_batch* b, uint32_t intervals, kpt_batch_tuning* out) {
    KPT_REQUIRE(b != nullptr, "kpt_batch_autotune: NULL handle");
    KPT_REQUIRE(!b->runs.empty(), "kpt_batch_autotune: no runs");
    kpt_context* ctx = b->ctx;
    if (int rc = activate(ctx)) return rc;
    cudaStream_t st = ctx->stream;
    intervals = intervals == 0 ? 1 : intervals;
    // save the pushed state of every run (x, y, p, t, step_dt, mu, status)
    size_t bytes = 0;
    for (const kpt_batch::Run& run : b->runs) bytes += run.parts->count * (6 * 8 + 4);
    KPT_CUDA(b->saved.reserve(std::max<size_t>(bytes, 8)));
    auto copy_state = [&](bool save) -> int {
        char* cur = static_cast<char*>(b->saved.ptr);
        for (const kpt_batch::Run& run : b->runs) {
            const kpt::ParticleArrays& a = run.parts->arrays;
            const size_t n = run.parts->count;
            void* arrays[7] = {a.x, a.y, a.p, a.t, a.step_dt, a.mu, a.status};
            for (int k = 0; k < 7; ++k) {
                const size_t sz = n * (k < 6 ? 8 : 4);
                if (sz == 0) continue;
                if (save) {
                    KPT_CUDA(cudaMemcpyAsync(cur, arrays[k], sz, cudaMemcpyDeviceToDevice, st));
                } else {
                    KPT_CUDA(cudaMemcpyAsync(arrays[k], cur, sz, cudaMemcpyDeviceToDevice, st));
                }
                cur += sz;
            }
        }
        return KPT_OK;
    };
    if (int rc = copy_state(true)) return rc;
    const std::vector<uint32_t> frames = [&] {
        std::vector<uint32_t> f;
        for (const kpt_batch::Run& run : b->runs) f.push_back(run.frame);
        return f;
    }();
    cudaEvent_t e0, e1;
    KPT_CUDA(cudaEventCreate(&e0));
    KPT_CUDA(cudaEventCreate(&e1));
    const int repeats = 3;
    // One candidate: its median over `repeats` timings of `intervals`
    // intervals from the saved state, and the spread (max - min) / median.
    auto time_candidate = [&](float* median, float* spread) -> int {
        batch_drop_graph(b);
        if (int rc = batch_prepare(b)) return rc;
        float ms[repeats];
        for (int r = 0; r < repeats; ++r) {
            KPT_CUDA(cudaEventRecord(e0, st));
            KPT_CUDA(batch_enqueue(b, intervals, st));
            KPT_CUDA(cudaEventRecord(e1, st));
            KPT_CUDA(cudaEventSynchronize(e1));
            KPT_CUDA(cudaEventElapsedTime(&ms[r], e0, e1));
            if (int rc = copy_state(false)) return rc;
            for (size_t k = 0; k < b->runs.size(); ++k) b->runs[k].frame = frames[k];
            if (int rc = batch_prepare(b)) return rc;
        }
        std::sort(ms, ms + repeats);
        *median = ms[repeats / 2];
        *spread = *median > 0.0f ? (ms[repeats - 1] - ms[0]) / *median : 0.0f;
        return KPT_OK;
    };
    struct Choice {
        int tile, every, bps, threads, ppl;
        float ms, spread;
    };
    Choice best{b->sort_tile, b->sort_every, b->blocks_per_sm, b->threads,
                b->particles_per_lane, 0.0f, 0.0f};
    int tried = 0;
    auto consider = [&](const Choice& c) -> int {
        b->sort_tile = c.tile;
        b->sort_every = c.every;
        b->blocks_per_sm = c.bps;
        b->threads = c.threads;
        b->particles_per_lane = c.ppl;
        float ms = 0.0f, spread = 0.0f;
        if (int rc = time_candidate(&ms, &spread)) return rc;
        if (tried == 0 || ms < best.ms) {
            best = c;
            best.ms = ms;
            best.spread = spread;
        }
        ++tried;
        return KPT_OK;
    };
    // Stage 1: the cell-sort tile and interval at the default launch shape.
    const int tiles[4] = {0, 8, 16, 32};
    const int every[2] = {1, 2};
    for (int tile : tiles) {
        for (int ev : every) {
            if (tile == 0 && ev != 1) continue;
            if (int rc = consider(Choice{tile, ev, 0, 128, 1, 0.0f, 0.0f})) return rc;
        }
    }
    // Stage 2: block shape, particles per lane and residency with that sort.
    // Residency candidates are resident threads per SM (all that fit, or the
    // threads of 3 or 2 blocks of 128), as blocks of the shape.
    const int sort_tile = best.tile, sort_every = best.every;
    const int shapes[3] = {64, 128, 256};
    const int lanes[2] = {1, 2};
    const int resident_threads[3] = {0, 384, 256};
    for (int threads : shapes) {
        for (int ppl : lanes) {
            for (int rt : resident_threads) {
                const int bps = rt == 0 ? 0 : std::max(1, rt / threads);
                if (threads == 128 && ppl == 1 && rt == 0) continue;  // timed in stage 1
                if (int rc = consider(Choice{sort_tile, sort_every, bps, threads, ppl, 0.0f,
                                             0.0f})) {
                    return rc;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    KPT_CUDA(cudaStreamSynchronize(st));
    for (size_t r = 0; r < b->runs.size(); ++r) b->runs[r].frame = frames[r];
    b->sort_tile = best.tile;
    b->blocks_per_sm = best.bps;
    b->sort_every = best.every;
    b->threads = best.threads;
    b->particles_per_lane = best.ppl;
    batch_drop_graph(b);
    if (out) {
        out->sort_tile = best.tile;
        out->blocks_per_sm = best.bps;
        out->sort_every = best.every;
        out->candidates = tried;
        out->best_ms = best.ms;
        out->spread = best.spread;
        out->threads_per_block = best.threads;
        out->particles_per_lane = best.ppl;
        out->repeats = repeats;
        out->pad = 0;
    }
    return KPT_OK;
}

}  // extern "C"
