/*
 * kpt.h — C ABI of the GB300-native Parker / focused-transport particle push.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (KPT_OK = 0, negative = error; kpt_last_error() describes the
 * last failure on the calling thread) and never falls back to the CPU: with
 * no usable CUDA device, kpt_context_create fails.
 *
 * Handles are opaque and owned by their creator; fields and particle stores
 * may be destroyed before or after their context.  Calls on one context are
 * ordered on the context's CUDA stream; calls that return host results
 * (counts, histograms, summaries, downloads) synchronise that stream.
 *
 * The entry points replace the reference's driver functions and library
 * types (paths relative to the reference project):
 *   kpt_field_create            src/main.cpp:932-962 load_*_coefficient_frame,
 *                               include/AthenaFieldReader.hpp:290-360 (reader),
 *                               include/Field.hpp:274-316 (ghost fill),
 *                               src/main.cpp:840-957 (coefficient tables)
 *   kpt_particles_*             src/main.cpp:292-333 ReconnectionParticleStorage
 *   kpt_inject_uniform          src/main.cpp:996-1048 inject_uniform_particles
 *   kpt_push_interval           src/main.cpp:1084-1327 move_parker_particles_one_interval,
 *                               src/main.cpp:1334-1755 move_particles_one_interval
 *   kpt_split                   src/main.cpp:1761-1839 split_particles
 *   kpt_histogram               src/main.cpp:1907-1964 write_momentum_histogram (binning)
 *   kpt_summarize               src/main.cpp:1845-1901 summarize_particles
 *   kpt_sample_table            include/FieldInterpolator.hpp:346-380 LinearPositionInterpolator
 *                               ::sample with src/main.cpp:1055-1077 time interpolation
 */
#ifndef KPT_H
#define KPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KPT_ABI_VERSION 2

enum kpt_status {
    KPT_OK = 0,
    KPT_ERROR_INVALID_ARGUMENT = -1,
    KPT_ERROR_CUDA = -2,
    KPT_ERROR_OUT_OF_MEMORY = -3,
    KPT_ERROR_IO = -4,
    KPT_ERROR_FORMAT = -5,
    KPT_ERROR_CAPACITY = -6,
    KPT_ERROR_NO_DEVICE = -7
};

/* Coefficient table layouts (component order of src/main.cpp:38-79). */
enum kpt_table_kind {
    KPT_TABLE_PARKER16 = 0,  /* Vx Vy Bx By Bz |B| dVx/dx dVy/dy dBx/dx dBx/dy dBy/dx
                                dBy/dy dBz/dx dBz/dy d|B|/dx d|B|/dy */
    KPT_TABLE_FOCUSED21 = 1  /* Vx Vy Vz Bx By Bz |B|, d(Vx,Vy,Vz)/d(x,y) (6),
                                d(Bx,By,Bz)/d(x,y) (6), d|B|/dx d|B|/dy */
};

/* Arithmetic of a table and of the push that reads it. */
enum kpt_precision {
    KPT_PRECISION_F64 = 0,   /* plain FP64 throughout */
    KPT_PRECISION_MIXED = 1  /* FP32 table, interpolation, coefficients and noise; FP64
                                position, time and momentum accumulation and cell search */
};

/* Pitch-angle scattering closure of the focused push. */
enum kpt_closure {
    KPT_CLOSURE_DRIVER = 0,    /* the driver's reduced D_mumu (src/main.cpp:1551-1589) */
    KPT_CLOSURE_QLT = 1,       /* slab-spectrum quasi-linear D_mumu, dD_mumu/dmu
                                  (include/LegencyModel.hpp:539-645) */
    KPT_CLOSURE_SURROGATE = 2  /* the QLT closure served by the trained MLP surrogate */
};

enum kpt_schedule {
    KPT_SCHEDULE_REFILL = 0,
    KPT_SCHEDULE_SIMPLE = 1
};

/* How the learned closure's network is served (push and evaluate). */
enum kpt_network_engine {
    KPT_ENGINE_TCGEN05 = 0,  /* block-collective tcgen05.mma, activations in tensor memory */
    KPT_ENGINE_MMA_SYNC = 1  /* warp-collective mma.sync, activations in registers */
};

/* Run parameters: the reference's Reconnection2DSettings physics block
 * (src/main.cpp:114-241).  Doubles first, then 32-bit ints. */
typedef struct kpt_settings {
    double mhd_dt;
    double p0;
    double pmin;
    double pmax;
    double gamma_turb;
    double kpara0;
    double kperp_over_kpara;
    double dt_min_rel;
    double dt_max_rel;
    double drift_param1;
    double drift_param2;
    double charge;
    double particle_v0;
    double duu0;
    double split_ratio;
    double pmin_split_over_p0;
    double mu_max;
    int32_t max_steps;
    int32_t momentum_dependency;
    int32_t magnetic_dependency;
    int32_t time_interpolation;
    int32_t split_particles;
    int32_t focused;
    /* Focused transport scattering closure (extension; KPT_CLOSURE_DRIVER
     * reproduces the reference driver).  The QLT closure evaluates, per
     * substep, Omega = qlt_omega0 |B| / gamma (gamma = sqrt(1 + p^2)),
     * v = particle_v0 p / p0, xi = Omega qlt_lc / v and the slab-spectrum
     * D_mumu of index qlt_spectral_index with regularisation qlt_h0. */
    int32_t closure;
    double qlt_sigma2;          /* dB^2 / B^2 */
    double qlt_spectral_index;  /* gamma_k */
    double qlt_h0;              /* |mu| regularisation */
    double qlt_omega0;          /* gyrofrequency at |B| = 1, gamma = 1 */
    double qlt_lc;              /* correlation length */
} kpt_settings;

/* Per-push counters, summed over the particles pushed. */
typedef struct kpt_push_stats {
    uint64_t particle_steps;   /* executed substep-loop iterations */
    uint64_t pushed;           /* particles active at the start of the push */
    uint64_t failed;           /* of those, particles that ended with status 2 */
    uint32_t max_steps;        /* largest per-particle substep count */
    uint32_t pad;
} kpt_push_stats;

/* summarize_particles output (src/main.cpp:255-270). */
typedef struct kpt_summary {
    uint64_t stored;
    uint64_t active;
    uint64_t inactive;
    double weight_sum;
    double p_min;
    double p_max;
    double p_avg;
    double dt_min;
    double dt_max;
    double dt_avg;
    int32_t max_split_level;
    int32_t pad;
} kpt_summary;

/* Device pointers of a particle store (SoA, length = capacity). */
typedef struct kpt_particle_arrays {
    double* x;
    double* y;
    double* p;
    double* t;
    double* step_dt;
    double* weight;
    double* mu;
    int32_t* status;
    int32_t* split_level;
} kpt_particle_arrays;

/* Training controls of the learned QLT closure (5 -> H -> H -> 3 tanh MLP,
 * inputs mu, ln p, ln|B|, dB^2/B^2, gamma_k; outputs D_mumu, dD_mumu/dmu,
 * ln kappa_parallel).  The box is where the network is trusted: outside it,
 * and for |mu| < mu_cut, the push evaluates the plain closure. */
enum kpt_surrogate_element {
    KPT_SURROGATE_BF16 = 0,  /* bfloat16 weights and activations (default) */
    KPT_SURROGATE_FP16 = 1   /* IEEE binary16: 3 more significand bits, same speed */
};

typedef struct kpt_surrogate_config {
    int32_t samples;          /* training set size (default 2,000,000) */
    int32_t steps;            /* Adam steps (default 16000) */
    int32_t batch;            /* minibatch (default 8192) */
    int32_t element_type;     /* kpt_surrogate_element of the served network */
    int32_t quantization_aware; /* 1: the last quarter of the steps trains through the
                                   served element type's rounding (default 0; measured
                                   no gain for BF16, whose error is activation rounding) */
    int32_t hidden_width;     /* H: 64 (default) or 32 */
    double learning_rate;     /* initial; cosine decay to 1 % (default 1e-2) */
    double mu_cut;            /* default 0.02 */
    double mu_max;            /* largest |mu| trained (default 0.999) */
    double p_lo_over_p0;      /* default 0.1 */
    double p_hi_over_p0;      /* default 1000 */
    double sigma2_lo;         /* default 0.01 */
    double sigma2_hi;         /* default 1 */
    double gk_lo;             /* default 1.5 */
    double gk_hi;             /* default 2 */
    double b_lo;              /* |B| range (default 0.05 .. 5) */
    double b_hi;
    uint64_t seed;
} kpt_surrogate_config;

typedef struct kpt_context kpt_context;
typedef struct kpt_field kpt_field;
typedef struct kpt_particles kpt_particles;
typedef struct kpt_surrogate kpt_surrogate;

/* ---- library ---------------------------------------------------------- */
int kpt_abi_version(void);
const char* kpt_last_error(void);
/* Reference defaults (src/main.cpp:136-154, Reconnection2DSettings). */
void kpt_default_settings(kpt_settings* out);

/* ---- context: one CUDA device and one stream --------------------------- */
int kpt_context_create(int device, kpt_context** out);
int kpt_context_destroy(kpt_context* ctx);
/* Order later calls on an external stream (cudaStream_t); NULL = own stream. */
int kpt_context_set_stream(kpt_context* ctx, void* cuda_stream);
int kpt_context_synchronize(kpt_context* ctx);
/* FP64 FMA throughput of the context's GPU in TFLOP/s, measured by a
 * project-written FMA-chain kernel (best of five launches, clocks as they
 * are).  No counterpart in the reference: it is the denominator of the plain
 * FP64 pushes' roofline, since GB300's FP64 pipe, not memory, bounds them. */
int kpt_context_fp64_fma_rate(kpt_context* ctx, double* tflops);
/* out[i] = x[i]^y[i] by the FP64 push's power function, evaluated on the GPU
 * (host arrays; parity and diagnostics).  The FP64 push computes every
 * Kokkos::pow of the reference's kernels (src/main.cpp:1180-1185,
 * :1439-1444, :1553-1580) with this function; the oracle and the reference
 * build on the shim use the same one, so powers round alike on both sides. */
int kpt_math_pow(kpt_context* ctx, uint64_t n, const double* x, const double* y, double* out);
/* Push scheduling: KPT_SCHEDULE_REFILL (persistent warps that refill lanes
 * from a work cursor; blocks_per_sm x SM count blocks of 128 threads, 0 =
 * as many as are resident) or KPT_SCHEDULE_SIMPLE (one particle per
 * thread).  Results do not depend on the choice. */
int kpt_context_set_push_schedule(kpt_context* ctx, int schedule, int blocks_per_sm);
/* Arithmetic of the plain FP64 push (precision KPT_PRECISION_F64):
 * KPT_FP64_STRICT (default) rounds every operation as the reference's code
 * is written (no FMA contraction) and computes powers with the library's
 * kpt_math_pow function, as the oracle does, so FP64 trajectories equal the
 * reference's on the Kokkos shim bit for bit over whole intervals;
 * KPT_FP64_CONTRACTED lets the compiler fuse multiply-adds and uses CUDA's
 * pow: about a quarter faster, trajectories within ~1e-15 per step of the
 * strict ones (the reference's own optimised builds contract too). */
enum kpt_fp64_arithmetic { KPT_FP64_STRICT = 0, KPT_FP64_CONTRACTED = 1 };
int kpt_context_set_fp64_arithmetic(kpt_context* ctx, int mode);
/* Cell records of the mixed pushes (no counterpart in the reference, whose
 * push samples its point tables): for a pair of FP32 tables the context
 * keeps one record per cell with each component's eight corner values of
 * both frames in one 32-byte sector, so four lanes of a warp read a
 * particle's cell one 128-byte line at a time.  KPT_RECORDS_AUTO (default)
 * builds them (record_floats x 4 bytes per table point: 768 focused, 512
 * Parker; rebuilt when the table pair changes) for a refill-scheduled
 * mixed push of at least a quarter as many particles as the table has
 * points; KPT_RECORDS_OFF never, KPT_RECORDS_ON for every refill-scheduled
 * mixed push.  Results are bit-identical either way.  The records are built
 * on the context's stream; a later push on another stream waits for them. */
enum kpt_records_mode { KPT_RECORDS_AUTO = 0, KPT_RECORDS_OFF = 1, KPT_RECORDS_ON = 2 };
int kpt_context_set_cell_records(kpt_context* ctx, int mode);

/* ---- fields: one MHD frame as a device coefficient table ---------------- */
/* Cells are 3 x ny x nx arrays (x fastest) of B and V, host memory.  Edges
 * (nx+1, ny+1) must be finite and ascending; uniform axes use the analytic
 * map, non-uniform axes the stored-edge map (extension). */
int kpt_field_create(kpt_context* ctx, int nx, int ny, const double* x_edges,
                     const double* y_edges, const double* b_cells, const double* v_cells,
                     int table_kind, int precision, kpt_field** out);
/* Read a compact field file (AthenaFieldReader.hpp:277-285 layout) and build
 * its table. */
int kpt_field_load(kpt_context* ctx, const char* path, int table_kind, int precision,
                   kpt_field** out);
int kpt_field_destroy(kpt_field* field);
/* The reader and the table build of kpt_field_load as two calls, so a host
 * thread can read frame f+2 from disk while the GPU pushes frame f (the
 * reference reads each frame between pushes, src/main.cpp:2300-2312).
 * kpt_field_data_read launches nothing on the device and may run on any host
 * thread; the cell data lands in page-locked memory (cudaHostAlloc) for a
 * full-bandwidth upload. */
typedef struct kpt_field_data kpt_field_data;
int kpt_field_data_read(const kpt_context* ctx, const char* path, kpt_field_data** out);
int kpt_field_data_free(kpt_field_data* data);
int kpt_field_data_shape(const kpt_field_data* data, int* nx, int* ny);
int kpt_field_create_from_data(kpt_context* ctx, const kpt_field_data* data, int table_kind,
                               int precision, kpt_field** out);
/* nx, ny, number of ghosted points and components. */
int kpt_field_shape(const kpt_field* field, int* nx, int* ny, uint64_t* points,
                    int* components);
/* Copy the table to host as float64 (points x components). */
int kpt_field_download_table(const kpt_field* field, double* out, uint64_t out_len);

/* ---- learned closure (no counterpart in the reference; replaces the QLT
 *      evaluation of include/LegencyModel.hpp:557-645 in the focused push) ---- */
void kpt_surrogate_default_config(kpt_surrogate_config* out);
/* Generate the training set from the plain closure (with the physics of
 * `settings`) and train on the GPU with the library's own forward/backward
 * kernels and Adam.  final_loss: mean squared error (normalised units) of
 * the last steps. */
int kpt_surrogate_train(kpt_context* ctx, const kpt_settings* settings,
                        const kpt_surrogate_config* config, kpt_surrogate** out,
                        double* final_loss);
int kpt_surrogate_destroy(kpt_surrogate* surrogate);
/* Network on n raw inputs (n x 5: mu, ln p, ln|B|, dB^2/B^2, gamma_k) ->
 * n x 3 (D_mumu, dD_mumu/dmu, ln kappa_parallel).  tensor_cores = 1 runs the
 * tensor-core path the push uses, 0 the FP32 SIMT forward.  Inputs
 * outside the box or with |mu| < mu_cut get the plain closure; served
 * (optional, n) is 1 where the network answered. */
int kpt_surrogate_evaluate(kpt_surrogate* surrogate, uint64_t n, const double* inputs,
                           int tensor_cores, double* outputs, int32_t* served);
/* Engine that serves the network in the push and in evaluate's
 * tensor-core path.  A trained network starts on the engine measured faster
 * for its width on GB300: KPT_ENGINE_TCGEN05 at width 64, KPT_ENGINE_MMA_SYNC
 * at width 32 (whose GEMMs are too small to repay the block-collective
 * engine's barriers and tensor-memory round trips).  The engines compute the
 * same BF16/FP16 network with FP32 accumulation; their sums associate
 * differently, so results agree to FP32 rounding, not bit for bit. */
int kpt_surrogate_set_engine(kpt_surrogate* surrogate, int engine);
int kpt_surrogate_get_engine(const kpt_surrogate* surrogate, int32_t* engine);
/* Failure-path check of the tcgen05 engine, no fault involved: `blocks`
 * blocks set up the width-64 network (weights, completion barrier, tensor
 * memory), wait `polls` polls for a completion that nothing signals, and
 * tear down as a timed-out push does (bounded second wait, tensor memory
 * freed).  timed_out / finished receive the blocks that reported the
 * timeout / got past the teardown (both = blocks when the bounds work). */
int kpt_surrogate_check_timeout(kpt_surrogate* surrogate, uint32_t blocks, uint32_t polls,
                                uint32_t* timed_out, uint32_t* finished);
/* Host only: the tcgen05 engine's weight block of a parameter block (the
 * FP32 layout of kpt_surrogate_parameters) as 16-bit values (BF16, or FP16
 * when fp16 != 0).  Three K-major, unswizzled tcgen05 B operands follow each
 * other: layer 1 (N = H rows, K = 16: inputs 0..4, bias head, bias
 * remainder, zeros), layer 2 (N = H, K = H + 16: weights, bias head,
 * remainder, zeros), layer 3 (N = 16, K = H + 16; rows 3..15 zero); element
 * (n, k) of an N x K operand sits at 16-bit index ((n/8) (K/8) 64 + (k/8) 64
 * + (n%8) 8 + k%8).  The bias head is the bias rounded to 16 bits, the
 * remainder the rounding of (bias - head).  out_len >= 16 H + H (H + 16) +
 * 16 (H + 16) values. */
int kpt_surrogate_pack_tc(const float* params, int32_t hidden_width, int32_t fp16,
                          uint16_t* out, uint64_t out_len);
/* Parameter block (FP32, W1[H][5] b1[H] W2[H][H] b2[H] W3[3][H] b3[3]:
 * 1379 floats for H = 32, 4739 for H = 64) and the box
 * normalisation (in_lo[5], in_hi[5], out_offset[3], out_scale[3], mu_cut);
 * the box is in feature units ln|mu|, ln p, ln|B|, ln(dB^2/B^2), gamma_k and
 * a feature f maps to 2 (f - lo) / (hi - lo) - 1. */
int kpt_surrogate_parameters(const kpt_surrogate* surrogate, float* params, int len,
                             float* normalisation, int norm_len);
/* Hidden width and parameter count of a trained network. */
int kpt_surrogate_shape(const kpt_surrogate* surrogate, int32_t* hidden_width,
                        int32_t* parameters);
/* Loss gradient (FP32) at `params` (a network of hidden width H, 0 = the
 * default) over n samples taken in order: normalised inputs (n x 5) and
 * normalised targets (n x 3). */
int kpt_surrogate_gradient(kpt_context* ctx, int32_t hidden_width, const float* params,
                           uint64_t n, const float* inputs, const float* targets, float* grad,
                           float* loss);
/* Pushes on this context with closure KPT_CLOSURE_SURROGATE use this
 * network (16-bit weights and activations, FP32 accumulation, on the tensor
 * cores).  The mixed focused push serves it on the surrogate's engine; the
 * FP64 focused push (precision KPT_PRECISION_F64, contracted FP64 arithmetic)
 * serves it on the mma.sync engine, where it replaces the plain closure's
 * five FP64 powers per substep.  The context keeps the pointer: unset it
 * (NULL) before destroying the surrogate. */
int kpt_context_set_surrogate(kpt_context* ctx, kpt_surrogate* surrogate);
/* Per-step judge of the surrogate in pushes since the last call: network
 * evaluations, evaluations checked against the plain closure, fallbacks to
 * the plain closure, largest relative error of D_mumu seen. */
int kpt_surrogate_judge(kpt_context* ctx, uint64_t* evaluations, uint64_t* judged,
                        uint64_t* fallbacks, double* max_rel_error);

/* ---- particles --------------------------------------------------------- */
int kpt_particles_create(kpt_context* ctx, uint64_t capacity, kpt_particles** out);
/* Non-owning store over existing device arrays (for example the CUDA-backend
 * Views of the reference's ReconnectionParticleStorage, src/main.cpp:292-333:
 * x = position.data(), y = position.data() + capacity under LayoutLeft).
 * The caller keeps the memory alive; destroy releases only the handle. */
int kpt_particles_wrap(kpt_context* ctx, uint64_t capacity, uint64_t count,
                       const kpt_particle_arrays* arrays, kpt_particles** out);
int kpt_particles_destroy(kpt_particles* particles);
int kpt_particles_count(const kpt_particles* particles, uint64_t* count,
                        uint64_t* capacity);
int kpt_particles_set_count(kpt_particles* particles, uint64_t count);
/* Host SoA in / out for the first `count` particles; NULL skips an array. */
int kpt_particles_upload(kpt_particles* particles, uint64_t count, const double* x,
                         const double* y, const double* p, const double* t,
                         const double* step_dt, const double* weight, const double* mu,
                         const int32_t* status, const int32_t* split_level);
int kpt_particles_download(const kpt_particles* particles, uint64_t count, double* x,
                           double* y, double* p, double* t, double* step_dt, double* weight,
                           double* mu, int32_t* status, int32_t* split_level);
int kpt_particles_device_arrays(const kpt_particles* particles, kpt_particle_arrays* out);
/* The driver's v4 snapshot records of the stored particles, packed on the
 * GPU (write_reconnection_particle_snapshot's record loop,
 * src/main.cpp:2155-2201): count x 100 bytes (id = storage index, status,
 * split level, sort key 0, position written as position, previous and
 * previous-step position, p, mu, weight, initial_kinetic_energy) copied to
 * `out` (page-locked memory from kpt_host_alloc copies fastest). */
int kpt_particles_pack_records(kpt_context* ctx, const kpt_particles* particles,
                               double initial_kinetic_energy, void* out, uint64_t out_len);
/* Page-locked host memory (for snapshot buffers and prefetched frames). */
int kpt_host_alloc(uint64_t bytes, void** out);
int kpt_host_free(void* ptr);

/* Cell sort of the work order: particle indices are ordered by spatial tile
 * (tile_x x tile_y cells, inactive particles last) and later pushes visit
 * particles in that order for cache locality.  Particle storage does not
 * move, so ids, noise streams and results are unchanged; the order is
 * dropped whenever the particle count changes (inject, split, upload). */
int kpt_particles_sort(kpt_context* ctx, kpt_particles* particles, const kpt_field* grid,
                       int tile_x, int tile_y);
int kpt_particles_clear_order(kpt_particles* particles);

/* ---- hot path ---------------------------------------------------------- */
/* Append min(requested, capacity - count) particles for the interval that
 * starts at frame * mhd_dt.  band_lo < band_hi draws y in that band instead
 * of the whole domain.  Noise: Philox4x32-10 keyed (seed, k, frame, 1). */
int kpt_inject_uniform(kpt_context* ctx, kpt_particles* particles, const kpt_field* grid,
                       const kpt_settings* settings, uint64_t requested, uint32_t frame,
                       uint64_t seed, double band_lo, double band_hi, uint64_t* injected);
/* Push every active particle across the interval [frame*mhd_dt,
 * frame*mhd_dt + mhd_dt) between tables `lower` and `upper` (same kind,
 * precision and grid).  Noise: Philox keyed (seed, index, frame, 2).
 * Replaces move_parker_particles_one_interval / move_particles_one_interval
 * (src/main.cpp:1084-1327, :1334-1755).  stats (optional) synchronises the
 * stream and receives the counters.  With the learned closure on the tcgen05
 * engine the call always synchronises (stats or not) and reads the counters
 * back, so a timed-out tensor-core completion wait is always reported
 * (KPT_ERROR_CUDA with the message; the push's results are then invalid). */
int kpt_push_interval(kpt_context* ctx, kpt_particles* particles, const kpt_field* lower,
                      const kpt_field* upper, const kpt_settings* settings, uint32_t frame,
                      uint64_t seed, kpt_push_stats* stats);
/* Momentum-threshold split, children appended in parent-index order. */
int kpt_split(kpt_context* ctx, kpt_particles* particles, const kpt_settings* settings,
              uint64_t* split, uint64_t* skipped);
/* Weight histogram of active particles over nbins log bins of [pmin, pmax]. */
int kpt_histogram(kpt_context* ctx, const kpt_particles* particles, double pmin, double pmax,
                  int nbins, double* bins);
int kpt_summarize(kpt_context* ctx, const kpt_particles* particles, kpt_summary* out);

/* Summary of particles in caller-owned device arrays, allocating nothing.
 * No counterpart in the reference: it serves callers that cannot allocate
 * device memory (a host application that owns all device memory through its
 * own pool or arena, or code that must not call cudaMalloc while other work
 * is being captured or timed).  Same result as kpt_summarize.  Its scratch is
 * one fixed device array of the library (about 0.7 MB per GPU, held until
 * the process exits), so count is limited to 16,777,216 particles
 * (KPT_ERROR_CAPACITY above that).  The first call in each CUDA context
 * looks up the array's device address in that context (kept under the
 * context's unique id, so a second context on a device, or a context
 * recreated after cudaDeviceReset, looks it up afresh), so make that first
 * call before any stream capture.  All calls
 * share the array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  Runs on cuda_stream
 * (NULL = legacy default stream) and synchronises it. */
int kpt_summarize_noalloc(const kpt_particle_arrays* arrays, uint64_t count, void* cuda_stream,
                          kpt_summary* out);

/* Interpolated table values at n host positions (x, y) and interval
 * fraction rt (parity and diagnostics); out is n x components float64. */
int kpt_sample_table(kpt_context* ctx, const kpt_field* lower, const kpt_field* upper,
                     uint64_t n, const double* x, const double* y, const double* rt,
                     int time_interpolation, double* out);

/* ======================================================================
 * Header-library step API (ParkerSolver / ParticleSystem), 2D Cartesian
 * grids with uniform (analytic) axes, FP64.  Same semantics as the
 * reference's templates; where the reference calls Kokkos::abort or throws,
 * these return KPT_ERROR_INVALID_ARGUMENT with the reference's message.
 * ====================================================================== */

/* ParticleProperties (ParticleSystem.hpp:145-160), dimensionless. */
typedef struct kpt_particle_properties {
    double rest_mass;
    double charge;
    double speed_of_light;
    double energy_scale_erg;
} kpt_particle_properties;

/* ParticleSplittingPolicy (ParticleSystem.hpp:280-295). */
typedef struct kpt_split_policy {
    double energy_split_ratio;   /* > 1 (reference default 2) */
    double minimum_child_weight; /* >= 0 */
} kpt_split_policy;

/* ParticleSplitStatistics (ParticleSystem.hpp:269-275). */
typedef struct kpt_split_statistics {
    uint64_t active_count;
    uint64_t split_count;
    uint64_t skipped_capacity_count;
    uint64_t skipped_invalid_baseline_count;
    uint64_t skipped_minimum_weight_count;
} kpt_split_statistics;

/* ParticleSystem<2> storage (ParticleSystem.hpp:340-350): host arrays for
 * upload/download, n entries each. */
typedef struct kpt_system_arrays {
    uint64_t* id;
    double* x;
    double* y;
    double* prev_x;
    double* prev_y;
    double* prevstep_x;
    double* prevstep_y;
    double* p;
    double* mu;
    double* weight;
    double* e0; /* initial_kinetic_energy */
    int32_t* status;
    int32_t* split_level;
    int32_t* sort_key;
} kpt_system_arrays;

/* PitchAngleScatteringParameters (LegencyModel.hpp:196-221). */
typedef struct kpt_scattering_parameters {
    double spectral_index;      /* > 1 (default 5/3) */
    double h0;                  /* resonance regularisation (default 1e-6) */
    double minimum_magnetic_field_magnitude;
    double minimum_sigma2;
    double minimum_correlation_length;
    double minimum_speed;
} kpt_scattering_parameters;

typedef struct kpt_grid kpt_grid;
typedef struct kpt_system kpt_system;
typedef struct kpt_parker_solver kpt_parker_solver;
typedef struct kpt_focus_solver kpt_focus_solver;

/* Uniform 2D Cartesian grid with two ghost layers (Grid.hpp:65,
 * AnalyticCoordinateGrid.hpp); edges nx+1 / ny+1 must be uniform (the field
 * reader's test, AthenaFieldReader.hpp:167-193); periodic[2] per axis. */
int kpt_grid_create(kpt_context* ctx, int nx, int ny, const double* x_edges,
                    const double* y_edges, const int32_t* periodic, kpt_grid** out);
/* StoredCoordinateGrid(metadata, face_coordinates) through
 * GridValidation::make_validated_stored_coordinate_grid
 * (StoredCoordinateGrid.hpp:53-66, GridValidation.hpp:773-784): a 2D
 * Cartesian grid on explicit, possibly non-uniform face coordinates.
 * x_faces / y_faces hold nx+5 / ny+5 faces in storage order, face -2 first
 * (the two ghost faces on each side included), strictly ascending; the
 * reference's validation messages on failure.  Every library call that takes
 * a kpt_grid accepts it: the solvers' sampling and limiters, boundary
 * conditions, the generator and the coefficient builders. */
int kpt_grid_create_stored(kpt_context* ctx, int nx, int ny, const double* x_faces,
                           const double* y_faces, const int32_t* periodic, kpt_grid** out);
int kpt_grid_destroy(kpt_grid* grid);

/* ParticleSystem(count, capacity, properties, policy) with
 * initialize_default_state (ParticleSystem.hpp:370-395, :1163-1198). */
int kpt_system_create(kpt_context* ctx, uint64_t count, uint64_t capacity,
                      const kpt_particle_properties* properties, const kpt_split_policy* policy,
                      kpt_system** out);
int kpt_system_destroy(kpt_system* system);
int kpt_system_count(const kpt_system* system, uint64_t* count, uint64_t* capacity);
int kpt_system_set_count(kpt_system* system, uint64_t count);
int kpt_system_upload(kpt_system* system, uint64_t n, const kpt_system_arrays* host);
int kpt_system_download(const kpt_system* system, uint64_t n, const kpt_system_arrays* host);
/* capture_previous_positions (ParticleSystem.hpp:623-629). */
int kpt_system_capture_previous_positions(kpt_context* ctx, kpt_system* system);
/* apply_grid_boundary_conditions, physical domain (ParticleSystem.hpp:653-699). */
int kpt_system_apply_boundary(kpt_context* ctx, kpt_system* system, const kpt_grid* grid);
/* sort_by_key(minimum_key, maximum_key) (ParticleSystem.hpp:723-759): a
 * stable sort, so equal keys keep index order (the reference's BinSort
 * leaves that order to its threads). */
int kpt_system_sort_by_key(kpt_context* ctx, kpt_system* system, int32_t minimum_key,
                           int32_t maximum_key);
/* compact_active_particles (ParticleSystem.hpp:768-789). */
int kpt_system_compact(kpt_context* ctx, kpt_system* system, uint64_t* active_count);
/* split_particles_on_energy_growth (ParticleSystem.hpp:791-905); children
 * in parent-index order (the serial order; the reference's atomics leave it
 * to its threads). */
int kpt_system_split_energy(kpt_context* ctx, kpt_system* system, kpt_split_statistics* out);
/* reset_split_baselines (ParticleSystem.hpp:634-650). */
int kpt_system_reset_split_baselines(kpt_context* ctx, kpt_system* system);

/* ParkerSolver(particles, grid, B, V, coefficients) with the packed
 * coefficient basis (ParkerSolver.hpp:122-198): basis holds, for every
 * ghosted point of the grid (x fastest), 18 values B(3) V(3) drift curl(3)
 * diffusion primary(3) secondary(3) kappa_par_1 kappa_perp_1 div V
 * (ParkerSolver.hpp:96-116); constant_ratio selects the constant
 * kappa_perp/kappa_par branch (secondary ignored).  courant: SolverBase's
 * courant_scale (default 0.3). */
int kpt_parker_solver_create(kpt_context* ctx, const kpt_grid* grid, const double* basis,
                             int constant_ratio, double courant, kpt_parker_solver** out);
int kpt_parker_solver_destroy(kpt_parker_solver* solver);
/* set_coefficient_fields (ParkerSolver.hpp:157-163). */
int kpt_parker_solver_set_basis(kpt_parker_solver* solver, const double* basis,
                                int constant_ratio);
int kpt_parker_solver_set_courant(kpt_parker_solver* solver, double courant);
/* Arithmetic of the steps (no counterpart in the reference, whose solvers
 * are FP64): KPT_PRECISION_F64 (default) follows the reference's FP64
 * arithmetic; KPT_PRECISION_MIXED samples an FP32 copy of the packed basis
 * and forms the terms, the local dt bounds and the Box-Muller noise in FP32,
 * keeping positions, momenta, the global dt and the boundary decisions in
 * FP64 (trajectories within a stated tolerance of the FP64 steps). */
int kpt_parker_solver_set_precision(kpt_parker_solver* solver, int precision);
/* compute_adaptive_time_step (ParkerSolver.hpp:209-222): courant x the
 * minimum local bound over active particles. */
int kpt_parker_compute_time_step(kpt_context* ctx, kpt_parker_solver* solver,
                                 kpt_system* system, double* dt);
/* advance_stochastic / advance_sde (ParkerSolver.hpp:261-294): boundary
 * conditions, adaptive dt, capture_previous_positions, Euler-Maruyama
 * update, boundary conditions.  The noise is the keyed Philox stream of
 * (seed, particle index, step); dt_used may be NULL. */
int kpt_parker_advance_stochastic(kpt_context* ctx, kpt_parker_solver* solver,
                                  kpt_system* system, uint64_t seed, uint32_t step,
                                  double* dt_used);
/* advance_deterministic (ParkerSolver.hpp:229-259). */
int kpt_parker_advance_deterministic(kpt_context* ctx, kpt_parker_solver* solver,
                                     kpt_system* system, double* dt_used);
/* Injected-noise step: advance_stochastic with the four standard normals of
 * every particle slot supplied by the caller instead of drawn from the
 * keyed stream: normals[k * count + i] is normal k of slot i (k = 0, 1, 2:
 * the spatial Wiener increments, 3: the parallel one; ParkerSolver.hpp:
 * 436-477), count = the system's particle count. */
int kpt_parker_advance_with_noise(kpt_context* ctx, kpt_parker_solver* solver,
                                  kpt_system* system, const double* normals, double* dt_used);
/* steps consecutive advance_stochastic calls (steps first_step ..
 * first_step+steps-1) recorded once into a CUDA graph and replayed, the dt
 * staying on the device between steps; dts (optional, steps entries)
 * receives each step's dt.  Same results as the single-step calls.  No
 * counterpart in the reference (a host loop of advance_stochastic). */
int kpt_parker_advance_stochastic_steps(kpt_context* ctx, kpt_parker_solver* solver,
                                        kpt_system* system, uint64_t seed, uint32_t first_step,
                                        uint32_t steps, double* dts);

/* FocusTransportSolver / FocusSolver(particles, grid, B, V, coefficients)
 * with the packed basis (FocusSolver.hpp:106-198): basis holds, for every
 * ghosted point (x fastest), 27 values B(3) b(3) V(3) gradient drift basis(3)
 * curvature drift basis(3) perpendicular diffusion advection(3) |B|
 * kappa_par_1 kappa_perp_1 div V magnetic focusing bb:grad V b.dV/dt sigma^2
 * L_c.  scattering NULL = reference defaults.  Pitch-angle scattering is the
 * slab-QLT closure evaluated four times per step (once for the limiters,
 * three Picard iterations, FocusSolver.hpp:697-740). */
int kpt_focus_solver_create(kpt_context* ctx, const kpt_grid* grid, const double* basis,
                            int constant_ratio, double courant,
                            const kpt_scattering_parameters* scattering,
                            kpt_focus_solver** out);
int kpt_focus_solver_destroy(kpt_focus_solver* solver);
int kpt_focus_solver_set_basis(kpt_focus_solver* solver, const double* basis,
                               int constant_ratio);
int kpt_focus_solver_set_courant(kpt_focus_solver* solver, double courant);
/* As kpt_parker_solver_set_precision; the mixed step also evaluates the
 * slab-QLT closure of the Picard pitch-angle update in FP32. */
int kpt_focus_solver_set_precision(kpt_focus_solver* solver, int precision);
/* set_maximum_pitch_angle_cosine (FocusSolver.hpp:219-226): 0 < value <= 1. */
int kpt_focus_solver_set_maximum_mu(kpt_focus_solver* solver, double maximum_mu);
/* compute_adaptive_time_step (FocusSolver.hpp:240-246). */
int kpt_focus_compute_time_step(kpt_context* ctx, kpt_focus_solver* solver,
                                kpt_system* system, double* dt);
/* advance_stochastic / advance_sde (FocusSolver.hpp:276-301); keyed noise of
 * (seed, particle index, step). */
int kpt_focus_advance_stochastic(kpt_context* ctx, kpt_focus_solver* solver,
                                 kpt_system* system, uint64_t seed, uint32_t step,
                                 double* dt_used);
/* advance_deterministic (FocusSolver.hpp:251-271). */
int kpt_focus_advance_deterministic(kpt_context* ctx, kpt_focus_solver* solver,
                                    kpt_system* system, double* dt_used);
/* Injected-noise step of the focused solver: normals[k * count + i], k = 0,
 * 1, 2 the spatial increments (projected perpendicular to b), 3 the
 * pitch-angle increment (FocusSolver.hpp:641-645, :1612). */
int kpt_focus_advance_with_noise(kpt_context* ctx, kpt_focus_solver* solver, kpt_system* system,
                                 const double* normals, double* dt_used);
/* steps consecutive advance_stochastic calls replayed from one CUDA graph
 * (as kpt_parker_advance_stochastic_steps). */
int kpt_focus_advance_stochastic_steps(kpt_context* ctx, kpt_focus_solver* solver,
                                       kpt_system* system, uint64_t seed, uint32_t first_step,
                                       uint32_t steps, double* dts);

/* ----------------------------------------------------------------------
 * Parker coefficient precompute on the library grid
 * (ParkerCoefficient::make_legacy_transport_coefficient_fields,
 * include/ParkerCoefficient.hpp:1102-1155, with LegencyModel's gamma-one
 * diffusion fields, LegencyModel.hpp:795-898, and FieldOperator's
 * divergence, FieldOperator.hpp:262-277, 487-530) straight into the packed
 * basis the solver samples (ParkerSolver.hpp:514-598).
 * ---------------------------------------------------------------------- */

/* TurbulenceProperties (TurbulenceProperties.hpp:294-484): storage 0 =
 * the constant state of TurbulencePropertyModel::constant_code_units(sigma2,
 * l2d, lslab, lc) (lc <= 0: the slab length); storage 1 = per-point fields
 * (host arrays over the ghosted cells, x fastest) as Field storage holds
 * them (lslab_field unused by the coefficients, may be NULL). */
typedef struct kpt_turbulence {
    int32_t storage;
    int32_t pad;
    double sigma2, l2d, lslab, lc;
    const double* sigma2_field;
    const double* l2d_field;
    const double* lslab_field;
    const double* lc_field;
} kpt_turbulence;

/* LegencyModel::DiffusionModelParameters (LegencyModel.hpp:33-117) plus
 * the drift floor and ghost-fill mode of make_legacy_transport_coefficient_
 * fields. perpendicular_model 0 README formula, 1 constant parallel ratio;
 * ghost_fill_mode 0 PeriodicOrClamped, 1 PeriodicOnly (Field.hpp:20-23). */
typedef struct kpt_diffusion_parameters {
    int32_t perpendicular_model;
    int32_t ghost_fill_mode;
    double parallel_prefactor;
    double perpendicular_prefactor;
    double perpendicular_parallel_ratio;
    double minimum_magnetic_field_magnitude;
    double minimum_solar_wind_speed;
    double minimum_sigma2;
    double minimum_magnetic_field_squared_for_drift;
} kpt_diffusion_parameters;

/* The reference defaults: README formula, 1.622, 0.198, zero floors. */
void kpt_default_diffusion_parameters(kpt_diffusion_parameters* out);

/* Packed Parker basis (grid points x 18, host) from cell-centred B and V
 * (grid points x 3, host, ghost cells as the caller filled them). */
int kpt_parker_coefficients(kpt_context* ctx, const kpt_grid* grid, const double* b,
                            const double* v, const kpt_turbulence* turbulence,
                            const kpt_particle_properties* properties,
                            const kpt_diffusion_parameters* parameters, double* packed);
/* Focused packed basis (grid points x 27, host) from cell-centred B, V and
 * partial_t V (grid points x 3, host; dvdt NULL = zero, the
 * make_legacy_transport_coefficient_fields overload): FocusCoefficient::
 * make_legacy_transport_coefficient_fields_with_time_derivative
 * (FocusCoefficient.hpp:852-993) and FocusSolver's packed layout
 * (FocusSolver.hpp:106-136).  minimum_magnetic_field_magnitude is the
 * builder's floor for b, ln |B| and the drift bases. */
int kpt_focus_coefficients(kpt_context* ctx, const kpt_grid* grid, const double* b,
                           const double* v, const double* dvdt, const kpt_turbulence* turbulence,
                           const kpt_particle_properties* properties,
                           const kpt_diffusion_parameters* parameters,
                           double minimum_magnetic_field_magnitude, double* packed);
/* FocusTransportSolver(particles, grid, B, V, coefficients) with the
 * coefficients built on the device and kept there. */
int kpt_focus_solver_create_from_fields(kpt_context* ctx, const kpt_grid* grid, const double* b,
                                        const double* v, const double* dvdt,
                                        const kpt_turbulence* turbulence,
                                        const kpt_particle_properties* properties,
                                        const kpt_diffusion_parameters* parameters,
                                        double minimum_magnetic_field_magnitude, double courant,
                                        const kpt_scattering_parameters* scattering,
                                        kpt_focus_solver** out);
/* ParkerSolver(particles, grid, B, V, make_legacy_transport_coefficient_
 * fields(...)): the basis is built on the device and stays there. */
int kpt_parker_solver_create_from_fields(kpt_context* ctx, const kpt_grid* grid, const double* b,
                                         const double* v, const kpt_turbulence* turbulence,
                                         const kpt_particle_properties* properties,
                                         const kpt_diffusion_parameters* parameters,
                                         double courant, kpt_parker_solver** out);

/* ======================================================================
 * ParticleGenerator (include/ParticleGenerator.hpp:659-1493): injection and
 * recycling on the library grid.  The reference draws from
 * RandomManager's XorShift pool; here each particle slot draws from its
 * own keyed stream (seed, slot, frame, tag 4), so the results do not depend
 * on thread scheduling.  Particle slot = local index for injection, particle
 * index for recycling (the reference's loop indices).
 * ====================================================================== */

typedef struct kpt_lib_field kpt_lib_field;
typedef struct kpt_candidates kpt_candidates;

enum kpt_centering { KPT_CELL_CENTERED = 0, KPT_FACE_CENTERED = 1 };
enum kpt_grid_domain { KPT_PHYSICAL_DOMAIN = 0, KPT_GHOSTED_DOMAIN = 1 };
/* FieldPredicateComparison (ParticleGenerator.hpp:117-124). */
enum kpt_field_comparison {
    KPT_GREATER = 0, KPT_GREATER_EQUAL = 1, KPT_LESS = 2, KPT_LESS_EQUAL = 3,
    KPT_ABS_GREATER = 4, KPT_ABS_LESS = 5
};
/* ParticleRecycleSelection (ParticleGenerator.hpp:129-133). */
enum kpt_recycle_selection {
    KPT_RECYCLE_ESCAPED_ONLY = 0, KPT_RECYCLE_INACTIVE_ONLY = 1, KPT_RECYCLE_RECYCLABLE = 2
};

/* AxisAlignedParticleRegion<2> (ParticleGenerator.hpp:18-62). */
typedef struct kpt_region {
    double lower[2];
    double upper[2];
} kpt_region;

/* ParticleInjectionKinematics<2> (ParticleGenerator.hpp:68-74); status as
 * ParticleStatus (0 active, 1 escaped, 2 inactive). */
typedef struct kpt_injection_kinematics {
    double momentum_magnitude;
    double mu;
    double weight;
    int32_t status;
    int32_t pad;
} kpt_injection_kinematics;

/* ParticleInjectionPlan (ParticleGenerator.hpp:107-112). */
typedef struct kpt_injection_plan {
    uint64_t first_particle_index;
    uint64_t particle_count;
    uint64_t first_particle_id;
    int32_t max_attempts;
    int32_t pad;
} kpt_injection_plan;

/* FieldThresholdParticlePredicate settings (ParticleGenerator.hpp:255-296). */
typedef struct kpt_field_predicate {
    const kpt_lib_field* field;
    double threshold;
    int32_t comparison;
    int32_t component;
    int32_t domain;
    int32_t pad;
} kpt_field_predicate;

/* Field<Grid, components> (Field.hpp:33-215) on a library grid: values
 * holds `components` doubles per stored point, dim 0 fastest over the
 * ghosted extent of the centering (cells n+4, faces n+5 per axis). */
int kpt_lib_field_create(kpt_context* ctx, const kpt_grid* grid, int32_t components,
                         const int32_t centering[2], const double* values, kpt_lib_field** out);
int kpt_lib_field_destroy(kpt_lib_field* field);
/* Stored points of the field (Field::point_count). */
int kpt_lib_field_points(const kpt_lib_field* field, uint64_t* points);

/* make_particle_region_from_grid (ParticleGenerator.hpp:208-226). */
int kpt_region_from_grid(const kpt_grid* grid, int32_t domain, kpt_region* out);

/* make_field_particle_candidate_set[_in_region] (ParticleGenerator.hpp:
 * 659-784); region NULL = the grid's domain. */
int kpt_candidates_from_field(kpt_context* ctx, const kpt_lib_field* field,
                              const kpt_region* region, double threshold, int32_t comparison,
                              int32_t component, int32_t domain, kpt_candidates** out);
/* make_grid_particle_candidate_set (ParticleGenerator.hpp:786-856). */
int kpt_candidates_from_grid(kpt_context* ctx, const kpt_grid* grid, int32_t domain,
                             kpt_candidates** out);
int kpt_candidates_info(const kpt_candidates* candidates, uint64_t* count, double* total_weight);
/* Candidate point indices (field sets; grid sets give cell ordinals) and
 * cumulative weights, either pointer may be NULL. */
int kpt_candidates_download(kpt_context* ctx, const kpt_candidates* candidates,
                            uint64_t* indices, double* cumulative_weights);
int kpt_candidates_destroy(kpt_candidates* candidates);

/* inject_particles_uniform / inject_particles_uniform_if with the field
 * threshold predicate (predicate NULL: accept all) (ParticleGenerator.hpp:
 * 885-960, :1106-1119). */
int kpt_generator_inject_uniform(kpt_context* ctx, kpt_system* system, uint64_t seed,
                                 uint32_t frame, const kpt_region* region,
                                 const kpt_injection_plan* plan,
                                 const kpt_injection_kinematics* kinematics,
                                 const kpt_field_predicate* predicate);
/* inject_particles_from_field_candidates / _from_grid_candidates
 * (ParticleGenerator.hpp:962-1104); with the candidate builders above this
 * covers inject_particles_uniform_where_field and _uniform_in_grid. */
int kpt_generator_inject_candidates(kpt_context* ctx, kpt_system* system, uint64_t seed,
                                    uint32_t frame, const kpt_candidates* candidates,
                                    const kpt_injection_plan* plan,
                                    const kpt_injection_kinematics* kinematics);
/* recycle_particles_uniform / _uniform_if (ParticleGenerator.hpp:1180-1272);
 * recycled (may be NULL) receives the number of particles rewritten. */
int kpt_generator_recycle_uniform(kpt_context* ctx, kpt_system* system, uint64_t seed,
                                  uint32_t frame, const kpt_region* region,
                                  const kpt_injection_kinematics* kinematics,
                                  const kpt_field_predicate* predicate, int32_t selection,
                                  int32_t max_attempts, uint64_t* recycled);
/* recycle_particles_from_grid_candidates / _from_field_candidates
 * (ParticleGenerator.hpp:1305-1447). */
int kpt_generator_recycle_candidates(kpt_context* ctx, kpt_system* system, uint64_t seed,
                                     uint32_t frame, const kpt_candidates* candidates,
                                     const kpt_injection_kinematics* kinematics,
                                     int32_t selection, uint64_t* recycled);

/* ======================================================================
 * Batched runs (no counterpart in the reference, which runs one simulation
 * per process): many independent driver runs -- each with its own particle
 * store, coefficient tables, settings, seed and frame -- pushed by one
 * persistent launch per interval, the interval loop recorded once into a
 * CUDA graph and replayed.  Results per run are bitwise those of
 * kpt_push_interval on that run (same seed and frame), whatever the batch
 * composition or schedule.  Mixed-precision tables, one transport model per
 * batch, plain closures.
 * ====================================================================== */
typedef struct kpt_batch kpt_batch;

typedef struct kpt_batch_tuning {
    int32_t sort_tile;      /* cell-sort tile (cells), 0 = no sort */
    int32_t blocks_per_sm;  /* resident blocks per SM, 0 = as many as fit */
    int32_t sort_every;     /* sort every k intervals */
    int32_t candidates;     /* schedules timed */
    float best_ms;          /* median time of the chosen schedule over the tuning intervals */
    float spread;           /* (max - min) / median of the chosen schedule's timings */
    int32_t threads_per_block;   /* 64, 128 or 256 */
    int32_t particles_per_lane;  /* 1 or 2 */
    int32_t repeats;        /* timings per candidate */
    int32_t pad;
} kpt_batch_tuning;

int kpt_batch_create(kpt_context* ctx, kpt_batch** out);
int kpt_batch_destroy(kpt_batch* batch);
/* Add a run; its next interval is first_frame.  The store, tables and
 * settings stay owned by the caller and must outlive the batch. */
int kpt_batch_add_run(kpt_batch* batch, kpt_particles* particles, const kpt_field* lower,
                      const kpt_field* upper, const kpt_settings* settings, uint64_t seed,
                      uint32_t first_frame, int* run_index);
int kpt_batch_set_schedule(kpt_batch* batch, int sort_tile, int blocks_per_sm, int sort_every);
int kpt_batch_get_schedule(const kpt_batch* batch, int* sort_tile, int* blocks_per_sm,
                           int* sort_every);
/* Launch shape of the batched push: threads per block (64, 128 or 256) and
 * particles per lane (1 or 2: a lane advances that many particles side by
 * side, each slot refilling from the work cursor on its own).  Results do not
 * depend on the shape (noise is keyed by particle). */
int kpt_batch_set_launch_shape(kpt_batch* batch, int threads_per_block, int particles_per_lane);
int kpt_batch_get_launch_shape(const kpt_batch* batch, int* threads_per_block,
                               int* particles_per_lane);
/* Push every run through `intervals` consecutive intervals (graph replay when
 * use_graph != 0 and the context's stream can be captured). */
int kpt_batch_run(kpt_batch* batch, uint32_t intervals, int use_graph);
/* Counters of a run's last interval. */
int kpt_batch_stats(const kpt_batch* batch, int run, kpt_push_stats* out);
/* A run's next interval (get / set). */
int kpt_batch_frame(const kpt_batch* batch, int run, uint32_t* frame);
int kpt_batch_set_frame(kpt_batch* batch, int run, uint32_t frame);
/* Time candidate schedules over `intervals` intervals on the current state,
 * restoring the state after each timing, and keep the fastest (median of
 * three timings per candidate).  Stage 1: cell-sort tile 0/8/16/32 and sort
 * every 1 or 2 intervals, at 128 threads, one particle per lane, all resident
 * blocks.  Stage 2, with the chosen sort: 64/128/256 threads per block x 1 or
 * 2 particles per lane x residency (all that fit, or the threads of 3 or 2
 * blocks of 128). */
int kpt_batch_autotune(kpt_batch* batch, uint32_t intervals, kpt_batch_tuning* out);

#ifdef __cplusplus
}
#endif

#endif
