// Internal interfaces between the C-ABI layer (kpt_api.cpp) and the kernel
// translation units.  Host-only code may include this header.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kpt_surrogate.cuh"
#include "kpt_types.h"

namespace kpt {

enum Precision : int { kPrecisionF64 = 0, kPrecisionMixed = 1 };
enum Schedule : int { kScheduleRefill = 0, kScheduleSimple = 1 };

// Table elements per point for a kind/precision (FP64 rows are 16-byte
// aligned and streamed with 128/256-bit loads).
inline int table_stride(int focused, int precision) {
    if (!focused) {
        return 16;
    }
    return precision == kPrecisionF64 ? 22 : 24;
}

// Layout of the FP32 tables.  FP64 tables are point-major rows of
// table_stride doubles.  An FP32 table is cut into planes of
// table_plane_floats(focused) floats per point, plane after plane: Parker
// tables are chunk-major (two planes of 8 floats: lanes sampling
// x-neighbouring points read neighbouring 32-byte sectors of one cache
// line), focused tables keep one plane of whole 24-float rows (their
// particles stream along x and rarely share lines, while a row then spans
// one or two lines instead of three).  Component c of point p sits at
// table_f32_offset.
__host__ __device__ constexpr int table_plane_floats(bool focused) { return focused ? 24 : 8; }
__host__ __device__ inline size_t table_f32_offset(bool focused, size_t points, size_t p, int c) {
    const int w = table_plane_floats(focused);
    return (static_cast<size_t>(c / w) * points + p) * w + c % w;
}

// Cell records of a pair of FP32 tables (the frames at the interval's two
// ends), for the mixed pushes.  The record of a cell is indexed by its
// lower-left ghosted point p and is made of 128-byte lines of four 32-byte
// sectors.  Line m holds frame m % 2 (lower, upper) of the component pairs
// 4 (m / 2) .. 4 (m / 2) + 3; the sector of pair k holds components 2k and
// 2k + 1 at the cell's corners p, p + 1, p + ex, p + ex + 1, pair by pair --
// the operands of the packed-pair interpolation, in the order the
// point-major sampler accumulates them.  Four lanes then read one line of a
// particle's record per request (four lines for the point-major rows), and
// a lane interpolates a component pair from its own two sectors.
// Components past the last are zero padding.
__host__ __device__ constexpr int record_sectors(bool focused) { return focused ? 24 : 16; }
__host__ __device__ constexpr int record_floats(bool focused) {
    return 8 * record_sectors(focused);
}

struct RecordLaunch {
    const float* lower;
    const float* upper;
    float* records;  // points x record_floats(focused)
    uint64_t points;
    int ex, ey;      // ghosted extents
    int focused;
};
cudaError_t launch_build_records(const RecordLaunch& launch, cudaStream_t stream);

struct PushLaunch {
    Grid grid;
    FixedGrid fixed;
    const uint32_t* order;  // optional permutation of [0, count) (cell sort)
    const void* lower;
    const void* upper;
    ParticleArrays parts;
    uint64_t count;
    DeviceSettings settings;
    double interval_start;
    double interval_end;
    uint32_t frame;
    uint64_t seed;
    PushCounters* counters;
    int precision;
    int focused;
    int schedule;
    int sm_count;
    int blocks_per_sm;
    int fp64_contracted;  // FP64 push: 0 strict rounding (oracle-exact), 1 FMA contraction
    // learned closure (mixed focused push only); nullptr = plain closures
    const SurrogateDevice* surrogate;
    // cell records of (lower, upper) for the mixed pushes; nullptr = sample
    // the point-major tables (the same values, bit for bit)
    const float* records;
};

cudaError_t launch_push_interval(const PushLaunch& launch, cudaStream_t stream);
// The plain FP64 push and FP64 table sampling, built in their own translation
// unit without FMA contraction (kpt_push_f64.cu).
cudaError_t launch_push_interval_f64(const PushLaunch& launch, cudaStream_t stream);
// The plain FP64 push with FMA contraction and CUDA's pow (kpt_push.cu).
cudaError_t launch_push_interval_f64_contracted(const PushLaunch& launch, cudaStream_t stream);
struct SampleLaunch;
cudaError_t launch_sample_f64(const SampleLaunch& launch, int blocks, cudaStream_t stream);

// Batched mixed-precision push over many independent runs (one launch).
// params: device array of per-run parameter blocks (push_params_size()
// bytes each, built by build_push_params); offsets: runs + 1 prefix sums of
// the runs' particle counts; cursor: one device word.
struct BatchLaunch {
    void* params;
    const uint64_t* offsets;
    int runs;
    int focused;
    unsigned long long* cursor;
    int sm_count;
    int blocks_per_sm;       // resident blocks per SM, 0 = as many as fit
    int threads;             // threads per block: 64, 128 or 256
    int particles_per_lane;  // particles a lane advances side by side: 1 or 2
    int records;             // every run's PushParams carries cell records
};
// The launch shapes the batched push is built for.
bool batch_shape_supported(int threads, int particles_per_lane);
size_t push_params_size();
void build_push_params(const PushLaunch& launch, void* out);
cudaError_t launch_push_batch(const BatchLaunch& launch, cudaStream_t stream);
cudaError_t launch_batch_next_frame(const BatchLaunch& launch, cudaStream_t stream);
int batch_max_runs();

// Coefficient table from cell-centred B and V (3 x ny x nx each, device).
struct TableLaunch {
    Grid grid;
    const double* b_cells;
    const double* v_cells;
    void* table;
    int focused;
    int precision;
};
cudaError_t launch_build_table(const TableLaunch& launch, cudaStream_t stream);

struct InjectLaunch {
    ParticleArrays parts;
    uint64_t first;
    uint64_t n;
    double x_lower, x_upper, y_lower, y_upper;
    double p0, interval_start, mhd_dt, dt_min, mu_max;
    uint32_t frame;
    uint64_t seed;
};
cudaError_t launch_inject(const InjectLaunch& launch, cudaStream_t stream);

// Split scratch: per-block counts (one per 1024 particles) and a 2-word
// result {children wanted, children written}.
struct SplitLaunch {
    ParticleArrays parts;
    uint64_t count;
    uint64_t capacity;
    const double* thresholds;  // per split level, host-computed
    const double* weights;     // 0.5^(level+1) per level
    int level_count;
    double pmax;
    unsigned int* block_counts;
    unsigned long long* block_offsets;
    unsigned long long* totals;
};
size_t split_scratch_blocks(uint64_t count);
cudaError_t launch_split(const SplitLaunch& launch, cudaStream_t stream);

struct HistogramLaunch {
    const double* p;
    const double* weight;
    const int32_t* status;
    uint64_t count;
    double pmin, pmax, log_pmin, inv_dlogp;
    int nbins;
    double* bins;                       // nbins, zeroed by the kernel launcher
    unsigned long long* edge_count;     // near-edge particles set aside
    unsigned int* edge_index;           // capacity >= count
};
cudaError_t launch_histogram(const HistogramLaunch& launch, cudaStream_t stream);

struct SummaryPartial {
    unsigned long long active;
    unsigned long long inactive;
    double weight_sum, p_sum, dt_sum;
    double p_min, p_max, dt_min, dt_max;
    int max_level;
    int pad;
};
struct SummaryLaunch {
    const double* p;
    const double* dt;
    const double* weight;
    const int32_t* status;
    const int32_t* level;
    uint64_t count;
    SummaryPartial* partials;  // summary_blocks(count) entries
    SummaryPartial* result;    // one entry
};
int summary_blocks(uint64_t count);
cudaError_t launch_summary(const SummaryLaunch& launch, cudaStream_t stream);
// Summary with its scratch in a fixed device array (no allocation); fills
// *host (pageable host memory) and synchronises the stream.
unsigned long long noalloc_summary_max_particles();
cudaError_t noalloc_summary(const SummaryLaunch& launch, cudaStream_t stream,
                            SummaryPartial* host);

// Counting sort of particle indices by spatial tile (inactive particles
// last).  counts/offsets hold tiles + 1 entries.
struct SortLaunch {
    Grid grid;
    ParticleArrays parts;
    uint64_t count;
    int tile_x, tile_y, tiles_x, tiles_y;
    unsigned int* keys;     // count
    unsigned int* counts;   // tiles + 1
    unsigned int* order;    // count
};
cudaError_t launch_sort(const SortLaunch& launch, cudaStream_t stream);
// v4 snapshot records (25 words each) of particles [0, count).
cudaError_t launch_pack_records(const ParticleArrays& a, uint64_t count, double e0,
                                uint32_t* out, cudaStream_t stream);

struct SurrogateTrainLaunch {
    const float* x;   // n x 5 raw features
    const float* t;   // n x 3 raw targets
    int n;
    uint64_t seed;
    int batch;
    SurrogateBox box;
    float* params;
    float* grad;
    float* m;
    float* v;
    float* xb;        // batch x 5 normalised inputs
    float* h1;        // batch x 64
    float* h2;
    float* g1;
    float* g2;
    float* gy;        // batch x 3
    float* loss;      // one float per step
    float* partial;   // ceil(batch / kGradChunk) x parameter-count gradient partials
    float beta1, beta2, lr;
    int quant;        // rounding emulated from step quant_from on: 0 none, 1 BF16, 2 FP16
    int quant_from;
};
constexpr int kGradChunk = 256;
cudaError_t surrogate_make_samples(uint64_t seed, int n, const SurrogateBox& box, float* x,
                                   float* t, cudaStream_t stream);
cudaError_t surrogate_train_step(const SurrogateTrainLaunch& launch, int step,
                                 cudaStream_t stream);
// Gradient of the loss over the first `batch` samples in order (step < 0).
cudaError_t surrogate_gradient(const SurrogateTrainLaunch& launch, cudaStream_t stream);
// Raw inputs (n x 5, device) -> D_mumu, dD_mumu/dmu, ln kappa_parallel
// (n x 3, device); served[i] = 1 where the network answered.
// How the network is served by surrogate_eval: engine -1 = the FP32 SIMT
// forward, kEngineMmaSync / kEngineTcgen05 = the tensor-core paths of the
// push; timeouts counts blocks stopped by a tcgen05 completion timeout.
struct SurrogateServe {
    const float* params;
    const uint2* block;
    const uint4* tc_block;
    int engine;
    unsigned int* timeouts;
};
cudaError_t surrogate_eval(int n, const double* inputs, const SurrogateBox& box,
                           const SurrogateServe& serve, double* out, int* served,
                           cudaStream_t stream);
// out[0]: blocks whose bounded completion wait timed out; out[1]: blocks that
// finished their teardown (a width-64 block of weights).
cudaError_t surrogate_tc_timeout_check(const uint4* block, int blocks, uint32_t polls,
                                       unsigned int* out, cudaStream_t stream);

// ---- header library (ParkerSolver / ParticleSystem), 2D Cartesian ---------
// One axis of an analytic uniform grid (AnalyticCoordinateGrid.hpp) with the
// MappedCoordinateGrid bound caches (MappedCoordinateGrid.hpp:118-147).
struct LibAxis {
    int n;
    int periodic;
    double x0, dx;                    // analytic uniform axis: face i at x0 + i dx
    double inv_dx;                    // 1 / dx (the mixed library step's stencil)
    double lower, upper;              // faces 0 and n
    double ghost_lower, ghost_upper;  // faces -2 and n+2
    double width, inv_width;          // periodic width (upper - lower) and 1/width
    // stored axis (StoredCoordinateGrid): explicit coordinates on the device,
    // storage index = logical index + 2; n + 5 faces, n + 4 cell centres
    int stored;
    const double* faces;
    const double* cells;
};
struct LibGrid {
    LibAxis axis[2];
    int ex;  // nx + 4 (ghosted points per row)
};

// ParticleSystem storage (ParticleSystem.hpp:340-350), SpaceDim 2.
struct SystemArrays {
    uint64_t* id;
    double *x, *y, *prev_x, *prev_y, *prevstep_x, *prevstep_y, *p, *mu, *weight, *e0;
    int *status, *split_level, *sort_key;
};

// Packed Parker coefficient basis (ParkerSolver.hpp:96-116) for VecDim 3:
// B(3) V(3) drift curl(3) primary(3) secondary(3) kappa_par kappa_perp divV.
constexpr int kLibBasis = 18;
constexpr int kLibBasisStride = 18;
constexpr int kLibBasisStrideF32 = 20;  // FP32 copy: rows of five 16-byte chunks
constexpr int kLibTermCount = 9;

struct LibParkerLaunch {
    LibGrid grid;
    const double* basis;      // ghosted points x kLibBasisStride
    const float* basis_f32;   // mixed step: ghosted points x kLibBasisStrideF32
    int mixed;                // 1: FP32 basis, terms and noise; FP64 positions and momenta
    int constant_ratio;
    SystemArrays sys;
    uint64_t count, capacity;
    double rest_mass, charge, speed_of_light, mc;
    double courant;
    double* terms;                  // count x kLibTermCount
    unsigned long long* min_bits;   // global minimum of the local dt bounds
    double* dt_device_out;          // courant * min (device)
    double* dt_history;             // optional per-step record (device)
    const double* dt_device;        // advance: dt read from the device
    double dt;
    int apply_boundary;             // boundary conditions before the terms
    int advance;                    // run the update pass
    int stochastic;
    int capture;                    // rotate previous positions
    uint2 key;
    uint32_t frame;
    const double* noise;            // caller normals [4][count] instead of the keyed stream
    int* error;                     // first abort condition met (code)
    unsigned long long* error_index;
};
cudaError_t lib_parker_step(const LibParkerLaunch& launch, cudaStream_t stream);
// FP32 copy of a packed basis (rows rounded, padded with zeros to dst_stride).
cudaError_t lib_basis_to_f32(const double* src, int src_stride, float* dst, int dst_stride,
                             int comps, uint64_t points, cudaStream_t stream);

// Packed focused basis (FocusSolver.hpp:106-136) for VecDim 3: B(3) b(3)
// V(3) gradient drift(3) curvature drift(3) perpendicular diffusion
// advection(3) |B| kappa_par kappa_perp divV focusing bb:gradV b.dV/dt
// sigma^2 Lc; rows padded to 28 doubles (16-byte aligned).
constexpr int kFocusBasis = 27;
constexpr int kFocusBasisStride = 28;
constexpr int kFocusBasisStrideF32 = 28;  // FP32 copy: rows of seven 16-byte chunks
constexpr int kFocusTermCount = 18;

struct LibFocusLaunch {
    LibGrid grid;
    const double* basis;      // ghosted points x kFocusBasisStride
    const float* basis_f32;   // mixed step: ghosted points x kFocusBasisStrideF32
    int mixed;                // 1: FP32 basis, terms, closure and noise; FP64 state
    int constant_ratio;
    SystemArrays sys;
    uint64_t count, capacity;
    double rest_mass, charge, abs_charge, speed_of_light, mc;
    double gk, h0, qlt_norm, min_b, min_sigma2, min_lc, min_speed, max_mu;
    double courant;
    double* terms;  // count x kFocusTermCount
    unsigned long long* min_bits;
    double* dt_device_out;
    double* dt_history;
    const double* dt_device;
    double dt;
    int apply_boundary, advance, stochastic, capture;
    uint2 key;
    uint32_t frame;
    const double* noise;  // caller normals [4][count] instead of the keyed stream
    int* error;
    unsigned long long* error_index;
};
cudaError_t lib_focus_step(const LibFocusLaunch& launch, cudaStream_t stream);

struct LibSplitLaunch {
    SystemArrays sys;
    uint64_t count, capacity;
    double rest_mass, speed_of_light, mc;
    double split_ratio, log_split_ratio, min_child_weight;
    int* flags;                    // count
    unsigned int* block_counts;    // one per 256 particles
    unsigned long long* tallies;   // active, skipped capacity, invalid baseline, min weight, wanted
};
cudaError_t system_split(const LibSplitLaunch& launch, cudaStream_t stream);
cudaError_t system_reset_baselines(const LibSplitLaunch& launch, cudaStream_t stream);

struct LibSortLaunch {
    SystemArrays sys;
    uint64_t count;
    int lo, hi;
    unsigned int *keys_a, *keys_b, *idx_a, *idx_b;
    unsigned int* hist;            // 256 x blocks
    unsigned long long* scratch_total;
    void* staging;                 // count x 8 bytes
};
cudaError_t system_sort(const LibSortLaunch& launch, cudaStream_t stream);
cudaError_t system_default_state(const SystemArrays& s, uint64_t count, uint64_t capacity,
                                 cudaStream_t stream);
cudaError_t system_boundary(const LibGrid& g, const SystemArrays& s, uint64_t count,
                            cudaStream_t stream);
cudaError_t system_capture(const SystemArrays& s, uint64_t capacity, cudaStream_t stream);
cudaError_t system_compact_keys(const SystemArrays& s, uint64_t count,
                                unsigned long long* active, cudaStream_t stream);

// ParticleGenerator (ParticleGenerator.hpp): a lattice field on the library
// grid (Field.hpp:33-215): `components` doubles per stored point, dim 0
// fastest over the ghosted extent of the field's centering (cells n+4,
// faces n+5; logical index -2 first).
struct GenField {
    const double* values;
    int components;
    int centering[2];  // 0 cell centred, 1 face centred
    int ext[2];
};

// FieldThresholdParticlePredicate (ParticleGenerator.hpp:255-358).
struct GenPredicate {
    int enabled;  // 0: AlwaysAcceptParticlePredicate
    GenField field;
    double threshold;
    int comparison, component, domain;
};

// Field or grid candidate set (ParticleGenerator.hpp:464-646).
struct GenCandidates {
    int kind;                    // 0 field points, 1 grid cells
    const uint64_t* indices;     // field point indices (kind 0)
    const double* cumulative;    // cumulative physical-volume weights
    uint64_t count;
    double total;
    int lower[2], extents[2];    // grid cells (kind 1)
    GenField field;              // centering and extents (kind 0)
};

struct GenLaunch {
    LibGrid grid;
    SystemArrays sys;
    int recycle;                 // 0 inject over a plan, 1 recycle selected particles
    int source;                  // 0 region sampling with predicate, 1 candidates
    double region_lo[2], region_hi[2];
    GenPredicate predicate;
    GenCandidates candidates;
    uint64_t first_index, count, first_id;  // inject: plan; recycle: count = particle count
    int max_attempts;
    int selection;               // ParticleRecycleSelection
    double momentum, mu, weight;
    int status;
    double rest_mass, speed_of_light, mc;
    uint2 key;
    uint32_t frame;
    unsigned long long* recycled;  // particles written by a recycle call
};
cudaError_t generator_run(const GenLaunch& launch, cudaStream_t stream);

// Field candidates: stable compaction of the points passing the predicate
// inside the region, then their cumulative cell volumes.  count_out is a
// device word; block_counts holds one entry per 256 points.
struct GenCandidateBuild {
    LibGrid grid;
    GenField field;
    double region_lo[2], region_hi[2];
    double threshold;
    int comparison, component, domain;
    uint64_t points;
    uint64_t* indices;           // points (upper bound)
    double* cumulative;          // points (upper bound)
    unsigned int* block_counts;  // (points + 255) / 256
    unsigned long long* count_out;
    double* block_sums;          // scan scratch
};
cudaError_t generator_field_candidates(const GenCandidateBuild& build, cudaStream_t stream);
cudaError_t generator_field_weights(const GenCandidateBuild& build, uint64_t count,
                                    cudaStream_t stream);
// Grid candidates: cumulative cell volumes of the domain's cells in order.
cudaError_t generator_grid_weights(const LibGrid& grid, const int lower[2], const int extents[2],
                                   uint64_t count, double* cumulative, double* block_sums,
                                   cudaStream_t stream);
// Scratch doubles generator_*_weights need for count candidates.
uint64_t generator_scan_scratch(uint64_t count);

// Parker coefficient precompute (ParkerCoefficient.hpp:1102-1155) into the
// packed basis (ParkerSolver.hpp:514-598) on the library grid: cell-centred
// B and V (3 doubles per ghosted point) in, kLibBasisStride doubles per
// point out.
struct CoefLaunch {
    LibGrid grid;
    const double* b;
    const double* v;
    int turbulence_fields;          // 0 constant state, 1 per-point fields
    double sigma2, l2d, lc;         // constant state (lc already resolved)
    const double* sigma2_field;     // per point (turbulence_fields = 1)
    const double* l2d_field;
    const double* lc_field;
    double abs_charge, rest_mass, speed_of_light;
    int constant_ratio;
    double parallel_prefactor, perpendicular_prefactor, ratio;
    double min_b, min_vsw, min_sigma2;
    double drift_floor;
    int ghost_mode;                 // 0 PeriodicOrClamped, 1 PeriodicOnly
    double* packed;
    int stride;                     // packed row length
    int kpar_slot, kperp_slot;      // gamma-one kappas in the packed row
    int* error;                     // failed check (device), parker_coefficients_no_error() if none
    // focused transport only
    const double* dvdt;             // partial_t V (3 per point) or nullptr (zero)
    double direction_floor;         // the builder's minimum |B| (direction, ln |B|, drifts)
    double* scratch;                // 8 doubles per point: ln|B|, grad ln|B| (3), curvature (3)
};
cudaError_t parker_coefficients(const CoefLaunch& launch, cudaStream_t stream);
// FocusCoefficient::make_legacy_transport_coefficient_fields_with_time_
// derivative (FocusCoefficient.hpp:852-993) into the focused packed basis
// (FocusSolver.hpp:106-136, :504-585), kFocusBasisStride doubles per point.
cudaError_t focus_coefficients(const CoefLaunch& launch, cudaStream_t stream);
int parker_coefficients_no_error();

struct SampleLaunch {
    Grid grid;
    const void* lower;
    const void* upper;
    const double* x;
    const double* y;
    const double* rt;
    uint64_t n;
    double shift_x, shift_y;
    int time_interpolation;
    int focused;
    int precision;
    double* out;
};
cudaError_t launch_sample(const SampleLaunch& launch, cudaStream_t stream);

// FP64 FMA throughput of the current device in TFLOP/s (best of five timed
// launches of a project-written FMA-chain kernel on `stream`).
cudaError_t fp64_fma_rate(int sm_count, cudaStream_t stream, double* tflops);
// out[i] = kpt_pow(x[i], y[i]) on the device (device arrays).
cudaError_t launch_pow(uint64_t n, const double* x, const double* y, double* out, int sm_count,
                       cudaStream_t stream);

}  // namespace kpt
