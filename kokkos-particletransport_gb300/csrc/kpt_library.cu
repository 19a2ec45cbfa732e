// The header library's step API on the GPU: ParkerSolver's lockstep
// global-dt step (include/ParkerSolver.hpp:209-294, kernels :443-477,
// :771-875, :956-1007, :1147-1174, :1477-1520) and the ParticleSystem
// lifecycle (include/ParticleSystem.hpp:623-917), on a 2D Cartesian grid with
// analytic uniform axes.  FP64 throughout, evaluation order as written in the
// reference; index arithmetic with explicit rounding so the branch decisions
// (wrap, cell index, stencil) match the reference bit for bit.
//
// One step is two kernels.  The first applies the boundary conditions,
// samples the packed coefficient basis once per particle, keeps the terms the
// update needs (coordinate rates, momentum rate, kappa_par, kappa_perp, the
// field direction, |p|) and folds the local stable time step into a global
// minimum (an atomic min on the bit pattern of a positive double, exact and
// order independent).  The second rotates the previous positions, draws the
// noise, updates every active particle from the kept terms and applies the
// boundary conditions again.  The reference evaluates the same terms twice
// (once for dt, once for the update) from the same positions; keeping them
// gives the same numbers with one gather pass instead of two.
#include <cuda_runtime.h>

#include <cstdint>

#include "kpt_device.cuh"
#include "kpt_internal.h"

namespace kpt {
namespace {

constexpr double kLargeTimeStep = 1.0e300;

// MappedCoordinateGrid::wrap_coordinate (MappedCoordinateGrid.hpp:294-315).
__device__ __forceinline__ double lib_wrap(const LibAxis& a, double x) {
    if (!a.periodic) {
        return x;
    }
    double wrapped = __dsub_rn(
        x, __dmul_rn(floor(__dmul_rn(__dsub_rn(x, a.lower), a.inv_width)), a.width));
    if (wrapped >= a.upper) {
        wrapped = __dsub_rn(wrapped, a.width);
    }
    if (wrapped < a.lower) {
        wrapped = __dadd_rn(wrapped, a.width);
    }
    return wrapped;
}

__device__ __forceinline__ bool lib_contains(double lower, double upper, double x) {
    return x >= lower && x <= upper;
}

// Face coordinate of logical index i: analytic uniform x0 + i dx
// (AnalyticCoordinateGrid.hpp:167-171), or the stored face
// (StoredCoordinateGrid.hpp:108-113).
__device__ __forceinline__ double lib_face(const LibAxis& a, double i) {
    if (a.stored) return a.faces[static_cast<int>(i) + 2];
    return __dadd_rn(a.x0, __dmul_rn(i, a.dx));
}

// StoredCoordinateGrid::cell_index (StoredCoordinateGrid.hpp:301-341): the
// cell [face k, face k + 1) holding x, cells lower_cell .. upper_cell of a
// domain whose faces span [lower_x, upper_x].  The interval is unique (faces
// ascend), so the bisection finds the reference's cell.
__device__ int stored_cell_index(const LibAxis& a, double x, int lower_cell, int upper_cell,
                                 double lower_x, double upper_x) {
    if (x < lower_x) return lower_cell - 1;
    if (x > upper_x) return upper_cell + 1;
    if (x == upper_x) return upper_cell;
    int left = lower_cell;
    int right = upper_cell;
    while (left <= right) {
        const int mid = left + (right - left) / 2;
        const double face_left = a.faces[mid + 2];
        const double face_right = a.faces[mid + 3];
        if (x >= face_left && x < face_right) return mid;
        if (x < face_left) {
            right = mid - 1;
        } else {
            left = mid + 1;
        }
    }
    return x < lower_x ? lower_cell - 1 : upper_cell + 1;
}

// StoredCoordinateGrid::grid_index over the ghosted domain
// (StoredCoordinateGrid.hpp:130-174): the logical index of x between the
// stored coordinates (cell centres -2 .. n+1, or faces -2 .. n+2),
// extrapolated linearly from the end intervals.
__device__ double stored_grid_index(const LibAxis& a, double x, bool faces) {
    const double* c = faces ? a.faces : a.cells;
    const int lower_index = -2;
    const int upper_index = faces ? a.n + 2 : a.n + 1;
    int left = lower_index;
    if (x <= c[lower_index + 2]) {
        left = lower_index;
    } else if (x >= c[upper_index + 2]) {
        left = upper_index - 1;
    } else {
        int lo = lower_index;
        int hi = upper_index - 1;
        while (lo <= hi) {
            const int mid = lo + (hi - lo) / 2;
            if (x >= c[mid + 2] && x < c[mid + 3]) {
                lo = mid;
                break;
            }
            if (x < c[mid + 2]) {
                hi = mid - 1;
            } else {
                lo = mid + 1;
            }
        }
        left = lo;
    }
    const double x_left = c[left + 2];
    const double x_right = c[left + 3];
    return __dadd_rn(static_cast<double>(left),
                     __ddiv_rn(__dsub_rn(x, x_left), __dsub_rn(x_right, x_left)));
}

// Cell index over the physical domain: MappedCoordinateGrid::cell_index
// (:255-276) on an analytic axis, StoredCoordinateGrid::cell_index on a
// stored one.
__device__ __forceinline__ int lib_cell_index(const LibAxis& a, double x) {
    if (a.stored) return stored_cell_index(a, x, 0, a.n - 1, a.lower, a.upper);
    if (x < a.lower) return -1;
    if (x > a.upper) return a.n;
    if (x == a.upper) return a.n - 1;
    return static_cast<int>(floor(__ddiv_rn(__dsub_rn(x, a.x0), a.dx)));
}

// Cell-centred stencil over the ghosted domain [-2, n+1]
// (FieldInterpolator.hpp:509-559) on the logical index of
// AnalyticCoordinateGrid.hpp:216-230 or StoredCoordinateGrid::grid_index.
__device__ __forceinline__ void stencil_from_logical(const LibAxis& a, double logical, int& lo,
                                                     int& hi, double& w);

__device__ __forceinline__ void lib_stencil(const LibAxis& a, double x, int& lo, int& hi,
                                            double& w) {
    const double logical = a.stored ? stored_grid_index(a, x, false)
                                    : __dsub_rn(__ddiv_rn(__dsub_rn(x, a.x0), a.dx), 0.5);
    stencil_from_logical(a, logical, lo, hi, w);
}

// The mixed step's stencil: on a uniform axis the logical index is the FP32
// product of the FP64 offset x - x0 and 1/dx (its rounding, ~1e-7 of a
// cell, moves the sample by less than the FP32 table's own precision; the
// bilinear weights are continuous across cells, so a cell index that differs
// from the FP64 one near a cell face gives the same value); stored axes keep
// their FP64 bisection.
__device__ __forceinline__ void lib_stencil_mixed(const LibAxis& a, double x, int& lo, int& hi,
                                                  float& w) {
    if (a.stored) {
        double wd;
        stencil_from_logical(a, stored_grid_index(a, x, false), lo, hi, wd);
        w = static_cast<float>(wd);
        return;
    }
    const float logical =
        fmaf(static_cast<float>(x - a.x0), static_cast<float>(a.inv_dx), -0.5f);
    const int lower_bound = -2;
    const int upper_bound = a.n + 1;
    if (logical <= static_cast<float>(lower_bound)) {
        lo = hi = lower_bound;
        w = 0.0f;
        return;
    }
    if (logical >= static_cast<float>(upper_bound)) {
        lo = hi = upper_bound;
        w = 0.0f;
        return;
    }
    const float cell = floorf(logical);
    lo = static_cast<int>(cell);
    hi = lo + 1;
    w = logical - cell;
    if (hi > upper_bound) {
        lo = hi = upper_bound;
        w = 0.0f;
    }
}

// FieldInterpolator's compute_axis_stencil on a logical index.
__device__ __forceinline__ void stencil_from_logical(const LibAxis& a, double logical, int& lo,
                                                     int& hi, double& w) {
    const int lower_bound = -2;
    const int upper_bound = a.n + 1;
    if (logical <= static_cast<double>(lower_bound)) {
        lo = hi = lower_bound;
        w = 0.0;
        return;
    }
    if (logical >= static_cast<double>(upper_bound)) {
        lo = hi = upper_bound;
        w = 0.0;
        return;
    }
    const int candidate = static_cast<int>(floor(logical));
    lo = candidate;
    hi = candidate + 1;
    w = __dsub_rn(logical, static_cast<double>(candidate));
    if (hi > upper_bound) {
        lo = hi = upper_bound;
        w = 0.0;
    }
}

// LinearPositionInterpolator::sample of the 18-component packed basis
// (FieldInterpolator.hpp:346-380): corners in order, weight = product of the
// per-axis factors, values accumulated in component order.
template <int C, int STRIDE>
__device__ __forceinline__ void lib_sample(const LibGrid& g, const double* __restrict__ basis,
                                           double x, double y, double (&out)[C]) {
    int lo[2], hi[2];
    double w[2];
    lib_stencil(g.axis[0], x, lo[0], hi[0], w[0]);
    lib_stencil(g.axis[1], y, lo[1], hi[1], w[1]);
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = 0.0;
#pragma unroll
    for (int corner = 0; corner < 4; ++corner) {
        const bool ux = (corner & 1) != 0;
        const bool uy = (corner & 2) != 0;
        double weight = 1.0;
        weight = __dmul_rn(weight, ux ? w[0] : __dsub_rn(1.0, w[0]));
        weight = __dmul_rn(weight, uy ? w[1] : __dsub_rn(1.0, w[1]));
        const int i = (ux ? hi[0] : lo[0]) + 2;
        const int j = (uy ? hi[1] : lo[1]) + 2;
        const double* row = basis + (static_cast<size_t>(j) * g.ex + i) * STRIDE;
#pragma unroll
        for (int c = 0; c + 1 < C; c += 2) {
            const double2 v = __ldg(reinterpret_cast<const double2*>(row + c));
            out[c] = __dadd_rn(out[c], __dmul_rn(weight, v.x));
            out[c + 1] = __dadd_rn(out[c + 1], __dmul_rn(weight, v.y));
        }
        if (C % 2 == 1) {
            out[C - 1] = __dadd_rn(out[C - 1], __dmul_rn(weight, __ldg(row + C - 1)));
        }
    }
}

// The mixed-precision library step samples an FP32 copy of the packed basis
// (rows padded to whole 16-byte chunks) with the same stencil and weights
// (formed in FP64 from the FP64 positions), accumulated in FP32.
template <int C, int STRIDE>
__device__ __forceinline__ void lib_sample(const LibGrid& g, const float* __restrict__ basis,
                                           double x, double y, float (&out)[C]) {
    static_assert(STRIDE % 4 == 0 && STRIDE >= C, "FP32 rows hold whole 16-byte chunks");
    int lo[2], hi[2];
    float w[2];
    lib_stencil_mixed(g.axis[0], x, lo[0], hi[0], w[0]);
    lib_stencil_mixed(g.axis[1], y, lo[1], hi[1], w[1]);
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = 0.0f;
#pragma unroll
    for (int corner = 0; corner < 4; ++corner) {
        const bool ux = (corner & 1) != 0;
        const bool uy = (corner & 2) != 0;
        const float weight = (ux ? w[0] : 1.0f - w[0]) * (uy ? w[1] : 1.0f - w[1]);
        const int i = (ux ? hi[0] : lo[0]) + 2;
        const int j = (uy ? hi[1] : lo[1]) + 2;
        const float4* row =
            reinterpret_cast<const float4*>(basis + (static_cast<size_t>(j) * g.ex + i) * STRIDE);
#pragma unroll
        for (int k = 0; k < (C + 3) / 4; ++k) {
            const float4 v = __ldg(row + k);
            const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (4 * k + m < C) out[4 * k + m] = fmaf(weight, e[m], out[4 * k + m]);
            }
        }
    }
}

// Math of the two library precisions.
template <typename T>
struct LibMath;
template <>
struct LibMath<double> {
    static __device__ __forceinline__ double sqrt(double v) { return ::sqrt(v); }
    static __device__ __forceinline__ double cbrt(double v) { return ::cbrt(v); }
    static __device__ __forceinline__ double pow(double a, double b) { return ::pow(a, b); }
    static __device__ __forceinline__ double abs(double v) { return fabs(v); }
};
template <>
struct LibMath<float> {
    static __device__ __forceinline__ float sqrt(float v) { return sqrtf(v); }
    static __device__ __forceinline__ float cbrt(float v) { return cbrtf(v); }
    static __device__ __forceinline__ float pow(float a, float b) { return powf(a, b); }
    static __device__ __forceinline__ float abs(float v) { return fabsf(v); }
};

// The momentum scalings gamma^(1/3) and gamma^(1/9) of the diffusion
// coefficients (LegencyModel.hpp:483-502, FocusSolver.hpp:820, :968 call
// pow(gamma, 1/3) and pow(gamma, 1/9)) as one and two cube roots: the same
// values to within two ulp, at a fraction of pow's FP64 work.  The kernels
// here are FP64-pipe bound, so every transcendental counts.
template <typename T>
struct GammaRoots {
    T third, ninth;
};
template <typename T>
__device__ __forceinline__ GammaRoots<T> gamma_roots(T gamma, bool ninth) {
    GammaRoots<T> r;
    r.third = LibMath<T>::cbrt(gamma);
    r.ninth = ninth ? LibMath<T>::cbrt(r.third) : r.third;
    return r;
}

template <typename T>
__device__ __forceinline__ bool finite_positive(T v) { return isfinite(v) && v > T(0); }
template <typename T>
__device__ __forceinline__ bool finite_nonnegative(T v) { return isfinite(v) && v >= T(0); }

// apply_grid_boundary_conditions for one active particle (ParticleSystem.hpp:
// 653-699).  Returns false when the particle escaped.
__device__ __forceinline__ bool lib_boundary(const LibGrid& g, const SystemArrays& s, size_t i) {
    bool escaped = false;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        double* pos = dim == 0 ? s.x : s.y;
        const double x = pos[i];
        if (a.periodic) {
            const double wrapped = lib_wrap(a, x);
            const double shift = __dsub_rn(wrapped, x);
            pos[i] = wrapped;
            double* prev = dim == 0 ? s.prev_x : s.prev_y;
            double* prevstep = dim == 0 ? s.prevstep_x : s.prevstep_y;
            prev[i] = __dadd_rn(prev[i], shift);
            prevstep[i] = __dadd_rn(prevstep[i], shift);
        } else if (!lib_contains(a.lower, a.upper, x)) {
            escaped = true;
        }
    }
    if (escaped) {
        s.status[i] = 1;
    }
    return !escaped;
}

// The mixed step's boundary pass: a coordinate already inside [lower, upper)
// of a periodic axis is its own wrap, so only coordinates outside take the
// reference's floor formula (two FP64 compares for most particles instead of
// the full wrap; GB300's FP64 pipe is the scarce one).
__device__ __forceinline__ bool lib_boundary_mixed(const LibGrid& g, const SystemArrays& s,
                                                   size_t i) {
    bool escaped = false;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        double* pos = dim == 0 ? s.x : s.y;
        const double x = pos[i];
        const bool inside = x >= a.lower && x < a.upper;
        if (a.periodic) {
            if (!inside) {
                const double wrapped = lib_wrap(a, x);
                const double shift = wrapped - x;
                pos[i] = wrapped;
                double* prev = dim == 0 ? s.prev_x : s.prev_y;
                double* prevstep = dim == 0 ? s.prevstep_x : s.prevstep_y;
                prev[i] = prev[i] + shift;
                prevstep[i] = prevstep[i] + shift;
            }
        } else if (!inside && !lib_contains(a.lower, a.upper, x)) {
            escaped = true;
        }
    }
    if (escaped) {
        s.status[i] = 1;
    }
    return !escaped;
}

template <typename T>
__device__ __forceinline__ bool lib_boundary_t(const LibGrid& g, const SystemArrays& s,
                                               size_t i) {
    if constexpr (sizeof(T) == 4) {
        return lib_boundary_mixed(g, s, i);
    } else {
        return lib_boundary(g, s, i);
    }
}

// Kept per-particle terms (one row per particle, kLibTermCount doubles).
enum TermSlot {
    kRateX = 0, kRateY, kMomentumRate, kKappaPar, kKappaPerp, kDirX, kDirY, kDirZ, kMomentum
};
static_assert(kMomentum + 1 == kLibTermCount, "term row layout");

// evaluate_terms_from_packed + local_stable_time_step
// (ParkerSolver.hpp:766-868, :689-760, :880-942).  Returns the local dt bound
// or a negative error code.  T = double: the reference's FP64 arithmetic;
// T = float: the mixed step (FP32 basis, terms and bounds in an FP32 term
// row; the positions and the boundary decisions stay FP64, wrapped once, and
// the momentum base is read from the FP64 state by the update).
template <typename T>
__device__ T lib_parker_terms(const LibParkerLaunch& L, size_t i, T* terms) {
    using M = LibMath<T>;
    constexpr bool kMixed = sizeof(T) == 4;
    const LibGrid& g = L.grid;
    const SystemArrays& s = L.sys;
    double pos[2] = {s.x[i], s.y[i]};
    // prepare_physical_position (:620-633)
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        if (!kMixed || !(pos[dim] >= a.lower && pos[dim] < a.upper)) {
            pos[dim] = lib_wrap(a, pos[dim]);
        }
        if (!lib_contains(a.lower, a.upper, pos[dim])) {
            // the reference's empty terms: zero rates, zero time step
            for (int k = 0; k < kLibTermCount; ++k) terms[k] = T(0);
            return T(0);
        }
    }
    T v[kLibBasis];
    if constexpr (kMixed) {
        // a wrapped physical position is its own wrap and inside the ghosts
        lib_sample<kLibBasis, kLibBasisStrideF32>(g, L.basis_f32, pos[0], pos[1], v);
    } else {
        // interpolator prepare_coordinate: wrap, then the ghosted-domain check
        double q[2];
#pragma unroll
        for (int dim = 0; dim < 2; ++dim) {
            q[dim] = lib_wrap(g.axis[dim], pos[dim]);
            if (!lib_contains(g.axis[dim].ghost_lower, g.axis[dim].ghost_upper, q[dim])) {
                return T(-1);  // "position lies outside the interpolation domain"
            }
        }
        lib_sample<kLibBasis, kLibBasisStride>(g, L.basis, q[0], q[1], v);
    }

    const T p_in = static_cast<T>(s.p[i]);
    const T p = p_in >= T(0) ? p_in : -p_in;
    const T normalized = p / static_cast<T>(L.mc);
    const T gamma = M::sqrt(T(1) + normalized * normalized);
    const T speed = p / (gamma * static_cast<T>(L.rest_mass));
    T b2 = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) b2 += v[c] * v[c];
    const T bmag = M::sqrt(b2);
    if (!finite_positive(bmag)) {
        return T(-2);  // "stochastic diffusion requires |B| > 0"
    }
    const T ib = T(1) / bmag;
    T dir[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) dir[c] = v[c] * ib;
    const GammaRoots<T> roots = gamma_roots<T>(gamma, !L.constant_ratio);
    const T g13 = roots.third;
    T diff[3];
    if (L.constant_ratio) {
#pragma unroll
        for (int c = 0; c < 3; ++c) diff[c] = g13 * v[9 + c];
    } else {
        const T g19 = roots.ninth;
#pragma unroll
        for (int c = 0; c < 3; ++c) diff[c] = g13 * v[9 + c] + g19 * v[12 + c];
    }
    const T kpar = v[15] * g13;
    const T kperp = v[16] * (L.constant_ratio ? g13 : roots.ninth);
    if (!finite_nonnegative(kpar) || !finite_nonnegative(kperp)) {
        return T(-3);  // "diffusion coefficients must be finite and non-negative"
    }
    T keff[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        keff[d] = kperp + (kpar - kperp) * dir[d] * dir[d];
        if (!finite_nonnegative(keff[d])) {
            return T(-4);  // "projected diffusion coefficient is invalid"
        }
    }
    const T divv = v[17];
    const T prefactor = p * speed * static_cast<T>(L.speed_of_light) /
                        (T(3) * static_cast<T>(L.charge));
    T total[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) total[c] = v[3 + c] + prefactor * v[6 + c] + diff[c];
    // Cartesian: h_inv = 1
    terms[kRateX] = total[0] * T(1);
    terms[kRateY] = total[1] * T(1);
    terms[kMomentumRate] = -(p / T(3)) * divv;
    terms[kKappaPar] = kpar;
    terms[kKappaPerp] = kperp;
    terms[kDirX] = dir[0];
    terms[kDirY] = dir[1];
    terms[kDirZ] = dir[2];
    if constexpr (!kMixed) terms[kMomentum] = p;

    // local_stable_time_step: prepare_physical_position again, then per-axis
    // cell widths at the physical cell index
    const T large = static_cast<T>(kLargeTimeStep);  // +inf in FP32
    T dmin = large;
    T amin = large;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        T dx;
        if (kMixed && !a.stored) {
            dx = static_cast<T>(a.dx);
        } else {
            const double x = kMixed ? pos[dim] : lib_wrap(a, pos[dim]);
            if (!lib_contains(a.lower, a.upper, x)) {
                return large;
            }
            const double cell = static_cast<double>(lib_cell_index(a, x));
            const double width =
                __dsub_rn(lib_face(a, __dadd_rn(cell, 1.0)), lib_face(a, cell));
            dx = static_cast<T>(fabs(__dmul_rn(1.0, width)));
        }
        if (!finite_positive(dx)) {
            return T(-5);  // "local physical cell width must be positive"
        }
        T diffusion_dt = large;
        if (keff[dim] > T(0)) {
            const T limited = T(0.5) * dx;
            diffusion_dt = limited * limited / (T(2) * keff[dim]);
        }
        const T adv = M::abs(total[dim]);
        T advection_dt = large;
        if (adv > T(0)) {
            advection_dt = T(1) * dx / adv;
        }
        dmin = diffusion_dt < dmin ? diffusion_dt : dmin;
        amin = advection_dt < amin ? advection_dt : amin;
    }
    T mdt = large;
    const T dm = M::abs(divv);
    if (dm > T(0)) {
        mdt = T(3) * T(1) / dm;
    }
    const T da = dmin < amin ? dmin : amin;
    return da < mdt ? da : mdt;
}

// The block's minimum of the local dt bounds to the global minimum: one
// atomic per block on the bit pattern of a positive double (exact and order
// independent); an FP32 bound of +inf (no limiter) is the reference's large
// step.
template <typename T>
__device__ __forceinline__ void block_min_to_global(T local, unsigned long long* min_bits) {
    for (int off = 16; off > 0; off >>= 1) {
        const T o = __shfl_down_sync(0xffffffffu, local, off);
        local = o < local ? o : local;
    }
    __shared__ T warp_min[8];
    if ((threadIdx.x & 31u) == 0u) warp_min[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        T m = warp_min[0];
        for (int k = 1; k < static_cast<int>(blockDim.x >> 5); ++k) m = warp_min[k] < m ? warp_min[k] : m;
        const double md = isinf(m) ? kLargeTimeStep : static_cast<double>(m);
        // positive doubles order like their bit patterns
        atomicMin(min_bits, static_cast<unsigned long long>(__double_as_longlong(md)));
    }
}

__device__ __forceinline__ void record_error(int* error, int code, uint32_t index,
                                             unsigned long long* error_index) {
    if (atomicCAS(error, 0, code) == 0) {
        *error_index = index;
    }
}

// Pass 1: boundary conditions, terms, local dt -> global min (bit pattern).
template <typename T>
__global__ void __launch_bounds__(256) lib_parker_terms_kernel(const LibParkerLaunch L) {
    T local = static_cast<T>(kLargeTimeStep);
    T* terms = reinterpret_cast<T*>(L.terms);
    const bool stopped = *L.error != 0;  // an earlier step of a replayed sequence failed
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
         !stopped && i < L.count; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        if (L.sys.status[i] != 0) {
            continue;
        }
        if (L.apply_boundary && !lib_boundary_t<T>(L.grid, L.sys, i)) {
            continue;
        }
        const T dt = lib_parker_terms<T>(L, i, terms + i * kLibTermCount);
        if (dt < T(0)) {
            record_error(L.error, static_cast<int>(-dt), static_cast<uint32_t>(i),
                         L.error_index);
            continue;
        }
        local = dt < local ? dt : local;
    }
    block_min_to_global(local, L.min_bits);
}

// Box-Muller pair from two stream draws (u1 = 1 - draw, u2 = draw): normals
// 2m and 2m+1 of a particle's step are r cos(theta) and r sin(theta) of
// block m, as the shim pool's normal() hands them out.  The FP32 pair takes
// the high word of each draw (24 bits), so it tracks the FP64 pair.
template <typename T>
struct NormalPair {
    T x, y;
};

template <typename T>
__device__ __forceinline__ NormalPair<T> lib_normal_pair(uint2 key, uint32_t block,
                                                         uint32_t index, uint32_t frame) {
    const uint4 r = philox4x32_10(make_uint4(block, index, frame, kTagLibrary), key);
    if constexpr (sizeof(T) == 8) {
        const double u1 = 1.0 - u01_f64(r.x, r.y);
        const double u2 = u01_f64(r.z, r.w);
        const double radius = sqrt(-2.0 * log(u1));
        double s, c;
        sincos(6.283185307179586 * u2, &s, &c);
        return NormalPair<T>{radius * c, radius * s};
    } else {
        const float u1 = 1.0f - u01_f32(r.y);
        const float u2 = u01_f32(r.w);
        const float radius = sqrtf(-2.0f * logf(u1));
        float s, c;
        sincosf(6.2831853071795865f * u2, &s, &c);
        return NormalPair<T>{radius * c, radius * s};
    }
}

// The four normals of a particle's step: the keyed stream's two pairs, or
// the caller's buffer [4][count].
template <typename T>
__device__ __forceinline__ void step_normals(uint2 key, uint32_t frame, const double* noise,
                                             uint64_t count, uint64_t i, NormalPair<T>& n01,
                                             NormalPair<T>& n23) {
    if (noise != nullptr) {
        n01 = NormalPair<T>{static_cast<T>(noise[i]), static_cast<T>(noise[count + i])};
        n23 = NormalPair<T>{static_cast<T>(noise[2 * count + i]),
                            static_cast<T>(noise[3 * count + i])};
    } else {
        n01 = lib_normal_pair<T>(key, 0u, static_cast<uint32_t>(i), frame);
        n23 = lib_normal_pair<T>(key, 1u, static_cast<uint32_t>(i), frame);
    }
}

// Pass 2: capture previous positions (whole capacity), update, boundary.
// The mixed step (T = float) forms the noise increments in FP32 and adds
// them, with the FP64 drift dt * rate, to the FP64 positions and momenta.
template <typename T>
__global__ void __launch_bounds__(256) lib_parker_advance_kernel(const LibParkerLaunch L) {
    const double dt = L.dt_device != nullptr ? *L.dt_device : L.dt;
    // a failed step (no positive dt, or an abort condition) changes nothing
    // beyond the boundary pass, as the reference throws before its update
    if (!(isfinite(dt) && dt > 0.0) || *L.error != 0) {
        return;
    }
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
         i < L.capacity; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const SystemArrays& s = L.sys;
        if (L.capture) {
            s.prevstep_x[i] = s.prev_x[i];
            s.prevstep_y[i] = s.prev_y[i];
            s.prev_x[i] = s.x[i];
            s.prev_y[i] = s.y[i];
        }
        if (i >= L.count || s.status[i] != 0) {
            continue;
        }
        const T* t = reinterpret_cast<const T*>(L.terms) + i * kLibTermCount;
        if constexpr (sizeof(T) == 8) {
            double inc[2] = {0.0, 0.0};
            if (L.stochastic) {
                NormalPair<double> n01, n23;
                step_normals<double>(L.key, L.frame, L.noise, L.count, i, n01, n23);
                const double gv[3] = {n01.x, n01.y, n23.x};
                double iso = 0.0;
#pragma unroll
                for (int c = 0; c < 3; ++c) iso += gv[c] * t[kDirX + c];
                const double pg = n23.y;
                const double kperp = t[kKappaPerp];
                const double kpar = t[kKappaPar];
                const double perp_scale = kperp > 0.0 ? sqrt(2.0 * kperp * dt) : 0.0;
                const double par_scale = kpar > 0.0 ? sqrt(2.0 * kpar * dt) : 0.0;
                const double replacement = par_scale * pg - perp_scale * iso;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    inc[c] = perp_scale * gv[c] + replacement * t[kDirX + c];
                }
            }
            if (L.stochastic) {
                s.x[i] += dt * t[kRateX] + inc[0] * 1.0;
                s.y[i] += dt * t[kRateY] + inc[1] * 1.0;
            } else {
                s.x[i] += dt * t[kRateX];
                s.y[i] += dt * t[kRateY];
            }
            const double updated = t[kMomentum] + dt * t[kMomentumRate];
            s.p[i] = updated > 0.0 ? updated : 0.0;
        } else {
            // the increments in FP32, added to the FP64 state
            const float tdt = static_cast<float>(dt);
            float inc[2] = {tdt * t[kRateX], tdt * t[kRateY]};
            if (L.stochastic) {
                NormalPair<float> n01, n23;
                step_normals<float>(L.key, L.frame, L.noise, L.count, i, n01, n23);
                const float gv[3] = {n01.x, n01.y, n23.x};
                const float iso = gv[0] * t[kDirX] + gv[1] * t[kDirY] + gv[2] * t[kDirZ];
                const float kperp = t[kKappaPerp];
                const float kpar = t[kKappaPar];
                const float perp_scale = kperp > 0.0f ? sqrtf(2.0f * kperp * tdt) : 0.0f;
                const float par_scale = kpar > 0.0f ? sqrtf(2.0f * kpar * tdt) : 0.0f;
                const float replacement = par_scale * n23.y - perp_scale * iso;
                inc[0] += perp_scale * gv[0] + replacement * t[kDirX];
                inc[1] += perp_scale * gv[1] + replacement * t[kDirY];
            }
            s.x[i] += static_cast<double>(inc[0]);
            s.y[i] += static_cast<double>(inc[1]);
            // the momentum base is the FP64 state, as the terms pass read it
            const double base = s.p[i] >= 0.0 ? s.p[i] : -s.p[i];
            const double updated = base + static_cast<double>(tdt * t[kMomentumRate]);
            s.p[i] = updated > 0.0 ? updated : 0.0;
        }
        lib_boundary_t<T>(L.grid, s, i);
    }
}

// dt = courant * min over the active particles, on the device (0 when no
// particle bounded it; the host reports that as an error).
__global__ void lib_finish_dt_kernel(const unsigned long long* min_bits, double courant,
                                     double* dt_out, double* dt_history, int* error,
                                     int require_positive) {
    const double m = __longlong_as_double(static_cast<long long>(*min_bits));
    const double dt = (!isfinite(m) || m >= 0.5 * kLargeTimeStep) ? 0.0 : courant * m;
    *dt_out = dt;
    if (dt_history != nullptr) *dt_history = *error != 0 ? 0.0 : dt;
    if (require_positive && !(isfinite(dt) && dt > 0.0) && *error == 0) {
        *error = 6;  // "adaptive time step is not positive and finite"
    }
}

__global__ void lib_reset_min_kernel(unsigned long long* min_bits) {
    *min_bits = static_cast<unsigned long long>(__double_as_longlong(kLargeTimeStep));
}

// ---- FocusTransportSolver ----------------------------------------------------

enum FocusSlot {
    fRateX = 0, fRateY, fMomentumRate, fKappaPerp, fDirX, fDirY, fDirZ, fMomentum, fMu, fSpeed,
    fGamma, fBmag, fDivV, fBBGradV, fConvective, fFocusing, fSigma2, fLc
};
static_assert(fLc + 1 <= kFocusTermCount, "focus term row layout");

// The first failure of a particle's step is the one reported, as the
// reference throws at its first failed check.
__device__ __forceinline__ void set_error(int* error, int code) {
    if (*error == 0) *error = code;
}

// reflected_pitch_angle_cosine (FocusSolver.hpp:453-470).
template <typename T>
__device__ __forceinline__ T focus_reflect(T mu, T max_mu, int* error) {
    if (!isfinite(mu)) {
        set_error(error, 8);  // "pitch-angle cosine is not finite"
        return T(0);
    }
    const T upper = max_mu;
    const T lower = -max_mu;
    for (int guard = 0; guard < 64 && (mu > upper || mu < lower); ++guard) {
        if (mu > upper) mu = T(2) * upper - mu;
        if (mu < lower) mu = T(2) * lower - mu;
    }
    return mu;
}

template <typename T>
__device__ __forceinline__ T positive_floor(T v, T floor_value) {
    if (floor_value <= T(0)) return v;
    return v < floor_value ? floor_value : v;
}

template <typename T>
struct PitchRates {
    T focusing, D, dD, rate;
};

// The parts of evaluate_pitch_angle_at_mu (FocusSolver.hpp:664-695) and of
// the slab-QLT D_mumu (LegencyModel.hpp:557-645) that do not depend on mu:
// one step evaluates the rates at four trial cosines (the time-step bound and
// three Picard iterations) of the same particle, so omega, xi, xi^gamma_k
// and the prefactor are formed once.  The reference forms pow(|mu|+h0, gk),
// pow(xi, gk) and pow(|mu|+h0, gk-1) in both D and D'; here one pow per trial
// cosine remains (|mu|+h0)^(gk-1), with (|mu|+h0)^gk as its product with
// |mu|+h0 (equal to within two ulp).
template <typename T>
struct PitchSetup {
    T speed, focusing0, convective, omega, xi, xi_gk, pref;
    int error;  // 12, 13 or 14: the input check that fails, in the reference's order
};

template <typename T>
__device__ PitchSetup<T> focus_pitch_setup(const LibFocusLaunch& L, const T* t) {
    PitchSetup<T> q{};
    q.speed = static_cast<T>(t[fSpeed]);
    if (q.speed <= T(0)) {
        q.error = 12;  // "pitch-angle stepping requires positive particle speed"
        return q;
    }
    q.focusing0 = -q.speed * static_cast<T>(t[fFocusing]);
    q.convective = T(2) * static_cast<T>(t[fConvective]) / q.speed;
    const T safe_b = positive_floor(static_cast<T>(t[fBmag]), static_cast<T>(L.min_b));
    const T safe_sigma2 = positive_floor(static_cast<T>(t[fSigma2]), static_cast<T>(L.min_sigma2));
    const T safe_lc = positive_floor(static_cast<T>(t[fLc]), static_cast<T>(L.min_lc));
    const T safe_speed = positive_floor(q.speed, static_cast<T>(L.min_speed));
    if (safe_b <= T(0) || safe_sigma2 <= T(0) || safe_lc <= T(0) || safe_speed <= T(0)) {
        q.error = 13;  // "pitch-angle scattering requires positive local inputs"
        return q;
    }
    q.omega = static_cast<T>(L.abs_charge) * safe_b /
              (static_cast<T>(L.rest_mass) * static_cast<T>(L.speed_of_light)) /
              static_cast<T>(t[fGamma]);
    if (q.omega <= T(0)) {
        q.error = 14;  // "D_mumu requires positive omega, speed, sigma2, and Lc"
        return q;
    }
    q.xi = q.omega * safe_lc / safe_speed;
    q.xi_gk = LibMath<T>::pow(q.xi, static_cast<T>(L.gk));
    q.pref = static_cast<T>(0.25 * 3.141592653589793238462643383279502884) * q.omega *
             safe_sigma2 * static_cast<T>(L.qlt_norm);
    return q;
}

// evaluate_pitch_angle_at_mu with the slab-QLT evaluate_pitch_angle_scattering
// (LegencyModel.hpp:539-693) at one trial cosine.
template <typename T>
__device__ PitchRates<T> focus_pitch(const LibFocusLaunch& L, const T* t,
                                     const PitchSetup<T>& q, T trial, int* error) {
    PitchRates<T> r{T(0), T(0), T(0), T(0)};
    const T mu = focus_reflect(trial, static_cast<T>(L.max_mu), error);
    if (q.error != 0) {
        set_error(error, q.error);
        return r;
    }
    const T mu2 = mu * mu;
    const T one_minus_mu2 = T(1) - mu2;
    r.focusing = T(0.5) * one_minus_mu2 *
                 (q.focusing0 + mu * static_cast<T>(t[fDivV]) -
                  T(3) * mu * static_cast<T>(t[fBBGradV]) - q.convective);
    T d = T(0);
    T dd = T(0);
    if (one_minus_mu2 > T(0)) {
        const T reg = (mu >= T(0) ? mu : -mu) + static_cast<T>(L.h0);
        const T gk = static_cast<T>(L.gk);
        const T reg_gk1 = LibMath<T>::pow(reg, gk - T(1));
        const T reg_gk = reg > T(0) ? reg_gk1 * reg : LibMath<T>::pow(reg, gk);
        const T den = reg_gk + q.xi_gk;
        if (den <= T(0)) {
            set_error(error, 15);  // "D_mumu denominator must be positive"
            return r;
        }
        d = q.pref * one_minus_mu2 * q.xi * reg_gk1 / den;
        // pitch_angle_diffusion_derivative (LegencyModel.hpp:599-645)
        const T sign = mu > T(0) ? T(1) : (mu < T(0) ? T(-1) : T(0));
        if (d != T(0) && sign != T(0)) {
            const T shape = sign * ((gk - T(1)) / reg - gk * reg_gk1 / den);
            dd = d * (T(-2) * mu / one_minus_mu2 + shape);
        }
    }
    r.D = d;
    r.dD = dd;
    r.rate = r.focusing + dd;
    return r;
}

// evaluate_terms_from_packed + local_stable_time_step
// (FocusSolver.hpp:904-1008, :1148-1233).  T = double: the reference's FP64
// arithmetic; T = float: the mixed step (FP32 basis, terms and closure; the
// positions, boundary and cell-width decisions and the momentum stay FP64).
template <typename T>
__device__ T focus_terms(const LibFocusLaunch& L, size_t i, T* t, int* error) {
    using M = LibMath<T>;
    constexpr bool kMixed = sizeof(T) == 4;
    const LibGrid& g = L.grid;
    const SystemArrays& s = L.sys;
    double pos[2] = {s.x[i], s.y[i]};
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        if (!kMixed || !(pos[dim] >= a.lower && pos[dim] < a.upper)) {
            pos[dim] = lib_wrap(a, pos[dim]);
        }
        if (!lib_contains(a.lower, a.upper, pos[dim])) {
            for (int k = 0; k < kFocusTermCount; ++k) t[k] = T(0);
            return T(0);
        }
    }
    T v[kFocusBasis];
    if constexpr (kMixed) {
        // a wrapped physical position is its own wrap and inside the ghosts
        lib_sample<kFocusBasis, kFocusBasisStrideF32>(g, L.basis_f32, pos[0], pos[1], v);
    } else {
        double q[2];
#pragma unroll
        for (int dim = 0; dim < 2; ++dim) {
            q[dim] = lib_wrap(g.axis[dim], pos[dim]);
            if (!lib_contains(g.axis[dim].ghost_lower, g.axis[dim].ghost_upper, q[dim])) {
                set_error(error, 1);
                return T(-1);
            }
        }
        lib_sample<kFocusBasis, kFocusBasisStride>(g, L.basis, q[0], q[1], v);
    }
    const T p_in = static_cast<T>(s.p[i]);
    const T p = p_in >= T(0) ? p_in : -p_in;
    const T mu = focus_reflect(static_cast<T>(s.mu[i]), static_cast<T>(L.max_mu), error);
    const T normalized = p / static_cast<T>(L.mc);
    const T gamma = M::sqrt(T(1) + normalized * normalized);
    const T speed = p / (gamma * static_cast<T>(L.rest_mass));
    const T bmag = v[18];
    if (!finite_positive(bmag)) {
        set_error(error, 9);  // "focused transport requires |B| > 0"
        return T(-1);
    }
    T s2 = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) s2 += v[3 + c] * v[3 + c];
    const T smag = M::sqrt(s2);
    if (!finite_positive(smag)) {
        set_error(error, 10);  // "interpolated magnetic direction is invalid"
        return T(-1);
    }
    const T inv = T(1) / smag;
    T dir[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) dir[c] = v[3 + c] * inv;
    const GammaRoots<T> roots = gamma_roots<T>(gamma, !L.constant_ratio);
    const T perp_factor = L.constant_ratio ? roots.third : roots.ninth;
    const T kpar = v[19] * roots.third;
    const T kperp = v[20] * perp_factor;
    if (!finite_nonnegative(kpar) || !finite_nonnegative(kperp)) {
        set_error(error, 11);  // "diffusion coefficients must be finite and non-negative"
        return T(-1);
    }
    const T mu2 = mu * mu;
    const T gdf = T(0.5) * (T(1) - mu2);
    const T cdf = mu2;
    const T prefactor = p * speed * static_cast<T>(L.speed_of_light) / static_cast<T>(L.charge);
    T total[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T streaming = speed * mu * dir[c];
        const T drift = prefactor * (gdf * v[9 + c] + cdf * v[12 + c]);
        const T diffadv = perp_factor * v[15 + c];
        total[c] = streaming + v[6 + c] + drift + diffadv;
    }
    T keff[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const T projection = T(1) - dir[d] * dir[d];
        keff[d] = projection > T(0) ? kperp * projection : T(0);
    }
    t[fRateX] = total[0] * T(1);
    t[fRateY] = total[1] * T(1);
    t[fKappaPerp] = kperp;
    t[fDirX] = dir[0];
    t[fDirY] = dir[1];
    t[fDirZ] = dir[2];
    if constexpr (!kMixed) t[fMomentum] = p;
    t[fMu] = mu;
    t[fSpeed] = speed;
    t[fGamma] = gamma;
    t[fBmag] = bmag;
    t[fDivV] = v[21];
    t[fFocusing] = v[22];
    t[fBBGradV] = v[23];
    t[fConvective] = v[24];
    t[fSigma2] = v[25];
    t[fLc] = v[26];
    const T one_minus_mu2 = T(1) - mu2;
    T acceleration = T(0);
    if (speed > T(0)) acceleration = mu * v[24] / speed;
    const T momentum_factor = T(0.5) * one_minus_mu2 * (v[21] - v[23]) + mu2 * v[23] +
                              acceleration;
    const T momentum_rate = -p * momentum_factor;
    t[fMomentumRate] = momentum_rate;
    const PitchRates<T> pitch = focus_pitch<T>(L, t, focus_pitch_setup<T>(L, t), mu, error);

    const T large = static_cast<T>(kLargeTimeStep);  // +inf in FP32
    T dmin = large;
    T amin = large;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        T dx;
        if (kMixed && !a.stored) {
            dx = static_cast<T>(a.dx);
        } else {
            const double x = kMixed ? pos[dim] : lib_wrap(a, pos[dim]);
            if (!lib_contains(a.lower, a.upper, x)) {
                return large;
            }
            const double cell = static_cast<double>(lib_cell_index(a, x));
            const double width =
                __dsub_rn(lib_face(a, __dadd_rn(cell, 1.0)), lib_face(a, cell));
            dx = static_cast<T>(fabs(__dmul_rn(1.0, width)));
        }
        if (!finite_positive(dx)) {
            set_error(error, 5);
            return T(-1);
        }
        T diffusion_dt = large;
        if (keff[dim] > T(0)) {
            const T limited = T(0.5) * dx;
            diffusion_dt = limited * limited / (T(2) * keff[dim]);
        }
        const T adv = M::abs(total[dim]);
        T advection_dt = large;
        if (adv > T(0)) advection_dt = T(1) * dx / adv;
        dmin = diffusion_dt < dmin ? diffusion_dt : dmin;
        amin = advection_dt < amin ? advection_dt : amin;
    }
    T mdt = large;
    const T mrate = M::abs(momentum_rate);
    if (p > T(0) && mrate > T(0)) mdt = T(1) * p / mrate;
    T padv = large;
    const T murate = M::abs(pitch.rate);
    if (murate > T(0)) padv = T(10) * T(0.1) / murate;
    T pdiff = large;
    if (pitch.D > T(0)) pdiff = T(10) * T(0.1) * T(0.1) / (T(2) * pitch.D);
    T pbal = large;
    if (pitch.D > T(0) && murate > T(0)) pbal = T(10) * T(2) * pitch.D / (murate * murate);
    const T a1 = dmin < amin ? dmin : amin;
    const T a2 = a1 < mdt ? a1 : mdt;
    const T b1 = pdiff < pbal ? pdiff : pbal;
    const T b2 = padv < b1 ? padv : b1;
    return a2 < b2 ? a2 : b2;
}

template <typename T>
__global__ void __launch_bounds__(256) focus_terms_kernel(const LibFocusLaunch L) {
    T local = static_cast<T>(kLargeTimeStep);
    T* terms = reinterpret_cast<T*>(L.terms);
    const bool stopped = *L.error != 0;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
         !stopped && i < L.count; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        if (L.sys.status[i] != 0) continue;
        if (L.apply_boundary && !lib_boundary_t<T>(L.grid, L.sys, i)) continue;
        int err = 0;
        const T dt = focus_terms<T>(L, i, terms + i * kFocusTermCount, &err);
        if (err != 0) {
            record_error(L.error, err, static_cast<uint32_t>(i), L.error_index);
            continue;
        }
        local = dt < local ? dt : local;
    }
    block_min_to_global(local, L.min_bits);
}

// advance_*_with_packed_interpolator (FocusSolver.hpp:1580-1637) with the
// Picard pitch-angle update (:697-740).  The mixed step (T = float) forms the
// noise increments and the pitch-angle update in FP32 and adds the
// increments, with the FP64 drift dt * rate, to the FP64 positions.
template <typename T>
__global__ void __launch_bounds__(256) focus_advance_kernel(const LibFocusLaunch L) {
    const double dt = L.dt_device != nullptr ? *L.dt_device : L.dt;
    if (!(isfinite(dt) && dt > 0.0) || *L.error != 0) {
        return;
    }
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
         i < L.capacity; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const SystemArrays& s = L.sys;
        if (L.capture) {
            s.prevstep_x[i] = s.prev_x[i];
            s.prevstep_y[i] = s.prev_y[i];
            s.prev_x[i] = s.x[i];
            s.prev_y[i] = s.y[i];
        }
        if (i >= L.count || s.status[i] != 0) continue;
        const T* t = reinterpret_cast<const T*>(L.terms) + i * kFocusTermCount;
        T inc[2] = {T(0), T(0)};
        T pitch_normal = T(0);
        const T tdt = static_cast<T>(dt);
        if (L.stochastic) {
            NormalPair<T> n01, n23;
            step_normals<T>(L.key, L.frame, L.noise, L.count, i, n01, n23);
            const T gv[3] = {n01.x, n01.y, n23.x};
            const T d[3] = {static_cast<T>(t[fDirX]), static_cast<T>(t[fDirY]),
                            static_cast<T>(t[fDirZ])};
            T parallel = T(0);
#pragma unroll
            for (int c = 0; c < 3; ++c) parallel += gv[c] * d[c];
            const T kperp = static_cast<T>(t[fKappaPerp]);
            const T scale = kperp > T(0) ? LibMath<T>::sqrt(T(2) * kperp * tdt) : T(0);
#pragma unroll
            for (int c = 0; c < 2; ++c) inc[c] = scale * (gv[c] - parallel * d[c]);
            pitch_normal = n23.y;
        }
        if constexpr (sizeof(T) == 8) {
            s.x[i] += dt * t[fRateX] + inc[0] * 1.0;
            s.y[i] += dt * t[fRateY] + inc[1] * 1.0;
            const double updated = t[fMomentum] + dt * t[fMomentumRate];
            s.p[i] = updated > 0.0 ? updated : 0.0;
        } else {
            // the increments in FP32, added to the FP64 state; the momentum
            // base is the FP64 state, as the terms pass read it
            s.x[i] += static_cast<double>(tdt * t[fRateX] + inc[0]);
            s.y[i] += static_cast<double>(tdt * t[fRateY] + inc[1]);
            const double base = s.p[i] >= 0.0 ? s.p[i] : -s.p[i];
            const double updated = base + static_cast<double>(tdt * t[fMomentumRate]);
            s.p[i] = updated > 0.0 ? updated : 0.0;
        }
        int err = 0;
        const T max_mu = static_cast<T>(L.max_mu);
        const T initial = focus_reflect(static_cast<T>(t[fMu]), max_mu, &err);
        const PitchSetup<T> setup = focus_pitch_setup<T>(L, t);
        T trial = initial;
        for (int it = 0; it < 3; ++it) {
            const PitchRates<T> pitch = focus_pitch<T>(L, t, setup, trial, &err);
            const T scale = pitch.D > T(0) ? LibMath<T>::sqrt(T(2) * pitch.D * tdt) : T(0);
            trial = initial + tdt * pitch.rate + scale * pitch_normal;
            trial = focus_reflect(trial, max_mu, &err);
        }
        if (err != 0) {
            record_error(L.error, err, static_cast<uint32_t>(i), L.error_index);
            continue;
        }
        s.mu[i] = trial;
        lib_boundary_t<T>(L.grid, s, i);
    }
}

// ---- ParticleSystem lifecycle ------------------------------------------------

__global__ void system_default_kernel(SystemArrays s, uint64_t count, uint64_t capacity) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < capacity;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        s.id[i] = i;
        s.mu[i] = 0.0;
        s.weight[i] = 1.0;
        s.e0[i] = 0.0;
        s.status[i] = i < count ? 0 : 2;
        s.split_level[i] = 0;
        s.sort_key[i] = 0;
        s.x[i] = s.y[i] = s.prev_x[i] = s.prev_y[i] = s.prevstep_x[i] = s.prevstep_y[i] = 0.0;
        s.p[i] = 0.0;
    }
}

__global__ void system_boundary_kernel(LibGrid g, SystemArrays s, uint64_t count) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        if (s.status[i] == 0) lib_boundary(g, s, i);
    }
}

__global__ void system_capture_kernel(SystemArrays s, uint64_t capacity) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < capacity;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        s.prevstep_x[i] = s.prev_x[i];
        s.prevstep_y[i] = s.prev_y[i];
        s.prev_x[i] = s.x[i];
        s.prev_y[i] = s.y[i];
    }
}

// kinetic energy (gamma - 1) m c^2 (ParticleSystem.hpp:171-193), every
// operation rounded on its own as the reference build evaluates it (the
// baselines it writes are compared bit for bit)
__device__ __forceinline__ double kinetic_energy_of(double p, double mc, double rest_mass,
                                                    double speed_of_light) {
    const double normalized = __ddiv_rn(p, mc);
    const double gamma = __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(normalized, normalized)));
    return __dmul_rn(__dmul_rn(__dmul_rn(__dsub_rn(gamma, 1.0), rest_mass), speed_of_light),
                     speed_of_light);
}
__device__ __forceinline__ double kinetic_energy(const LibSplitLaunch& L, double p) {
    return kinetic_energy_of(p, L.mc, L.rest_mass, L.speed_of_light);
}

__global__ void system_reset_baselines_kernel(LibSplitLaunch L) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < L.count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const double p = L.sys.p[i] >= 0.0 ? L.sys.p[i] : -L.sys.p[i];
        L.sys.e0[i] = kinetic_energy(L, p);
        L.sys.split_level[i] = 0;
    }
}

// Energy-growth split decision per active parent
// (ParticleSystem.hpp:791-905): 1 = wants a child.  Also counts the active
// parents, the invalid baselines (and repairs them) and the minimum-weight
// refusals.
__device__ __forceinline__ int split_decision(const LibSplitLaunch& L, uint64_t i,
                                              unsigned long long* tallies) {
    const SystemArrays& s = L.sys;
    if (s.status[i] != 0) return 0;
    atomicAdd(tallies + 0, 1ull);
    const double p = s.p[i] >= 0.0 ? s.p[i] : -s.p[i];
    const double current = kinetic_energy(L, p);
    const double baseline = s.e0[i];
    if (!isfinite(baseline) || baseline <= 0.0) {
        if (isfinite(current) && current > 0.0) s.e0[i] = current;
        atomicAdd(tallies + 2, 1ull);
        return 0;
    }
    const double ratio = __ddiv_rn(current, baseline);
    if (!isfinite(ratio) || ratio < L.split_ratio) return 0;
    const int target = static_cast<int>(floor(__ddiv_rn(log(ratio), L.log_split_ratio)));
    if (target <= s.split_level[i]) return 0;
    const double child_weight = __dmul_rn(0.5, s.weight[i]);
    if (!isfinite(child_weight) || child_weight <= 0.0 || child_weight < L.min_child_weight) {
        atomicAdd(tallies + 3, 1ull);
        return 0;
    }
    return 1;
}

// Per-block counts of children wanted (parents in index order).
__global__ void __launch_bounds__(256) system_split_count_kernel(LibSplitLaunch L) {
    __shared__ unsigned int block_total;
    if (threadIdx.x == 0) block_total = 0;
    __syncthreads();
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    int want = 0;
    if (i < L.count) {
        want = split_decision(L, i, L.tallies);
        L.flags[i] = want;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, want != 0);
    if ((threadIdx.x & 31u) == 0u && ballot) atomicAdd(&block_total, __popc(ballot));
    __syncthreads();
    if (threadIdx.x == 0) L.block_counts[blockIdx.x] = block_total;
}

// Exclusive scan of the block counts (one block; serial over blocks per
// thread chunk, then a block scan).
__global__ void __launch_bounds__(1024) system_split_scan_kernel(unsigned int* counts, int n,
                                                                 unsigned long long* total) {
    __shared__ unsigned long long partial[1024];
    const int t = threadIdx.x;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int begin = t * per;
    const int end = begin + per < n ? begin + per : n;
    unsigned long long sum = 0;
    for (int k = begin; k < end; ++k) sum += counts[k];
    partial[t] = sum;
    __syncthreads();
    for (int off = 1; off < static_cast<int>(blockDim.x); off <<= 1) {
        const unsigned long long v = t >= off ? partial[t - off] : 0ull;
        __syncthreads();
        partial[t] += v;
        __syncthreads();
    }
    unsigned long long run = t > 0 ? partial[t - 1] : 0ull;
    for (int k = begin; k < end; ++k) {
        const unsigned int c = counts[k];
        counts[k] = static_cast<unsigned int>(run);
        run += c;
    }
    if (t == static_cast<int>(blockDim.x) - 1) *total = partial[t];
}

// Children in parent-index order (the serial order of the reference loop).
__global__ void __launch_bounds__(256) system_split_scatter_kernel(LibSplitLaunch L) {
    __shared__ unsigned int warp_base[8];
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    const int want = i < L.count ? L.flags[i] : 0;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned ballot = __ballot_sync(0xffffffffu, want != 0);
    if (lane == 0) warp_base[threadIdx.x >> 5] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int run = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
            const unsigned int c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (!want) return;
    const uint64_t offset = static_cast<uint64_t>(L.block_counts[blockIdx.x]) +
                            warp_base[threadIdx.x >> 5] + __popc(ballot & ((1u << lane) - 1u));
    const uint64_t child = L.count + offset;
    const SystemArrays& s = L.sys;
    if (child >= L.capacity) {
        atomicAdd(L.tallies + 1, 1ull);
        return;
    }
    const double child_weight = 0.5 * s.weight[i];
    s.id[child] = child;
    s.x[child] = s.x[i];
    s.y[child] = s.y[i];
    s.prev_x[child] = s.prev_x[i];
    s.prev_y[child] = s.prev_y[i];
    s.prevstep_x[child] = s.prevstep_x[i];
    s.prevstep_y[child] = s.prevstep_y[i];
    s.p[child] = s.p[i];
    s.mu[child] = s.mu[i];
    s.weight[i] = child_weight;
    s.weight[child] = child_weight;
    s.e0[child] = s.e0[i];
    s.status[child] = 0;
    s.sort_key[child] = s.sort_key[i];
    const int next = s.split_level[i] + 1;
    s.split_level[i] = next;
    s.split_level[child] = next;
}

// sort_by_key (ParticleSystem.hpp:723-759, Kokkos::BinSort with BinOp1D):
// a stable LSD radix sort of (key - lo) with 8-bit digits, so particles with
// equal keys keep their index order (the serial BinSort order).  Per pass:
// block digit histograms, a digit-major scan, then a stable scatter whose
// in-block ranks come from warp match masks and per-warp digit counts.
constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;

__global__ void radix_init_kernel(const int* keys, uint64_t count, int lo, int bins,
                                  unsigned int* k_out, unsigned int* idx_out) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        long long b = static_cast<long long>(keys[i]) - lo;
        b = b < 0 ? 0 : (b >= bins ? bins - 1 : b);
        k_out[i] = static_cast<unsigned int>(b);
        idx_out[i] = static_cast<unsigned int>(i);
    }
}

__global__ void __launch_bounds__(kRadixThreads) radix_hist_kernel(const unsigned int* keys,
                                                                   uint64_t count, int shift,
                                                                   unsigned int* hist,
                                                                   int blocks) {
    __shared__ unsigned int local[256];
    local[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(kRadixThreads) + threadIdx.x;
    if (i < count) atomicAdd(&local[(keys[i] >> shift) & 255u], 1u);
    __syncthreads();
    hist[static_cast<size_t>(threadIdx.x) * blocks + blockIdx.x] = local[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixThreads) radix_scatter_kernel(
    const unsigned int* keys_in, const unsigned int* idx_in, uint64_t count, int shift,
    const unsigned int* offsets, int blocks, unsigned int* keys_out, unsigned int* idx_out) {
    __shared__ unsigned int warp_counts[kRadixWarps][257];
    for (int k = threadIdx.x; k < kRadixWarps * 257; k += kRadixThreads) {
        (&warp_counts[0][0])[k] = 0;
    }
    __syncthreads();
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(kRadixThreads) + threadIdx.x;
    const bool have = i < count;
    const unsigned int key = have ? keys_in[i] : 0u;
    const unsigned int digit = have ? ((key >> shift) & 255u) : 256u;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = threadIdx.x >> 5;
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const unsigned rank = __popc(peers & ((1u << lane) - 1u));
    if (rank == 0) warp_counts[warp][digit] = __popc(peers);
    __syncthreads();
    // exclusive prefix over the warps, per digit (thread t owns digit t)
    {
        unsigned int run = 0;
        for (int w = 0; w < kRadixWarps; ++w) {
            const unsigned int c = warp_counts[w][threadIdx.x];
            warp_counts[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
    if (!have) return;
    const unsigned int dest = offsets[static_cast<size_t>(digit) * blocks + blockIdx.x] +
                              warp_counts[warp][digit] + rank;
    keys_out[dest] = key;
    idx_out[dest] = idx_in[i];
}

template <typename T>
__global__ void gather_kernel(const T* __restrict__ src, T* __restrict__ dst,
                              const unsigned int* __restrict__ perm, uint64_t count) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        dst[i] = src[perm[i]];
    }
}

__global__ void compact_keys_kernel(const int* status, int* keys, uint64_t count,
                                    unsigned long long* active) {
    unsigned long long mine = 0;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const bool alive = status[i] == 0;
        keys[i] = alive ? 0 : 1;
        mine += alive ? 1 : 0;
    }
    for (int off = 16; off > 0; off >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, off);
    if ((threadIdx.x & 31u) == 0u && mine) atomicAdd(active, mine);
}

// ---- ParticleGenerator -------------------------------------------------------
//
// Injection and recycling (ParticleGenerator.hpp:659-1493).  Every particle's
// draws come from its own keyed stream (seed, particle slot, frame, tag 4), so
// the results do not depend on the launch shape; the shim's pool hands the
// reference templates the same stream.  Candidate sets are a stable
// compaction (field points in index order, the order of the reference's
// parallel_scan) plus an FP64 inclusive scan of the cell volumes.

// Uniform draws of one particle's stream: draw n is half n%2 of block n/2.
struct DrawStream {
    uint2 key;
    uint32_t index, frame, draw;
    uint4 block;
    __device__ double next() {
        if ((draw & 1u) == 0u) {
            block = philox4x32_10(make_uint4(draw >> 1, index, frame, kTagGenerator), key);
        }
        const double u = (draw & 1u) == 0u ? u01_f64(block.x, block.y) : u01_f64(block.z, block.w);
        ++draw;
        return u;
    }
    // drand(start, end) = start + (end - start) drand()
    __device__ double range(double start, double end) {
        return __dadd_rn(start, __dmul_rn(__dsub_rn(end, start), next()));
    }
};

// Logical index range of a domain for cells (Grid.hpp:253-287); faces end
// one further.
__device__ __forceinline__ int gen_lower_cell(const LibAxis& a, int domain) {
    return domain != 0 ? -2 : 0;
}
__device__ __forceinline__ int gen_upper_cell(const LibAxis& a, int domain) {
    return domain != 0 ? a.n + 1 : a.n - 1;
}
__device__ __forceinline__ int gen_lower_index(const LibAxis& a, int centering, int domain) {
    return gen_lower_cell(a, domain);
}
__device__ __forceinline__ int gen_upper_index(const LibAxis& a, int centering, int domain) {
    return gen_upper_cell(a, domain) + (centering != 0 ? 1 : 0);
}

// Field point coordinate: face x0 + i dx, cell centre the midpoint of its
// faces (AnalyticCoordinateGrid.hpp:109-187).
__device__ __forceinline__ double gen_coordinate(const LibAxis& a, int index, int centering) {
    const double i = static_cast<double>(index);
    if (centering != 0) return lib_face(a, i);
    return __dmul_rn(0.5, __dadd_rn(lib_face(a, i), lib_face(a, __dadd_rn(i, 1.0))));
}

// compare_field_predicate_value (ParticleGenerator.hpp:230-251).
__device__ __forceinline__ bool gen_compare(double value, double threshold, int comparison) {
    switch (comparison) {
        case 0: return value > threshold;
        case 1: return value >= threshold;
        case 2: return value < threshold;
        case 3: return value <= threshold;
        case 4: return fabs(value) > threshold;
        case 5: return fabs(value) < threshold;
    }
    return false;
}

// FieldThresholdParticlePredicate::operator() (ParticleGenerator.hpp:297-353)
// with MappedCoordinateGrid::cell_index and contains_coordinate for a domain
// (MappedCoordinateGrid.hpp:255-292).
__device__ bool gen_predicate(const LibGrid& g, const GenPredicate& P, const double (&pt)[2]) {
    if (!P.enabled) return true;
    int idx[2];
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        const double lower_x = P.domain != 0 ? a.ghost_lower : a.lower;
        const double upper_x = P.domain != 0 ? a.ghost_upper : a.upper;
        const double x = pt[dim];
        if (!(x >= lower_x && x <= upper_x)) return false;
        const int centering = P.field.centering[dim];
        int index;
        if (a.stored) {
            // StoredCoordinateGrid::cell_index for a cell-centred field, the
            // nearest face of StoredCoordinateGrid::grid_index for a
            // face-centred one (ParticleGenerator.hpp:317-326)
            if (centering == 0) {
                index = stored_cell_index(a, x, gen_lower_cell(a, P.domain),
                                          gen_upper_cell(a, P.domain), lower_x, upper_x);
            } else {
                index = static_cast<int>(floor(__dadd_rn(stored_grid_index(a, x, true), 0.5)));
            }
        } else if (centering == 0) {
            if (x == upper_x) {
                index = gen_upper_cell(a, P.domain);
            } else {
                index = static_cast<int>(floor(__ddiv_rn(__dsub_rn(x, a.x0), a.dx)));
            }
        } else {
            index = static_cast<int>(
                floor(__dadd_rn(__ddiv_rn(__dsub_rn(x, a.x0), a.dx), 0.5)));
        }
        if (index < gen_lower_index(a, centering, P.domain) ||
            index > gen_upper_index(a, centering, P.domain)) {
            return false;
        }
        idx[dim] = index;
    }
    const size_t point = static_cast<size_t>(idx[0] + 2) +
                         static_cast<size_t>(idx[1] + 2) * static_cast<size_t>(P.field.ext[0]);
    const double value = P.field.values[point * P.field.components + P.component];
    return gen_compare(value, P.threshold, P.comparison);
}

// sample_cumulative_weight_index (ParticleGenerator.hpp:437-461).
__device__ uint64_t gen_sample_index(const GenCandidates& C, DrawStream& st) {
    if (C.count == 0 || C.total <= 0.0) return 0;
    const double target = st.range(0.0, C.total);
    uint64_t left = 0;
    uint64_t right = C.count - 1;
    while (left < right) {
        const uint64_t middle = left + (right - left) / 2;
        if (target < C.cumulative[middle]) {
            right = middle;
        } else {
            left = middle + 1;
        }
    }
    return left;
}

// ParticleRecycleSelection (ParticleGenerator.hpp:129-151): 1 escaped, 2 inactive.
__device__ __forceinline__ bool gen_selected(int status, int selection) {
    switch (selection) {
        case 0: return status == 1;
        case 1: return status == 2;
        case 2: return status == 1 || status == 2;
    }
    return false;
}

// One particle of an inject_* or recycle_* call.
__global__ void __launch_bounds__(256) generator_kernel(const GenLaunch L) {
    unsigned long long written = 0;
    for (uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; k < L.count;
         k += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const SystemArrays& s = L.sys;
        const uint64_t slot = L.recycle ? k : L.first_index + k;
        if (L.recycle && !gen_selected(s.status[slot], L.selection)) continue;
        DrawStream st{L.key, static_cast<uint32_t>(k), L.frame, 0u, make_uint4(0, 0, 0, 0)};
        double pt[2] = {0.0, 0.0};
        bool accepted = true;
        if (L.source == 0) {
            accepted = false;
            for (int attempt = 0; attempt < L.max_attempts; ++attempt) {
                pt[0] = st.range(L.region_lo[0], L.region_hi[0]);
                pt[1] = st.range(L.region_lo[1], L.region_hi[1]);
                if (gen_predicate(L.grid, L.predicate, pt)) {
                    accepted = true;
                    break;
                }
            }
        } else {
            const GenCandidates& C = L.candidates;
            const uint64_t c = gen_sample_index(C, st);
            if (C.kind == 0) {
                // FieldParticleCandidateSet::coordinate (:530-541)
                uint64_t linear = C.indices[c];
#pragma unroll
                for (int dim = 0; dim < 2; ++dim) {
                    const uint64_t e = static_cast<uint64_t>(C.field.ext[dim]);
                    const int index = static_cast<int>(linear % e) - 2;
                    linear /= e;
                    pt[dim] = gen_coordinate(L.grid.axis[dim], index, C.field.centering[dim]);
                }
            } else {
                // GridParticleCandidateSet::sample_coordinate (:627-645)
                uint64_t linear = c;
#pragma unroll
                for (int dim = 0; dim < 2; ++dim) {
                    const uint64_t e = static_cast<uint64_t>(C.extents[dim]);
                    const int index = C.lower[dim] + static_cast<int>(linear % e);
                    linear /= e;
                    const LibAxis& a = L.grid.axis[dim];
                    const double lo = lib_face(a, static_cast<double>(index));
                    const double hi = lib_face(a, static_cast<double>(index + 1));
                    pt[dim] = lo <= hi ? st.range(lo, hi) : st.range(hi, lo);
                }
            }
        }
        if (!L.recycle) s.id[slot] = L.first_id + k;
        s.x[slot] = s.prev_x[slot] = s.prevstep_x[slot] = pt[0];
        s.y[slot] = s.prev_y[slot] = s.prevstep_y[slot] = pt[1];
        s.p[slot] = L.momentum;
        s.mu[slot] = L.mu;
        s.weight[slot] = L.weight;
        s.e0[slot] = kinetic_energy_of(L.momentum, L.mc, L.rest_mass, L.speed_of_light);
        s.status[slot] = accepted ? L.status : 2;
        s.split_level[slot] = 0;
        s.sort_key[slot] = 0;
        ++written;
    }
    if (L.recycled != nullptr) {
        for (int off = 16; off > 0; off >>= 1) written += __shfl_down_sync(0xffffffffu, written, off);
        if ((threadIdx.x & 31u) == 0u && written) atomicAdd(L.recycled, written);
    }
}

// make_field_particle_candidate_set_in_region's predicate over one stored
// point (ParticleGenerator.hpp:689-725).
__device__ bool gen_point_accepted(const GenCandidateBuild& B, uint64_t point) {
    uint64_t linear = point;
    double coord[2];
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const uint64_t e = static_cast<uint64_t>(B.field.ext[dim]);
        const int index = static_cast<int>(linear % e) - 2;
        linear /= e;
        const LibAxis& a = B.grid.axis[dim];
        const int centering = B.field.centering[dim];
        if (index < gen_lower_index(a, centering, B.domain) ||
            index > gen_upper_index(a, centering, B.domain)) {
            return false;
        }
        coord[dim] = gen_coordinate(a, index, centering);
    }
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        if (coord[dim] < B.region_lo[dim] || coord[dim] > B.region_hi[dim]) return false;
    }
    return gen_compare(B.field.values[point * B.field.components + B.component], B.threshold,
                       B.comparison);
}

__global__ void __launch_bounds__(256) gen_candidate_count_kernel(const GenCandidateBuild B) {
    __shared__ unsigned int block_total;
    if (threadIdx.x == 0) block_total = 0;
    __syncthreads();
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    const bool take = i < B.points && gen_point_accepted(B, i);
    const unsigned ballot = __ballot_sync(0xffffffffu, take);
    if ((threadIdx.x & 31u) == 0u && ballot) atomicAdd(&block_total, __popc(ballot));
    __syncthreads();
    if (threadIdx.x == 0) B.block_counts[blockIdx.x] = block_total;
}

// Accepted points in index order (the serial scan's order).
__global__ void __launch_bounds__(256) gen_candidate_scatter_kernel(const GenCandidateBuild B) {
    __shared__ unsigned int warp_base[8];
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    const bool take = i < B.points && gen_point_accepted(B, i);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned ballot = __ballot_sync(0xffffffffu, take);
    if (lane == 0) warp_base[threadIdx.x >> 5] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int run = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
            const unsigned int c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (!take) return;
    const uint64_t dest = static_cast<uint64_t>(B.block_counts[blockIdx.x]) +
                          warp_base[threadIdx.x >> 5] + __popc(ballot & ((1u << lane) - 1u));
    B.indices[dest] = i;
}

// approximate_grid_cell_physical_volume on the Cartesian grid
// (ParticleGenerator.hpp:379-394): |jacobian| = 1 times the face-to-face
// widths, each width face(i+1) - face(i) as the analytic mapping rounds it.
__device__ __forceinline__ double gen_cell_volume(const LibGrid& g, const int (&cell)[2]) {
    double volume = 1.0;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = g.axis[dim];
        const double i = static_cast<double>(cell[dim]);
        const double width = __dsub_rn(lib_face(a, __dadd_rn(i, 1.0)), lib_face(a, i));
        volume = __dmul_rn(volume, fabs(width));
    }
    return isfinite(volume) && volume > 0.0 ? volume : 0.0;
}

// Candidate weights: field points clamp to the domain's cells
// (field_indices_to_volume_cell_indices, :419-433); grid candidates are the
// domain's cells in order (:823-845).
__global__ void gen_field_weight_kernel(const GenCandidateBuild B, uint64_t count) {
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < count;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint64_t linear = B.indices[c];
        int cell[2];
#pragma unroll
        for (int dim = 0; dim < 2; ++dim) {
            const uint64_t e = static_cast<uint64_t>(B.field.ext[dim]);
            int index = static_cast<int>(linear % e) - 2;
            linear /= e;
            const int lo = gen_lower_cell(B.grid.axis[dim], B.domain);
            const int hi = gen_upper_cell(B.grid.axis[dim], B.domain);
            cell[dim] = index < lo ? lo : (index > hi ? hi : index);
        }
        B.cumulative[c] = gen_cell_volume(B.grid, cell);
    }
}

__global__ void gen_grid_weight_kernel(LibGrid g, int lower0, int lower1, int extent0,
                                       int extent1, uint64_t count, double* weights) {
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < count;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const int cell[2] = {lower0 + static_cast<int>(c % static_cast<uint64_t>(extent0)),
                             lower1 + static_cast<int>((c / static_cast<uint64_t>(extent0)) %
                                                       static_cast<uint64_t>(extent1))};
        weights[c] = gen_cell_volume(g, cell);
    }
}

// FP64 inclusive scan in place: tiles of kScanTile values per block, each
// thread adding kScanItems consecutive values serially from its running
// offset.  Pass 1 writes the tile sums, pass 2 scans them (one block),
// pass 3 rewrites the tile.  The association is fixed, so the result is
// deterministic; it differs from a one-thread serial sum only by rounding.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr uint64_t kScanTile = static_cast<uint64_t>(kScanThreads) * kScanItems;

__device__ double block_exclusive_sum(double v, double* shared_warp, double* block_total) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = threadIdx.x >> 5;
    double inclusive = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const double o = __shfl_up_sync(0xffffffffu, inclusive, off);
        if (lane >= static_cast<unsigned>(off)) inclusive += o;
    }
    if (lane == 31u) shared_warp[warp] = inclusive;
    __syncthreads();
    if (threadIdx.x == 0) {
        double run = 0.0;
        for (int w = 0; w < kScanThreads / 32; ++w) {
            const double t = shared_warp[w];
            shared_warp[w] = run;
            run += t;
        }
        *block_total = run;
    }
    __syncthreads();
    double exclusive = __shfl_up_sync(0xffffffffu, inclusive, 1);
    if (lane == 0u) exclusive = 0.0;
    return shared_warp[warp] + exclusive;
}

__global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(const double* values,
                                                                      uint64_t n,
                                                                      double* tile_sums) {
    __shared__ double warp_sums[kScanThreads / 32];
    __shared__ double total;
    const uint64_t base = blockIdx.x * kScanTile + static_cast<uint64_t>(threadIdx.x) * kScanItems;
    double sum = 0.0;
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) sum += values[base + k];
    }
    (void)block_exclusive_sum(sum, warp_sums, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) scan_offsets_kernel(double* tile_sums, int tiles) {
    __shared__ double partial[1024];
    const int t = threadIdx.x;
    const int per = (tiles + blockDim.x - 1) / blockDim.x;
    const int begin = t * per;
    const int end = begin + per < tiles ? begin + per : tiles;
    double sum = 0.0;
    for (int k = begin; k < end; ++k) sum += tile_sums[k];
    partial[t] = sum;
    __syncthreads();
    if (t == 0) {
        double run = 0.0;
        for (int k = 0; k < static_cast<int>(blockDim.x); ++k) {
            const double v = partial[k];
            partial[k] = run;
            run += v;
        }
    }
    __syncthreads();
    double run = partial[t];
    for (int k = begin; k < end; ++k) {
        const double v = tile_sums[k];
        tile_sums[k] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(double* values, uint64_t n,
                                                                  const double* tile_offsets) {
    __shared__ double warp_sums[kScanThreads / 32];
    __shared__ double total;
    const uint64_t base = blockIdx.x * kScanTile + static_cast<uint64_t>(threadIdx.x) * kScanItems;
    double local[kScanItems];
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        local[k] = base + k < n ? values[base + k] : 0.0;
        sum += local[k];
    }
    double run = tile_offsets[blockIdx.x] + block_exclusive_sum(sum, warp_sums, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        run += local[k];
        if (base + k < n) values[base + k] = run;
    }
}

cudaError_t scan_inclusive_f64(double* values, uint64_t n, double* scratch, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int tiles = static_cast<int>((n + kScanTile - 1) / kScanTile);
    scan_tile_sums_kernel<<<tiles, kScanThreads, 0, stream>>>(values, n, scratch);
    scan_offsets_kernel<<<1, 1024, 0, stream>>>(scratch, tiles);
    scan_apply_kernel<<<tiles, kScanThreads, 0, stream>>>(values, n, scratch);
    return cudaGetLastError();
}

// ---- Parker coefficient precompute ------------------------------------------
//
// make_legacy_transport_coefficient_fields (ParkerCoefficient.hpp:1102-1155)
// on the Cartesian library grid, written straight into the packed basis the
// solver samples: curl(B/B^2), the gamma-one kappas, the diffusion-tensor
// divergence bases, div V, each with its ghost cells filled.  Metric factors
// are 1 and enter as exact multiplications by 1; every other operation is
// rounded on its own in the reference's order, so only pow's last bits
// differ from the reference build.

__device__ __forceinline__ size_t coef_point(const LibGrid& g, int i, int j) {
    return static_cast<size_t>(i + 2) + static_cast<size_t>(j + 2) * static_cast<size_t>(g.ex);
}

// centered_three_point_derivative (ParkerCoefficient.hpp:215-234).
__device__ double coef_d3(double lc, double cc, double uc, double lv, double cv, double uv) {
    const double lw = __dsub_rn(cc, lc);
    const double uw = __dsub_rn(uc, cc);
    const double tw = __dsub_rn(uc, lc);
    const double a = __ddiv_rn(-uw, __dmul_rn(lw, tw));
    const double b = __ddiv_rn(__dsub_rn(uw, lw), __dmul_rn(lw, uw));
    const double c = __ddiv_rn(lw, __dmul_rn(uw, tw));
    return __dadd_rn(__dadd_rn(__dmul_rn(a, lv), __dmul_rn(b, cv)), __dmul_rn(c, uv));
}

__device__ __forceinline__ double coef_norm2(const double* row) {
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) s = __dadd_rn(s, __dmul_rn(row[c], row[c]));
    return s;
}

// Errors: the word starts at kCoefNoError and keeps the smallest code, the
// codes numbered in the reference's stage order (curl before the kappas
// before the divergence bases), so the message is the one the reference
// aborts with first.
constexpr int kCoefNoError = 0x7fffffff;
__device__ __forceinline__ void coef_set_error(int* error, int code) { atomicMin(error, code); }

// B_c / max(B^2, floor) (ParkerCoefficient.hpp:278-305), times h_c = 1.
__device__ __forceinline__ double coef_b_over_b2(const CoefLaunch& L, int i, int j, int c) {
    const double* row = L.b + 3 * coef_point(L.grid, i, j);
    const double b2 = coef_norm2(row);
    if (b2 <= 0.0 && L.drift_floor <= 0.0) {
        coef_set_error(L.error, 20);  // curl(B/B^2) is undefined where B^2 <= 0
    }
    const double den = b2 > L.drift_floor ? b2 : L.drift_floor;
    return __ddiv_rn(row[c], den);
}

// centered_metric_weighted_derivative (ParkerCoefficient.hpp:332-387):
// (upper - lower) / (x_upper - x_lower) along dim of h_c B_c / B^2.
__device__ double coef_curl_derivative(const CoefLaunch& L, int i, int j, int dim, int c) {
    if (dim >= 2 || L.grid.axis[dim].n <= 1) return 0.0;
    const int li = dim == 0 ? i - 1 : i, lj = dim == 1 ? j - 1 : j;
    const int ui = dim == 0 ? i + 1 : i, uj = dim == 1 ? j + 1 : j;
    const LibAxis& a = L.grid.axis[dim];
    const double width = __dsub_rn(gen_coordinate(a, dim == 0 ? ui : uj, 0),
                                   gen_coordinate(a, dim == 0 ? li : lj, 0));
    return __ddiv_rn(__dsub_rn(coef_b_over_b2(L, ui, uj, c), coef_b_over_b2(L, li, lj, c)),
                     width);
}

// The three-point weights of centered_three_point_derivative
// (ParkerCoefficient.hpp:215-234) at one logical index: a derivative is
// a lv + b cv + c uv, each product and sum rounded as coef_d3 rounds them.
struct D3Weights {
    double a, b, c;
};
__device__ __forceinline__ D3Weights coef_d3_weights(double lc, double cc, double uc) {
    const double lw = __dsub_rn(cc, lc);
    const double uw = __dsub_rn(uc, cc);
    const double tw = __dsub_rn(uc, lc);
    return D3Weights{__ddiv_rn(-uw, __dmul_rn(lw, tw)),
                     __ddiv_rn(__dsub_rn(uw, lw), __dmul_rn(lw, uw)),
                     __ddiv_rn(lw, __dmul_rn(uw, tw))};
}
__device__ __forceinline__ double coef_d3_apply(const D3Weights& w, double lv, double cv,
                                                double uv) {
    return __dadd_rn(__dadd_rn(__dmul_rn(w.a, lv), __dmul_rn(w.b, cv)), __dmul_rn(w.c, uv));
}

// The direction and kappas of one point of a diffusion tensor
// (ParkerCoefficient.hpp:606-641): b = B / max(|B|, floor).
struct TensorPoint {
    double b[3];
    double kpar, kperp;
};
__device__ TensorPoint coef_tensor_point(const CoefLaunch& L, int i, int j) {
    const size_t p = coef_point(L.grid, i, j);
    const double* row = L.b + 3 * p;
    const double magnitude = __dsqrt_rn(coef_norm2(row));
    if (magnitude <= 0.0 && L.min_b <= 0.0) {
        coef_set_error(L.error, 26);  // diffusion tensor direction is undefined where |B| <= 0
    }
    const double den = magnitude > L.min_b ? magnitude : L.min_b;
    TensorPoint t;
#pragma unroll
    for (int c = 0; c < 3; ++c) t.b[c] = __ddiv_rn(row[c], den);
    t.kpar = L.packed[p * L.stride + L.kpar_slot];
    t.kperp = L.packed[p * L.stride + L.kperp_slot];
    return t;
}

// One gamma-independent diffusion tensor basis component
// (ParkerCoefficient.hpp:606-641); basis 0 parallel projection, 1
// perpendicular projection, 2 constant parallel ratio.
__device__ __forceinline__ double coef_tensor(const CoefLaunch& L, const TensorPoint& t, int oc,
                                              int dc, int basis) {
    const double projection = __dmul_rn(t.b[oc], t.b[dc]);
    const double identity = oc == dc ? 1.0 : 0.0;
    if (basis == 0) return __dmul_rn(t.kpar, projection);
    if (basis == 1) return __dmul_rn(t.kperp, __dsub_rn(identity, projection));
    return __dmul_rn(t.kpar, __dadd_rn(__dmul_rn(L.ratio, identity),
                                       __dmul_rn(__dsub_rn(1.0, L.ratio), projection)));
}

// Everything a point's divergence bases read, formed once per point: the
// tensor points of the point and of its neighbours along each axis that has
// more than one cell, the three-point weights of each such axis, and the
// centred derivative of the Lame coefficient h = 1 along it
// (centered_lame_derivative, ParkerCoefficient.hpp:746-790).  The values are
// the ones the reference forms at every use, with the same rounding.
struct TensorStencil {
    TensorPoint centre, lower[2], upper[2];
    D3Weights weights[2];
    double lame[2];
    bool active[2];
};
__device__ __forceinline__ TensorStencil coef_tensor_stencil(const CoefLaunch& L, int i, int j) {
    TensorStencil s;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        const LibAxis& a = L.grid.axis[dim];
        s.active[dim] = a.n > 1;
        s.lame[dim] = 0.0;
        if (!s.active[dim]) continue;
        const int k = dim == 0 ? i : j;
        s.weights[dim] = coef_d3_weights(gen_coordinate(a, k - 1, 0), gen_coordinate(a, k, 0),
                                         gen_coordinate(a, k + 1, 0));
        s.lame[dim] = coef_d3_apply(s.weights[dim], 1.0, 1.0, 1.0);
        s.lower[dim] = coef_tensor_point(L, dim == 0 ? i - 1 : i, dim == 1 ? j - 1 : j);
        s.upper[dim] = coef_tensor_point(L, dim == 0 ? i + 1 : i, dim == 1 ? j + 1 : j);
    }
    s.centre = coef_tensor_point(L, i, j);
    return s;
}

// diffusion_tensor_divergence_basis_component (ParkerCoefficient.hpp:794-877).
__device__ __forceinline__ double coef_divergence_basis(const CoefLaunch& L,
                                                        const TensorStencil& s, int oc,
                                                        int basis) {
    double result = 0.0;
#pragma unroll
    for (int dim = 0; dim < 2; ++dim) {
        if (!s.active[dim]) {
            result = __dadd_rn(result, 0.0);
            continue;
        }
        const double lv = coef_tensor(L, s.lower[dim], oc, dim, basis);
        const double cv = coef_tensor(L, s.centre, oc, dim, basis);
        const double uv = coef_tensor(L, s.upper[dim], oc, dim, basis);
        result = __dadd_rn(result, coef_d3_apply(s.weights[dim], lv, cv, uv));
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c == oc) continue;
        if (c < 2) {
            const double t = coef_tensor(L, s.centre, oc, c, basis);
            result = __dadd_rn(result, __dmul_rn(t, s.lame[c]));
        }
        if (oc < 2) {
            const double t = coef_tensor(L, s.centre, c, c, basis);
            result = __dsub_rn(result, __dmul_rn(t, s.lame[oc]));
        }
    }
    return result;
}

__device__ __forceinline__ double coef_floor(double v, double f) {
    if (f <= 0.0) return v;
    return v < f ? f : v;
}

// The gamma-one kappas at one physical point (LegencyModel.hpp:434-470,
// :801-862); false after recording the failed check.
__device__ bool coef_kappas(const CoefLaunch& L, uint64_t p, const double* b, const double* v,
                            double& kpar_out, double& kperp_out) {
    const double safe_b = coef_floor(__dsqrt_rn(coef_norm2(b)), L.min_b);
    const double safe_vsw = coef_floor(__dsqrt_rn(coef_norm2(v)), L.min_vsw);
    const double sigma2 = L.turbulence_fields ? L.sigma2_field[p] : L.sigma2;
    const double l2d = L.turbulence_fields ? L.l2d_field[p] : L.l2d;
    const double lc = L.turbulence_fields ? L.lc_field[p] : L.lc;
    const double safe_sigma2 = coef_floor(sigma2, L.min_sigma2);
    if (safe_b <= 0.0) {
        coef_set_error(L.error, 21);  // gyrofrequency requires |B| > 0
        return false;
    }
    const double omega = __ddiv_rn(__dmul_rn(L.abs_charge, safe_b),
                                   __dmul_rn(L.rest_mass, L.speed_of_light));
    if (safe_vsw <= 0.0 || lc <= 0.0 || omega <= 0.0 || safe_sigma2 <= 0.0) {
        coef_set_error(L.error, 22);  // kappa_parallel requires positive inputs
        return false;
    }
    const double kpar = __ddiv_rn(
        __dmul_rn(__dmul_rn(L.parallel_prefactor, pow(safe_vsw, 4.0 / 3.0)), pow(lc, 2.0 / 3.0)),
        __dmul_rn(pow(omega, 1.0 / 3.0), safe_sigma2));
    double kperp;
    if (L.constant_ratio) {
        if (kpar <= 0.0 || L.ratio <= 0.0) {
            coef_set_error(L.error, 24);
            return false;
        }
        kperp = __dmul_rn(L.ratio, kpar);
    } else {
        if (safe_vsw <= 0.0 || l2d <= 0.0 || safe_sigma2 <= 0.0 || kpar <= 0.0) {
            coef_set_error(L.error, 23);
            return false;
        }
        kperp = __dmul_rn(
            __dmul_rn(__ddiv_rn(safe_vsw, 3.0),
                      pow(__ddiv_rn(__dmul_rn(3.0, kpar), safe_vsw), 1.0 / 3.0)),
            pow(__dmul_rn(__dmul_rn(L.perpendicular_prefactor, safe_sigma2), l2d), 2.0 / 3.0));
    }
    kpar_out = kpar;
    kperp_out = kperp;
    return true;
}

// Stage 1: B and V into the packed rows (every point, ghosts as given), the
// derived slots zeroed (the reference's freshly allocated fields), and the
// gamma-one kappas at the physical points
// (LegencyModel.hpp:434-470, :801-862).
__global__ void coef_kappa_kernel(const CoefLaunch L) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < points;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        double* out = L.packed + p * kLibBasisStride;
        const double* b = L.b + 3 * p;
        const double* v = L.v + 3 * p;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            out[c] = b[c];
            out[3 + c] = v[c];
        }
#pragma unroll
        for (int c = 6; c < kLibBasis; ++c) out[c] = 0.0;
        const int i = static_cast<int>(p % static_cast<uint64_t>(L.grid.ex)) - 2;
        const int j = static_cast<int>(p / static_cast<uint64_t>(L.grid.ex)) - 2;
        if (i < 0 || i >= L.grid.axis[0].n || j < 0 || j >= L.grid.axis[1].n) continue;
        // curl(B/B^2) reads B^2 at the x and y neighbours first
        if (L.drift_floor <= 0.0) {
#pragma unroll
            for (int dim = 0; dim < 2; ++dim) {
                if (L.grid.axis[dim].n <= 1) continue;
#pragma unroll
                for (int side = -1; side <= 1; side += 2) {
                    const size_t q = coef_point(L.grid, dim == 0 ? i + side : i,
                                                dim == 1 ? j + side : j);
                    if (coef_norm2(L.b + 3 * q) <= 0.0) coef_set_error(L.error, 20);
                }
            }
        }
        double kpar = 0.0, kperp = 0.0;
        if (!coef_kappas(L, p, b, v, kpar, kperp)) continue;
        out[15] = kpar;
        out[16] = kperp;
    }
}

// Field::fill_ghost_cells for cell-centred packed slots [first, last] and
// slot `extra` (Field.hpp:274-316): a ghost point copies its periodic image
// or, on an open axis, the nearest physical point (PeriodicOnly leaves it).
__global__ void coef_ghost_kernel(const CoefLaunch L, double* base, int stride, int first,
                                  int last, int extra) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < points;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        int idx[2] = {static_cast<int>(p % static_cast<uint64_t>(L.grid.ex)) - 2,
                      static_cast<int>(p / static_cast<uint64_t>(L.grid.ex)) - 2};
        bool ghost = false;
        bool skip = false;
#pragma unroll
        for (int dim = 0; dim < 2; ++dim) {
            const int n = L.grid.axis[dim].n;
            if (idx[dim] < 0 || idx[dim] > n - 1) {
                ghost = true;
                if (L.grid.axis[dim].periodic) {
                    int w = idx[dim] % n;
                    if (w < 0) w += n;
                    idx[dim] = w;
                } else if (L.ghost_mode == 1) {
                    skip = true;
                } else {
                    idx[dim] = idx[dim] < 0 ? 0 : n - 1;
                }
            }
        }
        if (!ghost || skip) continue;
        const double* src = base + coef_point(L.grid, idx[0], idx[1]) * stride;
        double* dst = base + p * stride;
        for (int c = first; c <= last; ++c) dst[c] = src[c];
        if (extra >= 0) dst[extra] = src[extra];
    }
}

// Stage 2 (after the kappas' ghosts): curl(B/B^2), the divergence bases
// and div V at the physical points.
__global__ void coef_derivative_kernel(const CoefLaunch L) {
    const int nx = L.grid.axis[0].n, ny = L.grid.axis[1].n;
    const uint64_t cells = static_cast<uint64_t>(nx) * ny;
    if (*L.error != kCoefNoError) return;
    for (uint64_t q = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; q < cells;
         q += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(q % static_cast<uint64_t>(nx));
        const int j = static_cast<int>(q / static_cast<uint64_t>(nx));
        double* out = L.packed + coef_point(L.grid, i, j) * kLibBasisStride;
        // magnetic_field_over_magnitude_squared_curl_component (:389-422)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int da = (c + 1) % 3, db = (c + 2) % 3;
            const double a = coef_curl_derivative(L, i, j, da, db);
            const double b = coef_curl_derivative(L, i, j, db, da);
            out[6 + c] = __dsub_rn(a, b);
        }
        // diffusion tensor divergence bases (:960-1095)
        const TensorStencil ts = coef_tensor_stencil(L, i, j);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (L.constant_ratio) {
                const double value = coef_divergence_basis(L, ts, c, 2);
                out[9 + c] = value;
                out[12 + c] = value;
            } else {
                out[9 + c] = coef_divergence_basis(L, ts, c, 0);
                out[12 + c] = coef_divergence_basis(L, ts, c, 1);
            }
        }
        // FieldOperator::divergence_value of V (FieldOperator.hpp:262-277)
        double div = 0.0;
        for (int dim = 0; dim < 2; ++dim) {
            if (L.grid.axis[dim].n <= 1) {
                div = __dadd_rn(div, 0.0);
                continue;
            }
            const LibAxis& a = L.grid.axis[dim];
            const int k = dim == 0 ? i : j;
            const double lv = L.v[3 * coef_point(L.grid, dim == 0 ? i - 1 : i,
                                                 dim == 1 ? j - 1 : j) + dim];
            const double cv = L.v[3 * coef_point(L.grid, i, j) + dim];
            const double uv = L.v[3 * coef_point(L.grid, dim == 0 ? i + 1 : i,
                                                 dim == 1 ? j + 1 : j) + dim];
            div = __dadd_rn(div, coef_d3(gen_coordinate(a, k - 1, 0), gen_coordinate(a, k, 0),
                                         gen_coordinate(a, k + 1, 0), lv, cv, uv));
        }
        out[17] = div;
    }
}

// ---- focused transport coefficient precompute --------------------------------
//
// make_legacy_transport_coefficient_fields_with_time_derivative
// (FocusCoefficient.hpp:852-993) into the focused packed basis
// (FocusSolver.hpp:106-136): B b V, drift bases over |B|, the perpendicular
// diffusion advection, |B|, the kappas, div V, b.grad ln|B|, bb:grad V,
// b.dV/dt, sigma^2 and Lc.  ln|B|, grad ln|B| and the curvature (b.grad)b
// live in an 8-double scratch row per point.  Fields the reference fills
// at every point (|B|, b, ln|B|, the drift bases, the scattering inputs)
// are computed at every point here too, before the same ghost fills.
constexpr int kFocusScratch = 8;

// Centred derivative of one component along dim at a physical point
// (FieldOperator.hpp:106-143), 0 on an ignorable or single-cell axis.
__device__ __forceinline__ double coef_component_derivative(const CoefLaunch& L,
                                                           const double* base, int stride,
                                                           int i, int j, int dim, int c) {
    if (dim >= 2 || L.grid.axis[dim].n <= 1) return 0.0;
    const LibAxis& a = L.grid.axis[dim];
    const int k = dim == 0 ? i : j;
    const double lv = base[coef_point(L.grid, dim == 0 ? i - 1 : i, dim == 1 ? j - 1 : j) * stride + c];
    const double cv = base[coef_point(L.grid, i, j) * stride + c];
    const double uv = base[coef_point(L.grid, dim == 0 ? i + 1 : i, dim == 1 ? j + 1 : j) * stride + c];
    return coef_d3(gen_coordinate(a, k - 1, 0), gen_coordinate(a, k, 0),
                   gen_coordinate(a, k + 1, 0), lv, cv, uv);
}

__device__ __forceinline__ bool coef_physical(const CoefLaunch& L, uint64_t p, int& i, int& j) {
    i = static_cast<int>(p % static_cast<uint64_t>(L.grid.ex)) - 2;
    j = static_cast<int>(p / static_cast<uint64_t>(L.grid.ex)) - 2;
    return i >= 0 && i < L.grid.axis[0].n && j >= 0 && j < L.grid.axis[1].n;
}

// Stage 1, every point: B, V, |B| (fill_magnitude), b (fill_direction with
// ZeroMagnitudePolicy::Abort), ln max(|B|, floor), the scattering sigma^2
// and Lc; the kappas at the physical points.
__global__ void focus_stage1_kernel(const CoefLaunch L) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < points;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        double* out = L.packed + p * L.stride;
        const double* b = L.b + 3 * p;
        const double* v = L.v + 3 * p;
        for (int c = 0; c < L.stride; ++c) out[c] = 0.0;
        const double magnitude = __dsqrt_rn(coef_norm2(b));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            out[c] = b[c];
            out[6 + c] = v[c];
        }
        out[18] = magnitude;
        if (magnitude <= L.direction_floor) {
            coef_set_error(L.error, 10);  // direction is undefined at zero magnitude
        } else {
            const double inverse = __ddiv_rn(1.0, magnitude);
#pragma unroll
            for (int c = 0; c < 3; ++c) out[3 + c] = __dmul_rn(b[c], inverse);
        }
        const double safe = magnitude > L.direction_floor ? magnitude : L.direction_floor;
        double* scratch = L.scratch + p * kFocusScratch;
#pragma unroll
        for (int c = 0; c < kFocusScratch; ++c) scratch[c] = 0.0;
        if (safe <= 0.0) {
            coef_set_error(L.error, 11);  // ln |B| requires a positive magnetic field
        } else {
            scratch[0] = log(safe);
        }
        out[25] = L.turbulence_fields ? L.sigma2_field[p] : L.sigma2;
        out[26] = L.turbulence_fields ? L.lc_field[p] : L.lc;
        int i, j;
        if (!coef_physical(L, p, i, j)) continue;
        double kpar = 0.0, kperp = 0.0;
        if (!coef_kappas(L, p, b, v, kpar, kperp)) continue;
        out[19] = kpar;
        out[20] = kperp;
    }
}

// Stage 2, physical points: grad ln|B| (fill_gradient) and the curvature
// (b.grad)b (FocusCoefficient.hpp:428-452, :559-595).
__global__ void focus_stage2_kernel(const CoefLaunch L) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < points;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        int i, j;
        if (!coef_physical(L, p, i, j)) continue;
        double* scratch = L.scratch + p * kFocusScratch;
        const double* dir = L.packed + p * L.stride + 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            scratch[1 + c] = c < 2 ? coef_component_derivative(L, L.scratch, kFocusScratch, i, j, c, 0)
                                   : 0.0;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double result = 0.0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double g = coef_component_derivative(L, L.packed + 3, L.stride, i, j, d, c);
                result = __dadd_rn(result, __dmul_rn(dir[d], g));
            }
            scratch[4 + c] = result;
        }
    }
}

__device__ __forceinline__ double coef_cross(const double* a, const double* b, int c) {
    if (c == 0) return __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
    if (c == 1) return __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
    return __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}

// Stage 3, every point: the drift bases b x grad ln|B| / |B| and
// b x (b.grad)b / |B| (FocusCoefficient.hpp:617-703).
__global__ void focus_stage3_kernel(const CoefLaunch L) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < points;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        double* out = L.packed + p * L.stride;
        const double* scratch = L.scratch + p * kFocusScratch;
        const double m = out[18] > L.direction_floor ? out[18] : L.direction_floor;
        if (m <= 0.0) {
            coef_set_error(L.error, 12);  // focused drift requires |B| > 0
            continue;
        }
        const double inverse = __ddiv_rn(1.0, m);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            out[9 + c] = __dmul_rn(coef_cross(out + 3, scratch + 1, c), inverse);
            out[12 + c] = __dmul_rn(coef_cross(out + 3, scratch + 4, c), inverse);
        }
    }
}

// Velocity gradient (grad V)_{oc, dc} in Cartesian components
// (FocusCoefficient.hpp:240-326).
__device__ __forceinline__ double coef_velocity_gradient(const CoefLaunch& L, int i, int j,
                                                         int oc, int dc) {
    return coef_component_derivative(L, L.v, 3, i, j, dc, oc);
}

// Stage 4, physical points: the perpendicular diffusion advection
// (FocusCoefficient.hpp:829-850), div V and the contractions
// (FocusCoefficient.hpp:705-781).
__global__ void focus_stage4_kernel(const CoefLaunch L) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    if (*L.error != kCoefNoError) return;
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < points;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        int i, j;
        if (!coef_physical(L, p, i, j)) continue;
        double* out = L.packed + p * L.stride;
        const double* scratch = L.scratch + p * kFocusScratch;
        const TensorStencil ts = coef_tensor_stencil(L, i, j);
#pragma unroll
        for (int c = 0; c < 3; ++c) out[15 + c] = coef_divergence_basis(L, ts, c, 1);
        double div = 0.0;
        for (int dim = 0; dim < 2; ++dim) {
            div = __dadd_rn(div, coef_component_derivative(L, L.v, 3, i, j, dim, dim));
        }
        out[21] = div;
        const double* dir = out + 3;
        const double* v = L.v + 3 * p;
        double focusing = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) focusing = __dadd_rn(focusing, __dmul_rn(dir[c], scratch[1 + c]));
        out[22] = focusing;
        double bb = 0.0;
        double convective = 0.0;
        for (int oc = 0; oc < 3; ++oc) {
            for (int dc = 0; dc < 3; ++dc) {
                const double g = coef_velocity_gradient(L, i, j, oc, dc);
                bb = __dadd_rn(bb, __dmul_rn(__dmul_rn(dir[oc], dir[dc]), g));
                convective = __dadd_rn(convective, __dmul_rn(__dmul_rn(dir[oc], v[dc]), g));
            }
        }
        out[23] = bb;
        double partial = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double dv = L.dvdt != nullptr ? L.dvdt[3 * p + c] : 0.0;
            partial = __dadd_rn(partial, __dmul_rn(dir[c], dv));
        }
        out[24] = __dadd_rn(partial, convective);
    }
}

int grid_for(uint64_t n, int threads) {
    const uint64_t want = (n + threads - 1) / threads;
    return static_cast<int>(want < 1 ? 1 : (want > 152u * 32u ? 152u * 32u : want));
}

}  // namespace

// The FP32 copy of a packed basis for the mixed step: each row rounded to
// FP32 and padded with zeros to dst_stride floats.
__global__ void basis_to_f32_kernel(const double* __restrict__ src, int src_stride,
                                    float* __restrict__ dst, int dst_stride, int comps,
                                    uint64_t points) {
    const uint64_t n = points * static_cast<uint64_t>(dst_stride);
    for (uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t point = k / dst_stride;
        const int c = static_cast<int>(k % dst_stride);
        dst[k] = c < comps ? static_cast<float>(src[point * src_stride + c]) : 0.0f;
    }
}

cudaError_t lib_basis_to_f32(const double* src, int src_stride, float* dst, int dst_stride,
                             int comps, uint64_t points, cudaStream_t stream) {
    if (points == 0) return cudaSuccess;
    basis_to_f32_kernel<<<grid_for(points * dst_stride, 256), 256, 0, stream>>>(
        src, src_stride, dst, dst_stride, comps, points);
    return cudaGetLastError();
}

cudaError_t lib_parker_step(const LibParkerLaunch& L, cudaStream_t stream) {
    lib_reset_min_kernel<<<1, 1, 0, stream>>>(L.min_bits);
    if (L.count > 0) {
        if (L.mixed) {
            lib_parker_terms_kernel<float><<<grid_for(L.count, 256), 256, 0, stream>>>(L);
        } else {
            lib_parker_terms_kernel<double><<<grid_for(L.count, 256), 256, 0, stream>>>(L);
        }
    }
    lib_finish_dt_kernel<<<1, 1, 0, stream>>>(L.min_bits, L.courant, L.dt_device_out,
                                              L.dt_history, L.error, L.advance);
    if (L.advance) {
        LibParkerLaunch A = L;
        A.dt_device = L.dt_device_out;
        if (L.mixed) {
            lib_parker_advance_kernel<float><<<grid_for(L.capacity, 256), 256, 0, stream>>>(A);
        } else {
            lib_parker_advance_kernel<double><<<grid_for(L.capacity, 256), 256, 0, stream>>>(A);
        }
    }
    return cudaGetLastError();
}

cudaError_t lib_focus_step(const LibFocusLaunch& L, cudaStream_t stream) {
    lib_reset_min_kernel<<<1, 1, 0, stream>>>(L.min_bits);
    if (L.count > 0) {
        if (L.mixed) {
            focus_terms_kernel<float><<<grid_for(L.count, 256), 256, 0, stream>>>(L);
        } else {
            focus_terms_kernel<double><<<grid_for(L.count, 256), 256, 0, stream>>>(L);
        }
    }
    lib_finish_dt_kernel<<<1, 1, 0, stream>>>(L.min_bits, L.courant, L.dt_device_out,
                                              L.dt_history, L.error, L.advance);
    if (L.advance) {
        LibFocusLaunch A = L;
        A.dt_device = L.dt_device_out;
        if (L.mixed) {
            focus_advance_kernel<float><<<grid_for(L.capacity, 256), 256, 0, stream>>>(A);
        } else {
            focus_advance_kernel<double><<<grid_for(L.capacity, 256), 256, 0, stream>>>(A);
        }
    }
    return cudaGetLastError();
}

cudaError_t system_default_state(const SystemArrays& s, uint64_t count, uint64_t capacity,
                                 cudaStream_t stream) {
    if (capacity == 0) return cudaSuccess;
    system_default_kernel<<<grid_for(capacity, 256), 256, 0, stream>>>(s, count, capacity);
    return cudaGetLastError();
}

cudaError_t system_boundary(const LibGrid& g, const SystemArrays& s, uint64_t count,
                            cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    system_boundary_kernel<<<grid_for(count, 256), 256, 0, stream>>>(g, s, count);
    return cudaGetLastError();
}

cudaError_t system_capture(const SystemArrays& s, uint64_t capacity, cudaStream_t stream) {
    if (capacity == 0) return cudaSuccess;
    system_capture_kernel<<<grid_for(capacity, 256), 256, 0, stream>>>(s, capacity);
    return cudaGetLastError();
}

cudaError_t system_reset_baselines(const LibSplitLaunch& L, cudaStream_t stream) {
    if (L.count == 0) return cudaSuccess;
    system_reset_baselines_kernel<<<grid_for(L.count, 256), 256, 0, stream>>>(L);
    return cudaGetLastError();
}

cudaError_t system_split(const LibSplitLaunch& L, cudaStream_t stream) {
    const int blocks = static_cast<int>((L.count + 255) / 256);
    system_split_count_kernel<<<blocks, 256, 0, stream>>>(L);
    system_split_scan_kernel<<<1, 1024, 0, stream>>>(L.block_counts, blocks, L.tallies + 4);
    system_split_scatter_kernel<<<blocks, 256, 0, stream>>>(L);
    return cudaGetLastError();
}

cudaError_t system_sort(const LibSortLaunch& L, cudaStream_t stream) {
    const long long range = static_cast<long long>(L.hi) - L.lo + 1;
    const int bins = static_cast<int>(range);
    int bits = 0;
    while (bits < 32 && (1ll << bits) < range) ++bits;
    const int passes = (bits + 7) / 8;
    const int blocks = static_cast<int>((L.count + kRadixThreads - 1) / kRadixThreads);
    unsigned int* k_cur = L.keys_a;
    unsigned int* i_cur = L.idx_a;
    unsigned int* k_alt = L.keys_b;
    unsigned int* i_alt = L.idx_b;
    radix_init_kernel<<<grid_for(L.count, 256), 256, 0, stream>>>(L.sys.sort_key, L.count, L.lo,
                                                                  bins, k_cur, i_cur);
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = 8 * pass;
        radix_hist_kernel<<<blocks, kRadixThreads, 0, stream>>>(k_cur, L.count, shift, L.hist,
                                                                blocks);
        system_split_scan_kernel<<<1, 1024, 0, stream>>>(L.hist, 256 * blocks, L.scratch_total);
        radix_scatter_kernel<<<blocks, kRadixThreads, 0, stream>>>(
            k_cur, i_cur, L.count, shift, L.hist, blocks, k_alt, i_alt);
        unsigned int* t = k_cur;
        k_cur = k_alt;
        k_alt = t;
        t = i_cur;
        i_cur = i_alt;
        i_alt = t;
    }
    const unsigned int* perm = i_cur;
    const int g = grid_for(L.count, 256);
    const SystemArrays& s = L.sys;
    cudaError_t err;
    // gather every array through the permutation via the staging buffer
    double* sd[10] = {s.x, s.y, s.prev_x, s.prev_y, s.prevstep_x, s.prevstep_y, s.p, s.mu,
                      s.weight, s.e0};
    for (double* a : sd) {
        gather_kernel<double><<<g, 256, 0, stream>>>(a, static_cast<double*>(L.staging), perm,
                                                     L.count);
        err = cudaMemcpyAsync(a, L.staging, sizeof(double) * L.count, cudaMemcpyDeviceToDevice,
                              stream);
        if (err != cudaSuccess) return err;
    }
    int* si[3] = {s.status, s.split_level, s.sort_key};
    for (int* a : si) {
        gather_kernel<int><<<g, 256, 0, stream>>>(a, static_cast<int*>(L.staging), perm, L.count);
        err = cudaMemcpyAsync(a, L.staging, sizeof(int) * L.count, cudaMemcpyDeviceToDevice,
                              stream);
        if (err != cudaSuccess) return err;
    }
    gather_kernel<unsigned long long><<<g, 256, 0, stream>>>(
        reinterpret_cast<const unsigned long long*>(s.id),
        static_cast<unsigned long long*>(L.staging), perm, L.count);
    err = cudaMemcpyAsync(s.id, L.staging, sizeof(uint64_t) * L.count, cudaMemcpyDeviceToDevice,
                          stream);
    if (err != cudaSuccess) return err;
    return cudaGetLastError();
}

cudaError_t system_compact_keys(const SystemArrays& s, uint64_t count, unsigned long long* active,
                                cudaStream_t stream) {
    cudaError_t err = cudaMemsetAsync(active, 0, sizeof(unsigned long long), stream);
    if (err != cudaSuccess) return err;
    if (count == 0) return cudaSuccess;
    compact_keys_kernel<<<grid_for(count, 256), 256, 0, stream>>>(s.status, s.sort_key, count,
                                                                  active);
    return cudaGetLastError();
}

cudaError_t generator_run(const GenLaunch& L, cudaStream_t stream) {
    if (L.recycled != nullptr) {
        const cudaError_t err = cudaMemsetAsync(L.recycled, 0, sizeof(unsigned long long), stream);
        if (err != cudaSuccess) return err;
    }
    if (L.count == 0) return cudaSuccess;
    generator_kernel<<<grid_for(L.count, 256), 256, 0, stream>>>(L);
    return cudaGetLastError();
}

cudaError_t generator_field_candidates(const GenCandidateBuild& B, cudaStream_t stream) {
    if (B.points == 0) {
        return cudaMemsetAsync(B.count_out, 0, sizeof(unsigned long long), stream);
    }
    const int blocks = static_cast<int>((B.points + 255) / 256);
    gen_candidate_count_kernel<<<blocks, 256, 0, stream>>>(B);
    system_split_scan_kernel<<<1, 1024, 0, stream>>>(B.block_counts, blocks, B.count_out);
    gen_candidate_scatter_kernel<<<blocks, 256, 0, stream>>>(B);
    return cudaGetLastError();
}

cudaError_t generator_field_weights(const GenCandidateBuild& B, uint64_t count,
                                    cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    gen_field_weight_kernel<<<grid_for(count, 256), 256, 0, stream>>>(B, count);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    return scan_inclusive_f64(B.cumulative, count, B.block_sums, stream);
}

cudaError_t generator_grid_weights(const LibGrid& g, const int lower[2], const int extents[2],
                                   uint64_t count, double* cumulative, double* block_sums,
                                   cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    gen_grid_weight_kernel<<<grid_for(count, 256), 256, 0, stream>>>(
        g, lower[0], lower[1], extents[0], extents[1], count, cumulative);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    return scan_inclusive_f64(cumulative, count, block_sums, stream);
}

uint64_t generator_scan_scratch(uint64_t count) {
    return (count + kScanTile - 1) / kScanTile + 1;
}

int parker_coefficients_no_error() { return kCoefNoError; }

cudaError_t parker_coefficients(const CoefLaunch& L, cudaStream_t stream) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    const uint64_t cells = static_cast<uint64_t>(L.grid.axis[0].n) * L.grid.axis[1].n;
    coef_kappa_kernel<<<grid_for(points, 256), 256, 0, stream>>>(L);
    coef_ghost_kernel<<<grid_for(points, 256), 256, 0, stream>>>(L, L.packed, L.stride, 15, 16,
                                                                 -1);
    coef_derivative_kernel<<<grid_for(cells, 128), 128, 0, stream>>>(L);
    coef_ghost_kernel<<<grid_for(points, 256), 256, 0, stream>>>(L, L.packed, L.stride, 6, 14,
                                                                 17);
    return cudaGetLastError();
}

cudaError_t focus_coefficients(const CoefLaunch& L, cudaStream_t stream) {
    const uint64_t points = static_cast<uint64_t>(L.grid.ex) * (L.grid.axis[1].n + 4);
    const int g = grid_for(points, 256);
    focus_stage1_kernel<<<g, 256, 0, stream>>>(L);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.scratch, kFocusScratch, 0, 0, -1);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.packed, L.stride, 19, 20, -1);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.packed, L.stride, 25, 26, -1);
    focus_stage2_kernel<<<grid_for(points, 128), 128, 0, stream>>>(L);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.scratch, kFocusScratch, 1, 6, -1);
    focus_stage3_kernel<<<g, 256, 0, stream>>>(L);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.packed, L.stride, 9, 14, -1);
    focus_stage4_kernel<<<grid_for(points, 128), 128, 0, stream>>>(L);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.packed, L.stride, 15, 17, -1);
    coef_ghost_kernel<<<g, 256, 0, stream>>>(L, L.packed, L.stride, 21, 24, -1);
    return cudaGetLastError();
}

}  // namespace kpt
