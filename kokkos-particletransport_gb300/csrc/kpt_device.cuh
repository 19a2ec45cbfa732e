// Device-side building blocks shared by the push, field and lifecycle kernels:
// the keyed Philox noise stream, the driver's periodic wrap, the grid maps
// (analytic uniform axis / stored-edge axis) and the bilinear stencil.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "kpt_types.h"

namespace kpt {

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon et al., SC'11).  Stream layout: key = seed halves,
// counter = (block, index, frame, tag); draw n uses block n/2, words
// 2(n%2) (low) and 2(n%2)+1 (high).
enum : uint32_t { kTagInject = 1u, kTagPush = 2u, kTagLibrary = 3u, kTagGenerator = 4u };

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        const uint32_t lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

__device__ __forceinline__ uint2 seed_key(uint64_t seed) {
    return make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
}

// u in [0,1) with 53 random bits from a (low, high) word pair.
__device__ __forceinline__ double u01_f64(uint32_t lo, uint32_t hi) {
    const uint64_t bits = ((static_cast<uint64_t>(hi) << 32) | lo) >> 11;
    return __dmul_rn(static_cast<double>(bits), 1.0 / 9007199254740992.0);
}

// u in [0,1) with 24 random bits from the high word of the same pair, so the
// FP32 stream tracks the FP64 stream to 2^-24.
__device__ __forceinline__ float u01_f32(uint32_t hi) {
    return static_cast<float>(hi >> 8) * (1.0f / 16777216.0f);
}

// ---------------------------------------------------------------- wrap
// wrap_periodic_coordinate (reference src/main.cpp:642-665).
__device__ __forceinline__ double wrap_driver(double value, double lower, double upper,
                                              double width) {
    double wrapped = value;
    if (wrapped >= upper) {
        wrapped = __dsub_rn(wrapped, width);
        if (wrapped >= upper) {
            wrapped = __dsub_rn(wrapped,
                                __dmul_rn(floor(__ddiv_rn(__dsub_rn(wrapped, lower), width)),
                                          width));
        }
    } else if (wrapped < lower) {
        wrapped = __dadd_rn(wrapped, width);
        if (wrapped < lower) {
            wrapped = __dsub_rn(wrapped,
                                __dmul_rn(floor(__ddiv_rn(__dsub_rn(wrapped, lower), width)),
                                          width));
        }
    }
    if (wrapped >= upper) {
        wrapped = __dsub_rn(wrapped, width);
    }
    if (wrapped < lower) {
        wrapped = __dadd_rn(wrapped, width);
    }
    return wrapped;
}

// Grid periodic wrap (MappedCoordinateGrid.hpp:284-306,
// StoredCoordinateGrid.hpp:357-377).
__device__ __forceinline__ double grid_wrap(const Axis& a, double x) {
    double wrapped =
        __dsub_rn(x, __dmul_rn(floor(__dmul_rn(__dsub_rn(x, a.lower), a.inv_width)), a.width));
    if (wrapped >= a.upper) {
        wrapped = __dsub_rn(wrapped, a.width);
    }
    if (wrapped < a.lower) {
        wrapped = __dadd_rn(wrapped, a.width);
    }
    return wrapped;
}

// Continuous cell-centred index over the ghosted domain
// (AnalyticCoordinateGrid.hpp:214-230; StoredCoordinateGrid.hpp:124-174).
__device__ __forceinline__ double cell_grid_index(const Axis& a, double x) {
    if (!a.stored) {
        return __dsub_rn(__ddiv_rn(__dsub_rn(x, a.start), a.step), 0.5);
    }
    const double* c = a.centers;  // logical -2 .. n+1 at c[0 .. n+3]
    const int upper_index = a.n + 1;
    int left;
    if (x <= __ldg(c)) {
        left = -2;
    } else if (x >= __ldg(c + upper_index + 2)) {
        left = upper_index - 1;
    } else {
        // Bucket guess then exact local scan: finds the same interval
        // [c[k], c[k+1]) as the reference's binary search.
        int k = -2;
        if (a.bucket_count > 0) {
            int b = static_cast<int>((x - a.bucket_origin) * a.bucket_scale);
            b = b < 0 ? 0 : (b >= a.bucket_count ? a.bucket_count - 1 : b);
            k = __ldg(a.buckets + b);
        }
        while (k > -2 && x < __ldg(c + k + 2)) {
            --k;
        }
        while (k < upper_index - 1 && x >= __ldg(c + k + 3)) {
            ++k;
        }
        left = k;
    }
    const double x_left = __ldg(c + left + 2);
    const double x_right = __ldg(c + left + 3);
    return __dadd_rn(static_cast<double>(left),
                     __ddiv_rn(__dsub_rn(x, x_left), __dsub_rn(x_right, x_left)));
}

// compute_axis_stencil (FieldInterpolator.hpp:509-559), cell-centred,
// ghosted domain [-2, n+1].
__device__ __forceinline__ void axis_stencil(const Axis& a, double coordinate, int& lo,
                                             int& hi, double& w) {
    const int lower_bound = -2;
    const int upper_bound = a.n + 1;
    const double logical = cell_grid_index(a, coordinate);
    if (logical <= static_cast<double>(lower_bound)) {
        lo = lower_bound;
        hi = lower_bound;
        w = 0.0;
        return;
    }
    if (logical >= static_cast<double>(upper_bound)) {
        lo = upper_bound;
        hi = upper_bound;
        w = 0.0;
        return;
    }
    const int candidate = static_cast<int>(floor(logical));
    lo = candidate;
    hi = candidate + 1;
    w = __dsub_rn(logical, static_cast<double>(candidate));
    if (hi > upper_bound) {
        lo = upper_bound;
        hi = upper_bound;
        w = 0.0;
    }
}

}  // namespace kpt
