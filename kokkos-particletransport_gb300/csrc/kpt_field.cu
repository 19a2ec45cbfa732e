// Per-frame coefficient tables on the device: one thread per ghosted point
// reads the cell-centred B and V (periodic ghosts are read through wrapped
// indices instead of being stored), and writes the 16 (Parker) or 21
// (focused) components of reference src/main.cpp:840-957 in the requested
// precision.  FP64 arithmetic uses explicitly rounded operations, so the FP64
// table is bit-identical to the reference's host build.
#include <cuda_runtime.h>

#include "kpt_internal.h"

namespace kpt {
namespace {

struct CellReader {
    const double* f;
    int nx, ny;
    size_t cells;
    __device__ __forceinline__ double operator()(int comp, int i, int j) const {
        int wi = i % nx;
        if (wi < 0) wi += nx;
        int wj = j % ny;
        if (wj < 0) wj += ny;
        return __ldg(f + static_cast<size_t>(comp) * cells + static_cast<size_t>(wj) * nx + wi);
    }
};

// Cell-centre coordinate (AnalyticCoordinateGrid.hpp:179-183 or stored
// centres, StoredCoordinateGrid.hpp:104-109).
__device__ __forceinline__ double cell_coordinate(const Axis& a, int index) {
    if (a.stored) {
        return __ldg(a.centers + index + 2);
    }
    const double ci = static_cast<double>(index);
    const double f0 = __dadd_rn(a.start, __dmul_rn(ci, a.step));
    const double f1 = __dadd_rn(a.start, __dmul_rn(__dadd_rn(ci, 1.0), a.step));
    return __dmul_rn(0.5, __dadd_rn(f0, f1));
}

__device__ __forceinline__ double bmag(const CellReader& b, int i, int j) {
    const double bx = b(0, i, j);
    const double by = b(1, i, j);
    const double bz = b(2, i, j);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(bx, bx), __dmul_rn(by, by)),
                                __dmul_rn(bz, bz)));
}

// derivative_component / derivative_magnetic_magnitude (src/main.cpp:716-834);
// comp < 0 differentiates |B|.
__device__ double derivative(const Grid& g, const CellReader& f, int i, int j, int dim,
                             int comp) {
    const Axis& a = g.axis[dim];
    if (a.n <= 1) {
        return 0.0;
    }
    const int lower = -2;
    const int upper = a.n + 1;
    const int idx = dim == 0 ? i : j;
    auto at = [&](int k) {
        const int ii = dim == 0 ? k : i;
        const int jj = dim == 0 ? j : k;
        return comp < 0 ? bmag(f, ii, jj) : f(comp, ii, jj);
    };
    if (idx <= lower) {
        const double x0 = cell_coordinate(a, lower);
        const double x2 = cell_coordinate(a, lower + 2);
        const double num = __dsub_rn(__dadd_rn(__dmul_rn(-3.0, at(lower)),
                                               __dmul_rn(4.0, at(lower + 1))),
                                     at(lower + 2));
        return __ddiv_rn(num, __dsub_rn(x2, x0));
    }
    if (idx >= upper) {
        const double x0 = cell_coordinate(a, upper - 2);
        const double x2 = cell_coordinate(a, upper);
        const double num = __dadd_rn(__dsub_rn(__dmul_rn(3.0, at(upper)),
                                               __dmul_rn(4.0, at(upper - 1))),
                                     at(upper - 2));
        return __ddiv_rn(num, __dsub_rn(x2, x0));
    }
    const double xl = cell_coordinate(a, idx - 1);
    const double xr = cell_coordinate(a, idx + 1);
    return __ddiv_rn(__dsub_rn(at(idx + 1), at(idx - 1)), __dsub_rn(xr, xl));
}

template <typename T, bool FOCUSED>
__global__ void build_table_kernel(const TableLaunch L) {
    constexpr int STRIDE = FOCUSED ? (sizeof(T) == 8 ? 22 : 24) : 16;
    const Grid& g = L.grid;
    const int nx = g.axis[0].n;
    const int ny = g.axis[1].n;
    const size_t points = static_cast<size_t>(nx + 4) * static_cast<size_t>(ny + 4);
    const CellReader b{L.b_cells, nx, ny, static_cast<size_t>(nx) * ny};
    const CellReader v{L.v_cells, nx, ny, static_cast<size_t>(nx) * ny};
    T* table = static_cast<T*>(L.table);
    for (size_t pnt = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; pnt < points;
         pnt += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(pnt % static_cast<size_t>(nx + 4)) - 2;
        const int j = static_cast<int>(pnt / static_cast<size_t>(nx + 4)) - 2;
        double out[24];
        const double bx = b(0, i, j);
        const double by = b(1, i, j);
        const double bz = b(2, i, j);
        const double bm = bmag(b, i, j);
        if (!FOCUSED) {
            out[0] = v(0, i, j);
            out[1] = v(1, i, j);
            out[2] = bx;
            out[3] = by;
            out[4] = bz;
            out[5] = bm;
            out[6] = derivative(g, v, i, j, 0, 0);
            out[7] = derivative(g, v, i, j, 1, 1);
            out[8] = derivative(g, b, i, j, 0, 0);
            out[9] = derivative(g, b, i, j, 1, 0);
            out[10] = derivative(g, b, i, j, 0, 1);
            out[11] = derivative(g, b, i, j, 1, 1);
            out[12] = derivative(g, b, i, j, 0, 2);
            out[13] = derivative(g, b, i, j, 1, 2);
            out[14] = derivative(g, b, i, j, 0, -1);
            out[15] = derivative(g, b, i, j, 1, -1);
        } else {
            out[0] = v(0, i, j);
            out[1] = v(1, i, j);
            out[2] = v(2, i, j);
            out[3] = bx;
            out[4] = by;
            out[5] = bz;
            out[6] = bm;
            out[7] = derivative(g, v, i, j, 0, 0);
            out[8] = derivative(g, v, i, j, 1, 0);
            out[9] = derivative(g, v, i, j, 0, 1);
            out[10] = derivative(g, v, i, j, 1, 1);
            out[11] = derivative(g, v, i, j, 0, 2);
            out[12] = derivative(g, v, i, j, 1, 2);
            out[13] = derivative(g, b, i, j, 0, 0);
            out[14] = derivative(g, b, i, j, 1, 0);
            out[15] = derivative(g, b, i, j, 0, 1);
            out[16] = derivative(g, b, i, j, 1, 1);
            out[17] = derivative(g, b, i, j, 0, 2);
            out[18] = derivative(g, b, i, j, 1, 2);
            out[19] = derivative(g, b, i, j, 0, -1);
            out[20] = derivative(g, b, i, j, 1, -1);
            for (int k = 21; k < STRIDE; ++k) {
                out[k] = 0.0;
            }
        }
        if constexpr (sizeof(T) == 8) {
            T* row = table + pnt * STRIDE;
#pragma unroll
            for (int k = 0; k < STRIDE; ++k) {
                row[k] = static_cast<T>(out[k]);
            }
        } else {
            // FP32 layout (table_f32_offset): 8 floats per 256-bit store
#pragma unroll
            for (int chunk = 0; chunk < STRIDE / 8; ++chunk) {
                float4 lo, hi;
                lo.x = static_cast<float>(out[8 * chunk + 0]);
                lo.y = static_cast<float>(out[8 * chunk + 1]);
                lo.z = static_cast<float>(out[8 * chunk + 2]);
                lo.w = static_cast<float>(out[8 * chunk + 3]);
                hi.x = static_cast<float>(out[8 * chunk + 4]);
                hi.y = static_cast<float>(out[8 * chunk + 5]);
                hi.z = static_cast<float>(out[8 * chunk + 6]);
                hi.w = static_cast<float>(out[8 * chunk + 7]);
                float4* dst = reinterpret_cast<float4*>(
                    table + table_f32_offset(FOCUSED, points, pnt, 8 * chunk));
                dst[0] = lo;
                dst[1] = hi;
            }
        }
    }
}

// One thread per (cell, sector): sector s of line m holds frame m % 2 of
// component pair 4 (m / 2) + s at the cell's four corners (zeros past the
// last component).  Cells on the last ghosted column or row have no
// upper-right corner and no record; no particle's stencil starts there.
template <bool FOCUSED>
__global__ void build_records_kernel(const RecordLaunch L) {
    constexpr int C = FOCUSED ? 21 : 16;
    constexpr int S = record_sectors(FOCUSED);
    const uint64_t total = L.points * S;
    const size_t ex = static_cast<size_t>(L.ex);
    for (uint64_t q = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; q < total;
         q += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const size_t p = static_cast<size_t>(q / S);
        const int sector = static_cast<int>(q % S);
        const size_t i = p % ex, j = p / ex;
        if (i + 1 >= ex || j + 2 > static_cast<size_t>(L.ey)) continue;
        const int line = sector / 4;
        const float* table = (line & 1) ? L.upper : L.lower;
        const int first = 2 * (4 * (line / 2) + sector % 4);
        const size_t corner[4] = {p, p + 1, p + ex, p + ex + 1};
        float v[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[2 * k] = first < C ? __ldg(table + table_f32_offset(FOCUSED, L.points, corner[k],
                                                                  first))
                                 : 0.0f;
            v[2 * k + 1] = first + 1 < C ? __ldg(table + table_f32_offset(FOCUSED, L.points,
                                                                          corner[k], first + 1))
                                         : 0.0f;
        }
        float4* out =
            reinterpret_cast<float4*>(L.records + p * record_floats(FOCUSED) + 8 * sector);
        out[0] = make_float4(v[0], v[1], v[2], v[3]);
        out[1] = make_float4(v[4], v[5], v[6], v[7]);
    }
}

}  // namespace

cudaError_t launch_build_records(const RecordLaunch& L, cudaStream_t stream) {
    const uint64_t total = L.points * static_cast<uint64_t>(record_sectors(L.focused != 0));
    const int threads = 256;
    const uint64_t want = (total + threads - 1) / threads;
    const int blocks = static_cast<int>(want < 1 ? 1 : (want > 152u * 64u ? 152u * 64u : want));
    if (L.focused) {
        build_records_kernel<true><<<blocks, threads, 0, stream>>>(L);
    } else {
        build_records_kernel<false><<<blocks, threads, 0, stream>>>(L);
    }
    return cudaGetLastError();
}

cudaError_t launch_build_table(const TableLaunch& L, cudaStream_t stream) {
    const size_t points = static_cast<size_t>(L.grid.axis[0].n + 4) *
                          static_cast<size_t>(L.grid.axis[1].n + 4);
    const int threads = 256;
    size_t want = (points + threads - 1) / threads;
    const int blocks = static_cast<int>(want < 1 ? 1 : (want > 152u * 64u ? 152u * 64u : want));
    if (L.precision == kPrecisionF64) {
        if (L.focused) {
            build_table_kernel<double, true><<<blocks, threads, 0, stream>>>(L);
        } else {
            build_table_kernel<double, false><<<blocks, threads, 0, stream>>>(L);
        }
    } else {
        if (L.focused) {
            build_table_kernel<float, true><<<blocks, threads, 0, stream>>>(L);
        } else {
            build_table_kernel<float, false><<<blocks, threads, 0, stream>>>(L);
        }
    }
    return cudaGetLastError();
}

}  // namespace kpt
