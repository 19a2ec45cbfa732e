// Particle lifecycle kernels: uniform injection, deterministic momentum
// split, weighted log-momentum histogram and the run summary reductions.
#include <cuda.h>  // CUcontext / CUresult types only; entry points come from the runtime
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kpt_device.cuh"
#include "kpt_internal.h"

namespace kpt {
namespace {

// ------------------------------------------------------------- inject
// inject_uniform_particles (reference src/main.cpp:996-1048): four draws per
// new particle in the order x, y, t, mu from the stream (seed, k, frame, 1).
__global__ void inject_kernel(const InjectLaunch L) {
    const uint2 key = seed_key(L.seed);
    for (uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; k < L.n;
         k += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t stream = static_cast<uint32_t>(k);
        const uint4 r0 = philox4x32_10(make_uint4(0u, stream, L.frame, kTagInject), key);
        const uint4 r1 = philox4x32_10(make_uint4(1u, stream, L.frame, kTagInject), key);
        const uint64_t n = L.first + k;
        const ParticleArrays& a = L.parts;
        a.x[n] = __dadd_rn(L.x_lower,
                           __dmul_rn(__dsub_rn(L.x_upper, L.x_lower), u01_f64(r0.x, r0.y)));
        a.y[n] = __dadd_rn(L.y_lower,
                           __dmul_rn(__dsub_rn(L.y_upper, L.y_lower), u01_f64(r0.z, r0.w)));
        a.p[n] = L.p0;
        a.t[n] = __dadd_rn(L.interval_start,
                           __dadd_rn(0.0, __dmul_rn(__dsub_rn(L.mhd_dt, 0.0),
                                                    u01_f64(r1.x, r1.y))));
        a.step_dt[n] = L.dt_min;
        a.weight[n] = 1.0;
        a.mu[n] = __dmul_rn(L.mu_max, __dsub_rn(__dmul_rn(2.0, u01_f64(r1.z, r1.w)), 1.0));
        a.status[n] = 0;
        a.split_level[n] = 0;
    }
}

// -------------------------------------------------------------- split
// split_particles (src/main.cpp:1761-1839) with children appended in parent
// order: per-block eligible counts, one exclusive scan over the blocks, then
// a ballot/popc rank inside each block.  Thresholds and child weights per
// split level come from the host (glibc pow), so eligibility is decided on
// the same doubles as the reference.
constexpr int kSplitBlock = 1024;

__device__ __forceinline__ bool split_eligible(const SplitLaunch& L, uint64_t i) {
    if (i >= L.count || L.parts.status[i] != 0) {
        return false;
    }
    const int level = L.parts.split_level[i];
    if (level < 0 || level >= L.level_count) {
        return false;
    }
    const double p = L.parts.p[i];
    return p > __ldg(L.thresholds + level) && p <= L.pmax;
}

__global__ void __launch_bounds__(kSplitBlock) split_count_kernel(const SplitLaunch L) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(kSplitBlock) + threadIdx.x;
    const int n = __syncthreads_count(split_eligible(L, i) ? 1 : 0);
    if (threadIdx.x == 0) {
        L.block_counts[blockIdx.x] = static_cast<unsigned int>(n);
    }
}

// Exclusive scan of the block counts by one block (fixed order).
__global__ void __launch_bounds__(1024) split_scan_kernel(const SplitLaunch L, int nblocks) {
    __shared__ unsigned long long warp_sums[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) {
        carry = 0;
    }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = threadIdx.x >> 5;
    for (int base = 0; base < nblocks; base += 1024) {
        const int idx = base + static_cast<int>(threadIdx.x);
        const unsigned long long v = idx < nblocks ? L.block_counts[idx] : 0ull;
        unsigned long long inclusive = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, inclusive, off);
            if (lane >= static_cast<unsigned>(off)) inclusive += y;
        }
        if (lane == 31u) warp_sums[warp] = inclusive;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = warp_sums[lane];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= static_cast<unsigned>(off)) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        const unsigned long long warp_prefix = warp == 0 ? 0ull : warp_sums[warp - 1];
        if (idx < nblocks) {
            L.block_offsets[idx] = carry + warp_prefix + inclusive - v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry += warp_sums[31];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        L.totals[0] = carry;
    }
}

__global__ void __launch_bounds__(kSplitBlock) split_scatter_kernel(const SplitLaunch L) {
    __shared__ unsigned int warp_counts[kSplitBlock / 32];
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(kSplitBlock) + threadIdx.x;
    const bool eligible = split_eligible(L, i);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = threadIdx.x >> 5;
    const unsigned ballot = __ballot_sync(0xffffffffu, eligible);
    if (lane == 0) {
        warp_counts[warp] = __popc(ballot);
    }
    __syncthreads();
    if (!eligible) {
        return;
    }
    unsigned int rank = __popc(ballot & ((1u << lane) - 1u));
    for (unsigned w = 0; w < warp; ++w) {
        rank += warp_counts[w];
    }
    const uint64_t child = L.count + L.block_offsets[blockIdx.x] + rank;
    if (child >= L.capacity) {
        return;  // counted as skipped by the host: wanted - written
    }
    const ParticleArrays& a = L.parts;
    const int new_level = a.split_level[i] + 1;
    const double new_weight = __ldg(L.weights + new_level - 1);
    a.x[child] = a.x[i];
    a.y[child] = a.y[i];
    a.p[child] = a.p[i];
    a.t[child] = a.t[i];
    a.step_dt[child] = a.step_dt[i];
    a.weight[i] = new_weight;
    a.weight[child] = new_weight;
    a.mu[child] = a.mu[i];
    a.status[child] = 0;
    a.split_level[i] = new_level;
    a.split_level[child] = new_level;
}

// ---------------------------------------------------------- histogram
// write_momentum_histogram binning (src/main.cpp:1915-1940).  Block-private
// shared bins, FP64 atomics (driver weights are dyadic, so any summation
// order gives the serial sum).  A particle whose bin coordinate lies within
// 1e-7 of a bin edge is set aside for the host, which re-bins it with the
// host log so bins match the reference's host computation exactly.
//
// Two things keep the kernel at memory speed: the bin coordinate is first
// formed in FP32 (a few 1e-6 from the FP64 one), and only particles whose
// FP32 coordinate lies within 1e-3 of an edge pay for the FP64 log; and the
// lanes of a warp that fall in the same bin add their weights together
// before one shared-memory atomic (the momentum spectra of a push sit in a
// handful of bins, so most of a warp's lanes share one).
__global__ void histogram_kernel(const HistogramLaunch L) {
    extern __shared__ double shared_bins[];
    for (int b = threadIdx.x; b < L.nbins; b += blockDim.x) {
        shared_bins[b] = 0.0;
    }
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warp_first = blockIdx.x * static_cast<uint64_t>(blockDim.x) +
                                (threadIdx.x & ~31u);
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const float log_pmin_f = static_cast<float>(L.log_pmin);
    const float inv_dlogp_f = static_cast<float>(L.inv_dlogp);
    // the loop bound is uniform over the warp, so every lane takes part in
    // the warp-wide bin match
    for (uint64_t base = warp_first; base < L.count; base += stride) {
        const uint64_t i = base + lane;
        int bin = -1;
        double w = 0.0;
        if (i < L.count && L.status[i] == 0) {
            const double p = L.p[i];
            if (p >= L.pmin && p <= L.pmax) {
                const float ff = (__logf(static_cast<float>(p)) - log_pmin_f) * inv_dlogp_f;
                bool edge = false;
                if (fabsf(ff - rintf(ff)) < 1.0e-3f) {
                    const double f = (log(p) - L.log_pmin) * L.inv_dlogp;
                    edge = fabs(f - rint(f)) < 1.0e-7;
                    bin = static_cast<int>(f);
                } else {
                    bin = static_cast<int>(ff);
                }
                if (edge) {
                    const unsigned long long slot = atomicAdd(L.edge_count, 1ull);
                    L.edge_index[slot] = static_cast<unsigned int>(i);
                    bin = -1;
                } else {
                    bin = bin < 0 ? 0 : (bin >= L.nbins ? L.nbins - 1 : bin);
                    w = L.weight[i];
                }
            }
        }
        const unsigned peers = __match_any_sync(full, bin);
        if (bin >= 0) {
            double sum = 0.0;
            for (unsigned m = peers; m != 0u; m &= m - 1u) {
                sum += __shfl_sync(peers, w, __ffs(m) - 1);
            }
            if (lane == static_cast<unsigned>(__ffs(peers) - 1)) {
                atomicAdd(shared_bins + bin, sum);
            }
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < L.nbins; b += blockDim.x) {
        const double v = shared_bins[b];
        if (v != 0.0) {
            atomicAdd(L.bins + b, v);
        }
    }
}

// ------------------------------------------------------------ summary
// summarize_particles (src/main.cpp:1845-1901).  Counts, min/max and the
// dyadic weight sum are exact in any order; the p and dt sums use a fixed
// two-level tree (per-block partials, then one block), so they are
// deterministic and differ from the reference's serial sums only by
// rounding.
constexpr int kSummaryThreads = 256;
constexpr int kSummaryPerThread = 8;

__device__ __forceinline__ SummaryPartial empty_partial() {
    SummaryPartial s;
    s.active = 0;
    s.inactive = 0;
    s.weight_sum = 0.0;
    s.p_sum = 0.0;
    s.dt_sum = 0.0;
    s.p_min = __longlong_as_double(0x7ff0000000000000ll);
    s.dt_min = s.p_min;
    s.p_max = 0.0;
    s.dt_max = 0.0;
    s.max_level = 0;
    s.pad = 0;
    return s;
}

__device__ __forceinline__ void combine(SummaryPartial& a, const SummaryPartial& b) {
    a.active += b.active;
    a.inactive += b.inactive;
    a.weight_sum += b.weight_sum;
    a.p_sum += b.p_sum;
    a.dt_sum += b.dt_sum;
    a.p_min = b.p_min < a.p_min ? b.p_min : a.p_min;
    a.dt_min = b.dt_min < a.dt_min ? b.dt_min : a.dt_min;
    a.p_max = a.p_max < b.p_max ? b.p_max : a.p_max;
    a.dt_max = a.dt_max < b.dt_max ? b.dt_max : a.dt_max;
    a.max_level = a.max_level < b.max_level ? b.max_level : a.max_level;
}

__device__ void block_reduce(SummaryPartial& mine, SummaryPartial* out) {
    __shared__ SummaryPartial shared[kSummaryThreads];
    shared[threadIdx.x] = mine;
    __syncthreads();
    for (int stride = kSummaryThreads / 2; stride > 0; stride >>= 1) {
        if (static_cast<int>(threadIdx.x) < stride) {
            combine(shared[threadIdx.x], shared[threadIdx.x + stride]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *out = shared[0];
    }
}

__global__ void __launch_bounds__(kSummaryThreads) summary_partial_kernel(const SummaryLaunch L) {
    SummaryPartial mine = empty_partial();
    const uint64_t base =
        (blockIdx.x * static_cast<uint64_t>(kSummaryThreads) + threadIdx.x) * kSummaryPerThread;
    for (int k = 0; k < kSummaryPerThread; ++k) {
        const uint64_t i = base + k;
        if (i >= L.count) {
            break;
        }
        if (L.status[i] == 0) {
            const double p = L.p[i];
            const double dt = L.dt[i];
            mine.active += 1;
            mine.weight_sum += L.weight[i];
            mine.p_sum += p;
            mine.dt_sum += dt;
            mine.p_min = p < mine.p_min ? p : mine.p_min;
            mine.p_max = mine.p_max < p ? p : mine.p_max;
            mine.dt_min = dt < mine.dt_min ? dt : mine.dt_min;
            mine.dt_max = mine.dt_max < dt ? dt : mine.dt_max;
            const int level = L.level[i];
            mine.max_level = mine.max_level < level ? level : mine.max_level;
        } else {
            mine.inactive += 1;
        }
    }
    block_reduce(mine, L.partials + blockIdx.x);
}

__global__ void __launch_bounds__(kSummaryThreads) summary_final_kernel(const SummaryLaunch L,
                                                                        int nblocks) {
    SummaryPartial mine = empty_partial();
    for (int b = threadIdx.x; b < nblocks; b += kSummaryThreads) {
        combine(mine, L.partials[b]);
    }
    block_reduce(mine, L.result);
}

// --------------------------------------------------------------- sort
// Tile key of each particle from its position (cell index by the grid map,
// mean-spacing estimate refined by the stored centres); inactive particles
// take the extra key so they sort last.
__device__ __forceinline__ int cell_of(const Axis& a, double x) {
    const double f = (x - a.lower) * a.inv_width;
    int k = static_cast<int>(floor(f * a.n));
    k = k < 0 ? 0 : (k >= a.n ? a.n - 1 : k);
    return k;
}

__global__ void sort_key_kernel(const SortLaunch L) {
    const unsigned tiles = static_cast<unsigned>(L.tiles_x) * static_cast<unsigned>(L.tiles_y);
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < L.count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        unsigned key = tiles;
        if (L.parts.status[i] == 0) {
            const int cx = cell_of(L.grid.axis[0], L.parts.x[i]);
            const int cy = cell_of(L.grid.axis[1], L.parts.y[i]);
            key = static_cast<unsigned>(cy / L.tile_y) * static_cast<unsigned>(L.tiles_x) +
                  static_cast<unsigned>(cx / L.tile_x);
        }
        L.keys[i] = key;
        atomicAdd(L.counts + key, 1u);
    }
}

// Exclusive scan of the tile counts in place (one block, fixed order).
__global__ void __launch_bounds__(1024) sort_scan_kernel(unsigned int* counts, int n) {
    __shared__ unsigned int warp_sums[32];
    __shared__ unsigned int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = threadIdx.x >> 5;
    for (int base = 0; base < n; base += 1024) {
        const int idx = base + static_cast<int>(threadIdx.x);
        const unsigned v = idx < n ? counts[idx] : 0u;
        unsigned inclusive = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, inclusive, off);
            if (lane >= static_cast<unsigned>(off)) inclusive += y;
        }
        if (lane == 31u) warp_sums[warp] = inclusive;
        __syncthreads();
        if (warp == 0) {
            unsigned w = warp_sums[lane];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= static_cast<unsigned>(off)) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        const unsigned prefix = warp == 0 ? 0u : warp_sums[warp - 1];
        if (idx < n) counts[idx] = carry + prefix + inclusive - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sums[31];
        __syncthreads();
    }
}

__global__ void sort_scatter_kernel(const SortLaunch L) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < L.count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const unsigned slot = atomicAdd(L.counts + L.keys[i], 1u);
        L.order[slot] = static_cast<unsigned int>(i);
    }
}

}  // namespace

cudaError_t launch_sort(const SortLaunch& L, cudaStream_t stream) {
    const int tiles = L.tiles_x * L.tiles_y + 1;
    cudaError_t err = cudaMemsetAsync(L.counts, 0, sizeof(unsigned int) * tiles, stream);
    if (err != cudaSuccess || L.count == 0) return err;
    const int threads = 256;
    const uint64_t want = (L.count + threads - 1) / threads;
    const int blocks = static_cast<int>(want > 152u * 16u ? 152u * 16u : want);
    sort_key_kernel<<<blocks, threads, 0, stream>>>(L);
    sort_scan_kernel<<<1, 1024, 0, stream>>>(L.counts, tiles);
    sort_scatter_kernel<<<blocks, threads, 0, stream>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_inject(const InjectLaunch& L, cudaStream_t stream) {
    if (L.n == 0) {
        return cudaSuccess;
    }
    const int threads = 256;
    const uint64_t want = (L.n + threads - 1) / threads;
    const int blocks = static_cast<int>(want > 152u * 32u ? 152u * 32u : want);
    inject_kernel<<<blocks, threads, 0, stream>>>(L);
    return cudaGetLastError();
}

size_t split_scratch_blocks(uint64_t count) {
    return static_cast<size_t>((count + kSplitBlock - 1) / kSplitBlock);
}

cudaError_t launch_split(const SplitLaunch& L, cudaStream_t stream) {
    const int nblocks = static_cast<int>(split_scratch_blocks(L.count));
    if (nblocks == 0) {
        return cudaMemsetAsync(L.totals, 0, sizeof(unsigned long long), stream);
    }
    split_count_kernel<<<nblocks, kSplitBlock, 0, stream>>>(L);
    split_scan_kernel<<<1, 1024, 0, stream>>>(L, nblocks);
    split_scatter_kernel<<<nblocks, kSplitBlock, 0, stream>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_histogram(const HistogramLaunch& L, cudaStream_t stream) {
    cudaError_t err = cudaMemsetAsync(L.bins, 0, sizeof(double) * L.nbins, stream);
    if (err != cudaSuccess) return err;
    err = cudaMemsetAsync(L.edge_count, 0, sizeof(unsigned long long), stream);
    if (err != cudaSuccess) return err;
    if (L.count == 0) {
        return cudaSuccess;
    }
    const int threads = 256;
    const uint64_t want = (L.count + threads - 1) / threads;
    const int blocks = static_cast<int>(want > 152u * 8u ? 152u * 8u : want);
    histogram_kernel<<<blocks, threads, sizeof(double) * L.nbins, stream>>>(L);
    return cudaGetLastError();
}

int summary_blocks(uint64_t count) {
    const uint64_t per_block = static_cast<uint64_t>(kSummaryThreads) * kSummaryPerThread;
    const uint64_t n = (count + per_block - 1) / per_block;
    return static_cast<int>(n < 1 ? 1 : n);
}

cudaError_t launch_summary(const SummaryLaunch& L, cudaStream_t stream) {
    const int nblocks = summary_blocks(L.count);
    summary_partial_kernel<<<nblocks, kSummaryThreads, 0, stream>>>(L);
    summary_final_kernel<<<1, kSummaryThreads, 0, stream>>>(L, nblocks);
    return cudaGetLastError();
}

}  // namespace kpt

// ------------------------------------------------- allocation-free summary
// For callers that must not allocate device memory (code running inside a
// host application's memory pool or arena, under a CUDA graph being built
// elsewhere, or in a host thread that is forbidden to call cudaMalloc), the
// summary reduction has a variant whose per-block partials live in this
// fixed device array instead of a context buffer.  Every GPU that loads the
// library holds the array (about 0.7 MB) until the process exits.
namespace {

constexpr int kNoAllocMaxBlocks = 8192;  // 8192 blocks x 2048 particles
constexpr unsigned long long kNoAllocMaxParticles =
    static_cast<unsigned long long>(kNoAllocMaxBlocks) * kpt::kSummaryThreads * kpt::kSummaryPerThread;

// [0, kNoAllocMaxBlocks): per-block partials; [kNoAllocMaxBlocks]: result.
static __device__ __align__(256) kpt::SummaryPartial g_noalloc_summary[kNoAllocMaxBlocks + 1];

// Device address of g_noalloc_summary per CUDA context.  The address is
// looked up (cudaGetSymbolAddress) the first time a context calls, and kept
// under the context's unique id (cuCtxGetId), so a second context on the
// same device, or a primary context recreated after cudaDeviceReset, gets its
// own lookup instead of another context's (possibly stale) address.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

struct NoAllocSlot {
    unsigned long long context_id;
    kpt::SummaryPartial* address;
};
constexpr int kNoAllocMaxContexts = 64;
std::mutex g_noalloc_mutex;
NoAllocSlot g_noalloc_slots[kNoAllocMaxContexts] = {};
int g_noalloc_used = 0;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Id of the calling thread's current context (0 when none is current).
// Caller holds g_noalloc_mutex.
cudaError_t current_context_id(unsigned long long* id) {
    *id = 0;
    if (g_ctx_get_current == nullptr || g_ctx_get_id == nullptr) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSuccess;
        cudaDriverEntryPointQueryResult q2 = cudaDriverEntryPointSuccess;
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaError_t err = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                           cudaEnableDefault, &q1);
        if (err != cudaSuccess) return err;
        err = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (err != cudaSuccess) return err;
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess ||
            f1 == nullptr || f2 == nullptr) {
            return cudaErrorNotSupported;
        }
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    if (ctx == nullptr) return cudaSuccess;
    if (g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    return cudaSuccess;
}

// Device address of g_noalloc_summary in the current context.
cudaError_t noalloc_address(kpt::SummaryPartial** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    cudaError_t err = current_context_id(&id);
    if (err != cudaSuccess) return err;
    for (int k = 0; k < g_noalloc_used && id != 0; ++k) {
        if (g_noalloc_slots[k].context_id == id) {
            *out = g_noalloc_slots[k].address;
            return cudaSuccess;
        }
    }
    // First call in this context (or no context current yet: the lookup
    // makes the device's primary context current, as any runtime call does).
    void* ptr = nullptr;
    err = cudaGetSymbolAddress(&ptr, g_noalloc_summary);
    if (err != cudaSuccess) return err;
    if (id == 0) {
        err = current_context_id(&id);
        if (err != cudaSuccess) return err;
    }
    if (id != 0 && g_noalloc_used < kNoAllocMaxContexts) {
        g_noalloc_slots[g_noalloc_used++] = NoAllocSlot{id, static_cast<kpt::SummaryPartial*>(ptr)};
    }
    *out = static_cast<kpt::SummaryPartial*>(ptr);
    return cudaSuccess;
}

}  // namespace

namespace kpt {

unsigned long long noalloc_summary_max_particles() { return kNoAllocMaxParticles; }

cudaError_t noalloc_summary(const SummaryLaunch& in, cudaStream_t stream, SummaryPartial* host) {
    SummaryPartial* scratch = nullptr;
    cudaError_t err = noalloc_address(&scratch);
    if (err != cudaSuccess) return err;
    SummaryLaunch L = in;
    L.partials = scratch;
    L.result = scratch + kNoAllocMaxBlocks;
    // Every partial that the final pass reads is written by this call, so no
    // clearing is needed between calls.
    err = launch_summary(L, stream);
    if (err != cudaSuccess) return err;
    err = cudaMemcpyAsync(host, L.result, sizeof(SummaryPartial), cudaMemcpyDeviceToHost, stream);
    if (err != cudaSuccess) return err;
    return cudaStreamSynchronize(stream);
}

// v4 snapshot records of the driver (src/main.cpp:2155-2201), 100 bytes
// each as 25 little-endian 32-bit words: id u64, status, split level,
// sort key 0, position / previous position / previous-step position (the
// driver writes the position three times), momentum, mu, weight, the initial
// kinetic energy.  8-byte fields sit on 4-byte boundaries, so they are
// written as word pairs.
namespace {
__device__ __forceinline__ void put64(uint32_t* w, double v) {
    const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(v));
    w[0] = static_cast<uint32_t>(bits);
    w[1] = static_cast<uint32_t>(bits >> 32);
}

__global__ void pack_records_kernel(ParticleArrays a, uint64_t count, double e0,
                                    uint32_t* out) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t* r = out + i * 25;
        r[0] = static_cast<uint32_t>(i);
        r[1] = static_cast<uint32_t>(i >> 32);
        r[2] = static_cast<uint32_t>(a.status[i]);
        r[3] = static_cast<uint32_t>(a.split_level[i]);
        r[4] = 0u;
        const double x = a.x[i];
        const double y = a.y[i];
        for (int k = 0; k < 3; ++k) {
            put64(r + 5 + 4 * k, x);
            put64(r + 7 + 4 * k, y);
        }
        put64(r + 17, a.p[i]);
        put64(r + 19, a.mu[i]);
        put64(r + 21, a.weight[i]);
        put64(r + 23, e0);
    }
}
}  // namespace

cudaError_t launch_pack_records(const ParticleArrays& a, uint64_t count, double e0,
                                uint32_t* out, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    const uint64_t want = (count + 255) / 256;
    const int blocks = static_cast<int>(want > 152u * 32u ? 152u * 32u : want);
    pack_records_kernel<<<blocks, 256, 0, stream>>>(a, count, e0, out);
    return cudaGetLastError();
}

}  // namespace kpt
