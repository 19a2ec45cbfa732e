// The learned closure shared by the trainer (kpt_surrogate.cu) and the push
// (kpt_push.cu): a 5 -> H -> H -> 3 tanh MLP (hidden width H = 32 or 64)
// standing in for the slab-QLT pitch-angle scattering closure
// (LegencyModel.hpp:557-645) and the kappa_parallel closure of the driver
// (src/main.cpp:1177-1193).
//
// Features (each mapped affinely from the training box onto [-1, 1]):
//   f0 = ln|mu|, f1 = ln p, f2 = ln|B|, f3 = ln(dB^2/B^2), f4 = gamma_k.
// D_mumu is even and dD_mumu/dmu odd in mu, so the network sees |mu| and the
// sign is applied analytically; logarithms turn the power laws of the
// closure into smooth, bounded functions.
// Targets (normalised by out_offset/out_scale):
//   y0 = ln D_mumu - ln(1 - mu^2)
//   y1 = sgn(mu) (|mu| + h0) (dD_mumu/dmu / D_mumu + 2 mu / (1 - mu^2))
//      = (gamma_k - 1) - gamma_k (|mu|+h0)^gamma_k / ((|mu|+h0)^gamma_k + xi^gamma_k)
//   y2 = ln kappa_parallel
// so D_mumu = (1 - mu^2) e^y0, dD_mumu/dmu = D_mumu (sgn(mu) y1 / (|mu|+h0)
// - 2 mu / (1 - mu^2)), kappa_parallel = e^y2.  For |mu| < mu_cut and outside
// the box the plain closure is evaluated instead.
//
// Inference is warp-collective: the 32 particles of a warp are the M = 32
// rows of three mma.sync.m16n8k16 GEMMs (BF16, or FP16 on request) with FP32
// accumulation.  The accumulator fragment of one layer is, after the
// activation and packing to 16-bit pairs, exactly the A fragment of the
// next, so activations never leave registers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace kpt {

constexpr int kMlpIn = 5;
constexpr int kMlpOut = 3;
constexpr int kMlpHiddenDefault = 32;

// Parameter block, FP32: W1[H][5] b1[H] W2[H][H] b2[H] W3[3][H] b3[3].
// Shared-memory block of the served network: 16-bit B fragments (one uint2
// per lane per 16x8 tile) in the order layer 1 [nt H/8], layer 2
// [kt H/16][nt H/8], layer 3 [kt H/16]; then FP32 biases b1[H], b2[H],
// b3[8] (zero padded).
template <int H>
struct Mlp {
    static_assert(H == 32 || H == 64, "hidden width 32 or 64");
    static constexpr int W1 = 0;
    static constexpr int B1 = W1 + H * kMlpIn;
    static constexpr int W2 = B1 + H;
    static constexpr int B2 = W2 + H * H;
    static constexpr int W3 = B2 + H;
    static constexpr int B3 = W3 + kMlpOut * H;
    static constexpr int Params = B3 + kMlpOut;
    static constexpr int NT = H / 8;   // 8-column tiles of a hidden layer
    static constexpr int KT = H / 16;  // 16-deep k tiles of a hidden layer
    static constexpr int FragW1 = 0;
    static constexpr int FragW2 = FragW1 + NT * 32;
    static constexpr int FragW3 = FragW2 + KT * NT * 32;
    static constexpr int FragCount = FragW3 + KT * 32;  // uint2 entries
    static constexpr int BiasCount = 2 * H + 8;
    static constexpr size_t SmemBytes = FragCount * sizeof(uint2) + BiasCount * sizeof(float);
};

__host__ __device__ constexpr int mlp_params(int hidden) {
    return hidden == 64 ? Mlp<64>::Params : Mlp<32>::Params;
}
__host__ __device__ constexpr size_t mlp_smem_bytes(int hidden) {
    return hidden == 64 ? Mlp<64>::SmemBytes : Mlp<32>::SmemBytes;
}
constexpr size_t kSurrogateSmemMax = Mlp<64>::SmemBytes;

// Training box and normalisation of one trained network.
struct SurrogateBox {
    float in_lo[kMlpIn];   // feature units (see above)
    float in_hi[kMlpIn];
    float in_scale[kMlpIn];   // 2 / (hi - lo)
    float in_offset[kMlpIn];  // -(hi + lo) / (hi - lo)
    float out_offset[kMlpOut];
    float out_scale[kMlpOut];
    float mu_cut;
    int fp16;    // element type of weights and activations: 0 BF16, 1 FP16
    int hidden;  // hidden width H (32 or 64)
    int magnetic_dependency, momentum_dependency;
    // physics constants the targets were generated with
    double p0, particle_v0, kpara0, gamma_turb, qlt_omega0, qlt_lc, qlt_h0;
};

// What a push needs: the fragment/bias block (Mlp<H>::SmemBytes, copied to
// shared memory by each block), the box, the run's constant features f3, f4
// (normalised) and the judge counters
// {evaluations, judged, fallbacks, max relative error (float bits)}.
struct SurrogateDevice {
    const uint2* block;
    SurrogateBox box;
    float f3, f4;
    int constants_in_box;
    int judge_period;  // judge one substep in judge_period per particle (power of 2)
    unsigned long long* judge;
};

#ifdef __CUDACC__

// Packed pair conversion, the activation and the m16n8k16 MMA for the two
// element types (FP16 = true: IEEE binary16, else BF16).
template <bool FP16>
__device__ __forceinline__ uint32_t pack_x2(float lo, float hi) {
    uint32_t r;
    // cvt packs its first source into the upper half
    if (FP16) {
        asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    } else {
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    }
    return r;
}

// tanh of two FP32 accumulators packed as the next layer's 16-bit pair.
// FP16: packed tanh.approx.f16x2 on the rounded pre-activations.  BF16:
// tanh.approx.f32 on each accumulator, then one rounding to BF16 -- faster on
// this GPU than the packed bf16x2 form and more accurate (one rounding after
// the activation instead of one before and one after).
template <bool FP16>
__device__ __forceinline__ uint32_t act_x2(float lo, float hi) {
    if (FP16) {
        uint32_t r;
        const uint32_t x = pack_x2<true>(lo, hi);
        asm("tanh.approx.f16x2 %0, %1;" : "=r"(r) : "r"(x));
        return r;
    }
    float tlo, thi;
    asm("tanh.approx.f32 %0, %1;" : "=f"(tlo) : "f"(lo));
    asm("tanh.approx.f32 %0, %1;" : "=f"(thi) : "f"(hi));
    return pack_x2<false>(tlo, thi);
}

template <bool FP16>
__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], uint2 b) {
    if (FP16) {
        asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
            "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
    } else {
        asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
            "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
    }
}

// Copy the fragment/bias block into shared memory (whole block, then sync).
template <int H>
__device__ __forceinline__ void load_surrogate_block(const uint2* src, uint2* smem) {
    constexpr int words = static_cast<int>(Mlp<H>::SmemBytes / sizeof(uint2));
    for (int k = threadIdx.x; k < words; k += blockDim.x) smem[k] = src[k];
    __syncthreads();
}

// Row tiles [0, MT) of the three layers: ax the input A fragments, out the
// output accumulators.  With MT = 2 both row tiles advance together: every
// weight fragment and bias read from shared memory feeds two MMAs, and the
// two tiles' dependency chains interleave, at the cost of twice the live
// activation registers.
template <bool FP16, int H, int MT>
__device__ __forceinline__ void mlp_rows(const uint2* smem, const uint32_t (*ax)[4],
                                         float (*out)[4]) {
    using M = Mlp<H>;
    const int lane = static_cast<int>(threadIdx.x & 31u);
    const int tig = lane & 3;
    const float* bias = reinterpret_cast<const float*>(smem + M::FragCount);
    // layer 1: NT column tiles -> A fragments of layer 2 (KT k tiles)
    uint32_t a2[MT][M::KT][4];
#pragma unroll
    for (int nt = 0; nt < M::NT; ++nt) {
        const float2 bv = *reinterpret_cast<const float2*>(bias + 8 * nt + 2 * tig);
        const uint2 w = smem[M::FragW1 + nt * 32 + lane];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
            float acc[4] = {bv.x, bv.y, bv.x, bv.y};
            mma_16816<FP16>(acc, ax[mt], w);
            a2[mt][nt >> 1][(nt & 1) * 2 + 0] = act_x2<FP16>(acc[0], acc[1]);
            a2[mt][nt >> 1][(nt & 1) * 2 + 1] = act_x2<FP16>(acc[2], acc[3]);
        }
    }
    // layer 2, with layer 3 accumulated as each pair of column tiles
    // completes a k tile of its A fragment
    const float2 b3 = *reinterpret_cast<const float2*>(bias + 2 * H + 2 * tig);
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
        out[mt][0] = b3.x;
        out[mt][1] = b3.y;
        out[mt][2] = b3.x;
        out[mt][3] = b3.y;
    }
#pragma unroll
    for (int kt3 = 0; kt3 < M::KT; ++kt3) {
        uint32_t a3[MT][4];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int nt = 2 * kt3 + half;
            const float2 bv = *reinterpret_cast<const float2*>(bias + H + 8 * nt + 2 * tig);
            float acc[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                acc[mt][0] = bv.x;
                acc[mt][1] = bv.y;
                acc[mt][2] = bv.x;
                acc[mt][3] = bv.y;
            }
#pragma unroll
            for (int kt = 0; kt < M::KT; ++kt) {
                const uint2 w = smem[M::FragW2 + (kt * M::NT + nt) * 32 + lane];
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) mma_16816<FP16>(acc[mt], a2[mt][kt], w);
            }
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                a3[mt][half * 2 + 0] = act_x2<FP16>(acc[mt][0], acc[mt][1]);
                a3[mt][half * 2 + 1] = act_x2<FP16>(acc[mt][2], acc[mt][3]);
            }
        }
        const uint2 w3 = smem[M::FragW3 + kt3 * 32 + lane];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) mma_16816<FP16>(out[mt], a3[mt], w3);
    }
}

// Warp-collective forward pass.  Every lane of the warp must call it with the
// warp converged; lane r supplies row r (its five normalised features; zeros
// for an idle lane) and receives the three normalised outputs of row r.
template <bool FP16, int H>
__device__ __forceinline__ void mlp_warp(const uint2* smem, const float (&f)[kMlpIn],
                                         float (&y)[kMlpOut]) {
    const unsigned full = 0xffffffffu;
    const int lane = static_cast<int>(threadIdx.x & 31u);
    const int g = lane >> 2;
    const int tig = lane & 3;
    const uint32_t pk0 = pack_x2<FP16>(f[0], f[1]);
    const uint32_t pk1 = pack_x2<FP16>(f[2], f[3]);
    const uint32_t pk2 = pack_x2<FP16>(f[4], 0.0f);
    // A fragments of the input tiles: columns 2tig, 2tig+1 of rows g and
    // g+8; columns 8..15 (and 5..7) are zero padding.
    uint32_t ax[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int src_lo = 16 * mt + g;
        const uint32_t l0 = __shfl_sync(full, pk0, src_lo);
        const uint32_t l1 = __shfl_sync(full, pk1, src_lo);
        const uint32_t l2 = __shfl_sync(full, pk2, src_lo);
        const uint32_t h0 = __shfl_sync(full, pk0, src_lo + 8);
        const uint32_t h1 = __shfl_sync(full, pk1, src_lo + 8);
        const uint32_t h2 = __shfl_sync(full, pk2, src_lo + 8);
        ax[mt][0] = tig == 0 ? l0 : (tig == 1 ? l1 : (tig == 2 ? l2 : 0u));
        ax[mt][1] = tig == 0 ? h0 : (tig == 1 ? h1 : (tig == 2 ? h2 : 0u));
        ax[mt][2] = 0u;
        ax[mt][3] = 0u;
    }
    // both row tiles together (one tile after the other spills at H = 64)
    float out[2][4];
    mlp_rows<FP16, H, 2>(smem, ax, out);
    // Row r = 16 mt + 8 h + g' sits in lane 4 g' (columns 0, 1; registers
    // 2h, 2h+1) and lane 4 g' + 1 (column 2; register 2h) of tile mt.
    const int src0 = 4 * (lane & 7);
    const int mt = lane >> 4;
    const int h = (lane >> 3) & 1;
    float c0[2][4], c2[2][2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
#pragma unroll
        for (int k = 0; k < 4; ++k) c0[t][k] = __shfl_sync(full, out[t][k], src0);
        c2[t][0] = __shfl_sync(full, out[t][0], src0 + 1);
        c2[t][1] = __shfl_sync(full, out[t][2], src0 + 1);
    }
    const bool second = mt != 0;
    const bool upper = h != 0;
    y[0] = second ? (upper ? c0[1][2] : c0[1][0]) : (upper ? c0[0][2] : c0[0][0]);
    y[1] = second ? (upper ? c0[1][3] : c0[1][1]) : (upper ? c0[0][3] : c0[0][1]);
    y[2] = second ? (upper ? c2[1][1] : c2[1][0]) : (upper ? c2[0][1] : c2[0][0]);
}

#endif  // __CUDACC__

}  // namespace kpt
