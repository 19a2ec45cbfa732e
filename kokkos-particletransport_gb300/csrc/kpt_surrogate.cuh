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
constexpr int kMlpHiddenDefault = 64;

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

// The same network served by the fifth-generation tensor cores (tcgen05),
// CTA-collective: the 128 threads of a block are the M = 128 rows.  Weights
// are the B operands in shared memory, K-major with no swizzle: 8-row x
// 16-byte core matrices, W[n][k] at byte (n/8) SBO + (k/8) 128 + (n%8) 16 +
// (k%8) 2 with SBO = K/8 x 128.  The biases ride in the GEMMs as two extra
// inputs fixed at 1 whose weights are the bias split into a 16-bit head and
// its 16-bit remainder (b = hi + lo to ~2^-16 relative): layer 1 is N = H x
// K = 16 (inputs 0..4, bias 5..6), layer 2 N = H x K = H + 16 (bias at
// H, H+1), layer 3 N = 16 x K = H + 16 (outputs 3..15 zero).  Activations
// live in tensor memory: the A operand of each layer (H/2 columns of 16-bit
// pairs, row = TMEM lane) followed by the constant block (one column of
// (1, 1), seven of zeros) and the hidden accumulators (H FP32 columns); the
// output accumulators (16 columns) reuse the first hidden columns, which the
// layer-2 epilogue has read before the layer-3 MMA is issued.  H = 32 then
// fits in 64 columns (eight blocks' worth per SM), H = 64 in 128.
template <int H>
struct TcMlp {
    static constexpr int K2 = H + 16;  // K of layers 2 and 3 (bias block included)
    static constexpr int W1 = 0;
    static constexpr int W2 = W1 + H * 16 * 2;
    static constexpr int W3 = W2 + H * K2 * 2;
    static constexpr int Bytes = W3 + 16 * K2 * 2;
    static constexpr uint32_t ColA = 0;
    static constexpr uint32_t ColOne = H / 2;  // constant block
    static constexpr uint32_t ColD = H / 2 + 8;
    static constexpr uint32_t ColOut = ColD;
    // TMEM allocation: a power of two >= 32 covering the hidden accumulators
    static constexpr uint32_t Cols = ColD + H <= 64 ? 64 : 128;
    static_assert(ColD + H <= Cols && ColOut + 16 <= Cols,
                  "tensor-memory layout exceeds the allocation");
};
__host__ __device__ constexpr size_t tc_block_bytes(int hidden) {
    return hidden == 64 ? TcMlp<64>::Bytes : TcMlp<32>::Bytes;
}
// Network engines of the push and of kpt_surrogate_evaluate.
constexpr int kEngineTcgen05 = 0;  // CTA-collective tcgen05.mma, TMEM activations
constexpr int kEngineMmaSync = 1;  // warp-collective mma.sync, register activations

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
    const uint4* tc_block;  // canonical-layout weights of the tcgen05 engine
    int engine;             // kEngineTcgen05 or kEngineMmaSync
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

// ------------------------------------------------------------ tcgen05
// Shared-memory address of a generic pointer into shared memory.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: start, leading (K-direction core-matrix)
// and stride (MN-direction 8-row group) byte offsets, descriptor version 1,
// no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) |
           (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, A and B both BF16
// (or both FP16), both K-major, M = 128, N.
__host__ __device__ constexpr uint32_t tc_idesc(bool fp16, int n) {
    return (1u << 4) | ((fp16 ? 0u : 1u) << 7) | ((fp16 ? 0u : 1u) << 10) |
           (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(128 >> 4) << 24);
}

// D[tmem] (+)= A[tmem] x B[smem]; accumulate = 0 overwrites D.
__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}"
        :
        : "r"(d), "r"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on the mbarrier once every MMA this thread issued has completed.
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :
                 : "r"(mbar)
                 : "memory");
}

// 4 (or 32) consecutive FP32 columns of this thread's row, waited for: the
// load and its wait sit in one asm statement, so no use of the registers
// can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
    uint32_t r[4];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// 16 consecutive 32-bit columns of this thread's row, waited for.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, "
        "%10, %11, %12, %13, %14, %15, %16};\n\t"
        "tcgen05.wait::st.sync.aligned;"
        :
        : "r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]),
          "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]),
          "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}

// 8 consecutive 32-bit columns of this thread's row, waited for.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n\t"
        "tcgen05.wait::st.sync.aligned;"
        :
        : "r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]),
          "r"(v[6]), "r"(v[7])
        : "memory");
}

// Completion waits give up after this many polls (each poll may suspend the
// thread for a while); the block then reports the timeout and stops.
#ifndef KPT_TC_WAIT_POLLS
#define KPT_TC_WAIT_POLLS (1u << 20)
#endif

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity,
                                          uint32_t polls = KPT_TC_WAIT_POLLS) {
    for (uint32_t i = 0; i < polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// One block's tensor-core network: TMEM base, shared-memory weights and the
// completion barrier with the parity of its next phase.
struct TcNet {
    uint32_t tmem;
    uint32_t w;
    uint32_t mbar;
    uint32_t phase;
};

// Shared-memory footprint of the tcgen05 engine: weights, then the
// mbarrier (8 B) and the TMEM address slot (4 B).
template <int H>
__host__ __device__ constexpr size_t tc_smem_bytes() {
    return static_cast<size_t>(TcMlp<H>::Bytes) + 16;
}

// Start of the push's record-sampler rows behind the engine's footprint.
template <int H>
__host__ __device__ constexpr size_t tc_xpose_offset() {
    return (tc_smem_bytes<H>() + 15) & ~static_cast<size_t>(15);
}

// Block prologue (all threads): weights to shared memory, barrier init,
// TMEM allocation by warp 0.
template <int H>
__device__ __forceinline__ TcNet tc_setup(const uint4* __restrict__ block, unsigned char* smem) {
    using T = TcMlp<H>;
    uint4* w = reinterpret_cast<uint4*>(smem);
    for (int k = threadIdx.x; k < T::Bytes / 16; k += blockDim.x) w[k] = block[k];
    const uint32_t mbar = smem_u32(smem + T::Bytes);
    const uint32_t slot = smem_u32(smem + T::Bytes + 8);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :
                     : "r"(slot), "r"(T::Cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // weights written by generic stores become visible to the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    TcNet net;
    net.tmem = *reinterpret_cast<volatile uint32_t*>(smem + T::Bytes + 8);
    net.w = smem_u32(smem);
    net.mbar = mbar;
    net.phase = 0;
    return net;
}

// Write this thread's row of the constant block (after tc_setup).
template <bool FP16, int H>
__device__ __forceinline__ void tc_constants(const TcNet& net) {
    const uint32_t row = (threadIdx.x & 0x60u) << 16;
    const uint32_t ones[8] = {pack_x2<FP16>(1.0f, 1.0f), 0u, 0u, 0u, 0u, 0u, 0u, 0u};
    tmem_st8(net.tmem + row + TcMlp<H>::ColOne, ones);
}

// Block epilogue (all threads, uniform): after a timeout, wait once more
// (bounded) for the MMAs in flight; then warp 0 frees the TMEM.  The TMEM is
// freed even when that second wait also gives up (keeping it would leave the
// blocks queued in tcgen05.alloc waiting forever); a late MMA may then write
// into columns another block of the same launch has allocated, so a false
// return means every result of the launch is invalid, not only this block's.
// Returns true when the block did not fail or its MMAs completed in time.
template <int H>
__device__ __forceinline__ bool tc_teardown(const TcNet& net, bool failed,
                                            uint32_t polls = KPT_TC_WAIT_POLLS) {
    __shared__ int drained;
    if (threadIdx.x == 0) {
        drained = failed ? (mbar_wait(net.mbar, net.phase ^ 1u, polls) ? 1 : 0) : 1;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :
                     : "r"(net.tmem), "r"(TcMlp<H>::Cols)
                     : "memory");
    }
    return drained != 0;
}

// Block-wide hand-over to the MMA issuer: TMEM stores ordered before the
// barrier, the failure flag made uniform.  Returns false (for every thread)
// once any thread has failed.
__device__ __forceinline__ bool tc_sync(bool& fail) {
    tc_fence_before();
    fail = __syncthreads_or(fail ? 1 : 0) != 0;
    tc_fence_after();
    return !fail;
}

// Wait for the MMAs of the current phase.
__device__ __forceinline__ void tc_complete(TcNet& net, bool& fail) {
    if (!mbar_wait(net.mbar, net.phase)) fail = true;
    net.phase ^= 1u;
    tc_fence_after();
}

// Hidden-layer epilogue of this thread's row: accumulators (bias included)
// -> activation -> 16-bit pairs, the next layer's A operand; 32 columns per
// TMEM round trip (0.7 % faster on the headline than 16).
template <bool FP16, int H>
__device__ __forceinline__ void tc_hidden(uint32_t td, uint32_t ta) {
#pragma unroll
    for (int c = 0; c < H / 32; ++c) {
        float acc[32];
        tmem_ld32(td + 32 * c, acc);
        uint32_t a[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) a[j] = act_x2<FP16>(acc[2 * j], acc[2 * j + 1]);
        tmem_st16(ta + 16 * c, a);
    }
}

// Block-collective forward pass: every thread of the block calls it (block
// converged); thread r supplies row r (its five normalised features; zeros
// for an idle thread) and receives the three normalised outputs of row r.
// Returns true when the block stops (a completion wait timed out: fail is
// then set in every thread); the outputs are then undefined.
template <bool FP16, int H>
__device__ __forceinline__ bool mlp_cta(TcNet& net, const float (&f)[kMlpIn],
                                        float (&y)[kMlpOut], bool& fail) {
    using T = TcMlp<H>;
    // warp w of the block owns TMEM lanes 32 w .. 32 w + 31
    const uint32_t row = (threadIdx.x & 0x60u) << 16;
    const uint32_t ta = net.tmem + row + T::ColA;
    const uint32_t td = net.tmem + row + T::ColD;
    const uint32_t a_op = net.tmem + T::ColA;
    const uint32_t d_op = net.tmem + T::ColD;
    const bool issuer = threadIdx.x == 0;
    {
        // inputs 0..4, then 1, 1 for the layer-1 bias head and remainder
        const uint32_t in[8] = {pack_x2<FP16>(f[0], f[1]), pack_x2<FP16>(f[2], f[3]),
                                pack_x2<FP16>(f[4], 1.0f), pack_x2<FP16>(1.0f, 0.0f),
                                0u, 0u, 0u, 0u};
        tmem_st8(ta, in);
    }
    // layer 1: K = 16
    if (!tc_sync(fail)) return true;
    if (issuer) {
        tc_mma(d_op, a_op, tc_desc(net.w + T::W1, 128, 256), tc_idesc(FP16, H), 0u);
        tc_commit(net.mbar);
    }
    tc_complete(net, fail);
    tc_hidden<FP16, H>(td, ta);
    // layer 2: K = H + 16 in steps of 16, the last step the bias block
    if (!tc_sync(fail)) return true;
    if (issuer) {
#pragma unroll
        for (int s = 0; s < T::K2 / 16; ++s) {
            tc_mma(d_op, a_op + 8 * s, tc_desc(net.w + T::W2 + 256 * s, 128, 16 * T::K2),
                   tc_idesc(FP16, H), s > 0 ? 1u : 0u);
        }
        tc_commit(net.mbar);
    }
    tc_complete(net, fail);
    tc_hidden<FP16, H>(td, ta);
    // layer 3: N = 16, K = H + 16
    if (!tc_sync(fail)) return true;
    if (issuer) {
#pragma unroll
        for (int s = 0; s < T::K2 / 16; ++s) {
            tc_mma(net.tmem + T::ColOut, a_op + 8 * s,
                   tc_desc(net.w + T::W3 + 256 * s, 128, 16 * T::K2), tc_idesc(FP16, 16),
                   s > 0 ? 1u : 0u);
        }
        tc_commit(net.mbar);
    }
    tc_complete(net, fail);
    float o[4];
    tmem_ld4(net.tmem + row + T::ColOut, o);
#pragma unroll
    for (int k = 0; k < kMlpOut; ++k) y[k] = o[k];
    return false;
}

#endif  // __CUDACC__

}  // namespace kpt
