// Training and evaluation of the learned QLT closure (the project's own
// forward and backward kernels, FP32 SIMT; the network is tiny).
//
// Samples are drawn uniformly over the training box (feature units) with the
// keyed Philox stream; targets come from the plain slab-QLT closure in FP64
// (LegencyModel.hpp:557-645) and the driver's kappa_parallel closure
// (src/main.cpp:1177-1193).  One optimisation step: forward + backward per
// sample (activations and deltas kept in HBM), batch reductions for the
// weight gradients, then Adam.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "kpt_device.cuh"
#include "kpt_internal.h"
#include "kpt_surrogate.cuh"

namespace kpt {
namespace {

constexpr double kPiD = 3.141592653589793238462643383279502884;

// Plain slab-QLT closure (LegencyModel.hpp:557-645) with per-sample sigma^2
// and gamma_k, FP64: D_mumu, dD_mumu/dmu and the two network targets
// y0 = ln D - ln(1 - mu^2), y1 = (gk - 1) - gk reg^gk / (reg^gk + xi^gk).
__device__ void qlt_targets(double mu, double omega, double speed, double sigma2, double lc,
                            double gk, double h0, double& d, double& dd, double& y0,
                            double& y1) {
    d = 0.0;
    dd = 0.0;
    y0 = 0.0;
    y1 = 0.0;
    const double one_minus_mu2 = 1.0 - mu * mu;
    if (one_minus_mu2 <= 0.0) return;
    const double reg = fabs(mu) + h0;
    const double xi = omega * lc / speed;
    const double reg_gk = pow(reg, gk);
    const double reg_gk1 = pow(reg, gk - 1.0);
    const double denominator = reg_gk + pow(xi, gk);
    const double norm = gk * sin(kPiD / gk) / kPiD;
    const double prefactor = 0.25 * kPiD * omega * sigma2 * norm;
    d = prefactor * one_minus_mu2 * xi * reg_gk1 / denominator;
    y0 = log(prefactor * xi) + (gk - 1.0) * log(reg) - log(denominator);
    y1 = (gk - 1.0) - gk * reg_gk / denominator;
    if (d == 0.0 || mu == 0.0) return;
    const double sign = mu > 0.0 ? 1.0 : -1.0;
    dd = d * (-2.0 * mu / one_minus_mu2 + sign * ((gk - 1.0) / reg - gk * reg_gk1 / denominator));
}

// The driver's kappa_parallel closure (src/main.cpp:1177-1193).
__device__ double kappa_parallel(const SurrogateBox& box, double p, double b) {
    double k = box.kpara0;
    if (box.magnetic_dependency == 1) k *= pow(b, box.gamma_turb - 2.0);
    if (box.momentum_dependency == 1) k *= pow(p / box.p0, 3.0 - box.gamma_turb);
    return k;
}

__device__ __forceinline__ double u32_open(uint32_t r) {
    return (static_cast<double>(r) + 0.5) * 2.3283064365386963e-10;
}

// Training samples, uniform over the box in feature units (ln|mu|, ln p,
// ln|B|, ln sigma^2, gamma_k); x holds the raw features, t the targets.
__global__ void make_samples_kernel(uint64_t seed, int n, SurrogateBox box, float* x, float* t) {
    const uint2 key = seed_key(seed);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 r0 = philox4x32_10(make_uint4(0u, static_cast<uint32_t>(i), 0u, 7u), key);
        const uint4 r1 = philox4x32_10(make_uint4(1u, static_cast<uint32_t>(i), 0u, 7u), key);
        const uint32_t words[5] = {r0.x, r0.y, r0.z, r0.w, r1.x};
        double f[kMlpIn];
        for (int k = 0; k < kMlpIn; ++k) {
            f[k] = box.in_lo[k] + (static_cast<double>(box.in_hi[k]) - box.in_lo[k]) *
                                      u32_open(words[k]);
        }
        const double mu = exp(f[0]);
        const double p = exp(f[1]);
        const double b = exp(f[2]);
        const double sigma2 = exp(f[3]);
        const double gk = f[4];
        const double speed = box.particle_v0 * p / box.p0;
        const double omega = box.qlt_omega0 * b / sqrt(1.0 + p * p);
        double d, dd, y0, y1;
        qlt_targets(mu, omega, speed, sigma2, box.qlt_lc, gk, box.qlt_h0, d, dd, y0, y1);
        float* xi = x + static_cast<size_t>(i) * kMlpIn;
        for (int k = 0; k < kMlpIn; ++k) xi[k] = static_cast<float>(f[k]);
        float* ti = t + static_cast<size_t>(i) * kMlpOut;
        ti[0] = static_cast<float>(y0);
        ti[1] = static_cast<float>(y1);
        ti[2] = static_cast<float>(log(kappa_parallel(box, p, b)));
    }
}

// Rounding of the served network's 16-bit element type (quantization-aware
// fine-tuning): 0 none, 1 BF16 (round to nearest even), 2 FP16.
__device__ __forceinline__ float quantize(float v, int q) {
    if (q == 1) {
        uint32_t bits = __float_as_uint(v);
        bits = (bits + 0x7fffu + ((bits >> 16) & 1u)) & 0xffff0000u;
        return __uint_as_float(bits);
    }
    if (q == 2) {
        return __half2float(__float2half_rn(v));
    }
    return v;
}

__device__ __forceinline__ float normalise_input(const SurrogateBox& box, int k, float v) {
    return v * box.in_scale[k] + box.in_offset[k];
}

// Forward and backward of one minibatch, one thread per sample.  Stores
// H1, H2 (activations) and G1, G2, GY (deltas) for the gradient reductions.
template <int H>
__global__ void __launch_bounds__(128) fwd_bwd_kernel(const float* __restrict__ x,
                                                      const float* __restrict__ t, int n,
                                                      uint64_t seed, int step, int batch,
                                                      SurrogateBox box,
                                                      const float* __restrict__ params,
                                                      float* xb, float* h1, float* h2, float* g1,
                                                      float* g2, float* gy, float* loss,
                                                      int quant) {
    // quant != 0: the forward sees the served network's rounding (weights,
    // inputs and activations in the 16-bit type, FP16 pre-activations too;
    // biases and accumulation FP32) and the backward passes straight
    // through it
    using M = Mlp<H>;
    __shared__ float w[M::Params];
    for (int k = threadIdx.x; k < M::Params; k += blockDim.x) {
        const bool bias = (k >= M::B1 && k < M::W2) || (k >= M::B2 && k < M::W3) || k >= M::B3;
        w[k] = bias ? params[k] : quantize(params[k], quant);
    }
    __syncthreads();
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    float sq = 0.0f;
    if (b < batch) {
        int i = b % n;
        if (step >= 0) {
            const uint4 r = philox4x32_10(make_uint4(static_cast<uint32_t>(b),
                                                     static_cast<uint32_t>(step), 0u, 9u),
                                          seed_key(seed));
            i = static_cast<int>(u01_f64(r.x, r.y) * n) % n;
        }
        float in[kMlpIn];
        for (int k = 0; k < kMlpIn; ++k) {
            in[k] = quantize(normalise_input(box, k, x[static_cast<size_t>(i) * kMlpIn + k]),
                             quant);
            xb[static_cast<size_t>(b) * kMlpIn + k] = in[k];
        }
        float a1[H];
        for (int j = 0; j < H; ++j) {
            float z = w[M::B1 + j];
            for (int k = 0; k < kMlpIn; ++k) z += w[M::W1 + j * kMlpIn + k] * in[k];
            a1[j] = quantize(tanhf(quant == 2 ? quantize(z, quant) : z), quant);
            h1[static_cast<size_t>(b) * H + j] = a1[j];
        }
        float y[kMlpOut];
        for (int o = 0; o < kMlpOut; ++o) y[o] = w[M::B3 + o];
        for (int j = 0; j < H; ++j) {
            float z = w[M::B2 + j];
            for (int k = 0; k < H; ++k) z += w[M::W2 + j * H + k] * a1[k];
            const float a2 = quantize(tanhf(quant == 2 ? quantize(z, quant) : z), quant);
            h2[static_cast<size_t>(b) * H + j] = a2;
            for (int o = 0; o < kMlpOut; ++o) y[o] += w[M::W3 + o * H + j] * a2;
        }
        float dy[kMlpOut];
        for (int o = 0; o < kMlpOut; ++o) {
            const float target = (t[static_cast<size_t>(i) * kMlpOut + o] - box.out_offset[o]) /
                                 box.out_scale[o];
            const float e = y[o] - target;
            sq += e * e;
            dy[o] = 2.0f * e / static_cast<float>(batch * kMlpOut);
            gy[static_cast<size_t>(b) * kMlpOut + o] = dy[o];
        }
        float d1[H];
        for (int k = 0; k < H; ++k) d1[k] = 0.0f;
        for (int j = 0; j < H; ++j) {
            const float a2 = h2[static_cast<size_t>(b) * H + j];
            float dh = 0.0f;
            for (int o = 0; o < kMlpOut; ++o) dh += w[M::W3 + o * H + j] * dy[o];
            const float dz = dh * (1.0f - a2 * a2);
            g2[static_cast<size_t>(b) * H + j] = dz;
            for (int k = 0; k < H; ++k) d1[k] += w[M::W2 + j * H + k] * dz;
        }
        for (int k = 0; k < H; ++k) {
            g1[static_cast<size_t>(b) * H + k] = d1[k] * (1.0f - a1[k] * a1[k]);
        }
    }
    // batch loss (mean squared error in normalised units)
    for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
    if ((threadIdx.x & 31u) == 0u && sq != 0.0f) {
        atomicAdd(loss, sq / static_cast<float>(batch * kMlpOut));
    }
}

// Weight and bias gradients, deterministic two-level reduction: block
// (row, chunk) sums its chunk of kGradChunk samples for one parameter row,
// threads over the row's columns; grad_sum_kernel then adds the chunk
// partials in chunk order.  Row r of:
//   W1 (H rows x 5):  sum_b G1[b][r] X[b][c];   b1[r] = sum_b G1[b][r]
//   W2 (H rows x H):  sum_b G2[b][r] H1[b][c];  b2[r] = sum_b G2[b][r]
//   W3 (3 rows x H):  sum_b GY[b][r] H2[b][c];  b3[r] = sum_b GY[b][r]
template <int H>
__global__ void __launch_bounds__(64) grad_partial_kernel(int batch, const float* xb,
                                                          const float* h1, const float* h2,
                                                          const float* g1, const float* g2,
                                                          const float* gy, float* partial) {
    using M = Mlp<H>;
    const int row = blockIdx.x;
    const int chunk = blockIdx.y;
    const int c = threadIdx.x;
    const float* delta;
    const float* input;
    int dstride, istride, cols, wbase, bbase, r;
    if (row < H) {
        r = row; delta = g1; dstride = H; input = xb; istride = kMlpIn; cols = kMlpIn;
        wbase = M::W1; bbase = M::B1;
    } else if (row < 2 * H) {
        r = row - H; delta = g2; dstride = H; input = h1; istride = H;
        cols = H; wbase = M::W2; bbase = M::B2;
    } else {
        r = row - 2 * H; delta = gy; dstride = kMlpOut; input = h2;
        istride = H; cols = H; wbase = M::W3; bbase = M::B3;
    }
    const int b0 = chunk * kGradChunk;
    const int b1 = b0 + kGradChunk < batch ? b0 + kGradChunk : batch;
    float acc = 0.0f, bacc = 0.0f;
    for (int b = b0; b < b1; ++b) {
        const float d = delta[static_cast<size_t>(b) * dstride + r];
        if (c < cols) acc += d * input[static_cast<size_t>(b) * istride + c];
        bacc += d;
    }
    float* out = partial + static_cast<size_t>(chunk) * M::Params;
    if (c < cols) out[wbase + r * cols + c] = acc;
    if (c == 0) out[bbase + r] = bacc;
}

__global__ void grad_sum_kernel(const float* partial, int chunks, int params, float* grad) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= params) return;
    float sum = 0.0f;
    for (int ch = 0; ch < chunks; ++ch) sum += partial[static_cast<size_t>(ch) * params + k];
    grad[k] = sum;
}

template <int H>
cudaError_t launch_gradients(const SurrogateTrainLaunch& L, cudaStream_t stream) {
    using M = Mlp<H>;
    const int chunks = (L.batch + kGradChunk - 1) / kGradChunk;
    grad_partial_kernel<H><<<dim3(2 * H + kMlpOut, chunks), 64, 0, stream>>>(
        L.batch, L.xb, L.h1, L.h2, L.g1, L.g2, L.gy, L.partial);
    grad_sum_kernel<<<(M::Params + 255) / 256, 256, 0, stream>>>(L.partial, chunks, M::Params,
                                                                 L.grad);
    return cudaGetLastError();
}

__global__ void adam_kernel(float* params, const float* grad, float* m, float* v, int count,
                            float lr, float beta1, float beta2, float eps, float bias1,
                            float bias2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const float g = grad[k];
    const float mk = beta1 * m[k] + (1.0f - beta1) * g;
    const float vk = beta2 * v[k] + (1.0f - beta2) * g * g;
    m[k] = mk;
    v[k] = vk;
    params[k] -= lr * (mk / bias1) / (sqrtf(vk / bias2) + eps);
}

// FP32 SIMT forward of normalised features -> normalised outputs.
template <int H>
__device__ void forward_fp32(const float* w, const float (&in)[kMlpIn], float (&y)[kMlpOut]) {
    using M = Mlp<H>;
    float a1[H];
    for (int j = 0; j < H; ++j) {
        float z = w[M::B1 + j];
        for (int k = 0; k < kMlpIn; ++k) z += w[M::W1 + j * kMlpIn + k] * in[k];
        a1[j] = tanhf(z);
    }
    for (int o = 0; o < kMlpOut; ++o) y[o] = w[M::B3 + o];
    for (int j = 0; j < H; ++j) {
        float z = w[M::B2 + j];
        for (int k = 0; k < H; ++k) z += w[M::W2 + j * H + k] * a1[k];
        const float a2 = tanhf(z);
        for (int o = 0; o < kMlpOut; ++o) y[o] += w[M::W3 + o * H + j] * a2;
    }
}

// Raw inputs (mu, ln p, ln|B|, sigma^2, gamma_k) -> (D_mumu, dD_mumu/dmu,
// ln kappa_parallel), FP64 out.  The network (FP32 SIMT, or a tensor-core
// engine of the push) serves inputs inside the box with |mu| >= mu_cut; the
// plain closure serves the rest.
//
// Features of input i (zeros for an idle thread and outside the box);
// returns whether the network serves it.
__device__ __forceinline__ bool eval_features(int i, bool have, const double* __restrict__ in,
                                              const SurrogateBox& box, double (&raw)[kMlpIn],
                                              float (&f)[kMlpIn]) {
    for (int k = 0; k < kMlpIn; ++k) raw[k] = 0.0;
    if (have) {
        for (int k = 0; k < kMlpIn; ++k) raw[k] = in[static_cast<size_t>(i) * kMlpIn + k];
    }
    const double mu = raw[0];
    const double feat[kMlpIn] = {log(fabs(mu)), raw[1], raw[2], log(raw[3]), raw[4]};
    bool inside = have && fabs(mu) >= box.mu_cut;
    for (int k = 0; k < kMlpIn; ++k) {
        inside = inside && feat[k] >= box.in_lo[k] && feat[k] <= box.in_hi[k];
        f[k] = static_cast<float>(feat[k]) * box.in_scale[k] + box.in_offset[k];
    }
    if (!inside) {
        for (int k = 0; k < kMlpIn; ++k) f[k] = 0.0f;
    }
    return inside;
}

// Closure values of input i from the network outputs y (or the plain
// closure outside the box), with the push's hand-over near mu_cut.
__device__ __forceinline__ void eval_store(int i, const double (&raw)[kMlpIn], bool inside,
                                           const float (&y)[kMlpOut], const SurrogateBox& box,
                                           double* __restrict__ out, int* __restrict__ served) {
    const double mu = raw[0];
    const double p = exp(raw[1]);
    const double b = exp(raw[2]);
    double d, dd, lk;
    const double speed = box.particle_v0 * p / box.p0;
    const double omega = box.qlt_omega0 * b / sqrt(1.0 + p * p);
    double pd, pdd, py0, py1;
    qlt_targets(mu, omega, speed, raw[3], box.qlt_lc, raw[4], box.qlt_h0, pd, pdd, py0, py1);
    const double plk = log(kappa_parallel(box, p, b));
    if (inside) {
        const double y0 = static_cast<double>(y[0]) * box.out_scale[0] + box.out_offset[0];
        const double y1 = static_cast<double>(y[1]) * box.out_scale[1] + box.out_offset[1];
        lk = static_cast<double>(y[2]) * box.out_scale[2] + box.out_offset[2];
        const double one_minus_mu2 = 1.0 - mu * mu;
        const double sign = mu > 0.0 ? 1.0 : -1.0;
        d = one_minus_mu2 * exp(y0);
        dd = d * (sign * y1 / (fabs(mu) + box.qlt_h0) - 2.0 * mu / one_minus_mu2);
        const double amu = fabs(mu);
        if (amu < 2.0 * box.mu_cut) {
            // the push's hand-over to the plain closure over [mu_cut, 2 mu_cut]
            const double w = (amu - box.mu_cut) / box.mu_cut;
            const double dw = sign / box.mu_cut;
            dd = pdd + w * (dd - pdd) + dw * (d - pd);
            d = pd + w * (d - pd);
            lk = log(exp(plk) + w * (exp(lk) - exp(plk)));
        }
    } else {
        d = pd;
        dd = pdd;
        lk = plk;
    }
    out[static_cast<size_t>(i) * kMlpOut + 0] = d;
    out[static_cast<size_t>(i) * kMlpOut + 1] = dd;
    out[static_cast<size_t>(i) * kMlpOut + 2] = lk;
    served[i] = inside ? 1 : 0;
}

// FP32 SIMT (MODE 0) or the warp-collective mma.sync engine (MODE 1 BF16,
// 2 FP16).  Warps stay converged (the loop bound is per warp) because the
// tensor-core path is collective.
template <int MODE, int H>
__global__ void __launch_bounds__(128) eval_kernel(int n, const double* __restrict__ in,
                                                   SurrogateBox box,
                                                   const float* __restrict__ params,
                                                   const uint2* __restrict__ block,
                                                   double* __restrict__ out,
                                                   int* __restrict__ served) {
    extern __shared__ uint2 smem[];
    if (MODE != 0) {
        load_surrogate_block<H>(block, smem);
    } else {
        float* w = reinterpret_cast<float*>(smem);
        for (int k = threadIdx.x; k < Mlp<H>::Params; k += blockDim.x) w[k] = params[k];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int base = warp * 32; base < n; base += warps * 32) {
        const int i = base + lane;
        const bool have = i < n;
        double raw[kMlpIn];
        float f[kMlpIn];
        const bool inside = eval_features(i, have, in, box, raw, f);
        float y[kMlpOut];
        if (MODE != 0) {
            mlp_warp<MODE == 2, H>(smem, f, y);
        } else {
            forward_fp32<H>(reinterpret_cast<const float*>(smem), f, y);
        }
        if (have) eval_store(i, raw, inside, y, box, out, served);
    }
}

// The tcgen05 engine: each block takes 128 inputs per trip (its rows), the
// trip count uniform over the block.
template <bool FP16, int H>
__global__ void __launch_bounds__(128) eval_tc_kernel(int n, const double* __restrict__ in,
                                                      SurrogateBox box,
                                                      const uint4* __restrict__ block,
                                                      double* __restrict__ out,
                                                      int* __restrict__ served,
                                                      unsigned int* __restrict__ timeouts) {
    extern __shared__ __align__(128) unsigned char tc_smem[];
    TcNet net = tc_setup<H>(block, tc_smem);
    tc_constants<FP16, H>(net);
    bool fail = false;
    for (int base = blockIdx.x * 128; base < n; base += gridDim.x * 128) {
        const int i = base + static_cast<int>(threadIdx.x);
        const bool have = i < n;
        double raw[kMlpIn];
        float f[kMlpIn];
        const bool inside = eval_features(i, have, in, box, raw, f);
        float y[kMlpOut];
        if (mlp_cta<FP16, H>(net, f, y, fail)) {
            break;
        }
        if (have) eval_store(i, raw, inside, y, box, out, served);
    }
    fail = __syncthreads_or(fail ? 1 : 0) != 0;
    if (fail && threadIdx.x == 0) {
        atomicAdd(timeouts, 1u);
    }
    tc_teardown<H>(net, fail);
}

// The failure path of the tcgen05 engine without a fault: every block sets
// up its network (weights, barrier, 128 TMEM columns), waits for a
// completion that nothing will signal (no MMA is issued) with `polls`
// polls, records the timeout, and tears down as a timed-out push block does
// (a second bounded wait, then the TMEM is freed).
__global__ void __launch_bounds__(128) tc_timeout_check_kernel(const uint4* __restrict__ block,
                                                               uint32_t polls,
                                                               unsigned int* __restrict__ out) {
    extern __shared__ __align__(128) unsigned char tc_smem[];
    TcNet net = tc_setup<64>(block, tc_smem);
    bool fail = !mbar_wait(net.mbar, net.phase, polls);
    net.phase ^= 1u;
    fail = __syncthreads_or(fail ? 1 : 0) != 0;
    if (fail && threadIdx.x == 0) {
        atomicAdd(out, 1u);
    }
    tc_teardown<64>(net, fail, polls);
    if (threadIdx.x == 0) {
        atomicAdd(out + 1, 1u);  // blocks that got past the teardown
    }
}

}  // namespace

cudaError_t surrogate_tc_timeout_check(const uint4* block, int blocks, uint32_t polls,
                                       unsigned int* out, cudaStream_t stream) {
    tc_timeout_check_kernel<<<blocks, 128, tc_smem_bytes<64>(), stream>>>(block, polls, out);
    return cudaGetLastError();
}

cudaError_t surrogate_make_samples(uint64_t seed, int n, const SurrogateBox& box, float* x,
                                   float* t, cudaStream_t stream) {
    const int threads = 256;
    const int blocks = (n + threads - 1) / threads < 152 * 16 ? (n + threads - 1) / threads
                                                              : 152 * 16;
    make_samples_kernel<<<blocks, threads, 0, stream>>>(seed, n, box, x, t);
    return cudaGetLastError();
}

namespace {

template <int H>
cudaError_t train_step(const SurrogateTrainLaunch& L, int step, cudaStream_t stream) {
    fwd_bwd_kernel<H><<<(L.batch + 127) / 128, 128, 0, stream>>>(
        L.x, L.t, L.n, L.seed, step, L.batch, L.box, L.params, L.xb, L.h1, L.h2, L.g1, L.g2, L.gy,
        L.loss + step, step >= L.quant_from ? L.quant : 0);
    launch_gradients<H>(L, stream);
    const float t1 = static_cast<float>(step + 1);
    const float bias1 = 1.0f - powf(L.beta1, t1);
    const float bias2 = 1.0f - powf(L.beta2, t1);
    adam_kernel<<<(Mlp<H>::Params + 255) / 256, 256, 0, stream>>>(
        L.params, L.grad, L.m, L.v, Mlp<H>::Params, L.lr, L.beta1, L.beta2, 1e-8f, bias1, bias2);
    return cudaGetLastError();
}

template <int H>
cudaError_t gradient(const SurrogateTrainLaunch& L, cudaStream_t stream) {
    fwd_bwd_kernel<H><<<(L.batch + 127) / 128, 128, 0, stream>>>(
        L.x, L.t, L.n, L.seed, -1, L.batch, L.box, L.params, L.xb, L.h1, L.h2, L.g1, L.g2, L.gy,
        L.loss, 0);
    return launch_gradients<H>(L, stream);
}

template <int H>
cudaError_t eval(int n, const double* inputs, const SurrogateBox& box, const SurrogateServe& sv,
                 double* out, int* served, cudaStream_t stream) {
    const int threads = 128;
    int blocks = (n + threads - 1) / threads;
    if (sv.engine == kEngineTcgen05) {
        // blocks beyond the 4 per SM whose TMEM fits wait in tcgen05.alloc
        // until a resident block frees its columns
        blocks = blocks < 1 ? 1 : (blocks > 152 * 4 ? 152 * 4 : blocks);
        const size_t smem = tc_smem_bytes<H>();
        if (box.fp16) {
            eval_tc_kernel<true, H><<<blocks, threads, smem, stream>>>(
                n, inputs, box, sv.tc_block, out, served, sv.timeouts);
        } else {
            eval_tc_kernel<false, H><<<blocks, threads, smem, stream>>>(
                n, inputs, box, sv.tc_block, out, served, sv.timeouts);
        }
        return cudaGetLastError();
    }
    blocks = blocks < 1 ? 1 : (blocks > 152 * 8 ? 152 * 8 : blocks);
    const size_t smem = Mlp<H>::SmemBytes;
    if (sv.engine == kEngineMmaSync && box.fp16) {
        eval_kernel<2, H><<<blocks, threads, smem, stream>>>(n, inputs, box, sv.params, sv.block,
                                                             out, served);
    } else if (sv.engine == kEngineMmaSync) {
        eval_kernel<1, H><<<blocks, threads, smem, stream>>>(n, inputs, box, sv.params, sv.block,
                                                             out, served);
    } else {
        eval_kernel<0, H><<<blocks, threads, Mlp<H>::Params * sizeof(float), stream>>>(
            n, inputs, box, sv.params, sv.block, out, served);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t surrogate_train_step(const SurrogateTrainLaunch& L, int step, cudaStream_t stream) {
    return L.box.hidden == 64 ? train_step<64>(L, step, stream) : train_step<32>(L, step, stream);
}

cudaError_t surrogate_gradient(const SurrogateTrainLaunch& L, cudaStream_t stream) {
    return L.box.hidden == 64 ? gradient<64>(L, stream) : gradient<32>(L, stream);
}

cudaError_t surrogate_eval(int n, const double* inputs, const SurrogateBox& box,
                           const SurrogateServe& serve, double* out, int* served,
                           cudaStream_t stream) {
    return box.hidden == 64 ? eval<64>(n, inputs, box, serve, out, served, stream)
                            : eval<32>(n, inputs, box, serve, out, served, stream);
}

}  // namespace kpt
