// imc_surrogate.cu -- training data, training and test entry points of the
// learned thick-cell surrogate (model in imc_surrogate.cuh).
//
//   k_surr_datagen  the analog in-cell walk (the physics of Transport.MC inside
//                   one cell, src/imc_transport.jl:72-193, in mean free paths)
//                   from random walk states; its outcomes are the training
//                   targets and, in the tests, the yardstick of the sampled ones
//   k_surr_grad     forward + backward of a 64-sample slice in FP32: the loss
//                   (cross entropy of the outcome + pinball losses of the
//                   outcome's quantile heads) and per-block weight gradients
//   k_surr_reduce   sums the per-block gradients in block order (deterministic)
//   k_surr_adam     Adam step on FP32 master weights
//   k_surr_forward  the transport kernel's tensor-core forward pass on given
//                   inputs (for the tests)
//   k_surr_sample   inverse-transform sampling of the network's outputs, as
//                   the transport kernel samples them (for the tests)
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "imc.h"  // include/imc.h (on the -I path)
#include "imc_device.cuh"
#include "imc_internal.h"
#include "imc_surrogate.cuh"

using namespace imc;
using namespace imc::surr;

namespace {

constexpr uint32_t kStageSurrData = 3;   // Philox stage tag of training walks
constexpr uint32_t kStageSurrTest = 4;   // stage tag of test sampling
constexpr int kWalkCapFactor = 8;        // flight cap: 8 * lmax + 64

// ----------------------------------------------------------- in-cell walk
// Analog walk from (d_n, d_f, mu', lmax), all in mean free paths, near face at
// 0, far face at d_n + d_f.  Returns the outcome and the two targets: for an
// exit ln(path / lmax) and |mu|, for truncation the displacement toward the
// far face / sqrt(lmax) and the final mu'.
__device__ int walk(Stream &rs, float d_n, float d_f, float mu, float lmax, float *y0, float *y1) {
    const float W = d_n + d_f;
    float pos = d_n, path = 0.0f;
    const int cap = kWalkCapFactor * (int)lmax + 64;
    for (int it = 0; it < cap; ++it) {
        const float s = Rand<float>::exp1(rs);
        const float dface = mu > 0.0f ? (W - pos) / mu : pos / (-mu);
        const float rem = lmax - path;
        if (rem <= s && rem <= dface) {
            pos += mu * rem;
            *y0 = (pos - d_n) / sqrtf(lmax);
            *y1 = mu;
            return kTrunc;
        }
        if (dface <= s) {
            path += dface;
            *y0 = logf(fmaxf(path, 1e-30f) / lmax);
            *y1 = fabsf(mu);
            return mu > 0.0f ? kFar : kNear;
        }
        pos += mu * s;
        path += s;
        mu = 0.0f;
        for (int r = 0; r < 64 && mu == 0.0f; ++r) mu = 1.0f - 2.0f * Rand<float>::u(rs);
        if (mu == 0.0f) mu = 1.0f;
    }
    *y0 = (pos - d_n) / sqrtf(lmax);
    *y1 = mu;
    return kTrunc;
}

// Random walk states covering the states the transport kernel asks about
// (lmax >= 32, cells >= 8 mean free paths, expected collisions
// min(lmax, 1.5 d_n d_f) >= 64) with a margin: lmax log-uniform on
// [40, 1.2e4]; cell width W log-uniform on [12, 2.5 lmax] for half of the
// states and on [12, min(2.5 lmax, 20 sqrt(lmax))] for the other half, so that
// cells thin enough for walks to cross them (diffusion length sqrt(lmax)) are
// well represented; the start uniform in the nearer half of the cell, redrawn
// (at most 16 times, then the cell centre) until 1.5 d_n d_f >= 48; mu'
// uniform on [-1, 1].
__device__ void draw_state(Stream &rs, float *d_n, float *d_f, float *mu, float *lmax) {
    const float lo = 1.6020600f, hi = 4.0791812f;  // log10 40, log10 1.2e4
    const float L = exp10f(lo + (hi - lo) * Rand<float>::u(rs));
    const float top = Rand<float>::u(rs) < 0.5f ? fminf(2.5f * L, 20.0f * sqrtf(L)) : 2.5f * L;
    const float lw0 = 1.0791812f, lw1 = log10f(fmaxf(top, 12.0f));  // log10 12
    const float W = exp10f(lw0 + (lw1 - lw0) * Rand<float>::u(rs));
    float dn = 0.5f * W;
    for (int r = 0; r < 16; ++r) {
        const float v = 0.5f * W * Rand<float>::u(rs);
        if (1.5f * v * (W - v) >= 48.0f) { dn = v; break; }
    }
    float m = 0.0f;
    for (int r = 0; r < 64 && m == 0.0f; ++r) m = 1.0f - 2.0f * Rand<float>::u(rs);
    if (m == 0.0f) m = 1.0f;
    *d_n = dn; *d_f = W - dn; *mu = m; *lmax = L;
}

__global__ void k_surr_datagen(unsigned long long seed, long long n, const float *state_in, float *x, int *cls,
                               float *tgt) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        Stream rs;
        rs.init(seed, 0u, (uint32_t)i, kStageSurrData);
        float dn, df, mu, L;
        if (state_in) {
            dn = state_in[4 * i]; df = state_in[4 * i + 1]; mu = state_in[4 * i + 2]; L = state_in[4 * i + 3];
        } else {
            draw_state(rs, &dn, &df, &mu, &L);
        }
        float y0, y1;
        const int c = walk(rs, dn, df, mu, L, &y0, &y1);
        float f[kIn];
        features(dn, df, mu, L, f);
        for (int k = 0; k < kIn; ++k) x[kIn * i + k] = f[k];
        cls[i] = c;
        tgt[2 * i] = y0;
        tgt[2 * i + 1] = y1;
    }
}

// ------------------------------------------------------------- training
constexpr int kSlice = 64;        // samples per block
constexpr int kTrainThreads = 256;

// gradient of the loss w.r.t. the 64 raw outputs of one sample; returns the loss
__device__ float output_grad(const float *out, int c, float y0, float y1, float *dout) {
    for (int j = 0; j < kOut; ++j) dout[j] = 0.0f;
    // cross entropy of the outcome
    const float m = fmaxf(out[0], fmaxf(out[1], out[2]));
    const float e0 = expf(out[0] - m), e1 = expf(out[1] - m), e2 = expf(out[2] - m);
    const float z = e0 + e1 + e2;
    float loss = -(out[c] - m - logf(z));
    dout[0] = e0 / z - (c == 0 ? 1.0f : 0.0f);
    dout[1] = e1 / z - (c == 1 ? 1.0f : 0.0f);
    dout[2] = e2 / z - (c == 2 ? 1.0f : 0.0f);
    // pinball losses of the outcome's two quantile heads
    int h0, k0, h1, k1;
    heads_of(c, &h0, &k0, &h1, &k1);
    const int heads[2] = {h0, h1}, ks[2] = {k0, k1};
    const float ys[2] = {y0, y1};
    for (int hh = 0; hh < 2; ++hh) {
        const float *h = out + heads[hh];
        const int K = ks[hh];
        float q[kQL], dq[kQL];
        knots(h, K, q);
        for (int k = 0; k < K; ++k) {
            const float tau = level(k, K), u = ys[hh] - q[k];
            loss += u >= 0.0f ? tau * u : (tau - 1.0f) * u;
            dq[k] = (u < 0.0f ? 1.0f : 0.0f) - tau;  // d loss / d q_k
        }
        // back through q_k = h_0 + sum_{j<=k, j>=1} softplus(h_j)
        float tail = 0.0f;
        for (int k = K - 1; k >= 1; --k) {
            tail += dq[k];
            const float sg = 1.0f / (1.0f + expf(-h[k]));
            dout[heads[hh] + k] = tail * sg;
        }
        dout[heads[hh]] = tail + dq[0];
    }
    return loss;
}

// shared-memory layout of k_surr_grad (floats)
constexpr int kSmWT = 0;                          // W1..W4 transposed: WT[k][j]
constexpr int kSmB = kSmWT + kParams - 4 * kHid;  // biases b1..b4 (256)
constexpr int kSmX = kSmB + 4 * kHid;             // inputs [64][4]
constexpr int kSmA1 = kSmX + kSlice * kIn;        // activations [64][64] x 3
constexpr int kSmA2 = kSmA1 + kSlice * kHid;
constexpr int kSmA3 = kSmA2 + kSlice * kHid;
constexpr int kSmO = kSmA3 + kSlice * kHid;       // outputs, then their gradients
constexpr int kSmD = kSmO + kSlice * kOut;        // back-propagated deltas
constexpr int kSmTotal = kSmD + kSlice * kHid;
constexpr int kGradSmemBytes = kSmTotal * 4;

// z[s][j] = b[j] + sum_k WT[k][j] a[s][k] for the 64 x 64 outputs of a layer
__device__ __forceinline__ void dense_fwd(const float *WT, const float *b, const float *a, int K, float *z, bool relu) {
    const int j = threadIdx.x & 63;
    for (int s = threadIdx.x >> 6; s < kSlice; s += kTrainThreads / 64) {
        float acc = b[j];
        for (int k = 0; k < K; ++k) acc += WT[k * kHid + j] * a[s * K + k];
        z[s * kHid + j] = relu ? fmaxf(acc, 0.0f) : acc;
    }
    __syncthreads();
}

// weight / bias gradients of one layer: gW[j][k] = sum_s dz[s][j] a[s][k]
__device__ __forceinline__ void dense_wgrad(const float *dz, const float *a, int K, float *gW, float *gb) {
    for (int e = threadIdx.x; e < kHid * K; e += kTrainThreads) {
        const int j = e / K, k = e % K;
        float acc = 0.0f;
        for (int s = 0; s < kSlice; ++s) acc += dz[s * kHid + j] * a[s * K + k];
        gW[e] = acc;
    }
    for (int j = threadIdx.x; j < kHid; j += kTrainThreads) {
        float acc = 0.0f;
        for (int s = 0; s < kSlice; ++s) acc += dz[s * kHid + j];
        gb[j] = acc;
    }
}

// delta of the layer below: da[s][k] = sum_j W[j][k] dz[s][j], masked by ReLU
__device__ __forceinline__ void dense_bwd(const float *W, const float *dz, const float *a_below, float *da) {
    const int k = threadIdx.x & 63;
    for (int s = threadIdx.x >> 6; s < kSlice; s += kTrainThreads / 64) {
        float acc = 0.0f;
        for (int j = 0; j < kHid; ++j) acc += W[j * kHid + k] * dz[s * kHid + j];
        da[s * kHid + k] = a_below[s * kHid + k] > 0.0f ? acc : 0.0f;
    }
    __syncthreads();
}

// Forward + backward of samples [off + 64 b, off + 64 b + 64) clipped to n;
// writes this block's gradient sums (kParams floats) and loss sum.
__global__ void __launch_bounds__(kTrainThreads) k_surr_grad(const float *P, const float *x, const int *cls,
                                                             const float *tgt, long long n, long long off,
                                                             float *gpart, float *lpart) {
    extern __shared__ float sm[];
    float *WT = sm + kSmWT, *B = sm + kSmB, *X = sm + kSmX;
    float *A1 = sm + kSmA1, *A2 = sm + kSmA2, *A3 = sm + kSmA3, *O = sm + kSmO, *D = sm + kSmD;
    // transposed weights: WT1 [4][64], WT2..WT4 [64][64]
    float *WT1 = WT, *WT2 = WT + kIn * kHid, *WT3 = WT2 + kHid * kHid, *WT4 = WT3 + kHid * kHid;
    for (int e = threadIdx.x; e < kHid * kIn; e += kTrainThreads) {
        const int j = e / kIn, k = e % kIn;
        WT1[k * kHid + j] = P[kW1 + e];
    }
    for (int e = threadIdx.x; e < kHid * kHid; e += kTrainThreads) {
        const int j = e / kHid, k = e % kHid;
        WT2[k * kHid + j] = P[kW2 + e];
        WT3[k * kHid + j] = P[kW3 + e];
        WT4[k * kHid + j] = P[kW4 + e];
    }
    for (int j = threadIdx.x; j < kHid; j += kTrainThreads) {
        B[j] = P[kB1 + j]; B[kHid + j] = P[kB2 + j]; B[2 * kHid + j] = P[kB3 + j]; B[3 * kHid + j] = P[kB4 + j];
    }
    const long long s0 = off + (long long)blockIdx.x * kSlice;
    for (int e = threadIdx.x; e < kSlice * kIn; e += kTrainThreads) {
        const long long i = s0 + e / kIn;
        X[e] = i < n ? x[i * kIn + e % kIn] : 0.0f;
    }
    __syncthreads();
    dense_fwd(WT1, B, X, kIn, A1, true);
    dense_fwd(WT2, B + kHid, A1, kHid, A2, true);
    dense_fwd(WT3, B + 2 * kHid, A2, kHid, A3, true);
    dense_fwd(WT4, B + 3 * kHid, A3, kHid, O, false);
    // output gradients, one thread per sample (zero for padding rows)
    __shared__ float sloss[kSlice];
    if (threadIdx.x < kSlice) {
        const long long i = s0 + threadIdx.x;
        float dout[kOut];
        float l = 0.0f;
        if (i < n) {
            l = output_grad(O + threadIdx.x * kOut, cls[i], tgt[2 * i], tgt[2 * i + 1], dout);
        } else {
            for (int j = 0; j < kOut; ++j) dout[j] = 0.0f;
        }
        for (int j = 0; j < kOut; ++j) O[threadIdx.x * kOut + j] = dout[j];
        sloss[threadIdx.x] = l;
    }
    __syncthreads();
    float *g = gpart + (size_t)blockIdx.x * kParams;
    dense_wgrad(O, A3, kHid, g + kW4, g + kB4);
    dense_bwd(P + kW4, O, A3, D);                 // delta at layer 3 output
    dense_wgrad(D, A2, kHid, g + kW3, g + kB3);
    __syncthreads();
    dense_bwd(P + kW3, D, A2, O);                 // delta at layer 2 output (reuses O)
    dense_wgrad(O, A1, kHid, g + kW2, g + kB2);
    __syncthreads();
    dense_bwd(P + kW2, O, A1, D);                 // delta at layer 1 output
    dense_wgrad(D, X, kIn, g + kW1, g + kB1);
    if (threadIdx.x == 0) {
        float l = 0.0f;
        for (int s = 0; s < kSlice; ++s) l += sloss[s];
        lpart[blockIdx.x] = l;
    }
}

// grad[p] = scale * sum_b gpart[b][p], in block order
__global__ void k_surr_reduce(const float *gpart, int nblk, float scale, float *grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    float acc = 0.0f;
    for (int b = 0; b < nblk; ++b) acc += gpart[(size_t)b * kParams + p];
    grad[p] = acc * scale;
}

__global__ void k_surr_adam(float *P, float *m, float *v, const float *grad, float lr, float b1t, float b2t) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gr = grad[p];
    const float mm = b1 * m[p] + (1.0f - b1) * gr;
    const float vv = b2 * v[p] + (1.0f - b2) * gr * gr;
    m[p] = mm;
    v[p] = vv;
    P[p] -= lr * (mm / (1.0f - b1t)) / (sqrtf(vv / (1.0f - b2t)) + eps);
}

// He-uniform weights, zero biases; deterministic in the seed
__global__ void k_surr_init(float *P, unsigned long long seed) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    int fan_in;
    bool is_w = true;
    if (p < kB1) fan_in = kIn;
    else if (p < kW2) is_w = false;
    else if (p < kB2) fan_in = kHid;
    else if (p < kW3) is_w = false;
    else if (p < kB3) fan_in = kHid;
    else if (p < kW4) is_w = false;
    else if (p < kB4) fan_in = kHid;
    else is_w = false;
    if (!is_w) { P[p] = 0.0f; return; }
    Stream rs;
    rs.init(seed, 1u, (uint32_t)p, kStageSurrData);
    const float bound = sqrtf(6.0f / (float)fan_in);
    float w = (2.0f * Rand<float>::u(rs) - 1.0f) * bound;
    if (p >= kW4) w *= 0.1f;  // small initial outputs
    P[p] = w;
}

// ------------------------------------------------------ tensor-core tests
constexpr int kFwdWarps = 4;
constexpr int kFwdSmemBytes = kImageBytes + kFwdWarps * kStageFloats * 4;

// network outputs of n given inputs, 16 rows per warp per pass
__global__ void __launch_bounds__(32 * kFwdWarps) k_surr_forward(const float *P, const float *x, long long n,
                                                                 float *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *frag = reinterpret_cast<uint32_t *>(smem);
    float *bias = reinterpret_cast<float *>(frag + kFragWords);
    float *stage = bias + kBiasFloats + (threadIdx.x >> 5) * kStageFloats;
    float *xin = stage, *yout = stage + 16 * kIn;
    build_image(P, frag, bias);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * kFwdWarps;
    for (long long r0 = ((long long)blockIdx.x * kFwdWarps + (threadIdx.x >> 5)) * 16; r0 < n; r0 += nwarps * 16) {
        for (int e = lane; e < 16 * kIn; e += 32) {
            const long long r = r0 + e / kIn;
            xin[e] = r < n ? x[r * kIn + e % kIn] : 0.0f;
        }
        __syncwarp();
        forward16(frag, bias, xin, yout);
        for (int e = lane; e < 16 * kOut; e += 32) {
            const long long r = r0 + e / kOut;
            if (r < n) out[r * kOut + e % kOut] = yout[e];
        }
        __syncwarp();
    }
}

// outcomes sampled from the network at n walk states (d_n, d_f, mu', lmax)
__global__ void __launch_bounds__(32 * kFwdWarps) k_surr_sample(const float *P, unsigned long long seed,
                                                                const float *state, long long n, int *cls,
                                                                float *y0, float *y1) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *frag = reinterpret_cast<uint32_t *>(smem);
    float *bias = reinterpret_cast<float *>(frag + kFragWords);
    float *stage = bias + kBiasFloats + (threadIdx.x >> 5) * kStageFloats;
    float *xin = stage, *yout = stage + 16 * kIn;
    build_image(P, frag, bias);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * kFwdWarps;
    for (long long r0 = ((long long)blockIdx.x * kFwdWarps + (threadIdx.x >> 5)) * 16; r0 < n; r0 += nwarps * 16) {
        if (lane < 16) {
            const long long r = r0 + lane;
            float f[kIn] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (r < n) features(state[4 * r], state[4 * r + 1], state[4 * r + 2], state[4 * r + 3], f);
            for (int k = 0; k < kIn; ++k) xin[lane * kIn + k] = f[k];
        }
        __syncwarp();
        forward16(frag, bias, xin, yout);
        if (lane < 16 && r0 + lane < n) {
            const long long r = r0 + lane;
            Stream rs;
            rs.init(seed, 0u, (uint32_t)r, kStageSurrTest);
            const float u0 = Rand<float>::u(rs), u1 = Rand<float>::u(rs), u2 = Rand<float>::u(rs);
            float a, b;
            cls[r] = sample_outcome(yout + lane * kOut, u0, u1, u2, &a, &b);
            y0[r] = a;
            y1[r] = b;
        }
        __syncwarp();
    }
}

}  // namespace

// ------------------------------------------------------------ entry points
namespace {

// device buffers of one call, released on every return path
struct DevScope {
    std::vector<void *> ptrs;
    cudaStream_t stream = nullptr;
    ~DevScope() {
        if (stream) cudaStreamSynchronize(stream);
        for (void *p : ptrs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
    template <class T> T *alloc(size_t count) {
        void *p = nullptr;
        if (count == 0) count = 1;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
};

int surr_device(DevScope &ds) {
    int dev = 0, major = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IMC_ERR_NO_DEVICE;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess || major < 10)
        return IMC_ERR_NO_DEVICE;
    if (cudaStreamCreateWithFlags(&ds.stream, cudaStreamNonBlocking) != cudaSuccess) return IMC_ERR_CUDA;
    return IMC_OK;
}

int h2d(void *d, const void *h, size_t bytes, cudaStream_t s) {
    return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess ? IMC_OK : IMC_ERR_CUDA;
}
int d2h(void *h, const void *d, size_t bytes, cudaStream_t s) {
    return cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s) == cudaSuccess ? IMC_OK : IMC_ERR_CUDA;
}
int finish(cudaStream_t s) {
    if (cudaGetLastError() != cudaSuccess) return IMC_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? IMC_OK : IMC_ERR_CUDA;
}

int grid_of(long long n, int per_block, int cap) {
    long long b = (n + per_block - 1) / per_block;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// per-slice gradients and the block-order reduction: grad = mean over n
int launch_grad(const float *P, const float *x, const int *cls, const float *tgt, long long n, long long off,
                float *gpart, float *lpart, float *grad, cudaStream_t s) {
    const int nblk = (int)((n + kSlice - 1) / kSlice);
    k_surr_grad<<<nblk, kTrainThreads, kGradSmemBytes, s>>>(P, x, cls, tgt, off + n, off, gpart, lpart);
    k_surr_reduce<<<(kParams + 255) / 256, 256, 0, s>>>(gpart, nblk, 1.0f / (float)n, grad);
    return cudaGetLastError() == cudaSuccess ? IMC_OK : IMC_ERR_CUDA;
}

bool smem_optin() {
    static bool done = false;
    if (done) return true;
    if (cudaFuncSetAttribute(k_surr_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradSmemBytes) != cudaSuccess)
        return false;
    done = true;
    return true;
}

}  // namespace

extern "C" {

int imc_surrogate_param_count(int *count) {
    if (!count) return IMC_ERR_INVALID_ARG;
    *count = kParams;
    return IMC_OK;
}

int imc_surrogate_walk(uint64_t seed, const float *state, int64_t n, float *x, int32_t *cls, float *tgt) {
    if (n < 0 || (n > 0 && (!x || !cls || !tgt)) || n > (int64_t)0xFFFFFFFF) return IMC_ERR_INVALID_ARG;
    if (n == 0) return IMC_OK;
    DevScope ds;
    int rc = surr_device(ds);
    if (rc) return rc;
    float *dstate = nullptr;
    if (state) {
        if (!(dstate = ds.alloc<float>(4 * n))) return IMC_ERR_OOM;
        if ((rc = h2d(dstate, state, 16 * (size_t)n, ds.stream))) return rc;
    }
    float *dx = ds.alloc<float>(kIn * n), *dt = ds.alloc<float>(2 * n);
    int *dc = ds.alloc<int>(n);
    if (!dx || !dt || !dc) return IMC_ERR_OOM;
    k_surr_datagen<<<grid_of(n, 256, 4096), 256, 0, ds.stream>>>(seed, n, dstate, dx, dc, dt);
    if ((rc = d2h(x, dx, 4 * kIn * (size_t)n, ds.stream)) || (rc = d2h(cls, dc, 4 * (size_t)n, ds.stream)) ||
        (rc = d2h(tgt, dt, 8 * (size_t)n, ds.stream)))
        return rc;
    return finish(ds.stream);
}

int imc_surrogate_grad(const float *params, const float *x, const int32_t *cls, const float *tgt, int64_t n,
                       float *grad, double *loss) {
    if (!params || !x || !cls || !tgt || !grad || n <= 0) return IMC_ERR_INVALID_ARG;
    for (int64_t i = 0; i < n; ++i)
        if (cls[i] < 0 || cls[i] > 2) return IMC_ERR_INVALID_ARG;
    DevScope ds;
    int rc = surr_device(ds);
    if (rc) return rc;
    if (!smem_optin()) return IMC_ERR_CUDA;
    const int nblk = (int)((n + kSlice - 1) / kSlice);
    float *dP = ds.alloc<float>(kParams), *dx = ds.alloc<float>(kIn * n), *dt = ds.alloc<float>(2 * n);
    int *dc = ds.alloc<int>(n);
    float *gpart = ds.alloc<float>((size_t)nblk * kParams), *lpart = ds.alloc<float>(nblk);
    float *dg = ds.alloc<float>(kParams);
    if (!dP || !dx || !dt || !dc || !gpart || !lpart || !dg) return IMC_ERR_OOM;
    if ((rc = h2d(dP, params, 4 * (size_t)kParams, ds.stream)) || (rc = h2d(dx, x, 4 * kIn * (size_t)n, ds.stream)) ||
        (rc = h2d(dc, cls, 4 * (size_t)n, ds.stream)) || (rc = h2d(dt, tgt, 8 * (size_t)n, ds.stream)))
        return rc;
    if ((rc = launch_grad(dP, dx, dc, dt, n, 0, gpart, lpart, dg, ds.stream))) return rc;
    std::vector<float> lp(nblk);
    if ((rc = d2h(grad, dg, 4 * (size_t)kParams, ds.stream)) || (rc = d2h(lp.data(), lpart, 4 * (size_t)nblk, ds.stream)))
        return rc;
    if ((rc = finish(ds.stream))) return rc;
    if (loss) {
        double l = 0.0;
        for (float v : lp) l += v;
        *loss = l / (double)n;
    }
    return IMC_OK;
}

int imc_surrogate_train(const ImcSurrogateTrainConfig *cfg, float *params, float *loss_history) {
    if (!cfg || !params) return IMC_ERR_INVALID_ARG;
    const long long n = cfg->n_samples;
    const int B = cfg->batch;
    if (n <= 0 || n > (int64_t)0xFFFFFFFF || B <= 0 || B % kSlice || n % B || cfg->iterations <= 0 ||
        !(cfg->lr > 0.0f) || cfg->lr_min < 0.0f)
        return IMC_ERR_INVALID_ARG;
    DevScope ds;
    int rc = surr_device(ds);
    if (rc) return rc;
    if (!smem_optin()) return IMC_ERR_CUDA;
    const int nblk = B / kSlice;
    float *dx = ds.alloc<float>(kIn * n), *dt = ds.alloc<float>(2 * n);
    int *dc = ds.alloc<int>(n);
    float *dP = ds.alloc<float>(kParams), *dm = ds.alloc<float>(kParams), *dv = ds.alloc<float>(kParams);
    float *gpart = ds.alloc<float>((size_t)nblk * kParams), *dg = ds.alloc<float>(kParams);
    float *lpart = ds.alloc<float>((size_t)nblk * cfg->iterations);
    if (!dx || !dt || !dc || !dP || !dm || !dv || !gpart || !dg || !lpart) return IMC_ERR_OOM;
    k_surr_datagen<<<grid_of(n, 256, 8192), 256, 0, ds.stream>>>(cfg->seed, n, nullptr, dx, dc, dt);
    k_surr_init<<<(kParams + 255) / 256, 256, 0, ds.stream>>>(dP, cfg->seed);
    if (cudaMemsetAsync(dm, 0, 4 * (size_t)kParams, ds.stream) != cudaSuccess ||
        cudaMemsetAsync(dv, 0, 4 * (size_t)kParams, ds.stream) != cudaSuccess)
        return IMC_ERR_CUDA;
    double b1t = 1.0, b2t = 1.0;
    const double pi = 3.14159265358979323846;
    for (int it = 0; it < cfg->iterations; ++it) {
        const long long off = ((long long)it * B) % n;
        k_surr_grad<<<nblk, kTrainThreads, kGradSmemBytes, ds.stream>>>(dP, dx, dc, dt, off + B, off, gpart,
                                                                        lpart + (size_t)it * nblk);
        k_surr_reduce<<<(kParams + 255) / 256, 256, 0, ds.stream>>>(gpart, nblk, 1.0f / (float)B, dg);
        b1t *= 0.9;
        b2t *= 0.999;
        const double lr = cfg->lr_min + 0.5 * (cfg->lr - cfg->lr_min) * (1.0 + cos(pi * it / cfg->iterations));
        k_surr_adam<<<(kParams + 255) / 256, 256, 0, ds.stream>>>(dP, dm, dv, dg, (float)lr, (float)b1t, (float)b2t);
        if (cudaGetLastError() != cudaSuccess) return IMC_ERR_CUDA;
    }
    if ((rc = d2h(params, dP, 4 * (size_t)kParams, ds.stream))) return rc;
    std::vector<float> lp;
    if (loss_history) {
        lp.resize((size_t)nblk * cfg->iterations);
        if ((rc = d2h(lp.data(), lpart, 4 * lp.size(), ds.stream))) return rc;
    }
    if ((rc = finish(ds.stream))) return rc;
    if (loss_history) {
        for (int it = 0; it < cfg->iterations; ++it) {
            double l = 0.0;
            for (int b = 0; b < nblk; ++b) l += lp[(size_t)it * nblk + b];
            loss_history[it] = (float)(l / B);
        }
    }
    return IMC_OK;
}

int imc_surrogate_forward(const float *params, const float *x, int64_t n, float *out) {
    if (!params || n < 0 || (n > 0 && (!x || !out))) return IMC_ERR_INVALID_ARG;
    if (n == 0) return IMC_OK;
    DevScope ds;
    int rc = surr_device(ds);
    if (rc) return rc;
    float *dP = ds.alloc<float>(kParams), *dx = ds.alloc<float>(kIn * n), *dout = ds.alloc<float>(kOut * n);
    if (!dP || !dx || !dout) return IMC_ERR_OOM;
    if ((rc = h2d(dP, params, 4 * (size_t)kParams, ds.stream)) || (rc = h2d(dx, x, 4 * kIn * (size_t)n, ds.stream)))
        return rc;
    k_surr_forward<<<grid_of(n, 16 * kFwdWarps, 1024), 32 * kFwdWarps, kFwdSmemBytes, ds.stream>>>(dP, dx, n, dout);
    if ((rc = d2h(out, dout, 4 * kOut * (size_t)n, ds.stream))) return rc;
    return finish(ds.stream);
}

int imc_surrogate_sample(const float *params, uint64_t seed, const float *state, int64_t n, int32_t *cls, float *y0,
                         float *y1) {
    if (!params || n < 0 || n > (int64_t)0xFFFFFFFF || (n > 0 && (!state || !cls || !y0 || !y1)))
        return IMC_ERR_INVALID_ARG;
    if (n == 0) return IMC_OK;
    DevScope ds;
    int rc = surr_device(ds);
    if (rc) return rc;
    float *dP = ds.alloc<float>(kParams), *dst = ds.alloc<float>(4 * n);
    float *d0 = ds.alloc<float>(n), *d1 = ds.alloc<float>(n);
    int *dc = ds.alloc<int>(n);
    if (!dP || !dst || !d0 || !d1 || !dc) return IMC_ERR_OOM;
    if ((rc = h2d(dP, params, 4 * (size_t)kParams, ds.stream)) || (rc = h2d(dst, state, 16 * (size_t)n, ds.stream)))
        return rc;
    k_surr_sample<<<grid_of(n, 16 * kFwdWarps, 1024), 32 * kFwdWarps, kFwdSmemBytes, ds.stream>>>(dP, seed, dst, n, dc,
                                                                                                d0, d1);
    if ((rc = d2h(cls, dc, 4 * (size_t)n, ds.stream)) || (rc = d2h(y0, d0, 4 * (size_t)n, ds.stream)) ||
        (rc = d2h(y1, d1, 4 * (size_t)n, ds.stream)))
        return rc;
    return finish(ds.stream);
}

}  // extern "C"
