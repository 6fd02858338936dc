// imc_surrogate.cuh -- the learned thick-cell transport surrogate: shape,
// parameter layout, input features, output heads and sampling.
//
// Inside one cell a history is a random walk: exponential flights with the
// effective scattering rate s = sigma_a(1 - f) + sigma_s, isotropic
// re-emission, and a weight that decays deterministically with path length l
// as exp(-sigma_a f l) (src/imc_transport.jl:72-193).  Measured in mean free
// paths, the walk therefore depends only on
//   d_n   distance to the nearer face        (mfp)
//   d_f   distance to the farther face       (mfp)
//   mu'   direction cosine, > 0 away from the nearer face
//   lmax  path after which the walk is cut: min(census path, cut-off path),
//         census path = s c (dt - t) ds, cut-off path = ln(E / Emin) s / (sigma_a f)
// and ends in one of three ways: exit through the near face, exit through
// the far face, or truncation at lmax (census, or the 1 % energy cut-off,
// src/imc_transport.jl:97-106).  The energy outcome is exact given the path:
// the absorbed fraction is 1 - exp(-sigma_a f l).
//
// The network (4 inputs, three hidden layers of 64 ReLU units, 64 outputs;
// BF16 weights in the transport kernel, FP32 accumulation) maps
//   x = (g(d_n / sqrt(lmax)), g(d_f / sqrt(lmax)), mu', (log10 lmax - 2)/2),
//   g(r) = min(ln(1 + r) / ln 11, 1),
// -- distances in diffusion lengths, which decide whether a face is within
// reach; ten or more are as good as infinity -- to the logits of the three
// outcomes and, for each outcome, the quantiles of its conditional
// distributions, sampled by inverse transform:
//   near / far exit:  y = ln(l / lmax) (12 quantiles), exit |mu| (6)
//   truncation:       displacement (x_end - x_start)/sqrt(lmax) toward the far
//                     face (6), final mu' (6)
// Quantile heads are monotone by construction: q_0 = h_0,
// q_k = q_{k-1} + softplus(h_k).
#pragma once
#include <cstdint>

#ifndef IMC_HD
#define IMC_HD __host__ __device__ __forceinline__
#endif

namespace imc {
namespace surr {

constexpr int kIn = 4;
constexpr int kHid = 64;
constexpr int kOut = 64;
// parameter layout (float, row-major W[out][in]):
constexpr int kW1 = 0;                       // [64][4]
constexpr int kB1 = kW1 + kHid * kIn;        // [64]
constexpr int kW2 = kB1 + kHid;              // [64][64]
constexpr int kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid;
constexpr int kB3 = kW3 + kHid * kHid;
constexpr int kW4 = kB3 + kHid;              // [64 out][64]
constexpr int kB4 = kW4 + kOut * kHid;
constexpr int kParams = kB4 + kOut;          // 12,800

// output heads
constexpr int kLogit = 0;                    // 3 logits: near, far, truncated
constexpr int kQL = 12, kQM = 6, kQP = 6;
constexpr int kNearL = 3;                    // ln(l/lmax) quantiles, near exit
constexpr int kNearM = kNearL + kQL;         // |mu| quantiles, near exit
constexpr int kFarL = kNearM + kQM;
constexpr int kFarM = kFarL + kQL;
constexpr int kTrP = kFarM + kQM;            // displacement / sqrt(lmax)
constexpr int kTrM = kTrP + kQP;             // final mu'
constexpr int kUsed = kTrM + kQM;            // 51
static_assert(kUsed <= kOut, "heads fit the output layer");

enum Outcome { kNear = 0, kFar = 1, kTrunc = 2 };

// domain in which the network is used; outside it the analog walk runs
constexpr float kLmaxMin = 32.0f;            // shorter walks are cheaper analog
constexpr float kLmaxMax = 1.0e4f;
constexpr float kCellMin = 8.0f;             // cell at least this many mfp wide
constexpr float kMinGain = 100.0f;           // ask only if the walk would take this many collisions

// network input from the walk's dimensionless state
IMC_HD float reach(float d, float lmax) {
    const float v = log1pf(d / sqrtf(lmax)) * 0.41703239f;  // 1 / ln 11
    return v < 1.0f ? v : 1.0f;
}
IMC_HD void features(float d_n, float d_f, float mu_p, float lmax, float x[kIn]) {
    x[0] = reach(d_n, lmax);
    x[1] = reach(d_f, lmax);
    x[2] = mu_p;
    x[3] = (log10f(lmax) - 2.0f) * 0.5f;
}

IMC_HD float softplusf(float v) { return v > 20.0f ? v : log1pf(expf(v)); }

// quantile level of knot k of K knots
IMC_HD float level(int k, int K) { return ((float)k + 0.5f) / (float)K; }

// monotone knots from raw head outputs
IMC_HD void knots(const float *h, int K, float *q) {
    float acc = h[0];
    q[0] = acc;
    for (int k = 1; k < K; ++k) {
        acc += softplusf(h[k]);
        q[k] = acc;
    }
}

// Inverse-transform sample of the piecewise-linear quantile function through
// (level(k), q_k), extended linearly by half a knot spacing to u = 0 and
// u = 1.  Only the knots up to the one needed are formed (lazy cumulative
// softplus).
IMC_HD float inv_cdf(const float *h, int K, float u) {
    float pos = u * (float)K - 0.5f;  // in [-0.5, K - 0.5]
    int k = (int)floorf(pos);
    k = k < 0 ? 0 : (k > K - 2 ? K - 2 : k);
    float q0 = h[0];
    for (int j = 1; j <= k; ++j) q0 += softplusf(h[j]);
    const float q1 = q0 + softplusf(h[k + 1]);
    return q0 + (pos - (float)k) * (q1 - q0);
}

// Expected number of collisions an in-cell walk from (d_n, d_f) takes before
// it leaves the cell or is cut at lmax, for a walk whose displacement
// variance grows by 2/3 per mean free path (diffusion limit): the exit time
// from the cell, 1.5 d_n d_f, the truncated exit time through the nearer
// face alone, E[min(tau, lmax)] ~ sqrt(12 lmax / pi) d_n = 1.95 d_n
// sqrt(lmax), and lmax itself bound it.  The transport kernel asks the
// network only when this is large enough to pay for the query.
IMC_HD float expected_collisions(float d_n, float d_f, float lmax) {
    float e = 1.5f * d_n * d_f;
    const float h = 1.95f * d_n * sqrtf(lmax);
    e = h < e ? h : e;
    return e < lmax ? e : lmax;
}

// first output and knot count of the two heads of an outcome
IMC_HD void heads_of(int c, int *h0, int *k0, int *h1, int *k1) {
    if (c == kNear) { *h0 = kNearL; *k0 = kQL; *h1 = kNearM; *k1 = kQM; }
    else if (c == kFar) { *h0 = kFarL; *k0 = kQL; *h1 = kFarM; *k1 = kQM; }
    else { *h0 = kTrP; *k0 = kQP; *h1 = kTrM; *k1 = kQM; }
}

// Outcome (softmax of the logits, by u0) and its two targets (inverse
// transform of the heads, by u1 and u2) from one row of network outputs.
IMC_HD int sample_outcome(const float *out, float u0, float u1, float u2, float *y0, float *y1) {
    const float m = fmaxf(out[0], fmaxf(out[1], out[2]));
    const float e0 = expf(out[0] - m), e1 = expf(out[1] - m), e2 = expf(out[2] - m);
    const float z = u0 * (e0 + e1 + e2);
    const int c = z < e0 ? kNear : (z < e0 + e1 ? kFar : kTrunc);
    int h0, k0, h1, k1;
    heads_of(c, &h0, &k0, &h1, &k1);
    *y0 = inv_cdf(out + h0, k0, u1);
    *y1 = inv_cdf(out + h1, k1, u2);
    return c;
}

}  // namespace surr
}  // namespace imc

#ifdef __CUDACC__
#include <cuda_bf16.h>

namespace imc {
namespace surr {

// Shared-memory image of the network for the tensor-core forward pass:
// B fragments of m16n8k16 (BF16) in the order lanes load them, FP32 biases.
//   layer 1: K = 4 padded to 16 (1 k-step), N = 64 (8 n-tiles)
//   layers 2-4: K = 64 (4 k-steps), N = 64
constexpr int kFragL1 = 1 * 8 * 32 * 2;          // uint32 words
constexpr int kFragL = 4 * 8 * 32 * 2;
constexpr int kFragWords = kFragL1 + 3 * kFragL;  // 6656 words = 26 KiB
constexpr int kBiasFloats = 3 * kHid + kOut;
constexpr int kImageBytes = kFragWords * 4 + kBiasFloats * 4;
// per-warp staging: 16 query rows of inputs and of outputs
constexpr int kStageFloats = 16 * kIn + 16 * kOut;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// word index of (layer, k-step, n-tile, lane) in the fragment image
__host__ __device__ __forceinline__ int frag_index(int layer, int kk, int nn, int lane) {
    int base = layer == 0 ? 0 : kFragL1 + (layer - 1) * kFragL;
    return base + ((kk * 8 + nn) * 32 + lane) * 2;
}

// Builds the image from FP32 parameters (one call per block, all threads).
__device__ __forceinline__ void build_image(const float *P, uint32_t *frag, float *bias) {
    for (int w = threadIdx.x; w < kFragWords / 2; w += blockDim.x) {
        int layer, rem;
        if (w < kFragL1 / 2) { layer = 0; rem = w; }
        else { layer = 1 + (w - kFragL1 / 2) / (kFragL / 2); rem = (w - kFragL1 / 2) % (kFragL / 2); }
        const int lane = rem % 32, knn = rem / 32, nn = knn % 8, kk = knn / 8;
        const int g = lane >> 2, t = lane & 3;
        const int n = nn * 8 + g, k0 = kk * 16 + 2 * t;
        const float *W;
        int K;
        if (layer == 0) { W = P + kW1; K = kIn; }
        else if (layer == 1) { W = P + kW2; K = kHid; }
        else if (layer == 2) { W = P + kW3; K = kHid; }
        else { W = P + kW4; K = kHid; }
        auto wv = [&](int k) { return k < K ? W[n * K + k] : 0.0f; };
        frag[frag_index(layer, kk, nn, lane)] = pack_bf16(wv(k0), wv(k0 + 1));
        frag[frag_index(layer, kk, nn, lane) + 1] = pack_bf16(wv(k0 + 8), wv(k0 + 9));
    }
    for (int i = threadIdx.x; i < kBiasFloats; i += blockDim.x) {
        float v;
        if (i < kHid) v = P[kB1 + i];
        else if (i < 2 * kHid) v = P[kB2 + i - kHid];
        else if (i < 3 * kHid) v = P[kB3 + i - 2 * kHid];
        else v = P[kB4 + i - 3 * kHid];
        bias[i] = v;
    }
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One layer: acc[nn][0..3] = A (16 x K) * W^T (K x 64), A given as k-step fragments.
__device__ __forceinline__ void layer_mma(const uint32_t *frag, int layer, int ksteps, const uint32_t (*a)[4],
                                          float (*acc)[4], int lane) {
#pragma unroll
    for (int nn = 0; nn < 8; ++nn) {
        acc[nn][0] = acc[nn][1] = acc[nn][2] = acc[nn][3] = 0.0f;
    }
    for (int kk = 0; kk < ksteps; ++kk) {
#pragma unroll
        for (int nn = 0; nn < 8; ++nn) {
            const uint2 b = *reinterpret_cast<const uint2 *>(frag + frag_index(layer, kk, nn, lane));
            mma_bf16(acc[nn], a[kk], b.x, b.y);
        }
    }
}

// bias + ReLU, then repack the accumulators as the next layer's A fragments
__device__ __forceinline__ void to_next(float (*acc)[4], const float *bias, uint32_t (*a)[4], int lane) {
    const int t = lane & 3;
#pragma unroll
    for (int nn = 0; nn < 8; ++nn) {
        const int c = nn * 8 + 2 * t;
        const float v0 = fmaxf(acc[nn][0] + bias[c], 0.0f), v1 = fmaxf(acc[nn][1] + bias[c + 1], 0.0f);
        const float v2 = fmaxf(acc[nn][2] + bias[c], 0.0f), v3 = fmaxf(acc[nn][3] + bias[c + 1], 0.0f);
        const int kk = nn >> 1;
        if ((nn & 1) == 0) { a[kk][0] = pack_bf16(v0, v1); a[kk][1] = pack_bf16(v2, v3); }
        else { a[kk][2] = pack_bf16(v0, v1); a[kk][3] = pack_bf16(v2, v3); }
    }
}

// Warp-collective forward pass of 16 queries.  All 32 lanes call it with the
// same arguments.  xin: 16 x kIn inputs (rows beyond the batch may hold any
// finite value); yout: 16 x kOut outputs.  Both in the warp's shared staging.
__device__ __forceinline__ void forward16(const uint32_t *frag, const float *bias, const float *xin, float *yout) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[4][4];
    float acc[8][4];
    // layer 1 input fragment: features in columns 0..3 of a 16-column tile
    {
        const float x0 = t < 2 ? xin[g * kIn + 2 * t] : 0.0f, x1 = t < 2 ? xin[g * kIn + 2 * t + 1] : 0.0f;
        const float x2 = t < 2 ? xin[(g + 8) * kIn + 2 * t] : 0.0f, x3 = t < 2 ? xin[(g + 8) * kIn + 2 * t + 1] : 0.0f;
        a[0][0] = pack_bf16(x0, x1);
        a[0][1] = pack_bf16(x2, x3);
        a[0][2] = 0u;
        a[0][3] = 0u;
    }
    layer_mma(frag, 0, 1, a, acc, lane);
    to_next(acc, bias, a, lane);
    layer_mma(frag, 1, 4, a, acc, lane);
    to_next(acc, bias + kHid, a, lane);
    layer_mma(frag, 2, 4, a, acc, lane);
    to_next(acc, bias + 2 * kHid, a, lane);
    layer_mma(frag, 3, 4, a, acc, lane);
    const float *b4 = bias + 3 * kHid;
#pragma unroll
    for (int nn = 0; nn < 8; ++nn) {
        const int c = nn * 8 + 2 * t;
        yout[g * kOut + c] = acc[nn][0] + b4[c];
        yout[g * kOut + c + 1] = acc[nn][1] + b4[c + 1];
        yout[(g + 8) * kOut + c] = acc[nn][2] + b4[c];
        yout[(g + 8) * kOut + c + 1] = acc[nn][3] + b4[c + 1];
    }
    __syncwarp();
}

}  // namespace surr
}  // namespace imc
#endif  // __CUDACC__
