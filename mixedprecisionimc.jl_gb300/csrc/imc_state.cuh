// imc_state.cuh -- particle-state precision policies (the PRECISION keyword).
//
//   StF64: FP64 storage, FP64 arithmetic  (reference Float64 semantics)
//   StF32: FP32 storage, FP32 arithmetic
//   StF16: binary16 storage of normalised fields (x/(dx*ds), t/dt, E/E0,
//          direction), binary32 E0, FP32 arithmetic in registers
//
// Loads expand a stored particle into arithmetic-type registers; stores round
// back.  The expansion formulas are the ones the oracle uses, so FP16 state
// round-trips identically on both sides.
#pragma once
#include <cuda_fp16.h>
#include "imc_internal.h"

namespace imc {

struct StF64 {
    typedef double T;
    typedef double S;
    typedef double E0S;
    static constexpr int prec = 0;
    static constexpr bool half = false;
};
struct StF32 {
    typedef float T;
    typedef float S;
    typedef float E0S;
    static constexpr int prec = 1;
    static constexpr bool half = false;
};
struct StF16 {
    typedef float T;
    typedef __half S;
    typedef float E0S;
    static constexpr int prec = 2;
    static constexpr bool half = true;
};

template <class St> struct PBuf {
    typedef typename St::S S;
    typedef typename St::E0S E0S;
    S *t, *x, *y, *ux, *uy, *E;
    E0S *E0;
    int32_t *cs;
    uint8_t *alive;
    __host__ __device__ explicit PBuf(const PBufRaw &r)
        : t((S *)r.t), x((S *)r.x), y((S *)r.y), ux((S *)r.ux), uy((S *)r.uy), E((S *)r.E), E0((E0S *)r.E0),
          cs(r.cs), alive(r.alive) {}
    __host__ __device__ explicit PBuf(const PBufRaw1D &r)
        : t((S *)r.t), x((S *)r.x), y(nullptr), ux((S *)r.ux), uy(nullptr), E((S *)r.E), E0((E0S *)r.E0),
          cs(r.cs), alive(r.alive) {}
};

template <class S> __device__ __forceinline__ float ld_f(const S *p) { return (float)*p; }
template <> __device__ __forceinline__ float ld_f<__half>(const __half *p) { return __half2float(*p); }

// store helpers: round a T value into storage type S
template <class S, class T> __device__ __forceinline__ void st_v(S *p, T v) { *p = (S)v; }
template <> __device__ __forceinline__ void st_v<__half, float>(__half *p, float v) { *p = __float2half_rn(v); }

}  // namespace imc
