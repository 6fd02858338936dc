// imc_transport.cuh -- device helpers shared by the transport kernels
// (imc_transport.cu, imc_transport_surr.cu): math overloads of the particle
// type, Neumaier accumulation, exact fixed-point tally flushes into global or
// block-shared accumulators, the per-cell table and the end-of-kernel
// counter reduction.
#pragma once
#include <cstdint>
#include "imc_device.cuh"
#include "imc_internal.h"
#include "imc_state.cuh"

namespace imc {

__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_expm1(float x) { return expm1f(x); }
__device__ __forceinline__ double m_expm1(double x) { return expm1(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ void m_sincos(float a, float *s, float *c) { sincosf(a, s, c); }
__device__ __forceinline__ void m_sincos(double a, double *s, double *c) { sincos(a, s, c); }

// Neumaier compensated add; all deposit terms are non-negative.
template <class T> __device__ __forceinline__ void nadd(T &s, T &c, T x) {
    T t = s + x;
    if (s >= x) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// Limb adds into global memory (64-bit integer reductions in L2) or into the
// block's private copy of the tally in shared memory.
template <bool SMT> __device__ __forceinline__ void add_limbs(long long *a, const Limbs &L) {
    if (SMT) {
        // the pointer is known to address shared memory
        unsigned long long *s = (unsigned long long *)a;
        if (L.l0) atomicAdd_block(s + 0, (unsigned long long)L.l0);
        if (L.l1) atomicAdd_block(s + 1, (unsigned long long)L.l1);
        if (L.l2) atomicAdd_block(s + 2, (unsigned long long)L.l2);
    } else {
        if (L.l0) atomicAdd((unsigned long long *)(a + 0), (unsigned long long)L.l0);
        if (L.l1) atomicAdd((unsigned long long *)(a + 1), (unsigned long long)L.l1);
        if (L.l2) atomicAdd((unsigned long long *)(a + 2), (unsigned long long)L.l2);
    }
}

// bytes of the per-cell transport table at the start of dynamic shared memory
__host__ __device__ __forceinline__ int table_bytes(const CellArgs &ca, int tsz) {
    int b = ca.geometry == 1 ? 4 * tsz * ca.nx : 2 * tsz * (ca.nc + ca.nx + ca.ny);
    return (b + 15) & ~15;
}

__device__ __forceinline__ long long *tally_smem(unsigned char *smem, int table) {
    return reinterpret_cast<long long *>(smem + table);
}

// Adds the block's shared tallies (deposition, then census energy, in the
// same 3-limb layout as the global accumulators) to the global ones.
__device__ __forceinline__ void flush_block_tallies(const CellArgs &ca, const long long *sm) {
    __syncthreads();
    const int n = 3 * ca.K * ca.nc;
    for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
        long long v = sm[i];
        if (v) atomicAdd((unsigned long long *)((i < n ? ca.dep_acc : ca.rad_acc) + (i < n ? i : i - n)),
                         (unsigned long long)v);
    }
}

// flush a compensated pair: the Neumaier result s + c, converted once
template <class T, bool SMT>
__device__ __forceinline__ void flush_pair(long long *acc, int slot, T s, T c, int b, unsigned &flags) {
    const T v = s + c;
    if (v == (T)0) return;
    Limbs A;
    if (!fix_split(v, b, A)) {
        flags |= (v != v) ? 1u /*NAN*/ : (1u << 5) /*FIXPOINT_RANGE*/;
        return;
    }
    add_limbs<SMT>(acc + 3 * (size_t)slot, A);
}

template <class T, bool SMT>
__device__ __forceinline__ void flush_one(long long *acc, int slot, T v, int b, unsigned &flags) {
    if (v == (T)0) return;
    Limbs A;
    if (!fix_split(v, b, A)) {
        flags |= (v != v) ? 1u : (1u << 5);
        return;
    }
    add_limbs<SMT>(acc + 3 * (size_t)slot, A);
}

template <class T> struct Tab1 { T saf, seff, dxs, dxT; };
template <class T> struct Tab2 { T saf, seff; };
template <class T> struct Face { T ws, wT; };  // width * distancescale, width

// end-of-kernel reduction of per-thread counters: one atomic per warp
template <class T>
__device__ __forceinline__ void finish_counters(Scalars *sc, unsigned long long segs, unsigned flags, T emax) {
    const unsigned full = 0xFFFFFFFFu;
    double em = (double)emax;
    for (int off = 16; off > 0; off >>= 1) {
        segs += __shfl_down_sync(full, segs, off);
        flags |= __shfl_down_sync(full, flags, off);
        double o = __shfl_down_sync(full, em, off);
        em = o > em ? o : em;
    }
    if ((threadIdx.x & 31) == 0) {
        if (segs) atomicAdd(&sc->segments, segs);
        if (flags) atomicOr(&sc->flags, flags);
        if (em > 0.0) atomicMax(&sc->emax_census_bits, (unsigned long long)d2u(em));
    }
}

}  // namespace imc
