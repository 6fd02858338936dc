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
#include "imc_surrogate.cuh"

namespace imc {

__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_expm1(float x) { return expm1f(x); }
__device__ __forceinline__ double m_expm1(double x) { return expm1(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ void m_sincos(float a, float *s, float *c) { sincosf(a, s, c); }
__device__ __forceinline__ void m_sincos(double a, double *s, double *c) { sincos(a, s, c); }

// e^x - 1 in the FP32 segment arithmetic: for |x| <= 1/16 the Taylor series
// to x^7 in Horner form with fused multiply-adds (the dropped terms are below
// 1e-13 of the result; rounding within about one ulp), else expm1f.  Segments
// of sigma_a f d below 1/16 -- every segment of the slab decks -- take the
// series.  The oracle's FP32 path evaluates the same expression.
__device__ __forceinline__ float expm1_seg(float x) {
    if (fabsf(x) <= 0.0625f) {
        float p = fmaf(x, 1.0f / 5040.0f, 1.0f / 720.0f);
        p = fmaf(p, x, 1.0f / 120.0f);
        p = fmaf(p, x, 1.0f / 24.0f);
        p = fmaf(p, x, 1.0f / 6.0f);
        p = fmaf(p, x, 0.5f);
        return fmaf(p * x, x, x);
    }
    return expm1f(x);
}

// Neumaier compensated add; all deposit terms are non-negative.
template <class T> __device__ __forceinline__ void nadd(T &s, T &c, T x) {
    T t = s + x;
    if (s >= x) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// Limb adds into global memory (64-bit integer reductions in L2) or into the
// block's private copy of the tally in shared memory.
//
// A shared-memory slot is six 32-bit words: the running sums of the three
// limb positions (w[0..2], same order as Limbs l0..l2, wrapping modulo 2^32)
// and their signed carry counts (cy[0..2]).  Each limb is added with a native
// 32-bit shared atomic; the returned old sum shows whether the add wrapped,
// and only then the carry count is bumped (a negative limb l is added as
// 2^32 + l with a carry of -1).  flush_block_tallies folds the carries into
// the next limb up.  Exact for any order of adds, like the 64-bit form, at
// the cost of a 32-bit atomic instead of a 64-bit one (which shared memory
// does not add natively).  The carry counts stay below 2^31 in magnitude
// while a block adds fewer than 2^31 limbs to one slot in one launch.
__device__ __forceinline__ void add_word_smem(unsigned *w, int *cy, long long l) {
    const unsigned u = (unsigned)l;
    const unsigned old = atomicAdd_block(w, u);
    const int c = (old + u < old ? 1 : 0) - (l < 0 ? 1 : 0);
    if (c) atomicAdd_block(cy, c);
}

// A positive FP32 value into a shared slot, without the signed three-limb
// split: its 24-bit mantissa occupies at most two adjacent 32-bit words of the
// 96-bit fixed-point value (f32_words), so at most two word adds (slot word
// 2 - j holds bits 32j..32j+31, as in add_limbs).  The same integers as
// fix_split + add_limbs<true>, so the same sums.  False (nothing added) for a
// value the general path must handle (see f32_words).
__device__ __forceinline__ void add_word_u(unsigned *w, int *cy, unsigned u) {
    const unsigned old = atomicAdd_block(w, u);
    if (old + u < old) atomicAdd_block(cy, 1);
}
__device__ __forceinline__ bool add_f32_smem(long long *slot, float v, int b) {
    int j;
    uint32_t lo, hi;
    if (!f32_words(v, b, j, lo, hi)) return false;
    unsigned *w = reinterpret_cast<unsigned *>(slot);
    int *cy = reinterpret_cast<int *>(slot) + 3;
    if (lo) add_word_u(w + 2 - j, cy + 2 - j, lo);
    if (hi) add_word_u(w + 1 - j, cy + 1 - j, hi);
    return true;
}

template <bool SMT> __device__ __forceinline__ void add_limbs(long long *a, const Limbs &L) {
    if (SMT) {
        // the pointer is known to address shared memory
        unsigned *w = reinterpret_cast<unsigned *>(a);
        int *cy = reinterpret_cast<int *>(a) + 3;
        if (L.l0) add_word_smem(w + 0, cy + 0, L.l0);
        if (L.l1) add_word_smem(w + 1, cy + 1, L.l1);
        if (L.l2) add_word_smem(w + 2, cy + 2, L.l2);
    } else {
        // Warp-aggregated: the lanes flushing to the same slot at this moment
        // add their limbs in registers (integer sums, exact in any order) and
        // one of them sends the reduction to L2.
        const unsigned active = __activemask();
        const unsigned peers = __match_any_sync(active, (unsigned long long)a);
        const int lane = threadIdx.x & 31;
        long long s0 = L.l0, s1 = L.l1, s2 = L.l2;
        if (peers != (1u << lane)) {
            const int rank = __popc(peers & ((1u << lane) - 1u));
            const int n = __popc(peers);
            for (int off = 1; off < n; off <<= 1) {
                const int pr = rank + off;
                const int src = pr < n ? (int)__fns(peers, 0u, pr + 1) : lane;
                const long long o0 = __shfl_sync(peers, s0, src);
                const long long o1 = __shfl_sync(peers, s1, src);
                const long long o2 = __shfl_sync(peers, s2, src);
                if ((rank & (2 * off - 1)) == 0 && pr < n) { s0 += o0; s1 += o1; s2 += o2; }
            }
            if (rank != 0) return;
        }
        if (s0) atomicAdd((unsigned long long *)(a + 0), (unsigned long long)s0);
        if (s1) atomicAdd((unsigned long long *)(a + 1), (unsigned long long)s1);
        if (s2) atomicAdd((unsigned long long *)(a + 2), (unsigned long long)s2);
    }
}

// bytes of the per-cell transport table at the start of dynamic shared memory
// (1D: one 32-byte Tab1 per cell for either type)
__host__ __device__ __forceinline__ int table_bytes(const CellArgs &ca, int tsz) {
    // 1D: 32-byte Tab1 rows; 2D: 16-byte Tab2 rows, then x and y Face rows
    int b = ca.geometry == 1 ? 32 * ca.nx : 16 * ca.nc + 2 * tsz * (ca.nx + ca.ny);
    return (b + 15) & ~15;
}
__host__ __device__ __forceinline__ int table_bytes(const Deck1DArgs &ca, int) { return (32 * ca.nx + 15) & ~15; }

__device__ __forceinline__ long long *tally_smem(unsigned char *smem, int table) {
    return reinterpret_cast<long long *>(smem + table);
}

// Adds the block's shared tallies (deposition, then census energy, in the
// same 3-limb layout as the global accumulators) to the global ones: limb
// q of a slot gets its word sum plus the carries out of the limb below it.
// with_rad false: the block holds only the deposition tallies.
template <class CA>
__device__ __forceinline__ void flush_block_tallies(const CA &ca, const long long *sm, bool with_rad) {
    __syncthreads();
    const int n = ca.K * ca.nc;
    for (int i = threadIdx.x; i < (with_rad ? 2 * n : n); i += blockDim.x) {
        const unsigned *w = reinterpret_cast<const unsigned *>(sm + 3 * (size_t)i);
        const int *cy = reinterpret_cast<const int *>(w + 3);
        long long *g = (i < n ? ca.dep_acc : ca.rad_acc) + 3 * (size_t)(i < n ? i : i - n);
        const long long v0 = (long long)w[0] + (long long)cy[1] + (long long)cy[0] * 4294967296ll;
        const long long v1 = (long long)w[1] + (long long)cy[2];
        const long long v2 = (long long)w[2];
        if (v0) atomicAdd((unsigned long long *)(g + 0), (unsigned long long)v0);
        if (v1) atomicAdd((unsigned long long *)(g + 1), (unsigned long long)v1);
        if (v2) atomicAdd((unsigned long long *)(g + 2), (unsigned long long)v2);
    }
}

// flush a compensated pair: the Neumaier result s + c, converted once
template <class T, bool SMT>
__device__ __forceinline__ void flush_pair(long long *acc, int slot, T s, T c, int b, unsigned &flags) {
    const T v = s + c;
    if (v == (T)0) return;
    if constexpr (SMT && sizeof(T) == 4)
        if (add_f32_smem(acc + 3 * (size_t)slot, v, b)) return;
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
    if constexpr (SMT && sizeof(T) == 4)
        if (add_f32_smem(acc + 3 * (size_t)slot, v, b)) return;
    Limbs A;
    if (!fix_split(v, b, A)) {
        flags |= (v != v) ? 1u : (1u << 5);
        return;
    }
    add_limbs<SMT>(acc + 3 * (size_t)slot, A);
}

// Work split of the transport over the particle list (or a resume pass's
// queue): warps take chunks in order from a counter (Scalars::work_next,
// zeroed before each transport and by each query pass) -- kListChunk1D- or
// kListChunk-entry chunks in the short-history schedule of the 1D and 2D
// kernels, 32-entry chunks in the refill schedule -- so the blocks (one per
// SM) run out of work together.  Measured against a fixed grid stride over 7/8
// of the list with the rest from the counter: the same on the slab (+0.7 %),
// 29 % faster transport on the 2D channel, whose history costs vary along the
// list.  256-entry chunks: 1.7 % faster 1D transport on the slab than 128,
// 2-4 % slower 2D transport on the channel.
constexpr int kListChunk = 128;
constexpr int kListChunk1D = 256;
// the counter's next value for the warp (warp-uniform; every lane calls)
__device__ __forceinline__ long long warp_counter_next(unsigned long long *counter) {
    unsigned long long c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(counter, 1ull);
    return (long long)__shfl_sync(0xFFFFFFFFu, c, 0);
}

// where the transport kernels add their tallies
enum { kTallyGlobal = 0, kTallyShared = 1, kTallySharedDep = 2 };

// threads per block of the shared-tally transport kernels: FP32 / FP16 state
// and FP64 state (one block per SM: the table and the private tallies take
// most of the shared memory)
constexpr int kSmtBlock32 = 1024;
constexpr int kSmtBlock64 = 512;
// threads per block of the global-tally kernels (meshes whose private
// tallies do not fit): FP32 / FP16 state as one 1024-thread block per SM,
// FP64 in 256-thread blocks
constexpr int kGlbBlock32 = 1024;
constexpr int kGlbBlock64 = 256;

// 1D per-cell table: sigma_a f, effective scatter, width * distancescale,
// width; the FP32 table adds the reciprocals its arithmetic multiplies by
template <class T> struct Tab1;
template <> struct Tab1<double> { double saf, seff, dxs, dxT; };
template <> struct Tab1<float> { float saf, seff, dxs, dxT, rseff, rdxT, pad0, pad1; };
static_assert(sizeof(Tab1<double>) == 32 && sizeof(Tab1<float>) == 32, "32-byte table rows");

template <class T>
__device__ __forceinline__ Tab1<T> make_tab1(double sa, double f, double ss, double dx, T ds) {
    Tab1<T> e;
    const T saT = (T)sa, fT = (T)f, ssT = (T)ss;
    e.saf = saT * fT;
    e.seff = saT * ((T)1 - fT) + ssT;
    e.dxT = (T)dx;
    e.dxs = e.dxT * ds;
    if constexpr (sizeof(T) == 4) {
        e.rseff = 1.0f / e.seff;  // inf for a zero opacity: the flight is then inf, as seff/0 is
        e.rdxT = 1.0f / e.dxT;
        e.pad0 = e.pad1 = 0.0f;
    }
    return e;
}

// Segment arithmetic of Transport.MC (src/imc_transport.jl:84-123).  FP64
// evaluates the reference's expressions as written.  FP32 (and FP16 state)
// evaluates the same quantities with fewer instructions: the collision
// distance as -log(v) * (1/seff) with the hardware logarithm, the weight
// after the segment as E + E expm1(-sigma_a f d) -- one transcendental for
// both the attenuation and the deposit, so the two add up to E up to one
// rounding -- and reciprocals instead of divisions.
template <class T> struct SegMath;
template <> struct SegMath<double> {
    static __device__ __forceinline__ double flight(Stream &rs, const Tab1<double> &ce) {
        return Rand<double>::exp1(rs) / ce.seff;
    }
    // new weight; *dep = the deposit per unit width
    static __device__ __forceinline__ double attenuate(double E, const Tab1<double> &ce, double d, double *dep) {
        *dep = -(E / ce.dxT) * expm1(-ce.saf * d);
        return E * exp(-ce.saf * d);
    }
    static __device__ __forceinline__ double all_in(double E, const Tab1<double> &ce) { return E / ce.dxT; }
};
template <> struct SegMath<float> {
    static __device__ __forceinline__ float flight(Stream &rs, const Tab1<float> &ce) {
        const float v = (float)((rs.next() >> 8) | 1u) * 0x1p-24f;
        return -__logf(v) * ce.rseff;
    }
    static __device__ __forceinline__ float attenuate(float E, const Tab1<float> &ce, float d, float *dep) {
        const float em1 = expm1_seg(-ce.saf * d);
        *dep = -(E * ce.rdxT) * em1;
        return E + E * em1;
    }
    static __device__ __forceinline__ float all_in(float E, const Tab1<float> &ce) { return E * ce.rdxT; }
};
// 2D per-cell table: sigma_a f, effective scatter; FP32 adds 1/seff and the
// reciprocal cell area
template <class T> struct Tab2;
template <> struct Tab2<double> { double saf, seff; };
template <> struct Tab2<float> { float saf, seff, rseff, rarea; };
static_assert(sizeof(Tab2<double>) == 16 && sizeof(Tab2<float>) == 16, "16-byte table rows");
template <class T> struct Face { T ws, wT; };  // width * distancescale, width

// end-of-kernel reduction of per-thread counters: one atomic per warp
// (segments, histories removed from the list, error flags, and the census
// maximum as the exponent of its true energy, see scale_exp)
__device__ __forceinline__ void finish_counters(Scalars *sc, unsigned long long segs, unsigned long long killed,
                                                unsigned flags, int emax_e) {
    const unsigned full = 0xFFFFFFFFu;
    for (int off = 16; off > 0; off >>= 1) {
        segs += __shfl_down_sync(full, segs, off);
        killed += __shfl_down_sync(full, killed, off);
        flags |= __shfl_down_sync(full, flags, off);
        const int o = __shfl_down_sync(full, emax_e, off);
        emax_e = o > emax_e ? o : emax_e;
    }
    if ((threadIdx.x & 31) == 0) {
        if (segs) atomicAdd(&sc->segments, segs);
        if (killed) atomicAdd(&sc->killed, killed);
        if (flags) atomicOr(&sc->flags, flags);
        if (emax_e != kNoExp) atomicMax(&sc->emax_census_exp, emax_e);
    }
}

// the exponents scale_exp(scale_k) of the deck's energy scales, in shared
// memory (every thread calls; a barrier must follow before use)
template <class CA> __device__ __forceinline__ void load_scale_exps(const CA &ca, int *s_sexp) {
    for (int i = threadIdx.x; i < ca.K; i += blockDim.x) s_sexp[i] = scale_exp(ca.scales[i]);
}

// ------------------------------------------------ learned surrogate: when to ask
// The walk's state in mean free paths, for the network (imc_surrogate.cuh).
struct Query {
    float W, dn, df, mup, L;
    bool near_left;  // the nearer face is the left one
    bool cut;        // the 1 % energy cut-off ends the walk at L (truncation = kill)
    bool census;     // census ends the walk at L
};

enum { kAnalog = 0, kAsk = 1, kCertainKill = 2 };

// Whether a history at (x, mu, t, E) in a cell should walk analog, ask the
// network, or die here for certain (no face within reach before the cut-off).
template <class T>
__device__ __forceinline__ int surr_decide(const Tab1<T> &ce, T x, T mu, T t, T E, T minenergy, T c, T ds, T dt,
                                           Query &q) {
    using namespace surr;
    const float seff = (float)ce.seff;
    const float W = (float)ce.dxs * seff;
    if (!(W >= kCellMin)) return kAnalog;
    const float lcen = seff * (float)(c * (dt - t) * ds);
    const float lcut = ce.saf > (T)0 ? logf((float)E / (float)minenergy) * seff / (float)ce.saf : INFINITY;
    const float L = fminf(lcen, lcut);
    if (!(L >= kLmaxMin)) return kAnalog;
    const float xm = (float)x * seff;
    q.W = W;
    q.near_left = xm <= 0.5f * W;
    q.dn = fmaxf(q.near_left ? xm : W - xm, 0.0f);
    q.df = W - q.dn;
    q.mup = q.near_left ? (float)mu : -(float)mu;
    q.cut = lcut <= lcen && lcut <= kLmaxMax;
    q.census = !q.cut && lcen <= kLmaxMax;
    q.L = fminf(L, kLmaxMax);
    if (q.cut && q.dn >= q.L) return kCertainKill;
    return expected_collisions(q.dn, q.df, q.L) >= kMinGain ? kAsk : kAnalog;
}

// Per-cell gate of the analog passes: the least distance from the nearer
// face, in mean free paths, at which a history of this cell can want a query
// this step (infinity where none can: cell narrower than kCellMin mean free
// paths, or lmax below kMinGain even at the step's start with full energy).
// With lmax at most Lc = min(census path seff c dt ds, cut-off path
// ln(100) seff / (sigma_a f)), asking needs 1.95 d_n sqrt(Lc) >= kMinGain,
// so histories nearer the face than kMinGain / (1.95 sqrt(Lc)) skip the test.
template <class T>
__device__ __forceinline__ void fill_gate(const CellArgs &ca, float *gate, T ds, T c, T dt) {
    using namespace surr;
    for (int i = threadIdx.x; i < ca.nx; i += blockDim.x) {
        const float sa = (float)ca.sa[i], f = (float)ca.fleck[i], ss = (float)ca.ss[i];
        const float saf = sa * f, seff = sa * (1.0f - f) + ss;
        const float W = (float)ca.dx[i] * (float)ds * seff;
        const float lcen = seff * (float)(c * dt * ds);
        const float lcut = saf > 0.0f ? 4.6051702f * seff / saf : INFINITY;
        const float Lc = fminf(lcen, lcut);
        gate[i] = (W >= kCellMin && Lc >= kMinGain) ? kMinGain / (1.95f * sqrtf(Lc)) : INFINITY;
    }
}

// whether this thread's share of the filled gate holds an open cell
__device__ __forceinline__ bool gate_open(const CellArgs &ca, const float *gate) {
    bool open = false;
    for (int i = threadIdx.x; i < ca.nx; i += blockDim.x) open |= gate[i] < INFINITY;
    return open;
}

// shared-memory bytes of the 1D analog kernel: table, private tallies (SMT),
// and the per-cell gate when histories may be set aside for queries
template <class CA>
__host__ __device__ __forceinline__ int analog1d_smem(const CA &ca, int tsz, bool smt, bool gate) {
    return table_bytes(ca, tsz) + (smt ? 48 * ca.K * ca.nc : 0) + (gate ? ((4 * ca.nx + 15) & ~15) : 0);
}

}  // namespace imc
