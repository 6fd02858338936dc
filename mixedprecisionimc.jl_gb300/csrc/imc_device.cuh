// imc_device.cuh -- device-side building blocks of the IMC engine (sm_103a).
//
//  * Philox-4x32-10 (Salmon et al., SC'11) keyed (SEED, step, particle index,
//    stage): every history draws its own reproducible stream, independent of
//    which thread runs it.
//  * Julia-semantics helpers used by the restated reference arithmetic
//    (NaN-propagating min, isless ordering for the sorter).
//  * Utilities.sorter (src/imc_utilities.jl:23-54) as a device function.
//  * Exact fixed-point tally accumulation: a non-negative double v is scaled by
//    2^-b (b fixed per step and tally) and rounded to a 96-bit integer split in
//    three 32-bit limbs, each added to its own 64-bit accumulator.  Integer
//    addition is associative, so the tally does not depend on the order in
//    which histories finish: GPU runs are bit-reproducible run to run.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_fp16.h>

#ifndef IMC_HD
#define IMC_HD __host__ __device__ __forceinline__
#endif

namespace imc {

// ------------------------------------------------------------------ Philox
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

// stream stage tags: transport, sourcing; the surrogate transport gives each
// resumed analog pass and each query pass of round r its own stream
enum : uint32_t { kStageTransport = 0, kStageSource = 1, kStageResume = 16, kStageQuery = 32 };

IMC_HD void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                           uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        uint32_t lo0 = kPhiloxM0 * c0, hi0 = __umulhi(kPhiloxM0, c0);
        uint32_t lo1 = kPhiloxM1 * c2, hi1 = __umulhi(kPhiloxM1, c2);
#else
        uint64_t p0 = (uint64_t)kPhiloxM0 * c0, p1 = (uint64_t)kPhiloxM1 * c2;
        uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += kPhiloxW0; k1 += kPhiloxW1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// One history's stream: counter {block, step, pid, stage}, key = SEED.
struct Stream {
    uint32_t k0, k1, step, pid, stage, block;
    uint32_t buf[4];
    int idx;
    IMC_HD void init(uint64_t seed, uint32_t step_, uint32_t pid_, uint32_t stage_) {
        k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
        step = step_; pid = pid_; stage = stage_; block = 0; idx = 4;
    }
    IMC_HD uint32_t next() {
        if (idx == 4) {
            philox4x32_10(block, step, pid, stage, k0, k1, buf);
            block += 1u;
            idx = 0;
        }
        // buf is indexed dynamically; keep it in registers via a select chain
        uint32_t v = idx == 0 ? buf[0] : idx == 1 ? buf[1] : idx == 2 ? buf[2] : buf[3];
        ++idx;
        return v;
    }
};

// uniform [0,1) and exponential variates, per arithmetic type
template <class T> struct Rand;
template <> struct Rand<float> {
    static IMC_HD float u(Stream &s) { return (float)(s.next() >> 8) * 0x1p-24f; }
    // v = odd multiple of 2^-24 on (0,1): -log(v) is never 0 (so 0/0 cannot
    // arise when the effective scatter opacity rounds to 0) and never inf
    static IMC_HD float exp1(Stream &s) {
        float v = (float)((s.next() >> 8) | 1u) * 0x1p-24f;
        return -logf(v);
    }
};
template <> struct Rand<double> {
    static IMC_HD double u(Stream &s) {
        uint64_t hi = s.next(), lo = s.next();
        return (double)(((hi << 32) | lo) >> 11) * 0x1p-53;
    }
    static IMC_HD double exp1(Stream &s) {
        uint64_t hi = s.next(), lo = s.next();
        double v = (double)((((hi << 32) | lo) >> 11) | 1u) * 0x1p-53;
        return -log(v);
    }
};

// The reference's Float64 angle 2 pi rand rounded to binary32, for the 24-bit
// uniforms of Rand<float>::u (u = m 2^-24, m = the stream word >> 8):
// RN32(RN64(2 pi_64 u)) = fma(m, hi, RN32(m lo)) 2^-24, where hi + lo is
// 2 pi_64 split into binary32 (hi = RN32(2 pi_64), lo = RN32(2 pi_64 - hi)).
// No FP64 operation; equal for every m < 2^24 (exhaustive host check in
// tests/test_device_header.py).
IMC_HD float two_pi_u24(uint32_t m) {
    const float mf = (float)m;
    return fmaf(mf, 0x1.921fb6p+2f, mf * -0x1.777a5cp-23f) * 0x1p-24f;
}

// The reference's Float64 angles -pi rand and pi (1/2 - rand) of the 2D
// surface births, rounded to binary32, for the 24-bit uniforms u = m 2^-24:
// each is pi_64 n 2^-24 for an integer n (1/2 - u = (2^23 - m) 2^-24 exactly
// in binary64), and RN32(RN64(pi_64 n 2^-24)) = fma(n, hi, RN32(n lo)) 2^-24
// with hi + lo the binary32 split of pi_64 for every |n| <= 2^24 (n itself
// exact in binary32; exhaustive host check in tests/test_device_header.py).
// pi (1/2 + rand) reaches n = 2^24 + 2^23, beyond that, and keeps its FP64
// product.
IMC_HD float pi_n24(int n) {
    const float nf = (float)n;
    return fmaf(nf, 0x1.921fb6p+1f, nf * -0x1.777a5cp-24f) * 0x1p-24f;
}

// The reference's cut-off energy 0.01 E0, a Float64 product, rounded to the
// arithmetic type.  Binary32 without FP64 where the cut-off is a normal
// number: with hi + lo the binary32 split of 0.01_64 (hi = RN32(0.01_64), lo
// = RN32(0.01_64 - hi)), RN32(RN64(0.01_64 E0)) = fma(E0, hi, RN32(E0 lo))
// for E0 >= 2^-114, and the same of E0 2^64, times 2^-64, for 0x1.9p-120 <=
// E0 < 2^-114.  Smaller E0 (a subnormal cut-off), negative and NaN take the
// FP64 product in a call kept out of line, so the common path holds no FP64
// registers.  The whole function equals the FP64 form for every
// non-negative binary32 and infinity (host check in
// tests/test_device_header.py).
static __host__ __device__ __noinline__ float cutoff_energy_fp64(float e0) { return (float)(0.01 * (double)e0); }
IMC_HD float cutoff_energy(float e0) {
    const bool tiny = e0 < 0x1p-114f;
    const float xs = tiny ? e0 * 0x1p64f : e0;
    const float y = fmaf(xs, 0x1.47ae14p-7f, xs * 0x1.eb851ep-33f);
    if (!(e0 >= 0x1.9p-120f)) return cutoff_energy_fp64(e0);
    return tiny ? y * 0x1p-64f : y;
}
IMC_HD double cutoff_energy(double e0) { return 0.01 * e0; }

// ------------------------------------------------------- Julia semantics
template <class T> IMC_HD T jmin(T a, T b) {
    if (a != a) return a;
    if (b != b) return b;
    return b < a ? b : a;
}
IMC_HD bool jisless(double a, double b) {
    bool an = a != a, bn = b != b;
    if (an || bn) return !an && bn;
    if (a < b) return true;
    if (a == b) return signbit(a) && !signbit(b);
    return false;
}

// precision tags for the sorter's scale choice
template <int P> struct SelType;
template <> struct SelType<0> { typedef double T; };
template <> struct SelType<1> { typedef float T; };

IMC_HD bool sel_finite_half(float v) {
    // binary16 overflow threshold: 65520 rounds to +inf
    return v == v && fabsf(v) < 65520.0f;
}

// Julia's isless order on Float64 as an unsigned integer key: -Inf < ... <
// -0.0 < +0.0 < ... < +Inf < NaN, every NaN equal (the sign-magnitude bits
// flipped into a two's-complement-free order).  Sorting by the key is sorting
// with jisless, with integer compares instead of FP64 ones (1/64 rate).
IMC_HD uint64_t isless_key(double v) {
    uint64_t b;
#ifdef __CUDA_ARCH__
    b = (uint64_t)__double_as_longlong(v);
#else
    memcpy(&b, &v, 8);
#endif
    if (v != v) return ~0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
IMC_HD double isless_value(uint64_t k) {
    uint64_t b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;  // NaN key -> a NaN
    double v;
#ifdef __CUDA_ARCH__
    v = __longlong_as_double((long long)b);
#else
    memcpy(&v, &b, 8);
#endif
    return v;
}

// Utilities.sorter (src/imc_utilities.jl:23-54): append scale j, sort
// ascending, multiply smallest by largest pairwise; the first scale whose
// product is finite in the selection precision wins.  Returns the FP64
// product; *jout = -1 if no scale works.  N values (compile time).
//
// The sort is a stable adjacent-swap insertion sort, unrolled over the
// compile-time size so the keys stay in registers.  Values that compare
// equal under isless have equal bits, except NaNs, whose products are never
// finite, so the product is the reference's in every case.
template <int SEL, int N>
IMC_HD double sorter_n(const double *vals, const double *scales, int nsc, int *jout) {
    constexpr int m = N + 1;
    uint64_t base[N];
#pragma unroll
    for (int i = 0; i < N; ++i) base[i] = isless_key(vals[i]);
    for (int j = 0; j < nsc; ++j) {
        uint64_t k[m];
#pragma unroll
        for (int i = 0; i < N; ++i) k[i] = base[i];
        k[N] = isless_key(scales[j]);
#pragma unroll
        for (int i = 1; i < m; ++i) {
#pragma unroll
            for (int q = i - 1; q >= 0; --q) {
                const uint64_t a = k[q], b = k[q + 1];
                const bool sw = b < a;
                k[q] = sw ? b : a;
                k[q + 1] = sw ? a : b;
            }
        }
        double arr[m];
#pragma unroll
        for (int i = 0; i < m; ++i) arr[i] = isless_value(k[i]);
        double prod = 1.0;
        bool ok;
        if (SEL == 2) {
            // binary16 evaluation: products of two binary16 values are exact
            // in binary32, so one rounding to binary16 per step reproduces
            // native half arithmetic.
            float ph = 1.0f;
#pragma unroll
            for (int i = 0; i < m / 2; ++i) {
                prod *= arr[i] * arr[m - 1 - i];
                float a = __half2float(__double2half(arr[i])), b = __half2float(__double2half(arr[m - 1 - i]));
                float pair = __half2float(__float2half_rn(a * b));
                ph = __half2float(__float2half_rn(ph * pair));
            }
            if (m & 1) {
                prod *= arr[m / 2];
                float a = __half2float(__double2half(arr[m / 2]));
                ph = __half2float(__float2half_rn(ph * a));
            }
            ok = sel_finite_half(ph);
        } else if (SEL == 1) {
            float pf = 1.0f;
#pragma unroll
            for (int i = 0; i < m / 2; ++i) {
                prod *= arr[i] * arr[m - 1 - i];
                pf = pf * ((float)arr[i] * (float)arr[m - 1 - i]);
            }
            if (m & 1) {
                prod *= arr[m / 2];
                pf = pf * (float)arr[m / 2];
            }
            ok = isfinite(pf);
        } else {
#pragma unroll
            for (int i = 0; i < m / 2; ++i) prod *= arr[i] * arr[m - 1 - i];
            if (m & 1) prod *= arr[m / 2];
            ok = true;
        }
        if (ok && isfinite(prod)) {
            *jout = j;
            return prod;
        }
    }
    *jout = -1;
    return 0.0;
}

// the same with the number of values at run time (host checks); n <= 15
template <int SEL>
IMC_HD double sorter(const double *vals, int n, const double *scales, int nsc, int *jout) {
    switch (n) {
    case 1: return sorter_n<SEL, 1>(vals, scales, nsc, jout);
    case 2: return sorter_n<SEL, 2>(vals, scales, nsc, jout);
    case 3: return sorter_n<SEL, 3>(vals, scales, nsc, jout);
    case 4: return sorter_n<SEL, 4>(vals, scales, nsc, jout);
    case 5: return sorter_n<SEL, 5>(vals, scales, nsc, jout);
    case 6: return sorter_n<SEL, 6>(vals, scales, nsc, jout);
    case 7: return sorter_n<SEL, 7>(vals, scales, nsc, jout);
    case 8: return sorter_n<SEL, 8>(vals, scales, nsc, jout);
    case 9: return sorter_n<SEL, 9>(vals, scales, nsc, jout);
    case 10: return sorter_n<SEL, 10>(vals, scales, nsc, jout);
    case 11: return sorter_n<SEL, 11>(vals, scales, nsc, jout);
    case 12: return sorter_n<SEL, 12>(vals, scales, nsc, jout);
    case 13: return sorter_n<SEL, 13>(vals, scales, nsc, jout);
    case 14: return sorter_n<SEL, 14>(vals, scales, nsc, jout);
    case 15: return sorter_n<SEL, 15>(vals, scales, nsc, jout);
    default: *jout = -1; return 0.0;
    }
}

// ------------------------------------------------- fixed-point tallies
// Signed 3-limb fixed point: V = round_half_up(v * 2^-b) with |V| < 2^94,
// limbs of weight 2^64, 2^32 and 1 held in separate int64 accumulators.  Each
// accumulator holds the exact signed sum of its limbs (|sum| < n * 2^32 for n
// additions, far below 2^63), so the recombined total is exact whatever the
// order of additions.  The conversion is pure integer arithmetic: no FP64 on
// the FP32 hot path.
struct Limbs { long long l0, l1, l2; };

IMC_HD uint32_t f2u(float v) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(v);
#else
    uint32_t u; memcpy(&u, &v, 4); return u;
#endif
}
IMC_HD uint64_t d2u(double v) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t u; memcpy(&u, &v, 8); return u;
#endif
}
IMC_HD int bitlen64(uint64_t m) {
#ifdef __CUDA_ARCH__
    return 64 - __clzll((long long)m);
#else
    return m ? 64 - __builtin_clzll(m) : 0;
#endif
}

// man * 2^sh (man < 2^53), rounded half-up, signed; false if |V| >= 2^94
IMC_HD bool fix_place(uint64_t man, int sh, bool neg, Limbs &o) {
    uint64_t lo = 0, hi = 0;
    if (man == 0) { o.l0 = o.l1 = o.l2 = 0; return true; }
    if (sh >= 0) {
        if (bitlen64(man) + sh > 94) return false;
        if (sh == 0) { lo = man; hi = 0; }
        else if (sh < 64) { lo = man << sh; hi = man >> (64 - sh); }
        else { lo = 0; hi = man << (sh - 64); }
    } else {
        int r = -sh;
        if (r >= 60) { lo = 0; }
        else { lo = (man + (1ull << (r - 1))) >> r; }
        hi = 0;
    }
    long long l2 = (long long)(lo & 0xFFFFFFFFull);
    long long l1 = (long long)(lo >> 32);
    long long l0 = (long long)hi;
    if (neg) { l0 = -l0; l1 = -l1; l2 = -l2; }
    o.l0 = l0; o.l1 = l1; o.l2 = l2;
    return true;
}

IMC_HD int bitlen32(uint32_t m) {
#ifdef __CUDA_ARCH__
    return 32 - __clz((int)m);
#else
    return m ? 32 - __builtin_clz(m) : 0;
#endif
}

// FP32 values: the 24-bit mantissa lands in at most two of the three 32-bit
// words, placed with 32-bit shifts (the same result as fix_place).
IMC_HD bool fix_split(float v, int b, Limbs &o) {
    uint32_t bits = f2u(v);
    bool neg = (bits >> 31) != 0;
    int ex = (int)((bits >> 23) & 0xFFu);
    if (ex == 0xFF) return false;
    uint32_t man = bits & 0x7FFFFFu;
    int e2;
    if (ex == 0) e2 = 1 - 127 - 23;
    else { man |= 0x800000u; e2 = ex - 127 - 23; }
    const int sh = e2 - b;
    if (sh < 0 || man == 0) return fix_place(man, sh, neg, o);
    if (bitlen32(man) + sh > 94) return false;
    const int w = sh >> 5, off = sh & 31;
    const uint32_t lo = man << off;
    const uint32_t hi = off ? man >> (32 - off) : 0u;
    uint32_t w0 = 0u, w1 = 0u, w2 = 0u;  // bits 0-31, 32-63, 64-95
    if (w == 0) { w0 = lo; w1 = hi; }
    else if (w == 1) { w1 = lo; w2 = hi; }
    else { w2 = lo; }
    long long l2 = (long long)w0, l1 = (long long)w1, l0 = (long long)w2;
    if (neg) { l0 = -l0; l1 = -l1; l2 = -l2; }
    o.l0 = l0; o.l1 = l1; o.l2 = l2;
    return true;
}
// The same placement for a positive normal FP32 value, as two 32-bit words:
// bits [32j, 32j + 32) of the fixed-point value get lo, the next word hi (0
// when j == 2).  False where fix_split would round (below the resolution),
// fail (above the range, not finite) or negate; the shared-memory tally
// flush takes this path and leaves the rest to fix_split.
IMC_HD bool f32_words(float v, int b, int &j, uint32_t &lo, uint32_t &hi) {
    const uint32_t bits = f2u(v);
    const int ex = (int)(bits >> 23);  // the sign bit makes it >= 256
    if (ex == 0 || ex >= 255) return false;
    const int sh = ex - 150 - b;  // exponent of the mantissa's lowest bit, relative to b
    if (sh < 0 || sh > 94 - 24) return false;
    const uint32_t man = (bits & 0x7FFFFFu) | 0x800000u;
    j = sh >> 5;
    const int off = sh & 31;
    lo = man << off;
    hi = off ? man >> (32 - off) : 0u;
    return true;
}
IMC_HD bool fix_split(double v, int b, Limbs &o) {
    uint64_t bits = d2u(v);
    bool neg = (bits >> 63) != 0;
    int ex = (int)((bits >> 52) & 0x7FFu);
    if (ex == 0x7FF) return false;
    uint64_t man = bits & 0xFFFFFFFFFFFFFull;
    int e2;
    if (ex == 0) e2 = 1 - 1023 - 52;
    else { man |= 0x10000000000000ull; e2 = ex - 1023 - 52; }
    return fix_place(man, e2 - b, neg, o);
}

// Energy scales and the tally exponents.  A particle of scale k carries
// E = e_true * scale_k; each tally slot of scale k holds its values times
// 2^-scale_exp(scale_k), i.e. within a factor two of true energies, so one
// exponent per tally (set from the largest true energy) fits every scale --
// scale lists that span more than the fixed point's 2^93 (the binary32
// fallback of the sorter) lose nothing.  The tallies' exponent of scale k is
// that base plus scale_exp(scale_k); exact powers of two throughout.
IMC_HD int scale_exp(double s) {
    const int e = (int)((d2u(s) >> 52) & 0x7FFu);
    return e == 0 ? -1023 : e - 1023;  // ilogb of a normal scale
}
// an upper bound of ilogb(v) for v > 0: exact for normal v
IMC_HD int exp_bound(float v) {
    const int e = (int)((f2u(v) >> 23) & 0xFFu);
    return e == 0 ? -127 : e - 127;
}
IMC_HD int exp_bound(double v) {
    const int e = (int)((d2u(v) >> 52) & 0x7FFu);
    return e == 0 ? -1023 : e - 1023;
}
// no census particle (emax_census_exp of an empty census)
constexpr int kNoExp = -100000;
// the largest double whose ilogb is e (every value of that exponent is <= it)
IMC_HD double exp_top(int e) {
#ifdef __CUDA_ARCH__
    return ldexp(1.9999999999999998, e);
#else
    return std::ldexp(1.9999999999999998, e);
#endif
}

// Exponent b with every |v| <= vmax mapping below 2^93 (one spare bit for a
// value a rounding step above vmax, one for the compensation term).
IMC_HD int fix_exponent(double vmax) {
    if (!(vmax > 0.0) || !(vmax < 1.0e308)) return -1074;
    int e = ilogb(vmax);
    return e + 1 - 93;
}

// signed total of accumulator words a[0..2] times 2^b
IMC_HD double fix_value(const long long *a, int b) {
    uint64_t hi = (uint64_t)a[0], lo = 0;
    // + a1 * 2^32 (sign-extended)
    uint64_t lo1 = (uint64_t)a[1] << 32;
    uint64_t hi1 = (uint64_t)(a[1] >> 32);
    lo += lo1;
    hi += hi1 + (lo < lo1 ? 1ull : 0ull);
    // + a2 (sign-extended)
    uint64_t lo2 = (uint64_t)a[2];
    uint64_t hi2 = a[2] < 0 ? ~0ull : 0ull;
    uint64_t plo = lo;
    lo += lo2;
    hi += hi2 + (lo < plo ? 1ull : 0ull);
    double v = (double)(long long)hi * 0x1p64 + (double)lo;
    return scalbn(v, b);
}

// ------------------------------------------------ double-double summation
// no constructor, so arrays of DD may live in __shared__ memory
struct DD {
    double hi, lo;
    IMC_HD void clear() { hi = 0.0; lo = 0.0; }
    IMC_HD void add(double x) {
        double s = hi + x;
        double bp = s - hi;
        double e = (hi - (s - bp)) + (x - bp);
        hi = s;
        lo += e;
    }
    IMC_HD void add(const DD &o) {
        add(o.hi);
        lo += o.lo;
    }
    IMC_HD double val() const { return hi + lo; }
};

}  // namespace imc
