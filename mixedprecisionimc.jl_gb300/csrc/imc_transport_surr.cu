// imc_transport_surr.cu -- 1D transport (Transport.MC, src/imc_transport.jl:
// 13-210) with the learned thick-cell surrogate of imc_surrogate.cuh.
//
// Outside the surrogate's domain every segment is the analog one of
// k_transport1d (same event logic, same tallies).  A history in a cell at
// least kCellMin mean free paths wide, with at least kLmaxMin mean free paths
// of path left before census or the 1 % energy cut-off, and whose walk would
// take at least kMinGain collisions (min(lmax, 1.5 d_n d_f)), instead asks the
// network where its walk inside this cell ends: through the near face,
// through the far face, or at the cut (census position and direction, or the
// cut-off kill).  Energy follows exactly from the sampled path l:
// E -> E exp(-sigma_a f l), the difference deposited in the cell, as the
// analog segments would deposit it.  A history that cannot reach either face
// before the cut-off kills it is killed at once, without the network (exact).
//
// Wavefront layout.  The network runs as a warp-collective BF16 m16n8k16
// tensor-core pass over 16 queries, which wants 16 queries ready at once;
// analog segments want every lane walking its own history.  So a step runs
// as separate passes (all launched on the stream, replayed in the step's
// CUDA graph):
//   list pass              the 1D transport kernel (imc_transport.cu) in its
//                          list mode: a history that wants a query flushes
//                          its deposits and is set aside in the `ask` queue
//   k_wave_query (round r) every queued history gets one query, 32 per warp
//                          (two MMA passes of 16 rows, all lanes sampling);
//                          census, kill and escape finish the history,
//                          face exits and 1e4-path pieces continue in the
//                          `resume` queue
//   resume pass            the 1D transport kernel over the resume queue,
//                          which may set histories aside again, except in
//                          the last of kSurrRounds rounds
// A resumed history draws from its own Philox stream per round (stage tags
// kStageResume + r, kStageQuery + r), so results do not depend on the order
// of the queues, which atomics fill; tallies are exact fixed-point sums.
#include <cstdint>
#include "imc_surrogate.cuh"
#include "imc_transport.cuh"

namespace imc {
namespace {

using namespace imc::surr;

constexpr int kQueryWarps = 8;
constexpr int kQueryBlock = 32 * kQueryWarps;
constexpr unsigned kFull = 0xFFFFFFFFu;
// query pass shared memory: network image | per-warp staging | cell table
constexpr int kQueryHead = kImageBytes + kQueryWarps * kStageFloats * 4;
static_assert(kQueryHead % 16 == 0, "16-byte aligned sections");

// per-lane history state
template <class T> struct Hist {
    long long i;
    int cell, k, cs;
    T t, x, mu, E, E0, minenergy;
    T acc_s, acc_c;
    int acc_cell;
    long long seg;
    Stream rs;
};

// census: write the state back (src/imc_transport.jl:185-193) and tally it
// (b_rad: the census tally's exponent of this history's scale, se that
// scale's scale_exp)
template <class St, class T, bool SMT>
__device__ __forceinline__ void census(PBuf<St> &pb, const Tab1<T> *tab, Hist<T> &h, long long *rad_acc, int nc,
                                       int b_rad, int se, unsigned &flags, int &emax_e) {
    const long long i = h.i;
    T Est = h.E;
    if (St::half) {
        st_v(pb.t + i, 0.0f);
        st_v(pb.x + i, (float)h.x / (float)tab[h.cell].dxs);
        st_v(pb.ux + i, (float)h.mu);
        __half ef = __float2half_rn((float)h.E / (float)h.E0);
        pb.E[i] = ef;
        Est = __half2float(ef) * (float)h.E0;
    } else {
        pb.t[i] = (typename St::S)0;
        pb.x[i] = (typename St::S)h.x;
        pb.ux[i] = (typename St::S)h.mu;
        pb.E[i] = (typename St::S)h.E;
    }
    if (h.cell != (h.cs & 0xFFFFFF)) pb.cs[i] = h.cell | (h.k << 24);
    flush_one<T, SMT>(rad_acc, h.k * nc + h.cell, Est, b_rad, flags);
    const int ee = exp_bound(Est) - se;
    emax_e = ee > emax_e ? ee : emax_e;
}

// Face crossing after a segment that ended on a face, in the reference's
// order (src/imc_transport.jl:130-169): mu > 0 moves right (or reflects /
// escapes at the right boundary), then mu < 0 moves left.  Returns false if
// the history escaped (its energy tallied as lost).
template <class T>
__device__ __forceinline__ bool cross_face(const CellArgs &ca, const Tab1<T> *tab, Hist<T> &h, int N,
                                           bool reflect_l, bool reflect_r, int b_lost, unsigned &flags) {
    if (h.mu > (T)0) {
        if (h.cell == N - 1) {
            if (reflect_r) {
                h.mu = -h.mu;
            } else {
                flush_one<T, false>(ca.lost_acc, h.k, h.E, b_lost, flags);
                return false;
            }
        }
        h.cell += 1;
        h.x = (T)0;
    }
    if (h.mu < (T)0) {
        if (h.cell == 0) {
            if (reflect_l) {
                h.mu = -h.mu;
            } else {
                flush_one<T, false>(ca.lost_acc, h.k, h.E, b_lost, flags);
                return false;
            }
        } else {
            h.cell -= 1;
            h.x = tab[h.cell].dxs;
        }
    }
    return true;
}

enum { kGo = 0, kKilled = 1, kCensus = 2, kPaused = 3 };

template <class T>
__device__ __forceinline__ int decide(const Tab1<T> &ce, const Hist<T> &h, T c, T ds, T dt, Query &q) {
    return surr_decide<T>(ce, h.x, h.mu, h.t, h.E, h.minenergy, c, ds, dt, q);
}

// applies a sampled outcome (cls, y0, y1) of the walk described by q
template <class T>
__device__ __forceinline__ int apply_outcome(const CellArgs &ca, const Tab1<T> *tab, Hist<T> &h, const Query &q,
                                             int cls, float y0, float y1, T c, T ds, bool ds_one, T dt, long long cap,
                                             int N, bool reflect_l, bool reflect_r, int b_lost, unsigned &flags) {
    if (++h.seg > cap) { flags |= (1u << 2); return kKilled; }
    const Tab1<T> ce = tab[h.cell];
    if (cls == kTrunc && q.cut) {
        nadd(h.acc_s, h.acc_c, SegMath<T>::all_in(h.E, ce));
        return kKilled;
    }
    const float seff = (float)ce.seff;
    T dist, xn, mun;
    bool face = false;
    if (cls == kTrunc) {
        const float pos = fminf(fmaxf(q.dn + y0 * sqrtf(q.L), 0.0f), q.W);  // from the near face
        const float xm = q.near_left ? pos : q.W - pos;
        xn = (T)(xm / seff);
        xn = xn < (T)0 ? (T)0 : (xn > ce.dxs ? ce.dxs : xn);
        float mp = fminf(fmaxf(y1, -1.0f), 1.0f);
        if (mp == 0.0f) mp = 1.0f;
        mun = (T)(q.near_left ? mp : -mp);
        dist = q.census ? c * (dt - h.t) * ds : (T)(q.L / seff);
    } else {
        const bool far = cls == kFar;
        const float l = fminf(fmaxf(q.L * expf(y0), far ? q.df : q.dn), q.L);
        const float ma = fminf(fmaxf(y1, 1.0e-3f), 1.0f);
        const bool right = q.near_left == far;
        xn = right ? ce.dxs : (T)0;
        mun = (T)(right ? ma : -ma);
        dist = (T)(l / seff);
        face = true;
    }
    T dep;
    const T newenergy = SegMath<T>::attenuate(h.E, ce, dist, &dep);
    if (newenergy <= h.minenergy) {
        nadd(h.acc_s, h.acc_c, SegMath<T>::all_in(h.E, ce));
        return kKilled;
    }
    nadd(h.acc_s, h.acc_c, dep);
    h.t += (ds_one ? dist : dist / ds) / c;
    if (h.t > dt) h.t = dt;
    h.E = newenergy;
    h.x = xn;
    h.mu = mun;
    if (face) return cross_face<T>(ca, tab, h, N, reflect_l, reflect_r, b_lost, flags) ? kGo : kKilled;
    return q.census ? kCensus : kGo;
}


// --------------------------------------------------------------- queues
template <class T>
__device__ __forceinline__ void store_queued(const SurrQueue &qq, unsigned long long j, const Hist<T> &h) {
    qq.x[j] = (float)h.x;
    qq.mu[j] = (float)h.mu;
    qq.t[j] = (float)h.t;
    qq.E[j] = (float)h.E;
    qq.E0[j] = (float)h.E0;
    qq.cs[j] = h.cell | (h.k << 24);
    qq.cs_list[j] = h.cs;
    qq.idx[j] = h.i;
}

template <class T>
__device__ __forceinline__ void load_queued(const SurrQueue &qq, long long e, unsigned long long seed, unsigned step,
                                            uint32_t stage, Hist<T> &h) {
    h.i = qq.idx[e];
    const int cs = qq.cs[e];
    h.cs = qq.cs_list[e];
    h.cell = cs & 0xFFFFFF;
    h.k = cs >> 24;
    h.E0 = (T)qq.E0[e];
    h.x = (T)qq.x[e];
    h.mu = (T)qq.mu[e];
    h.t = (T)qq.t[e];
    h.E = (T)qq.E[e];
    h.rs.init(seed, step, (uint32_t)h.i, stage);
    h.minenergy = cutoff_energy(h.E0);  // (T)(0.01 * (double)E0)
    h.acc_s = (T)0;
    h.acc_c = (T)0;
    h.acc_cell = h.cell;
    h.seg = 0;
}

template <class T>
__device__ __forceinline__ void fill_table(const CellArgs &ca, Tab1<T> *tab, T ds) {
    for (int i = threadIdx.x; i < ca.nx; i += blockDim.x) tab[i] = make_tab1<T>(ca.sa[i], ca.fleck[i], ca.ss[i], ca.dx[i], ds);
}

// ------------------------------------------------------------- query pass
// One network query for every history of the ask queue of round `round`:
// 32 histories per warp, two tensor-core passes of 16 rows, all lanes
// sampling.  Census, kill and escape end the history; face exits and
// 1e4-path pieces continue in the resume queue.
template <class St>
__global__ void __launch_bounds__(kQueryBlock, 2) k_wave_query(CellArgs ca, Scalars *sc, PBufPair bufs, SurrWave w,
                                                               int round) {
    typedef float T;
    // the resume pass after this one takes its queue chunks from the work
    // counter, which the pass before this one has finished using
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->work_next = 0ull;
    const long long n = (long long)sc->qcount[2 * round];
    if (n == 0) return;
    PBuf<St> pb(bufs.b[sc->cur]);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t *frag = reinterpret_cast<const uint32_t *>(smem_raw);
    const float *bias = reinterpret_cast<const float *>(smem_raw + kFragWords * 4);
    float *stage_all = reinterpret_cast<float *>(smem_raw + kImageBytes);
    Tab1<T> *tab = reinterpret_cast<Tab1<T> *>(smem_raw + kQueryHead);
    const int N = ca.nx, nc = ca.nc;
    const T ds = (T)ca.ds, c = (T)ca.c;
    const bool ds_one = ds == (T)1;
    {
        uint4 *dst = reinterpret_cast<uint4 *>(smem_raw);
        for (int v = threadIdx.x; v < kImageBytes / 16; v += blockDim.x) dst[v] = ca.surr_image[v];
        for (int v = threadIdx.x; v < kQueryWarps * kStageFloats; v += blockDim.x) stage_all[v] = 0.0f;
    }
    fill_table<T>(ca, tab, ds);
    __shared__ int s_sexp[16];
    load_scale_exps(ca, s_sexp);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    float *xin = stage_all + warp * kStageFloats;
    float *yout = xin + 16 * kIn;
    const T dt = (T)sc->dt;
    unsigned long long *resume_count = &sc->qcount[2 * round + 1];
    const uint32_t stage = kStageQuery + (uint32_t)round;
    const int b_dep = sc->b_dep, b_rad = sc->b_rad, b_lost = sc->b_lost;
    const unsigned step = sc->step;
    const unsigned long long seed = ca.seed;
    const long long cap = ca.seg_cap;
    const bool reflect_r = ca.bc[1] == 1, reflect_l = ca.bc[0] == 1;
    unsigned long long calls = 0, killed = 0;
    unsigned flags = 0;
    int emax_e = kNoExp;
    const long long wstride = (long long)gridDim.x * kQueryWarps * 32;
    for (long long base = ((long long)blockIdx.x * kQueryWarps + warp) * 32; base < n; base += wstride) {
        const long long e = base + lane;
        const bool valid = e < n;
        Hist<T> h;
        Query q;
        int kind = kAnalog;
        if (valid) {
            load_queued<T>(w.ask, e, seed, step, stage, h);
            kind = decide<T>(tab[h.cell], h, c, ds, dt, q);  // the state the history was set aside with
        }
        int cls = kTrunc;
        float y0 = 0.0f, y1 = 0.0f;
        for (int half = 0; half < 2; ++half) {
            const bool mine = (lane >> 4) == half;
            if (mine) {
                float f[kIn] = {0.0f, 0.0f, 0.0f, 0.0f};
                if (valid && kind == kAsk) features(q.dn, q.df, q.mup, q.L, f);
                for (int j = 0; j < kIn; ++j) xin[(lane & 15) * kIn + j] = f[j];
            }
            __syncwarp();
            forward16(frag, bias, xin, yout);
            if (mine && valid && kind == kAsk) {
                const float u0 = Rand<float>::u(h.rs), u1 = Rand<float>::u(h.rs), u2 = Rand<float>::u(h.rs);
                cls = sample_outcome(yout + (lane & 15) * kOut, u0, u1, u2, &y0, &y1);
            }
            __syncwarp();
        }
        int res = kGo;
        if (valid) {
            if (kind == kAsk) {
                res = apply_outcome<T>(ca, tab, h, q, cls, y0, y1, c, ds, ds_one, dt, cap, N, reflect_l, reflect_r,
                                       b_lost + s_sexp[h.k], flags);
                calls += 1;
            } else if (kind == kCertainKill) {
                nadd(h.acc_s, h.acc_c, SegMath<T>::all_in(h.E, tab[h.cell]));
                calls += 1;
                res = kKilled;
            }
            const int se = s_sexp[h.k];
            flush_pair<T, false>(ca.dep_acc, h.k * nc + h.acc_cell, h.acc_s, h.acc_c, b_dep + se, flags);
            if (res == kCensus) census<St, T, false>(pb, tab, h, ca.rad_acc, nc, b_rad + se, se, flags, emax_e);
            else if (res == kKilled) {
                pb.alive[h.i] = 0;
                ++killed;
            }
        }
        // continuing histories go to the resume queue, one atomic per warp
        const bool go = valid && res == kGo;
        const unsigned m = __ballot_sync(kFull, go);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long b0 = 0;
            if (lane == leader) b0 = atomicAdd(resume_count, (unsigned long long)__popc(m));
            b0 = __shfl_sync(kFull, b0, leader);
            if (go) store_queued<T>(w.resume, b0 + __popc(m & lt), h);
        }
    }
    for (int off = 16; off > 0; off >>= 1) calls += __shfl_down_sync(kFull, calls, off);
    if (lane == 0 && calls) atomicAdd(&sc->surrogate_calls, calls);
    finish_counters(sc, 0ull, killed, flags, emax_e);
}

// BF16 fragment image of FP32 parameters (one block)
__global__ void k_surr_image(const float *P, uint4 *dst) {
    __shared__ __align__(16) unsigned char img[kImageBytes];
    uint32_t *frag = reinterpret_cast<uint32_t *>(img);
    float *bias = reinterpret_cast<float *>(img + kFragWords * 4);
    build_image(P, frag, bias);
    __syncthreads();
    const uint4 *src = reinterpret_cast<const uint4 *>(img);
    for (int v = threadIdx.x; v < kImageBytes / 16; v += blockDim.x) dst[v] = src[v];
}

template <class St>
void launch_wave(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, const SurrWave &w, const SurrShapes &sh,
                 cudaStream_t st) {
    launch_surr_analog(ca, sc, prec, bufs, w, 0, 0, sh.analog_grid, sh.analog_smem, st);
    for (int r = 0; r < kSurrRounds; ++r) {
        k_wave_query<St><<<sh.query_grid, kQueryBlock, sh.query_smem, st>>>(ca, sc, bufs, w, r);
        launch_surr_analog(ca, sc, prec, bufs, w, r + 1 < kSurrRounds ? 1 : 2, r, sh.analog_grid, sh.analog_smem, st);
    }
}

}  // namespace

SurrShapes surr_shapes(const CellArgs &ca, int prec) {
    SurrShapes s{};
    const TransportShape ts = transport_shape(ca, prec);
    s.analog_block = ts.block;
    s.analog_smem = surr_analog_smem(ca, prec);
    s.analog_smt = ts.smem_tally;
    s.query_block = kQueryBlock;
    s.query_smem = kQueryHead + table_bytes(ca, 4);
    return s;
}

const void *surr_kernel_ptr(const CellArgs &ca, int prec, int which) {
    if (which == 3) return prec == 2 ? (const void *)k_wave_query<StF16> : (const void *)k_wave_query<StF32>;
    return surr_analog_ptr(ca, prec, which);
}

void launch_transport_surr(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, const SurrWave &w,
                           const SurrShapes &sh, cudaStream_t st) {
    if (prec == 2) launch_wave<StF16>(ca, sc, prec, bufs, w, sh, st);
    else launch_wave<StF32>(ca, sc, prec, bufs, w, sh, st);
}

void launch_surr_image(const float *params, void *dst, cudaStream_t st) {
    k_surr_image<<<1, 256, 0, st>>>(params, reinterpret_cast<uint4 *>(dst));
}

}  // namespace imc
