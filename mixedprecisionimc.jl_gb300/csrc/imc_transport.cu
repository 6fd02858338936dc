// imc_transport.cu -- history-based particle transport, one thread per history.
//
//   k_transport1d <- Transport.MC   (src/imc_transport.jl:13-210)
//   k_transport2d <- Transport.MC2D (src/imc_transport.jl:483-732)
//
// A persistent grid walks the particle list in chunks of consecutive entries
// that warps take from a counter, so every warp loads 32 consecutive
// particles (coalesced structure-of-arrays loads) and the blocks run out of
// work together; a history stays in registers: each particle's state is read
// once and written once per step.  The per-cell transport table (sigma_a*f,
// effective scatter, face widths) is built in shared memory by every block.
//
// Tallies: a history accumulates its deposits for the cell it is in as a
// Neumaier-compensated pair in the arithmetic type, and flushes the pair when
// it leaves the cell or ends, as exact fixed-point limbs (imc_device.cuh) with
// 64-bit integer atomics.  Census energy and escaped energy are tallied the
// same way.  All tallies are therefore independent of scheduling.
//
// The event logic restates the reference line by line: distances to the face,
// to collision (randexp over the effective scatter opacity) and to census; the
// minimum wins; events are tested by float equality in the reference's
// if/if/if order, so ties run every matching branch, as they do there.
#include <cstdint>
#include "imc_transport.cuh"

namespace imc {

// segments per history at and above which the 1D kernel refills lanes
constexpr float kRefillSegments = 3.0f;

// 1D analog kernel modes: the plain transport, and the passes of the
// surrogate transport (imc_transport_surr.cu) -- the list pass and the resume
// passes set aside histories that want a network query; the last resume
// pass walks everything to its end.
enum { kModePlain = 0, kModeList = 1, kModeResume = 2, kModeResumeLast = 3 };

// The transport of one deck's list by one block (every thread calls; the
// block's dynamic shared memory at smem_raw).  TM: where the flushes go
// (kTallyGlobal, kTallyShared, or kTallySharedDep: deposition tallies shared,
// census tallies global; the plain pass only).  The block's shared tallies
// and counters are flushed to the deck's before it returns; the caller puts a
// barrier between two calls.
template <class St, int BLOCK, int TM, int MODE, class CA, class BP>
__device__ __forceinline__ void transport1d_block(const CA &ca, Scalars *sc, const BP &bufs, const SurrWave &w,
                                                  int round, unsigned char *smem_raw) {
    constexpr bool SMT = TM != kTallyGlobal;      // deposition flushes to shared memory
    constexpr bool RAD_SMT = TM == kTallyShared;  // census flushes to shared memory
    typedef typename St::T T;
    typedef SegMath<T> M;
    constexpr bool kFromQueue = MODE == kModeResume || MODE == kModeResumeLast;
    constexpr bool kPause = MODE == kModeList || MODE == kModeResume;
    const long long n = kFromQueue ? (long long)sc->qcount[2 * round + 1] : sc->n_particles;
    if (kFromQueue && n == 0) return;
    PBuf<St> pb(bufs.b[sc->cur]);
    Tab1<T> *tab = reinterpret_cast<Tab1<T> *>(smem_raw);
    const int N = ca.nx;
    const T ds = (T)ca.ds, c = (T)ca.c;
    const bool ds_one = ds == (T)1;
    const T rdsc = (T)1 / (ds * c);
    long long *dep_acc = ca.dep_acc, *rad_acc = ca.rad_acc;
    if (SMT) {
        dep_acc = tally_smem(smem_raw, table_bytes(ca, sizeof(T)));
        if (RAD_SMT) rad_acc = dep_acc + 3 * (size_t)ca.K * ca.nc;
        for (int i = threadIdx.x; i < (RAD_SMT ? 6 : 3) * ca.K * ca.nc; i += blockDim.x) dep_acc[i] = 0;
    }
    static_assert(TM != kTallySharedDep || MODE == kModePlain, "deposition-only tallies: plain pass only");
    const T endsteptime = (T)sc->dt;
    float *gate = reinterpret_cast<float *>(smem_raw + analog1d_smem(ca, sizeof(T), RAD_SMT, false));
    for (int i = threadIdx.x; i < N; i += blockDim.x) tab[i] = make_tab1<T>(ca.sa[i], ca.fleck[i], ca.ss[i], ca.dx[i], ds);
    __shared__ int s_sexp[16];
    load_scale_exps(ca, s_sexp);
    if constexpr (kPause) fill_gate<T>(ca, gate, ds, c, endsteptime);
    // the barrier after the table; with the gate, also whether any cell's
    // gate is open this step (each thread tests the entries it filled; every
    // block fills the whole gate, so all blocks agree): if none is, no
    // history is tested
    bool gating = false;
    if constexpr (kPause) gating = __syncthreads_or(gate_open(ca, gate)) && sc->surr_gate != 0;
    else __syncthreads();
    const int b_dep = sc->b_dep, b_rad = sc->b_rad, b_lost = sc->b_lost;
    const unsigned step = sc->step;
    const unsigned long long seed = ca.seed;
    const long long cap = ca.seg_cap;
    const int nc = ca.nc;
    const bool reflect_r = ca.bc[1] == 1, reflect_l = ca.bc[0] == 1;
    unsigned long long *ask_count = &sc->qcount[kFromQueue ? 2 * round + 2 : 0];
    const uint32_t stage = kFromQueue ? kStageResume + (uint32_t)round : kStageTransport;
    unsigned long long segs = 0, calls = 0, killed = 0;
    unsigned flags = 0;
    int emax_e = kNoExp;
    // Lane state of the history in flight (cs: as stored in the list; the
    // current cell and scale are cell, k).  Deposits go to the compensated
    // pair (acc_s, acc_c) of the current cell acc_cell; the pair of the cell
    // the history left last waits in (prv_s, prv_c, prv_cell) and is flushed
    // only when a third cell is entered, so a history that visits at most
    // two cells flushes both pairs at its end, with the warp converged.
    long long i = 0;
    int cs = 0, cell = 0, k = 0, acc_cell = 0, prv_cell = -1;
    T t = (T)0, x = (T)0, mu = (T)0, E = (T)0, E0 = (T)0, minenergy = (T)0, acc_s = (T)0, acc_c = (T)0, rmu = (T)0;
    T prv_s = (T)0, prv_c = (T)0;
    long long seg = 0;
    Stream rs;
    auto start = [&](int cs_now) {
        cell = cs_now & 0xFFFFFF;
        k = cs_now >> 24;
        rs.init(seed, step, (uint32_t)i, stage);
        minenergy = cutoff_energy(E0);  // (T)(0.01 * (double)E0), without FP64 in binary32
        acc_s = (T)0;
        acc_c = (T)0;
        acc_cell = cell;
        prv_cell = -1;
        seg = 0;
        rmu = (T)1 / mu;  // FP32: the face distance as a product (reset at each new direction)
    };
    // one entry of the list (or of the resume queue): false if it holds no history
    auto load = [&](long long e, int &cs_now, T &lt, T &lx, T &lmu, T &lE, T &lE0, long long &li, int &lcs) -> bool {
        if (kFromQueue) {
            li = w.resume.idx[e];
            lcs = w.resume.cs_list[e];
            cs_now = w.resume.cs[e];
            lt = (T)w.resume.t[e]; lx = (T)w.resume.x[e]; lmu = (T)w.resume.mu[e];
            lE = (T)w.resume.E[e]; lE0 = (T)w.resume.E0[e];
            return true;
        }
        if (!pb.alive[e]) return false;
        li = e;
        lcs = cs_now = pb.cs[e];
        lE0 = (T)pb.E0[e];
        if (St::half) {
            lt = ld_f(pb.t + e) * (float)endsteptime;
            lx = ld_f(pb.x + e) * (float)tab[cs_now & 0xFFFFFF].dxs;
            lmu = ld_f(pb.ux + e);
            lE = ld_f(pb.E + e) * (float)lE0;
        } else {
            lt = (T)pb.t[e]; lx = (T)pb.x[e]; lmu = (T)pb.ux[e]; lE = (T)pb.E[e];
        }
        return true;
    };
    // the history is in `cell`: on a cell change the current pair moves to
    // the waiting slot, whose earlier pair (a third cell) is flushed now
    auto enter_cell = [&]() {
        if (cell != acc_cell) {
            if (prv_cell >= 0) flush_pair<T, SMT>(dep_acc, k * nc + prv_cell, prv_s, prv_c, b_dep + s_sexp[k], flags);
            prv_cell = acc_cell; prv_s = acc_s; prv_c = acc_c;
            acc_s = (T)0; acc_c = (T)0; acc_cell = cell;
        }
    };
    // one pass of the reference's while loop; 0 = go on, 1 = killed, 2 =
    // census, 3 = set aside for a query (kPause), 4 = escaped through a
    // vacuum face.  The census write and the escape tally are left to
    // finish(), which the warp runs converged once per history.
    auto segment = [&]() -> int {
        if (gating && (float)(x < tab[cell].dxs - x ? x : tab[cell].dxs - x) * (float)tab[cell].seff >= gate[cell]) {
            Query q;
            const int kind = surr_decide<T>(tab[cell], x, mu, t, E, minenergy, c, ds, endsteptime, q);
            if (kind == kCertainKill) {
                enter_cell();
                nadd(acc_s, acc_c, M::all_in(E, tab[cell]));
                ++seg;
                ++calls;
                return 1;
            }
            if (kind == kAsk) return 3;
        }
        int end = 0;
        // one pass of the reference's while loop (src/imc_transport.jl:73-195)
        if (++seg > cap) {
            flags |= (1u << 2);
            end = 1;
        } else {
            const Tab1<T> ce = tab[cell];
            T dist_b;
            if constexpr (sizeof(T) == 4) dist_b = mu > (T)0 ? (ce.dxs - x) * rmu : m_abs(x * rmu);
            else dist_b = mu > (T)0 ? (ce.dxs - x) / mu : m_abs(x / mu);
            const T dist_col = M::flight(rs, ce);
            const T dist_cen = c * (endsteptime - t) * ds;
            const T dist = jmin(jmin(dist_b, dist_col), dist_cen);
            if (dist != dist) {
                flags |= 1u;
                end = 1;
            } else {
                T dep;
                const T newenergy = M::attenuate(E, ce, dist, &dep);
                enter_cell();
                if (newenergy <= minenergy) {
                    nadd(acc_s, acc_c, M::all_in(E, ce));
                    end = 1;
                } else {
                    nadd(acc_s, acc_c, dep);
                    x += mu * dist;
                    if constexpr (sizeof(T) == 4) t += dist * rdsc;
                    else t += (ds_one ? dist : dist / ds) / c;
                    E = newenergy;
                    if (dist == dist_b) {
                        if (mu > (T)0) {
                            if (cell == N - 1) {
                                if (reflect_r) {
                                    mu = -mu;
                                    rmu = -rmu;
                                } else {
                                    end = 4;
                                }
                            }
                            if (!end) {
                                cell += 1;
                                x = (T)0;
                            }
                        }
                        if (!end && mu < (T)0) {
                            if (cell == 0) {
                                if (reflect_l) {
                                    mu = -mu;
                                    rmu = -rmu;
                                } else {
                                    end = 4;
                                }
                            } else {
                                cell -= 1;
                                x = tab[cell].dxs;
                            }
                        }
                    }
                    if (!end && dist == dist_col) {
                        // mu = 1 - 2*rand, redrawn while zero (src/imc_transport.jl:178-181);
                        // a zero needs rand == 0.5 exactly, so 64 redraws never run out
                        mu = (T)0;
                        for (int r = 0; r < 64 && mu == (T)0; ++r) mu = (T)1 - (T)2 * Rand<T>::u(rs);
                        if (mu == (T)0) mu = (T)1;
                        rmu = (T)1 / mu;
                    }
                    // census: t = 0 and the state written back by finish()
                    // (src/imc_transport.jl:185-193)
                    if (!end && dist == dist_cen) end = 2;
                }
            }
        }
        return end;
    };
    auto finish = [&](int end) {
        const int se = s_sexp[k];
        if (prv_cell >= 0) flush_pair<T, SMT>(dep_acc, k * nc + prv_cell, prv_s, prv_c, b_dep + se, flags);
        flush_pair<T, SMT>(dep_acc, k * nc + acc_cell, acc_s, acc_c, b_dep + se, flags);
        if (end == 2) {
            // census: t = 0, write the state back (src/imc_transport.jl:185-193)
            T Est = E;
            if (St::half) {
                st_v(pb.t + i, 0.0f);
                st_v(pb.x + i, (float)x / (float)tab[cell].dxs);
                st_v(pb.ux + i, (float)mu);
                __half ef = __float2half_rn((float)E / (float)E0);
                pb.E[i] = ef;
                Est = __half2float(ef) * (float)E0;
            } else {
                pb.t[i] = (typename St::S)0;
                pb.x[i] = (typename St::S)x;
                pb.ux[i] = (typename St::S)mu;
                pb.E[i] = (typename St::S)E;
            }
            if (cell != (cs & 0xFFFFFF)) pb.cs[i] = cell | (k << 24);
            flush_one<T, RAD_SMT>(rad_acc, k * nc + cell, Est, b_rad + se, flags);
            const int ee = exp_bound(Est) - se;
            emax_e = ee > emax_e ? ee : emax_e;
        } else if (end == 3) {
            // set aside with its state for the query pass (its deposits flushed)
            const unsigned long long j = atomicAdd(ask_count, 1ull);
            w.ask.x[j] = (float)x; w.ask.mu[j] = (float)mu; w.ask.t[j] = (float)t; w.ask.E[j] = (float)E;
            w.ask.E0[j] = (float)E0; w.ask.cs[j] = cell | (k << 24); w.ask.cs_list[j] = cs; w.ask.idx[j] = i;
        } else {
            // killed, or escaped with E through a vacuum face
            if (end == 4) flush_one<T, false>(ca.lost_acc, k, E, b_lost + se, flags);
            pb.alive[i] = 0;
            ++killed;
        }
        segs += (unsigned long long)seg;
    };
    const int lane = threadIdx.x & 31;
    if (sc->seg_per_hist < kRefillSegments) {
        // Short histories (the last transport averaged fewer than
        // kRefillSegments segments each): each lane walks one history to its
        // end, and the warp moves on together to 32 consecutive entries, so
        // every load and store of the list is coalesced.
        auto walk = [&](long long e) {
            int cs_now;
            if (!load(e, cs_now, t, x, mu, E, E0, i, cs)) return;
            start(cs_now);
            int end;
            do end = segment(); while (!end);
            finish(end);
        };
        if constexpr (!kFromQueue && !St::half) {
            // the list in chunks from the counter; the next entry's fields
            // are loaded while the current history walks (FP32 / FP64 state:
            // their stored fields are the arithmetic values; measured on the
            // 2000-cell slab, 0.496 -> 0.474 ms per launch)
            typedef typename St::S S;
            typedef typename St::E0S E0S;
            uint8_t pa = 0;
            int pcs = 0;
            S pt = (S)0, px = (S)0, pmu = (S)0, pE = (S)0;
            E0S pE0 = (E0S)0;
            auto fetch = [&](long long e) {
                pa = e < n ? pb.alive[e] : (uint8_t)0;
                if (pa) { pcs = pb.cs[e]; pt = pb.t[e]; px = pb.x[e]; pmu = pb.ux[e]; pE = pb.E[e]; pE0 = pb.E0[e]; }
            };
            for (long long base = warp_counter_next(&sc->work_next) * kListChunk1D; base < n;
                 base = warp_counter_next(&sc->work_next) * kListChunk1D) {
                fetch(base + lane);
                for (int r = 0; r < kListChunk1D; r += 32) {
                    const long long e = base + r + lane;
                    const bool a = pa != 0;
                    const int ccs = pcs;
                    t = (T)pt; x = (T)px; mu = (T)pmu; E = (T)pE; E0 = (T)pE0;
                    if (r + 32 < kListChunk1D) fetch(e + 32);
                    if (a) {
                        i = e;
                        cs = ccs;
                        start(ccs);
                        int end;
                        do end = segment(); while (!end);
                        finish(end);
                    }
                }
            }
        } else {
            // the list (or a resume pass's queue) in chunks from the counter
            for (long long base = warp_counter_next(&sc->work_next) * kListChunk1D; base < n;
                 base = warp_counter_next(&sc->work_next) * kListChunk1D)
                for (int r = 0; r < kListChunk1D; r += 32)
                    if (base + r + lane < n) walk(base + r + lane);
        }
    } else {
        // Long histories of unequal length: each lane starts the next history
        // as soon as its current one ends.  The warp reads the entries in
        // chunks of 32 (coalesced: lane l prefetches entry 32 c + l into
        // registers); idle lanes take the chunk's entries in order through
        // register shuffles.
        const unsigned lt = (1u << lane) - 1u;
        const long long nchunks = (n + 31) / 32;
        // chunks of the list (or of a resume pass's queue) from the counter
        long long chunk = warp_counter_next(&sc->work_next);
        auto advance = [&]() { chunk = warp_counter_next(&sc->work_next); };
        int p_now = -1, p_cs = 0;  // prefetched entry (p_now -1: none / dead)
        long long p_i = 0;
        T p_t = (T)0, p_x = (T)0, p_mu = (T)0, p_E = (T)0, p_E0 = (T)0;
        auto prefetch = [&]() {
            const long long e = chunk * 32 + lane;
            p_now = -1;
            if (e < n) {
                int cn;
                if (load(e, cn, p_t, p_x, p_mu, p_E, p_E0, p_i, p_cs)) p_now = cn;
            }
        };
        bool more = chunk < nchunks;  // warp-uniform: the current chunk has entries left
        int pos = 0;                  // warp-uniform: next entry of the chunk to hand out
        if (more) prefetch();
        bool has = false;
        while (true) {
            unsigned idle = __ballot_sync(0xFFFFFFFFu, !has);
            while (idle && more) {
                const int r = __popc(idle & lt);
                const int avail = 32 - pos;
                const int sl = (pos + r) & 31;
                const int q_now = __shfl_sync(0xFFFFFFFFu, p_now, sl);
                const int q_cs = __shfl_sync(0xFFFFFFFFu, p_cs, sl);
                const long long q_i = __shfl_sync(0xFFFFFFFFu, p_i, sl);
                const T q_t = __shfl_sync(0xFFFFFFFFu, p_t, sl), q_x = __shfl_sync(0xFFFFFFFFu, p_x, sl);
                const T q_mu = __shfl_sync(0xFFFFFFFFu, p_mu, sl), q_E = __shfl_sync(0xFFFFFFFFu, p_E, sl);
                const T q_E0 = __shfl_sync(0xFFFFFFFFu, p_E0, sl);
                if (!has && r < avail && q_now >= 0) {
                    i = q_i;
                    cs = q_cs;
                    t = q_t; x = q_x; mu = q_mu; E = q_E; E0 = q_E0;
                    start(q_now);
                    has = true;
                }
                const int nidle = __popc(idle);
                pos += nidle < avail ? nidle : avail;
                if (pos >= 32) {
                    advance();
                    more = chunk < nchunks;
                    pos = 0;
                    if (more) prefetch();
                }
                idle = __ballot_sync(0xFFFFFFFFu, !has);
            }
            if (idle == 0xFFFFFFFFu) break;  // no history left for this warp
            if (!has) continue;
            const int end = segment();
            if (end) {
                finish(end);
                has = false;
            }
        }
    }
    if (SMT) flush_block_tallies(ca, dep_acc, RAD_SMT);
    if (kPause) {
        for (int off = 16; off > 0; off >>= 1) calls += __shfl_down_sync(0xFFFFFFFFu, calls, off);
        if (lane == 0 && calls) atomicAdd(&sc->surrogate_calls, calls);
    }
    finish_counters(sc, segs, killed, flags, emax_e);
}

template <class St, int BLOCK, int TM, int MODE>
__global__ void __launch_bounds__(BLOCK) k_transport1d(CellArgs ca, Scalars *sc, PBufPair bufs, SurrWave w,
                                                       int round) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    transport1d_block<St, BLOCK, TM, MODE>(ca, sc, bufs, w, round, smem_raw);
}

// One transport launch over the lists of many 1D decks (the fused batch,
// imc_run_batch_fused), whose arguments sit in constant memory.  Blocks go
// through the decks in order; a block sets up a deck (its cell table and
// private tallies) only while the deck's work counter still has chunks, takes
// chunks from that counter like the single-deck kernel, and flushes the
// deck's tallies and counters before it moves on.  Every history runs the
// single-deck code with the deck's own streams and exact tallies, so each
// deck's result is bit-identical to its own launch's.
__constant__ Deck1DArgs c_multi_ca[kFusedMaxDecks];
__constant__ PBufPair1D c_multi_bufs[kFusedMaxDecks];
__constant__ Scalars *c_multi_sc[kFusedMaxDecks];

template <class St, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_transport1d_multi(int ndecks) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_go;
    for (int d = 0; d < ndecks; ++d) {
        Scalars *sc = c_multi_sc[d];
        if (threadIdx.x == 0) {
            // chunks left: 128-entry chunks for short histories, 32-entry in
            // the refill schedule (a stale, low counter only costs a setup)
            const long long n = *(volatile long long *)&sc->n_particles;
            const unsigned long long used = *(volatile unsigned long long *)&sc->work_next;
            const long long per = *(volatile float *)&sc->seg_per_hist < kRefillSegments ? kListChunk1D : 32;
            s_go = (long long)used * per < n;
        }
        __syncthreads();
        if (s_go)
            transport1d_block<St, BLOCK, kTallyShared, kModePlain>(c_multi_ca[d], sc, c_multi_bufs[d], SurrWave{}, 0,
                                                                    smem_raw);
        __syncthreads();
    }
}

// TM, where the flushes go: kTallyGlobal, kTallyShared (deposition and
// census tallies block-private in shared memory) or kTallySharedDep (the
// deposition tallies only; census energy, one flush per census particle, to
// global memory)
template <class St, int BLOCK, int TM>
__global__ void __launch_bounds__(BLOCK) k_transport2d(CellArgs ca, Scalars *sc, PBufPair bufs) {
    constexpr bool SMT = TM != kTallyGlobal;        // deposition flushes to shared memory
    constexpr bool RAD_SMT = TM == kTallyShared;    // census flushes to shared memory
    typedef typename St::T T;
    PBuf<St> pb(bufs.b[sc->cur]);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int NX = ca.nx, NY = ca.ny, nc = ca.nc;
    Tab2<T> *tab = reinterpret_cast<Tab2<T> *>(smem_raw);
    Face<T> *fx = reinterpret_cast<Face<T> *>(tab + nc);
    Face<T> *fy = fx + NX;
    const T ds = (T)ca.ds, c = (T)ca.c;
    const bool ds_one = ds == (T)1;
    const T rdsc = (T)1 / (ds * c);
    long long *dep_acc = ca.dep_acc, *rad_acc = ca.rad_acc;
    if (SMT) {
        dep_acc = tally_smem(smem_raw, table_bytes(ca, sizeof(T)));
        if (RAD_SMT) rad_acc = dep_acc + 3 * (size_t)ca.K * ca.nc;
        for (int i = threadIdx.x; i < (RAD_SMT ? 6 : 3) * ca.K * ca.nc; i += blockDim.x) dep_acc[i] = 0;
    }
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        T sa = (T)ca.sa[i], f = (T)ca.fleck[i], ss = (T)ca.ss[i];
        Tab2<T> e;
        e.saf = sa * f;
        e.seff = sa * ((T)1 - f) + ss;
        if constexpr (sizeof(T) == 4) {
            e.rseff = 1.0f / e.seff;
            e.rarea = 1.0f / ((float)ca.dx[i % NX] * (float)ca.dy[i / NX]);
        }
        tab[i] = e;
    }
    for (int i = threadIdx.x; i < NX; i += blockDim.x) { fx[i].wT = (T)ca.dx[i]; fx[i].ws = fx[i].wT * ds; }
    for (int i = threadIdx.x; i < NY; i += blockDim.x) { fy[i].wT = (T)ca.dy[i]; fy[i].ws = fy[i].wT * ds; }
    __shared__ int s_sexp[16];
    load_scale_exps(ca, s_sexp);
    __syncthreads();
    const T dtT = (T)sc->dt;
    const long long n = sc->n_particles;
    const int b_dep = sc->b_dep, b_rad = sc->b_rad, b_lost = sc->b_lost;
    const unsigned step = sc->step;
    const unsigned long long seed = ca.seed;
    const long long cap = ca.seg_cap;
    const bool refl_l = ca.bc[0] == 1, refl_r = ca.bc[1] == 1, refl_t = ca.bc[2] == 1, refl_b = ca.bc[3] == 1;
    unsigned long long segs = 0, killed = 0;
    unsigned flags = 0;
    int emax_e = kNoExp;
    // Lane state of the history in flight.
    long long i = 0;
    int cs = 0, xi = 0, yi = 0, k = 0, acc_cell = 0;
    T t = (T)0, xp = (T)0, yp = (T)0, vx = (T)0, vy = (T)0, E = (T)0, E0 = (T)0, minenergy = (T)0;
    T acc_s = (T)0, acc_c = (T)0;
    long long seg = 0;
    Stream rs;
    auto start = [&]() {
        const int cell0 = cs & 0xFFFFFF;
        k = cs >> 24;
        xi = cell0 % NX;
        yi = cell0 / NX;
        rs.init(seed, step, (uint32_t)i, kStageTransport);
        minenergy = cutoff_energy(E0);  // (T)(0.01 * (double)E0), without FP64 in binary32
        acc_s = (T)0;
        acc_c = (T)0;
        acc_cell = cell0;
        seg = 0;
    };
    auto load = [&](long long e, int &lcs, T &lt, T &lx, T &ly, T &lvx, T &lvy, T &lE, T &lE0) -> bool {
        if (!pb.alive[e]) return false;
        lcs = pb.cs[e];
        const int c0 = lcs & 0xFFFFFF;
        lE0 = (T)pb.E0[e];
        if (St::half) {
            lt = ld_f(pb.t + e) * (float)dtT;
            lx = ld_f(pb.x + e) * (float)fx[c0 % NX].ws;
            ly = ld_f(pb.y + e) * (float)fy[c0 / NX].ws;
            lvx = ld_f(pb.ux + e);
            lvy = ld_f(pb.uy + e);
            lE = ld_f(pb.E + e) * (float)lE0;
        } else {
            lt = (T)pb.t[e]; lx = (T)pb.x[e]; ly = (T)pb.y[e];
            lvx = (T)pb.ux[e]; lvy = (T)pb.uy[e]; lE = (T)pb.E[e];
        }
        return true;
    };
    // one pass of the reference's while loop (src/imc_transport.jl:533-717);
    // 0 = go on, 1 = killed, 2 = census, 4 = escaped through a vacuum face.
    // The census write and the escape tally are left to finish(), which
    // the warp runs converged once per history.
    auto segment = [&]() -> int {
        if (++seg > cap) { flags |= (1u << 2); return 1; }
        const T dist_bx = vx > (T)0 ? m_abs((fx[xi].ws - xp) / vx) : m_abs(xp / vx);
        const T dist_by = vy > (T)0 ? m_abs((fy[yi].ws - yp) / vy) : m_abs(yp / vy);
        T dist_b;
        if (dist_bx != dist_bx) dist_b = dist_by;
        else if (dist_by != dist_by) dist_b = dist_bx;
        else dist_b = jmin(dist_bx, dist_by);
        const int cell = xi + yi * NX;
        const Tab2<T> ce = tab[cell];
        T dist_col, Edens, newenergy, dep;
        if constexpr (sizeof(T) == 4) {
            // FP32: the 1D kernels' formulation (SegMath<float>)
            const float v = (float)((rs.next() >> 8) | 1u) * 0x1p-24f;
            dist_col = -__logf(v) * ce.rseff;
        } else {
            dist_col = Rand<T>::exp1(rs) / ce.seff;
        }
        const T dist_cen = c * (dtT - t) * ds;
        const T dist = jmin(jmin(dist_b, dist_col), dist_cen);
        if (dist != dist) { flags |= 1u; return 1; }
        if constexpr (sizeof(T) == 4) {
            const float em1 = expm1_seg(-ce.saf * dist);
            newenergy = E + E * em1;
            Edens = E * ce.rarea;
            dep = -Edens * em1;
        } else {
            newenergy = E * m_exp(-ce.saf * dist);
            Edens = (E / fx[xi].wT) / fy[yi].wT;
            dep = -Edens * m_expm1(-ce.saf * dist);
        }
        if (cell != acc_cell) {
            flush_pair<T, SMT>(dep_acc, k * nc + acc_cell, acc_s, acc_c, b_dep + s_sexp[k], flags);
            acc_s = (T)0; acc_c = (T)0; acc_cell = cell;
        }
        if (newenergy <= minenergy) {
            nadd(acc_s, acc_c, Edens);
            return 1;
        }
        nadd(acc_s, acc_c, dep);
        xp += dist * vx;
        yp += dist * vy;
        if constexpr (sizeof(T) == 4) t += dist * rdsc;
        else t += (ds_one ? dist : dist / ds) / c;
        E = newenergy;
        if (dist == dist_bx || dist == dist_by) {
            if (dist_bx < dist_by) {
                if (vx > (T)0) {
                    if (xi == NX - 1) {
                        if (refl_r) { vx = -vx; return 0; }
                        return 4;
                    }
                    xi += 1; xp = (T)0;
                } else {
                    if (xi == 0) {
                        if (refl_l) { vx = -vx; return 0; }
                        return 4;
                    }
                    xi -= 1; xp = fx[xi].ws;
                }
            } else {
                if (vy > (T)0) {
                    if (yi == NY - 1) {
                        if (refl_t) { vy = -vy; return 0; }
                        return 4;
                    }
                    yi += 1; yp = (T)0;
                } else {
                    if (yi == 0) {
                        if (refl_b) { vy = -vy; return 0; }
                        return 4;
                    }
                    yi -= 1; yp = fy[yi].ws;
                }
            }
            return 0;
        }
        if (dist == dist_col) {
            // isotropic re-emission: angle 2*pi*rand in Float64, rounded to T
            // (binary32: two_pi_u24, the same value without FP64; the
            // hardware sine and cosine)
            T ang;
            if constexpr (sizeof(T) == 4) ang = two_pi_u24(rs.next() >> 8);
            else ang = (T)(6.283185307179586 * (double)Rand<T>::u(rs));
            if constexpr (sizeof(T) == 4) __sincosf(ang, &vy, &vx);
            else m_sincos(ang, &vy, &vx);
        }
        // census: t = 0 and the state written back by finish()
        if (dist == dist_cen) return 2;
        return 0;
    };
    auto finish = [&](int end) {
        flush_pair<T, SMT>(dep_acc, k * nc + acc_cell, acc_s, acc_c, b_dep + s_sexp[k], flags);
        if (end == 2) {
            // census: t = 0, write the state back (src/imc_transport.jl:700-717)
            const int cellf = xi + yi * NX;
            T Est = E;
            if (St::half) {
                st_v(pb.t + i, 0.0f);
                st_v(pb.x + i, (float)xp / (float)fx[xi].ws);
                st_v(pb.y + i, (float)yp / (float)fy[yi].ws);
                st_v(pb.ux + i, (float)vx);
                st_v(pb.uy + i, (float)vy);
                __half ef = __float2half_rn((float)E / (float)E0);
                pb.E[i] = ef;
                Est = __half2float(ef) * (float)E0;
            } else {
                pb.t[i] = (typename St::S)0;
                pb.x[i] = (typename St::S)xp;
                pb.y[i] = (typename St::S)yp;
                pb.ux[i] = (typename St::S)vx;
                pb.uy[i] = (typename St::S)vy;
                pb.E[i] = (typename St::S)E;
            }
            if (cellf != (cs & 0xFFFFFF)) pb.cs[i] = cellf | (k << 24);
            flush_one<T, RAD_SMT>(rad_acc, k * nc + cellf, Est, b_rad + s_sexp[k], flags);
            const int ee = exp_bound(Est) - s_sexp[k];
            emax_e = ee > emax_e ? ee : emax_e;
        } else {
            // killed, or escaped with E through a vacuum face
            if (end == 4) flush_one<T, false>(ca.lost_acc, k, E, b_lost + s_sexp[k], flags);
            pb.alive[i] = 0;
            ++killed;
        }
        segs += (unsigned long long)seg;
    };
    if (sc->seg_per_hist < kRefillSegments) {
        // short histories: one history per lane to its end (see k_transport1d)
        auto walk = [&](long long e) {
            if (!load(e, cs, t, xp, yp, vx, vy, E, E0)) return;
            i = e;
            start();
            int end;
            do end = segment(); while (!end);
            finish(end);
        };
        // the list in chunks from the counter
        const int lane = threadIdx.x & 31;
        for (long long base = warp_counter_next(&sc->work_next) * kListChunk; base < n;
             base = warp_counter_next(&sc->work_next) * kListChunk)
            for (int r = 0; r < kListChunk; r += 32)
                if (base + r + lane < n) walk(base + r + lane);
    } else {
        // long histories: lanes refill from 32-entry chunks (see k_transport1d)
        const int lane = threadIdx.x & 31;
        const unsigned lt = (1u << lane) - 1u;
        const long long nchunks = (n + 31) / 32;
        // chunks from the counter
        long long chunk = warp_counter_next(&sc->work_next);
        auto advance = [&]() { chunk = warp_counter_next(&sc->work_next); };
        int p_cs = -1;
        T p_t = (T)0, p_x = (T)0, p_y = (T)0, p_vx = (T)0, p_vy = (T)0, p_E = (T)0, p_E0 = (T)0;
        auto prefetch = [&]() {
            const long long e = chunk * 32 + lane;
            int lcs = -1;
            if (!(e < n && load(e, lcs, p_t, p_x, p_y, p_vx, p_vy, p_E, p_E0))) lcs = -1;
            p_cs = lcs;
        };
        bool more = chunk < nchunks;
        int pos = 0;
        if (more) prefetch();
        bool has = false;
        while (true) {
            unsigned idle = __ballot_sync(0xFFFFFFFFu, !has);
            while (idle && more) {
                const int r = __popc(idle & lt);
                const int avail = 32 - pos;
                const int sl = (pos + r) & 31;
                const int q_cs = __shfl_sync(0xFFFFFFFFu, p_cs, sl);
                const T q_t = __shfl_sync(0xFFFFFFFFu, p_t, sl), q_x = __shfl_sync(0xFFFFFFFFu, p_x, sl);
                const T q_y = __shfl_sync(0xFFFFFFFFu, p_y, sl), q_vx = __shfl_sync(0xFFFFFFFFu, p_vx, sl);
                const T q_vy = __shfl_sync(0xFFFFFFFFu, p_vy, sl), q_E = __shfl_sync(0xFFFFFFFFu, p_E, sl);
                const T q_E0 = __shfl_sync(0xFFFFFFFFu, p_E0, sl);
                if (!has && r < avail && q_cs >= 0) {
                    i = chunk * 32 + pos + r;
                    cs = q_cs;
                    t = q_t; xp = q_x; yp = q_y; vx = q_vx; vy = q_vy; E = q_E; E0 = q_E0;
                    start();
                    has = true;
                }
                const int nidle = __popc(idle);
                pos += nidle < avail ? nidle : avail;
                if (pos >= 32) {
                    advance();
                    more = chunk < nchunks;
                    pos = 0;
                    if (more) prefetch();
                }
                idle = __ballot_sync(0xFFFFFFFFu, !has);
            }
            if (idle == 0xFFFFFFFFu) break;
            if (!has) continue;
            const int end = segment();
            if (end) {
                finish(end);
                has = false;
            }
        }
    }
    if (SMT) flush_block_tallies(ca, dep_acc, RAD_SMT);
    finish_counters(sc, segs, killed, flags, emax_e);
}

// Launch shape of the transport kernel.  When the table and the block's
// private tallies fit in shared memory the kernel runs one large block per
// SM with shared tallies (kSmtBlock32 threads for FP32 / FP16 state,
// kSmtBlock64 for FP64).  When only the table and the deposition tallies fit
// in the opt-in maximum, the deposition tallies are shared and the census
// flushes (one per census particle) go to global memory (the analog passes
// of the surrogate transport then keep every tally global).
// Otherwise every flush goes to global memory (kGlbBlock32 / kGlbBlock64
// threads).
constexpr int kSmemBudget = 200 * 1024;
constexpr int kSmemOptInMax = 227 * 1024;  // sm_100-family dynamic shared memory per block

TransportShape transport_shape(const CellArgs &ca, int prec) {
    TransportShape sh;
    const int tsz = prec == 0 ? 8 : 4;
    const int table = table_bytes(ca, tsz);
    const long long dep = 3ll * 8 * (long long)ca.K * ca.nc;
    sh.smem_tally = table + 2 * dep <= kSmemBudget;
    sh.dep_only = !sh.smem_tally && table + dep <= kSmemOptInMax;
    sh.smem = table + (int)(sh.smem_tally ? 2 * dep : sh.dep_only ? dep : 0);
    const bool shared = sh.smem_tally || sh.dep_only;
    sh.block = shared ? (prec == 0 ? kSmtBlock64 : kSmtBlock32) : (prec == 0 ? kGlbBlock64 : kGlbBlock32);
    return sh;
}

// the plain 1D or 2D transport kernel of one state type, block size and
// tally mode
template <class St, int B, int TM> static const void *kptr(int geometry) {
    if (geometry == 1) return (const void *)k_transport1d<St, B, TM, kModePlain>;
    return (const void *)k_transport2d<St, B, TM>;
}

template <class St, int B, int TM>
static void launch_one(const CellArgs &ca, Scalars *sc, PBufPair buf, int grid, int smem, cudaStream_t st) {
    if (ca.geometry == 1) k_transport1d<St, B, TM, kModePlain><<<grid, B, smem, st>>>(ca, sc, buf, SurrWave{}, 0);
    else k_transport2d<St, B, TM><<<grid, B, smem, st>>>(ca, sc, buf);
}

template <class St> struct StBlocks {
    static constexpr int smt = sizeof(typename St::T) == 8 ? kSmtBlock64 : kSmtBlock32;
    static constexpr int glb = sizeof(typename St::T) == 8 ? kGlbBlock64 : kGlbBlock32;
};

template <class St> static const void *kernel_of(const CellArgs &ca, const TransportShape &sh) {
    if (sh.smem_tally) return kptr<St, StBlocks<St>::smt, kTallyShared>(ca.geometry);
    if (sh.dep_only) return kptr<St, StBlocks<St>::smt, kTallySharedDep>(ca.geometry);
    return kptr<St, StBlocks<St>::glb, kTallyGlobal>(ca.geometry);
}

template <class St>
static void launch_of(const CellArgs &ca, const TransportShape &sh, Scalars *sc, PBufPair buf, int grid,
                      cudaStream_t st) {
    if (sh.smem_tally) launch_one<St, StBlocks<St>::smt, kTallyShared>(ca, sc, buf, grid, sh.smem, st);
    else if (sh.dep_only) launch_one<St, StBlocks<St>::smt, kTallySharedDep>(ca, sc, buf, grid, sh.smem, st);
    else launch_one<St, StBlocks<St>::glb, kTallyGlobal>(ca, sc, buf, grid, sh.smem, st);
}

const void *transport_kernel_ptr(const CellArgs &ca, int prec) {
    TransportShape sh = transport_shape(ca, prec);
    if (prec == 0) return kernel_of<StF64>(ca, sh);
    if (prec == 1) return kernel_of<StF32>(ca, sh);
    return kernel_of<StF16>(ca, sh);
}

void launch_transport(const CellArgs &ca, Scalars *sc, int prec, PBufPair buf, int grid, cudaStream_t st) {
    TransportShape sh = transport_shape(ca, prec);
    if (prec == 0) launch_of<StF64>(ca, sh, sc, buf, grid, st);
    else if (prec == 1) launch_of<StF32>(ca, sh, sc, buf, grid, st);
    else launch_of<StF16>(ca, sh, sc, buf, grid, st);
}

const void *transport_multi_ptr(int prec) {
    if (prec == 0) return (const void *)k_transport1d_multi<StF64, kSmtBlock64>;
    if (prec == 1) return (const void *)k_transport1d_multi<StF32, kSmtBlock32>;
    return (const void *)k_transport1d_multi<StF16, kSmtBlock32>;
}

int transport_multi_block(int prec) { return prec == 0 ? kSmtBlock64 : kSmtBlock32; }

cudaError_t set_transport_multi_decks(const Deck1DArgs *ca, const PBufPair1D *bufs, Scalars *const *sc, int n,
                                      cudaStream_t st) {
    if (n < 0 || n > kFusedMaxDecks) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyToSymbolAsync(c_multi_ca, ca, sizeof(Deck1DArgs) * (size_t)n, 0,
                                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbolAsync(c_multi_bufs, bufs, sizeof(PBufPair1D) * (size_t)n, 0, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbolAsync(c_multi_sc, sc, sizeof(Scalars *) * (size_t)n, 0, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}


// ------------------------------------------- analog passes of the surrogate transport
// which: 0 the list pass, 1 a resume pass that sets aside, 2 the last resume pass
template <class St, int B, bool SMT> static const void *wave_ptr(int which) {
    if (which == 0) return (const void *)k_transport1d<St, B, SMT, kModeList>;
    if (which == 1) return (const void *)k_transport1d<St, B, SMT, kModeResume>;
    return (const void *)k_transport1d<St, B, SMT, kModeResumeLast>;
}

const void *surr_analog_ptr(const CellArgs &ca, int prec, int which) {
    const bool smt = transport_shape(ca, prec).smem_tally;
    if (prec == 2) return smt ? wave_ptr<StF16, kSmtBlock32, true>(which) : wave_ptr<StF16, kGlbBlock32, false>(which);
    return smt ? wave_ptr<StF32, kSmtBlock32, true>(which) : wave_ptr<StF32, kGlbBlock32, false>(which);
}

int surr_analog_smem(const CellArgs &ca, int prec) {
    return analog1d_smem(ca, 4, transport_shape(ca, prec).smem_tally, true);
}

template <class St, int B, bool SMT>
static void wave_one(const CellArgs &ca, Scalars *sc, PBufPair bufs, const SurrWave &w, int which, int round,
                     int grid, int smem, cudaStream_t st) {
    if (which == 0) k_transport1d<St, B, SMT, kModeList><<<grid, B, smem, st>>>(ca, sc, bufs, w, round);
    else if (which == 1) k_transport1d<St, B, SMT, kModeResume><<<grid, B, smem, st>>>(ca, sc, bufs, w, round);
    else k_transport1d<St, B, SMT, kModeResumeLast><<<grid, B, smem, st>>>(ca, sc, bufs, w, round);
}

void launch_surr_analog(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, const SurrWave &w, int which,
                        int round, int grid, int smem, cudaStream_t st) {
    const bool smt = transport_shape(ca, prec).smem_tally;
    if (prec == 2) {
        if (smt) wave_one<StF16, kSmtBlock32, true>(ca, sc, bufs, w, which, round, grid, smem, st);
        else wave_one<StF16, kGlbBlock32, false>(ca, sc, bufs, w, which, round, grid, smem, st);
    } else {
        if (smt) wave_one<StF32, kSmtBlock32, true>(ca, sc, bufs, w, which, round, grid, smem, st);
        else wave_one<StF32, kGlbBlock32, false>(ca, sc, bufs, w, which, round, grid, smem, st);
    }
}

}  // namespace imc
