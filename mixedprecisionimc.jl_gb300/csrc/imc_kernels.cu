// imc_kernels.cu -- the O(ncells) stages (FP64) and the particle-list stages
// around transport.
//
//   k_update           <- Update.update                 src/imc_update.jl:12-56
//   k_source_slots     <- Sourcing.sourcing, energies     src/imc_sourcing.jl:56-111
//   k_source_total     <- Sourcing.sourcing, total/budget src/imc_sourcing.jl:121-136
//   k_source_counts    <- Sourcing.sourcing, counts       src/imc_sourcing.jl:138-157
//   k_source_emit      <- Sourcing.sourcing, births        src/imc_sourcing.jl:159-366
//   k_compact_*        <- Clean.clean                    src/imc_clean.jl:6-19
//   k_tally            <- Tally.tally                    src/imc_tally.jl:22-142
//   k_energycheck      <- EnergyCheck.energychecker      src/imc_energycheck.jl:19-38
//   k_timestep         <- timestep                       src/MixedPrecisionIMC.jl:181-222
//
// Sums over cells are double-double: a fixed-order tree inside each 64-thread
// block, then the block partials in block order -- deterministic, and within
// a rounding of the exact sum.  Every launch has a fixed grid and reads its sizes from
// device scalars, so a whole step can be captured once as a CUDA graph.
#include <cstdint>
#include "imc_device.cuh"
#include "imc_internal.h"
#include "imc_state.cuh"

namespace imc {

constexpr int kPlanThreads = 1024;

// GB300 executes FP64 at 1/64 of the FP32 rate, so every per-cell FP64 stage
// runs as many one-warp blocks (kCellThreads) spread over the SMs; sums are
// double-double per block over a fixed partition of the cells, combined in
// block order.

__device__ __forceinline__ DD block_reduce_dd(DD v, DD *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = kCellThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            DD x = sh[threadIdx.x];
            x.add(sh[threadIdx.x + w]);
            sh[threadIdx.x] = x;
        }
        __syncthreads();
    }
    DD r = sh[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ DD dd_of(double x) {
    DD d;
    d.hi = x;
    d.lo = 0.0;
    return d;
}

// ------------------------------------------------------------------ update
__global__ void __launch_bounds__(kCellThreads) k_update(CellArgs ca, Scalars *sc) {
    const double a = ca.a, c = ca.c, dt = sc->dt;
    const double one[1] = {1.0};
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->flags = 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ca.nc) return;
    double T = ca.temp[i];
    double T3 = T * T * T;
    double beta;
    if (ca.linearized) {
        ca.bee[i] = (4.0 * a) * T3;
        beta = 1.0;
    } else {
        beta = ((4.0 * a) * T3) / ca.bee[i];
    }
    ca.beta[i] = beta;
    double Tc = (ca.temp_floor > 0.0 && T < ca.temp_floor) ? ca.temp_floor : T;
    // pow(x, 0) is 1 for every x (NaN included): skip the FP64 pow there
    const double psa = ca.sa_pow[i], pss = ca.ss_pow[i];
    double sa = ca.sa_val[i] * (psa == 0.0 ? 1.0 : pow(Tc, psa));
    if (ca.marshak) sa = ca.sa_val[i] / Tc / Tc / Tc;
    ca.sa[i] = sa;
    ca.ss[i] = ca.ss_val[i] * (pss == 0.0 ? 1.0 : pow(Tc, pss));
    double v[6] = {ca.ds, ca.alpha, beta, c, dt, sa};
    int j;
    double prod = sorter_n<0, 6>(v, one, 1, &j);
    ca.fleck[i] = 1.0 / (1.0 + prod);
}

void launch_update(const CellArgs &ca, Scalars *sc, cudaStream_t st) {
    k_update<<<ca.nblk_cell, kCellThreads, 0, st>>>(ca, sc);
}

// ---------------------------------------------------------------- sourcing

__device__ __forceinline__ int nsurf_slots(const CellArgs &ca) {
    return ca.geometry == 1 ? 2 : 2 * ca.nx + 2 * ca.ny;
}

// source-slot groups for the energy sums: 0 body, 1 radiation source,
// 2..5 the faces bottom, top, left, right (2D); 1D surfaces are added directly
__device__ __forceinline__ int slot_group(const CellArgs &ca, int s) {
    const int ns = nsurf_slots(ca);
    if (s >= ns + ca.nc) return 1;
    if (s >= ns) return 0;
    if (ca.geometry == 1) return -1;
    if (s < ca.nx) return 2;
    if (s < 2 * ca.nx) return 3;
    if (s < 2 * ca.nx + ca.ny) return 4;
    return 5;
}

// Energies per source slot (src/imc_sourcing.jl:56-111).  Slot order is the
// reference's push! order: 1D [left, right, body cells, source cells]; 2D
// [bottom x, top x, left y, right y, body cells, source cells].  Each block
// also leaves double-double partial sums of e/escale per slot group.
template <int G, int SEL>
__global__ void __launch_bounds__(kCellThreads) k_source_slots(CellArgs ca, Scalars *sc) {
    __shared__ DD sh[kCellThreads];
    const double a = ca.a, c = ca.c, ds = ca.ds, dt = sc->dt;
    const int ns = nsurf_slots(ca), nc = ca.nc, K = ca.K;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double q = 0.0;
    int grp = -2;
    if (s < ca.nslots) {
        double e = 0.0;
        int j = -1;
        if (s < ns) {
            double Ts = ca.tsurf[s], w = 0.0;
            if (G == 1) {
                double v[8] = {a, c, Ts, Ts, Ts, Ts, dt, 0.25};
                e = sorter_n<SEL, 8>(v, ca.scales, K, &j);
            } else {
                if (s < 2 * ca.nx) w = ca.dx[s % ca.nx];
                else w = ca.dy[(s - 2 * ca.nx) % ca.ny];
                double v[9] = {a, c, Ts, Ts, Ts, Ts, w, dt, 0.25};
                e = sorter_n<SEL, 9>(v, ca.scales, K, &j);
            }
        } else if (s < ns + nc) {
            const int i = s - ns;
            const int ix = G == 1 ? i : i % ca.nx;
            const int iy = G == 1 ? 0 : i / ca.nx;
            const double T = ca.temp[i], f = ca.fleck[i], sa = ca.sa[i];
            if (G == 1) {
                double v[11] = {f, sa, a, c, T, T, T, T, ca.dx[i], dt, ds};
                e = sorter_n<SEL, 11>(v, ca.scales, K, &j);
            } else {
                double v[12] = {f, sa, a, c, T, T, T, T, ca.dx[ix], ca.dy[iy], dt, ds};
                e = sorter_n<SEL, 12>(v, ca.scales, K, &j);
            }
            // emitted energy density (src/imc_sourcing.jl:69-70)
            double ve[10] = {f, sa, a, c, T, T, T, T, dt, ds};
            int je;
            double em = sorter_n<SEL, 10>(ve, ca.scales, K, &je);
            for (int k = 0; k < K; ++k) ca.emitted[(size_t)k * nc + i] = 0.0;
            if (je >= 0) ca.emitted[(size_t)je * nc + i] = em;
            else atomicOr(&sc->flags, 1u << 5);
        } else {
            const int i = s - ns - nc;
            const int ix = G == 1 ? i : i % ca.nx;
            const int iy = G == 1 ? 0 : i / ca.nx;
            if (G == 1) {
                double v[3] = {ca.radsource[i], ca.dx[i], dt};
                e = sorter_n<SEL, 3>(v, ca.scales, K, &j);
            } else {
                double v[4] = {ca.radsource[i], ca.dx[ix], ca.dy[iy], dt};
                e = sorter_n<SEL, 4>(v, ca.scales, K, &j);
            }
        }
        if (j < 0) atomicOr(&sc->flags, 1u << 5);
        const double sv = j >= 0 ? ca.scales[j] : 0.0;
        q = e / sv;
        ca.slot_e[s] = e;
        ca.slot_s[s] = sv;
        ca.slot_j[s] = j;
        ca.slot_q[s] = q;
        grp = slot_group(ca, s);
    }
    for (int g = 0; g < 6; ++g) {
        // most blocks hold one group: reduce only the groups present
        if (!__syncthreads_or(grp == g)) {
            if (threadIdx.x == 0) {
                ca.part_src[(blockIdx.x * 6 + g) * 2] = 0.0;
                ca.part_src[(blockIdx.x * 6 + g) * 2 + 1] = 0.0;
            }
            continue;
        }
        DD r = block_reduce_dd(dd_of(grp == g ? q : 0.0), sh);
        if (threadIdx.x == 0) {
            ca.part_src[(blockIdx.x * 6 + g) * 2] = r.hi;
            ca.part_src[(blockIdx.x * 6 + g) * 2 + 1] = r.lo;
        }
    }
}

__device__ __forceinline__ long long round_count(double q, double n_source, double E, bool withmin,
                                                 double cellmin) {
    double r = rint((q * n_source) / E);
    if (withmin) r = fmax(r, cellmin);
    return (long long)r;
}

// Sum of the double-double block partials of one group by one warp: lane l
// takes blocks l, l+32, ..., then a fixed shuffle tree.  Deterministic.
__device__ __forceinline__ double warp_sum_partials(const double *part, int nb, int stride, int g) {
    const int lane = threadIdx.x & 31;
    DD d;
    d.clear();
    for (int bb = lane; bb < nb; bb += 32) {
        DD p;
        p.hi = part[(bb * stride + g) * 2];
        p.lo = part[(bb * stride + g) * 2 + 1];
        d.add(p);
    }
    for (int off = 16; off > 0; off >>= 1) {
        DD o;
        o.hi = __shfl_down_sync(0xFFFFFFFFu, d.hi, off);
        o.lo = __shfl_down_sync(0xFFFFFFFFu, d.lo, off);
        if (lane < off) d.add(o);
    }
    return __shfl_sync(0xFFFFFFFFu, d.val(), 0);
}

// Sums of the slot groups (src/imc_sourcing.jl:121): one one-warp block per
// group, so each sum has an SM's FP64 pipe to itself (1D needs only the body
// and radiation-source groups; its two surfaces are added directly).
__global__ void __launch_bounds__(32) k_source_total(CellArgs ca, Scalars *sc) {
    const double v = warp_sum_partials(ca.part_src, ca.nblk_slot, 6, blockIdx.x);
    if (threadIdx.x == 0) sc->src_group[blockIdx.x] = v;
}

// Total energy (src/imc_sourcing.jl:121) and particle budget (:132-136) from
// the group sums, in a fixed order: every block of k_source_counts computes
// the same values.
__device__ __forceinline__ void source_total(const CellArgs &ca, const Scalars *sc, double &E, double &n_source) {
    const double *g = sc->src_group;
    double e_surface;
    if (ca.geometry == 1) {
        e_surface = ca.slot_q[0] + ca.slot_q[1];
    } else {
        e_surface = 0.0;
        e_surface += g[2];
        e_surface += g[3];
        e_surface += g[4];
        e_surface += g[5];
    }
    E = g[0] + g[1] + e_surface;
    const long long n_census = sc->n_census;
    n_source = (double)ca.n_input;
    if (ca.n_input + n_census > ca.n_max) {
        double lenN = ca.geometry == 1 ? 1.0 : 2.0;
        n_source = fmax(ca.cellmin, (double)(ca.n_max - n_census) - lenN - 1.0);
    }
}

// Births per slot (src/imc_sourcing.jl:138-157) and per-particle energy;
// block 0 also records the step's total energy and budget.
__global__ void __launch_bounds__(kCellThreads) k_source_counts(CellArgs ca, Scalars *sc) {
    __shared__ double wm[kCellThreads / 32];
    const int ns = nsurf_slots(ca), nc = ca.nc;
    double E, n_source;
    source_total(ca, sc, E, n_source);
    const bool ok = (E > 0.0) && isfinite(E);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->totalenergy = E;
        sc->n_source = n_source;
        if (!ok) atomicOr(&sc->flags, 1u << 4);
    }
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double my = 0.0;
    if (q < ca.nslots) {
        const double *e = ca.slot_e, *qv = ca.slot_q;
        long long n = 0, nd = 0;
        if (ok) {
            if (q < ns) {
                if (e[q] > 0) n = round_count(qv[q], n_source, E, ca.geometry == 2, ca.cellmin);
                nd = n;
            } else if (q < ns + nc) {
                n = round_count(qv[q], n_source, E, true, ca.cellmin);
                nd = n;
            } else if (e[q] > 0) {
                n = round_count(qv[q], n_source, E, true, ca.cellmin);
                nd = n;
                // 2D births n_body particles per source cell (src/imc_sourcing.jl:357)
                if (ca.geometry == 2 && n > 0) n = round_count(qv[q - nc], n_source, E, true, ca.cellmin);
            }
            if (n < 0) n = 0;
        }
        const double nrg = n > 0 ? e[q] / (double)nd : 0.0;
        ca.slot_n[q] = n;
        ca.slot_nrg[q] = nrg;
        ca.slot_nrg_f[q] = (float)nrg;
        // the largest birth energy in true units (see scale_exp)
        if (n > 0) my = ldexp(nrg, -scale_exp(ca.scales[ca.slot_j[q]]));
    }
    for (int off = 16; off > 0; off >>= 1) {
        double o = __shfl_down_sync(0xFFFFFFFFu, my, off);
        my = o > my ? o : my;
    }
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = my;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = wm[0];
        for (int w = 1; w < kCellThreads / 32; ++w) m = wm[w] > m ? wm[w] : m;
        ca.part_emax[blockIdx.x] = m;
    }
}

// Exclusive scan of the births, capacity check, fixed-point exponents.
__global__ void __launch_bounds__(kPlanThreads) k_source_scan(CellArgs ca, Scalars *sc) {
    __shared__ long long warp_tot[32];
    __shared__ long long s_run;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_run = 0;
    __syncthreads();
    for (int base = 0; base < ca.nslots; base += blockDim.x) {
        int q = base + threadIdx.x;
        long long v = q < ca.nslots ? ca.slot_n[q] : 0;
        long long x = v;
        for (int off = 1; off < 32; off <<= 1) {
            long long y = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
            for (int off = 1; off < 32; off <<= 1) {
                long long y = __shfl_up_sync(0xFFFFFFFFu, w, off);
                if (lane >= off) w += y;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        long long excl = s_run + (warp > 0 ? warp_tot[warp - 1] : 0) + x - v;
        if (q < ca.nslots) ca.slot_off[q] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_run = excl + v;
        __syncthreads();
    }
    // largest birth energy over the per-block maxima, one warp wide (the
    // loads are independent; a single thread would wait for each in turn)
    __shared__ double s_emax;
    if (warp == 0) {
        double m = 0.0;
        for (int bb = lane; bb < ca.nblk_slot; bb += 32) m = fmax(m, ca.part_emax[bb]);
        for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xFFFFFFFFu, m, off));
        if (lane == 0) s_emax = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long n_census = sc->n_census;  // live particles
        const long long len = sc->n_particles;    // list length, holes included
        long long n_new = s_run;
        unsigned fl = 0;
        if (len + n_new > ca.capacity) {
            n_new = ca.capacity - len;
            if (n_new < 0) n_new = 0;
            fl |= 1u << 3;
        }
        const int ce = sc->emax_census_exp;
        const double emax = fmax(ce == kNoExp ? 0.0 : exp_top(ce), s_emax);
        sc->n_census_in = n_census;
        sc->n_sourced = n_new;
        sc->birth_base = len;
        sc->n_particles = len + n_new;
        sc->emax = emax;
        sc->emax_census_exp = kNoExp;
        sc->segments = 0ull;
        sc->surrogate_calls = 0ull;
        sc->killed = 0ull;
        sc->work_next = 0ull;
        for (int r = 0; r <= 2 * kSurrRounds; ++r) sc->qcount[r] = 0ull;
        sc->b_dep = fix_exponent(emax / ca.vol_min);
        sc->b_lost = fix_exponent(emax);
        sc->b_rad = fix_exponent(emax);
        if (fl) sc->flags |= fl;
    }
}

template <class T> struct RT;
template <> struct RT<float> { static __device__ float sqrt_(float x) { return sqrtf(x); } };
template <> struct RT<double> { static __device__ double sqrt_(double x) { return sqrt(x); } };

template <class St>
__device__ __forceinline__ void store_birth(const CellArgs &ca, PBuf<St> &pb, long long pid, typename St::T t,
                                            typename St::T x, typename St::T y, typename St::T ux,
                                            typename St::T uy, typename St::T E0, int cell, int k, float dtf) {
    typedef typename St::S S;
    if (St::half) {
        const int ix = ca.geometry == 1 ? cell : cell % ca.nx;
        float dxs = (float)ca.dx[ix] * (float)ca.ds;
        st_v(pb.x + pid, (float)x / dxs);
        if (ca.geometry == 2) {
            const int iy = cell / ca.nx;
            float dys = (float)ca.dy[iy] * (float)ca.ds;
            st_v(pb.y + pid, (float)y / dys);
            st_v(pb.uy + pid, (float)uy);
        }
        st_v(pb.t + pid, (float)t / dtf);
        st_v(pb.ux + pid, (float)ux);
        st_v(pb.E + pid, 1.0f);
        pb.E0[pid] = (float)E0;
    } else {
        pb.t[pid] = (S)t;
        pb.x[pid] = (S)x;
        pb.ux[pid] = (S)ux;
        if (ca.geometry == 2) { pb.y[pid] = (S)y; pb.uy[pid] = (S)uy; }
        pb.E[pid] = (S)E0;
        pb.E0[pid] = (typename St::E0S)E0;
    }
    pb.cs[pid] = cell | (k << 24);
    pb.alive[pid] = 1;
}

// One thread per newborn particle; its stream is keyed by its list index.
template <class St>
__global__ void __launch_bounds__(256) k_source_emit(CellArgs ca, Scalars *sc, PBufPair bufs) {
    typedef typename St::T T;
    PBuf<St> pb(bufs.b[sc->cur]);
    const long long n_new = sc->n_sourced, n_census = sc->birth_base;
    const unsigned step = sc->step;
    const double dtd = sc->dt;
    const T dtT = (T)dtd, dsT = (T)ca.ds;
    const int ns = nsurf_slots(ca), nc = ca.nc, nslots = ca.nslots;
    const double pd = 3.141592653589793;
    // the surface births' fixed positions, the same for every birth of a
    // face (computed on the host, CellArgs::surf_f / surf_d)
    auto surf = [&](int w) -> T { return sizeof(T) == 4 ? (T)ca.surf_f[w] : (T)ca.surf_d[w]; };
    const T x1_l = surf(0), x1_r = surf(1), x2_l = surf(2), x2_r = surf(3), y2_b = surf(4), y2_t = surf(5);
    // Each warp takes `run` consecutive births at a time, lane l the births
    // base + l + 32 i (every store coalesced).  A lane finds the slot of its
    // first birth by binary search over the slot offsets (slot = last q with
    // slot_off[q] <= j) and the later ones by galloping forward from there
    // (q + 1, q + 2, q + 4, ... then bisection): one or two loads where the
    // slot holds many births (the channel's surface segment), a few where
    // it holds a handful (the CELLMIN births of every body cell).  The run
    // is the births per warp of the grid, rounded up to a multiple of 32 in
    // [32, 256], so a small step's births still spread over every warp.
    const int lane = threadIdx.x & 31;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long per_warp = (n_new + nw - 1) / nw;
    const int run = per_warp >= 256 ? 256 : per_warp <= 32 ? 32 : (int)((per_warp + 31) & ~31ll);
    for (long long base = wid * run; base < n_new; base += nw * run)
    for (int q = -1, r = 0; r < run; r += 32) {
        const long long j = base + r + lane;
        if (j >= n_new) break;
        if (q < 0) {
            int lo = 0, hi = nslots;
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (ca.slot_off[mid] <= j) lo = mid;
                else hi = mid;
            }
            q = lo;
        } else if (q + 1 < nslots && ca.slot_off[q + 1] <= j) {
            int lo = q + 1, step = 2, hi = q + 2;  // slot_off[lo] <= j
            while (hi < nslots && ca.slot_off[hi] <= j) {
                lo = hi;
                step <<= 1;
                hi = q + step;
            }
            if (hi > nslots) hi = nslots;  // slot_off[hi] > j, or hi == nslots
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (ca.slot_off[mid] <= j) lo = mid;
                else hi = mid;
            }
            q = lo;
        }
        const long long pid = n_census + j;
        Stream rs;
        rs.init(ca.seed, step, (uint32_t)pid, kStageSource);
        const T E0 = sizeof(T) == 4 ? (T)ca.slot_nrg_f[q] : (T)ca.slot_nrg[q];
        const int k = ca.slot_j[q] < 0 ? 0 : ca.slot_j[q];
        if (ca.geometry == 1) {
            if (q < 2) {
                // surface births (src/imc_sourcing.jl:161-189)
                const int cell = q == 0 ? 0 : ca.nx - 1;
                T xpos = q == 0 ? x1_l : x1_r;
                T mu = (T)0;
                for (int r = 0; r < 64 && mu == (T)0; ++r) {
                    T rr = RT<T>::sqrt_(Rand<T>::u(rs));
                    mu = q == 0 ? rr : -rr;
                }
                if (mu == (T)0) mu = q == 0 ? (T)1 : (T)-1;
                T st = dtT * Rand<T>::u(rs);
                store_birth<St>(ca, pb, pid, st, xpos, (T)0, mu, (T)0, E0, cell, k, (float)dtT);
            } else {
                // body / source births (src/imc_sourcing.jl:193-236)
                const int cell = q < ns + nc ? q - ns : q - ns - nc;
                T xpos = (sizeof(T) == 4 ? (T)ca.dxf[cell] : (T)ca.dx[cell]) * Rand<T>::u(rs) * dsT;
                T mu = (T)0;
                for (int r = 0; r < 64 && mu == (T)0; ++r) mu = (T)1 - (T)2 * Rand<T>::u(rs);
                if (mu == (T)0) mu = (T)1;
                T st = dtT * Rand<T>::u(rs);
                store_birth<St>(ca, pb, pid, st, xpos, (T)0, mu, (T)0, E0, cell, k, (float)dtT);
            }
        } else {
            T st, xpos, ypos, ang;
            int ix, iy;
            if (q < ns) {
                // surface births (src/imc_sourcing.jl:265-323)
                const int nx = ca.nx, ny = ca.ny;
                int face, idx;
                if (q < nx) { face = 0; idx = q; }
                else if (q < 2 * nx) { face = 1; idx = q - nx; }
                else if (q < 2 * nx + ny) { face = 2; idx = q - 2 * nx; }
                else { face = 3; idx = q - 2 * nx - ny; }
                st = dtT * Rand<T>::u(rs);
                // the angles are the reference's Float64 products rounded to T
                // (binary32: pi_n24 of the uniform's integer m, the same value
                // without FP64; the widths binary32 copies)
                if (face < 2) {
                    ix = idx;
                    iy = face == 0 ? 0 : ny - 1;
                    xpos = (sizeof(T) == 4 ? (T)ca.dxf[ix] : (T)ca.dx[ix]) * Rand<T>::u(rs) * dsT;
                    ypos = face == 0 ? y2_b : y2_t;
                    if constexpr (sizeof(T) == 4) {
                        const uint32_t m = rs.next() >> 8;
                        ang = face == 0 ? (T)pd * ((T)m * 0x1p-24f) : -pi_n24((int)m);
                    } else {
                        T u = Rand<T>::u(rs);
                        ang = face == 0 ? (T)((T)pd * u) : (T)(-pd * (double)u);
                    }
                } else {
                    iy = idx;
                    ix = face == 2 ? 0 : nx - 1;
                    xpos = face == 2 ? x2_l : x2_r;
                    // the reference scales y by mesh.dx[j] (src/imc_sourcing.jl:301,316)
                    if constexpr (sizeof(T) == 4) {
                        ypos = (iy < nx ? ca.dxf[iy] : ca.dyf[iy]) * Rand<T>::u(rs) * dsT;
                        const uint32_t m = rs.next() >> 8;
                        ang = face == 2 ? pi_n24((1 << 23) - (int)m)
                                        : (T)(pd * (0.5 + (double)((T)m * 0x1p-24f)));
                    } else {
                        const double wq = iy < nx ? ca.dx[iy] : ca.dy[iy];
                        ypos = (T)wq * Rand<T>::u(rs) * dsT;
                        T u = Rand<T>::u(rs);
                        ang = face == 2 ? (T)(pd * (0.5 - (double)u)) : (T)(pd * (0.5 + (double)u));
                    }
                }
            } else {
                // body / source births (src/imc_sourcing.jl:326-366)
                const int cell = q < ns + nc ? q - ns : q - ns - nc;
                ix = cell % ca.nx;
                iy = cell / ca.nx;
                // binary32 widths precomputed (no per-birth conversion); the
                // angle is the reference's Float64 2 pi rand rounded to T
                // (binary32: two_pi_u24, the same value without FP64)
                xpos = (sizeof(T) == 4 ? (T)ca.dxf[ix] : (T)ca.dx[ix]) * Rand<T>::u(rs) * dsT;
                ypos = (sizeof(T) == 4 ? (T)ca.dyf[iy] : (T)ca.dy[iy]) * Rand<T>::u(rs) * dsT;
                if constexpr (sizeof(T) == 4) ang = two_pi_u24(rs.next() >> 8);
                else ang = (T)(2.0 * pd * (double)Rand<T>::u(rs));
                st = dtT * Rand<T>::u(rs);
            }
            T ux, uy;
            if (sizeof(T) == 4) { float s_, c_; sincosf((float)ang, &s_, &c_); ux = (T)c_; uy = (T)s_; }
            else { double s_, c_; sincos((double)ang, &s_, &c_); ux = (T)c_; uy = (T)s_; }
            store_birth<St>(ca, pb, pid, st, xpos, ypos, ux, uy, E0, ix + iy * ca.nx, k, (float)dtT);
        }
    }
}

void launch_source(const CellArgs &ca, Scalars *sc, int prec, PBufPair buf, int grid, cudaStream_t st) {
    const int nb = ca.nblk_slot;
    // one instantiation per geometry and scale-selection precision, so each
    // holds only its own unrolled sorters
    auto slots = ca.geometry == 1 ? (ca.sel_prec == 2 ? k_source_slots<1, 2> : ca.sel_prec == 1 ? k_source_slots<1, 1> : k_source_slots<1, 0>)
                                  : (ca.sel_prec == 2 ? k_source_slots<2, 2> : ca.sel_prec == 1 ? k_source_slots<2, 1> : k_source_slots<2, 0>);
    slots<<<nb, kCellThreads, 0, st>>>(ca, sc);
    k_source_total<<<ca.geometry == 1 ? 2 : 6, 32, 0, st>>>(ca, sc);
    k_source_counts<<<nb, kCellThreads, 0, st>>>(ca, sc);
    k_source_scan<<<1, kPlanThreads, 0, st>>>(ca, sc);
    if (prec == 0) k_source_emit<StF64><<<grid, 256, 0, st>>>(ca, sc, buf);
    else if (prec == 1) k_source_emit<StF32><<<grid, 256, 0, st>>>(ca, sc, buf);
    else k_source_emit<StF16><<<grid, 256, 0, st>>>(ca, sc, buf);
}

// ------------------------------------------------------------- compaction
// Stable three-pass compaction: per-tile alive counts, one-block exclusive
// scan of the tile counts, then a per-tile block scan that scatters the
// survivors in order into the other buffer.
__global__ void __launch_bounds__(kCompactThreads) k_compact_count(const Scalars *sc, PBufPair bufs,
                                                                   long long *tile_cnt) {
    if (!sc->compact_now) return;
    const uint8_t *alive = bufs.b[sc->cur].alive;
    const long long n = sc->n_particles;
    const long long base = (long long)blockIdx.x * kCompactTile;
    if (base >= n) return;
    int cnt = 0;
    if (base + kCompactTile <= n) {
        // a full tile: 16 alive bytes per thread in one 16-byte load (tiles
        // start at multiples of 4096 bytes, so every load is aligned)
        static_assert(kCompactTile == 16 * kCompactThreads, "one uint4 per thread");
        const uint4 v = reinterpret_cast<const uint4 *>(alive + base)[threadIdx.x];
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        for (int q = 0; q < 4; ++q)
            for (int b = 0; b < 4; ++b) cnt += ((w[q] >> (8 * b)) & 0xFFu) != 0u;
    } else {
        for (int r = threadIdx.x; r < kCompactTile; r += blockDim.x) {
            long long i = base + r;
            if (i < n && alive[i]) ++cnt;
        }
    }
    cnt = __reduce_add_sync(0xFFFFFFFFu, (unsigned)cnt);
    __shared__ int wt[kCompactThreads / 32];
    if ((threadIdx.x & 31) == 0) wt[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) s += wt[w];
        tile_cnt[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(1024) k_compact_scan(Scalars *sc, const long long *tile_cnt, long long *tile_off,
                                                      int force) {
    __shared__ long long warp_tot[32];
    __shared__ long long s_run;
    if (!sc->compact_now) return;  // k_compact_decide set the live count
    const long long n = sc->n_particles;
    const long long ntiles = (n + kCompactTile - 1) / kCompactTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_run = 0;
    __syncthreads();
    for (long long base = 0; base < ntiles; base += blockDim.x) {
        long long q = base + threadIdx.x;
        long long v = q < ntiles ? tile_cnt[q] : 0;
        long long x = v;
        for (int off = 1; off < 32; off <<= 1) {
            long long y = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long w = warp_tot[lane];
            for (int off = 1; off < 32; off <<= 1) {
                long long y = __shfl_up_sync(0xFFFFFFFFu, w, off);
                if (lane >= off) w += y;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        long long excl = s_run + (warp > 0 ? warp_tot[warp - 1] : 0) + x - v;
        if (q < ntiles) tile_off[q] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_run = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // compact when forced (Clean.clean) or when the holes exceed 1/16 of the list
        const long long alive = s_run;
        (void)force;
        sc->n_census = alive;
        sc->compact_src = sc->cur;
        sc->cur ^= 1;
        sc->n_particles = alive;
    }
}

template <class St>
__global__ void __launch_bounds__(kCompactThreads) k_compact_scatter(int geometry, const Scalars *sc,
                                                                     const long long *tile_off, PBufPair bufs,
                                                                     const long long *n_before) {
    if (!sc->compact_now) return;
    PBuf<St> src(bufs.b[sc->compact_src]), dst(bufs.b[sc->compact_src ^ 1]);
    __shared__ unsigned short src_idx[kCompactTile];
    __shared__ int wt[kCompactThreads / 32];
    __shared__ int s_tot;
    const long long n = *n_before;
    const long long base = (long long)blockIdx.x * kCompactTile;
    if (base >= n) return;
    const int tile_n = (int)((n - base) < kCompactTile ? (n - base) : kCompactTile);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // survivor list of the tile, in order: thread t owns tile positions
    // [16t, 16t + 16) and reads their alive bytes with one 16-byte load
    constexpr int kPer = kCompactTile / kCompactThreads;
    static_assert(kPer == 16, "one uint4 of alive bytes per thread");
    const int first = threadIdx.x * kPer;
    unsigned char flags[kPer];
    const uint8_t *ap = src.alive + base + first;
    if (first + kPer <= tile_n && (((uintptr_t)ap) & 15u) == 0) {
        uint4 v = *reinterpret_cast<const uint4 *>(ap);
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
        for (int q = 0; q < kPer; ++q) flags[q] = (unsigned char)((w[q >> 2] >> (8 * (q & 3))) & 0xFFu);
    } else {
        for (int q = 0; q < kPer; ++q) flags[q] = first + q < tile_n ? ap[q] : 0;
    }
    int mine = 0;
    for (int q = 0; q < kPer; ++q) mine += flags[q] ? 1 : 0;
    int incl = mine;
    for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) wt[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) { int v = wt[w]; wt[w] = acc; acc += v; }
        s_tot = acc;
    }
    __syncthreads();
    int pos = wt[warp] + incl - mine;
    for (int q = 0; q < kPer; ++q)
        if (flags[q]) src_idx[pos++] = (unsigned short)(first + q);
    const int run = s_tot;
    __syncthreads();
    const int cnt = run;
    const long long out = tile_off[blockIdx.x];
    // Every field of a survivor in one pass: stores coalesced, loads gathered
    // from the tile (whole sectors when most entries survive; when most are
    // holes, only the sectors that hold a survivor), all fields' loads of a
    // survivor in flight together.
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
        const long long f = base + src_idx[j], d = out + j;
        const auto t = src.t[f], x = src.x[f], ux = src.ux[f];
        const auto E = src.E[f];
        const auto E0 = src.E0[f];
        const int cs = src.cs[f];
        if (geometry == 2) {
            const auto y = src.y[f], uy = src.uy[f];
            dst.y[d] = y;
            dst.uy[d] = uy;
        }
        dst.t[d] = t; dst.x[d] = x; dst.ux[d] = ux;
        dst.E[d] = E;
        dst.E0[d] = E0;
        dst.cs[d] = cs;
        dst.alive[d] = 1;
    }
}

// Before compaction: the list length (for the scatter) and whether this step
// compacts.  The live count follows from the transport's kills (census
// carried in + births - removed), so the holes are known without reading the
// alive bytes; they are counted per tile only when the list is compacted.
__global__ void k_compact_decide(Scalars *sc, long long *n_before, int force) {
    const long long n = sc->n_particles;
    *n_before = n;
    const long long live = sc->n_census_in + sc->n_sourced - (long long)sc->killed;
    const bool compact = force || (n - live) * kDeferHoles > n;
    sc->compact_now = compact ? 1 : 0;
    if (!compact) sc->n_census = live;
}

void launch_compact(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, long long *tile_cnt,
                    long long *tile_off, long long ntiles_cap, bool force, cudaStream_t st) {
    // tile_off has ntiles_cap + 1 entries; the last holds the pre-compaction length
    long long *n_before = tile_off + ntiles_cap;
    k_compact_decide<<<1, 1, 0, st>>>(sc, n_before, force ? 1 : 0);
    k_compact_count<<<(unsigned)ntiles_cap, kCompactThreads, 0, st>>>(sc, bufs, tile_cnt);
    k_compact_scan<<<1, 1024, 0, st>>>(sc, tile_cnt, tile_off, force ? 1 : 0);
    if (prec == 0)
        k_compact_scatter<StF64><<<(unsigned)ntiles_cap, kCompactThreads, 0, st>>>(ca.geometry, sc, tile_off, bufs, n_before);
    else if (prec == 1)
        k_compact_scatter<StF32><<<(unsigned)ntiles_cap, kCompactThreads, 0, st>>>(ca.geometry, sc, tile_off, bufs, n_before);
    else
        k_compact_scatter<StF16><<<(unsigned)ntiles_cap, kCompactThreads, 0, st>>>(ca.geometry, sc, tile_off, bufs, n_before);
}

void launch_compact(const CellArgs &ca, Scalars *sc, int prec, PBufRaw src, PBufRaw dst, long long *tile_cnt,
                    long long *tile_off, long long ntiles_cap, cudaStream_t st) {
    PBufPair p;
    p.b[0] = src;
    p.b[1] = dst;
    launch_compact(ca, sc, prec, p, tile_cnt, tile_off, ntiles_cap, true, st);
}

// ------------------------------------------------------------------- tally
__device__ __forceinline__ double cell_vol(const CellArgs &ca, int i) {
    return ca.geometry == 1 ? ca.dx[i] : ca.dx[i % ca.nx] * ca.dy[i / ca.nx];
}

// Converts this transport's fixed-point tallies to FP64 mesh fields and
// clears the accumulators: energydep and the escaped energy as
// Transport.MC leaves them (src/imc_transport.jl:198-205), and the census
// radiation energy density of src/imc_tally.jl:81-113.  Cell i, and the
// escaped energy and segment statistics in block 0, thread 0.
__device__ __forceinline__ void finalize_cell(const CellArgs &ca, Scalars *sc, int i) {
    const int nc = ca.nc, K = ca.K;
    const int b_dep = sc->b_dep, b_rad = sc->b_rad, b_lost = sc->b_lost;
    if (i < nc) {
        const double vol = cell_vol(ca, i);
        double r = 0.0;
        for (int k = 0; k < K; ++k) {
            const size_t idx = (size_t)k * nc + i;
            const int se = scale_exp(ca.scales[k]);
            long long *d = ca.dep_acc + 3 * idx;
            ca.energydep[idx] = fix_value(d, b_dep + se);
            d[0] = d[1] = d[2] = 0;
            long long *g = ca.rad_acc + 3 * idx;
            r += fix_value(g, b_rad + se) / (vol * ca.scales[k]);
            g[0] = g[1] = g[2] = 0;
        }
        ca.radenergydens[i] = r;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double lost = 0.0;
        for (int k = 0; k < K; ++k) {
            long long *d = ca.lost_acc + 3 * k;
            lost += fix_value(d, b_lost + scale_exp(ca.scales[k])) / ca.scales[k];
            d[0] = d[1] = d[2] = 0;
        }
        sc->lost_step = lost;
        // mean transport segments per history of this step: the next
        // transport picks its lane schedule from it
        const double hist = (double)(sc->n_census_in + sc->n_sourced);
        sc->seg_per_hist = hist > 0.0 ? (float)((double)sc->segments / hist) : 0.0f;
        sc->lostenergy += lost;
    }
}

// Tally.tally per cell (src/imc_tally.jl:29-75); each block leaves partial
// sums of the deposited energy per scale and of the radiation energy.
__device__ __forceinline__ void tally_cell(const CellArgs &ca, Scalars *sc, int i, DD *sh) {
    const int nc = ca.nc, K = ca.K;
    const double a = ca.a, c = ca.c, dt = sc->dt;
    const bool first = sc->t == 0.0;
    const double one[1] = {1.0};
    double vol = 0.0;
    if (i < nc) {
        vol = cell_vol(ca, i);
        if (first) {
            double T = ca.temp[i];
            double v[10] = {ca.fleck[i], ca.sa[i], a, c, T, T, T, T, dt, ca.ds};
            int j;
            ca.matenergydens[i] = sorter_n<0, 10>(v, one, 1, &j);
        }
        double inc = 0.0;
        for (int k = 0; k < K; ++k)
            inc += (ca.energydep[(size_t)k * nc + i] - ca.emitted[(size_t)k * nc + i]) / ca.scales[k];
        double m = ca.matenergydens[i] + inc;
        ca.matenergydens[i] = m;
        if (ca.linearized) ca.temp[i] = pow(m, 0.25);
        else ca.temp[i] = ca.temp[i] + inc / ca.bee[i];
    }
    const int np = K + 1;
    for (int k = 0; k < K; ++k) {
        double x = i < nc ? (ca.energydep[(size_t)k * nc + i] * vol) / ca.scales[k] : 0.0;
        DD r = block_reduce_dd(dd_of(x), sh);
        if (threadIdx.x == 0) {
            ca.part_tally[(blockIdx.x * np + k) * 2] = r.hi;
            ca.part_tally[(blockIdx.x * np + k) * 2 + 1] = r.lo;
        }
    }
    DD r = block_reduce_dd(dd_of(i < nc ? ca.radenergydens[i] * vol : 0.0), sh);
    if (threadIdx.x == 0) {
        ca.part_tally[(blockIdx.x * np + K) * 2] = r.hi;
        ca.part_tally[(blockIdx.x * np + K) * 2 + 1] = r.lo;
    }
}

__global__ void __launch_bounds__(kCellThreads) k_finalize(CellArgs ca, Scalars *sc) {
    finalize_cell(ca, sc, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(kCellThreads) k_tally(CellArgs ca, Scalars *sc) {
    __shared__ DD sh[kCellThreads];
    tally_cell(ca, sc, blockIdx.x * blockDim.x + threadIdx.x, sh);
}

// Both in one launch (the step sequence): the tally of cell i reads only
// what the finalize of cell i wrote, in the same thread, and nothing that
// the compaction between them in the reference's order changes.
__global__ void __launch_bounds__(kCellThreads) k_finalize_tally(CellArgs ca, Scalars *sc) {
    __shared__ DD sh[kCellThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    finalize_cell(ca, sc, i);
    tally_cell(ca, sc, i, sh);
}

void launch_finalize(const CellArgs &ca, Scalars *sc, cudaStream_t st) {
    k_finalize<<<ca.nblk_cell, kCellThreads, 0, st>>>(ca, sc);
}

void launch_tally(const CellArgs &ca, Scalars *sc, cudaStream_t st) {
    k_tally<<<ca.nblk_cell, kCellThreads, 0, st>>>(ca, sc);
}

void launch_finalize_tally(const CellArgs &ca, Scalars *sc, cudaStream_t st) {
    k_finalize_tally<<<ca.nblk_cell, kCellThreads, 0, st>>>(ca, sc);
}

// timestep (src/MixedPrecisionIMC.jl:181-222), FP64 on the device so a run
// can replay without host round trips.
__device__ __forceinline__ void advance_clock(const CellArgs &ca, Scalars *sc) {
    double t = sc->t, dt = sc->dt;
    const double t_end = ca.t_end;
    if (t == t_end) {
        t = t_end + dt;
    } else if (ca.timestepping == 0) {
        if (t + dt > t_end) { dt = t_end - t; t = t_end; }
        else t = t + dt;
    } else {
        if (dt < ca.dtmax) {
            dt = dt * ca.kfac;
            if (dt > ca.dtmax) dt = ca.dtmax;
        }
        if (t + dt > t_end) { dt = t_end - t; t = t_end; }
        else t = t + dt;
    }
    sc->t = t;
    sc->dt = dt;
    sc->finished = t > t_end ? 1 : 0;
    sc->step += 1u;
}

// EnergyCheck.energychecker (src/imc_energycheck.jl:19-38) from the sums of
// the tally's per-block partials (g[k]: deposited energy of scale k, g[K]:
// radiation energy), by one thread: the balance, the step's statistics, the
// learned surrogate's gate, and with STEP the clock.
__device__ void energycheck_done(const CellArgs &ca, Scalars *sc, DevStats *stats, long long stats_cap,
                                 const double *g, bool step) {
    double totdep = 0.0;
    for (int k = 0; k < ca.K; ++k) totdep += g[k];
    const double radenergy = g[ca.K];
    sc->totalenergydep = totdep;
    double err = (sc->totalenergy - totdep - (radenergy - sc->radenergyold) - sc->lostenergy) / sc->totalenergy;
    if (stats && stats_cap > 0) {
        DevStats &d = stats[sc->step % (unsigned long long)stats_cap];
        d.t = sc->t; d.dt = sc->dt;
        d.total_energy = sc->totalenergy;
        d.energy_dep = totdep;
        d.rad_energy = radenergy;
        d.rad_energy_old = sc->radenergyold;
        d.lost_energy = sc->lostenergy;
        d.energy_error = err;
        d.n_census_in = sc->n_census_in;
        d.n_sourced = sc->n_sourced;
        d.n_census_out = sc->n_census;
        d.segments = (long long)sc->segments;
        d.surrogate_calls = (long long)sc->surrogate_calls;
        d.error_flags = sc->flags;
        d.step_index = sc->step;
    }
    sc->energy_err = err;
    sc->radenergy = radenergy;
    sc->radenergyold = radenergy;
    sc->lostenergy = 0.0;
    // Learned surrogate gate for the next step.  Its extra passes (a query
    // pass and an analog resume pass after the list pass) pay only when a
    // step holds enough queries to fill the GPU about twice over; with
    // fewer, the passes' latency outweighs the collisions the queries save
    // (measured on the 256-deck ensemble).  A step that ran with the gate
    // open keeps it open only if it made ca.surr_min_calls queries.  A
    // closed gate opens again to measure when the step's histories have
    // doubled since it closed (a census still filling up) and every
    // kSurrProbe-th step.  The decision uses the step's own counts, so runs
    // stay reproducible.
    if (ca.surr_image) {
        const long long hist = sc->n_census_in + sc->n_sourced;
        if (sc->surr_gate) {
            sc->surr_gate = (long long)sc->surrogate_calls >= ca.surr_min_calls ? 1 : 0;
            if (!sc->surr_gate) sc->surr_closed_h = hist;
        } else if (hist >= 2 * sc->surr_closed_h) {
            sc->surr_gate = 1;
        }
        if ((sc->step + 1u) % kSurrProbe == 0u) sc->surr_gate = 1;
    }
    if (step) advance_clock(ca, sc);  // the step sequence: timestep in the same launch
}

// EnergyCheck.energychecker as its own launch: one warp per partial-sum
// group (K deposition scales, then the radiation energy).
template <bool STEP>
__global__ void __launch_bounds__(544) k_energycheck(CellArgs ca, Scalars *sc, DevStats *stats, long long stats_cap) {
    __shared__ double g[17];
    const int warp = threadIdx.x >> 5, np = ca.K + 1;
    if (warp < np) {
        double v = warp_sum_partials(ca.part_tally, ca.nblk_cell, np, warp);
        if ((threadIdx.x & 31) == 0) g[warp] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) energycheck_done(ca, sc, stats, stats_cap, g, STEP);
}

// Finalize + tally per cell, then, in the block that finishes last, the
// energy check and the timestep: one launch for the step's tail.  Each
// block publishes its partial sums before taking a ticket; the last block
// sums every block's partials in block order (the same fixed order as
// k_energycheck, so the same values).
__global__ void __launch_bounds__(kCellThreads) k_tally_check(CellArgs ca, Scalars *sc, DevStats *stats,
                                                             long long stats_cap) {
    static_assert(kCellThreads == 32, "one-warp blocks");
    __shared__ DD sh[kCellThreads];
    __shared__ double g[17];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    finalize_cell(ca, sc, i);
    tally_cell(ca, sc, i, sh);
    __threadfence();
    unsigned ticket = 0;
    if (threadIdx.x == 0) ticket = atomicAdd(&sc->tally_blocks_done, 1u);
    ticket = __shfl_sync(0xFFFFFFFFu, ticket, 0);
    if (ticket != gridDim.x - 1u) return;
    __threadfence();
    const int np = ca.K + 1;
    for (int q = 0; q < np; ++q) {
        const double v = warp_sum_partials(ca.part_tally, ca.nblk_cell, np, q);
        if (threadIdx.x == 0) g[q] = v;
    }
    if (threadIdx.x == 0) {
        sc->tally_blocks_done = 0u;
        energycheck_done(ca, sc, stats, stats_cap, g, true);
    }
}

__global__ void k_timestep(CellArgs ca, Scalars *sc) { advance_clock(ca, sc); }

void launch_timestep(const CellArgs &ca, Scalars *sc, cudaStream_t st) { k_timestep<<<1, 1, 0, st>>>(ca, sc); }

void launch_energycheck(const CellArgs &ca, Scalars *sc, DevStats *stats, long long stats_cap, cudaStream_t st) {
    k_energycheck<false><<<1, 32 * (ca.K + 1), 0, st>>>(ca, sc, stats, stats_cap);
}

void launch_tally_check_timestep(const CellArgs &ca, Scalars *sc, DevStats *stats, long long stats_cap,
                                 cudaStream_t st) {
    k_tally_check<<<ca.nblk_cell, kCellThreads, 0, st>>>(ca, sc, stats, stats_cap);
}

// Transport of a list that was set directly (no sourcing this step): take the
// fixed-point exponents from the census maximum.
__global__ void k_prepare_transport(CellArgs ca, Scalars *sc) {
    const int ce = sc->emax_census_exp;
    const double emax = ce == kNoExp ? 0.0 : exp_top(ce);
    sc->emax = emax;
    sc->emax_census_exp = kNoExp;
    sc->segments = 0ull;
    sc->surrogate_calls = 0ull;
    sc->killed = 0ull;
    sc->work_next = 0ull;
    for (int r = 0; r <= 2 * kSurrRounds; ++r) sc->qcount[r] = 0ull;
    sc->n_census_in = sc->n_census;
    sc->n_sourced = 0;
    sc->birth_base = sc->n_particles;
    sc->b_dep = fix_exponent(emax / ca.vol_min);
    sc->b_lost = fix_exponent(emax);
    sc->b_rad = fix_exponent(emax);
}

void launch_prepare_transport(const CellArgs &ca, Scalars *sc, cudaStream_t st) {
    k_prepare_transport<<<1, 1, 0, st>>>(ca, sc);
}

}  // namespace imc
