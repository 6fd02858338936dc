/*
 * imc_oracle.cpp -- ORACLE.  Test infrastructure only: the test suite, the
 * smoke check and bench.py's CPU-baseline leg load it as the CHECKER of the
 * GPU engine.  Nothing in the product links, imports or calls it.
 *
 * A single-threaded CPU restatement of the per-timestep particle path of
 * MixedPrecisionIMC.jl, one function per reference function, each citing the
 * reference lines it follows (paths are relative to the reference project):
 *
 *   orc_update      <- Update.update            src/imc_update.jl:12-56
 *   sorter          <- Utilities.sorter         src/imc_utilities.jl:23-54
 *   orc_sourcing    <- Sourcing.sourcing        src/imc_sourcing.jl:23-367
 *   transport_1d    <- Transport.MC             src/imc_transport.jl:13-210
 *   transport_2d    <- Transport.MC2D           src/imc_transport.jl:483-732
 *   orc_clean       <- Clean.clean              src/imc_clean.jl:6-19
 *   orc_tally       <- Tally.tally              src/imc_tally.jl:22-142
 *   orc_energycheck <- EnergyCheck.energychecker src/imc_energycheck.jl:19-38
 *   orc_timestep    <- timestep                 src/MixedPrecisionIMC.jl:181-222
 *
 * Parity status: the reference is Julia and cannot run in this build
 * environment, and its own tests (test/runtests.jl) hold no numeric golden
 * vectors, so this restatement is "parity unpinned" against reference runs.
 * It is pinned instead by the reference tests' structural checks, by closed-
 * form known answers (Fleck factor, emission, surface flux, attenuation,
 * energy balance) and by the benchmark curves carried in the reference decks.
 *
 * Deliberate, documented differences from the reference:
 *   - RNG: Julia's global Xoshiro stream is replaced by Philox-4x32-10 keyed
 *     (SEED, step, particle index, stage), identical to the GPU kernels, so a
 *     history here and on the GPU consume the same variates.  randexp() is
 *     -log(v), v uniform on (0,1) (the reference uses a ziggurat: same law).
 *   - Mesh-side arithmetic (update, sourcing energies, tally) is FP64 for every
 *     PRECISION; particle arithmetic follows PRECISION.  The energy-scale
 *     choice of sorter is still evaluated in the deck precision.
 *   - Tally sums are double-double (effectively exact) instead of Julia's
 *     sequential or pairwise `sum`; they differ only by rounding.
 *   - A history whose distance turns NaN is killed and flagged instead of
 *     looping; a history stops at a segment cap and is flagged.
 *   - FP32 particle arithmetic in 1D and 2D transport takes the kernels' shorter
 *     formulation of the same quantities: collision distance -log(v)/seff as
 *     -log(v) * (1/seff), the weight after a segment E exp(-a) as
 *     E + E expm1(-a) (the deposit uses the same expm1, so attenuation and
 *     deposit add up to E; expm1 of |a| <= 1/16 as the kernels' Taylor series
 *     to a^7, expm1_seg), and reciprocals of dx and ds*c instead of
 *     divisions (also 1/mu, set at each new direction, for the face
 *     distance).  They differ from the reference's FP32 evaluation by
 *     roundings only; FP64 keeps the reference's expressions.
 */
#include "../include/imc.h"
#include "philox.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include <chrono>

/* e^x - 1 of the kernels' FP32 segment arithmetic: the Taylor series to x^7
 * in Horner form with fused multiply-adds for |x| <= 1/16, expm1f beyond. */
static float expm1_seg(float x) {
    if (std::fabs(x) <= 0.0625f) {
        float p = std::fma(x, 1.0f / 5040.0f, 1.0f / 720.0f);
        p = std::fma(p, x, 1.0f / 120.0f);
        p = std::fma(p, x, 1.0f / 24.0f);
        p = std::fma(p, x, 1.0f / 6.0f);
        p = std::fma(p, x, 0.5f);
        return std::fma(p * x, x, x);
    }
    return std::expm1(x);
}

/* exported for the CPU test of its error bound */
extern "C" float orc_expm1_seg(float x) { return expm1_seg(x); }

namespace {

const double kPi = 3.141592653589793;  /* Float64(pi) */

/* Julia's min(x, y) for floats: NaN-propagating (base/math.jl). */
template <class T> inline T jmin(T a, T b) {
    if (a != a) return a;
    if (b != b) return b;
    return b < a ? b : a;
}

/* Julia isless for floats: NaN after everything, -0.0 before 0.0. */
inline bool jisless(double a, double b) {
    bool an = a != a, bn = b != b;
    if (an || bn) return !an && bn;
    if (a < b) return true;
    if (a == b) return std::signbit(a) && !std::signbit(b);
    return false;
}

/* double-double accumulator (TwoSum) */
struct DD {
    double hi = 0.0, lo = 0.0;
    void add(double x) {
        double s = hi + x;
        double bp = s - hi;
        double e = (hi - (s - bp)) + (x - bp);
        hi = s;
        lo += e;
    }
    double val() const { return hi + lo; }
};

/* Utilities.sorter (src/imc_utilities.jl:23-54): for each energy scale in turn,
 * append it to the factors, sort ascending, multiply the smallest by the
 * largest pairwise, and keep the first scale whose product is finite in the
 * selection precision P.  The product returned is the FP64 pairwise product. */
template <class P>
double sorter(const double *vals, int n, const double *scales, int nsc, double *scale_out, int *j_out) {
    double arr[32];
    for (int j = 0; j < nsc; ++j) {
        int m = n + 1;
        for (int i = 0; i < n; ++i) arr[i] = vals[i];
        arr[n] = scales[j];
        std::stable_sort(arr, arr + m, jisless);
        double prod = 1.0;
        P prodp = (P)1.0;
        for (int i = 0; i < m / 2; ++i) {
            prod *= arr[i] * arr[m - 1 - i];
            prodp = (P)(prodp * (P)((P)arr[i] * (P)arr[m - 1 - i]));
        }
        if (m & 1) {
            prod *= arr[m / 2];
            prodp = (P)(prodp * (P)arr[m / 2]);
        }
        double chk = (double)prodp;
        if (std::isfinite(chk) && std::isfinite(prod)) {
            if (scale_out) *scale_out = scales[j];
            if (j_out) *j_out = j;
            return prod;
        }
    }
    if (scale_out) *scale_out = 0.0;
    if (j_out) *j_out = -1;
    return 0.0;
}

double sorter_sel(int prec, const double *vals, int n, const double *scales, int nsc, double *scale_out, int *j_out) {
    if (prec == IMC_FP32) return sorter<float>(vals, n, scales, nsc, scale_out, j_out);
    if (prec == IMC_FP16) return sorter<_Float16>(vals, n, scales, nsc, scale_out, j_out);
    return sorter<double>(vals, n, scales, nsc, scale_out, j_out);
}

/* Julia round(x): nearest, ties to even */
inline double jround(double x) { return std::nearbyint(x); }

/* Particle as stored.  FP64/FP32: physical values (rounded to the state
 * type).  FP16: x holds x/(dx*ds), t holds t/dt, E holds E/E0, each rounded to
 * binary16; E0 is binary32.  2D direction: ux, uy (state type); the reference's
 * angle is kept in ang for the 2D restatement. */
struct OP {
    double t, x, y, mu, ux, uy, ang, E, E0;
    int32_t cell, k;
    bool alive;
};

struct Sim {
    ImcDeck d;
    int nx, ny, nc, K;
    std::vector<double> dx, dy, temp, bee, beta, fleck, sa, ss;
    std::vector<double> sa_val, sa_pow, ss_val, ss_pow, radsource, tsurf, scales;
    std::vector<double> energydep, emitted, radenergydens, matenergydens;
    double totalenergy = 0, totalenergydep = 0, lostenergy = 0, radenergyold = 0;
    double t = 0, dt = 0;
    int64_t step = 0;
    bool finished = false;
    std::vector<OP> parts;
    /* per-step bookkeeping */
    int64_t n_census_in = 0, n_sourced = 0, segments = 0;
    uint32_t flags = 0;
    double last_err = 0, last_rad = 0, last_radold = 0, last_lost = 0;
    ImcStepStats last{};
    std::vector<DD> lost_k;   /* per scale, this step */
    std::vector<DD> dep_acc;  /* per slot k*nc+c, this step */
    bool transported = false;
};

inline double Kscale(const Sim &s, int k) { return s.scales[k]; }

/* ---------------------------------------------------------------- update */
/* Update.update (src/imc_update.jl:12-56), FP64. */
void orc_update_impl(Sim &s) {
    const double a = s.d.phys_a, c = s.d.phys_c;
    const double one[1] = {1.0};
    for (int i = 0; i < s.nc; ++i) {
        double T = s.temp[i];
        double T3 = T * T * T;
        if (s.d.linearized) {
            s.bee[i] = (4.0 * a) * T3;
            s.beta[i] = 1.0;
        } else {
            s.beta[i] = ((4.0 * a) * T3) / s.bee[i];
        }
        double Tc = (s.d.temp_floor > 0.0 && T < s.d.temp_floor) ? s.d.temp_floor : T;
        s.sa[i] = s.sa_val[i] * std::pow(Tc, s.sa_pow[i]);
        if (s.d.marshak_opacity) s.sa[i] = s.sa_val[i] / Tc / Tc / Tc;
        s.ss[i] = s.ss_val[i] * std::pow(Tc, s.ss_pow[i]);
        double v[6] = {s.d.distancescale, s.d.alpha, s.beta[i], c, s.dt, s.sa[i]};
        double prod = sorter<double>(v, 6, one, 1, nullptr, nullptr);
        s.fleck[i] = 1.0 / (1.0 + prod);
    }
}

/* --------------------------------------------------------------- helpers */
template <class T> struct RandT;
template <> struct RandT<double> {
    static double rand(OrcStream *s) { return orc_rand_f64(s); }
    static double randexp(OrcStream *s) { return orc_randexp_f64(s); }
};
template <> struct RandT<float> {
    static float rand(OrcStream *s) { return orc_rand_f32(s); }
    static float randexp(OrcStream *s) { return orc_randexp_f32(s); }
};

/* state rounding for storage */
inline double h16(double v) { return (double)(_Float16)v; }

/* ------------------------------------------------------------- sourcing */
struct SourceSlot {
    int64_t count;
    int kind;   /* 0 surf L, 1 surf R (1D); 10 bottom, 11 top, 12 left, 13 right (2D); 2 body; 3 rad */
    int idx;    /* cell or face-segment index */
    double nrg; /* per-particle energy (deck arithmetic, FP64) */
    int k;      /* scale index */
};

template <class T>
void store_new_particle(Sim &s, OP &p, T t, T x, T y, T mu, T ux, T uy, double ang, T E, int cell, int k) {
    p.alive = true;
    p.cell = cell;
    p.k = k;
    p.ang = ang;
    p.E0 = (double)E;
    if (s.d.precision == IMC_FP16) {
        int ix = s.d.geometry == IMC_GEOM_1D ? cell : cell % s.nx;
        float dxs = (float)s.dx[ix] * (float)s.d.distancescale;
        p.x = h16((double)((float)x / dxs));
        if (s.d.geometry == IMC_GEOM_2D) {
            int iy = cell / s.nx;
            float dys = (float)s.dy[iy] * (float)s.d.distancescale;
            p.y = h16((double)((float)y / dys));
        } else p.y = 0;
        p.t = h16((double)((float)t / (float)s.dt));
        p.mu = h16((double)mu);
        p.ux = h16((double)ux);
        p.uy = h16((double)uy);
        p.E = h16(1.0);
        p.E0 = (double)(float)E;
    } else {
        p.t = (double)t; p.x = (double)x; p.y = (double)y; p.mu = (double)mu;
        p.ux = (double)ux; p.uy = (double)uy; p.E = (double)E;
    }
}

/* Sourcing.sourcing (src/imc_sourcing.jl:23-367) with particle math in T. */
template <class T>
void orc_sourcing_impl(Sim &s) {
    const int K = s.K;
    const double *sc = s.scales.data();
    const int sp = s.d.scale_select_precision;
    const double a = s.d.phys_a, c = s.d.phys_c, ds = s.d.distancescale, dt = s.dt;
    const int nc = s.nc;
    std::vector<double> e_body(nc), sb(nc), e_rad(nc), sr(nc);
    std::vector<int> jb(nc), jr(nc);
    std::fill(s.emitted.begin(), s.emitted.end(), 0.0);
    std::vector<SourceSlot> slots;
    double e_surface = 0.0;
    DD surf_sum;
    /* surface energies */
    std::vector<double> e_sf, s_sf;
    std::vector<int> j_sf, kind_sf, idx_sf;
    if (s.d.geometry == IMC_GEOM_1D) {
        for (int side = 0; side < 2; ++side) {
            double Ts = s.tsurf[side];
            double v[8] = {a, c, Ts, Ts, Ts, Ts, dt, 0.25};
            double sv; int j;
            double e = sorter_sel(sp, v, 8, sc, K, &sv, &j);
            e_sf.push_back(e); s_sf.push_back(sv); j_sf.push_back(j);
            kind_sf.push_back(side); idx_sf.push_back(side == 0 ? 0 : s.nx - 1);
        }
        e_surface = (e_sf[0] / s_sf[0]) + (e_sf[1] / s_sf[1]);
    } else {
        /* bottom, top over x; left, right over y (src/imc_sourcing.jl:86-95) */
        const int nfx = s.nx, nfy = s.ny;
        for (int face = 0; face < 4; ++face) {
            int nseg = face < 2 ? nfx : nfy;
            const double *Tf = s.tsurf.data() + (face == 0 ? 0 : face == 1 ? nfx : face == 2 ? 2 * nfx : 2 * nfx + nfy);
            DD fs;
            for (int i = 0; i < nseg; ++i) {
                double Ts = Tf[i];
                double w = face < 2 ? s.dx[i] : s.dy[i];
                double v[9] = {a, c, Ts, Ts, Ts, Ts, w, dt, 0.25};
                double sv; int j;
                double e = sorter_sel(sp, v, 9, sc, K, &sv, &j);
                e_sf.push_back(e); s_sf.push_back(sv); j_sf.push_back(j);
                kind_sf.push_back(10 + face); idx_sf.push_back(i);
                fs.add(e / sv);
            }
            e_surface += fs.val();
        }
    }
    DD sum_body, sum_rad;
    for (int i = 0; i < nc; ++i) {
        int ix = s.d.geometry == IMC_GEOM_1D ? i : i % s.nx;
        int iy = s.d.geometry == IMC_GEOM_1D ? 0 : i / s.nx;
        double Tk = s.temp[i], f = s.fleck[i], sa = s.sa[i];
        double sv; int j;
        if (s.d.geometry == IMC_GEOM_1D) {
            double vb[11] = {f, sa, a, c, Tk, Tk, Tk, Tk, s.dx[i], dt, ds};
            e_body[i] = sorter_sel(sp, vb, 11, sc, K, &sb[i], &jb[i]);
            double vr[3] = {s.radsource[i], s.dx[i], dt};
            e_rad[i] = sorter_sel(sp, vr, 3, sc, K, &sr[i], &jr[i]);
        } else {
            double vb[12] = {f, sa, a, c, Tk, Tk, Tk, Tk, s.dx[ix], s.dy[iy], dt, ds};
            e_body[i] = sorter_sel(sp, vb, 12, sc, K, &sb[i], &jb[i]);
            double vr[4] = {s.radsource[i], s.dx[ix], s.dy[iy], dt};
            e_rad[i] = sorter_sel(sp, vr, 4, sc, K, &sr[i], &jr[i]);
        }
        double ve[10] = {f, sa, a, c, Tk, Tk, Tk, Tk, dt, ds};
        double em = sorter_sel(sp, ve, 10, sc, K, &sv, &j);
        if (j >= 0) s.emitted[(size_t)j * nc + i] = em;
        if (jb[i] < 0 || jr[i] < 0 || j < 0) s.flags |= IMC_FLAG_FIXPOINT_RANGE;
        sum_body.add(e_body[i] / sb[i]);
        sum_rad.add(e_rad[i] / sr[i]);
    }
    s.totalenergy = sum_body.val() + sum_rad.val() + e_surface;
    const double E = s.totalenergy;

    /* particle budget (src/imc_sourcing.jl:132-136) on the live census;
     * length(Ncells) is 1 in 1D, 2 in 2D */
    int64_t n_census = 0;
    for (const OP &q : s.parts) n_census += q.alive ? 1 : 0;
    double n_source = (double)s.d.n_input;
    if (s.d.n_input + n_census > s.d.n_max) {
        double lenN = s.d.geometry == IMC_GEOM_1D ? 1.0 : 2.0;
        n_source = std::max(s.d.cellmin, (double)(s.d.n_max - n_census) - lenN - 1.0);
    }
    s.n_census_in = n_census;
    if (!(E > 0.0) || !std::isfinite(E)) {
        s.flags |= IMC_FLAG_NO_ENERGY;
        s.n_sourced = 0;
        return;
    }
    auto cnt = [&](double e, double sv, bool withmin) -> int64_t {
        double r = jround(((e / sv) * n_source) / E);
        if (withmin) r = std::max(r, s.d.cellmin);
        return (int64_t)r;
    };
    std::vector<int64_t> n_body(nc), n_rad(nc);
    for (int i = 0; i < nc; ++i) {
        n_body[i] = cnt(e_body[i], sb[i], true);
        n_rad[i] = e_rad[i] > 0 ? cnt(e_rad[i], sr[i], true) : 0;
    }
    /* slots in the reference's push! order */
    for (size_t q = 0; q < e_sf.size(); ++q) {
        int64_t n = 0;
        if (e_sf[q] > 0) n = cnt(e_sf[q], s_sf[q], s.d.geometry == IMC_GEOM_2D);
        SourceSlot sl{n, kind_sf[q], idx_sf[q], n > 0 ? (double)(T)(e_sf[q] / (double)n) : 0.0, j_sf[q]};
        slots.push_back(sl);
    }
    for (int i = 0; i < nc; ++i) {
        if (n_body[i] <= 0) continue;
        slots.push_back(SourceSlot{n_body[i], 2, i, (double)(T)(e_body[i] / (double)n_body[i]), jb[i]});
    }
    for (int i = 0; i < nc; ++i) {
        if (n_rad[i] <= 0) continue;
        /* 2D births n_body particles per source cell (src/imc_sourcing.jl:357) */
        int64_t n = s.d.geometry == IMC_GEOM_1D ? n_rad[i] : n_body[i];
        slots.push_back(SourceSlot{n, 3, i, (double)(T)(e_rad[i] / (double)n_rad[i]), jr[i]});
    }
    int64_t total = 0;
    for (auto &sl : slots) total += sl.count;
    s.n_sourced = total;
    const T dtT = (T)dt, dsT = (T)ds;
    int64_t pid = (int64_t)s.parts.size();  /* births follow the list, holes included */
    s.parts.reserve(s.parts.size() + total);
    for (auto &sl : slots) {
        for (int64_t q = 0; q < sl.count; ++q, ++pid) {
            OrcStream rs;
            orc_stream_init(&rs, s.d.seed, (uint32_t)s.step, (uint32_t)pid, ORC_STAGE_SOURCE);
            OP p{};
            T E0 = (T)sl.nrg;
            if (s.d.geometry == IMC_GEOM_1D) {
                if (sl.kind == 0 || sl.kind == 1) {
                    /* src/imc_sourcing.jl:161-189 */
                    int cell = sl.kind == 0 ? 0 : s.nx - 1;
                    double frac = sl.kind == 0 ? 0.01 : 0.99;
                    T xpos = (T)(frac * (double)(T)s.dx[cell] * (double)dsT);
                    T mu = (T)0;
                    for (int r = 0; r < 64 && mu == (T)0; ++r) {
                        T rr = std::sqrt(RandT<T>::rand(&rs));
                        mu = sl.kind == 0 ? rr : -rr;
                    }
                    if (mu == (T)0) mu = sl.kind == 0 ? (T)1 : (T)-1;
                    T st = dtT * RandT<T>::rand(&rs);
                    store_new_particle<T>(s, p, st, xpos, (T)0, mu, (T)0, (T)0, 0.0, E0, cell, sl.k);
                } else {
                    /* body / radiation source: src/imc_sourcing.jl:193-236 */
                    int cell = sl.idx;
                    T xpos = (T)s.dx[cell] * RandT<T>::rand(&rs) * dsT;
                    T mu = (T)0;
                    for (int r = 0; r < 64 && mu == (T)0; ++r) mu = (T)1 - (T)2 * RandT<T>::rand(&rs);
                    if (mu == (T)0) mu = (T)1;
                    T st = dtT * RandT<T>::rand(&rs);
                    store_new_particle<T>(s, p, st, xpos, (T)0, mu, (T)0, (T)0, 0.0, E0, cell, sl.k);
                }
            } else {
                T st, xpos, ypos, ang;
                int ix, iy;
                const double pd = kPi;
                if (sl.kind >= 10) {
                    /* surfaces: src/imc_sourcing.jl:265-323 */
                    int face = sl.kind - 10;
                    st = dtT * RandT<T>::rand(&rs);
                    if (face == 0 || face == 1) {
                        ix = sl.idx;
                        iy = face == 0 ? 0 : s.ny - 1;
                        xpos = (T)s.dx[ix] * RandT<T>::rand(&rs) * dsT;
                        ypos = face == 0 ? (T)(0.001 * (double)(T)s.dy[0] * (double)dsT)
                                         : (T)(0.999 * (double)(T)s.dy[s.ny - 1] * (double)dsT);
                        T u = RandT<T>::rand(&rs);
                        ang = face == 0 ? (T)((T)pd * u) : (T)(-pd * (double)u);
                    } else {
                        iy = sl.idx;
                        ix = face == 2 ? 0 : s.nx - 1;
                        xpos = face == 2 ? (T)(0.001 * (double)(T)s.dx[0] * (double)dsT)
                                         : (T)(0.999 * (double)(T)s.dx[s.nx - 1] * (double)dsT);
                        /* the reference scales y by mesh.dx[j] here (src/imc_sourcing.jl:301,316) */
                        double wq = iy < s.nx ? s.dx[iy] : s.dy[iy];
                        ypos = (T)wq * RandT<T>::rand(&rs) * dsT;
                        T u = RandT<T>::rand(&rs);
                        ang = face == 2 ? (T)(pd * (0.5 - (double)u)) : (T)(pd * (0.5 + (double)u));
                    }
                } else {
                    /* body / source: src/imc_sourcing.jl:326-366 */
                    ix = sl.idx % s.nx;
                    iy = sl.idx / s.nx;
                    xpos = (T)s.dx[ix] * RandT<T>::rand(&rs) * dsT;
                    ypos = (T)s.dy[iy] * RandT<T>::rand(&rs) * dsT;
                    ang = (T)(2.0 * pd * (double)RandT<T>::rand(&rs));
                    st = dtT * RandT<T>::rand(&rs);
                }
                T ux = std::cos(ang), uy = std::sin(ang);
                store_new_particle<T>(s, p, st, xpos, ypos, (T)0, ux, uy, (double)ang, E0, ix + iy * s.nx, sl.k);
            }
            s.parts.push_back(p);
        }
    }
}

/* ------------------------------------------------------------- transport */
inline void dep_add(Sim &s, int k, int cell, double v) {
    if (!(v >= 0.0)) {
        s.flags |= (v != v) ? IMC_FLAG_NAN : IMC_FLAG_NEG_TALLY;
        return;
    }
    s.dep_acc[(size_t)k * s.nc + cell].add(v);
}

/* Transport.MC (src/imc_transport.jl:13-210) with particle arithmetic in T.
 * FP16 state (Half = true) loads binary16 fields into T = float. */
template <class T, bool Half>
void transport_1d(Sim &s) {
    const int N = s.nx;
    const T endsteptime = (T)s.dt, c = (T)s.d.phys_c, ds = (T)s.d.distancescale;
    const int64_t cap = s.d.segment_cap > 0 ? s.d.segment_cap : 10000000;
    std::vector<T> saf(N), seff(N), dxs(N), dxT(N), rseff(N), rdxT(N);
    for (int i = 0; i < N; ++i) {
        T sa = (T)s.sa[i], f = (T)s.fleck[i], ss = (T)s.ss[i];
        saf[i] = sa * f;
        seff[i] = sa * ((T)1 - f) + ss;
        dxT[i] = (T)s.dx[i];
        dxs[i] = dxT[i] * ds;
        rseff[i] = (T)1 / seff[i];
        rdxT[i] = (T)1 / dxT[i];
    }
    // FP32 evaluates the segment with the kernels' formulation: collision
    // distance -log(v) * (1/seff), weight E + E expm1(-sigma_a f d) (one
    // transcendental for attenuation and deposit), reciprocals for divisions.
    // FP64 evaluates the reference's expressions as written.
    constexpr bool kF32 = sizeof(T) == 4;
    const T rdsc = (T)1 / (ds * c);
    for (size_t pi = 0; pi < s.parts.size(); ++pi) {
        OP &p = s.parts[pi];
        if (!p.alive) continue;
        OrcStream rs;
        orc_stream_init(&rs, s.d.seed, (uint32_t)s.step, (uint32_t)pi, ORC_STAGE_TRANSPORT);
        int cell = p.cell, k = p.k;
        T currenttime, position, mu, energy, startenergy;
        if (Half) {
            currenttime = (T)((float)p.t * (float)endsteptime);
            position = (T)((float)p.x * (float)dxs[cell]);
            mu = (T)p.mu;
            startenergy = (T)p.E0;
            energy = (T)((float)p.E * (float)p.E0);
        } else {
            currenttime = (T)p.t; position = (T)p.x; mu = (T)p.mu;
            energy = (T)p.E; startenergy = (T)p.E0;
        }
        const T minenergy = (T)(0.01 * (double)startenergy);
        int64_t seg = 0;
        T rmu = (T)1 / mu;
        while (true) {
            ++s.segments;
            if (++seg > cap) { s.flags |= IMC_FLAG_SEGMENT_CAP; p.alive = false; break; }
            T dist_b = kF32 ? (mu > (T)0 ? (dxs[cell] - position) * rmu : std::fabs(position * rmu))
                            : (mu > (T)0 ? (dxs[cell] - position) / mu : std::fabs(position / mu));
            T dist_col = kF32 ? RandT<T>::randexp(&rs) * rseff[cell] : RandT<T>::randexp(&rs) / seff[cell];
            T dist_cen = c * (endsteptime - currenttime) * ds;
            T dist = jmin(jmin(dist_b, dist_col), dist_cen);
            if (dist != dist) { s.flags |= IMC_FLAG_NAN; p.alive = false; break; }
            T newenergy, dep;
            if (kF32) {
                const T em1 = (T)expm1_seg((float)(-saf[cell] * dist));
                newenergy = energy + energy * em1;
                dep = -(energy * rdxT[cell]) * em1;
            } else {
                newenergy = energy * std::exp(-saf[cell] * dist);
                dep = -(energy / dxT[cell]) * std::expm1(-saf[cell] * dist);
            }
            if (newenergy <= minenergy) {
                dep_add(s, k, cell, (double)(kF32 ? energy * rdxT[cell] : energy / dxT[cell]));
                p.alive = false;
                break;
            }
            dep_add(s, k, cell, (double)dep);
            position += mu * dist;
            if (kF32) currenttime += dist * rdsc;
            else currenttime += (dist / ds) / c;
            energy = newenergy;
            if (dist == dist_b) {
                if (mu > (T)0) {
                    if (cell == N - 1) {
                        if (s.d.bc[IMC_RIGHT] == IMC_BC_REFLECT) {
                            mu = -mu;
                            rmu = -rmu;
                        } else {
                            s.lost_k[k].add((double)energy);
                            p.alive = false;
                            break;
                        }
                    }
                    cell += 1;
                    position = (T)0;
                }
                if (mu < (T)0) {
                    if (cell == 0) {
                        if (s.d.bc[IMC_LEFT] == IMC_BC_REFLECT) {
                            mu = -mu;
                            rmu = -rmu;
                        } else {
                            s.lost_k[k].add((double)energy);
                            p.alive = false;
                            break;
                        }
                    } else {
                        cell -= 1;
                        position = dxs[cell];
                    }
                }
            }
            if (dist == dist_col) {
                mu = (T)0;
                for (int r = 0; r < 64 && mu == (T)0; ++r) mu = (T)1 - (T)2 * RandT<T>::rand(&rs);
                if (mu == (T)0) mu = (T)1;
                rmu = (T)1 / mu;
            }
            if (dist == dist_cen) {
                p.cell = cell;
                if (Half) {
                    p.t = 0.0;
                    p.x = h16((double)((float)position / (float)dxs[cell]));
                    p.mu = h16((double)mu);
                    p.E = h16((double)((float)energy / (float)startenergy));
                } else {
                    p.t = 0.0; p.x = (double)position; p.mu = (double)mu; p.E = (double)energy;
                }
                break;
            }
        }
    }
}

/* Transport.MC2D (src/imc_transport.jl:483-732), particle arithmetic in T.
 * The direction is kept as the reference keeps it, an angle whose cosine and
 * sine are taken at every segment; reflections go through atan. */
template <class T, bool Half>
void transport_2d(Sim &s) {
    const int NX = s.nx, NY = s.ny;
    const T c = (T)s.d.phys_c, ds = (T)s.d.distancescale, dtT = (T)s.dt;
    const int64_t cap = s.d.segment_cap > 0 ? s.d.segment_cap : 10000000;
    std::vector<T> saf(s.nc), seff(s.nc), rseff(s.nc), rarea(s.nc), dxT(NX), dyT(NY), dxs(NX), dys(NY);
    for (int i = 0; i < s.nc; ++i) {
        T sa = (T)s.sa[i], f = (T)s.fleck[i], ss = (T)s.ss[i];
        saf[i] = sa * f;
        seff[i] = sa * ((T)1 - f) + ss;
        rseff[i] = (T)1 / seff[i];
        rarea[i] = (T)1 / ((T)s.dx[i % NX] * (T)s.dy[i / NX]);
    }
    // FP32: the kernels' shorter formulation (as in transport_1d)
    constexpr bool kF32 = sizeof(T) == 4;
    const T rdsc = (T)1 / (ds * c);
    for (int i = 0; i < NX; ++i) { dxT[i] = (T)s.dx[i]; dxs[i] = dxT[i] * ds; }
    for (int j = 0; j < NY; ++j) { dyT[j] = (T)s.dy[j]; dys[j] = dyT[j] * ds; }
    for (size_t pi = 0; pi < s.parts.size(); ++pi) {
        OP &p = s.parts[pi];
        if (!p.alive) continue;
        OrcStream rs;
        orc_stream_init(&rs, s.d.seed, (uint32_t)s.step, (uint32_t)pi, ORC_STAGE_TRANSPORT);
        int xi = p.cell % NX, yi = p.cell / NX, k = p.k;
        T t, xp, yp, energy, startenergy, mu;
        if (Half) {
            t = (T)((float)p.t * (float)dtT);
            xp = (T)((float)p.x * (float)dxs[xi]);
            yp = (T)((float)p.y * (float)dys[yi]);
            startenergy = (T)p.E0;
            energy = (T)((float)p.E * (float)p.E0);
        } else {
            t = (T)p.t; xp = (T)p.x; yp = (T)p.y; energy = (T)p.E; startenergy = (T)p.E0;
        }
        mu = (T)p.ang;
        const T minenergy = (T)(0.01 * (double)startenergy);
        int64_t seg = 0;
        while (true) {
            ++s.segments;
            if (++seg > cap) { s.flags |= IMC_FLAG_SEGMENT_CAP; p.alive = false; break; }
            T vx = std::cos(mu), vy = std::sin(mu);
            T dist_bx = vx > (T)0 ? std::fabs((dxs[xi] - xp) / vx) : std::fabs(xp / vx);
            T dist_by = vy > (T)0 ? std::fabs((dys[yi] - yp) / vy) : std::fabs(yp / vy);
            T dist_b;
            if (dist_bx != dist_bx) dist_b = dist_by;
            else if (dist_by != dist_by) dist_b = dist_bx;
            else dist_b = jmin(dist_bx, dist_by);
            int cell = xi + yi * NX;
            T dist_col = kF32 ? RandT<T>::randexp(&rs) * rseff[cell] : RandT<T>::randexp(&rs) / seff[cell];
            T dist_cen = c * (dtT - t) * ds;
            T dist = jmin(jmin(dist_b, dist_col), dist_cen);
            if (dist != dist) { s.flags |= IMC_FLAG_NAN; p.alive = false; break; }
            const T edens = kF32 ? energy * rarea[cell] : (energy / dxT[xi]) / dyT[yi];
            T newenergy, dep;
            if (kF32) {
                const T em1 = (T)expm1_seg((float)(-saf[cell] * dist));
                newenergy = energy + energy * em1;
                dep = -edens * em1;
            } else {
                newenergy = energy * std::exp(-saf[cell] * dist);
                dep = -edens * std::expm1(-saf[cell] * dist);
            }
            if (newenergy <= minenergy) {
                dep_add(s, k, cell, (double)edens);
                p.alive = false;
                break;
            }
            dep_add(s, k, cell, (double)dep);
            xp += dist * vx;
            yp += dist * vy;
            if (kF32) t += dist * rdsc;
            else t += (dist / ds) / c;
            energy = newenergy;
            if (dist == dist_bx || dist == dist_by) {
                bool killed = false;
                if (dist_bx < dist_by) {
                    if (vx > (T)0) {
                        if (xi == NX - 1) {
                            if (s.d.bc[IMC_RIGHT] == IMC_BC_REFLECT) mu = std::atan2(vy, -vx);
                            else { s.lost_k[k].add((double)energy); killed = true; }
                            if (killed) { p.alive = false; break; }
                            continue;
                        }
                        xi += 1; xp = (T)0;
                    } else {
                        if (xi == 0) {
                            if (s.d.bc[IMC_LEFT] == IMC_BC_REFLECT) mu = std::atan2(vy, -vx);
                            else { s.lost_k[k].add((double)energy); killed = true; }
                            if (killed) { p.alive = false; break; }
                            continue;
                        }
                        xi -= 1; xp = dxs[xi];
                    }
                } else {
                    if (vy > (T)0) {
                        if (yi == NY - 1) {
                            if (s.d.bc[IMC_TOP] == IMC_BC_REFLECT) mu = std::atan2(-vy, vx);
                            else { s.lost_k[k].add((double)energy); killed = true; }
                            if (killed) { p.alive = false; break; }
                            continue;
                        }
                        yi += 1; yp = (T)0;
                    } else {
                        if (yi == 0) {
                            if (s.d.bc[IMC_BOTTOM] == IMC_BC_REFLECT) mu = std::atan2(-vy, vx);
                            else { s.lost_k[k].add((double)energy); killed = true; }
                            if (killed) { p.alive = false; break; }
                            continue;
                        }
                        yi -= 1; yp = dys[yi];
                    }
                }
                continue;
            }
            if (dist == dist_col) mu = (T)(2.0 * kPi * (double)RandT<T>::rand(&rs));
            if (dist == dist_cen) {
                p.cell = xi + yi * NX;
                p.ang = (double)mu;
                T ux = std::cos(mu), uy = std::sin(mu);
                if (Half) {
                    p.t = 0.0;
                    p.x = h16((double)((float)xp / (float)dxs[xi]));
                    p.y = h16((double)((float)yp / (float)dys[yi]));
                    p.ux = h16((double)ux); p.uy = h16((double)uy);
                    p.E = h16((double)((float)energy / (float)startenergy));
                } else {
                    p.t = 0.0; p.x = (double)xp; p.y = (double)yp;
                    p.ux = (double)ux; p.uy = (double)uy; p.E = (double)energy;
                }
                break;
            }
        }
    }
}

void orc_transport_impl(Sim &s) {
    s.dep_acc.assign((size_t)s.K * s.nc, DD());
    s.lost_k.assign(s.K, DD());
    s.segments = 0;
    bool two = s.d.geometry == IMC_GEOM_2D;
    if (s.d.precision == IMC_FP64) { if (two) transport_2d<double, false>(s); else transport_1d<double, false>(s); }
    else if (s.d.precision == IMC_FP32) { if (two) transport_2d<float, false>(s); else transport_1d<float, false>(s); }
    else { if (two) transport_2d<float, true>(s); else transport_1d<float, true>(s); }
    for (size_t i = 0; i < s.energydep.size(); ++i) s.energydep[i] = s.dep_acc[i].val();
    double lost = 0.0;
    for (int k = 0; k < s.K; ++k) lost += s.lost_k[k].val() / s.scales[k];
    s.lostenergy += lost;
    s.transported = true;
}

/* Clean.clean (src/imc_clean.jl:6-19): drop killed particles, keep order. */
void orc_clean_impl(Sim &s) {
    size_t w = 0;
    for (size_t r = 0; r < s.parts.size(); ++r)
        if (s.parts[r].alive) s.parts[w++] = s.parts[r];
    s.parts.resize(w);
}

/* The engine's whole-step list policy: killed particles stay in the list as
 * holes until they exceed 1/16 of its length, then the list is compacted as
 * Clean.clean does.  Births are appended after the holes, so a history's list
 * index -- the key of its random stream -- is the same here and on the GPU. */
void step_clean(Sim &s) {
    int64_t len = (int64_t)s.parts.size(), live = 0;
    for (const OP &q : s.parts) live += q.alive ? 1 : 0;
    if ((len - live) * 16 > len) orc_clean_impl(s);
}

int64_t live_count(const Sim &s) {
    int64_t n = 0;
    for (const OP &q : s.parts) n += q.alive ? 1 : 0;
    return n;
}

/* physical energy of a stored particle */
inline double part_energy(const Sim &s, const OP &p) {
    if (s.d.precision == IMC_FP16) return (double)((float)p.E * (float)p.E0);
    return p.E;
}

/* Tally.tally (src/imc_tally.jl:22-142), FP64. */
void orc_tally_impl(Sim &s) {
    const double a = s.d.phys_a, c = s.d.phys_c;
    const int nc = s.nc;
    const double one[1] = {1.0};
    if (s.t == 0.0) {
        for (int i = 0; i < nc; ++i) {
            double T = s.temp[i];
            double v[10] = {s.fleck[i], s.sa[i], a, c, T, T, T, T, s.dt, s.d.distancescale};
            s.matenergydens[i] = sorter<double>(v, 10, one, 1, nullptr, nullptr);
        }
    }
    std::vector<double> inc(nc, 0.0);
    double totdep = 0.0;
    for (int k = 0; k < s.K; ++k) {
        DD sum;
        for (int i = 0; i < nc; ++i) {
            double dep = s.energydep[(size_t)k * nc + i];
            double em = s.emitted[(size_t)k * nc + i];
            inc[i] += (dep - em) / s.scales[k];
            double area = s.d.geometry == IMC_GEOM_1D ? s.dx[i] : (s.dx[i % s.nx] * s.dy[i / s.nx]);
            sum.add((dep * area) / s.scales[k]);
        }
        totdep += sum.val();
    }
    s.totalenergydep = totdep;
    for (int i = 0; i < nc; ++i) {
        s.matenergydens[i] += inc[i];
        if (s.d.linearized) s.temp[i] = std::pow(s.matenergydens[i], 0.25);
        else s.temp[i] = s.temp[i] + inc[i] / s.bee[i];
    }
    /* radiation energy density from the census (src/imc_tally.jl:81-113):
     * sum E per (scale, cell) exactly, then divide by volume * scale */
    std::vector<DD> rad((size_t)s.K * nc);
    for (const OP &p : s.parts) {
        if (!p.alive) continue;
        rad[(size_t)p.k * nc + p.cell].add(part_energy(s, p));
    }
    for (int i = 0; i < nc; ++i) {
        double vol = s.d.geometry == IMC_GEOM_1D ? s.dx[i] : (s.dx[i % s.nx] * s.dy[i / s.nx]);
        double r = 0.0;
        for (int k = 0; k < s.K; ++k) r += rad[(size_t)k * nc + i].val() / (vol * s.scales[k]);
        s.radenergydens[i] = r;
    }
}

/* EnergyCheck.energychecker (src/imc_energycheck.jl:19-38), FP64. */
double orc_energycheck_impl(Sim &s) {
    DD r;
    for (int i = 0; i < s.nc; ++i) {
        double vol = s.d.geometry == IMC_GEOM_1D ? s.dx[i] : (s.dx[i % s.nx] * s.dy[i / s.nx]);
        r.add(s.radenergydens[i] * vol);
    }
    double radenergy = r.val();
    double err = (s.totalenergy - s.totalenergydep - (radenergy - s.radenergyold) - s.lostenergy) / s.totalenergy;
    s.last_radold = s.radenergyold;
    s.last_rad = radenergy;
    s.last_lost = s.lostenergy;
    s.last_err = err;
    s.radenergyold = radenergy;
    s.lostenergy = 0.0;
    return err;
}

/* timestep (src/MixedPrecisionIMC.jl:181-222) */
void orc_timestep_impl(Sim &s) {
    if (s.t == s.d.t_end) {
        s.t = s.d.t_end + s.dt;
        s.finished = true;
        return;
    }
    if (s.d.timestepping == IMC_TS_CONSTANT) {
        if (s.t + s.dt > s.d.t_end) { s.dt = s.d.t_end - s.t; s.t = s.d.t_end; }
        else s.t = s.t + s.dt;
    } else {
        if (s.dt < s.d.dtmax) {
            s.dt = s.dt * s.d.k;
            if (s.dt > s.d.dtmax) s.dt = s.d.dtmax;
        }
        if (s.t + s.dt > s.d.t_end) { s.dt = s.d.t_end - s.t; s.t = s.d.t_end; }
        else s.t = s.t + s.dt;
    }
    if (s.t > s.d.t_end) s.finished = true;
}

void orc_sourcing_dispatch(Sim &s) {
    if (s.d.precision == IMC_FP64) orc_sourcing_impl<double>(s);
    else orc_sourcing_impl<float>(s);
}

Sim *make_sim(const ImcDeck *d) {
    if (!d || d->abi_version != IMC_ABI_VERSION) return nullptr;
    if (d->nx <= 0 || d->ny <= 0 || d->n_scales <= 0 || d->n_scales > 16) return nullptr;
    Sim *s = new Sim();
    s->d = *d;
    s->nx = d->nx; s->ny = d->geometry == IMC_GEOM_1D ? 1 : d->ny;
    s->nc = s->nx * s->ny;
    s->K = d->n_scales;
    const int nc = s->nc;
    s->dx.assign(d->dx, d->dx + s->nx);
    if (d->geometry == IMC_GEOM_2D) s->dy.assign(d->dy, d->dy + s->ny);
    else s->dy.assign(1, 1.0);
    s->temp.assign(d->temp, d->temp + nc);
    s->sa_val.assign(d->sigma_a_val, d->sigma_a_val + nc);
    s->sa_pow.assign(d->sigma_a_pow, d->sigma_a_pow + nc);
    s->ss_val.assign(d->sigma_s_val, d->sigma_s_val + nc);
    s->ss_pow.assign(d->sigma_s_pow, d->sigma_s_pow + nc);
    s->bee.assign(d->bee, d->bee + nc);
    s->radsource.assign(d->radsource, d->radsource + nc);
    int nts = d->geometry == IMC_GEOM_1D ? 2 : 2 * s->nx + 2 * s->ny;
    s->tsurf.assign(d->t_surface, d->t_surface + nts);
    s->scales.assign(d->energyscales, d->energyscales + s->K);
    s->beta.assign(nc, 1.0);
    s->fleck.assign(nc, 0.0);
    s->sa = s->sa_val;
    s->ss = s->ss_val;
    s->energydep.assign((size_t)s->K * nc, 0.0);
    s->emitted.assign((size_t)s->K * nc, 0.0);
    s->radenergydens.assign(nc, 0.0);
    s->matenergydens.assign(nc, 0.0);
    s->t = 0.0;
    s->dt = d->timestepping == IMC_TS_RAMP ? d->dt0 : d->dt;
    return s;
}

void fill_stats(Sim &s, ImcStepStats *st, double t, double dt) {
    st->t = t; st->dt = dt;
    st->total_energy = s.totalenergy;
    st->energy_dep = s.totalenergydep;
    st->rad_energy = s.last_rad;
    st->rad_energy_old = s.last_radold;
    st->lost_energy = s.last_lost;
    st->energy_error = s.last_err;
    st->n_census_in = s.n_census_in;
    st->n_sourced = s.n_sourced;
    st->n_census_out = live_count(s);
    st->segments = s.segments;
    st->surrogate_calls = 0;
    st->error_flags = s.flags;
    st->step_index = (uint32_t)s.step;
}

int step_impl(Sim &s, ImcStepStats *st, int *done) {
    double t0 = s.t, dt0 = s.dt;
    s.flags = 0;
    orc_update_impl(s);
    orc_sourcing_dispatch(s);
    orc_transport_impl(s);
    step_clean(s);
    orc_tally_impl(s);
    orc_energycheck_impl(s);
    fill_stats(s, &s.last, t0, dt0);
    if (st) *st = s.last;
    orc_timestep_impl(s);
    s.step += 1;
    if (done) *done = s.finished ? 1 : 0;
    return 0;
}

}  // namespace

extern "C" {

void *orc_create(const ImcDeck *deck) { return make_sim(deck); }
void orc_destroy(void *h) { delete (Sim *)h; }

int orc_update(void *h) { orc_update_impl(*(Sim *)h); return 0; }
int orc_sourcing(void *h) {
    Sim &s = *(Sim *)h;
    s.flags = 0;
    orc_sourcing_dispatch(s);
    return 0;
}
int orc_transport(void *h) { orc_transport_impl(*(Sim *)h); return 0; }
int orc_clean(void *h) { orc_clean_impl(*(Sim *)h); return 0; }
int orc_tally(void *h) { orc_tally_impl(*(Sim *)h); return 0; }
int orc_energycheck(void *h, double *err) {
    double e = orc_energycheck_impl(*(Sim *)h);
    if (err) *err = e;
    return 0;
}
int orc_timestep(void *h, int *done) {
    Sim &s = *(Sim *)h;
    orc_timestep_impl(s);
    s.step += 1;
    if (done) *done = s.finished ? 1 : 0;
    return 0;
}
int orc_step(void *h, ImcStepStats *st, int *done) { return step_impl(*(Sim *)h, st, done); }
int orc_run(void *h, int64_t max_steps, ImcStepStats *stats, int64_t *nsteps) {
    Sim &s = *(Sim *)h;
    int64_t n = 0;
    int done = s.finished ? 1 : 0;
    while (!done && n < max_steps) {
        step_impl(s, stats ? &stats[n] : nullptr, &done);
        ++n;
    }
    if (nsteps) *nsteps = n;
    return 0;
}
int orc_get_time(void *h, double *t, double *dt, int64_t *step) {
    Sim &s = *(Sim *)h;
    if (t) *t = s.t;
    if (dt) *dt = s.dt;
    if (step) *step = s.step;
    return 0;
}
int orc_set_time(void *h, double t, double dt) {
    Sim &s = *(Sim *)h;
    s.t = t; s.dt = dt;
    return 0;
}
int orc_set_step(void *h, int64_t step) { ((Sim *)h)->step = step; return 0; }
int64_t orc_num_particles(void *h) { return (int64_t)((Sim *)h)->parts.size(); }

/* physical view of the particle list (FP16 state expanded as the kernels do) */
int orc_get_particles(void *h, ImcParticles *p) {
    Sim &s = *(Sim *)h;
    if ((int64_t)s.parts.size() > p->n) return IMC_ERR_INVALID_ARG;
    p->n = (int64_t)s.parts.size();
    bool half = s.d.precision == IMC_FP16;
    for (int64_t i = 0; i < p->n; ++i) {
        const OP &q = s.parts[i];
        int ix = s.d.geometry == IMC_GEOM_1D ? q.cell : q.cell % s.nx;
        int iy = s.d.geometry == IMC_GEOM_1D ? 0 : q.cell / s.nx;
        double x = q.x, y = q.y, t = q.t, E = q.E;
        if (half) {
            float dxs = (float)s.dx[ix] * (float)s.d.distancescale;
            x = (double)((float)q.x * dxs);
            if (s.d.geometry == IMC_GEOM_2D) y = (double)((float)q.y * ((float)s.dy[iy] * (float)s.d.distancescale));
            t = (double)((float)q.t * (float)s.dt);
            E = (double)((float)q.E * (float)q.E0);
        }
        if (p->t) p->t[i] = t;
        if (p->x) p->x[i] = x;
        if (p->y) p->y[i] = y;
        if (p->mu) p->mu[i] = q.mu;
        if (p->ux) p->ux[i] = q.ux;
        if (p->uy) p->uy[i] = q.uy;
        if (p->E) p->E[i] = E;
        if (p->E0) p->E0[i] = q.alive ? q.E0 : -1.0;
        if (p->cell) p->cell[i] = q.cell;
        if (p->scale) p->scale[i] = q.k;
    }
    return 0;
}

/* Replace the list.  Values are rounded to the state precision. */
int orc_set_particles(void *h, const ImcParticles *p) {
    Sim &s = *(Sim *)h;
    s.parts.assign(p->n, OP{});
    for (int64_t i = 0; i < p->n; ++i) {
        OP &q = s.parts[i];
        q.cell = p->cell[i];
        q.k = p->scale ? p->scale[i] : 0;
        q.alive = p->E0[i] >= 0.0;
        int ix = s.d.geometry == IMC_GEOM_1D ? q.cell : q.cell % s.nx;
        int iy = s.d.geometry == IMC_GEOM_1D ? 0 : q.cell / s.nx;
        double t = p->t ? p->t[i] : 0.0;
        double x = p->x ? p->x[i] : 0.0, y = p->y ? p->y[i] : 0.0;
        double mu = p->mu ? p->mu[i] : 0.0, ux = p->ux ? p->ux[i] : 0.0, uy = p->uy ? p->uy[i] : 0.0;
        double E = p->E[i], E0 = p->E0[i];
        if (s.d.precision == IMC_FP64) {
            q.t = t; q.x = x; q.y = y; q.mu = mu; q.ux = ux; q.uy = uy; q.E = E; q.E0 = E0;
            q.ang = std::atan2(uy, ux);
        } else if (s.d.precision == IMC_FP32) {
            q.t = (float)t; q.x = (float)x; q.y = (float)y; q.mu = (float)mu; q.ux = (float)ux; q.uy = (float)uy;
            q.E = (float)E; q.E0 = (float)E0;
            q.ang = (double)std::atan2((float)q.uy, (float)q.ux);
        } else {
            float dxs = (float)s.dx[ix] * (float)s.d.distancescale;
            q.x = h16((double)((float)x / dxs));
            if (s.d.geometry == IMC_GEOM_2D) q.y = h16((double)((float)y / ((float)s.dy[iy] * (float)s.d.distancescale)));
            q.t = h16((double)((float)t / (float)s.dt));
            q.mu = h16(mu); q.ux = h16(ux); q.uy = h16(uy);
            q.E0 = (float)E0;
            q.E = h16((double)((float)E / (float)q.E0));
            q.ang = (double)std::atan2((float)q.uy, (float)q.ux);
        }
    }
    return 0;
}

int orc_get_field(void *h, int field, double *out, int64_t count) {
    Sim &s = *(Sim *)h;
    const std::vector<double> *v = nullptr;
    switch (field) {
        case IMC_FIELD_TEMP: v = &s.temp; break;
        case IMC_FIELD_RADENERGY: v = &s.radenergydens; break;
        case IMC_FIELD_MATENERGY: v = &s.matenergydens; break;
        case IMC_FIELD_FLECK: v = &s.fleck; break;
        case IMC_FIELD_BETA: v = &s.beta; break;
        case IMC_FIELD_SIGMA_A: v = &s.sa; break;
        case IMC_FIELD_SIGMA_S: v = &s.ss; break;
        case IMC_FIELD_BEE: v = &s.bee; break;
        case IMC_FIELD_ENERGYDEP: v = &s.energydep; break;
        case IMC_FIELD_EMITTED: v = &s.emitted; break;
        default: return IMC_ERR_INVALID_ARG;
    }
    if ((int64_t)v->size() != count) return IMC_ERR_INVALID_ARG;
    std::memcpy(out, v->data(), sizeof(double) * count);
    return 0;
}

int orc_set_field(void *h, int field, const double *in, int64_t count) {
    Sim &s = *(Sim *)h;
    std::vector<double> *v = nullptr;
    switch (field) {
        case IMC_FIELD_TEMP: v = &s.temp; break;
        case IMC_FIELD_RADENERGY: v = &s.radenergydens; break;
        case IMC_FIELD_MATENERGY: v = &s.matenergydens; break;
        case IMC_FIELD_FLECK: v = &s.fleck; break;
        case IMC_FIELD_BETA: v = &s.beta; break;
        case IMC_FIELD_SIGMA_A: v = &s.sa; break;
        case IMC_FIELD_SIGMA_S: v = &s.ss; break;
        case IMC_FIELD_BEE: v = &s.bee; break;
        case IMC_FIELD_ENERGYDEP: v = &s.energydep; break;
        case IMC_FIELD_EMITTED: v = &s.emitted; break;
        default: return IMC_ERR_INVALID_ARG;
    }
    if ((int64_t)v->size() != count) return IMC_ERR_INVALID_ARG;
    std::memcpy(v->data(), in, sizeof(double) * count);
    return 0;
}

int orc_get_stats(void *h, ImcStepStats *st) { *st = ((Sim *)h)->last; return 0; }
int orc_get_scalars(void *h, double *out4) {
    Sim &s = *(Sim *)h;
    out4[0] = s.totalenergy; out4[1] = s.totalenergydep; out4[2] = s.lostenergy; out4[3] = s.radenergyold;
    return 0;
}
int64_t orc_segments(void *h) { return ((Sim *)h)->segments; }
uint32_t orc_flags(void *h) { return ((Sim *)h)->flags; }

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { orc_philox4x32_10(ctr, key, out); }

double orc_sorter(int prec, const double *vals, int n, const double *scales, int nsc, double *scale_out, int *j_out) {
    return sorter_sel(prec, vals, n, scales, nsc, scale_out, j_out);
}

/* CPU baseline: `nthreads` independent replicas (seeds SEED+i), each running
 * up to max_steps steps; returns wall seconds, total segments and histories. */
int orc_bench(const ImcDeck *deck, int nthreads, int64_t max_steps, double *seconds, int64_t *segments,
              int64_t *histories) {
    if (nthreads < 1) nthreads = 1;
    std::vector<int64_t> seg(nthreads, 0), his(nthreads, 0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int i = 0; i < nthreads; ++i) {
        th.emplace_back([&, i]() {
            ImcDeck d = *deck;
            d.seed = deck->seed + (uint64_t)i;
            Sim *s = make_sim(&d);
            if (!s) return;
            int done = 0;
            for (int64_t n = 0; n < max_steps && !done; ++n) {
                ImcStepStats st;
                step_impl(*s, &st, &done);
                seg[i] += st.segments;
                his[i] += st.n_census_in + st.n_sourced;
            }
            delete s;
        });
    }
    for (auto &t : th) t.join();
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    int64_t S = 0, H = 0;
    for (int i = 0; i < nthreads; ++i) { S += seg[i]; H += his[i]; }
    if (segments) *segments = S;
    if (histories) *histories = H;
    return 0;
}

/* Analog in-cell walk of the learned surrogate's training data: the in-cell
 * part of Transport.MC's loop (src/imc_transport.jl:72-193) in mean free
 * paths -- exponential flights, isotropic re-emission (mu = 1 - 2 rand,
 * redrawn while zero), the walk cut at path lmax.  Near face at 0, far face
 * at d_n + d_f.  Same variates as the kernel: stream (seed, 0, i, 3). */
int orc_surr_walk(uint64_t seed, const float *state, int64_t n, float *x, int32_t *cls, float *tgt) {
    for (int64_t i = 0; i < n; ++i) {
        OrcStream rs;
        orc_stream_init(&rs, seed, 0u, (uint32_t)i, ORC_STAGE_SURR_DATA);
        const float d_n = state[4 * i], d_f = state[4 * i + 1], lmax = state[4 * i + 3];
        float mu = state[4 * i + 2];
        const float W = d_n + d_f;
        float pos = d_n, path = 0.0f, y0 = 0.0f, y1 = 0.0f;
        int c = 2;
        const int cap = 8 * (int)lmax + 64;
        bool ended = false;
        for (int it = 0; it < cap && !ended; ++it) {
            const float s = orc_randexp_f32(&rs);
            const float dface = mu > 0.0f ? (W - pos) / mu : pos / (-mu);
            const float rem = lmax - path;
            if (rem <= s && rem <= dface) {
                pos += mu * rem;
                y0 = (pos - d_n) / sqrtf(lmax); y1 = mu; c = 2; ended = true;
            } else if (dface <= s) {
                path += dface;
                y0 = logf(std::max(path, 1e-30f) / lmax); y1 = fabsf(mu); c = mu > 0.0f ? 1 : 0; ended = true;
            } else {
                pos += mu * s;
                path += s;
                mu = 0.0f;
                for (int r = 0; r < 64 && mu == 0.0f; ++r) mu = 1.0f - 2.0f * orc_rand_f32(&rs);
                if (mu == 0.0f) mu = 1.0f;
            }
        }
        if (!ended) { y0 = (pos - d_n) / sqrtf(lmax); y1 = mu; c = 2; }
        const float r0 = log1pf(d_n / sqrtf(lmax)) * 0.41703239f, r1 = log1pf(d_f / sqrtf(lmax)) * 0.41703239f;
        x[4 * i] = r0 < 1.0f ? r0 : 1.0f;
        x[4 * i + 1] = r1 < 1.0f ? r1 : 1.0f;
        x[4 * i + 2] = state[4 * i + 2];
        x[4 * i + 3] = (log10f(lmax) - 2.0f) * 0.5f;
        cls[i] = c;
        tgt[2 * i] = y0;
        tgt[2 * i + 1] = y1;
    }
    return 0;
}

}  // extern "C"
