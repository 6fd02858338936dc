// imc_internal.h -- device data layout and kernel launchers shared by the
// translation units of libimc.so.  Not part of the public ABI (include/imc.h).
//
// Layout in HBM
//   cell state      FP64 arrays of ncells (temp, bee, beta, fleck, sigma_a,
//                   sigma_s, matenergydens, radenergydens) and ncells*K
//                   (energydep, emittedenergy), K = number of energy scales.
//   particles       two ping-pong structure-of-arrays buffers; one field per
//                   array so every load and store is coalesced:
//                     1D: t, x, mu, E, E0, cs      2D: t, x, y, ux, uy, E, E0, cs
//                   FP64 / FP32 store physical values; FP16 stores x/(dx*ds),
//                   y/(dy*ds), t/dt, E/E0 and the direction in binary16 with E0
//                   in binary32.  cs = cell | scale_index << 24.  alive is one
//                   byte per particle.
//   tallies         3-limb fixed-point accumulators (int64) per (scale, cell)
//                   for deposition and census energy, per scale for escaped
//                   energy; finalised to FP64 by the tally kernel.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

namespace imc {

// query rounds per step of the surrogate transport (launch_transport_surr)
constexpr unsigned kSurrProbe = 32;  // steps between re-openings of the surrogate gate (k_energycheck)
constexpr int kSurrRounds = 1;  // measured best on GB300 (thick slab: 1 round 84 ms, 3 rounds 104 ms, 6 rounds 134 ms)

// scalars that live in device memory so a whole step can replay as a graph
struct Scalars {
    double t, dt;
    double totalenergy, totalenergydep, lostenergy, radenergyold, radenergy, energy_err;
    double lost_step;                  // escaped energy of this step
    int emax_census_exp;               // max over the census of ilogb(E) - scale_exp(scale_k) (kNoExp: none)
    double emax;                       // max true particle energy at transport start (an upper bound)
    long long n_census;                // live particles in the list (the census after transport)
    long long n_census_in;             // census carried into this step
    long long n_particles;             // list length (live particles and holes left by kills)
    long long birth_base;              // list index of this step's first birth
    long long n_sourced;
    double n_source;                   // particle budget of this step
    double src_group[6];               // sourcing: energy/escale sum of each slot group
    unsigned long long segments;
    unsigned long long surrogate_calls;
    unsigned long long killed;         // histories this transport removed (kill, escape, cap)
    float seg_per_hist;                // segments per history of the last transport
    unsigned long long work_next;      // transport: next chunk of the list's tail to hand out
    unsigned long long qcount[2 * kSurrRounds + 1];  // surrogate transport: ask queue of round r at 2r, resume queue at 2r + 1
    unsigned int flags;
    int b_dep, b_rad, b_lost;          // fixed-point exponents of this transport in true energy;
                                       // scale k's tallies use b + scale_exp(scale_k)
    unsigned int step;                 // step index (RNG key, stats slot)
    int finished;                      // t > t_end
    int cur;                           // particle buffer holding the list (0 or 1)
    int compact_src;                   // buffer compacted from this step
    int compact_now;                   // this step compacts the list
    int surr_gate;                     // learned surrogate: this step may set histories aside
    long long surr_closed_h;           // histories of the step that last closed the gate
    unsigned int tally_blocks_done;    // fused tally + energy check: blocks finished (the last one checks)
};

struct CellArgs {
    int geometry, nx, ny, nc, K;
    const double *dx, *dy;
    double *temp, *bee, *beta, *fleck, *sa, *ss;
    const double *sa_val, *sa_pow, *ss_val, *ss_pow, *radsource, *tsurf, *scales;
    double *energydep, *emitted, *radenergydens, *matenergydens;
    long long *dep_acc, *rad_acc, *lost_acc;   // 3 limbs per slot
    // sourcing scratch (per source slot)
    int nslots;
    double *slot_e, *slot_s, *slot_nrg, *slot_q;
    float *slot_nrg_f;                 // slot_nrg rounded to binary32 (FP32 / FP16 births)
    const float *dxf, *dyf;            // cell widths rounded to binary32 (FP32 / FP16 births)
    // fixed positions of the surface births, in binary32 (FP32 / FP16 state)
    // and binary64, each the reference's Float64 product rounded to the
    // arithmetic type: 1D 0.01 / 0.99 of the end cells
    // (src/imc_sourcing.jl:163,178), 2D 0.001 / 0.999 of the first / last
    // column (x, :300,315) and row (y, :271,286); order x1 left, x1 right,
    // x2 left, x2 right, y2 bottom, y2 top
    float surf_f[6];
    double surf_d[6];
    int *slot_j;
    long long *slot_n, *slot_off;
    // per-block partial sums (double-double pairs) and maxima
    int nblk_slot, nblk_cell;          // kCellThreads-thread blocks over slots / cells
    double *part_src;                  // [nblk_slot][6 groups][hi, lo]
    double *part_emax;                 // [nblk_slot]
    double *part_tally;                // [nblk_cell][K + 1][hi, lo]
    // physics / control
    int bc[4];
    double c, a, alpha, ds, temp_floor, cellmin;
    int linearized, marshak, sel_prec, timestepping;
    long long n_input, n_max, capacity, seg_cap;
    unsigned long long seed;
    double vol_min, scale_min;
    double t_end, dtmax, kfac;
    // learned thick-cell surrogate: tensor-core image of the network
    // (imc_surrogate.cuh), or null for analog transport everywhere
    const uint4 *surr_image;
    long long surr_min_calls;          // queries a step needs to keep the network on (surr_gate)
};

// type-erased particle buffer
struct PBufRaw {
    void *t, *x, *y, *ux, *uy, *E, *E0;
    int32_t *cs;
    uint8_t *alive;
};

// the two particle buffers; Scalars::cur says which one holds the list, so
// the kernels of a step need no host-side knowledge of it
struct PBufPair {
    PBufRaw b[2];
};

// per-step statistics slot written on the device
struct DevStats {
    double t, dt, total_energy, energy_dep, rad_energy, rad_energy_old, lost_energy, energy_error;
    long long n_census_in, n_sourced, n_census_out, segments, surrogate_calls;
    unsigned int error_flags, step_index;
};

// launchers (imc_kernels.cu / imc_transport.cu); all asynchronous on `st`
void launch_update(const CellArgs &ca, Scalars *sc, cudaStream_t st);
void launch_source(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, int grid, cudaStream_t st);
struct TransportShape {
    bool smem_tally;  // block-private tallies in shared memory
    bool dep_only;    // only the deposition tallies in shared memory
    int smem;         // dynamic shared memory bytes
    int block;        // threads per block
};
TransportShape transport_shape(const CellArgs &ca, int prec);
void launch_transport(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, int grid, cudaStream_t st);
// 1D transport with the learned surrogate in thick cells (ca.surr_image set;
// FP32 or FP16 state), as 1 + 2 kSurrRounds kernels per step: an analog pass
// over the list that sets aside the histories that want a network query,
// then rounds of (query pass, analog pass over the continuing histories).
// histories set aside between passes (FP32 state)
struct SurrQueue {
    float *x, *mu, *t, *E, *E0;
    int32_t *cs;        // cell | scale_index << 24 now
    int32_t *cs_list;   // as stored in the list (census rewrites it on change)
    long long *idx;     // list index
};
struct SurrWave {
    SurrQueue ask;      // waiting for a query
    SurrQueue resume;   // continuing after a query
};
struct SurrShapes {
    int analog_block, analog_smem, analog_grid;  // list pass
    bool analog_smt;
    int query_block, query_smem, query_grid;     // query passes
};
SurrShapes surr_shapes(const CellArgs &ca, int prec);
// the analog passes are the 1D transport kernel in its pass modes
// (imc_transport.cu); which: 0 list pass, 1 resume pass, 2 last resume pass
const void *surr_analog_ptr(const CellArgs &ca, int prec, int which);
int surr_analog_smem(const CellArgs &ca, int prec);
void launch_surr_analog(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, const SurrWave &w, int which,
                        int round, int grid, int smem, cudaStream_t st);
// kernel pointers for attribute / occupancy set-up: which = 0 list pass,
// 1 resume pass that sets aside, 2 last resume pass, 3 query pass
const void *surr_kernel_ptr(const CellArgs &ca, int prec, int which);
void launch_transport_surr(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, const SurrWave &w,
                           const SurrShapes &sh, cudaStream_t st);
// writes the tensor-core image of FP32 parameters into dst (device, kImageBytes)
void launch_surr_image(const float *params, void *dst, cudaStream_t st);
// Removes killed particles from the list.  With force = false the list is
// compacted only when the holes exceed 1/16 of its length (kDeferHoles);
// otherwise the holes stay and only the live count is updated.
constexpr long long kDeferHoles = 16;
void launch_compact(const CellArgs &ca, Scalars *sc, int prec, PBufPair bufs, long long *tile_cnt,
                    long long *tile_off, long long ntiles_cap, bool force, cudaStream_t st);
// forced compaction of `src` into `dst` (the list must be in src: Scalars::cur == 0)
void launch_compact(const CellArgs &ca, Scalars *sc, int prec, PBufRaw src, PBufRaw dst, long long *tile_cnt,
                    long long *tile_off, long long ntiles_cap, cudaStream_t st);
void launch_finalize(const CellArgs &ca, Scalars *sc, cudaStream_t st);
void launch_tally(const CellArgs &ca, Scalars *sc, cudaStream_t st);
void launch_energycheck(const CellArgs &ca, Scalars *sc, DevStats *stats, long long stats_cap, cudaStream_t st);
void launch_timestep(const CellArgs &ca, Scalars *sc, cudaStream_t st);
// the step sequence's fused launches: finalize + tally, energycheck + timestep
void launch_finalize_tally(const CellArgs &ca, Scalars *sc, cudaStream_t st);
// finalize + tally + energycheck + timestep in one launch (the step sequence)
void launch_tally_check_timestep(const CellArgs &ca, Scalars *sc, DevStats *stats, long long stats_cap,
                                 cudaStream_t st);
void launch_prepare_transport(const CellArgs &ca, Scalars *sc, cudaStream_t st);
const void *transport_kernel_ptr(const CellArgs &ca, int prec);
// One deck of the fused batch transport (1D): what the transport reads of
// its CellArgs, and its two particle buffers' 1D arrays.  The fused kernel
// reads them from constant memory (kFusedMaxDecks entries), so that, like a
// single deck's kernel parameters, they cost no registers in the history loop.
struct Deck1DArgs {
    int nx, nc, K, bc[2];
    const double *dx;
    double *sa, *fleck, *ss;
    const double *scales;
    long long *dep_acc, *rad_acc, *lost_acc;
    double c, ds;
    long long seg_cap;
    unsigned long long seed;
};
struct PBufRaw1D {
    void *t, *x, *ux, *E, *E0;
    int32_t *cs;
    uint8_t *alive;
};
struct PBufPair1D {
    PBufRaw1D b[2];
};
constexpr int kFusedMaxDecks = 256;
// the fused batch transport (1D, shared tallies): a kernel taking the number
// of decks, launched (as a graph kernel node) with transport_multi_block
// threads per block and the largest deck's dynamic shared memory over the
// decks set by set_transport_multi_decks
const void *transport_multi_ptr(int prec);
int transport_multi_block(int prec);
cudaError_t set_transport_multi_decks(const Deck1DArgs *ca, const PBufPair1D *bufs, Scalars *const *sc, int n,
                                      cudaStream_t st);

// threads per block of the per-cell / per-slot FP64 kernels: one warp, so that
// a 2000-cell mesh spreads over 63 SMs (FP64 runs at 1/64 of the FP32 rate,
// and these kernels are latency bound)
constexpr int kCellThreads = 32;
constexpr int kCompactTile = 4096;     // particles per compaction tile
constexpr int kCompactThreads = 256;

}  // namespace imc
