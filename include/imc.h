/*
 * imc.h -- C ABI of the GB300 Implicit Monte Carlo (IMC) particle engine.
 *
 * This is the drop-in boundary for the per-timestep particle path of
 * MixedPrecisionIMC.jl.  The reference runs that path as plain Julia module
 * functions that mutate `mesh`, `simvars` and `particles` in place:
 *
 *   Update.update(inputs, mesh, simvars)                 src/imc_update.jl:12
 *   Sourcing.sourcing(mesh, simvars, particles)          src/imc_sourcing.jl:12
 *   Transport.MC(mesh, simvars, particles)               src/imc_transport.jl:13
 *   Transport.MC2D(mesh, simvars, particles)             src/imc_transport.jl:483
 *   Clean.clean(particles)                               src/imc_clean.jl:6
 *   Tally.tally(inputs, mesh, simvars, particles)        src/imc_tally.jl:11
 *   EnergyCheck.energychecker(inputs, mesh, simvars, p)  src/imc_energycheck.jl:10
 *   timestep(timestepping, simvars)                      src/MixedPrecisionIMC.jl:181
 *
 * called in that order by main(args) (src/MixedPrecisionIMC.jl:136-152, 2D
 * :165-176).  Here each stage is one entry point acting on an opaque handle
 * that owns all device memory (mesh state in FP64, particle state as
 * structure-of-arrays in FP64, FP32 or FP16).  The caller keeps the input deck
 * and the mesh geometry on the host and passes them once, as plain arrays, in
 * an ImcDeck.
 *
 * Conventions
 *   - Every function returns an int status: 0 (IMC_OK) or one of IMC_ERR_*.
 *     Nothing throws across the ABI.  imc_last_error() gives a message.
 *   - A handle is not thread-safe; it owns one CUDA stream and every call is
 *     ordered on it.  Calls return once their work is complete on the GPU,
 *     except where stated.
 *   - 2D cell arrays are x-fastest: cell (ix, iy) is element ix + iy*nx, the
 *     memory order of a Julia Nx-by-Ny array.  Cell indices are 0-based.
 *   - Times, energies and all mesh quantities cross the ABI as double.
 */
#ifndef IMC_H_
#define IMC_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IMC_ABI_VERSION 1

/* status codes */
enum {
    IMC_OK = 0,
    IMC_ERR_INVALID_ARG = 1,  /* bad deck field, null pointer, size mismatch */
    IMC_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    IMC_ERR_OOM = 3,          /* device allocation failed */
    IMC_ERR_CAPACITY = 4,     /* particle buffer would overflow */
    IMC_ERR_NUMERIC = 5,      /* NaN / negative tally contribution seen */
    IMC_ERR_SEGMENT_CAP = 6,  /* a history hit the per-history segment cap */
    IMC_ERR_NO_ENERGY = 7,    /* total source energy is zero or not finite */
    IMC_ERR_STATE = 8,        /* call out of order (e.g. transport before sourcing) */
    IMC_ERR_NO_DEVICE = 9,    /* no CUDA device, or not an sm_103 device */
    IMC_ERR_TIMEOUT = 10      /* a bounded device-side wait gave up */
};

/* device error-flag bits, reported in ImcStepStats.error_flags */
enum {
    IMC_FLAG_NAN = 1u << 0,          /* NaN energy / distance in a history */
    IMC_FLAG_NEG_TALLY = 1u << 1,    /* negative tally contribution dropped */
    IMC_FLAG_SEGMENT_CAP = 1u << 2,  /* history stopped at the segment cap */
    IMC_FLAG_CAPACITY = 1u << 3,     /* sourcing clipped at buffer capacity */
    IMC_FLAG_NO_ENERGY = 1u << 4,    /* total energy 0 / NaN: nothing sourced */
    IMC_FLAG_FIXPOINT_RANGE = 1u << 5,  /* tally value above the fixed-point range */
    IMC_FLAG_SURROGATE_DOMAIN = 1u << 6 /* surrogate query outside its domain (fell back) */
};

enum { IMC_GEOM_1D = 1, IMC_GEOM_2D = 2 };
/* particle-state precision (PRECISION deck keyword) */
enum { IMC_FP64 = 0, IMC_FP32 = 1, IMC_FP16 = 2 };
enum { IMC_BC_VACUUM = 0, IMC_BC_REFLECT = 1 };
enum { IMC_TS_CONSTANT = 0, IMC_TS_RAMP = 1 };
/* boundary slots in ImcDeck.bc: order of src/MixedPrecisionIMC.jl:121-162 */
enum { IMC_LEFT = 0, IMC_RIGHT = 1, IMC_TOP = 2, IMC_BOTTOM = 3 };

/*
 * ImcDeck: the input deck after keyword parsing and mesh generation
 * (src/imc_input.jl:20-129, src/constants.jl:6-15, src/imc_mesh.jl:42-259).
 * All pointers are read during imc_create only; the caller keeps ownership.
 */
typedef struct ImcDeck {
    int32_t abi_version;       /* IMC_ABI_VERSION */
    int32_t geometry;          /* IMC_GEOM_1D / IMC_GEOM_2D (GEOMETRY) */
    int32_t nx, ny;            /* cells; ny = 1 in 1D */
    int32_t precision;         /* IMC_FP64 / IMC_FP32 / IMC_FP16 (PRECISION) */
    int32_t scale_select_precision; /* precision in which the energy-scale choice of
                                       Utilities.sorter is evaluated
                                       (src/imc_utilities.jl:23-54); IMC_FP64 etc. */
    const double *dx;          /* nx cell widths (DX / XMESHNODES / MESHNODES) */
    const double *dy;          /* ny cell heights (2D only; NULL in 1D) */
    const double *temp;        /* nx*ny initial temperature (T_INIT) */
    const double *sigma_a_val; /* nx*ny absorption-opacity constant, already / DISTANCESCALE */
    const double *sigma_a_pow; /* nx*ny absorption-opacity temperature power */
    const double *sigma_s_val; /* nx*ny scattering-opacity constant, already / DISTANCESCALE */
    const double *sigma_s_pow; /* nx*ny scattering-opacity temperature power */
    const double *bee;         /* nx*ny heat capacity (BEE_VALS) */
    const double *radsource;   /* nx*ny radiation source (RADSOURCE_VALS) */
    const double *t_surface;   /* 1D: [left, right]; 2D: bottom[nx], top[nx], left[ny], right[ny] */
    int32_t bc[4];             /* IMC_BC_* for LEFTBC, RIGHTBC, TOPBC, BOTTOMBC */
    double phys_c, phys_a, alpha;   /* PHYS_C, PHYS_A, ALPHA */
    int32_t n_scales;          /* number of ENERGYSCALES (1..16) */
    const double *energyscales;/* sorted descending, as src/imc_mesh.jl:130 */
    double distancescale;      /* DISTANCESCALE */
    int64_t n_input, n_max;    /* NINPUT, NMAX */
    double cellmin;            /* CELLMIN */
    int32_t linearized;        /* LINEARIZED = TRUE */
    int32_t marshak_opacity;   /* NAME == "MARSHAK WAVE": sigma_a = val/T^3 (src/imc_update.jl:32-34) */
    double temp_floor;         /* opacity temperature clamp T >= temp_floor (0 = off; not in the reference) */
    uint64_t seed;             /* SEED */
    int32_t timestepping;      /* IMC_TS_CONSTANT / IMC_TS_RAMP (TIMESTEPPING) */
    int32_t sort_census;       /* reserved, must be 0 */
    double dt, dt0, k, dtmax, t_end;  /* DT, DT0, K, DTMAX, ENDTIME */
    int64_t capacity;          /* particle-buffer capacity; 0 = derived from NMAX */
    int64_t segment_cap;       /* per-history segment cap; 0 = 1e7 */
} ImcDeck;

/* One timestep's scalars, as printed by the reference each step
 * (src/imc_energycheck.jl:31-38, src/imc_transport.jl:208). */
typedef struct ImcStepStats {
    double t, dt;
    double total_energy;      /* mesh.totalenergy       (src/imc_sourcing.jl:121) */
    double energy_dep;        /* mesh.totalenergydep    (src/imc_tally.jl:51) */
    double rad_energy;        /* sum(radenergydens*dx)  (src/imc_energycheck.jl:26) */
    double rad_energy_old;    /* mesh.radenergyold before this step */
    double lost_energy;       /* mesh.lostenergy        */
    double energy_error;      /* (E - Edep - dErad - Elost)/E (src/imc_energycheck.jl:34) */
    int64_t n_census_in;      /* particles carried into the step */
    int64_t n_sourced;        /* particles born this step */
    int64_t n_census_out;     /* survivors after Clean.clean */
    int64_t segments;         /* while-loop passes this step (src/imc_transport.jl:73) */
    int64_t surrogate_calls;  /* thick-cell surrogate evaluations */
    uint32_t error_flags;     /* IMC_FLAG_* bits raised during the step */
    uint32_t step_index;      /* 0-based step counter */
} ImcStepStats;

/* Host-side particle view (structure of arrays).  1D uses t,x,mu; 2D uses
 * t,x,y,ux,uy (direction cosines).  cell is 0-based (2D: ix + iy*nx); scale is
 * the 0-based index into ImcDeck.energyscales.  Energies are in scaled units,
 * as the reference stores them (src/imc_sourcing.jl:173,276). */
typedef struct ImcParticles {
    int64_t n;
    double *t, *x, *y, *mu, *ux, *uy, *E, *E0;
    int32_t *cell, *scale;
} ImcParticles;

/* cell fields for imc_get_field / imc_set_field */
enum {
    IMC_FIELD_TEMP = 0,        /* mesh.temp */
    IMC_FIELD_RADENERGY = 1,   /* mesh.radenergydens */
    IMC_FIELD_MATENERGY = 2,   /* mesh.matenergydens */
    IMC_FIELD_FLECK = 3,       /* mesh.fleck */
    IMC_FIELD_BETA = 4,        /* mesh.beta */
    IMC_FIELD_SIGMA_A = 5,     /* mesh.sigma_a[:,1] */
    IMC_FIELD_SIGMA_S = 6,     /* mesh.sigma_s[:,1] */
    IMC_FIELD_BEE = 7,         /* mesh.bee */
    IMC_FIELD_ENERGYDEP = 8,   /* mesh.energydep, ncells*n_scales, scale-major */
    IMC_FIELD_EMITTED = 9,     /* mesh.emittedenergy, ncells*n_scales, scale-major */
    IMC_FIELD_COUNT = 10
};

typedef struct ImcHandle ImcHandle;

/* ---- lifetime ---------------------------------------------------------- */

/* Validate the deck, allocate device state and upload the mesh.  Replaces the
 * set-up half of main(args): src/MixedPrecisionIMC.jl:78-125 (Mesh state of
 * src/imc_mesh.jl:10-40, SimVars of :35-51, Random.seed! of :86). */
int imc_create(const ImcDeck *deck, ImcHandle **out);
int imc_destroy(ImcHandle *h);
/* Copies the last error message of h (or of the last failed imc_create when
 * h is NULL) into buf; returns the status that produced it. */
int imc_last_error(const ImcHandle *h, char *buf, size_t len);
/* Returns IMC_ABI_VERSION; lets a binding check it loaded the right library. */
int imc_abi_version(void);
/* Device name and SM count of the current device, or IMC_ERR_NO_DEVICE. */
int imc_device_info(char *name, size_t len, int *sm_count, int *cc_major, int *cc_minor);

/* ---- per-stage entry points (one per reference function) --------------- */

/* Update.update: opacities, beta, Fleck factor, FP64 (src/imc_update.jl:12-56).
 * Uses the current dt. */
int imc_update(ImcHandle *h);
/* Sourcing.sourcing: emission energies, particle budget and births appended
 * after the census (src/imc_sourcing.jl:12-370). */
int imc_sourcing(ImcHandle *h);
/* Transport.MC (1D, src/imc_transport.jl:13-210) or Transport.MC2D (2D,
 * :483-732): every particle history to census, escape or cut-off; tallies
 * energy deposition, escaped energy and census radiation energy. */
int imc_transport(ImcHandle *h);
/* Clean.clean: stable removal of killed particles (src/imc_clean.jl:6-19). */
int imc_clean(ImcHandle *h);
/* Tally.tally: material energy, temperature and radiation energy density
 * (src/imc_tally.jl:11-149), FP64. */
int imc_tally(ImcHandle *h);
/* EnergyCheck.energychecker (src/imc_energycheck.jl:10-56), FP64.  Writes the
 * relative balance error to *energy_error (may be NULL). */
int imc_energycheck(ImcHandle *h, double *energy_error);
/* timestep(timestepping, simvars): CONSTANT / RAMP control
 * (src/MixedPrecisionIMC.jl:181-222).  *done = 1 once t > t_end. */
int imc_timestep(ImcHandle *h, int *done);

/* ---- whole-step / whole-run entry points -------------------------------- */

/* One timestep: update -> sourcing -> transport -> clean -> tally ->
 * energycheck -> timestep (src/MixedPrecisionIMC.jl:136-152).  stats may be
 * NULL.  *done = 1 once t > t_end.  In imc_step and imc_run the clean stage
 * removes killed particles only once they exceed 1/16 of the list; until then
 * they stay in place as holes (alive byte 0; E0 = -1 in imc_get_particles)
 * and births are appended after them.  imc_clean always removes them all. */
int imc_step(ImcHandle *h, ImcStepStats *stats, int *done);
/* Run steps until t > t_end or max_steps steps ran, replaying one captured
 * CUDA graph per step.  stats (may be NULL) receives up to max_steps entries;
 * *n_steps the number run; *device_ms (may be NULL) the device time of the
 * run measured with CUDA events on the handle's stream. */
int imc_run(ImcHandle *h, int64_t max_steps, ImcStepStats *stats,
            int64_t *n_steps, double *device_ms);

/* Batched ensemble: runs every handle to the end of its clock (at most
 * max_steps steps each), `n_threads` host threads driving the handles' own
 * CUDA streams, so the decks' kernels run side by side on the GPU (each
 * handle's transport grid is sized to its particle buffer).  Handles must be
 * distinct.  steps[i] (optional) = steps run by handle i; *wall_ms (optional)
 * = host wall time of the whole batch.  Returns IMC_OK or the status of the
 * first handle that failed, whose index goes to *failed (-1 if none). */
int imc_run_batch(ImcHandle *const *hs, int32_t n, int64_t max_steps, int32_t n_threads, int64_t *steps,
                  double *wall_ms, int32_t *failed);
/* Batched ensemble with one transport launch per step over every deck: each
 * step is one CUDA graph -- every deck's update + sourcing, then a single
 * persistent transport kernel whose blocks take work chunks from each deck's
 * list in turn (with that deck's cell table and private tallies), then every
 * deck's compaction and tally + energycheck + timestep.  Each deck's result
 * is bit-identical to imc_run's.  The decks step together; a deck whose clock
 * ends leaves the group.  Requires every handle 1D, on one device, of one
 * state precision, without the surrogate, and with its tallies in shared
 * memory (up to 2560 cells for FP32 or FP16 state with one energy scale);
 * otherwise IMC_ERR_INVALID_ARG with *failed = the first handle that does
 * not qualify.  At most 256 decks per call (IMC_ERR_INVALID_ARG beyond).
 * Arguments and results as imc_run_batch; the batch stops at the first deck
 * that raises an error flag.  No counterpart in the reference (a loop over
 * its decks is the user's). */
int imc_run_batch_fused(ImcHandle *const *hs, int32_t n, int64_t max_steps, int64_t *steps, double *wall_ms,
                        int32_t *failed);

/* Checkpoint / resume.  imc_save_state copies the whole simulation state --
 * clock, device scalars (energy balance, fixed-point ranges), cell fields and
 * the particle list in its storage types -- into a host buffer: with buf
 * NULL it sets *len to the size needed; otherwise *len is the buffer size on
 * input and the size written on return.  imc_load_state restores such a blob
 * into a handle created from the same deck (precision, geometry, mesh and
 * scales must match); the run then continues exactly as the saved one would
 * have (every random stream is keyed by the step index, which is restored). */
int imc_save_state(const ImcHandle *h, void *buf, size_t *len);
int imc_load_state(ImcHandle *h, const void *buf, size_t len);

/* Totals over every step run by imc_step / imc_run since imc_create:
 * segments, histories (census carried in + births, per step) and surrogate
 * queries; any pointer may be NULL. */
int imc_get_totals(const ImcHandle *h, int64_t *segments, int64_t *histories, int64_t *surrogate_calls);

/* ---- state access ------------------------------------------------------- */


/* simulation clock (simvars.t, simvars.dt) and step counter */
int imc_get_time(const ImcHandle *h, double *t, double *dt, int64_t *step_index);
/* Overrides t and dt (the reference tests build SimVars by hand,
 * test/runtests.jl:67). */
int imc_set_time(ImcHandle *h, double t, double dt);
/* length of the particle list: live particles, births not yet transported,
 * and killed particles not yet removed */
int imc_num_particles(const ImcHandle *h, int64_t *n);
/* copy a cell field (IMC_FIELD_*) to / from the host; count = ncells, or
 * ncells*n_scales for ENERGYDEP / EMITTED. */
int imc_get_field(const ImcHandle *h, int field, double *out, int64_t count);
int imc_set_field(ImcHandle *h, int field, const double *in, int64_t count);
/* Copy the particle list to the host; p->n on entry is the capacity of the
 * arrays, on return the number copied (all of them, or IMC_ERR_INVALID_ARG). */
int imc_get_particles(const ImcHandle *h, ImcParticles *p);
/* Replace the particle list (census) with p->n host particles.  E0 < 0 marks a
 * killed particle, as slot 8 == -1.0 does in the reference
 * (src/imc_transport.jl:104, src/imc_clean.jl:10). */
int imc_set_particles(ImcHandle *h, const ImcParticles *p);
/* Most recent step's scalars. */
int imc_get_stats(const ImcHandle *h, ImcStepStats *stats);
/* Per-launch timing of the transport kernel.  With timing on, imc_run and
 * imc_step bracket every transport launch with CUDA events on the handle's
 * stream (imc_run then launches each step's kernels directly instead of
 * replaying the captured graph). */
int imc_set_timing(ImcHandle *h, int enable);
/* Average device time (ms) of the transport kernel over the launches since
 * the last call; resets the accumulator.  *launches receives the count. */
int imc_transport_timing(ImcHandle *h, double *avg_ms, int64_t *launches);
/* Number of kernel launches one step issues (for launch accounting). */
int imc_kernels_per_step(const ImcHandle *h, int *count);

/* ---- compaction for callers that cannot allocate ------------------------ */

/* Device-resident particle arrays owned by the caller (structure of arrays,
 * element type by precision: double / float / binary16 state, double or
 * float E0).  1D uses t, x, ux (mu), E, E0; 2D also y, uy.  cs = cell |
 * scale_index << 24; alive = 1 byte per particle. */
typedef struct ImcDeviceParticles {
    void *t, *x, *y, *ux, *uy, *E, *E0;
    int32_t *cs;
    uint8_t *alive;
} ImcDeviceParticles;

/* No counterpart in the reference.  Stable removal of the particles whose
 * alive byte is 0 -- the compaction imc_clean performs -- from caller-owned
 * device arrays `src` into caller-owned `dst`, for callers that cannot call
 * cudaMalloc: hosts whose device memory belongs to their own pool allocator
 * (which must account for every byte on the device), and loops that cannot
 * take the device-wide synchronisation of an allocation.  It allocates
 * nothing: its scratch is a fixed 72 KiB __device__ array that every GPU
 * loading the library holds until exit, which limits n to 16,777,216
 * particles (larger n returns IMC_ERR_INVALID_ARG).  The first call on a
 * device looks the array's address up with that device current.  All calls
 * share the array, so calls that overlap on the GPU race.
 * Requirements, checked before any device work (IMC_ERR_INVALID_ARG):
 * t, x, ux, E, E0, cs, alive non-NULL in both src and dst (2D: also y, uy);
 * each array aligned to its element size, alive to 16 bytes; no dst array
 * sharing memory with a src array over n elements (no in-place compaction).
 * dst arrays hold at least n elements; with n = 0 no array is read (NULL
 * is accepted) and *n_out = 0.  Work is ordered on `stream` (a
 * cudaStream_t; NULL = the default stream); the call returns once *n_out,
 * the number of survivors, is known.
 * Returns IMC_OK, IMC_ERR_INVALID_ARG, IMC_ERR_NO_DEVICE or IMC_ERR_CUDA. */
int imc_clean_noalloc(int precision, int geometry, const ImcDeviceParticles *src, ImcDeviceParticles *dst,
                      int64_t n, int64_t *n_out, void *stream);

/* ---- learned thick-cell surrogate --------------------------------------- */

/* Replaces the analog collision loop of Transport.MC (src/imc_transport.jl:
 * 72-193) inside cells many mean free paths thick.  Inside one cell a history
 * is a random walk whose outcome depends only on its state in mean free
 * paths: distance to the nearer face d_n, to the farther face d_f, direction
 * cosine mu' (> 0 away from the nearer face) and lmax, the path after which
 * the walk is cut (census, or the 1 % energy cut-off).  A 4-64-64-64-64
 * ReLU network (IMC_SURROGATE_PARAMS floats, W[out][in] row-major then the
 * bias, per layer) maps (min(d_n/lmax,1), min(d_f/lmax,1), mu',
 * (log10 lmax - 2)/2) to the probabilities of exit near / exit far /
 * truncation and the quantiles of the exit path ln(l/lmax) and exit |mu|, or
 * of the displacement/lmax toward the far face and final mu' at truncation.
 * The transport kernel evaluates it with BF16 tensor-core MMA and FP32
 * accumulation on batches of 16 histories per warp. */
#define IMC_SURROGATE_PARAMS 12800

typedef struct ImcSurrogateTrainConfig {
    uint64_t seed;       /* training walks and initial weights */
    int64_t n_samples;   /* analog in-cell walks generated on the device */
    int32_t batch;       /* walks per Adam step; a multiple of 64 dividing n_samples */
    int32_t iterations;  /* Adam steps */
    float lr;            /* peak learning rate (cosine decay) */
    float lr_min;        /* final learning rate */
} ImcSurrogateTrainConfig;

/* *count = IMC_SURROGATE_PARAMS. */
int imc_surrogate_param_count(int *count);
/* Generates walks and trains the network on the GPU (FP32 forward and
 * backward, Adam).  params: IMC_SURROGATE_PARAMS floats out; loss_history:
 * `iterations` mean batch losses out, or NULL.  Deterministic in the config. */
int imc_surrogate_train(const ImcSurrogateTrainConfig *cfg, float *params, float *loss_history);
/* Analog in-cell walks (the training targets) on the GPU.  state: n x 4
 * (d_n, d_f, mu', lmax) in host memory, or NULL to draw training states.
 * Out (host): x n x 4 network inputs, cls n outcomes (0 near, 1 far,
 * 2 truncated), tgt n x 2 (ln(l/lmax), |mu|) or (displacement/lmax, mu'). */
int imc_surrogate_walk(uint64_t seed, const float *state, int64_t n, float *x, int32_t *cls, float *tgt);
/* Training loss (mean over the n samples) and its gradient with respect to
 * the parameters, on the GPU in FP32; all buffers in host memory. */
int imc_surrogate_grad(const float *params, const float *x, const int32_t *cls, const float *tgt, int64_t n,
                       float *grad, double *loss);
/* Network outputs (n x 64, host) for n inputs (n x 4, host) by the transport
 * kernel's BF16 tensor-core forward pass. */
int imc_surrogate_forward(const float *params, const float *x, int64_t n, float *out);
/* Outcomes sampled from the network at n walk states (n x 4, host) as the
 * transport kernel samples them: cls, y0, y1 as imc_surrogate_walk's. */
int imc_surrogate_sample(const float *params, uint64_t seed, const float *state, int64_t n, int32_t *cls,
                         float *y0, float *y1);
/* Turns the surrogate on for this handle's transport (params: n_params ==
 * IMC_SURROGATE_PARAMS floats, host) or off (params NULL).  1D geometry with
 * FP32 or FP16 particle state only.  In a cell at least 8 mean free paths
 * wide, a history with at least 32 mean free paths of path left before census
 * or the cut-off is moved by one network query instead of its analog
 * collisions (lmax above 1e4 is walked in 1e4 pieces); elsewhere transport
 * is analog.  ImcStepStats.surrogate_calls counts the queries.  A step gate
 * keeps the network on for the next step only when this step made at least
 * two queries per GPU thread (2 x SMs x 1024); below that the step runs the
 * analog transport alone.  A closed gate re-opens to measure when the step's
 * histories have doubled since it closed and every 32 steps.  The gate reads
 * only the step's own counts, so runs stay bit-reproducible. */
int imc_set_surrogate(ImcHandle *h, const float *params, int64_t n_params);
/* *active = 1 while the surrogate is on. */
int imc_get_surrogate_active(const ImcHandle *h, int *active);

#ifdef __cplusplus
}
#endif
#endif /* IMC_H_ */
