// imc_api.cu -- the C ABI of include/imc.h: handle lifetime, one entry point
// per reference stage, whole-step and whole-run drivers, state access.
//
// One handle owns one CUDA stream and all device memory of one simulation.
// Sizes that change from step to step (census length, births) live in device
// scalars, so the host never needs them to launch: a step is a fixed sequence
// of launches, captured once per ping-pong parity as a CUDA graph.  The host
// keeps an exact mirror of the simulation clock (the timestep arithmetic is
// deterministic FP64), so it knows how many steps a run has without reading
// the device.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>
#include <thread>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "imc.h"  // include/imc.h (on the -I path)
#include "imc_device.cuh"
#include "imc_internal.h"
#include "imc_surrogate.cuh"

using namespace imc;

namespace {

std::string g_create_err;
int g_create_code = IMC_OK;

struct Stage { enum { Fresh = 0, Updated, Sourced, Transported, Cleaned, Tallied, Checked }; };

}  // namespace

struct ImcHandle {
    // the deck's scalars; the arrays read after imc_create (cell widths,
    // energy scales) point into host_dx / host_dy / host_scales, copies the
    // handle owns: the caller's arrays are read during imc_create only
    ImcDeck deck;
    std::vector<double> host_dx, host_dy, host_scales;
    int device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    int prec = 1, geometry = 1, nx = 1, ny = 1, nc = 1, K = 1, nslots = 0;
    CellArgs ca{};
    Scalars *d_sc = nullptr;
    std::vector<void *> allocs;  // cell / scratch allocations
    // particle buffers
    PBufRaw buf[2]{};   // which one holds the list is Scalars::cur, on the device
    std::vector<void *> pallocs;
    long long capacity = 0, ntiles_cap = 0;
    long long *tile_cnt = nullptr, *tile_off = nullptr;
    DevStats *d_stats = nullptr;
    long long stats_cap = 0;
    int grid_transport = 0, block_transport = 256, grid_emit = 0;
    int grid_full = 0;  // resident transport blocks on the whole GPU
    // learned surrogate: device image of the network (ca.surr_image points
    // into it while the surrogate is on) and its kernel's persistent grid
    void *d_surr_image = nullptr;
    SurrWave wave{};                   // queues of the surrogate transport passes
    std::vector<void *> qallocs;
    long long qcap = 0;
    SurrShapes sshape{};
    cudaGraphExec_t graph = nullptr;  // one step, captured once
    bool timing = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> ev_pool;
    double transport_ms = 0.0;
    int64_t transport_launches = 0;
    // host mirror of the clock
    double t = 0.0, dt = 0.0;
    int64_t step = 0;
    bool finished = false;
    // totals over every step run since imc_create
    int64_t tot_segments = 0, tot_histories = 0, tot_calls = 0;
    int stage = Stage::Fresh;
    long long n_census_host = 0;
    ImcStepStats last{};
    std::string err;
    int err_code = IMC_OK;
};

namespace {

int fail(ImcHandle *h, int code, const std::string &msg) {
    if (h) { h->err = msg; h->err_code = code; }
    else { g_create_err = msg; g_create_code = code; }
    return code;
}

#define CK(h, call)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail((h), e_ == cudaErrorMemoryAllocation ? IMC_ERR_OOM : IMC_ERR_CUDA,       \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

#define CKL(h)                                                                                   \
    do {                                                                                         \
        cudaError_t e_ = cudaGetLastError();                                                     \
        if (e_ != cudaSuccess) return fail((h), IMC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
    } while (0)

template <class T> int dalloc(ImcHandle *h, T **p, size_t n, std::vector<void *> &list) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return fail(h, IMC_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    list.push_back(q);
    *p = (T *)q;
    return IMC_OK;
}

// Synchronous copy on the handle's own stream (never the legacy default
// stream), so handles driven from different host threads -- one of them
// possibly capturing its step graph -- do not interact.
cudaError_t hcopy(const ImcHandle *h, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, h->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(h->stream);
}
cudaError_t hset(const ImcHandle *h, void *dst, int v, size_t bytes) {
    cudaError_t e = cudaMemsetAsync(dst, v, bytes, h->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(h->stream);
}

template <class T> int upload(ImcHandle *h, T **p, const T *src, size_t n) {
    int rc = dalloc(h, p, n, h->allocs);
    if (rc) return rc;
    if (src && n) CK(h, hcopy(h, *p, src, n * sizeof(T), cudaMemcpyHostToDevice));
    else CK(h, hset(h, *p, 0, std::max<size_t>(n, 1) * sizeof(T)));
    return IMC_OK;
}

size_t state_elem(int prec) { return prec == 0 ? 8 : prec == 1 ? 4 : 2; }
size_t e0_elem(int prec) { return prec == 0 ? 8 : 4; }

int alloc_particles(ImcHandle *h, long long cap, PBufRaw out[2], std::vector<void *> &list) {
    const size_t se = state_elem(h->prec), e0 = e0_elem(h->prec);
    for (int b = 0; b < 2; ++b) {
        PBufRaw &r = out[b];
        r = PBufRaw{};
        int rc;
        if ((rc = dalloc(h, (char **)&r.t, se * cap, list))) return rc;
        if ((rc = dalloc(h, (char **)&r.x, se * cap, list))) return rc;
        if ((rc = dalloc(h, (char **)&r.ux, se * cap, list))) return rc;
        if (h->geometry == 2) {
            if ((rc = dalloc(h, (char **)&r.y, se * cap, list))) return rc;
            if ((rc = dalloc(h, (char **)&r.uy, se * cap, list))) return rc;
        }
        if ((rc = dalloc(h, (char **)&r.E, se * cap, list))) return rc;
        if ((rc = dalloc(h, (char **)&r.E0, e0 * cap, list))) return rc;
        if ((rc = dalloc(h, &r.cs, cap, list))) return rc;
        if ((rc = dalloc(h, &r.alive, cap, list))) return rc;
    }
    return IMC_OK;
}

void free_list(std::vector<void *> &list) {
    for (void *p : list) cudaFree(p);
    list.clear();
}

void drop_graphs(ImcHandle *h) {
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
}

// Transport blocks for this handle: the resident grid of the whole GPU, or
// fewer for a small particle buffer (16 entries per thread at capacity), so
// that the kernels of small decks run side by side in a batch.
int sized_grid(const ImcHandle *h, int full, int block) {
    const long long want = (h->capacity + 16ll * block - 1) / (16ll * block);
    return (int)std::max<long long>(1, std::min<long long>(full, want));
}

PBufPair pair(const ImcHandle *h) {
    PBufPair p;
    p.b[0] = h->buf[0];
    p.b[1] = h->buf[1];
    return p;
}

long long births_bound(const ImcHandle *h, long long n_census) {
    const ImcDeck &d = h->deck;
    double cm = std::max(d.cellmin, 0.0);
    double nsrc = (double)d.n_input;
    if (d.n_input + n_census > d.n_max) nsrc = std::max(cm, (double)(d.n_max - n_census));
    return (long long)nsrc + (long long)h->nslots * ((long long)cm + 2) + 16;
}

int tile_alloc(ImcHandle *h) {
    h->ntiles_cap = (h->capacity + kCompactTile - 1) / kCompactTile;
    int rc;
    if ((rc = dalloc(h, &h->tile_cnt, h->ntiles_cap + 1, h->pallocs))) return rc;
    if ((rc = dalloc(h, &h->tile_off, h->ntiles_cap + 1, h->pallocs))) return rc;
    return IMC_OK;
}

// Grow both particle buffers so that `need` particles fit; keeps the list.
// queues of the surrogate transport: every live history fits in each
int surr_queue_alloc(ImcHandle *h) {
    if (h->qcap >= h->capacity) return IMC_OK;
    free_list(h->qallocs);
    h->qcap = 0;
    const long long cap = h->capacity;
    auto take = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        h->qallocs.push_back(p);
        return p;
    };
    for (SurrQueue *q : {&h->wave.ask, &h->wave.resume}) {
        q->x = (float *)take(4 * cap);
        q->mu = (float *)take(4 * cap);
        q->t = (float *)take(4 * cap);
        q->E = (float *)take(4 * cap);
        q->E0 = (float *)take(4 * cap);
        q->cs = (int32_t *)take(4 * cap);
        q->cs_list = (int32_t *)take(4 * cap);
        q->idx = (long long *)take(8 * cap);
        if (!q->x || !q->mu || !q->t || !q->E || !q->E0 || !q->cs || !q->cs_list || !q->idx) {
            free_list(h->qallocs);
            return fail(h, IMC_ERR_OOM, "surrogate queues");
        }
    }
    h->qcap = cap;
    return IMC_OK;
}

int grow(ImcHandle *h, long long need) {
    if (need <= h->capacity) return IMC_OK;
    long long ncap = std::max<long long>(need + need / 2, h->capacity + h->capacity / 2);
    CK(h, cudaStreamSynchronize(h->stream));
    Scalars sc;
    CK(h, hcopy(h, &sc, h->d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost));
    const long long n = sc.n_particles;
    PBufRaw nb[2];
    std::vector<void *> nlist;
    long long old_cap = h->capacity;
    h->capacity = ncap;
    int rc = alloc_particles(h, ncap, nb, nlist);
    if (rc) { free_list(nlist); h->capacity = old_cap; return rc; }
    const size_t se = state_elem(h->prec), e0 = e0_elem(h->prec);
    const PBufRaw &o = h->buf[sc.cur];
    PBufRaw &w = nb[0];
    if (n > 0) {
        CK(h, hcopy(h, w.t, o.t, se * n, cudaMemcpyDeviceToDevice));
        CK(h, hcopy(h, w.x, o.x, se * n, cudaMemcpyDeviceToDevice));
        CK(h, hcopy(h, w.ux, o.ux, se * n, cudaMemcpyDeviceToDevice));
        if (h->geometry == 2) {
            CK(h, hcopy(h, w.y, o.y, se * n, cudaMemcpyDeviceToDevice));
            CK(h, hcopy(h, w.uy, o.uy, se * n, cudaMemcpyDeviceToDevice));
        }
        CK(h, hcopy(h, w.E, o.E, se * n, cudaMemcpyDeviceToDevice));
        CK(h, hcopy(h, w.E0, o.E0, e0 * n, cudaMemcpyDeviceToDevice));
        CK(h, hcopy(h, w.cs, o.cs, 4 * n, cudaMemcpyDeviceToDevice));
        CK(h, hcopy(h, w.alive, o.alive, n, cudaMemcpyDeviceToDevice));
    }
    free_list(h->pallocs);
    h->pallocs = nlist;
    h->buf[0] = nb[0];
    h->buf[1] = nb[1];
    sc.cur = 0;
    CK(h, hcopy(h, h->d_sc, &sc, sizeof(Scalars), cudaMemcpyHostToDevice));
    h->ca.capacity = ncap;
    h->grid_transport = sized_grid(h, h->grid_full, h->block_transport);
    if ((rc = tile_alloc(h))) return rc;
    if (h->ca.surr_image && (rc = surr_queue_alloc(h))) return rc;
    drop_graphs(h);
    return IMC_OK;
}

int read_scalars(ImcHandle *h, Scalars *sc) {
    CK(h, cudaMemcpyAsync(sc, h->d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return IMC_OK;
}

void to_stats(const DevStats &d, ImcStepStats *s) {
    s->t = d.t; s->dt = d.dt;
    s->total_energy = d.total_energy;
    s->energy_dep = d.energy_dep;
    s->rad_energy = d.rad_energy;
    s->rad_energy_old = d.rad_energy_old;
    s->lost_energy = d.lost_energy;
    s->energy_error = d.energy_error;
    s->n_census_in = d.n_census_in;
    s->n_sourced = d.n_sourced;
    s->n_census_out = d.n_census_out;
    s->segments = d.segments;
    s->surrogate_calls = d.surrogate_calls;
    s->error_flags = d.error_flags;
    s->step_index = d.step_index;
}

int flags_status(ImcHandle *h, unsigned flags) {
    if (flags & IMC_FLAG_CAPACITY) return fail(h, IMC_ERR_CAPACITY, "particle buffer capacity reached; births clipped");
    if (flags & IMC_FLAG_SEGMENT_CAP) return fail(h, IMC_ERR_SEGMENT_CAP, "a history reached the segment cap");
    if (flags & IMC_FLAG_NO_ENERGY) return fail(h, IMC_ERR_NO_ENERGY, "total source energy is zero or not finite");
    if (flags & (IMC_FLAG_NAN | IMC_FLAG_FIXPOINT_RANGE))
        return fail(h, IMC_ERR_NUMERIC, "non-finite or out-of-range tally contribution");
    return IMC_OK;
}

// host mirror of timestep (src/MixedPrecisionIMC.jl:181-222)
void host_timestep(const ImcDeck &d, double &t, double &dt, bool &finished) {
    if (t == d.t_end) {
        t = d.t_end + dt;
    } else if (d.timestepping == IMC_TS_CONSTANT) {
        if (t + dt > d.t_end) { dt = d.t_end - t; t = d.t_end; }
        else t = t + dt;
    } else {
        if (dt < d.dtmax) {
            dt = dt * d.k;
            if (dt > d.dtmax) dt = d.dtmax;
        }
        if (t + dt > d.t_end) { dt = d.t_end - t; t = d.t_end; }
        else t = t + dt;
    }
    finished = t > d.t_end;
}

// the transport kernel of this handle: analog, or with the learned surrogate
void run_transport(ImcHandle *h, PBufPair bufs, cudaStream_t st) {
    if (h->ca.surr_image) {
        SurrShapes sh = h->sshape;
        sh.analog_grid = sized_grid(h, sh.analog_grid, sh.analog_block);
        sh.query_grid = sized_grid(h, sh.query_grid, sh.query_block);
        launch_transport_surr(h->ca, h->d_sc, h->prec, bufs, h->wave, sh, st);
    }
    else launch_transport(h->ca, h->d_sc, h->prec, bufs, h->grid_transport, st);
}

// The kernel sequence of one step, asynchronous on `st`; the list's buffer is
// chosen on the device, so the same sequence serves every step.  Its halves
// around the transport: update + sourcing, then the compaction (it reads no
// cell field and the tally no particle) and finalize + tally + energycheck +
// timestep in one launch.
void enqueue_before_transport(ImcHandle *h, cudaStream_t st) {
    launch_update(h->ca, h->d_sc, st);
    launch_source(h->ca, h->d_sc, h->prec, pair(h), h->grid_emit, st);
}
void enqueue_after_transport(ImcHandle *h, cudaStream_t st) {
    launch_compact(h->ca, h->d_sc, h->prec, pair(h), h->tile_cnt, h->tile_off, h->ntiles_cap, false, st);
    launch_tally_check_timestep(h->ca, h->d_sc, h->d_stats, h->stats_cap, st);
}

int enqueue_step(ImcHandle *h, bool with_events, int ev_slot) {
    cudaStream_t st = h->stream;
    enqueue_before_transport(h, st);
    if (with_events) CK(h, cudaEventRecord(h->ev_pool[2 * ev_slot], st));
    run_transport(h, pair(h), st);
    if (with_events) CK(h, cudaEventRecord(h->ev_pool[2 * ev_slot + 1], st));
    enqueue_after_transport(h, st);
    CKL(h);
    return IMC_OK;
}

int ensure_events(ImcHandle *h, size_t pairs) {
    while (h->ev_pool.size() < 2 * pairs) {
        cudaEvent_t e;
        CK(h, cudaEventCreate(&e));
        h->ev_pool.push_back(e);
    }
    return IMC_OK;
}

int collect_events(ImcHandle *h, size_t pairs) {
    for (size_t i = 0; i < pairs; ++i) {
        float ms = 0.f;
        CK(h, cudaEventElapsedTime(&ms, h->ev_pool[2 * i], h->ev_pool[2 * i + 1]));
        h->transport_ms += ms;
        h->transport_launches += 1;
    }
    return IMC_OK;
}

int ensure_stats(ImcHandle *h, long long n) {
    if (h->stats_cap >= n) return IMC_OK;
    if (h->d_stats) { cudaFree(h->d_stats); h->d_stats = nullptr; }
    long long cap = std::max<long long>(n, 64);
    void *p = nullptr;
    CK(h, cudaMalloc(&p, sizeof(DevStats) * cap));
    h->d_stats = (DevStats *)p;
    h->stats_cap = cap;
    drop_graphs(h);
    return IMC_OK;
}

std::mutex g_capture_mutex;  // one step-graph capture at a time in the process
std::mutex g_attr_mutex;     // kernel attributes are per process, shared by every handle

// Raises a kernel's dynamic shared-memory limit to at least `smem`, never
// lowering it: handles of different meshes share the kernel, and a handle
// created later must not shrink the limit under one that runs now.
cudaError_t raise_smem_limit(const void *kp, int smem) {
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, kp);
    if (e != cudaSuccess) return e;
    if (smem <= a.maxDynamicSharedSizeBytes) return cudaSuccess;
    return cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

int capture(ImcHandle *h) {
    if (h->graph) return IMC_OK;
    std::lock_guard<std::mutex> lock(g_capture_mutex);
    cudaGraph_t g;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_step(h, false, 0);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(h, IMC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, IMC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    return IMC_OK;
}

int validate(const ImcDeck *d, std::string &why) {
    if (!d) { why = "deck is NULL"; return IMC_ERR_INVALID_ARG; }
    if (d->abi_version != IMC_ABI_VERSION) { why = "abi_version mismatch"; return IMC_ERR_INVALID_ARG; }
    if (d->geometry != IMC_GEOM_1D && d->geometry != IMC_GEOM_2D) { why = "geometry must be 1 or 2"; return IMC_ERR_INVALID_ARG; }
    if (d->nx <= 0 || d->ny <= 0) { why = "nx, ny must be positive"; return IMC_ERR_INVALID_ARG; }
    long long nc = (long long)d->nx * (d->geometry == IMC_GEOM_2D ? d->ny : 1);
    if (nc >= (1ll << 24)) { why = "at most 2^24 - 1 cells"; return IMC_ERR_INVALID_ARG; }
    if (d->precision < IMC_FP64 || d->precision > IMC_FP16) { why = "precision must be 0, 1 or 2"; return IMC_ERR_INVALID_ARG; }
    if (d->scale_select_precision < IMC_FP64 || d->scale_select_precision > IMC_FP16) { why = "scale_select_precision must be 0, 1 or 2"; return IMC_ERR_INVALID_ARG; }
    if (d->n_scales < 1 || d->n_scales > 16 || !d->energyscales) { why = "1..16 energy scales required"; return IMC_ERR_INVALID_ARG; }
    if (!d->dx || !d->temp || !d->sigma_a_val || !d->sigma_a_pow || !d->sigma_s_val || !d->sigma_s_pow ||
        !d->bee || !d->radsource || !d->t_surface) { why = "a mesh array is NULL"; return IMC_ERR_INVALID_ARG; }
    if (d->geometry == IMC_GEOM_2D && !d->dy) { why = "dy is NULL in 2D"; return IMC_ERR_INVALID_ARG; }
    for (int i = 0; i < d->nx; ++i) if (!(d->dx[i] > 0)) { why = "dx must be positive"; return IMC_ERR_INVALID_ARG; }
    if (d->geometry == IMC_GEOM_2D)
        for (int j = 0; j < d->ny; ++j) if (!(d->dy[j] > 0)) { why = "dy must be positive"; return IMC_ERR_INVALID_ARG; }
    for (int k = 0; k < d->n_scales; ++k) if (!(d->energyscales[k] > 0)) { why = "energy scales must be positive"; return IMC_ERR_INVALID_ARG; }
    if (!(d->distancescale > 0) || !(d->phys_c > 0)) { why = "PHYS_C and DISTANCESCALE must be positive"; return IMC_ERR_INVALID_ARG; }
    if (d->timestepping == IMC_TS_CONSTANT && !(d->dt > 0)) { why = "DT must be positive"; return IMC_ERR_INVALID_ARG; }
    if (d->timestepping == IMC_TS_RAMP && (!(d->dt0 > 0) || !(d->dtmax > 0) || !(d->k > 0))) { why = "DT0, DTMAX, K must be positive"; return IMC_ERR_INVALID_ARG; }
    if (d->n_input < 0 || d->n_max < 0) { why = "NINPUT, NMAX must be non-negative"; return IMC_ERR_INVALID_ARG; }
    for (int b = 0; b < (d->geometry == IMC_GEOM_2D ? 4 : 2); ++b)
        if (d->bc[b] != IMC_BC_VACUUM && d->bc[b] != IMC_BC_REFLECT) { why = "bc must be VACUUM or REFLECT"; return IMC_ERR_INVALID_ARG; }
    return IMC_OK;
}

int check_device(ImcHandle *h, int *dev, int *sms) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(h, IMC_ERR_NO_DEVICE, "no CUDA device");
    CK(h, cudaGetDevice(dev));
    cudaDeviceProp p;
    CK(h, cudaGetDeviceProperties(&p, *dev));
    if (!(p.major == 10 && p.minor == 3))
        return fail(h, IMC_ERR_NO_DEVICE, std::string("libimc is built for sm_103a; device is ") + p.name);
    *sms = p.multiProcessorCount;
    return IMC_OK;
}

// ------------------------------------------------------------- fused batch
// One half of a handle's step sequence (before or after the transport),
// captured as a graph.
int capture_half(ImcHandle *h, bool before, cudaGraph_t *g) {
    std::lock_guard<std::mutex> lock(g_capture_mutex);
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    if (before) enqueue_before_transport(h, h->stream);
    else enqueue_after_transport(h, h->stream);
    const cudaError_t le = cudaGetLastError();
    const cudaError_t e = cudaStreamEndCapture(h->stream, g);
    if (e != cudaSuccess) return fail(h, IMC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    if (le != cudaSuccess) {
        cudaGraphDestroy(*g);
        return fail(h, IMC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(le));
    }
    return IMC_OK;
}

// The fused batch's step graph.
struct FusedBatch {
    cudaStream_t st = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int> members;    // deck indices of the graph, in launch order
    ~FusedBatch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (st) cudaStreamDestroy(st);
    }
    void drop() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
};
// the fused transport's deck arguments live in one constant-memory table:
// one fused batch at a time in the process
std::mutex g_fused_mutex;

Deck1DArgs deck1d_args(const CellArgs &ca) {
    Deck1DArgs a{};
    a.nx = ca.nx; a.nc = ca.nc; a.K = ca.K;
    a.bc[0] = ca.bc[0]; a.bc[1] = ca.bc[1];
    a.dx = ca.dx; a.sa = ca.sa; a.fleck = ca.fleck; a.ss = ca.ss; a.scales = ca.scales;
    a.dep_acc = ca.dep_acc; a.rad_acc = ca.rad_acc; a.lost_acc = ca.lost_acc;
    a.c = ca.c; a.ds = ca.ds;
    a.seg_cap = ca.seg_cap;
    a.seed = ca.seed;
    return a;
}

PBufPair1D pair1d(const ImcHandle *h) {
    PBufPair1D p{};
    for (int b = 0; b < 2; ++b) {
        const PBufRaw &r = h->buf[b];
        p.b[b].t = r.t; p.b[b].x = r.x; p.b[b].ux = r.ux; p.b[b].E = r.E; p.b[b].E0 = r.E0;
        p.b[b].cs = r.cs; p.b[b].alive = r.alive;
    }
    return p;
}

// Builds the step graph over `members`: every deck's update + sourcing, one
// fused transport launch over all of them, then every deck's compaction and
// tally + energycheck + timestep.  *bad: the deck whose capture failed (the
// first member for a failure of the batch as a whole, whose message it holds).
int build_fused(FusedBatch &F, ImcHandle *const *hs, const std::vector<int> &members, int prec, int *bad) {
    F.drop();
    F.members.clear();
    const int n = (int)members.size();
    ImcHandle *h0 = hs[members[0]];
    *bad = members[0];
    std::vector<Deck1DArgs> cas((size_t)n);
    std::vector<PBufPair1D> bufs((size_t)n);
    std::vector<Scalars *> scs((size_t)n);
    int smem = 0;
    for (int j = 0; j < n; ++j) {
        ImcHandle *h = hs[members[j]];
        cas[j] = deck1d_args(h->ca);
        bufs[j] = pair1d(h);
        scs[j] = h->d_sc;
        smem = std::max(smem, transport_shape(h->ca, prec).smem);
    }
    CK(h0, set_transport_multi_decks(cas.data(), bufs.data(), scs.data(), n, F.st));
    const void *kp = transport_multi_ptr(prec);
    const int block = transport_multi_block(prec);
    CK(h0, raise_smem_limit(kp, smem));
    int per_sm = 0;
    CK(h0, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kp, block, smem));
    if (per_sm < 1) return fail(h0, IMC_ERR_CUDA, "fused transport: no block fits on an SM");
    const int grid = per_sm * h0->sm_count;
    cudaGraph_t G = nullptr;
    CK(h0, cudaGraphCreate(&G, 0));
    int rc = IMC_OK;
    std::vector<cudaGraphNode_t> before((size_t)n);
    cudaGraphNode_t tn = nullptr;
    auto add_half = [&](int j, bool first, const cudaGraphNode_t *deps, size_t ndeps, cudaGraphNode_t *node) {
        ImcHandle *h = hs[members[j]];
        cudaGraph_t g = nullptr;
        if ((rc = capture_half(h, first, &g))) { *bad = members[j]; return; }
        const cudaError_t e = cudaGraphAddChildGraphNode(node, G, deps, ndeps, g);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            rc = fail(h, IMC_ERR_CUDA, std::string("child graph: ") + cudaGetErrorString(e));
            *bad = members[j];
        }
    };
    for (int j = 0; j < n && !rc; ++j) add_half(j, true, nullptr, 0, &before[j]);
    if (!rc) {
        int nd = n;
        void *args[] = {&nd};
        cudaKernelNodeParams p{};
        p.func = const_cast<void *>(kp);
        p.gridDim = dim3((unsigned)grid);
        p.blockDim = dim3((unsigned)block);
        p.sharedMemBytes = (unsigned)smem;
        p.kernelParams = args;
        p.extra = nullptr;
        const cudaError_t e = cudaGraphAddKernelNode(&tn, G, before.data(), (size_t)n, &p);
        if (e != cudaSuccess) rc = fail(h0, IMC_ERR_CUDA, std::string("fused transport node: ") + cudaGetErrorString(e));
    }
    for (int j = 0; j < n && !rc; ++j) {
        cudaGraphNode_t after = nullptr;
        add_half(j, false, &tn, 1, &after);
    }
    if (!rc) {
        const cudaError_t e = cudaGraphInstantiate(&F.exec, G, 0);
        if (e != cudaSuccess) {
            F.exec = nullptr;
            rc = fail(h0, IMC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        }
    }
    cudaGraphDestroy(G);
    if (!rc) F.members = members;
    return rc;
}

// The host clock mirror and the totals after `done` steps run on the device,
// whose statistics start at ring slot `slot0` (copied in at most two pieces).
int absorb_steps(ImcHandle *h, unsigned long long slot0, int64_t done, ImcStepStats *stats, unsigned *allflags) {
    std::vector<DevStats> ds((size_t)done);
    const unsigned long long cap = (unsigned long long)h->stats_cap;
    for (int64_t s = 0; s < done;) {
        const unsigned long long slot = (slot0 + (unsigned long long)s) % cap;
        const int64_t len = std::min<int64_t>(done - s, (int64_t)(cap - slot));
        CK(h, hcopy(h, &ds[(size_t)s], h->d_stats + slot, sizeof(DevStats) * (size_t)len, cudaMemcpyDeviceToHost));
        s += len;
    }
    for (int64_t s = 0; s < done; ++s) {
        if (stats) to_stats(ds[s], &stats[s]);
        *allflags |= ds[s].error_flags;
        h->tot_segments += ds[s].segments;
        h->tot_histories += ds[s].n_census_in + ds[s].n_sourced;
        h->tot_calls += ds[s].surrogate_calls;
        bool fin;
        host_timestep(h->deck, h->t, h->dt, fin);
        h->finished = fin;
        h->step += 1;
    }
    if (done > 0) to_stats(ds[done - 1], &h->last);
    h->stage = Stage::Fresh;
    return IMC_OK;
}

}  // namespace

extern "C" {

int imc_abi_version(void) { return IMC_ABI_VERSION; }

int imc_device_info(char *name, size_t len, int *sm_count, int *cc_major, int *cc_minor) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return IMC_ERR_NO_DEVICE;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return IMC_ERR_NO_DEVICE;
    if (name && len) { std::strncpy(name, p.name, len - 1); name[len - 1] = 0; }
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return IMC_OK;
}

int imc_last_error(const ImcHandle *h, char *buf, size_t len) {
    const std::string &m = h ? h->err : g_create_err;
    int code = h ? h->err_code : g_create_code;
    if (buf && len) { std::strncpy(buf, m.c_str(), len - 1); buf[len - 1] = 0; }
    return code;
}

int imc_create(const ImcDeck *d, ImcHandle **out) {
    if (!out) return fail(nullptr, IMC_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    std::string why;
    int rc = validate(d, why);
    if (rc) return fail(nullptr, rc, why);
    ImcHandle *h = new ImcHandle();
    h->deck = *d;
    h->host_dx.assign(d->dx, d->dx + d->nx);
    if (d->geometry == IMC_GEOM_2D) h->host_dy.assign(d->dy, d->dy + d->ny);
    h->host_scales.assign(d->energyscales, d->energyscales + d->n_scales);
    h->deck.dx = h->host_dx.data();
    h->deck.dy = d->geometry == IMC_GEOM_2D ? h->host_dy.data() : nullptr;
    h->deck.energyscales = h->host_scales.data();
    auto bail = [&](int code) {
        g_create_err = h->err; g_create_code = code;
        imc_destroy(h);
        return code;
    };
    if ((rc = check_device(h, &h->device, &h->sm_count))) return bail(rc);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(h, IMC_ERR_CUDA, "cudaStreamCreate failed"));
    h->prec = d->precision;
    h->geometry = d->geometry;
    h->nx = d->nx;
    h->ny = d->geometry == IMC_GEOM_2D ? d->ny : 1;
    h->nc = h->nx * h->ny;
    h->K = d->n_scales;
    h->nslots = (d->geometry == IMC_GEOM_1D ? 2 : 2 * h->nx + 2 * h->ny) + 2 * h->nc;
    const int nc = h->nc, K = h->K;
    CellArgs &ca = h->ca;
    ca.geometry = d->geometry; ca.nx = h->nx; ca.ny = h->ny; ca.nc = nc; ca.K = K;
    std::vector<double> ones(std::max(nc, 1), 1.0);
    const int nts = d->geometry == IMC_GEOM_1D ? 2 : 2 * h->nx + 2 * h->ny;
    double *p;
    if ((rc = upload(h, &p, d->dx, h->nx))) return bail(rc); ca.dx = p;
    if ((rc = upload(h, &p, d->geometry == IMC_GEOM_2D ? d->dy : ones.data(), h->ny))) return bail(rc); ca.dy = p;
    {
        // binary32 copies of the widths for the FP32 / FP16 births
        std::vector<float> wf(d->dx, d->dx + h->nx);
        float *fp;
        if ((rc = upload(h, &fp, wf.data(), h->nx))) return bail(rc); ca.dxf = fp;
        wf.assign(h->ny, 1.0f);
        if (d->geometry == IMC_GEOM_2D) for (int j = 0; j < h->ny; ++j) wf[j] = (float)d->dy[j];
        if ((rc = upload(h, &fp, wf.data(), h->ny))) return bail(rc); ca.dyf = fp;
        // surface birth positions: frac * width * DISTANCESCALE in Float64 with
        // the width and scale first rounded to the arithmetic type
        const double fr[6] = {0.01, 0.99, 0.001, 0.999, 0.001, 0.999};
        const double w[6] = {d->dx[0], d->dx[h->nx - 1], d->dx[0], d->dx[h->nx - 1],
                             d->geometry == IMC_GEOM_2D ? d->dy[0] : 1.0,
                             d->geometry == IMC_GEOM_2D ? d->dy[h->ny - 1] : 1.0};
        const float dsf = (float)d->distancescale;
        for (int q = 0; q < 6; ++q) {
            ca.surf_f[q] = (float)(fr[q] * (double)(float)w[q] * (double)dsf);
            ca.surf_d[q] = fr[q] * w[q] * d->distancescale;
        }
    }
    if ((rc = upload(h, &ca.temp, d->temp, nc))) return bail(rc);
    if ((rc = upload(h, &ca.bee, d->bee, nc))) return bail(rc);
    if ((rc = upload(h, &ca.beta, ones.data(), nc))) return bail(rc);
    if ((rc = upload<double>(h, &ca.fleck, nullptr, nc))) return bail(rc);
    if ((rc = upload(h, &ca.sa, d->sigma_a_val, nc))) return bail(rc);
    if ((rc = upload(h, &ca.ss, d->sigma_s_val, nc))) return bail(rc);
    if ((rc = upload(h, &p, d->sigma_a_val, nc))) return bail(rc); ca.sa_val = p;
    if ((rc = upload(h, &p, d->sigma_a_pow, nc))) return bail(rc); ca.sa_pow = p;
    if ((rc = upload(h, &p, d->sigma_s_val, nc))) return bail(rc); ca.ss_val = p;
    if ((rc = upload(h, &p, d->sigma_s_pow, nc))) return bail(rc); ca.ss_pow = p;
    if ((rc = upload(h, &p, d->radsource, nc))) return bail(rc); ca.radsource = p;
    if ((rc = upload(h, &p, d->t_surface, nts))) return bail(rc); ca.tsurf = p;
    if ((rc = upload(h, &p, d->energyscales, K))) return bail(rc); ca.scales = p;
    if ((rc = upload<double>(h, &ca.energydep, nullptr, (size_t)K * nc))) return bail(rc);
    if ((rc = upload<double>(h, &ca.emitted, nullptr, (size_t)K * nc))) return bail(rc);
    if ((rc = upload<double>(h, &ca.radenergydens, nullptr, nc))) return bail(rc);
    if ((rc = upload<double>(h, &ca.matenergydens, nullptr, nc))) return bail(rc);
    if ((rc = upload<long long>(h, &ca.dep_acc, nullptr, 3 * (size_t)K * nc))) return bail(rc);
    if ((rc = upload<long long>(h, &ca.rad_acc, nullptr, 3 * (size_t)K * nc))) return bail(rc);
    if ((rc = upload<long long>(h, &ca.lost_acc, nullptr, 3 * (size_t)K))) return bail(rc);
    ca.nslots = h->nslots;
    if ((rc = upload<double>(h, &ca.slot_e, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<double>(h, &ca.slot_s, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<double>(h, &ca.slot_nrg, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<float>(h, &ca.slot_nrg_f, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<int>(h, &ca.slot_j, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<long long>(h, &ca.slot_n, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<long long>(h, &ca.slot_off, nullptr, h->nslots))) return bail(rc);
    if ((rc = upload<double>(h, &ca.slot_q, nullptr, h->nslots))) return bail(rc);
    ca.nblk_slot = (h->nslots + kCellThreads - 1) / kCellThreads;
    ca.nblk_cell = (nc + kCellThreads - 1) / kCellThreads;
    if ((rc = upload<double>(h, &ca.part_src, nullptr, (size_t)ca.nblk_slot * 12))) return bail(rc);
    if ((rc = upload<double>(h, &ca.part_emax, nullptr, (size_t)ca.nblk_slot))) return bail(rc);
    if ((rc = upload<double>(h, &ca.part_tally, nullptr, (size_t)ca.nblk_cell * (K + 1) * 2))) return bail(rc);
    for (int b = 0; b < 4; ++b) ca.bc[b] = d->bc[b];
    ca.c = d->phys_c; ca.a = d->phys_a; ca.alpha = d->alpha; ca.ds = d->distancescale;
    ca.temp_floor = d->temp_floor; ca.cellmin = d->cellmin;
    ca.linearized = d->linearized ? 1 : 0; ca.marshak = d->marshak_opacity ? 1 : 0;
    ca.sel_prec = d->scale_select_precision;
    ca.timestepping = d->timestepping;
    ca.n_input = d->n_input; ca.n_max = d->n_max;
    ca.seg_cap = d->segment_cap > 0 ? d->segment_cap : 10000000;
    ca.seed = d->seed;
    double dxmin = *std::min_element(d->dx, d->dx + h->nx);
    double dymin = d->geometry == IMC_GEOM_2D ? *std::min_element(d->dy, d->dy + h->ny) : 1.0;
    ca.vol_min = dxmin * dymin;
    ca.scale_min = *std::min_element(d->energyscales, d->energyscales + K);
    ca.t_end = d->t_end; ca.dtmax = d->dtmax; ca.kfac = d->k;
    // particle buffers
    long long cap = d->capacity > 0 ? d->capacity : (d->n_max + 2 * births_bound(h, 0));
    if (cap < 1024) cap = 1024;
    h->capacity = cap;
    ca.capacity = cap;
    if ((rc = alloc_particles(h, cap, h->buf, h->pallocs))) return bail(rc);
    if ((rc = tile_alloc(h))) return bail(rc);
    // scalars
    Scalars sc{};
    sc.emax_census_exp = kNoExp;
    sc.surr_gate = 1;
    h->t = 0.0;
    h->dt = d->timestepping == IMC_TS_RAMP ? d->dt0 : d->dt;
    sc.t = h->t; sc.dt = h->dt;
    void *q = nullptr;
    if (cudaMalloc(&q, sizeof(Scalars)) != cudaSuccess) return bail(fail(h, IMC_ERR_OOM, "cudaMalloc scalars"));
    h->allocs.push_back(q);
    h->d_sc = (Scalars *)q;
    if (hcopy(h, h->d_sc, &sc, sizeof(Scalars), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(h, IMC_ERR_CUDA, "upload scalars"));
    if ((rc = ensure_stats(h, 64))) return bail(rc);
    // launch shapes: persistent grids sized by occupancy on this GPU
    TransportShape shape = transport_shape(ca, h->prec);
    const int smem = shape.smem;
    h->block_transport = shape.block;
    const void *kp = transport_kernel_ptr(ca, h->prec);
    if (smem > 227 * 1024) return bail(fail(h, IMC_ERR_INVALID_ARG, "mesh too large for the shared-memory transport table"));
    if (smem > 48 * 1024)
        if (raise_smem_limit(kp, smem) != cudaSuccess)
            return bail(fail(h, IMC_ERR_CUDA, "cudaFuncSetAttribute(smem)"));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kp, h->block_transport, smem) != cudaSuccess || per_sm < 1)
        return bail(fail(h, IMC_ERR_CUDA, "transport kernel cannot be resident"));
    h->grid_full = h->sm_count * per_sm;
    ca.surr_min_calls = 2ll * h->sm_count * 1024;  // two queries per thread of the GPU
    h->grid_transport = sized_grid(h, h->grid_full, h->block_transport);
    h->grid_emit = h->sm_count * 4;
    if (cudaEventCreate(&h->ev[0]) != cudaSuccess || cudaEventCreate(&h->ev[1]) != cudaSuccess)
        return bail(fail(h, IMC_ERR_CUDA, "cudaEventCreate"));
    *out = h;
    return IMC_OK;
}

int imc_destroy(ImcHandle *h) {
    if (!h) return IMC_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graphs(h);
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    for (int i = 0; i < 2; ++i) if (h->ev[i]) cudaEventDestroy(h->ev[i]);
    if (h->d_stats) cudaFree(h->d_stats);
    if (h->d_surr_image) cudaFree(h->d_surr_image);
    free_list(h->qallocs);
    free_list(h->pallocs);
    free_list(h->allocs);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return IMC_OK;
}

int imc_update(ImcHandle *h) {
    if (!h) return IMC_ERR_INVALID_ARG;
    launch_update(h->ca, h->d_sc, h->stream);
    CKL(h);
    CK(h, cudaStreamSynchronize(h->stream));
    h->stage = Stage::Updated;
    return IMC_OK;
}

int imc_sourcing(ImcHandle *h) {
    if (!h) return IMC_ERR_INVALID_ARG;
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    if ((rc = grow(h, sc.n_particles + births_bound(h, sc.n_particles)))) return rc;
    launch_source(h->ca, h->d_sc, h->prec, pair(h), h->grid_emit, h->stream);
    CKL(h);
    if ((rc = read_scalars(h, &sc))) return rc;
    h->stage = Stage::Sourced;
    if (sc.flags & (IMC_FLAG_CAPACITY | IMC_FLAG_NO_ENERGY)) return flags_status(h, sc.flags);
    return IMC_OK;
}

int imc_transport(ImcHandle *h) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (h->stage != Stage::Sourced) launch_prepare_transport(h->ca, h->d_sc, h->stream);
    if (h->timing) CK(h, cudaEventRecord(h->ev[0], h->stream));
    run_transport(h, pair(h), h->stream);
    CKL(h);
    if (h->timing) {
        CK(h, cudaEventRecord(h->ev[1], h->stream));
        CK(h, cudaEventSynchronize(h->ev[1]));
        float ms = 0;
        CK(h, cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
        h->transport_ms += ms;
        h->transport_launches += 1;
    }
    launch_finalize(h->ca, h->d_sc, h->stream);
    CKL(h);
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    h->stage = Stage::Transported;
    return flags_status(h, sc.flags & (IMC_FLAG_SEGMENT_CAP | IMC_FLAG_NAN | IMC_FLAG_FIXPOINT_RANGE));
}

int imc_clean(ImcHandle *h) {
    if (!h) return IMC_ERR_INVALID_ARG;
    // Clean.clean removes every killed particle (forced compaction)
    launch_compact(h->ca, h->d_sc, h->prec, pair(h), h->tile_cnt, h->tile_off, h->ntiles_cap, true, h->stream);
    CKL(h);
    CK(h, cudaStreamSynchronize(h->stream));
    h->stage = Stage::Cleaned;
    return IMC_OK;
}

int imc_tally(ImcHandle *h) {
    if (!h) return IMC_ERR_INVALID_ARG;
    launch_tally(h->ca, h->d_sc, h->stream);
    CKL(h);
    CK(h, cudaStreamSynchronize(h->stream));
    h->stage = Stage::Tallied;
    return IMC_OK;
}

int imc_energycheck(ImcHandle *h, double *energy_error) {
    if (!h) return IMC_ERR_INVALID_ARG;
    launch_energycheck(h->ca, h->d_sc, h->d_stats, h->stats_cap, h->stream);
    CKL(h);
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    DevStats ds;
    CK(h, hcopy(h, &ds, h->d_stats + (sc.step % (unsigned long long)h->stats_cap), sizeof(DevStats),
                     cudaMemcpyDeviceToHost));
    to_stats(ds, &h->last);
    if (energy_error) *energy_error = sc.energy_err;
    h->stage = Stage::Checked;
    return IMC_OK;
}

int imc_timestep(ImcHandle *h, int *done) {
    if (!h) return IMC_ERR_INVALID_ARG;
    launch_timestep(h->ca, h->d_sc, h->stream);
    CKL(h);
    CK(h, cudaStreamSynchronize(h->stream));
    bool fin;
    host_timestep(h->deck, h->t, h->dt, fin);
    h->finished = fin;
    h->step += 1;
    h->stage = Stage::Fresh;
    if (done) *done = fin ? 1 : 0;
    return IMC_OK;
}

int imc_step(ImcHandle *h, ImcStepStats *stats, int *done) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (h->finished) { if (done) *done = 1; return IMC_OK; }
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    if ((rc = grow(h, sc.n_particles + births_bound(h, sc.n_particles)))) return rc;
    if (h->timing) {
        if ((rc = ensure_events(h, 1))) return rc;
        if ((rc = enqueue_step(h, true, 0))) return rc;
    } else {
        if ((rc = capture(h))) return rc;
        CK(h, cudaGraphLaunch(h->graph, h->stream));
    }
    if ((rc = read_scalars(h, &sc))) return rc;
    if (h->timing && (rc = collect_events(h, 1))) return rc;
    DevStats ds;
    CK(h, hcopy(h, &ds, h->d_stats + ((sc.step - 1u) % (unsigned long long)h->stats_cap), sizeof(DevStats),
                     cudaMemcpyDeviceToHost));
    to_stats(ds, &h->last);
    h->tot_segments += ds.segments;
    h->tot_histories += ds.n_census_in + ds.n_sourced;
    h->tot_calls += ds.surrogate_calls;
    if (stats) *stats = h->last;
    bool fin;
    host_timestep(h->deck, h->t, h->dt, fin);
    h->finished = fin;
    h->step += 1;
    h->stage = Stage::Fresh;
    if (done) *done = fin ? 1 : 0;
    return flags_status(h, ds.error_flags);
}

int imc_run(ImcHandle *h, int64_t max_steps, ImcStepStats *stats, int64_t *n_steps, double *device_ms) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (n_steps) *n_steps = 0;
    if (device_ms) *device_ms = 0.0;
    // steps this run will take, from the host clock mirror
    std::vector<std::pair<double, double>> sched;
    {
        double t = h->t, dt = h->dt;
        bool fin = h->finished;
        while (!fin && (int64_t)sched.size() < max_steps) {
            sched.emplace_back(t, dt);
            host_timestep(h->deck, t, dt, fin);
        }
    }
    const int64_t N = (int64_t)sched.size();
    if (N == 0) return IMC_OK;
    int rc;
    if ((rc = ensure_stats(h, N))) return rc;
    Scalars sc;
    if ((rc = read_scalars(h, &sc))) return rc;
    // first stats slot of this run
    const unsigned long long slot0 = sc.step;
    CK(h, cudaEventRecord(h->ev[0], h->stream));
    int64_t done_steps = 0;
    long long n_census = sc.n_particles;
    while (done_steps < N) {
        // largest chunk whose worst-case births fit the buffers
        int64_t m = 0;
        long long bound = n_census;
        while (m < 64 && done_steps + m < N) {
            long long nb = bound + births_bound(h, bound);
            if (nb > h->capacity) break;
            bound = nb;
            ++m;
        }
        if (m == 0) {
            CK(h, cudaEventRecord(h->ev[1], h->stream));
            if ((rc = grow(h, n_census + 4 * births_bound(h, n_census)))) return rc;
            continue;
        }
        if (h->timing) {
            if ((rc = ensure_events(h, (size_t)m))) return rc;
            for (int64_t s = 0; s < m; ++s)
                if ((rc = enqueue_step(h, true, (int)s))) return rc;
        } else {
            if ((rc = capture(h))) return rc;
            for (int64_t s = 0; s < m; ++s) CK(h, cudaGraphLaunch(h->graph, h->stream));
        }
        done_steps += m;
        if ((rc = read_scalars(h, &sc))) return rc;
        if (h->timing && (rc = collect_events(h, (size_t)m))) return rc;
        n_census = sc.n_particles;
        if (sc.flags & (IMC_FLAG_CAPACITY | IMC_FLAG_SEGMENT_CAP | IMC_FLAG_NAN | IMC_FLAG_FIXPOINT_RANGE | IMC_FLAG_NO_ENERGY))
            break;
    }
    CK(h, cudaEventRecord(h->ev[1], h->stream));
    CK(h, cudaEventSynchronize(h->ev[1]));
    float ms = 0.f;
    CK(h, cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
    if (device_ms) *device_ms = ms;
    unsigned allflags = 0;
    if ((rc = absorb_steps(h, slot0, done_steps, stats, &allflags))) return rc;
    if (n_steps) *n_steps = done_steps;
    return flags_status(h, allflags);
}

int imc_run_batch(ImcHandle *const *hs, int32_t n, int64_t max_steps, int32_t n_threads, int64_t *steps,
                  double *wall_ms, int32_t *failed) {
    if (!hs || n < 0 || n_threads < 1) return IMC_ERR_INVALID_ARG;
    for (int32_t i = 0; i < n; ++i)
        if (!hs[i]) return IMC_ERR_INVALID_ARG;
    for (int32_t i = 0; i < n; ++i)
        for (int32_t j = 0; j < i; ++j)
            if (hs[i] == hs[j]) return IMC_ERR_INVALID_ARG;  // a handle is not thread-safe
    if (failed) *failed = -1;
    std::atomic<int32_t> next(0);
    std::atomic<int> first_rc(IMC_OK);
    std::atomic<int32_t> first_bad(-1);
    auto worker = [&]() {
        while (true) {
            const int32_t i = next.fetch_add(1);
            if (i >= n) return;
            ImcHandle *h = hs[i];
            int64_t st = 0;
            int rc = cudaSetDevice(h->device) == cudaSuccess ? imc_run(h, max_steps, nullptr, &st, nullptr)
                                                             : fail(h, IMC_ERR_CUDA, "cudaSetDevice");
            if (steps) steps[i] = st;
            if (rc != IMC_OK) {
                int expect = IMC_OK;
                if (first_rc.compare_exchange_strong(expect, rc)) first_bad.store(i);
            }
        }
    };
    const auto t0 = std::chrono::steady_clock::now();
    const int nt = (int)std::min<int32_t>(n_threads, std::max<int32_t>(n, 1));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto &th : pool) th.join();
    const auto t1 = std::chrono::steady_clock::now();
    if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (failed) *failed = first_bad.load();
    return first_rc.load();
}

int imc_run_batch_fused(ImcHandle *const *hs, int32_t n, int64_t max_steps, int64_t *steps, double *wall_ms,
                        int32_t *failed) {
    if (!hs || n < 1 || n > kFusedMaxDecks) return IMC_ERR_INVALID_ARG;
    for (int32_t i = 0; i < n; ++i)
        if (!hs[i]) return IMC_ERR_INVALID_ARG;
    for (int32_t i = 0; i < n; ++i)
        for (int32_t j = 0; j < i; ++j)
            if (hs[i] == hs[j]) return IMC_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> fused_lock(g_fused_mutex);
    if (failed) *failed = -1;
    if (steps)
        for (int32_t i = 0; i < n; ++i) steps[i] = 0;
    if (wall_ms) *wall_ms = 0.0;
    const int prec = hs[0]->prec, dev = hs[0]->device;
    for (int32_t i = 0; i < n; ++i) {
        ImcHandle *h = hs[i];
        if (h->device != dev || h->geometry != 1 || h->prec != prec || h->ca.surr_image ||
            !transport_shape(h->ca, prec).smem_tally) {
            if (failed) *failed = i;
            return fail(h, IMC_ERR_INVALID_ARG,
                        "fused batch: every deck 1D, on one device, of one state precision, without the "
                        "surrogate, with its tallies in shared memory");
        }
    }
    if (cudaSetDevice(dev) != cudaSuccess) return fail(hs[0], IMC_ERR_CUDA, "cudaSetDevice");
    const auto t0 = std::chrono::steady_clock::now();
    // steps of each deck from the host clock mirrors, as imc_run counts them
    std::vector<int64_t> N((size_t)n, 0), done((size_t)n, 0);
    std::vector<unsigned long long> slot0((size_t)n, 0);
    std::vector<long long> ncen((size_t)n, 0);
    int rc = IMC_OK, bad = -1;
    for (int32_t i = 0; i < n && !rc; ++i) {
        ImcHandle *h = hs[i];
        double t = h->t, dt = h->dt;
        bool fin = h->finished;
        while (!fin && N[i] < max_steps) {
            ++N[i];
            host_timestep(h->deck, t, dt, fin);
        }
        Scalars sc;
        if (N[i] > 0 && ((rc = ensure_stats(h, N[i])) || (rc = read_scalars(h, &sc)))) { bad = i; break; }
        if (N[i] > 0) { slot0[i] = sc.step; ncen[i] = sc.n_particles; }
    }
    FusedBatch F;
    if (!rc && cudaStreamCreateWithFlags(&F.st, cudaStreamNonBlocking) != cudaSuccess) {
        rc = fail(hs[0], IMC_ERR_CUDA, "cudaStreamCreateWithFlags");
        bad = 0;
    }
    // launch order: the larger particle budgets first (the order is scheduling
    // only: no deck's result depends on it)
    std::vector<int> order((size_t)n);
    for (int32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return hs[a]->deck.n_max > hs[b]->deck.n_max; });
    const unsigned fatal = IMC_FLAG_CAPACITY | IMC_FLAG_SEGMENT_CAP | IMC_FLAG_NAN | IMC_FLAG_FIXPOINT_RANGE |
                           IMC_FLAG_NO_ENERGY;
    while (!rc) {
        std::vector<int> members;
        for (int i : order)
            if (done[i] < N[i]) members.push_back(i);
        if (members.empty()) break;
        // the largest chunk of steps whose worst-case births fit every deck's buffers
        int64_t m = 64;
        for (int i : members) m = std::min<int64_t>(m, N[i] - done[i]);
        bool grew = false;
        for (int i : members) {
            ImcHandle *h = hs[i];
            int64_t mi = 0;
            long long bound = ncen[i];
            while (mi < m) {
                const long long nb = bound + births_bound(h, bound);
                if (nb > h->capacity) break;
                bound = nb;
                ++mi;
            }
            if (mi == 0) {
                if ((rc = grow(h, ncen[i] + 4 * births_bound(h, ncen[i])))) { bad = i; break; }
                grew = true;
            } else {
                m = std::min(m, mi);
            }
        }
        if (rc) break;
        if (grew) {
            F.drop();
            continue;
        }
        if (!F.exec || members != F.members)
            if ((rc = build_fused(F, hs, members, prec, &bad))) break;
        for (int64_t s = 0; s < m && !rc; ++s) {
            const cudaError_t e = cudaGraphLaunch(F.exec, F.st);
            if (e != cudaSuccess) {
                rc = fail(hs[members[0]], IMC_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
                bad = members[0];
            }
        }
        const cudaError_t e = cudaStreamSynchronize(F.st);
        if (!rc && e != cudaSuccess) {
            rc = fail(hs[members[0]], IMC_ERR_CUDA, std::string("fused batch: ") + cudaGetErrorString(e));
            bad = members[0];
        }
        if (rc) break;
        bool stop = false;
        for (int i : members) {
            done[i] += m;
            Scalars sc;
            if ((rc = read_scalars(hs[i], &sc))) { bad = i; break; }
            ncen[i] = sc.n_particles;
            if (sc.flags & fatal) stop = true;
        }
        if (stop) break;
    }
    // host clock mirrors, totals, and each deck's own status
    for (int32_t i = 0; i < n; ++i) {
        unsigned fl = 0;
        int r = absorb_steps(hs[i], slot0[i], done[i], nullptr, &fl);
        if (steps) steps[i] = done[i];
        if (!r) r = flags_status(hs[i], fl);
        if (r && !rc) { rc = r; bad = i; }
    }
    const auto t1 = std::chrono::steady_clock::now();
    if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (failed) *failed = rc ? bad : -1;
    return rc;
}

int imc_get_totals(const ImcHandle *h, int64_t *segments, int64_t *histories, int64_t *surrogate_calls) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (segments) *segments = h->tot_segments;
    if (histories) *histories = h->tot_histories;
    if (surrogate_calls) *surrogate_calls = h->tot_calls;
    return IMC_OK;
}

int imc_get_time(const ImcHandle *h, double *t, double *dt, int64_t *step_index) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (t) *t = h->t;
    if (dt) *dt = h->dt;
    if (step_index) *step_index = h->step;
    return IMC_OK;
}

int imc_set_time(ImcHandle *h, double t, double dt) {
    if (!h) return IMC_ERR_INVALID_ARG;
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    sc.t = t; sc.dt = dt;
    sc.finished = t > h->deck.t_end ? 1 : 0;
    CK(h, hcopy(h, h->d_sc, &sc, sizeof(Scalars), cudaMemcpyHostToDevice));
    h->t = t; h->dt = dt; h->finished = t > h->deck.t_end;
    return IMC_OK;
}

int imc_num_particles(const ImcHandle *h, int64_t *n) {
    if (!h || !n) return IMC_ERR_INVALID_ARG;
    Scalars sc;
    int rc = read_scalars(const_cast<ImcHandle *>(h), &sc);
    if (rc) return rc;
    *n = sc.n_particles;
    return IMC_OK;
}

static double *field_ptr(const ImcHandle *h, int field, int64_t *count) {
    const CellArgs &ca = h->ca;
    *count = h->nc;
    switch (field) {
        case IMC_FIELD_TEMP: return ca.temp;
        case IMC_FIELD_RADENERGY: return ca.radenergydens;
        case IMC_FIELD_MATENERGY: return ca.matenergydens;
        case IMC_FIELD_FLECK: return ca.fleck;
        case IMC_FIELD_BETA: return ca.beta;
        case IMC_FIELD_SIGMA_A: return ca.sa;
        case IMC_FIELD_SIGMA_S: return ca.ss;
        case IMC_FIELD_BEE: return ca.bee;
        case IMC_FIELD_ENERGYDEP: *count = (int64_t)h->nc * h->K; return ca.energydep;
        case IMC_FIELD_EMITTED: *count = (int64_t)h->nc * h->K; return ca.emitted;
        default: return nullptr;
    }
}

int imc_get_field(const ImcHandle *h, int field, double *out, int64_t count) {
    if (!h || !out) return IMC_ERR_INVALID_ARG;
    ImcHandle *hh = const_cast<ImcHandle *>(h);
    int64_t n;
    double *p = field_ptr(h, field, &n);
    if (!p) return fail(hh, IMC_ERR_INVALID_ARG, "unknown field");
    if (n != count) return fail(hh, IMC_ERR_INVALID_ARG, "field size mismatch");
    CK(hh, cudaStreamSynchronize(h->stream));
    CK(hh, hcopy(hh, out, p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return IMC_OK;
}

int imc_set_field(ImcHandle *h, int field, const double *in, int64_t count) {
    if (!h || !in) return IMC_ERR_INVALID_ARG;
    int64_t n;
    double *p = field_ptr(h, field, &n);
    if (!p) return fail(h, IMC_ERR_INVALID_ARG, "unknown field");
    if (n != count) return fail(h, IMC_ERR_INVALID_ARG, "field size mismatch");
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, hcopy(h, p, in, sizeof(double) * n, cudaMemcpyHostToDevice));
    return IMC_OK;
}

namespace {
// layout of a state blob (imc_save_state): header, host clock and totals,
// the device Scalars, the cell arrays, then the particle list's fields in
// their storage types (buffer Scalars::cur)
struct StateHeader {
    char magic[8];
    int32_t version, prec, geometry, nx, ny, K;
    int64_t n_particles;
    double t, dt;
    int64_t step, finished, tot_segments, tot_histories, tot_calls;
    int64_t scalars_bytes;  // the device scalars' layout must match too
};
constexpr int32_t kStateVersion = 3;  // 3: census maximum kept as an exponent per true energy

struct Piece {
    void *dev;
    size_t bytes;
};

std::vector<Piece> cell_pieces(const ImcHandle *h) {
    const size_t nc = (size_t)h->nc, nk = (size_t)h->nc * h->K;
    const CellArgs &c = h->ca;
    return {{c.temp, 8 * nc}, {c.bee, 8 * nc}, {c.beta, 8 * nc}, {c.fleck, 8 * nc}, {c.sa, 8 * nc}, {c.ss, 8 * nc},
            {c.radenergydens, 8 * nc}, {c.matenergydens, 8 * nc}, {c.energydep, 8 * nk}, {c.emitted, 8 * nk}};
}

std::vector<Piece> particle_pieces(const ImcHandle *h, const PBufRaw &b, long long n) {
    const size_t se = state_elem(h->prec), e0 = e0_elem(h->prec), m = (size_t)n;
    std::vector<Piece> v = {{b.t, se * m}, {b.x, se * m}, {b.ux, se * m}, {b.E, se * m}, {b.E0, e0 * m},
                            {b.cs, 4 * m}, {b.alive, m}};
    if (h->geometry == 2) {
        v.push_back({b.y, se * m});
        v.push_back({b.uy, se * m});
    }
    return v;
}
}  // namespace

int imc_save_state(const ImcHandle *hc, void *buf, size_t *len) {
    if (!hc || !len) return IMC_ERR_INVALID_ARG;
    ImcHandle *h = const_cast<ImcHandle *>(hc);
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    const long long n = sc.n_particles;
    auto cells = cell_pieces(h);
    auto parts = particle_pieces(h, h->buf[sc.cur], n);
    size_t need = sizeof(StateHeader) + sizeof(Scalars);
    for (auto &p : cells) need += p.bytes;
    for (auto &p : parts) need += p.bytes;
    if (!buf) { *len = need; return IMC_OK; }
    if (*len < need) { *len = need; return fail(h, IMC_ERR_INVALID_ARG, "state buffer too small"); }
    unsigned char *o = static_cast<unsigned char *>(buf);
    StateHeader hd{};
    std::memcpy(hd.magic, "IMCSTATE", 8);
    hd.version = kStateVersion; hd.prec = h->prec; hd.geometry = h->geometry; hd.nx = h->nx; hd.ny = h->ny; hd.K = h->K;
    hd.n_particles = n; hd.t = h->t; hd.dt = h->dt; hd.step = h->step; hd.finished = h->finished ? 1 : 0;
    hd.tot_segments = h->tot_segments; hd.tot_histories = h->tot_histories; hd.tot_calls = h->tot_calls;
    hd.scalars_bytes = (int64_t)sizeof(Scalars);
    std::memcpy(o, &hd, sizeof hd); o += sizeof hd;
    std::memcpy(o, &sc, sizeof sc); o += sizeof sc;
    for (auto &p : cells) { CK(h, hcopy(h, o, p.dev, p.bytes, cudaMemcpyDeviceToHost)); o += p.bytes; }
    for (auto &p : parts) { if (p.bytes) CK(h, hcopy(h, o, p.dev, p.bytes, cudaMemcpyDeviceToHost)); o += p.bytes; }
    *len = need;
    return IMC_OK;
}

int imc_load_state(ImcHandle *h, const void *buf, size_t len) {
    if (!h || !buf || len < sizeof(StateHeader) + sizeof(Scalars)) return IMC_ERR_INVALID_ARG;
    const unsigned char *in = static_cast<const unsigned char *>(buf);
    StateHeader hd;
    std::memcpy(&hd, in, sizeof hd); in += sizeof hd;
    if (std::memcmp(hd.magic, "IMCSTATE", 8) != 0 || hd.version != kStateVersion ||
        hd.scalars_bytes != (int64_t)sizeof(Scalars))
        return fail(h, IMC_ERR_INVALID_ARG, "not a state blob of this library version");
    if (hd.prec != h->prec || hd.geometry != h->geometry || hd.nx != h->nx || hd.ny != h->ny || hd.K != h->K)
        return fail(h, IMC_ERR_INVALID_ARG, "state blob of another deck (precision, geometry, mesh or scales)");
    Scalars sc;
    std::memcpy(&sc, in, sizeof sc); in += sizeof sc;
    const long long n = hd.n_particles;
    int rc = grow(h, n);
    if (rc) return rc;
    auto cells = cell_pieces(h);
    auto parts = particle_pieces(h, h->buf[0], n);
    size_t need = sizeof(StateHeader) + sizeof(Scalars);
    for (auto &p : cells) need += p.bytes;
    for (auto &p : parts) need += p.bytes;
    if (len < need) return fail(h, IMC_ERR_INVALID_ARG, "state blob truncated");
    CK(h, cudaStreamSynchronize(h->stream));
    for (auto &p : cells) { CK(h, hcopy(h, p.dev, in, p.bytes, cudaMemcpyHostToDevice)); in += p.bytes; }
    for (auto &p : parts) { if (p.bytes) CK(h, hcopy(h, p.dev, in, p.bytes, cudaMemcpyHostToDevice)); in += p.bytes; }
    sc.cur = 0;
    sc.compact_src = 0;
    CK(h, hcopy(h, h->d_sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
    h->t = hd.t; h->dt = hd.dt; h->step = hd.step; h->finished = hd.finished != 0;
    h->tot_segments = hd.tot_segments; h->tot_histories = hd.tot_histories; h->tot_calls = hd.tot_calls;
    h->stage = Stage::Fresh;
    drop_graphs(h);
    return IMC_OK;
}

int imc_get_particles(const ImcHandle *hc, ImcParticles *p) {
    ImcHandle *h = const_cast<ImcHandle *>(hc);
    if (!h || !p) return IMC_ERR_INVALID_ARG;
    Scalars sc;
    int rc = read_scalars(h, &sc);
    if (rc) return rc;
    const long long n = sc.n_particles;
    if (n > p->n) return fail(h, IMC_ERR_INVALID_ARG, "particle arrays too small");
    const PBufRaw &b = h->buf[sc.cur];
    const size_t se = state_elem(h->prec), e0 = e0_elem(h->prec);
    std::vector<unsigned char> t(se * n), x(se * n), y(se * n), ux(se * n), uy(se * n), E(se * n), E0(e0 * n);
    std::vector<int32_t> cs(n);
    std::vector<uint8_t> alive(n);
    if (n > 0) {
        CK(h, hcopy(h, t.data(), b.t, se * n, cudaMemcpyDeviceToHost));
        CK(h, hcopy(h, x.data(), b.x, se * n, cudaMemcpyDeviceToHost));
        CK(h, hcopy(h, ux.data(), b.ux, se * n, cudaMemcpyDeviceToHost));
        if (h->geometry == 2) {
            CK(h, hcopy(h, y.data(), b.y, se * n, cudaMemcpyDeviceToHost));
            CK(h, hcopy(h, uy.data(), b.uy, se * n, cudaMemcpyDeviceToHost));
        }
        CK(h, hcopy(h, E.data(), b.E, se * n, cudaMemcpyDeviceToHost));
        CK(h, hcopy(h, E0.data(), b.E0, e0 * n, cudaMemcpyDeviceToHost));
        CK(h, hcopy(h, cs.data(), b.cs, 4 * n, cudaMemcpyDeviceToHost));
        CK(h, hcopy(h, alive.data(), b.alive, n, cudaMemcpyDeviceToHost));
    }
    auto rd = [&](const std::vector<unsigned char> &v, long long i) -> double {
        if (h->prec == 0) return ((const double *)v.data())[i];
        if (h->prec == 1) return (double)((const float *)v.data())[i];
        return (double)__half2float(((const __half *)v.data())[i]);
    };
    auto rd0 = [&](long long i) -> double {
        if (h->prec == 0) return ((const double *)E0.data())[i];
        return (double)((const float *)E0.data())[i];
    };
    for (long long i = 0; i < n; ++i) {
        const int cell = cs[i] & 0xFFFFFF, k = cs[i] >> 24;
        const int ix = h->geometry == 1 ? cell : cell % h->nx;
        const int iy = h->geometry == 1 ? 0 : cell / h->nx;
        double vt = rd(t, i), vx = rd(x, i), vy = h->geometry == 2 ? rd(y, i) : 0.0;
        double vE = rd(E, i), vE0 = rd0(i);
        if (h->prec == 2) {
            float dxs = (float)h->deck.dx[ix] * (float)h->deck.distancescale;
            vx = (double)((float)vx * dxs);
            if (h->geometry == 2) vy = (double)((float)vy * ((float)h->deck.dy[iy] * (float)h->deck.distancescale));
            vt = (double)((float)vt * (float)h->dt);
            vE = (double)((float)vE * (float)vE0);
        }
        if (p->t) p->t[i] = vt;
        if (p->x) p->x[i] = vx;
        if (p->y) p->y[i] = vy;
        if (h->geometry == 1) { if (p->mu) p->mu[i] = rd(ux, i); }
        else { if (p->ux) p->ux[i] = rd(ux, i); if (p->uy) p->uy[i] = rd(uy, i); }
        if (p->E) p->E[i] = vE;
        if (p->E0) p->E0[i] = alive[i] ? vE0 : -1.0;
        if (p->cell) p->cell[i] = cell;
        if (p->scale) p->scale[i] = k;
    }
    p->n = n;
    return IMC_OK;
}

int imc_set_particles(ImcHandle *h, const ImcParticles *p) {
    if (!h || !p || p->n < 0 || !p->E || !p->E0 || !p->cell) return IMC_ERR_INVALID_ARG;
    const long long n = p->n;
    int rc;
    if ((rc = grow(h, n + births_bound(h, n)))) return rc;
    CK(h, cudaStreamSynchronize(h->stream));
    const int prec = h->prec;
    const size_t se = state_elem(prec), e0s = e0_elem(prec);
    std::vector<unsigned char> t(se * n), x(se * n), y(se * n), ux(se * n), uy(se * n), E(se * n), E0(e0s * n);
    std::vector<int32_t> cs(n);
    std::vector<uint8_t> alive(n);
    int emax_e = kNoExp;  // census maximum as the ilogb of its true energy
    auto wr = [&](std::vector<unsigned char> &v, long long i, double val) {
        if (prec == 0) ((double *)v.data())[i] = val;
        else if (prec == 1) ((float *)v.data())[i] = (float)val;
        else ((__half *)v.data())[i] = __float2half_rn((float)val);
    };
    for (long long i = 0; i < n; ++i) {
        const int cell = p->cell[i];
        if (cell < 0 || cell >= h->nc) return fail(h, IMC_ERR_INVALID_ARG, "particle cell out of range");
        const int k = p->scale ? p->scale[i] : 0;
        if (k < 0 || k >= h->K) return fail(h, IMC_ERR_INVALID_ARG, "particle scale index out of range");
        const int se = scale_exp(h->deck.energyscales[k]);
        const int ix = h->geometry == 1 ? cell : cell % h->nx;
        const int iy = h->geometry == 1 ? 0 : cell / h->nx;
        const double vt = p->t ? p->t[i] : 0.0, vx = p->x ? p->x[i] : 0.0, vy = p->y ? p->y[i] : 0.0;
        const double vE = p->E[i], vE0 = p->E0[i];
        double dirx = h->geometry == 1 ? (p->mu ? p->mu[i] : 0.0) : (p->ux ? p->ux[i] : 0.0);
        double diry = h->geometry == 2 && p->uy ? p->uy[i] : 0.0;
        alive[i] = vE0 >= 0.0 ? 1 : 0;
        cs[i] = cell | (k << 24);
        if (prec == 2) {
            float dxs = (float)h->deck.dx[ix] * (float)h->deck.distancescale;
            wr(x, i, (double)((float)vx / dxs));
            if (h->geometry == 2) wr(y, i, (double)((float)vy / ((float)h->deck.dy[iy] * (float)h->deck.distancescale)));
            wr(t, i, (double)((float)vt / (float)h->dt));
            ((float *)E0.data())[i] = (float)vE0;
            float ef = (float)vE / (float)vE0;
            wr(E, i, (double)ef);
            if (alive[i]) emax_e = std::max(emax_e, exp_bound(__half2float(__float2half_rn(ef)) * (float)vE0) - se);
        } else {
            wr(t, i, vt); wr(x, i, vx); wr(y, i, vy); wr(E, i, vE);
            if (prec == 0) ((double *)E0.data())[i] = vE0;
            else ((float *)E0.data())[i] = (float)vE0;
            if (alive[i]) emax_e = std::max(emax_e, (prec == 0 ? exp_bound(vE) : exp_bound((float)vE)) - se);
        }
        wr(ux, i, dirx);
        wr(uy, i, diry);
    }
    Scalars sc;
    if ((rc = read_scalars(h, &sc))) return rc;
    const PBufRaw &b = h->buf[sc.cur];
    if (n > 0) {
        CK(h, hcopy(h, b.t, t.data(), se * n, cudaMemcpyHostToDevice));
        CK(h, hcopy(h, b.x, x.data(), se * n, cudaMemcpyHostToDevice));
        CK(h, hcopy(h, b.ux, ux.data(), se * n, cudaMemcpyHostToDevice));
        if (h->geometry == 2) {
            CK(h, hcopy(h, b.y, y.data(), se * n, cudaMemcpyHostToDevice));
            CK(h, hcopy(h, b.uy, uy.data(), se * n, cudaMemcpyHostToDevice));
        }
        CK(h, hcopy(h, b.E, E.data(), se * n, cudaMemcpyHostToDevice));
        CK(h, hcopy(h, b.E0, E0.data(), e0s * n, cudaMemcpyHostToDevice));
        CK(h, hcopy(h, b.cs, cs.data(), 4 * n, cudaMemcpyHostToDevice));
        CK(h, hcopy(h, b.alive, alive.data(), n, cudaMemcpyHostToDevice));
    }
    long long live = 0;
    for (long long i = 0; i < n; ++i) live += alive[i];
    sc.n_census = live;
    sc.n_particles = n;
    sc.emax_census_exp = emax_e;
    CK(h, hcopy(h, h->d_sc, &sc, sizeof(Scalars), cudaMemcpyHostToDevice));
    h->stage = Stage::Fresh;
    return IMC_OK;
}

int imc_get_stats(const ImcHandle *h, ImcStepStats *stats) {
    if (!h || !stats) return IMC_ERR_INVALID_ARG;
    *stats = h->last;
    return IMC_OK;
}

int imc_set_timing(ImcHandle *h, int enable) {
    if (!h) return IMC_ERR_INVALID_ARG;
    h->timing = enable != 0;
    return IMC_OK;
}

int imc_transport_timing(ImcHandle *h, double *avg_ms, int64_t *launches) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (avg_ms) *avg_ms = h->transport_launches ? h->transport_ms / (double)h->transport_launches : 0.0;
    if (launches) *launches = h->transport_launches;
    h->transport_ms = 0.0;
    h->transport_launches = 0;
    return IMC_OK;
}

int imc_set_surrogate(ImcHandle *h, const float *params, int64_t n_params) {
    if (!h) return IMC_ERR_INVALID_ARG;
    if (!params) {
        h->ca.surr_image = nullptr;
        drop_graphs(h);
        return IMC_OK;
    }
    if (n_params != surr::kParams) return fail(h, IMC_ERR_INVALID_ARG, "surrogate: expected IMC_SURROGATE_PARAMS floats");
    if (h->geometry != IMC_GEOM_1D) return fail(h, IMC_ERR_INVALID_ARG, "surrogate: 1D geometry only");
    if (h->prec == IMC_FP64) return fail(h, IMC_ERR_INVALID_ARG, "surrogate: FP32 or FP16 particle state only");
    for (int64_t i = 0; i < n_params; ++i)
        if (!std::isfinite(params[i])) return fail(h, IMC_ERR_INVALID_ARG, "surrogate: non-finite parameter");
    CK(h, cudaStreamSynchronize(h->stream));
    if (!h->d_surr_image) CK(h, cudaMalloc(&h->d_surr_image, surr::kImageBytes));
    float *dP = nullptr;
    CK(h, cudaMalloc(&dP, sizeof(float) * surr::kParams));
    cudaError_t e = cudaMemcpyAsync(dP, params, sizeof(float) * surr::kParams, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        launch_surr_image(dP, h->d_surr_image, h->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dP);
    if (e != cudaSuccess) return fail(h, IMC_ERR_CUDA, std::string("surrogate image: ") + cudaGetErrorString(e));
    CellArgs ca = h->ca;
    ca.surr_image = reinterpret_cast<const uint4 *>(h->d_surr_image);
    SurrShapes sh = surr_shapes(ca, h->prec);
    if (sh.analog_smem > 227 * 1024 || sh.query_smem > 227 * 1024)
        return fail(h, IMC_ERR_INVALID_ARG, "surrogate: mesh too large for shared memory");
    int grids[4] = {0, 0, 0, 0};
    for (int which = 0; which < 4; ++which) {
        const void *kp = surr_kernel_ptr(ca, h->prec, which);
        const int block = which == 3 ? sh.query_block : sh.analog_block;
        const int smem = which == 3 ? sh.query_smem : sh.analog_smem;
        CK(h, raise_smem_limit(kp, smem));
        int per_sm = 0;
        CK(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kp, block, smem));
        if (per_sm < 1) return fail(h, IMC_ERR_CUDA, "surrogate transport kernel cannot be resident");
        grids[which] = h->sm_count * per_sm;
    }
    sh.analog_grid = std::min(grids[0], std::min(grids[1], grids[2]));
    sh.query_grid = grids[3];
    int rc = surr_queue_alloc(h);
    if (rc) return rc;
    h->sshape = sh;
    h->ca = ca;
    drop_graphs(h);
    return IMC_OK;
}

int imc_get_surrogate_active(const ImcHandle *h, int *active) {
    if (!h || !active) return IMC_ERR_INVALID_ARG;
    *active = h->ca.surr_image != nullptr;
    return IMC_OK;
}

int imc_kernels_per_step(const ImcHandle *h, int *count) {
    if (!h || !count) return IMC_ERR_INVALID_ARG;
    // update, source x5, transport, compact x4, finalize + tally +
    // energycheck + timestep; the surrogate transport is 1 + 2 kSurrRounds
    // kernels
    *count = 12 + (h->ca.surr_image ? 2 * kSurrRounds : 0);
    return IMC_OK;
}

}  // extern "C"
