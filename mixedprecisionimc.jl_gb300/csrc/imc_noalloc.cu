// imc_noalloc.cu -- imc_clean_noalloc: the stable compaction of Clean.clean
// for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc: code that enqueues
// work inside a CUDA stream capture (allocation is not a capturable
// operation), hosts whose device memory is owned by their own pool allocator
// (a Julia CUDA.jl or PyTorch caching pool that must see every byte), and
// loops that cannot afford the device-wide synchronisation cudaMalloc
// implies.  They own the particle arrays and pass them in; the only other
// memory the compaction needs -- per-tile survivor counts, their prefix sums
// and a small scalar block -- lives in the file-scope __device__ array below.
//
// That array is a fixed 72 KiB region that every GPU loading the library
// holds until the process exits.  It bounds the list to kNoAllocMaxTiles
// tiles of 4096 particles (16,777,216 particles); longer lists are rejected
// with IMC_ERR_INVALID_ARG.  All calls share it: calls that overlap on the
// GPU (on different streams, or from different threads, without ordering)
// race on it and give wrong results.
//
// Its device address is looked up once per device (cudaGetSymbolAddress with
// that device current) by the first call made on that device; make that first
// call before any stream capture begins.
#include <cuda_runtime.h>

#include <mutex>

#include "imc.h"  // include/imc.h (on the -I path)
#include "imc_internal.h"

using namespace imc;

namespace {

constexpr long long kNoAllocMaxTiles = 4096;
// layout: Scalars | tile counts [max + 1] | tile offsets [max + 1]
constexpr size_t kNoAllocScalarsBytes = (sizeof(Scalars) + 255) / 256 * 256;
constexpr size_t kNoAllocBytes = kNoAllocScalarsBytes + 2 * (kNoAllocMaxTiles + 1) * sizeof(long long);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {nullptr};

// sets the list length the compaction kernels read
__global__ void k_noalloc_set_n(Scalars *sc, long long n) {
    sc->n_particles = n;
    sc->n_census = n;
}

}  // namespace

extern "C" int imc_clean_noalloc(int precision, int geometry, const ImcDeviceParticles *src,
                                 ImcDeviceParticles *dst, int64_t n, int64_t *n_out, void *stream) {
    if (!src || !dst || !n_out || n < 0) return IMC_ERR_INVALID_ARG;
    if (precision < IMC_FP64 || precision > IMC_FP16 || (geometry != IMC_GEOM_1D && geometry != IMC_GEOM_2D))
        return IMC_ERR_INVALID_ARG;
    const long long ntiles = (n + kCompactTile - 1) / kCompactTile;
    if (ntiles > kNoAllocMaxTiles)
        return IMC_ERR_INVALID_ARG;
    if (!src->alive || !src->cs || !src->E || !src->E0 || !dst->alive || !dst->cs || !dst->E || !dst->E0)
        return IMC_ERR_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return IMC_ERR_NO_DEVICE;
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return IMC_ERR_CUDA;
            g_addr[dev] = (unsigned char *)p;
        }
        base = g_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    *n_out = 0;
    if (n == 0) return IMC_OK;
    Scalars *sc = (Scalars *)base;
    long long *tile_cnt = (long long *)(base + kNoAllocScalarsBytes);
    long long *tile_off = tile_cnt + (kNoAllocMaxTiles + 1);
    // the scratch keeps the previous call's contents: clear the scalars
    if (cudaMemsetAsync(sc, 0, sizeof(Scalars), st) != cudaSuccess)
        return IMC_ERR_CUDA;
    k_noalloc_set_n<<<1, 1, 0, st>>>(sc, n);
    PBufRaw s{src->t, src->x, src->y, src->ux, src->uy, src->E, src->E0, src->cs, src->alive};
    PBufRaw d{dst->t, dst->x, dst->y, dst->ux, dst->uy, dst->E, dst->E0, dst->cs, dst->alive};
    CellArgs ca{};
    ca.geometry = geometry;
    launch_compact(ca, sc, precision, s, d, tile_cnt, tile_off, ntiles, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return IMC_ERR_CUDA;
    long long kept = 0;
    e = cudaMemcpyAsync(&kept, &sc->n_census, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return IMC_ERR_CUDA;
    *n_out = kept;
    return IMC_OK;
}
