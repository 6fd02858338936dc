// imc_noalloc.cu -- imc_clean_noalloc: the stable compaction of Clean.clean
// for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc: hosts whose device
// memory is owned by their own pool allocator (a Julia CUDA.jl or PyTorch
// caching pool that must account for every byte on the device), and loops
// that cannot afford the device-wide synchronisation that cudaMalloc and
// cudaFree imply.  They own the particle arrays and pass them in; the only
// other memory the compaction needs -- per-tile survivor counts, their prefix
// sums and a small scalar block -- lives in the file-scope __device__ array
// below.
//
// That array is a fixed 72 KiB region that every GPU loading the library
// holds until the process exits.  It bounds the list to kNoAllocMaxTiles
// tiles of 4096 particles (16,777,216 particles); longer lists are rejected
// with IMC_ERR_INVALID_ARG.  All calls share it: calls that overlap on the
// GPU (on different streams, or from different threads, without ordering)
// race on it and give wrong results.
//
// Its device address is looked up once per device (cudaGetSymbolAddress with
// that device current) by the first call made on that device.
#include <cuda_runtime.h>

#include <cstdint>
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

// one caller array: its base pointer, element size and required alignment
struct Field {
    const void *p;
    size_t elem, align;
};

// The arrays the compaction reads (src) or writes (dst) for this precision
// and geometry; false if one of them is missing or misaligned.  The alive
// bytes are read 16 at a time from tile starts (multiples of 4096 bytes past
// the base), so they need a 16-byte aligned base.
bool fields_of(const ImcDeviceParticles *a, int precision, int geometry, Field out[9], int *count) {
    const size_t ss = precision == IMC_FP64 ? 8 : precision == IMC_FP32 ? 4 : 2;
    const size_t e0 = precision == IMC_FP64 ? 8 : 4;
    int n = 0;
    out[n++] = {a->t, ss, ss};
    out[n++] = {a->x, ss, ss};
    out[n++] = {a->ux, ss, ss};
    out[n++] = {a->E, ss, ss};
    out[n++] = {a->E0, e0, e0};
    out[n++] = {a->cs, 4, 4};
    out[n++] = {a->alive, 1, 16};
    if (geometry == IMC_GEOM_2D) {
        out[n++] = {a->y, ss, ss};
        out[n++] = {a->uy, ss, ss};
    }
    *count = n;
    for (int i = 0; i < n; ++i)
        if (!out[i].p || ((uintptr_t)out[i].p % out[i].align) != 0) return false;
    return true;
}

// whether the n-element ranges of two arrays share a byte
bool overlap(const Field &a, const Field &b, long long n) {
    const uintptr_t a0 = (uintptr_t)a.p, a1 = a0 + (uintptr_t)n * a.elem;
    const uintptr_t b0 = (uintptr_t)b.p, b1 = b0 + (uintptr_t)n * b.elem;
    return a0 < b1 && b0 < a1;
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
    // an empty list reads and writes no array (which may then be NULL)
    if (n == 0) {
        *n_out = 0;
        return IMC_OK;
    }
    Field fs[9], fd[9];
    int ns = 0, nd = 0;
    if (!fields_of(src, precision, geometry, fs, &ns) || !fields_of(dst, precision, geometry, fd, &nd))
        return IMC_ERR_INVALID_ARG;
    // the scatter reads survivors while other blocks write earlier output
    // positions: an output array that shares memory with any input array
    // would be read after it was overwritten
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j < nd; ++j)
            if (overlap(fs[i], fd[j], n)) return IMC_ERR_INVALID_ARG;
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
