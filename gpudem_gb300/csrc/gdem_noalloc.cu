// gdem_sort_keys_noalloc: the stable radix sort of gdem_sort_keys on device
// pointers and the caller's stream, with no device allocation.
//
// Who needs it.  Some callers must not allocate while they run:
//  * a host loop stepping a scene sized to fill HBM, where a cudaMalloc of the
//    sort's scratch can fail after the state has been laid out;
//  * a caller that must not stall the device: cudaFree synchronises the whole
//    device, and cudaMalloc may too, so an allocating sort inside a frame
//    serialises every stream of the process;
//  * a caller that owns its memory budget (a framework's caching allocator or
//    a fixed pool) and counts every byte the process takes.
// gdem_sort_keys allocates and frees its scratch on every call; this entry
// point uses a fixed scratch array instead.
//
// Scratch.  One file-scope __device__ array holds the second ping-pong side
// (keys and payload) and the per-tile digit histogram for up to
// GDEM_SORT_NOALLOC_MAX_KEYS keys: 8 bytes per key plus 1 KiB per 2048-key
// tile, 8.5 MiB in all.  The array is part of this module's static device
// memory, so it exists as soon as the module is loaded on a device.  The first
// call on each device looks its address up with cudaGetSymbolAddress (which
// loads the module there if it is not loaded yet) and keeps it for later
// calls, together with the id of the context it belongs to.  Make that first
// call on each device before any stream capture begins.  A context torn down
// and made again (cudaDeviceReset, then any CUDA call) loads the module anew,
// possibly at another address: the next call sees the new context id and
// looks the address up again, so that call too belongs before any capture.
//
// Nothing in the scratch must start at zero: every pass overwrites the whole
// histogram it reads (one count per digit and tile) and every position of the
// ping-pong side below n.  The caller's output buffers are the first side:
// the keys and an identity payload are copied there, and after the four
// passes the sorted keys and the permutation are back in them.
//
// One scratch array per device means calls on the same device must not
// overlap on the GPU: two calls in flight at once (on different streams, or
// from different host threads without ordering) race on the scratch and give
// wrong results.  Order them on one stream or with events.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "gdem.h"
#include "gdem_internal.cuh"

namespace {

constexpr int kMaxKeys = GDEM_SORT_NOALLOC_MAX_KEYS;
constexpr int kTile = 2048;  // keys per radix-sort tile, as gdem::rs_blocks_for counts them
constexpr int kMaxTiles = (kMaxKeys + kTile - 1) / kTile;
constexpr size_t kKeysOff = 0;
constexpr size_t kValsOff = kKeysOff + sizeof(uint32_t) * (size_t)kMaxKeys;
constexpr size_t kHistOff = kValsOff + sizeof(int) * (size_t)kMaxKeys;
constexpr size_t kTotOff = kHistOff + sizeof(uint32_t) * 256 * (size_t)kMaxTiles;
constexpr size_t kScratchBytes = kTotOff + sizeof(uint32_t) * 256;
static_assert(kKeysOff % 256 == 0 && kValsOff % 256 == 0 && kHistOff % 256 == 0 && kTotOff % 256 == 0,
              "scratch sections must stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// Id of the current context (unique for the life of the process, unlike its
// handle), through the driver entry points the runtime hands out, so the
// library needs no link against the driver library.
cudaError_t current_context_id(unsigned long long* id) {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess)
            return cudaErrorNotSupported;
        get_current = reinterpret_cast<GetCurrent>(a);
        get_id = reinterpret_cast<GetId>(b);
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorContextIsDestroyed;
    return cudaSuccess;
}

// Address of this device's scratch in the current context: looked up on the
// first call per device and again whenever the context has changed (or no
// context is current on this thread yet: the lookup makes the device's
// primary context current).
cudaError_t scratch_for(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    unsigned long long ctx = 0;
    const bool known = current_context_id(&ctx) == cudaSuccess;
    if (!known || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return e;
        const cudaError_t ce = current_context_id(&ctx);
        if (ce != cudaSuccess) return ce;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// First ping-pong side: the caller's keys and the payload 0..n-1.
__global__ void k_seed_pairs(const uint32_t* keys, int n, uint32_t* keys_out, int* vals_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys_out[i] = keys[i];
    vals_out[i] = i;
}

}  // namespace

extern "C" int gdem_sort_keys_noalloc(const uint32_t* d_keys, int n, uint32_t* d_keys_sorted, int* d_perm,
                                      void* stream) {
    if (n < 0 || (n > 0 && (!d_keys || !d_keys_sorted || !d_perm))) return GDEM_ERR_ARG;
    if (n > kMaxKeys) return GDEM_ERR_CAPACITY;
    if (n == 0) return GDEM_OK;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return GDEM_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return GDEM_ERR_ARG;
    unsigned char* base = nullptr;
    if (scratch_for(dev, &base) != cudaSuccess) return GDEM_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* k1 = reinterpret_cast<uint32_t*>(base + kKeysOff);
    int* v1 = reinterpret_cast<int*>(base + kValsOff);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + kHistOff);
    uint32_t* tot = reinterpret_cast<uint32_t*>(base + kTotOff);
    const int nb = gdem::rs_blocks_for(n);
    if (nb > kMaxTiles) return GDEM_ERR_CAPACITY;
    k_seed_pairs<<<(n + 255) / 256, 256, 0, st>>>(d_keys, n, d_keys_sorted, d_perm);
    gdem::radix_sort_pairs(d_keys_sorted, d_perm, k1, v1, hist, tot, n, nb, 0, 4, st);
    return cudaGetLastError() == cudaSuccess ? GDEM_OK : GDEM_ERR_CUDA;
}
