// pg_noalloc.cu — pg_rss_matmul_u64_noalloc: the limb tensor-core RSS
// share-GEMM with its scratch in one fixed device array, for callers that
// must not allocate device memory once they are running.
//
// The regular entry point grows the context's scratch with cudaMalloc and
// releases the old block with cudaFree, which waits for the whole device.
// A host that owns all device memory through its own pool, a serving loop
// that must not stall its other streams on that wait, or one that must not
// meet an out-of-memory error halfway through a request cannot allow either.
// This entry point takes its scratch from `noalloc_scratch` below instead,
// which the CUDA runtime reserves on a device when it loads this file's
// module there. With the default lazy module loading (CUDA_MODULE_LOADING
// unset or LAZY) that happens at the first call of this entry point on the
// device, so a process that never calls it never holds the array. With
// CUDA_MODULE_LOADING=EAGER every module of the library is loaded when the
// process creates its CUDA context on a device, and the array is then held
// on every device the process uses, whether it calls this entry point or not.
//
// Set-up: the first call on a device, with the context's device current,
// looks up the array's device address with cudaGetSymbolAddress (which also
// loads the module) and raises the GEMM kernel's shared-memory limit. Every
// call looks the address up again (a lookup in the loaded module, no
// allocation) and repeats the set-up if it changed, as it does after a
// cudaDeviceReset. Make the first call before any stream capture on the
// device.
//
// Sharing: every call on a device, from every context and thread, uses the
// same array. Calls whose execution can overlap on the device (different
// streams with no ordering between them) corrupt each other's results;
// order them on one stream or with events.
#include <mutex>

#include "pg_common.cuh"

namespace pg {
int limb_prepare_current_device(Ctx *c, bool again);
int limb_rss_matmul_u64_fixed(Ctx *c, uint8_t *scr, size_t cap, const uint64_t *const a[6],
                              const uint64_t *const b[6], uint64_t *const out[6], int M, int N, int K, int tA, int tB,
                              int tC, int trunc);
}  // namespace pg

using namespace pg;

namespace {

static __device__ __align__(256) uint8_t noalloc_scratch[PG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex setup_mutex;
uint8_t *scratch_addr[kMaxDevices];  // per device: the address the last set-up saw

int setup_device(Ctx *c, uint8_t **out) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, PG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    }
    if (cur != c->device)
        return set_error(c, PG_ERR_INVALID_ARG, "the context's device %d must be current (device %d is)", c->device,
                         cur);
    if (cur < 0 || cur >= kMaxDevices)
        return set_error(c, PG_ERR_UNSUPPORTED, "device ordinal %d is above %d", cur, kMaxDevices - 1);
    std::lock_guard<std::mutex> lock(setup_mutex);
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return set_error(c, PG_ERR_CUDA, "cudaGetSymbolAddress of the fixed scratch: %s", cudaGetErrorString(e));
    }
    if (scratch_addr[cur] != (uint8_t *)p) {
        // first call on this device, or the module was loaded anew (a device reset)
        int st = limb_prepare_current_device(c, scratch_addr[cur] != nullptr);
        if (st) return st;
        scratch_addr[cur] = (uint8_t *)p;
    }
    *out = scratch_addr[cur];
    return PG_OK;
}

}  // namespace

extern "C" int pg_rss_matmul_u64_noalloc(pg_ctx *c, const uint64_t *const a[6], const uint64_t *const b[6],
                                         uint64_t *const out[6], int M, int N, int K, int tA, int tB, int tC,
                                         int trunc) {
    if (!c) return PG_ERR_INVALID_ARG;
    uint8_t *scr = nullptr;
    int st = setup_device(c, &scr);
    if (st) return st;
    return limb_rss_matmul_u64_fixed(c, scr, PG_NOALLOC_SCRATCH_BYTES, a, b, out, M, N, K, tA, tB, tC, trunc);
}
