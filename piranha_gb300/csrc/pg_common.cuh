// pg_common.cuh — shared definitions of the piranha_gb300 CUDA library:
// the context, status handling, share-pointer bundles and the ring helpers
// that every kernel uses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "piranha_gb300.h"

namespace pg {

// ------------------------------------------------------------------ context

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int form = PG_FORM_LIMB_TC;
    std::string err;
    uint64_t comm[9] = {0};
    std::atomic<uint64_t> launches{0};
    // scratch owned by the context (grown on demand, freed at destroy)
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // split-K partial sums of the CUDA-core ring GEMM (separate from scratch,
    // which callers of that GEMM may be using for its operands)
    void *partial = nullptr;
    size_t partial_bytes = 0;
    int sm_count = 0;
    int *dev_err = nullptr;  // device word that bounded waits set on timeout
    // buffers that scratch / partial outgrew: a captured graph may still
    // point into them, so they are freed only with the context
    std::vector<void *> retired;
    // counters at pg_graph_begin (capture does no work: they are put back at the end)
    uint64_t capture_comm[9] = {0};
    uint64_t capture_launches = 0;
    bool capturing = false;
    // split-K autotuner of the limb GEMM: on/off, and the timed choice
    // (split, chunks per split) per problem shape
    int autotune = 1;
    std::unordered_map<std::string, std::pair<int, int>> split_cache;
    // set by the network executor around a standalone share-GEMM / convolution
    // call whose A (rep_a) or B (rep_b) share buffers hold a replicated sharing,
    // so that the limb form's digit image of that operand stores each share once
    bool rep_a = false, rep_b = false;
    // the limb GEMM's schedule (MMA order, issue lag) of a tuner's timing run; -1: none
    int lsched_order = -1, lsched_lag = -1;
    // set by the network executor around a maxpool / ReLU layer whose input's
    // shares 1-4 (party A's shareB, party B's two, party C's shareA) are known
    // to be 0 (a bias-free FC / CNN output, [v, 0, 0, 0, 0, v]): those are not read
    bool in_zero_mid = false;
    // AES counter-mode masks of the resharing steps (off: the reference's
    // unfilled masks); round keys of the three pairwise keys and the next block
    bool prg_on = false;
    uint32_t prg_rk[3][60];
    uint64_t prg_ctr = 0;
    // bound on every device-side wait of the limb kernels, and the diagnostic
    // stage whose copies the limb GEMM's producer withholds (-1: none)
    uint64_t wait_ns = 2000000000ull;
    int withhold_stage = -1;
};

int set_error(Ctx *c, int code, const char *fmt, ...);

#define PG_CHECK_CUDA(ctx, expr)                                                               \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return ::pg::set_error((ctx), PG_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
    } while (0)

// Status after a launch: configuration errors surface here.
int launch_status(Ctx *c, const char *what);

void *scratch(Ctx *c, size_t bytes);  // nullptr on failure (error set)
void *gemm_partial(Ctx *c, size_t bytes);  // the split-K buffer; nullptr on failure (error set)

// ---------------------------------------------------------- communication

// The accounting of one protocol message step in which every one of the 3
// parties sends tx bytes and receives rx bytes (DeviceData.h:93,111).
inline void comm_msg(Ctx *c, uint64_t tx, uint64_t rx) {
    for (int p = 0; p < 3; p++) {
        c->comm[p] += tx;
        c->comm[4 + p] += rx;
    }
}
inline void comm_round(Ctx *c, uint64_t n = 1) { c->comm[8] += n; }

// ------------------------------------------------------------ share bundles

template <typename T> struct Sh6 {
    T *p[6];
};
template <typename T> struct CSh6 {
    const T *p[6];
};
template <typename T> struct Pub3 {
    T *p[3];
};

template <typename T> inline bool load6(CSh6<T> &o, const T *const *a) {
    if (!a) return false;
    for (int i = 0; i < 6; i++) {
        if (!a[i]) return false;
        o.p[i] = a[i];
    }
    return true;
}
template <typename T> inline bool load6(Sh6<T> &o, T *const *a) {
    if (!a) return false;
    for (int i = 0; i < 6; i++) {
        if (!a[i]) return false;
        o.p[i] = a[i];
    }
    return true;
}

// Operand segments of one fused ring GEMM: sum over i of A_i (B0_i + B1_i),
// B1_i optional; every segment has the same shape and layout.
template <typename T> struct SegList {
    int nseg = 0;
    const T *a[12];
    const T *b0[12];
    const T *b1[12];
};

// party helpers (RSS.inl:348-369)
__host__ __device__ constexpr int next_party(int p) { return p == 2 ? 0 : p + 1; }
__host__ __device__ constexpr int prev_party(int p) { return p == 0 ? 2 : p - 1; }

// ------------------------------------------------------------ ring division

template <typename T> struct Signed;
template <> struct Signed<uint64_t> { typedef int64_t type; };
template <> struct Signed<uint32_t> { typedef int32_t type; };

// (T)(S)((double)(S)x / (double)(S)d) of functors.cuh:33-45,94-105, for
// d = 2^t with 0 <= t <= 62 (t <= 30 for 32-bit rings), restated in integer
// arithmetic: round |x| to 53 significant bits (ties to even), divide by 2^t
// truncating toward zero, saturate like cvt.rzi.
__device__ __forceinline__ uint64_t div_pow2(uint64_t x, int t) {
    int64_t sx = (int64_t)x;
    uint64_t ax = sx < 0 ? (uint64_t)0 - x : x;
    int bits = 64 - __clzll(ax);
    if (bits > 53) {
        int sh = bits - 53;
        uint64_t base = ax >> sh;
        uint64_t rem = ax & ((1ull << sh) - 1);
        uint64_t half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (base & 1))) base++;
        ax = base << sh;
    }
    uint64_t qa = ax >> t;
    if (sx >= 0) return qa >= (1ull << 63) ? (uint64_t)INT64_MAX : qa;
    return (uint64_t)0 - qa;
}
__device__ __forceinline__ uint32_t div_pow2(uint32_t x, int t) {
    int32_t sx = (int32_t)x;
    uint32_t ax = sx < 0 ? 0u - x : x;  // exact in double
    uint32_t qa = ax >> t;
    if (sx >= 0) return qa >= 0x80000000u ? (uint32_t)INT32_MAX : qa;
    return 0u - qa;
}
// General denominator: the reference's device double arithmetic.
__device__ __forceinline__ uint64_t div_general(uint64_t x, uint64_t d) {
    double q = __ddiv_rn(__ll2double_rn((long long)x), __ll2double_rn((long long)d));
    return (uint64_t)__double2ll_rz(q);
}
__device__ __forceinline__ uint32_t div_general(uint32_t x, uint32_t d) {
    double q = __ddiv_rn((double)(int32_t)x, (double)(int32_t)d);
    return (uint32_t)__double2int_rz(q);
}
// t >= 0: power-of-two denominator 2^t; t < 0: general denominator d
template <typename T> __device__ __forceinline__ T div_public(T x, T d, int t) {
    return t >= 0 ? div_pow2(x, t) : div_general(x, d);
}
// device-side: log2 of d when d is a power of two in the integer-path range, else -1
template <typename T> __device__ __forceinline__ int pow2_shift_dev(T d) {
    if (d == 0 || (d & (d - 1))) return -1;
    const int t = (int)(sizeof(T) * 8) - 1 - (sizeof(T) == 8 ? __clzll((long long)d) : __clz((int)d));
    return t <= (int)(sizeof(T) * 8 - 2) ? t : -1;
}
// host-side: log2 of d when d is a power of two in the integer-path range
template <typename T> inline int pow2_shift(T d) {
    if (d == 0 || (d & (d - 1))) return -1;
    int t = 0;
    while (((T)1 << t) != d) t++;
    return t <= (int)(sizeof(T) * 8 - 2) ? t : -1;
}

inline unsigned grid_for(size_t n, int threads, int max_blocks = 1 << 20) {
    size_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > (size_t)max_blocks) b = max_blocks;
    return (unsigned)b;
}

}  // namespace pg

struct pg_ctx : public pg::Ctx {};
