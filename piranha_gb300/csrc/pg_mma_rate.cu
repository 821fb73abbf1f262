// pg_mma_rate.cu — sustained throughput of the tensor-core instruction forms
// an exact limb decomposition of the ring GEMM could ride on, measured on the
// device it runs on. This is how the limb form's operand type was chosen:
//
//   PG_RATE_TC_F16  tcgen05.mma kind::f16, M=128 N=256 K=16, fp16 x fp16 ->
//                   fp32 in tensor memory (the form the limb GEMM uses);
//   PG_RATE_TC_F8   tcgen05.mma kind::f8f6f4 (e4m3), M=128 N=256 K=32 -> fp32
//                   (integers up to 16 are exact: 4-bit limbs, 136 pairs);
//   PG_RATE_MMA_S8  mma.sync m16n8k32 s8 x s8 -> s32, the only INT8 tensor
//                   instruction sm_103a accepts (ptxas rejects tcgen05.mma
//                   kind::i8 for sm_103a: "Feature '.kind::i8' not supported
//                   on .target 'sm_103a'");
//   PG_RATE_MMA_F16 mma.sync m16n8k16 f16 x f16 -> f32, the legacy path.
//
// The tcgen05 forms run one CTA per SM whose one elected thread issues `iters`
// MMAs back to back from fixed shared-memory operands into two alternating
// 256-column accumulators; the mma.sync forms run 16 warps per SM, each with
// eight independent accumulator chains. Every wait is bounded.
#include <cuda_fp16.h>

#include "pg_common.cuh"
#include "pg_tcgen05.cuh"

namespace pg {
namespace rate {

constexpr uint64_t WAIT_NS = 2000000000ull;
constexpr int TC_M = 128, TC_N = 256;
constexpr int A_BYTES = TC_M * 32, B_BYTES = TC_N * 32;  // 32 bytes of K per row

// byte offset of (row r, K byte kb) in the no-swizzle K-major layout of 8 x 16-byte
// core matrices, LBO = 128 (K-adjacent core matrices), SBO = 256 (8-row groups)
__device__ __forceinline__ int core_off(int r, int kb) { return (r >> 3) * 256 + (kb >> 4) * 128 + (r & 7) * 16 + (kb & 15); }

template <int F8>
__global__ void __launch_bounds__(128, 1) tc_rate_kernel(int iters, unsigned long long *cycles, int *err) {
    __shared__ __align__(1024) uint8_t sa[A_BYTES];
    __shared__ __align__(1024) uint8_t sb[B_BYTES];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    __shared__ int never;
    const int t = threadIdx.x, warp = t >> 5;
    // operands: small integers (fp16) or e4m3 bytes without the NaN codes
    for (int i = t; i < A_BYTES / 2; i += blockDim.x) {
        const int r = i / 16, k = i % 16;
        if (F8) {
            sa[core_off(r, 2 * k)] = (uint8_t)((r * 37 + 2 * k) & 0x77);
            sa[core_off(r, 2 * k + 1)] = (uint8_t)((r * 37 + 2 * k + 1) & 0x77);
        } else {
            *reinterpret_cast<__half *>(sa + core_off(r, 2 * k)) = __int2half_rn(((r * 7 + k * 13) & 255) - 128);
        }
    }
    for (int i = t; i < B_BYTES / 2; i += blockDim.x) {
        const int r = i / 16, k = i % 16;
        if (F8) {
            sb[core_off(r, 2 * k)] = (uint8_t)((r * 11 + 2 * k) & 0x77);
            sb[core_off(r, 2 * k + 1)] = (uint8_t)((r * 11 + 2 * k + 1) & 0x77);
        } else {
            *reinterpret_cast<__half *>(sb + core_off(r, 2 * k)) = __int2half_rn(((r * 5 + k * 3) & 255) - 128);
        }
    }
    if (t == 0) {
        tc::mbar_init(tc::smem_u32(&bar), 1);
        never = 0;
        tc::fence_mbar_init();
    }
    tc::fence_proxy_async_smem();
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_u32(&tbase), 512);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tm = tbase;
    if (t == 0) {
        const uint64_t ad = tc::smem_desc(tc::smem_u32(sa), 128, 256);
        const uint64_t bd = tc::smem_desc(tc::smem_u32(sb), 128, 256);
        const uint32_t id = tc::idesc_f16_f32(TC_M, TC_N);  // f32 D; A/B code 0 = f16 or e4m3
        const unsigned long long c0 = clock64();
        for (int i = 0; i < iters; i++) {
            const uint32_t d = tm + (uint32_t)((i & 1) * TC_N);
            const uint32_t acc = i >= 2 ? 1u : 0u;
            if (F8)
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(d),
                    "l"(ad), "l"(bd), "r"(id), "r"(acc)
                    : "memory");
            else
                tc::mma_f16(d, ad, bd, id, acc);
        }
        tc::mma_commit(tc::smem_u32(&bar));
        const bool ok = tc::mbar_wait(tc::smem_u32(&bar), 0, &never, WAIT_NS);
        const unsigned long long c1 = clock64();
        if (!ok) {
            if (err) atomicCAS(err, 0, 0x800);
            tc::mbar_wait(tc::smem_u32(&bar), 0, &never, WAIT_NS);  // once more before freeing tensor memory
        }
        cycles[blockIdx.x] = c1 - c0;
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tm, 512);
    }
}

constexpr int CHAINS = 8;

// mma.sync throughput: eight independent accumulator chains per warp.
template <int S8>
__global__ void __launch_bounds__(512, 1) mma_sync_rate_kernel(int iters, const uint32_t *in, uint32_t *out,
                                                                unsigned long long *cycles) {
    const int t = threadIdx.x;
    uint32_t a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = in[(t + i) & 63];
    b[0] = in[(t + 5) & 63];
    b[1] = in[(t + 9) & 63];
    uint32_t c[CHAINS][4];
#pragma unroll
    for (int j = 0; j < CHAINS; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) c[j][i] = 0;
    const unsigned long long c0 = clock64();
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int j = 0; j < CHAINS; j++) {
            if (S8)
                asm volatile(
                    "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
            else
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
        }
    }
    const unsigned long long c1 = clock64();
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < CHAINS; j++) s += c[j][0] ^ c[j][1] ^ c[j][2] ^ c[j][3];
    out[blockIdx.x * blockDim.x + t] = s;
    if (t == 0) cycles[blockIdx.x] = c1 - c0;
}

}  // namespace rate
}  // namespace pg

using namespace pg;

extern "C" int pg_tensor_rate(pg_ctx *c, int form, int iters, double *out) {
    if (!c || !out) return PG_ERR_INVALID_ARG;
    if (form < PG_RATE_TC_F16 || form > PG_RATE_MMA_F16 || iters <= 0 || iters > (1 << 24))
        return set_error(c, PG_ERR_INVALID_ARG, "tensor_rate: form %d, iters %d", form, iters);
    PG_CHECK_CUDA(c, cudaSetDevice(c->device));
    const bool tc = form == PG_RATE_TC_F16 || form == PG_RATE_TC_F8;
    const int blocks = c->sm_count;
    const int threads = tc ? 128 : 512;
    unsigned long long *cyc = nullptr;
    uint32_t *io = nullptr;
    PG_CHECK_CUDA(c, cudaMalloc(&cyc, sizeof(unsigned long long) * blocks));
    const size_t io_words = 64 + (size_t)blocks * threads;
    if (cudaMalloc(&io, io_words * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(cyc);
        return set_error(c, PG_ERR_NO_MEMORY, "tensor_rate: buffers");
    }
    int st = PG_OK;
    // tcgen05 forms: an unused dynamic shared-memory reservation keeps one CTA
    // (one 512-column tensor-memory allocation) per SM
    const int pad_smem = tc ? 160 * 1024 : 0;
    if (tc && (cudaFuncSetAttribute(rate::tc_rate_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, pad_smem) !=
                   cudaSuccess ||
               cudaFuncSetAttribute(rate::tc_rate_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, pad_smem) !=
                   cudaSuccess)) {
        cudaGetLastError();
        st = set_error(c, PG_ERR_CUDA, "tensor_rate: shared-memory limit");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    if (st == PG_OK && cudaMemsetAsync(io, 0x35, 64 * sizeof(uint32_t), c->stream) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        st = set_error(c, PG_ERR_CUDA, "tensor_rate: set-up");
    }
    for (int rep = 0; rep < 2 && st == PG_OK; rep++) {  // one warm-up launch, one timed
        const int n = rep == 0 ? (iters / 8 > 0 ? iters / 8 : 1) : iters;
        cudaEventRecord(e0, c->stream);
        switch (form) {
            case PG_RATE_TC_F16: rate::tc_rate_kernel<0><<<blocks, threads, pad_smem, c->stream>>>(n, cyc, c->dev_err); break;
            case PG_RATE_TC_F8: rate::tc_rate_kernel<1><<<blocks, threads, pad_smem, c->stream>>>(n, cyc, c->dev_err); break;
            case PG_RATE_MMA_S8:
                rate::mma_sync_rate_kernel<1><<<blocks, threads, 0, c->stream>>>(n, io, io + 64, cyc);
                break;
            default: rate::mma_sync_rate_kernel<0><<<blocks, threads, 0, c->stream>>>(n, io, io + 64, cyc); break;
        }
        cudaEventRecord(e1, c->stream);
        st = launch_status(c, "tensor_rate");
        c->launches++;
    }
    if (st == PG_OK && cudaEventSynchronize(e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "tensor_rate: sync");
    if (st == PG_OK) {
        cudaEventElapsedTime(&ms, e0, e1);
        unsigned long long *hc = new unsigned long long[blocks];
        cudaMemcpy(hc, cyc, sizeof(unsigned long long) * blocks, cudaMemcpyDeviceToHost);
        double cmax = 0;
        for (int i = 0; i < blocks; i++) cmax = hc[i] > cmax ? (double)hc[i] : cmax;
        delete[] hc;
        // operations of one instruction, and instructions per CTA (tcgen05) or per warp (mma.sync)
        double ops_per_inst, inst_per_stream, streams;
        if (tc) {
            ops_per_inst = 2.0 * rate::TC_M * rate::TC_N * (form == PG_RATE_TC_F8 ? 32 : 16);
            inst_per_stream = iters;
            streams = blocks;
        } else {
            ops_per_inst = 2.0 * 16 * 8 * (form == PG_RATE_MMA_S8 ? 32 : 16);
            inst_per_stream = (double)iters * rate::CHAINS;
            streams = (double)blocks * threads / 32;
        }
        out[0] = ops_per_inst * inst_per_stream * streams / (ms * 1e-3) / 1e12;  // tera-ops per second
        out[1] = cmax / inst_per_stream;                                         // SM cycles per instruction
        out[2] = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(io);
    cudaFree(cyc);
    return st;
}
