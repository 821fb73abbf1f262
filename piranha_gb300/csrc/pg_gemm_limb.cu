// pg_gemm_limb.cu — the 8-bit-limb tensor-core form of the RSS share-GEMM and
// implicit-GEMM convolution (tcgen05, fp16 operands, fp32 accumulators in
// tensor memory), exact modulo 2^64.
//
// Arithmetic. Every 64-bit operand v is written as eight signed digits
// d_i = byte_i(v) - 128 in [-128, 127], so v = sum_i d_i 2^(8i) + C with
// C = 0x8080808080808080 (mod 2^64). A digit is exact in fp16 and a digit
// product has magnitude <= 2^14. For a contraction over K' terms
//   sum a*b = sum_s 2^(8s) D_s + C*(sum a) + C*(sum b) - K'*C^2   (mod 2^64)
// with D_s = sum_{i+j=s} sum_k d_i(a_k) d_j(b_k) for the 36 digit pairs with
// i+j < 8 (pairs with i+j >= 8 vanish mod 2^64). One tcgen05.mma per pair and
// K step of 16 accumulates D_s in fp32 tensor memory. Each output tile runs
// two passes over K': the high pass (diagonals 4-7, 26 pairs, needed only
// modulo 2^32) and the low pass (diagonals 0-3, 10 pairs, digits 0-3 only).
// A pass keeps four accumulators and two tensor-memory buffers, so the
// epilogue warps drain one buffer into 64-bit registers while the MMAs fill
// the other; chunk lengths keep every |D_s| <= 2^24, so every fp32 sum is an
// exact integer. The row sums of A are accumulated by the producer warps and
// the column sums of B by the packing kernel.
//
// Protocol. The K' dimension is the concatenation of the six RSS segments
// [x_p0 | x_p1] x [y_p0 + y_p1 ; y_p0] of the three parties (localMatMul,
// src/mpc/RSS.inl:1097-1110; localFprop :614-639), so Z = sum_p z_p, which
// the epilogue truncates with dividePublic3out3 (:1077-1094).
//
// Operands. B (weights, y_p0 + y_p1 and y_p0 per party) is converted once per
// call by pack_b_kernel into limb planes laid out exactly as the kernel's
// shared-memory stages (16 KB per segment, K block of 16 and N tile of 64), with
// its column sums; the GEMM streams it in with one bulk async copy per stage.
// A (activations, implicit im2col for conv) is converted on chip.
//
// Roles (448 threads): warps 0-3 load A rows (one row per thread, two
// 8-value units per stage, loads for the next stage in flight while the
// current one is converted) and accumulate the row sums; warp 4 issues the B
// bulk copies; warp 5 owns the tensor memory and one lane issues the MMAs;
// warps 6-13 drain tensor memory (two warps per 32-lane quarter, 32 columns
// each) and run the epilogue. Every mbarrier wait is
// bounded; on a timeout the kernel records an error word, stops issuing work,
// waits for its own MMAs and frees tensor memory before returning.
#include <cuda_fp16.h>

#include <cstring>

#include "pg_common.cuh"
#include "pg_tcgen05.cuh"

namespace pg {

namespace limb {

constexpr int BM = 128, BN = 64, BK = 16, STAGES = 4;
// K' per fp32 accumulation chunk: the high pass (diagonals 4-7, up to 8 pairs
// per diagonal) drains every 128 K' (8 stages), the low pass (diagonals 0-3,
// up to 4 pairs) every 256 K' (16 stages): |D_s| <= (pairs * K'chunk) * 2^14 <= 2^24.
constexpr int CHUNK_STAGES = 8, CHUNK_STAGES_LO = 16;
constexpr int A_LIMB_BYTES = BM * BK * 2;                               // 4096
constexpr int B_LIMB_BYTES = BN * BK * 2;                               // 2048
constexpr int B_STAGE_BYTES = 8 * B_LIMB_BYTES;                         // 16384
constexpr int STAGE_BYTES = 8 * A_LIMB_BYTES + B_STAGE_BYTES;           // 49152
constexpr int NTHREADS = 448;
constexpr int W_BPROD = 4, W_MMA = 5, W_EPI0 = 6;
constexpr uint32_t TMEM_COLS = 512;  // 2 buffers x 4 diagonals x 64 columns
constexpr uint64_t CDIG = 0x8080808080808080ull;
constexpr uint64_t WAIT_NS = 2000000000ull;  // 2 s bound on any single wait

enum { KIND_GEMM = 0, KIND_FPROP = 1 };

struct FastDivL {
    uint32_t d, m;
    int s;
    __host__ void init(uint32_t dd) {
        d = dd;
        if (dd <= 1) { m = 0; s = 0; return; }
        s = 0;
        while ((1ull << s) < dd) s++;
        m = (uint32_t)((((1ull << 32) * ((1ull << s) - dd)) / dd) + 1);
    }
    __device__ __forceinline__ uint32_t div(uint32_t x) const {
        if (d == 1) return x;
        uint32_t hi = __umulhi(x, m);
        return (hi + ((x - hi) >> 1)) >> (s - 1);
    }
};

struct Args {
    int M, N, Kseg, nseg;
    const uint64_t *a[6];
    const uint8_t *packB;      // [seg][kb][ntile][16 KB] limb planes of B
    const uint64_t *colsum;    // [split][ntiles*64] column sums of B over each K' slice
    int kind, tA, tC;
    int ntiles_n, kblocks;     // kblocks = Kseg / 16
    // conv fprop geometry
    int ch, cw, cc, cs, cp, cq, pad, stride;
    FastDivL dQ, dP, dC, dS;
    // K' split: chunks [z*chunks_per_split, ...) of the total
    int total_stages, chunks_per_split;
    // epilogue
    int direct;           // 1: RSS epilogue here; 0: write the slice's Z to partial
    uint64_t *partial;    // [gridDim.z][M][N]
    uint64_t *out[6];
    const uint64_t *bias[6];
    uint64_t d;
    int dshift;
    int *err;
};

struct __align__(16) Smem {
    uint8_t stage[STAGES][STAGE_BYTES];
    Args args;  // kernel arguments, copied here so that dynamic indexing stays out of local memory
    uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], done;
    uint64_t rowsum[BM], colsum[BN];
    uint32_t tmem_base;
    int abort;
};

// ---------------------------------------------------------------- loaders

// 8 consecutive K' values of row m of A (K' offset k of segment seg)
__device__ __forceinline__ void load_a8(const Args &g, int seg, int m, int k, uint64_t (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = 0;
    if (m >= g.M) return;
    const uint64_t *a = g.a[seg];
    if (g.kind == KIND_FPROP) {
        uint32_t nq = g.dQ.div(m), q = m - nq * g.cq;
        uint32_t n = g.dP.div(nq), p = nq - n * g.cp;
        uint32_t rs = g.dC.div(k), c = k - rs * g.cc;
        uint32_t r = g.dS.div(rs), s = rs - r * g.cs;
        int h = (int)(p * g.stride) - g.pad + (int)r, w = (int)(q * g.stride) - g.pad + (int)s;
        if (h < 0 || h >= g.ch || w < 0 || w >= g.cw) return;
        const ulonglong2 *src = (const ulonglong2 *)(a + ((((size_t)n * g.ch + h) * g.cw + w) * g.cc + c));
#pragma unroll
        for (int i = 0; i < 4; i++) {
            ulonglong2 t = __ldg(src + i);
            v[2 * i] = t.x;
            v[2 * i + 1] = t.y;
        }
    } else if (g.tA) {
        const ulonglong2 *src = (const ulonglong2 *)(a + (size_t)m * g.Kseg + k);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            ulonglong2 t = __ldg(src + i);
            v[2 * i] = t.x;
            v[2 * i + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = __ldg(a + (size_t)m + (size_t)(k + i) * g.M);
    }
}

// byte i of each of v[k], v[k+1] as fp16 (byte - 128), packed in one half2 word
__device__ __forceinline__ uint32_t digit_pair(uint32_t wk, uint32_t wk1, uint32_t sel) {
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(wk), "r"(wk1), "r"(sel));
    d = (d & 0x00FF00FFu) | 0x64006400u;  // fp16 1024 + byte
    __half2 h = *reinterpret_cast<__half2 *>(&d);
    h = __hsub2(h, __halves2half2(__ushort_as_half(0x6480), __ushort_as_half(0x6480)));  // - 1152
    return *reinterpret_cast<uint32_t *>(&h);
}

// Convert 8 u64 values (consecutive K' of one row) into the 8 limb planes:
// limb i goes to plane_base + i*plane_bytes at core-matrix offset off.
__device__ __forceinline__ void store_limbs(uint8_t *plane_base, int plane_bytes, uint32_t off,
                                            const uint64_t (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint32_t w[4];
#pragma unroll
        for (int p = 0; p < 4; p++) {
            uint32_t a = i < 4 ? (uint32_t)v[2 * p] : (uint32_t)(v[2 * p] >> 32);
            uint32_t b = i < 4 ? (uint32_t)v[2 * p + 1] : (uint32_t)(v[2 * p + 1] >> 32);
            // prmt selector: d.byte0 = a.byte(i&3), d.byte2 = b.byte(i&3) (bytes 1, 3 masked off)
            const uint32_t sel = (uint32_t)(i & 3) | ((uint32_t)(i & 3) << 4) | ((uint32_t)(4 + (i & 3)) << 8) |
                                 ((uint32_t)(4 + (i & 3)) << 12);
            w[p] = digit_pair(a, b, sel);
        }
        uint4 q = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4 *>(plane_base + i * plane_bytes + off) = q;
    }
}

// Limbs 0-3 only (the low 32 bits of each value), for the low-digit pass.
__device__ __forceinline__ void store_limbs_lo(uint8_t *plane_base, int plane_bytes, uint32_t off,
                                               const uint64_t (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint32_t w[4];
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const uint32_t sel = (uint32_t)i | ((uint32_t)i << 4) | ((uint32_t)(4 + i) << 8) | ((uint32_t)(4 + i) << 12);
            w[p] = digit_pair((uint32_t)v[2 * p], (uint32_t)v[2 * p + 1], sel);
        }
        *reinterpret_cast<uint4 *>(plane_base + i * plane_bytes + off) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// core-matrix offset of (row, 8-element chunk kc) inside a limb plane
__host__ __device__ __forceinline__ uint32_t cm_off(int row, int kc) {
    return (uint32_t)((row >> 3) * 256 + kc * 128 + (row & 7) * 16);
}

__device__ __forceinline__ void flag_error(Smem &sm, const Args &g, int code) {
    sm.abort = 1;
    if (g.err) atomicCAS(g.err, 0, code);
}

// Move four diagonal accumulators (32 columns of this thread's TMEM lane)
// into the 64-bit running sums. HI: diagonals 4-7, which matter only modulo
// 2^32 (shift >= 32), so only the high word is touched; LO: diagonals 0-3,
// added as sign-extended 64-bit values shifted by 8s.
template <bool HI>
__device__ __forceinline__ void drain4(uint32_t taddr, uint64_t (&run)[32]) {
#pragma unroll
    for (int a = 0; a < 4; a++) {
        uint32_t r[32];
        tc::tmem_ld32(taddr + (uint32_t)(a * BN), r);
        tc::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; j++) {
            int v = __float2int_rz(__uint_as_float(r[j]));  // exact: |v| <= 2^24
            if (HI) run[j] += (uint64_t)((uint32_t)v << (8 * a)) << 32;
            else run[j] += (uint64_t)(int64_t)v << (8 * a);
        }
    }
}

// Final epilogue for 32 columns of one row: add the digit-offset correction,
// then either store the slice's partial Z or apply dividePublic3out3 and
// write the six output shares (+ bias shares).
__device__ __forceinline__ void finish32(const Args &g, const Smem &sm, int z, int m, int row, int nbase, int cbase,
                                         uint64_t kc2, uint64_t (&run)[32]) {
    const uint64_t rs = sm.rowsum[row];
#pragma unroll
    for (int j = 0; j < 32; j++) run[j] += CDIG * (rs + sm.colsum[cbase + j]) - kc2;
    const int ncols = g.N - nbase < 32 ? g.N - nbase : 32;
    if (!g.direct) {
        uint64_t *dst = g.partial + ((size_t)z * g.M + m) * g.N + nbase;
#pragma unroll
        for (int j = 0; j < 32; j++)
            if (j < ncols) dst[j] = run[j];
        return;
    }
    const bool colmajor = (g.kind == KIND_GEMM && !g.tC);
#pragma unroll
    for (int j8 = 0; j8 < 32; j8 += 8) {
        uint64_t v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = 1 + div_public<uint64_t>(run[j8 + j] - g.d, g.d, g.dshift);
#pragma unroll 1
        for (int ps = 0; ps < 6; ps++) {
            uint64_t *o = g.out[ps];
            const uint64_t *b = g.bias[ps];
            const bool val = (ps == 0 || ps == 5);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (j8 + j < ncols) {
                    const int n = nbase + j8 + j;
                    uint64_t base = val ? v[j] : 0;
                    if (b) base += b[n];
                    o[colmajor ? (size_t)m + (size_t)n * g.M : (size_t)m * g.N + n] = base;
                }
            }
        }
    }
}

// All MMAs of one stage for the diagonals D0..D0+3. For a fixed A digit
// plane i, the pairs (i, j) with i + j in the pass's range use consecutive B
// digit planes j = jlo..jhi, which sit in shared memory exactly as one
// (64*cnt)-row operand, and land in consecutive 64-column accumulators
// d - D0 = i + jlo - D0 ... So one MMA with N = 64*cnt covers them all: 8
// MMAs per stage for the high pass (N = 256 x5, 192, 128, 64) and 4 for the
// low pass (N = 256, 192, 128, 64).
template <int D0>
__device__ __forceinline__ void issue_stage(uint32_t acc, uint64_t adesc, uint64_t bdesc, bool first_stage) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int jlo = D0 - i > 0 ? D0 - i : 0;
        const int jhi = D0 + 3 - i;  // inclusive
        const int cnt = jhi - jlo + 1;
        if (cnt <= 0) continue;
        const uint64_t ad = adesc + (uint64_t)((i * A_LIMB_BYTES) >> 4);
        const uint64_t bd = bdesc + (uint64_t)((jlo * B_LIMB_BYTES) >> 4);
        const uint32_t d = acc + (uint32_t)((i + jlo - D0) * BN);
        const uint32_t accum = (!first_stage || i > 0) ? 1u : 0u;  // i = 0 writes all four accumulators first
        tc::mma_f16(d, ad, bd, tc::idesc_f16_f32(BM, BN * cnt), accum);
    }
}

// ------------------------------------------------------------------ kernel

__global__ void __launch_bounds__(NTHREADS, 1) limb_gemm_kernel(const __grid_constant__ Args gp) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&gp);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sm.args);
        for (int i = threadIdx.x; i < (int)(sizeof(Args) / 4); i += blockDim.x) dst[i] = src[i];
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int z = blockIdx.z;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(tc::smem_u32(&sm.full[s]), 128 + 1);  // A producers + the B bulk-copy arrive
            tc::mbar_init(tc::smem_u32(&sm.empty[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(tc::smem_u32(&sm.acc_full[b]), 1);
            tc::mbar_init(tc::smem_u32(&sm.acc_empty[b]), 256);
        }
        tc::mbar_init(tc::smem_u32(&sm.done), 1);
        sm.abort = 0;
        tc::fence_mbar_init();
    }
    if (warp == W_MMA) {
        tc::tmem_alloc(tc::smem_u32(&sm.tmem_base), TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const Args &g = sm.args;
    const uint32_t tmem = sm.tmem_base;
    const int stage_begin = z * g.chunks_per_split * CHUNK_STAGES;
    int stage_end = stage_begin + g.chunks_per_split * CHUNK_STAGES;
    if (stage_end > g.total_stages) stage_end = g.total_stages;
    const int nst = stage_end > stage_begin ? stage_end - stage_begin : 0;
    const int stages_per_seg = g.kblocks;

    if (warp < 4) {
        // ----------------------------------------------------- A producers
        const int row = threadIdx.x;  // tile row; units (row, chunk 0) and (row, chunk 1) per stage
        uint64_t rsum = 0;
        uint64_t bufA[2][8], bufB[2][8];
        auto load_stage = [&](int it, uint64_t (&buf)[2][8]) {
            const int gst = stage_begin + it;
            const int seg = gst / stages_per_seg;
            const int k0 = (gst - seg * stages_per_seg) * BK;
            load_a8(g, seg, m0 + row, k0, buf[0]);
            load_a8(g, seg, m0 + row, k0 + 8, buf[1]);
        };
        // global ring position: pass 0 (high digits) stages 0..nst-1, pass 1 (low) nst..2*nst-1
        auto step = [&](int it, bool lo_pass, uint64_t (&cur)[2][8], uint64_t (&nxt)[2][8]) -> bool {
            const int git = it + (lo_pass ? nst : 0);
            const int s = git % STAGES;
            const uint32_t ph = (uint32_t)(git / STAGES) & 1;
            if (!tc::mbar_wait(tc::smem_u32(&sm.empty[s]), ph ^ 1, &sm.abort, WAIT_NS)) {
                flag_error(sm, g, 0x100 + s);
                return false;
            }
            if (it + 1 < nst) load_stage(it + 1, nxt);
            else if (!lo_pass) load_stage(0, nxt);  // first stage of the low pass
#pragma unroll
            for (int kc = 0; kc < 2; kc++) {
                if (!lo_pass) {
#pragma unroll
                    for (int i = 0; i < 8; i++) rsum += cur[kc][i];
                    store_limbs(sm.stage[s], A_LIMB_BYTES, cm_off(row, kc), cur[kc]);
                } else {
                    store_limbs_lo(sm.stage[s], A_LIMB_BYTES, cm_off(row, kc), cur[kc]);
                }
            }
            tc::fence_proxy_async_smem();
            tc::mbar_arrive(tc::smem_u32(&sm.full[s]));
            return true;
        };
        bool ok = true;
        if (nst > 0) load_stage(0, bufA);
        // both passes together have 2*nst stages; nst parity decides which buffer starts the low pass
        for (int pass = 0; pass < 2 && ok; pass++) {
            const bool lo = pass == 1;
            const bool startA = !lo || (nst % 2 == 0);
            for (int it = 0; it < nst && ok; it += 2) {
                if (startA) {
                    ok = step(it, lo, bufA, bufB);
                    if (ok && it + 1 < nst) ok = step(it + 1, lo, bufB, bufA);
                } else {
                    ok = step(it, lo, bufB, bufA);
                    if (ok && it + 1 < nst) ok = step(it + 1, lo, bufA, bufB);
                }
            }
        }
        sm.rowsum[row] = rsum;
        if (row < BN) sm.colsum[row] = g.colsum[(size_t)z * g.ntiles_n * BN + n0 + row];
        asm volatile("bar.sync 1, 384;" ::: "memory");  // A producers + epilogue
    } else if (warp == W_BPROD) {
        // ------------------------------------------------ B bulk copies
        if (lane == 0) {
            for (int git = 0; git < 2 * nst; git++) {
                const bool lo = git >= nst;
                const int it = lo ? git - nst : git;
                const int s = git % STAGES;
                const uint32_t ph = (uint32_t)(git / STAGES) & 1;
                if (!tc::mbar_wait(tc::smem_u32(&sm.empty[s]), ph ^ 1, &sm.abort, WAIT_NS)) {
                    flag_error(sm, g, 0x180 + s);
                    break;
                }
                const int gst = stage_begin + it;  // = seg * kblocks + kb
                const uint8_t *src = g.packB + ((size_t)gst * g.ntiles_n + blockIdx.x) * B_STAGE_BYTES;
                const uint32_t bar = tc::smem_u32(&sm.full[s]);
                const uint32_t bytes = lo ? B_STAGE_BYTES / 2 : B_STAGE_BYTES;  // limbs 0-3 lead the image
                tc::mbar_arrive_expect_tx(bar, bytes);
                tc::bulk_g2s(tc::smem_u32(sm.stage[s] + 8 * A_LIMB_BYTES), src, bytes, bar);
            }
        }
        __syncwarp();
    } else if (warp == W_MMA) {
        // ------------------------------------------------------------- MMA
        if (lane == 0) {
            const uint64_t desc0 = tc::smem_desc(tc::smem_u32(sm.stage[0]), 128, 256);
            int git = 0, gc = 0;  // ring position, global chunk (buffer = gc & 1)
            bool ok = true;
            for (int pass = 0; pass < 2 && ok; pass++) {
                const bool lo = pass == 1;
                const int cstages = lo ? CHUNK_STAGES_LO : CHUNK_STAGES;
                const int nch = (nst + cstages - 1) / cstages;
                for (int c = 0; c < nch && ok; c++, gc++) {
                    const int buf = gc & 1;
                    if (gc >= 2 && !tc::mbar_wait(tc::smem_u32(&sm.acc_empty[buf]), (uint32_t)((gc - 2) >> 1) & 1,
                                                  &sm.abort, WAIT_NS)) {
                        flag_error(sm, g, 0x200 + buf);
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t acc = tmem + (uint32_t)(buf * 4 * BN);
                    const int cst = (nst - c * cstages) < cstages ? nst - c * cstages : cstages;
                    for (int st = 0; st < cst; st++, git++) {
                        const int s = git % STAGES;
                        const uint32_t ph = (uint32_t)(git / STAGES) & 1;
                        if (!tc::mbar_wait(tc::smem_u32(&sm.full[s]), ph, &sm.abort, WAIT_NS)) {
                            flag_error(sm, g, 0x300 + s);
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
                        const uint64_t ad = desc0 + (uint64_t)((s * STAGE_BYTES) >> 4);
                        const uint64_t bd = ad + (uint64_t)((8 * A_LIMB_BYTES) >> 4);
                        if (lo) issue_stage<0>(acc, ad, bd, st == 0);
                        else issue_stage<4>(acc, ad, bd, st == 0);
                        tc::mma_commit(tc::smem_u32(&sm.empty[s]));
                    }
                    if (!ok) break;
                    tc::mma_commit(tc::smem_u32(&sm.acc_full[buf]));
                }
            }
            // all MMAs this thread issued are complete once `done` fires
            tc::mma_commit(tc::smem_u32(&sm.done));
            if (!tc::mbar_wait(tc::smem_u32(&sm.done), 0, &sm.abort, WAIT_NS) && g.err) atomicCAS(g.err, 0, 0x400);
        }
        __syncwarp();
    } else {
        // -------------------------------------------------------- epilogue
        const int q = warp & 3;                  // TMEM lane quarter this warp may access
        const int colh = (warp - W_EPI0) >> 2;   // which 32 of the 64 columns
        const int row = q * 32 + lane;           // tile row = TMEM lane
        uint64_t run[32];
#pragma unroll
        for (int j = 0; j < 32; j++) run[j] = 0;
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(colh * 32);
        const int nch_hi = (nst + CHUNK_STAGES - 1) / CHUNK_STAGES;
        const int nch_lo = (nst + CHUNK_STAGES_LO - 1) / CHUNK_STAGES_LO;
        for (int gc = 0; gc < nch_hi + nch_lo; gc++) {
            const int buf = gc & 1;
            if (!tc::mbar_wait(tc::smem_u32(&sm.acc_full[buf]), (uint32_t)(gc >> 1) & 1, &sm.abort, WAIT_NS)) {
                flag_error(sm, g, 0x500);
                break;
            }
            tc::tc_fence_after();
            if (gc < nch_hi) drain4<true>(taddr + (uint32_t)(buf * 4 * BN), run);
            else drain4<false>(taddr + (uint32_t)(buf * 4 * BN), run);
            tc::tc_fence_before();
            tc::mbar_arrive(tc::smem_u32(&sm.acc_empty[buf]));
        }
        asm volatile("bar.sync 1, 384;" ::: "memory");
        const int m = m0 + row;
        if (!sm.abort && m < g.M) {
            const uint64_t kc2 = (uint64_t)nst * BK * (CDIG * CDIG);
            finish32(g, sm, z, m, row, n0 + colh * 32, colh * 32, kc2, run);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == W_MMA) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// Convert B (segment seg: y_p0 + y_p1 for even seg, y_p0 for odd) into the
// stage image layout and accumulate the column sums. One thread per
// (segment, column, K block of 16, chunk of 8).
struct PackArgs {
    const uint64_t *b[6];
    int N, Kseg, ntiles_n, kblocks, tB, kind;
    int stages_per_split;  // column sums are kept per K' slice of this many stages
    uint8_t *packB;
    uint64_t *colsum;
};

__global__ void pack_b_kernel(const __grid_constant__ PackArgs pa) {
    const size_t total = (size_t)6 * pa.ntiles_n * BN * pa.kblocks * 2;
    for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < total; u += (size_t)gridDim.x * blockDim.x) {
        const int kc = (int)(u & 1);
        size_t t = u >> 1;
        const int kb = (int)(t % pa.kblocks);
        t /= pa.kblocks;
        const int n = (int)(t % ((size_t)pa.ntiles_n * BN));
        const int seg = (int)(t / ((size_t)pa.ntiles_n * BN));
        const int p = seg >> 1;
        const int k = kb * BK + kc * 8;
        uint64_t v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = 0;
        if (n < pa.N) {
            const uint64_t *b0 = pa.b[2 * p], *b1 = (seg & 1) ? nullptr : pa.b[2 * p + 1];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                size_t idx = (pa.kind == KIND_FPROP || !pa.tB) ? (size_t)n * pa.Kseg + k + i : (size_t)(k + i) * pa.N + n;
                v[i] = b0[idx] + (b1 ? b1[idx] : 0);
            }
            uint64_t sum = 0;
#pragma unroll
            for (int i = 0; i < 8; i++) sum += v[i];
            const int slice = (seg * pa.kblocks + kb) / pa.stages_per_split;
            atomicAdd((unsigned long long *)&pa.colsum[(size_t)slice * pa.ntiles_n * BN + n], (unsigned long long)sum);
        }
        const int nt = n / BN, nr = n % BN;
        uint8_t *dst = pa.packB + (((size_t)seg * pa.kblocks + kb) * pa.ntiles_n + nt) * B_STAGE_BYTES;
        store_limbs(dst, B_LIMB_BYTES, cm_off(nr, kc), v);
    }
}

// sum the split-K partials and apply dividePublic3out3 (+ bias)
__global__ void limb_reduce_kernel(const Args g, int nsplit) {
    size_t total = (size_t)g.M * g.N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        uint64_t zv = 0;
        for (int s = 0; s < nsplit; s++) zv += g.partial[(size_t)s * total + e];
        int m = (int)(e / g.N), n = (int)(e % g.N);
        size_t idx = (g.kind == KIND_GEMM && !g.tC) ? (size_t)m + (size_t)n * g.M : e;
        uint64_t vv = 1 + div_public<uint64_t>(zv - g.d, g.d, g.dshift);
#pragma unroll
        for (int ps = 0; ps < 6; ps++) {
            uint64_t base = (ps == 0 || ps == 5) ? vv : 0;
            if (g.bias[ps]) base += g.bias[ps][n];
            g.out[ps][idx] = base;
        }
    }
}

// ------------------------------------------------------------- self test

// One 128x64x16 MMA of fp16 integers: D = A * B^T with A, B given K-major
// (row-major 128x16 and 64x16 halves). Checks descriptors, instruction
// descriptor and the TMEM lane/column layout against a host reference.
__global__ void __launch_bounds__(128, 1) selftest_kernel(const uint16_t *A, const uint16_t *B, float *D, int *err) {
    __shared__ __align__(1024) uint8_t sa[A_LIMB_BYTES];
    __shared__ __align__(1024) uint8_t sb[B_LIMB_BYTES];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    __shared__ int abort_flag;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int kc = 0; kc < 2; kc++) {
        *reinterpret_cast<uint4 *>(sa + cm_off(t, kc)) = *reinterpret_cast<const uint4 *>(A + t * 16 + kc * 8);
        if (t < 64) *reinterpret_cast<uint4 *>(sb + cm_off(t, kc)) = *reinterpret_cast<const uint4 *>(B + t * 16 + kc * 8);
    }
    if (t == 0) {
        tc::mbar_init(tc::smem_u32(&bar), 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    tc::fence_proxy_async_smem();
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_u32(&tbase), 64);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tm = tbase;
    if (t == 0) {
        tc::mma_f16(tm, tc::smem_desc(tc::smem_u32(sa), 128, 256), tc::smem_desc(tc::smem_u32(sb), 128, 256),
                    tc::idesc_f16_f32(128, 64), 0u);
        tc::mma_commit(tc::smem_u32(&bar));
    }
    __syncwarp();
    bool ok = tc::mbar_wait(tc::smem_u32(&bar), 0, &abort_flag, WAIT_NS);
    if (!ok && err) atomicCAS(err, 0, 0x600);
    tc::tc_fence_after();
    if (ok) {
        for (int half = 0; half < 2; half++) {
            uint32_t r[32];
            tc::tmem_ld32(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)(half * 32), r);
            tc::tmem_wait_ld();
            for (int j = 0; j < 32; j++) D[(warp * 32 + lane) * 64 + half * 32 + j] = __uint_as_float(r[j]);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tm, 64);
    }
}

static size_t smem_bytes() { return sizeof(Smem) + 1024; }

}  // namespace limb

int *device_error_word(Ctx *c);
template <typename T>
int rss_matmul(Ctx *, const T *const *, const T *const *, T *const *, const T *const *, int, int, int, int, int, int,
               int);
template <typename T>
int rss_conv(Ctx *, const T *const *, const T *const *, T *const *, int, int, int, int, int, int, int, int, int, int);

// b: the six B share pointers (layout per g.kind / tB)
static int limb_launch(Ctx *c, limb::Args &g, int tB, const uint64_t *const *b) {
    using namespace limb;
    static bool attr_set = false;
    if (!attr_set) {
        PG_CHECK_CUDA(c, cudaFuncSetAttribute(limb_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem_bytes()));
        attr_set = true;
    }
    const int tiles_m = (g.M + BM - 1) / BM, tiles_n = (g.N + BN - 1) / BN;
    const int tiles = tiles_m * tiles_n;
    g.ntiles_n = tiles_n;
    g.kblocks = g.Kseg / BK;
    const int total_stages = 6 * g.kblocks;
    const int chunks = (total_stages + CHUNK_STAGES - 1) / CHUNK_STAGES;
    int sms = c->sm_count > 0 ? c->sm_count : 148;
    int split = tiles >= sms ? 1 : sms / tiles;
    if (split > chunks) split = chunks;
    if (split < 1) split = 1;
    int cps = (chunks + split - 1) / split;
    split = (chunks + cps - 1) / cps;
    g.total_stages = total_stages;
    g.chunks_per_split = cps;
    g.err = device_error_word(c);
    // scratch: packed B stages, column sums, then [split][M][N] partials (all 256-byte aligned)
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t pack_bytes = (size_t)total_stages * tiles_n * B_STAGE_BYTES;
    const size_t col_bytes = al((size_t)split * tiles_n * BN * 8);
    const size_t part_bytes = split > 1 ? (size_t)split * g.M * g.N * 8 : 0;
    uint8_t *scr = (uint8_t *)scratch(c, pack_bytes + col_bytes + part_bytes);
    if (!scr) return PG_ERR_NO_MEMORY;
    g.packB = scr;
    g.colsum = (uint64_t *)(scr + pack_bytes);
    PG_CHECK_CUDA(c, cudaMemsetAsync((void *)g.colsum, 0, col_bytes, c->stream));
    {
        PackArgs pa;
        memset(&pa, 0, sizeof(pa));
        for (int i = 0; i < 6; i++) pa.b[i] = b[i];
        pa.N = g.N; pa.Kseg = g.Kseg; pa.ntiles_n = tiles_n; pa.kblocks = g.kblocks; pa.tB = tB; pa.kind = g.kind;
        pa.stages_per_split = cps * CHUNK_STAGES;
        pa.packB = scr;
        pa.colsum = (uint64_t *)(scr + pack_bytes);
        size_t units = (size_t)6 * tiles_n * BN * g.kblocks * 2;
        unsigned blocks = (unsigned)((units + 255) / 256);
        if (blocks > (unsigned)sms * 16) blocks = sms * 16;
        pack_b_kernel<<<blocks, 256, 0, c->stream>>>(pa);
        c->launches++;
        int st = launch_status(c, "pack_b_kernel");
        if (st) return st;
    }
    if (split > 1) {
        g.partial = (uint64_t *)(scr + pack_bytes + col_bytes);
        g.direct = 0;
    } else {
        g.direct = 1;
    }
    dim3 grid(tiles_n, tiles_m, split);
    limb_gemm_kernel<<<grid, NTHREADS, smem_bytes(), c->stream>>>(g);
    c->launches++;
    int st = launch_status(c, "limb_gemm_kernel");
    if (st) return st;
    if (split > 1) {
        size_t total = (size_t)g.M * g.N;
        unsigned blocks = (unsigned)((total + 255) / 256);
        if (blocks > (unsigned)sms * 8) blocks = sms * 8;
        limb_reduce_kernel<<<blocks, 256, 0, c->stream>>>(g, split);
        c->launches++;
        st = launch_status(c, "limb_reduce_kernel");
        if (st) return st;
    }
    return PG_OK;
}

static void limb_segments(limb::Args &g, const uint64_t *const *a) {
    g.nseg = 6;
    for (int i = 0; i < 6; i++) g.a[i] = a[i];  // segment 2p: x_p0, segment 2p+1: x_p1
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

int limb_rss_matmul_u64(Ctx *c, const uint64_t *const a[6], const uint64_t *const b[6], uint64_t *const out[6],
                        const uint64_t *const bias[6], int M, int N, int K, int tA, int tB, int tC, int trunc) {
    CSh6<uint64_t> ca, cb;
    Sh6<uint64_t> co;
    if (!load6(ca, a) || !load6(cb, b) || !load6(co, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    bool ok = (K % limb::BK) == 0;
    for (int i = 0; i < 6 && ok; i++) ok = aligned16(a[i]) && aligned16(b[i]);
    if (tA && (K % 2)) ok = false;
    if (!ok)  // shapes the limb tiles do not cover run on the integer CUDA cores
        return rss_matmul<uint64_t>(c, a, b, out, bias, M, N, K, tA, tB, tC, trunc);
    limb::Args g;
    memset(&g, 0, sizeof(g));
    g.M = M; g.N = N; g.Kseg = K; g.kind = limb::KIND_GEMM; g.tA = tA; g.tC = tC;
    limb_segments(g, a);
    for (int i = 0; i < 6; i++) { g.out[i] = out[i]; g.bias[i] = bias ? bias[i] : nullptr; }
    g.d = 1ull << trunc;
    g.dshift = pow2_shift<uint64_t>(g.d);
    int st = limb_launch(c, g, tB, b);
    if (st) return st;
    comm_msg(c, 2ull * M * N * 8, 2ull * M * N * 8);
    comm_round(c);
    return PG_OK;
}

int limb_rss_conv_u64(Ctx *c, const uint64_t *const A[6], const uint64_t *const B[6], uint64_t *const C[6], int op,
                      int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    CSh6<uint64_t> ca, cb;
    Sh6<uint64_t> co;
    if (!load6(ca, A) || !load6(cb, B) || !load6(co, C)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    bool ok = op == PG_CONV_FPROP && (Din % 16) == 0;
    for (int i = 0; i < 6 && ok; i++) ok = aligned16(A[i]) && aligned16(B[i]);
    if (!ok || batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Dout <= 0 || stride <= 0 || pad < 0 || H + 2 * pad < f ||
        W + 2 * pad < f)
        return rss_conv<uint64_t>(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc);
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    limb::Args g;
    memset(&g, 0, sizeof(g));
    int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    g.M = batch * P * Q; g.N = Dout; g.Kseg = f * f * Din; g.kind = limb::KIND_FPROP; g.tC = 1;
    g.ch = H; g.cw = W; g.cc = Din; g.cs = f; g.cp = P; g.cq = Q; g.pad = pad; g.stride = stride;
    g.dQ.init(Q); g.dP.init(P); g.dC.init(Din); g.dS.init(f);
    limb_segments(g, A);
    for (int i = 0; i < 6; i++) { g.out[i] = C[i]; g.bias[i] = nullptr; }
    g.d = 1ull << trunc;
    g.dshift = pow2_shift<uint64_t>(g.d);
    int st = limb_launch(c, g, 0, B);
    if (st) return st;
    uint64_t n_out = (uint64_t)g.M * g.N;
    comm_msg(c, 2 * n_out * 8, 2 * n_out * 8);
    comm_round(c);
    return PG_OK;
}

int limb_selftest(Ctx *c, const uint16_t *A, const uint16_t *B, float *D) {
    if (!A || !B || !D) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    limb::selftest_kernel<<<1, 128, 0, c->stream>>>(A, B, D, device_error_word(c));
    c->launches++;
    return launch_status(c, "selftest_kernel");
}

// ------------------------------------------------ fixed-scratch share-GEMM

// Raise the GEMM kernel's dynamic shared-memory limit on the current device.
int limb_prepare_current_device(Ctx *c) {
    PG_CHECK_CUDA(c, cudaFuncSetAttribute(limb::limb_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)limb::smem_bytes()));
    return PG_OK;
}

// The limb-form RSS share-GEMM of limb_rss_matmul_u64 (no bias), with every
// scratch byte taken from [scr, scr + cap) instead of the context's scratch.
// It allocates nothing. Split-K is used only when its partial sums fit too;
// a problem whose unsplit need exceeds cap is refused with PG_ERR_SIZE, and
// shapes the limb tiles do not cover with PG_ERR_UNSUPPORTED. The column
// sums are zeroed on the stream before use; the packed weights and the
// partial sums are written in full by their producers before they are read.
int limb_rss_matmul_u64_fixed(Ctx *c, uint8_t *scr, size_t cap, const uint64_t *const a[6],
                              const uint64_t *const b[6], uint64_t *const out[6], int M, int N, int K, int tA, int tB,
                              int tC, int trunc) {
    using namespace limb;
    CSh6<uint64_t> ca, cb;
    Sh6<uint64_t> co;
    if (!load6(ca, a) || !load6(cb, b) || !load6(co, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    if (K % BK) return set_error(c, PG_ERR_UNSUPPORTED, "K = %d is not a multiple of %d", K, BK);
    for (int i = 0; i < 6; i++)
        if (!aligned16(a[i]) || !aligned16(b[i]))
            return set_error(c, PG_ERR_UNSUPPORTED, "share pointers must be 16-byte aligned");
    if (!scr || ((uintptr_t)scr & 255)) return set_error(c, PG_ERR_INVALID_ARG, "scratch must be 256-byte aligned");

    Args g;
    memset(&g, 0, sizeof(g));
    g.M = M; g.N = N; g.Kseg = K; g.kind = KIND_GEMM; g.tA = tA; g.tC = tC;
    limb_segments(g, a);
    for (int i = 0; i < 6; i++) { g.out[i] = out[i]; g.bias[i] = nullptr; }
    g.d = 1ull << trunc;
    g.dshift = pow2_shift<uint64_t>(g.d);

    const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
    const int tiles = tiles_m * tiles_n;
    g.ntiles_n = tiles_n;
    g.kblocks = K / BK;
    const int total_stages = 6 * g.kblocks;
    const int chunks = (total_stages + CHUNK_STAGES - 1) / CHUNK_STAGES;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t pack_bytes = (size_t)total_stages * tiles_n * B_STAGE_BYTES;
    auto need = [&](int split) {
        return pack_bytes + al((size_t)split * tiles_n * BN * 8) + (split > 1 ? (size_t)split * M * N * 8 : 0);
    };
    int split = tiles >= sms ? 1 : sms / tiles;
    if (split > chunks) split = chunks;
    if (split < 1) split = 1;
    int cps = (chunks + split - 1) / split;
    split = (chunks + cps - 1) / cps;
    if (need(split) > cap) {
        split = 1;
        cps = chunks;
    }
    if (need(split) > cap)
        return set_error(c, PG_ERR_SIZE,
                         "M=%d N=%d K=%d needs %zu bytes of scratch; the fixed scratch holds %zu (the packed "
                         "weights alone take 96 * K * (N rounded up to 64) bytes)",
                         M, N, K, need(split), cap);
    g.total_stages = total_stages;
    g.chunks_per_split = cps;
    g.err = device_error_word(c);
    const size_t col_bytes = al((size_t)split * tiles_n * BN * 8);
    uint64_t *colsum = (uint64_t *)(scr + pack_bytes);
    g.packB = scr;
    g.colsum = colsum;
    PG_CHECK_CUDA(c, cudaMemsetAsync((void *)colsum, 0, col_bytes, c->stream));
    {
        PackArgs pa;
        memset(&pa, 0, sizeof(pa));
        for (int i = 0; i < 6; i++) pa.b[i] = b[i];
        pa.N = N; pa.Kseg = K; pa.ntiles_n = tiles_n; pa.kblocks = g.kblocks; pa.tB = tB; pa.kind = KIND_GEMM;
        pa.stages_per_split = cps * CHUNK_STAGES;
        pa.packB = scr;
        pa.colsum = colsum;
        size_t units = (size_t)6 * tiles_n * BN * g.kblocks * 2;
        unsigned blocks = (unsigned)((units + 255) / 256);
        if (blocks > (unsigned)sms * 16) blocks = sms * 16;
        pack_b_kernel<<<blocks, 256, 0, c->stream>>>(pa);
        c->launches++;
        int st = launch_status(c, "pack_b_kernel");
        if (st) return st;
    }
    g.direct = split > 1 ? 0 : 1;
    if (split > 1) g.partial = (uint64_t *)(scr + pack_bytes + col_bytes);
    dim3 grid(tiles_n, tiles_m, split);
    limb_gemm_kernel<<<grid, NTHREADS, smem_bytes(), c->stream>>>(g);
    c->launches++;
    int st = launch_status(c, "limb_gemm_kernel");
    if (st) return st;
    if (split > 1) {
        size_t total = (size_t)M * N;
        unsigned blocks = (unsigned)((total + 255) / 256);
        if (blocks > (unsigned)sms * 8) blocks = sms * 8;
        limb_reduce_kernel<<<blocks, 256, 0, c->stream>>>(g, split);
        c->launches++;
        st = launch_status(c, "limb_reduce_kernel");
        if (st) return st;
    }
    comm_msg(c, 2ull * M * N * 8, 2ull * M * N * 8);
    comm_round(c);
    return PG_OK;
}

}  // namespace pg
