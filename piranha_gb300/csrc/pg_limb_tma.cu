// pg_limb_tma.cu — the 8-bit-limb tensor-core RSS share-GEMM and implicit
// convolution, fed by TMA (tcgen05, fp16 digits, fp32 accumulators in tensor
// memory), exact modulo 2^64.
//
// Digits. Every 64-bit operand v is written with eight signed digits
//   e_i = byte_i(v + 0x8080808080808080) - 128  in [-128, 127],
// for which v = sum_i e_i 2^(8i) (mod 2^64) holds exactly (adding 128 to
// every byte and removing it again digit by digit leaves the value). So a
// contraction over K' terms is
//   sum_k a_k b_k = sum_s 2^(8s) D_s (mod 2^64),  D_s = sum_{i+j=s} sum_k e_i(a_k) e_j(b_k),
// with no correction terms, and only the 36 digit pairs with i+j < 8 matter.
// The value 0 has all digits 0, so zero padding (tensor-map out-of-bounds
// fill, ragged tiles) stands for the value 0. A digit product is at most 2^14
// in magnitude; diagonals 4-7 have at most 8 pairs and are drained every
// 128 K', diagonals 0-3 at most 4 pairs and are drained every 256 K', so
// every partial sum is an integer of magnitude <= 2^24, exact in fp32.
//
// Operands. A (activations, or the GEMM's left operand) is first written by
// image_kernel as an image of digit planes in global memory,
//   img[seg][plane][C/8][pixel][8]  (fp16),
// so that for a tile of output pixels and one conv tap, the 16 channels of a
// K block in all eight digit planes are one 5-D tensor-map box: (8 channels
// x Wt pixels, as one contiguous line of 16*Wt bytes) x Ht rows x Nt images
// x 2 channel groups x 8 planes, one copy per stage.
// A tap is a shift of the box (16 bytes per pixel along the line), and
// padding is the box running out of bounds. The GEMM case reads lines of 32
// consecutive image rows instead. B (weights, with
// y_p0 + y_p1 precomputed) is packed once by pack_kernel into the exact
// shared-memory stage image and streamed with bulk async copies.
//
// Protocol. The K' dimension concatenates the six RSS segments
// [x_p0 | x_p1] x [y_p0 + y_p1 ; y_p0] of the three parties (localMatMul,
// src/mpc/RSS.inl:1097-1110; localFprop :614-639); the epilogue truncates
// Z = sum_p z_p with dividePublic3out3 (:1077-1094).
//
// Roles (384 threads): warp 0 issues the TMA and bulk copies of each stage,
// warp 1 owns tensor memory and one lane issues the MMAs of diagonals 0-3,
// one lane of warp 2 issues those of diagonals 4-7, warp 3 is spare, warps
// 4-11 drain the accumulators (two warps per 32-lane quarter, 32 columns
// each) and run the epilogue; warpgroup 0 hands most of its registers to
// them (setmaxnreg). Each output tile makes one pass over K' with all eight digit
// diagonals in tensor memory (8 x 64 columns) in two groups, diagonals 0-3
// and 4-7, whose drains into 64-bit registers are staggered: while the
// epilogue drains one group, the other group's MMA warp runs ahead over the
// stages already loaded. A stage is released when both MMA warps have
// committed it (the empty barrier counts two arrivals); the low group's
// issuer trails the high group's by a stage (the issue lag). The grid is one
// CTA per SM: each walks a host-balanced list of work items (an output tile
// and its K' slice), with the ring and chunk counts running on across them,
// and stores a tile's output from the epilogue registers while the next
// tile's copies and MMAs run. Every mbarrier wait is bounded; on a timeout
// the kernel records an error word, stops issuing, waits for its own copies
// and MMAs, and frees tensor memory.
//
// Replicated sharings. Where the six share buffers hold one (party p's
// second share equal to party p+1's first), the image stores each share once
// (three blocks of digit planes) and segment s is read from block
// ((s + 1) / 2) mod 3.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <functional>
#include <vector>
#include <cstring>
#include <memory>
#include <mutex>
#include <unordered_map>

#include "pg_common.cuh"
#include "pg_limb_tma.cuh"
#include "pg_relu_value.cuh"
#include "pg_tcgen05.cuh"

namespace pg {
int *device_error_word(Ctx *c);
namespace lt {

constexpr int BM = 128, BN = 64, BK = 16, STAGES = 4;
// Accumulator drains: diagonals 4-7 (up to 8 pairs) every 128 K', diagonals
// 0-3 (up to 4 pairs) every 256 K', with the low group's boundaries falling
// between the high group's (its first chunk is 192 K').
constexpr int CHUNK_STAGES = 8;     // high group, and the split-K granule
constexpr int CHUNK_STAGES_LO = 16;
constexpr int LO_FIRST = 12;
constexpr int A_PLANE_BYTES = BM * BK * 2;                      // 4096
constexpr int B_PLANE_BYTES = BN * BK * 2;                      // 2048
constexpr int B_STAGE_BYTES = 8 * B_PLANE_BYTES;                // 16384
constexpr int STAGE_BYTES = 8 * A_PLANE_BYTES + B_STAGE_BYTES;  // 49152
// Warp roles: warpgroup 0 = the copy producer, the two MMA issuers and one
// spare warp; warpgroups 1-2 = the eight drain / epilogue warps (warp w reads
// tensor-memory lanes 32 * (w % 4), so each lane quarter has two of them).
constexpr int NTHREADS = 384;
constexpr int W_PROD = 0, W_MMA = 1, W_MMA2 = 2, W_EPI0 = 4;
// Register split (setmaxnreg): the block is launched at REGS_LAUNCH per thread
// (the most that 3 warps on each SM sub-partition allow); warpgroup 0 gives
// registers back down to REGS_CTRL and the epilogue warpgroups take them up to
// REGS_EPI, enough to hold a group's four accumulators (4 x 32 values) beside
// the 32 running 64-bit sums, so that tensor memory is handed back to the
// MMA warp before any of them is converted. The split must add up to the
// launch's registers, or the increase would wait forever; the host checks the
// kernel's register count against REGS_LAUNCH before the first launch.
constexpr int REGS_LAUNCH = 168, REGS_CTRL = 56, REGS_EPI = 224;
static_assert(4 * 32 * REGS_CTRL + 8 * 32 * REGS_EPI <= NTHREADS * REGS_LAUNCH, "register split over the launch");
static_assert(3 * REGS_LAUNCH * 32 <= 16384 && REGS_CTRL + 2 * REGS_EPI <= 512,
              "three warps per sub-partition at launch; one control and two epilogue warps after the split");
constexpr uint32_t TMEM_COLS = 512;  // 8 diagonals x 64 columns
constexpr uint64_t DIGIT_OFFSET = 0x8080808080808080ull;
constexpr uint64_t WAIT_NS = 2000000000ull;  // 2 s bound on any single wait (the context can set a shorter one)

struct Args {
    int M, N;
    int kblocks, cblocks, C8, f, pad;
    int Wt, Ht, Nt, R, tiles_w, tiles_h, P, Q, Nimg;
    int Himg, Wimg;
    int rows_mode;  // 1: the image holds one row per output row (GEMM, im2col)
    int ntiles_n, total_stages, chunks_per_split;
    int tiles_m, nsplit, n_items;  // row tiles; K' slices; work items (ntiles_n x tiles_m x nsplit)
    int direct, colmajor;
    int posmajor;  // tiles by output position (Plan::posmajor); H, W: input extents then
    int wgt;       // implicit weight gradient (Plan::wgt): a tile is 128 input channels of one filter tap
    int cdim, nb16;  // wgt: input channels, images / 16
    int zeros_kept;  // the four zero output shares already hold 0: write only value / bias shares
    int tma_out;     // the two value shares go out as tensor-map stores of the staged tile (see tma_store_4d)
    uint32_t a_box_bytes;  // bytes of one digit plane of a stage (16 * 2 * Wt * Ht * Nt)
    const uint8_t *packB;
    uint64_t *partial;
    uint64_t *raw;  // non-null: write the untruncated Z (row-major M x N) here instead of output shares
    uint64_t *out[6];
    const uint64_t *bias[6];
    uint64_t d;
    int dshift;
    int *err;
    uint64_t wait_ns;  // bound on every wait of the kernel
    int withhold;      // diagnostic: K stage (of each CTA's range) whose copies the producer never issues; -1: none
    int lag;           // the low group's issuer issues stage t once the high group's has issued stage t + lag
    int order;         // 1: narrow and wide MMAs interleaved within a group's stage (issue_lo / issue_hi)
    int seg_block[6];  // digit-plane block of the image holding each K segment (the identity, or 0,1,1,2,2,0
                       // for an image of a replicated sharing stored once per share)
    const int *rep_flag;  // non-null: the blocks 0,1,1,2,2,0 when the device word is set (the image's layout)
};

struct __align__(16) Smem {
    uint8_t stage[STAGES][STAGE_BYTES];
    Args args;
    uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], done;  // [0] low group, [1] high group
    uint32_t tmem_base;
    int abort;
    int never;      // stays 0: a wait that must not be cut short by the abort flag
    int hi_issued;  // stages whose MMAs the high group's issuer has issued
    int gsel;       // the accumulator group whose chunk the epilogue drains next (-1: stop)
};

static size_t smem_bytes() { return sizeof(Smem) + 1024; }

// ------------------------------------------------------------------ digits

// fp16 digits of byte b of two words, packed in one half2 word:
// low half from x, high half from y, each (1024 + byte) - 1152 = byte - 128.
__device__ __forceinline__ uint32_t digit_pair(uint32_t x, uint32_t y, uint32_t b) {
    const uint32_t sel = b | (b << 4) | ((4 + b) << 8) | ((4 + b) << 12);
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(x), "r"(y), "r"(sel));
    d = (d & 0x00FF00FFu) | 0x64006400u;
    __half2 h = *reinterpret_cast<__half2 *>(&d);
    h = __hsub2(h, __halves2half2(__ushort_as_half(0x6480), __ushort_as_half(0x6480)));
    return *reinterpret_cast<uint32_t *>(&h);
}

// The digit planes (8 fp16 each, one uint4 per plane) of 8 values.
template <int NPL>
__device__ __forceinline__ void digits8(const uint64_t (&v)[8], uint4 (&pl)[NPL]) {
    uint32_t lo[8], hi[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint64_t u = v[k] + DIGIT_OFFSET;
        lo[k] = (uint32_t)u;
        hi[k] = (uint32_t)(u >> 32);
    }
#pragma unroll
    for (int i = 0; i < NPL; i++) {
        uint32_t w[4];
#pragma unroll
        for (int p = 0; p < 4; p++)
            w[p] = i < 4 ? digit_pair(lo[2 * p], lo[2 * p + 1], (uint32_t)(i & 3))
                         : digit_pair(hi[2 * p], hi[2 * p + 1], (uint32_t)(i & 3));
        pl[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// ------------------------------------------------------------ image kernel

enum { SRC_ROWS = 0, SRC_COLS = 1, SRC_IM2COL = 2, SRC_WGRAD = 3, SRC_WGRAD_T = 4 };

struct ImageArgs {
    const uint64_t *a[6];
    int mode;
    long long pixels;  // image rows written (source rows, then zero rows up to a whole line)
    long long pixels_src;  // image rows that come from A
    int C8;            // image channel groups of 8
    int Kreal;         // values at k >= Kreal are 0
    long long ld;      // ROWS: row stride; COLS: column stride
    int vec;           // ROWS: rows are 16-byte aligned and Kreal is a multiple of 8
    int H, W, Din, f, stride, pad, P, Q;
    long long bi_n, bi_hw;  // ROWS, batch-innermost image: image row (h * W + w) * bi_n + n holds source row
                            // n * bi_hw + h * W + w (bi_n = 0: image row = source row)
    int nseg;               // 6: a block per share buffer; 3: block b from party b's first share (a
                            // replicated sharing stored once per share, run_image's shared flag)
    const int *rep_flag;    // non-null: 3 blocks when the device word is set (checked on the device)
    uint4 *img;
};

// One thread per (segment, pair of 8-channel groups, pixel); consecutive
// threads take consecutive pixels, so the plane stores are coalesced, and a
// thread reads its 16 channels of a row as one whole 128-byte line (with one
// group per thread each line was fetched twice from DRAM). C8 is even (the
// image's channels are a multiple of 16).
__global__ void image_kernel(const __grid_constant__ ImageArgs ia) {
    const int C16 = ia.C8 >> 1;
    const int nseg = ia.rep_flag && *ia.rep_flag ? 3 : ia.nseg;
    const long long total = (long long)nseg * C16 * ia.pixels;
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < total;
         u += (long long)gridDim.x * blockDim.x)
#pragma unroll 1
    for (int half = 0; half < 2; half++) {
        const long long pix = u % ia.pixels;
        const long long t = u / ia.pixels;
        const int cb = 2 * (int)(t % C16) + half;
        const int seg = (int)(t / C16);
        const uint64_t *a = ia.a[nseg == 3 ? 2 * seg : seg];
        const int k0 = cb * 8;
        uint64_t v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = 0;
        if (pix >= ia.pixels_src) {
            // zero row padding the image to whole lines
        } else if (ia.mode == SRC_ROWS) {
            const long long srow = ia.bi_n ? (pix % ia.bi_n) * ia.bi_hw + pix / ia.bi_n : pix;
            const uint64_t *src = a + srow * ia.ld + k0;
            if (ia.vec && k0 < ia.Kreal) {
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const ulonglong2 q = __ldg(reinterpret_cast<const ulonglong2 *>(src) + i);
                    v[2 * i] = q.x;
                    v[2 * i + 1] = q.y;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++)
                    if (k0 + i < ia.Kreal) v[i] = __ldg(src + i);
            }
        } else if (ia.mode == SRC_WGRAD) {
            // weight gradient: row pix = (r, s, c) of the filter, K index k =
            // (n, p, q) of an output pixel, value = the forward input at
            // (n, p*stride - pad + r, q*stride - pad + s, c)
            const int c = (int)(pix % ia.Din);
            const int rs = (int)(pix / ia.Din);
            const int s = rs % ia.f, r = rs / ia.f;
            int q = k0 % ia.Q;
            const int np = k0 / ia.Q;
            int p = np % ia.P;
            long long n = np / ia.P;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                if (k0 + i < ia.Kreal) {
                    const int h = p * ia.stride - ia.pad + r, w = q * ia.stride - ia.pad + s;
                    if (h >= 0 && h < ia.H && w >= 0 && w < ia.W)
                        v[i] = __ldg(a + ((n * ia.H + h) * ia.W + w) * (long long)ia.Din + c);
                }
                if (++q == ia.Q) {
                    q = 0;
                    if (++p == ia.P) {
                        p = 0;
                        ++n;
                    }
                }
            }
        } else if (ia.mode == SRC_COLS) {
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (k0 + i < ia.Kreal) v[i] = __ldg(a + (long long)(k0 + i) * ia.ld + pix);
        } else {
            const int q = (int)(pix % ia.Q);
            const long long np = pix / ia.Q;
            const int p = (int)(np % ia.P);
            const long long n = np / ia.P;
            // k = (r * f + s) * Din + c, split once and then carried
            int c = k0 % ia.Din;
            const int rs = k0 / ia.Din;
            int s = rs % ia.f, r = rs / ia.f;
            const int h0 = p * ia.stride - ia.pad, w0 = q * ia.stride - ia.pad;
            const uint64_t *img0 = a + n * ia.H * ia.W * (long long)ia.Din;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                if (k0 + i < ia.Kreal) {
                    const int h = h0 + r, w = w0 + s;
                    if (h >= 0 && h < ia.H && w >= 0 && w < ia.W)
                        v[i] = __ldg(img0 + ((long long)h * ia.W + w) * ia.Din + c);
                }
                if (++c == ia.Din) {
                    c = 0;
                    if (++s == ia.f) {
                        s = 0;
                        ++r;
                    }
                }
            }
        }
        uint4 pl[8];
        digits8<8>(v, pl);
#pragma unroll
        for (int i = 0; i < 8; i++) ia.img[((long long)(seg * 8 + i) * ia.C8 + cb) * ia.pixels + pix] = pl[i];
    }
}

// The digit image of the implicit weight gradient: the forward input X
// (NHWC, batch x HW pixels x C channels) as img[seg][plane][pixel][n / 8][c][n % 8],
// so that 8 consecutive images of one channel are one 16-byte core row and a
// filter tap is a shift of the pixel coordinate. One thread per (segment,
// pixel, 8-image block, channel): consecutive threads take consecutive
// channels (coalesced reads of each image's row, coalesced 16-byte writes).
struct WgtImageArgs {
    const uint64_t *a[6];
    long long hw, nb8, cdim;  // cdim: image channels (>= the input's, zero past it)
    int din;                  // the input's channels
    int nseg;                 // 6 or 3 plane blocks (see ImageArgs)
    uint4 *img;
};

__global__ void wgt_image_kernel(const __grid_constant__ WgtImageArgs ia) {
    const long long per_seg = ia.hw * ia.nb8 * ia.cdim;
    const long long total = ia.nseg * per_seg;
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < total;
         u += (long long)gridDim.x * blockDim.x) {
        const long long c = u % ia.cdim;
        long long t = u / ia.cdim;
        const long long nb = t % ia.nb8;
        t /= ia.nb8;
        const long long pix = t % ia.hw;
        const int seg = (int)(t / ia.hw);
        const uint64_t *a = ia.a[ia.nseg == 3 ? 2 * seg : seg];
        uint64_t v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = c < ia.din ? __ldg(a + ((nb * 8 + i) * ia.hw + pix) * ia.din + c) : 0;
        uint4 pl[8];
        digits8<8>(v, pl);
#pragma unroll
        for (int i = 0; i < 8; i++) ia.img[(long long)(seg * 8 + i) * per_seg + (pix * ia.nb8 + nb) * ia.cdim + c] = pl[i];
    }
}

// ReLU fused with the digit image of the convolution it feeds: a block of
// 256 threads takes 16 pixels x 16 channels (one 128-byte line of each
// share per pixel). Each thread runs the ReLU of one value (dReLU +
// selectShare, RSS.inl:807-865, all three parties) and writes the layer's
// shares and bit shares; then 192 threads turn the block's 16 pixels x 2
// channel groups x 6 shares into the next convolution's fp16 digit planes,
// consecutive threads on consecutive pixels. The image launch and its
// re-read of the ReLU output are saved. With out[0] null the ReLU output is
// kept in the digit image alone (image_decode_kernel restores the shares),
// with dout[k] null bit share k is not written.
struct ReluImageArgs {
    const uint64_t *in[6];
    uint64_t *out[6];
    uint8_t *dout[6];
    uint4 *img;
    long long pixels, pixels_alloc;
    int C8;
    long long bi_n, bi_hw;  // batch-innermost image (see ImageArgs); 0: image pixel = NHWC pixel
    int nseg;               // 6 or 3 plane blocks (see ImageArgs)
    int zmid;               // shares 1-4 of the input are 0 (Ctx::in_zero_mid): not read
};

constexpr int RI_PIX = 16, RI_CH = 16, RI_PITCH = RI_PIX + 1;  // pitch 17: two-way bank conflicts at most

// ZM: a.zmid (shares 1-4 of the input are 0, not read) as a compile-time fact;
// RELU = false: no ReLU, the digit image of the input itself (run_image's
// rows of a position-major image, whose consecutive image rows are rows of
// different images: read here as whole 128-byte lines of a row), and with
// three plane blocks only shares 0, 2 and 4 are read. At most 40 registers,
// so that six blocks of 256 threads fit on an SM.
template <bool ZM, bool RELU>
__global__ void __launch_bounds__(256, 6) relu_image_kernel(const __grid_constant__ ReluImageArgs a) {
    // two staging buffers, alternating by round: a round's ReLU writes one
    // while nothing reads it (the other round's digit phase reads the other),
    // so one barrier per tile suffices
    __shared__ uint64_t zbuf[2][6][RI_CH][RI_PITCH];
    // 32-bit tile and pixel arithmetic (relu_image_fits keeps both below 2^31)
    const uint32_t C16 = (uint32_t)(a.C8 >> 1);
    const uint64_t C = 8ull * a.C8;
    const uint32_t pixels = (uint32_t)a.pixels;
    const uint32_t tiles = (pixels + RI_PIX - 1) / RI_PIX * C16;
    const uint32_t bi_n = (uint32_t)a.bi_n, bi_hw = (uint32_t)a.bi_hw;
    const int t = threadIdx.x;
    int round = 0;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x, round ^= 1) {
        uint64_t (*zs)[RI_CH][RI_PITCH] = zbuf[round];
        const uint32_t pt = tile / C16;
        const uint32_t cp = tile - pt * C16;
        const uint32_t p0 = pt * RI_PIX;
        {
            const int pl = t / RI_CH, ch = t % RI_CH;
            const uint32_t pix = p0 + pl;
            uint64_t z[3][2];
            if (pix < pixels) {
                uint32_t src = pix;
                if (bi_n) {
                    const uint32_t n = pix / bi_n;
                    src = (pix - n * bi_n) * bi_hw + n;
                }
                const uint64_t idx = src * C + cp * RI_CH + ch;
                uint64_t x[3][2], zero[3][2];
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    const bool skip = (ZM && k > 0 && k < 5) || (!RELU && a.nseg == 3 && (k & 1));
                    x[k >> 1][k & 1] = skip ? 0 : __ldg(a.in[k] + idx);
                    zero[k >> 1][k & 1] = 0;
                }
                if constexpr (RELU) {
                    uint8_t r[3][2];
                    drelu_value<uint64_t, uint8_t>(x, r);
                    select_value<uint64_t, uint8_t>(zero, x, r, z);
#pragma unroll
                    for (int k = 0; k < 6; k++) {
                        if (a.out[0]) a.out[k][idx] = z[k >> 1][k & 1];
                        if (a.dout[k]) a.dout[k][idx] = r[k >> 1][k & 1];
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < 6; k++) z[k >> 1][k & 1] = x[k >> 1][k & 1];
                }
            } else {
#pragma unroll
                for (int k = 0; k < 6; k++) z[k >> 1][k & 1] = 0;
            }
#pragma unroll
            for (int k = 0; k < 6; k++) zs[k][ch][pl] = z[k >> 1][k & 1];
        }
        __syncthreads();
        if (t < a.nseg * 2 * RI_PIX) {
            const int seg = t / (2 * RI_PIX), half = (t / RI_PIX) & 1, pl = t % RI_PIX;
            const int sh = a.nseg == 3 ? 2 * seg : seg;
            const uint32_t pix = p0 + pl;
            if (pix < pixels) {
                uint64_t v[8];
#pragma unroll
                for (int i = 0; i < 8; i++) v[i] = zs[sh][half * 8 + i][pl];
                uint4 plv[8];
                digits8<8>(v, plv);
                const int cb = 2 * cp + half;
#pragma unroll
                for (int i = 0; i < 8; i++)
                    a.img[((long long)(seg * 8 + i) * a.C8 + cb) * a.pixels_alloc + pix] = plv[i];
            }
        }
        // no barrier here: the next round writes the other buffer, and the
        // round after it passes the next round's barrier first, which every
        // thread reaches only after this digit phase
    }
}

// The inverse of relu_image_kernel's image: the six u64 shares of every
// (NHWC pixel, channel) value rebuilt from its eight fp16 digit planes,
// v = sum_i (digit_i + 128) * 2^(8 i) - DIGIT_OFFSET. With three plane blocks
// (a replicated sharing, block b = share 2b) share s is block ((s + 1) / 2) % 3.
// One thread per (value, share); not on the forward's path (it serves reads
// of a layer output that the forward kept as a digit image).
struct ImageDecodeArgs {
    const uint4 *img;
    uint64_t *out[6];
    long long pixels, pixels_alloc;
    int C8, nseg;
    long long bi_n, bi_hw;  // batch-innermost image (see ReluImageArgs)
};

__global__ void image_decode_kernel(const __grid_constant__ ImageDecodeArgs a) {
    const long long C = 8ll * a.C8;
    const long long total = 6 * a.pixels * C;
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < total;
         u += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(u / (a.pixels * C));
        const long long idx = u - (long long)k * a.pixels * C;  // NHWC value index
        const long long src = idx / C;
        const int ch = (int)(idx - src * C);
        const long long pix = a.bi_n ? (src % a.bi_hw) * a.bi_n + src / a.bi_hw : src;
        const int seg = a.nseg == 3 ? ((k + 1) / 2) % 3 : k;
        const __half *pl = reinterpret_cast<const __half *>(a.img);
        uint64_t u64 = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const long long at = (((long long)(seg * 8 + i) * a.C8 + ch / 8) * a.pixels_alloc + pix) * 8 + ch % 8;
            const int digit = (int)__half2float(pl[at]);
            u64 |= (uint64_t)(uint32_t)(digit + 128) << (8 * i);
        }
        a.out[k][idx] = u64 - DIGIT_OFFSET;
    }
}

// ------------------------------------------------------------- B packing

struct PackArgs {
    const uint64_t *b[6];
    int N, Kreal, kblocks, ntiles_n;
    int kn;  // 1: b[k * N + n]; 0: b[n * Kreal + k]
    long long wg_pq;  // > 0: K index k = pixel * wg_batch + image of b = dY[image][pixel][n] (wg_pq pixels)
    int wg_batch;
    int cpad, creal;  // cpad > 0: K index k = tap * cpad + c of the channel-padded image, b's k = tap * creal + c
    int flip_f;       // > 0: K index k = tap * cpad + kk (kk < creal), column n: b = W[kk][f-1-r][f-1-s][n], N = Din
    uint8_t *packB;
};

// core-matrix offset of (row, 8-element K chunk kc) inside a B digit plane:
// 8 rows x 16 bytes per core matrix, K-adjacent core matrices 128 bytes
// apart, 8-row groups 256 bytes apart
__host__ __device__ __forceinline__ uint32_t b_off(int row, int kc) {
    return (uint32_t)((row >> 3) * 256 + kc * 128 + (row & 7) * 16);
}

// One thread per (party, K block, N tile, column, chunk of 8), with the
// chunk and then the column varying fastest: a warp writes 512 contiguous
// bytes of a digit plane (16 columns x both 8-element chunks) and reads runs
// of consecutive columns (b[k * N + n]) or of consecutive k (b[n * K + k]).
// Segment 2p holds y_p0 + y_p1 and segment 2p+1 holds y_p0 of party p; the
// thread reads each of the party's two shares once and writes both segments.
__global__ void pack_kernel(const __grid_constant__ PackArgs pa) {
    const long long total = 3ll * pa.kblocks * pa.ntiles_n * BN * 2;
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < total;
         u += (long long)gridDim.x * blockDim.x) {
        const int kc = (int)(u & 1);
        const int row = (int)((u >> 1) % BN);
        long long t = (u >> 1) / BN;
        const int nt = (int)(t % pa.ntiles_n);
        t /= pa.ntiles_n;
        const int kb = (int)(t % pa.kblocks);
        const int p = (int)(t / pa.kblocks);
        const int n = nt * BN + row;
        const int k0 = kb * BK + kc * 8;
        uint64_t v0[8], v1[8];  // y_p0, y_p1
#pragma unroll
        for (int i = 0; i < 8; i++) v0[i] = v1[i] = 0;
        if (n < pa.N) {
            const uint64_t *b0 = pa.b[2 * p], *b1 = pa.b[2 * p + 1];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                int k = k0 + i;
                long long idx = -1;
                if (pa.flip_f) {
                    const int tap = k / pa.cpad, kk = k - tap * pa.cpad;
                    if (kk < pa.creal && tap < pa.flip_f * pa.flip_f) {
                        const int r = tap / pa.flip_f, sx = tap - r * pa.flip_f;
                        idx = ((long long)(kk * pa.flip_f + (pa.flip_f - 1 - r)) * pa.flip_f + (pa.flip_f - 1 - sx)) *
                                  pa.N + n;
                    }
                } else {
                    if (pa.cpad) {
                        const int tap = k / pa.cpad, ch = k - tap * pa.cpad;
                        k = ch < pa.creal ? tap * pa.creal + ch : pa.Kreal;  // padding channels: 0
                    }
                    if (k < pa.Kreal) {
                        idx = pa.kn ? (long long)k * pa.N + n : (long long)n * pa.Kreal + k;
                        if (pa.wg_pq) idx = ((long long)(k % pa.wg_batch) * pa.wg_pq + k / pa.wg_batch) * pa.N + n;
                    }
                }
                if (idx >= 0) {
                    v0[i] = __ldg(b0 + idx);
                    v1[i] = __ldg(b1 + idx);
                }
            }
        }
        uint4 pl[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v1[i] += v0[i];
        digits8<8>(v1, pl);  // segment 2p: y_p0 + y_p1
        uint8_t *dst = pa.packB + (((long long)(2 * p) * pa.kblocks + kb) * pa.ntiles_n + nt) * B_STAGE_BYTES;
#pragma unroll
        for (int i = 0; i < 8; i++)
            *reinterpret_cast<uint4 *>(dst + i * B_PLANE_BYTES + b_off(row, kc)) = pl[i];
        digits8<8>(v0, pl);  // segment 2p + 1: y_p0
        dst = pa.packB + (((long long)(2 * p + 1) * pa.kblocks + kb) * pa.ntiles_n + nt) * B_STAGE_BYTES;
#pragma unroll
        for (int i = 0; i < 8; i++)
            *reinterpret_cast<uint4 *>(dst + i * B_PLANE_BYTES + b_off(row, kc)) = pl[i];
    }
}

// ------------------------------------------------------------- GEMM kernel

// One 5-D box: all eight digit planes of a stage's A tile in one copy.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void flag_error(Smem &sm, const Args &g, int code) {
    sm.abort = 1;
    if (g.err) atomicCAS(g.err, 0, code);
}

// The low group's issuer trails the high group's: it issues stage t only
// once the high one has issued stage t + lag (both run one thread of
// warpgroup 0). Then, while the high group waits for its accumulators to be
// drained, the tensor pipe still holds the low group's MMAs of the stages
// the high one has already passed, instead of running dry. A lag below the
// ring depth cannot deadlock: the high issuer's stages up to t + lag are
// loaded once the low one has released stage t + lag - STAGES < t. Bounded,
// and cut short by the abort flag.
__device__ __forceinline__ bool wait_issued(Smem &sm, int need, uint64_t limit_ns) {
    const volatile int *hi = &sm.hi_issued;
    if (*hi >= need) return true;
    const uint64_t t0 = tc::globaltimer();
    for (uint32_t it = 1;; it++) {
        if (*hi >= need) return true;
        if ((it & 63) == 0) {
            if (*reinterpret_cast<volatile int *>(&sm.abort)) return false;
            if (tc::globaltimer() - t0 > limit_ns) return false;
        }
    }
}

// The MMAs of one stage for the low diagonals 0-3 (columns 0-255): for A
// digit plane i < 4 the B planes j = 0..3-i are adjacent in shared memory and
// their products go to the adjacent accumulators of diagonals i..3, so one
// MMA with N = 64 (4 - i) covers them. i = 0 writes all four accumulators,
// so it comes first (it resets them at a chunk's first stage).
// ORDER 1 issues the narrow MMAs between the wide ones (low: N = 256, 64,
// 192, 128; high: 256, 64, 256, 128, 256, 192, 256, 256): a narrow MMA reads
// more shared memory per tensor-pipe cycle than a wide one, and interleaved
// they keep both busy (measured on the GB300: 1362 -> 1256 cycles per stage
// for the stage mix without drains, 1574 -> 1525 with them).
template <int ORDER>
__device__ __forceinline__ void issue_lo(uint32_t acc, uint64_t adesc, uint32_t aplane16, uint64_t bdesc,
                                         bool first_stage) {
#pragma unroll
    for (int ii = 0; ii < 4; ii++) {
        const int i = ORDER ? (ii == 0 ? 0 : ii == 1 ? 3 : ii == 2 ? 1 : 2) : ii;
        tc::mma_f16(acc + (uint32_t)(i * BN), adesc + (uint64_t)(i * aplane16), bdesc,
                    tc::idesc_f16_f32(BM, BN * (4 - i)), (!first_stage || i > 0) ? 1u : 0u);
    }
}

// The MMAs of one stage for the high diagonals 4-7 (columns 256-511): for A
// plane i the B planes j = max(0, 4-i)..7-i, one MMA each (8 per stage).
template <int ORDER>
__device__ __forceinline__ void issue_hi(uint32_t acc, uint64_t adesc, uint32_t aplane16, uint64_t bdesc,
                                         bool first_stage) {
#pragma unroll
    for (int ii = 0; ii < 8; ii++) {
        const int i = ORDER ? (ii == 0 ? 0 : ii == 1 ? 7 : ii == 2 ? 1 : ii == 3 ? 6 : ii == 4 ? 2 : ii == 5 ? 5
                                                                                    : ii == 6 ? 3 : 4)
                            : ii;
        const int jlo = 4 - i > 0 ? 4 - i : 0;
        const int cnt = 8 - i < 4 ? 8 - i : 4;
        tc::mma_f16(acc + (uint32_t)((i + jlo) * BN), adesc + (uint64_t)(i * aplane16),
                    bdesc + (uint64_t)((jlo * B_PLANE_BYTES) >> 4), tc::idesc_f16_f32(BM, BN * cnt),
                    (!first_stage || i > 0) ? 1u : 0u);
    }
}

__device__ __forceinline__ int f2i(uint32_t x) { return __float2int_rz(__uint_as_float(x)); }

// Move accumulators into the running 64-bit sums of this thread's 32
// columns. Low group: diagonals 0-3 in full 64-bit precision. High group:
// diagonals 4-7 (shift >= 32) only into the high word. The next
// accumulator's tensor-memory load is in flight while the current one is
// folded in (tcgen05.wait::ld waits for all of a thread's loads, so each
// wait covers exactly the one load issued since the previous wait).
__device__ __forceinline__ void fold_lo(int a, const uint32_t (&r)[32], uint64_t (&acc)[32]) {
#pragma unroll
    for (int j = 0; j < 32; j++) {
        // acc += D * 2^(8a) as one widening multiply-add
        const int32_t dv = f2i(r[j]);
        uint64_t t;
        asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(t) : "r"(dv), "r"(1 << (8 * a)), "l"(acc[j]));
        acc[j] = t;
    }
}
__device__ __forceinline__ void fold_hi(int a, const uint32_t (&r)[32], uint64_t (&acc)[32]) {
#pragma unroll
    for (int j = 0; j < 32; j++) acc[j] += (uint64_t)((uint32_t)f2i(r[j]) << (8 * (a - 4))) << 32;
}
// The whole drain of a group with the four accumulators in registers: load,
// wait, hand tensor memory back to the group's MMA warp, then fold all four.
template <bool HI> __device__ __forceinline__ void drain4(uint32_t taddr, uint64_t (&acc)[32], uint32_t bar_empty) {
    constexpr int a0 = HI ? 4 : 0;
    uint32_t r0[32], r1[32], r2[32], r3[32];
    tc::tmem_ld32(taddr + (uint32_t)(a0 * BN), r0);
    tc::tmem_ld32(taddr + (uint32_t)((a0 + 1) * BN), r1);
    tc::tmem_ld32(taddr + (uint32_t)((a0 + 2) * BN), r2);
    tc::tmem_ld32(taddr + (uint32_t)((a0 + 3) * BN), r3);
    tc::tmem_wait_ld();
    tc::tc_fence_before();
    tc::mbar_arrive(bar_empty);
    if (HI) {
        fold_hi(a0, r0, acc);
        fold_hi(a0 + 1, r1, acc);
        fold_hi(a0 + 2, r2, acc);
        fold_hi(a0 + 3, r3, acc);
    } else {
        fold_lo(a0, r0, acc);
        fold_lo(a0 + 1, r1, acc);
        fold_lo(a0 + 2, r2, acc);
        fold_lo(a0 + 3, r3, acc);
    }
}

// number of low-group chunks of a K' range of nst stages
__device__ __forceinline__ int lo_chunks(int nst) {
    return nst <= 0 ? 0 : nst <= LO_FIRST ? 1 : 1 + (nst - LO_FIRST + CHUNK_STAGES_LO - 1) / CHUNK_STAGES_LO;
}

// The tile's output, staged in shared memory once the accumulators are all
// drained (the stage ring is free then: every MMA has completed, so every
// load it read has landed). Each epilogue thread puts its row's 32 values
// (Z, or 1 + (Z - d) / d for a direct output) into STG[row][col]; then the 256
// epilogue threads write each output share as whole row segments (a warp
// stores 32 consecutive columns of one row, or 32 consecutive rows of one
// column for a column-major GEMM output), adding the bias shares.
constexpr int STG_PITCH = BN + 1;  // u64 per staged row: two-way bank conflicts at most
static_assert(BM * STG_PITCH * 8 + BM * 8 <= STAGES * STAGE_BYTES, "the staged tile must fit in the stage ring");
static_assert(BM * STG_PITCH * 8 + BM * 8 <= 2 * STAGE_BYTES && BM * BN * 8 <= 2 * STAGE_BYTES,
              "the pitched tile fits in stages 0-1 and the dense one in stages 2-3");
static_assert(NTHREADS - W_EPI0 * 32 == 256, "eight epilogue warps");

__device__ __forceinline__ void named_bar_epilogue() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
// the epilogue warps' drain hand-offs (see the drain loop)
__device__ __forceinline__ void named_bar_poll() { asm volatile("bar.sync 2, 256;" ::: "memory"); }
__device__ __forceinline__ void named_bar_poll2() { asm volatile("bar.sync 3, 256;" ::: "memory"); }

__device__ __forceinline__ void stage_row(const Args &g, uint64_t *stg, long long *mrow, int row, int colh,
                                          long long m, const uint64_t (&zs)[32]) {
    if (colh == 0) mrow[row] = m;
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const uint64_t v = g.direct ? 1 + div_public<uint64_t>(zs[j] - g.d, g.d, g.dshift) : zs[j];
        stg[row * STG_PITCH + colh * 32 + j] = v;
    }
}

__device__ __forceinline__ void store_tile(const Args &g, int z, int nbase, const uint64_t *stg, const long long *mrow,
                                           int te) {
    const int ncols = g.N - nbase < BN ? g.N - nbase : BN;
    if (!g.direct) {
        for (int e = te; e < BM * BN; e += 256) {
            const int r = e >> 6, c = e & (BN - 1);
            const long long m = mrow[r];
            if (m >= 0 && c < ncols) g.partial[((long long)z * g.M + m) * g.N + nbase + c] = stg[r * STG_PITCH + c];
        }
        return;
    }
#pragma unroll 1
    for (int ps = 0; ps < 6; ps++) {
        uint64_t *o = g.out[ps];
        const uint64_t *b = g.bias[ps];
        const bool val = (ps == 0 || ps == 5);
        if (!val && !b && g.zeros_kept) continue;
        for (int e = te; e < BM * BN; e += 256) {
            const int r = g.colmajor ? (e & (BM - 1)) : (e >> 6);
            const int c = g.colmajor ? (e >> 7) : (e & (BN - 1));
            const long long m = mrow[r];
            if (m < 0 || c >= ncols) continue;
            const int n = nbase + c;
            uint64_t v = val ? stg[r * STG_PITCH + c] : 0;
            if (b) v += b[n];
            o[g.colmajor ? m + (long long)n * g.M : m * g.N + n] = v;
        }
    }
}

// One 4-D tensor-map store of a staged tile from shared memory (bulk group).
__device__ __forceinline__ void tma_store_4d(const CUtensorMap *map, uint32_t src, int c0, int c1, int c2, int c3) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(src), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
                 : "memory");
}

// One work item of the kernel: an output tile (N tile bx, row tile by) and
// its K' slice z, with the tile's geometry and its stage range. Items are
// numbered bx fastest, then by, then z; a CTA takes items blockIdx.x,
// blockIdx.x + gridDim.x, ... (one item per CTA when the grid holds them
// all, a loop over items when the grid is one CTA per SM).
struct Item {
    int bx, by, z;
    int tw, t2, w0, h0, n0;
    int r_lo, s_lo, ns, tile_stages, stage_begin, nst;
};

__host__ __device__ __forceinline__ void item_geometry(const Args &g, int item, Item &it) {
    it.bx = item % g.ntiles_n;
    const int rest = item / g.ntiles_n;
    it.by = rest % g.tiles_m;
    it.z = rest / g.tiles_m;
    it.tw = it.by % g.tiles_w;
    it.t2 = it.by / g.tiles_w;
    const int th = it.t2 % g.tiles_h, tn = it.t2 / g.tiles_h;
    it.w0 = it.tw * g.Wt;
    it.h0 = th * g.Ht;
    it.n0 = tn * g.Nt;
    // Position-major tiles (output pixel (h0, w0) of Nt images) run only the
    // taps inside the input: rows r_lo..r_lo+nr-1, columns s_lo..s_lo+ns-1 of
    // the filter. Their K' range (6 segments x taps x channel blocks) is split
    // evenly over the nsplit slices.
    it.r_lo = 0;
    it.s_lo = 0;
    it.ns = 1;
    it.tile_stages = g.total_stages;
    if (g.wgt) {
        // Weight gradient of filter tap (r, s) = t2 for input channels tw *
        // 128 ...: K runs over the output pixels (p, q) whose input pixel
        // (p + r - pad, q + s - pad) is inside the image (rows r_lo...,
        // columns s_lo..s_lo+ns-1) and 16 images per stage.
        const int tap = it.t2, r = tap / g.f, sx = tap - r * g.f;
        it.r_lo = g.pad - r > 0 ? g.pad - r : 0;
        const int p_hi = g.Himg - 1 + g.pad - r < g.P - 1 ? g.Himg - 1 + g.pad - r : g.P - 1;
        it.s_lo = g.pad - sx > 0 ? g.pad - sx : 0;
        const int q_hi = g.Wimg - 1 + g.pad - sx < g.Q - 1 ? g.Wimg - 1 + g.pad - sx : g.Q - 1;
        it.ns = q_hi - it.s_lo + 1;
        it.tile_stages = (p_hi >= it.r_lo && it.ns > 0) ? 6 * (p_hi - it.r_lo + 1) * it.ns * g.nb16 : 0;
    } else if (g.posmajor) {
        it.r_lo = g.pad - it.h0 > 0 ? g.pad - it.h0 : 0;
        const int r_hi = g.Himg - 1 + g.pad - it.h0 < g.f - 1 ? g.Himg - 1 + g.pad - it.h0 : g.f - 1;
        it.s_lo = g.pad - it.w0 > 0 ? g.pad - it.w0 : 0;
        const int s_hi = g.Wimg - 1 + g.pad - it.w0 < g.f - 1 ? g.Wimg - 1 + g.pad - it.w0 : g.f - 1;
        it.ns = s_hi - it.s_lo + 1;
        it.tile_stages = 6 * (r_hi - it.r_lo + 1) * it.ns * g.cblocks;
    }
    int stage_end;
    if (g.posmajor || g.wgt) {
        const int per = (it.tile_stages + g.nsplit - 1) / g.nsplit;
        it.stage_begin = it.z * per;
        stage_end = it.stage_begin + per;
    } else {
        it.stage_begin = it.z * g.chunks_per_split * CHUNK_STAGES;
        stage_end = it.stage_begin + g.chunks_per_split * CHUNK_STAGES;
    }
    if (stage_end > it.tile_stages) stage_end = it.tile_stages;
    it.nst = stage_end > it.stage_begin ? stage_end - it.stage_begin : 0;
}

// The CTAs' item lists, balanced on the host: items taken longest first
// (by stage count), each given to the CTA with the fewest stages so far, so
// that position-major tiles of 4, 6 and 9 taps, split-K slices and
// weight-gradient taps of different lengths even out across the CTAs (a
// round-robin deal left some CTAs with more long tiles: the 8x8x256
// convolutions of VGG16 1.10 -> 1.13 ms). CTA b runs order[start[b]] ..
// order[start[b+1] - 1]; n == 0: round-robin (item b, b + gridDim.x, ...).
constexpr int SCHED_MAX_CTAS = 256, SCHED_MAX_ITEMS = 8192;
struct Sched {
    int n;
    uint16_t start[SCHED_MAX_CTAS + 1];
    uint16_t order[SCHED_MAX_ITEMS];
};

// k-th item of this CTA, or -1
__device__ __forceinline__ int cta_item(const Sched &sc, const Args &g, int k) {
    if (sc.n) {
        const int i = sc.start[blockIdx.x] + k;
        return i < sc.start[blockIdx.x + 1] ? sc.order[i] : -1;
    }
    const long long item = blockIdx.x + (long long)k * gridDim.x;
    return item < g.n_items ? (int)item : -1;
}

// The stage count of an item alone (for the MMA issuers, which need nothing else).
__device__ __forceinline__ int item_nst(const Args &g, int item) {
    Item it;
    item_geometry(g, item, it);
    return it.nst;
}

// A tile's output straight from the epilogue thread's registers (row m,
// columns nb .. nb+31 of its half), while the stage ring already holds the
// next item's operands: 16-byte stores of a row's consecutive columns where
// the row is 16-byte aligned, one column per store for a column-major output
// (the warp's 32 consecutive rows make those coalesced).
__device__ __forceinline__ void put_row(uint64_t *dst, int ncols, const uint64_t (&v)[32], const uint64_t *b) {
    if (!b && ncols == 32 && !((uintptr_t)dst & 15)) {
#pragma unroll
        for (int j = 0; j < 32; j += 2)
            asm volatile("st.global.v2.u64 [%0], {%1, %2};" ::"l"(dst + j), "l"(v[j]), "l"(v[j + 1]) : "memory");
        return;
    }
#pragma unroll
    for (int j = 0; j < 32; j++)
        if (j < ncols) dst[j] = v[j] + (b ? b[j] : 0);
}

__device__ __forceinline__ void store_row_direct(const Args &g, int z, long long m, int nb, uint64_t (&zs)[32]) {
    const int ncols = g.N - nb < 32 ? g.N - nb : 32;
    if (m < 0 || ncols <= 0) return;
    if (!g.direct) {
        put_row(g.partial + ((long long)z * g.M + m) * g.N + nb, ncols, zs, nullptr);
        return;
    }
#pragma unroll
    for (int j = 0; j < 32; j++) zs[j] = 1 + div_public<uint64_t>(zs[j] - g.d, g.d, g.dshift);
#pragma unroll 1
    for (int ps = 0; ps < 6; ps++) {
        uint64_t *o = g.out[ps];
        const uint64_t *b = g.bias[ps] ? g.bias[ps] + nb : nullptr;
        const bool val = (ps == 0 || ps == 5);
        if (!val && !b && g.zeros_kept) continue;
        if (g.colmajor) {
#pragma unroll
            for (int j = 0; j < 32; j++)
                if (j < ncols) o[m + (long long)(nb + j) * g.M] = (val ? zs[j] : 0) + (b ? b[j] : 0);
        } else if (val) {
            put_row(o + m * g.N + nb, ncols, zs, b);
        } else {
            uint64_t zero[32];
#pragma unroll
            for (int j = 0; j < 32; j++) zero[j] = 0;
            put_row(o + m * g.N + nb, ncols, zero, b);
        }
    }
}

__global__ void __launch_bounds__(NTHREADS, 1)
    limb_tma_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmOut0,
                    const __grid_constant__ CUtensorMap tmOut5, const __grid_constant__ Args gp,
                    const __grid_constant__ Sched sc) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
    Smem &sm = *reinterpret_cast<Smem *>(smem_raw + pad);
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&gp);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sm.args);
        for (int i = threadIdx.x; i < (int)(sizeof(Args) / 4); i += blockDim.x) dst[i] = src[i];
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(tc::smem_u32(&sm.full[s]), 1);
            tc::mbar_init(tc::smem_u32(&sm.empty[s]), 2);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(tc::smem_u32(&sm.acc_full[b]), 1);
            tc::mbar_init(tc::smem_u32(&sm.acc_empty[b]), 256);
        }
        tc::mbar_init(tc::smem_u32(&sm.done), 2);
        sm.abort = 0;
        sm.never = 0;
        sm.hi_issued = 0;
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
    const uint64_t wait_ns = g.wait_ns;

    if (warp < W_EPI0) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(REGS_CTRL));
    if (warp == W_PROD) {
        // ------------------------------------------------ TMA + bulk copies
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
            const bool rep = g.rep_flag && *g.rep_flag;  // the image holds one block per share
            int R = 0;  // ring position: stages issued by this CTA over its items
            bool ok = true;
            for (int k = 0, item; ok && (item = cta_item(sc, g, k)) >= 0; k++) {
                Item it;
                item_geometry(g, item, it);
                for (int git = 0; git < it.nst; git++) {
                    const int s = R % STAGES;
                    const uint32_t ph = (uint32_t)(R / STAGES) & 1;
                    if (!tc::mbar_wait(tc::smem_u32(&sm.empty[s]), ph ^ 1, &sm.abort, wait_ns)) {
                        flag_error(sm, g, 0x100 + s);
                        ok = false;
                        break;
                    }
                    int gst = it.stage_begin + git;
                    int seg, x, y, zc, c3;
                    if (g.wgt) {
                        // (segment, valid output pixel, 16-image block) -> the packed dY stage
                        const int per_seg = it.tile_stages / 6;
                        seg = gst / per_seg;
                        const int rem = gst - seg * per_seg;
                        const int pi = rem / g.nb16, nb = rem - pi * g.nb16;
                        const int pp = it.r_lo + pi / it.ns, qq = it.s_lo + pi % it.ns;
                        const int r = it.t2 / g.f, sx = it.t2 - r * g.f;
                        gst = seg * g.kblocks + (pp * g.Q + qq) * g.nb16 + nb;
                        // box: 8 images x 128 channels x 2 image blocks at input pixel (h, w), 8 planes
                        x = 0;
                        y = it.tw * BM;
                        zc = 2 * nb;
                        c3 = (pp + r - g.pad) * g.Wimg + (qq + sx - g.pad);
                    } else if (g.posmajor) {
                        // compacted K' index (segment, inside tap, channel block) -> the packed stage
                        const int per_seg = it.tile_stages / 6;
                        seg = gst / per_seg;
                        const int kb = gst - seg * per_seg;
                        const int ti = kb / g.cblocks;
                        const int cb = kb - ti * g.cblocks;
                        const int r = it.r_lo + ti / it.ns, sx = it.s_lo + ti % it.ns;
                        gst = seg * g.kblocks + (r * g.f + sx) * g.cblocks + cb;
                        // 32-row line of the batch-innermost image: pixel (h * W + w) * Nimg + n0
                        x = 0;
                        y = (int)((((long long)(it.h0 + r - g.pad) * g.Wimg + (it.w0 + sx - g.pad)) * g.Nimg + it.n0) >>
                                  5);
                        zc = 0;
                        c3 = 2 * cb;
                    } else {
                        seg = gst / g.kblocks;
                        const int kb = gst - seg * g.kblocks;
                        const int tap = kb / g.cblocks;
                        const int cb = kb - tap * g.cblocks;
                        const int r = tap / g.f, sx = tap - r * g.f;
                        // line offset (16 bytes per pixel, so always 16-byte aligned), row, image
                        x = g.rows_mode ? 0 : 8 * (it.w0 + sx - g.pad);
                        y = g.rows_mode ? it.n0 >> 5 : it.h0 + r - g.pad;
                        zc = g.rows_mode ? 0 : it.n0;
                        c3 = 2 * cb;
                    }
                    const int this_R = R++;
                    if (this_R == g.withhold) continue;  // diagnostic: this stage's data never arrives
                    const uint32_t bar = tc::smem_u32(&sm.full[s]);
                    tc::mbar_arrive_expect_tx(bar, 8 * g.a_box_bytes + B_STAGE_BYTES);
                    const uint32_t dst = tc::smem_u32(sm.stage[s]);
                    tma_load_5d(dst, &tmA, x, y, zc, c3, (rep ? ((seg + 1) >> 1) % 3 : g.seg_block[seg]) * 8, bar);
                    const uint8_t *src = g.packB + ((size_t)gst * g.ntiles_n + it.bx) * B_STAGE_BYTES;
                    tc::bulk_g2s(dst + 8 * A_PLANE_BYTES, src, B_STAGE_BYTES, bar);
                }
            }
            if (!ok) {
                // wait (bounded, not cut short by the abort flag) for the copies still in flight
                const int from = R - STAGES > 0 ? R - STAGES : 0;
                for (int r = from; r < R; r++)
                    tc::mbar_wait(tc::smem_u32(&sm.full[r % STAGES]), (uint32_t)(r / STAGES) & 1, &sm.never, wait_ns);
            }
        }
        __syncwarp();
    } else if (warp == W_MMA || warp == W_MMA2) {
        // --------------------------------------------- MMA: one warp per group
        // Each group's issuer blocks on its own barriers only: the drain wait
        // at its chunk starts and the stage data. (One thread interleaving both
        // groups, polling both sets of barriers, issued 12-17 % slower.)
        if (lane == 0) {
            const int gi = warp == W_MMA ? 0 : 1;
            const uint32_t s0 = tc::smem_u32(sm.stage[0]);
            const uint64_t adesc0 = tc::smem_desc(s0, g.a_box_bytes / 2, 128);
            const uint64_t bdesc0 = tc::smem_desc(s0 + 8 * A_PLANE_BYTES, 128, 256);
            const uint32_t aplane16 = g.a_box_bytes >> 4;
            const int len = gi == 0 ? CHUNK_STAGES_LO : CHUNK_STAGES;
            int R_total = 0;  // stages of all of this CTA's items
            for (int k = 0, item; (item = cta_item(sc, g, k)) >= 0; k++) R_total += item_nst(g, item);
            int R = 0, chunk = 0;  // ring position and chunks committed, over the items
            bool ok = true;
            for (int k = 0, item; ok && (item = cta_item(sc, g, k)) >= 0; k++) {
                const int nst = item_nst(g, item);
                int cstart = 0;
                int cend = gi == 0 ? (nst < LO_FIRST ? nst : LO_FIRST) : (nst < CHUNK_STAGES ? nst : CHUNK_STAGES);
                for (int t = 0; t < nst; t++, R++) {
                    if (t == cstart && chunk > 0) {
                        if (!tc::mbar_wait(tc::smem_u32(&sm.acc_empty[gi]), (uint32_t)(chunk - 1) & 1, &sm.abort,
                                           wait_ns)) {
                            flag_error(sm, g, 0x300 + gi);
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
                    }
                    if (!tc::mbar_wait(tc::smem_u32(&sm.full[R % STAGES]), (uint32_t)(R / STAGES) & 1, &sm.abort,
                                       wait_ns)) {
                        flag_error(sm, g, 0x310 + gi);
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    if (gi == 0 && g.lag > 0 && !wait_issued(sm, R + g.lag < R_total ? R + g.lag : R_total, wait_ns)) {
                        flag_error(sm, g, 0x320);
                        ok = false;
                        break;
                    }
                    const uint64_t off = (uint64_t)(((R % STAGES) * STAGE_BYTES) >> 4);
                    if (gi == 0) {
                        if (g.order) issue_lo<1>(tmem, adesc0 + off, aplane16, bdesc0 + off, t == cstart);
                        else issue_lo<0>(tmem, adesc0 + off, aplane16, bdesc0 + off, t == cstart);
                    } else {
                        if (g.order) issue_hi<1>(tmem, adesc0 + off, aplane16, bdesc0 + off, t == cstart);
                        else issue_hi<0>(tmem, adesc0 + off, aplane16, bdesc0 + off, t == cstart);
                    }
                    if (R < R_total - STAGES) tc::mma_commit(tc::smem_u32(&sm.empty[R % STAGES]));
                    if (gi == 1) *reinterpret_cast<volatile int *>(&sm.hi_issued) = R + 1;
                    if (t + 1 == cend) {
                        tc::mma_commit(tc::smem_u32(&sm.acc_full[gi]));
                        chunk++;
                        cstart = t + 1;
                        cend = nst < cstart + len ? nst : cstart + len;
                    }
                }
            }
            if (R_total > 0) {
                tc::mma_commit(tc::smem_u32(&sm.done));
                if (!tc::mbar_wait(tc::smem_u32(&sm.done), 0, &sm.never, wait_ns) && g.err) atomicCAS(g.err, 0, 0x400);
            }
        }
        __syncwarp();
    }
    } else {
        asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(REGS_EPI));
        // -------------------------------------------------------- epilogue
        const int q = warp & 3;
        const int colh = (warp - W_EPI0) >> 2;
        const int row = q * 32 + lane;
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(colh * 32);
        int drained[2] = {0, 0};  // chunks drained per group, over the items
        for (int k = 0, item; (item = cta_item(sc, g, k)) >= 0; k++) {
            Item it;
            item_geometry(g, item, it);
            const bool last = cta_item(sc, g, k + 1) < 0;
            uint64_t zs[32];  // running Z of this thread's 32 columns
#pragma unroll
            for (int j = 0; j < 32; j++) zs[j] = 0;
            // drain each group's chunks in order, whichever group is ready first:
            // one lane of the first epilogue warp polls the two groups' barriers
            // and names the group; the other warps sleep on a named barrier
            // meanwhile (256 threads spinning on the barriers cost the MMA and
            // copy warps about 4 % of their issue slots: measured on the stage
            // pipeline)
            const int nch[2] = {lo_chunks(it.nst), (it.nst + CHUNK_STAGES - 1) / CHUNK_STAGES};
            int done_ch[2] = {0, 0};
            while (done_ch[0] < nch[0] || done_ch[1] < nch[1]) {
                if (warp == W_EPI0) {
                    if (lane == 0) {
                        int sel = -1;
                        const uint64_t t0 = tc::globaltimer();
                        for (uint32_t it_ = 0;; it_++) {
                            if (done_ch[1] < nch[1] &&
                                tc::mbar_test_wait(tc::smem_u32(&sm.acc_full[1]), (uint32_t)drained[1] & 1)) {
                                sel = 1;
                                break;
                            }
                            if (done_ch[0] < nch[0] &&
                                tc::mbar_test_wait(tc::smem_u32(&sm.acc_full[0]), (uint32_t)drained[0] & 1)) {
                                sel = 0;
                                break;
                            }
                            if ((it_ & 15) == 0) {
                                if (*reinterpret_cast<volatile int *>(&sm.abort)) break;
                                if (tc::globaltimer() - t0 > wait_ns) {
                                    flag_error(sm, g, 0x500);
                                    break;
                                }
                            }
                        }
                        sm.gsel = sel;
                    }
                    __syncwarp();
                }
                named_bar_poll();
                const int gi = *reinterpret_cast<volatile int *>(&sm.gsel);
                named_bar_poll2();  // every thread has read gsel before the next poll writes it
                if (gi < 0) break;
                tc::tc_fence_after();
                if (gi == 0) drain4<false>(taddr, zs, tc::smem_u32(&sm.acc_empty[0]));
                else drain4<true>(taddr, zs, tc::smem_u32(&sm.acc_empty[1]));
                done_ch[gi]++;
                drained[gi]++;
            }
            // output row of this thread's accumulator lane (-1: padding or past the image)
            long long m = -1;
            if (g.wgt) {
                // row = input channel tw * 128 + row of filter tap t2: output row (r, s, c)
                const int ch = it.tw * BM + row;
                if (ch < g.cdim) m = (long long)it.t2 * g.cdim + ch;
            } else if (row < g.R) {
                const int wh = g.Wt * g.Ht;
                const int nn = row / wh, rem = row - nn * wh;
                const int hh = rem / g.Wt, ww = rem - hh * g.Wt;
                const int n = it.n0 + nn, h = it.h0 + hh, w = it.w0 + ww;
                if (n < g.Nimg && h < g.P && w < g.Q) m = ((long long)n * g.P + h) * g.Q + w;
            }
            if (!last) {
                // the stage ring already holds the next item's operands; after
                // an abort the items are still walked (without stores), so that
                // every epilogue thread reaches the last item's barriers
                if (!sm.abort) store_row_direct(g, it.z, m, it.bx * BN + colh * 32, zs);
                continue;
            }
            // The CTA's last item: every MMA has completed and no copy is
            // pending, so the tile is staged in the stage ring and written as
            // whole row segments or by tensor-map stores. Every epilogue warp
            // reaches both barriers (the drain loop only ever breaks out, and
            // no role sets the abort flag any more once the last item's
            // chunks are drained).
            uint64_t *stg = reinterpret_cast<uint64_t *>(sm.stage[0]);
            long long *mrow = reinterpret_cast<long long *>(stg + BM * STG_PITCH);
            tc::fence_proxy_async_smem();
            stage_row(g, stg, mrow, row, colh, sm.abort ? -1 : m, zs);
            named_bar_epilogue();
            if (!sm.abort && g.tma_out) {
                // The tile's value (the same for party A's shareA and party C's
                // shareB) repacked densely, row by row in the box's order (BN
                // columns, then Wt, Ht, Nt), then stored by the tensor maps of the
                // two value shares; the maps clip rows and columns past the tensor.
                const int te = threadIdx.x - W_EPI0 * 32;
                uint64_t *dense = reinterpret_cast<uint64_t *>(sm.stage[2]);
                for (int e = te; e < g.R * BN; e += 256) dense[e] = stg[(e >> 6) * STG_PITCH + (e & (BN - 1))];
                tc::fence_proxy_async_smem();
                named_bar_epilogue();
                if (te == 0) {
                    const int c0 = it.bx * BN;
                    const int c1 = g.rows_mode ? it.n0 : it.w0, c2 = g.rows_mode ? 0 : it.h0,
                              c3 = g.rows_mode ? 0 : it.n0;
                    const uint32_t src = tc::smem_u32(dense);
                    tma_store_4d(&tmOut0, src, c0, c1, c2, c3);
                    tma_store_4d(&tmOut5, src, c0, c1, c2, c3);
                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    // the shared memory must stay valid until the stores have read it
                    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                }
            } else if (!sm.abort) {
                store_tile(g, it.z, it.bx * BN, stg, mrow, threadIdx.x - W_EPI0 * 32);
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == W_MMA) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// sum the split-K partials and apply dividePublic3out3 (+ bias)
__global__ void reduce_kernel(const __grid_constant__ Args g, int nsplit) {
    const long long total = (long long)g.M * g.N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        uint64_t zv = 0;
        for (int s = 0; s < nsplit; s++) zv += g.partial[(long long)s * total + e];
        if (g.raw) {
            g.raw[e] = zv;
            continue;
        }
        const long long m = e / g.N;
        const int n = (int)(e - m * g.N);
        const long long idx = g.colmajor ? m + (long long)n * g.M : e;
        const uint64_t vv = 1 + div_public<uint64_t>(zv - g.d, g.d, g.dshift);
#pragma unroll
        for (int ps = 0; ps < 6; ps++) {
            const bool val = (ps == 0 || ps == 5);
            if (!val && !g.bias[ps] && g.zeros_kept) continue;
            uint64_t base = val ? vv : 0;
            if (g.bias[ps]) base += g.bias[ps][n];
            g.out[ps][idx] = base;
        }
    }
}

// ------------------------------------------------------ input gradient

struct Col2ImArgs {
    const uint64_t *cols;  // [n][p][q][r][s][c]: untruncated Z of dY x W per output pixel and tap
    uint64_t *out[6];
    long long total;       // batch * H * W * Din
    int H, W, Din, f, stride, pad, P, Q;
    uint64_t d;
    int dshift;
};

// The input gradient of a convolution (CNNLayer backward, dL/dX): Z at
// (n, h, w, c) is the sum of the per-tap products cols[(n, p, q)][(r, s, c)]
// over the taps with p * stride = h + pad - r, q * stride = w + pad - s; then
// dividePublic3out3 (r = 1 at party A's shareA and party C's shareB).
__global__ void col2im_kernel(const __grid_constant__ Col2ImArgs ca) {
    const long long fd = (long long)ca.f * ca.f * ca.Din;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ca.total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % ca.Din);
        long long t = e / ca.Din;
        const int w = (int)(t % ca.W);
        t /= ca.W;
        const int h = (int)(t % ca.H);
        const long long n = t / ca.H;
        uint64_t z = 0;
        for (int r = 0; r < ca.f; r++) {
            const int ph = h + ca.pad - r;
            if (ph < 0 || ph % ca.stride) continue;
            const int p = ph / ca.stride;
            if (p >= ca.P) continue;
            for (int s = 0; s < ca.f; s++) {
                const int qw = w + ca.pad - s;
                if (qw < 0 || qw % ca.stride) continue;
                const int q = qw / ca.stride;
                if (q >= ca.Q) continue;
                z += __ldg(ca.cols + ((n * ca.P + p) * ca.Q + q) * fd + (r * ca.f + s) * ca.Din + c);
            }
        }
        const uint64_t v = 1 + div_public<uint64_t>(z - ca.d, ca.d, ca.dshift);
#pragma unroll
        for (int ps = 0; ps < 6; ps++) ca.out[ps][e] = (ps == 0 || ps == 5) ? v : 0;
    }
}

// ------------------------------------------------------------- self test

// One 128x64x16 MMA of fp16 integers, D = A * B^T, with A and B given as
// K-major row-major halves (128 x 16 and 64 x 16). Checks the shared-memory
// descriptors, the instruction descriptor and the tensor-memory lane/column
// layout against a host reference.
__global__ void __launch_bounds__(128, 1) selftest_kernel(const uint16_t *A, const uint16_t *B, float *D, int *err) {
    __shared__ __align__(1024) uint8_t sa[A_PLANE_BYTES];
    __shared__ __align__(1024) uint8_t sb[B_PLANE_BYTES];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    __shared__ int abort_flag;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int kc = 0; kc < 2; kc++) {
        *reinterpret_cast<uint4 *>(sa + b_off(t, kc)) = *reinterpret_cast<const uint4 *>(A + t * 16 + kc * 8);
        if (t < 64) *reinterpret_cast<uint4 *>(sb + b_off(t, kc)) = *reinterpret_cast<const uint4 *>(B + t * 16 + kc * 8);
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
    const bool ok = tc::mbar_wait(tc::smem_u32(&bar), 0, &abort_flag, WAIT_NS);
    if (!ok && err) atomicCAS(err, 0, 0x700);
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

// ------------------------------------------------------------------- host

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn(Ctx *c) {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    });
    if (!fn) set_error(c, PG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    return fn;
}

// Once per device (with it current): the GEMM kernel's shared-memory limit
// and the tensor-map encoder.
int prepare_device(Ctx *c, bool again) {
    static std::mutex mu;
    static bool done[64];
    std::lock_guard<std::mutex> lock(mu);
    if (c->device < 0 || c->device >= 64) return set_error(c, PG_ERR_UNSUPPORTED, "device ordinal %d", c->device);
    if (!done[c->device] || again) {
        PG_CHECK_CUDA(c, cudaFuncSetAttribute(limb_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem_bytes()));
        // the register split inside the kernel assumes this launch size
        cudaFuncAttributes fa;
        PG_CHECK_CUDA(c, cudaFuncGetAttributes(&fa, limb_tma_kernel));
        if (fa.numRegs != REGS_LAUNCH || fa.maxThreadsPerBlock < NTHREADS)
            return set_error(c, PG_ERR_UNSUPPORTED,
                             "limb_tma_kernel built with %d registers per thread (%d threads); its register split "
                             "needs %d", fa.numRegs, fa.maxThreadsPerBlock, REGS_LAUNCH);
        if (!encode_fn(c)) return PG_ERR_CUDA;
        done[c->device] = true;
    }
    return PG_OK;
}

static void tile_geometry(Plan &p) {
    if (p.posmajor) {
        // one output position of BM images per tile
        p.Wt = 1;
        p.Ht = 1;
        p.Nt = BM;
        p.tiles_w = p.Q;
        p.tiles_h = p.P;
    } else if (!p.implicit) {
        // rows of the image, 32 per tensor-map line
        p.Wt = 1;
        p.Ht = 1;
        const int r32 = (p.M + 31) / 32 * 32;
        p.Nt = r32 < BM ? r32 : BM;
        p.tiles_w = 1;
        p.tiles_h = 1;
    } else {
        // up to 32 output columns per line; then rows, then whole images, up to 128 pixels
        p.Wt = p.Q < 32 ? p.Q : 32;
        p.tiles_w = (p.Q + p.Wt - 1) / p.Wt;
        p.Ht = p.P < BM / p.Wt ? p.P : BM / p.Wt;
        p.Nt = 1;
        if (p.Ht == p.P && p.tiles_w == 1) {
            const int per = BM / (p.P * p.Wt);
            p.Nt = per < p.Nimg ? per : p.Nimg;
        }
        p.tiles_h = (p.P + p.Ht - 1) / p.Ht;
    }
    p.R = p.Wt * p.Ht * p.Nt;
    p.tiles_m = p.tiles_w * p.tiles_h * ((p.Nimg + p.Nt - 1) / p.Nt);
}

static void finish_plan(Plan &p) {
    p.kblocks = p.C / BK * (p.implicit ? p.f * p.f : 1);
    p.cblocks = p.C / BK;
    p.ntiles_n = (p.N + BN - 1) / BN;
    // the GEMM / im2col image is padded with zero rows to whole 32-row lines
    p.pixels_alloc = p.implicit ? p.pixels : (p.pixels + 31) / 32 * 32;
    p.image_bytes = 96ull * (size_t)p.C * (size_t)p.pixels_alloc;
    p.packB_bytes = (size_t)6 * p.kblocks * p.ntiles_n * B_STAGE_BYTES;
    tile_geometry(p);
}

int plan_gemm(Ctx *c, Plan &p, int M, int N, int K, int tA, int tB, int tC) {
    memset(&p, 0, sizeof(p));
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    p.implicit = 0;
    p.M = M; p.N = N; p.Kreal = K;
    p.C = (K + BK - 1) / BK * BK;
    p.pixels = M;
    p.src_mode = tA ? SRC_ROWS : SRC_COLS;
    p.ld = tA ? K : M;
    p.tB_kn = tB;
    p.colmajor = !tC;
    p.f = 1; p.pad = 0;
    p.Wimg = 1; p.Himg = 1; p.Nimg = M;
    p.P = 1; p.Q = 1;
    finish_plan(p);
    return PG_OK;
}

// The implicit weight gradient (Plan::wgt) is used wherever it applies
// (stride 1, a multiple of 16 images) unless PG_WGT=0 in the environment.
static bool wgt_enabled() {
    static const bool on = [] {
        const char *e = getenv("PG_WGT");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Implicit convolutions over input channels that are not a multiple of 16
// pad the image's channels with zeros up to the next multiple (PG_CPAD=0
// turns this off), when that adds at most 60 % to the tensor work: LeNet's
// second convolution (20 -> 32 channels) then reads a 57 MB digit image
// instead of a 403 MB im2col image.
static bool cpad_enabled() {
    static const bool on = [] {
        const char *e = getenv("PG_CPAD");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Stages by which the low accumulator group's MMA issuer trails the high
// group's (PG_LAG, 0..STAGES-1; 0 turns the lag off). Measured on one GB300
// with the same tuned plans (VGG16 b128 img/s, 4096^3 share-GEMM T
// ring-MAC/s): order 0 lag 2 12.84k / 22.36 T, order 0 lag 1 12.91k /
// 23.18 T, order 1 lag 2 12.99k / 22.60 T, order 1 lag 1 13.10k / 23.48 T.
// On another, order 0: lag 0 12.06k, lag 1 12.99k, lag 2 12.98k, lag 3
// 11.03k (a lag of the ring depth less one starves the low group).
static int issue_lag() {
    static const int lag = [] {
        const char *e = getenv("PG_LAG");
        const int v = e && *e ? atoi(e) : 1;
        return v < 0 ? 0 : v > STAGES - 1 ? STAGES - 1 : v;
    }();
    return lag;
}

// Longest-first balanced item lists of a grid of `ctas` CTAs (Sched); the
// round-robin deal where the grid holds every item, or where the lists do
// not fit the parameter's tables.
static void build_schedule(const Args &g, int ctas, Sched &sc) {
    static const bool on = [] {
        const char *e = getenv("PG_SCHED");  // 0: round-robin deal
        return !(e && *e == '0');
    }();
    sc.n = 0;
    if (!on || ctas >= g.n_items || ctas > SCHED_MAX_CTAS || g.n_items > SCHED_MAX_ITEMS) return;
    std::vector<std::pair<int, int>> len((size_t)g.n_items);  // (stages, item)
    for (int i = 0; i < g.n_items; i++) {
        Item it;
        item_geometry(g, i, it);
        len[(size_t)i] = {it.nst, i};
    }
    std::stable_sort(len.begin(), len.end(), [](const std::pair<int, int> &a, const std::pair<int, int> &b) {
        return a.first > b.first;
    });
    std::vector<long long> load((size_t)ctas, 0);
    std::vector<std::vector<int>> lists((size_t)ctas);
    // least-loaded CTA first (a binary heap of (load, cta))
    std::vector<std::pair<long long, int>> heap;
    for (int b = 0; b < ctas; b++) heap.push_back({0, b});
    auto cmp = [](const std::pair<long long, int> &a, const std::pair<long long, int> &b) {
        return a.first != b.first ? a.first > b.first : a.second > b.second;
    };
    std::make_heap(heap.begin(), heap.end(), cmp);
    for (const auto &e : len) {
        std::pop_heap(heap.begin(), heap.end(), cmp);
        auto &top = heap.back();
        lists[(size_t)top.second].push_back(e.second);
        top.first += e.first + 4;  // + a few stages' worth of per-item cost
        std::push_heap(heap.begin(), heap.end(), cmp);
    }
    int pos = 0;
    for (int b = 0; b < ctas; b++) {
        sc.start[b] = (uint16_t)pos;
        // a CTA's items in increasing index (neighbouring tiles share operands in L2)
        std::sort(lists[(size_t)b].begin(), lists[(size_t)b].end());
        for (int it : lists[(size_t)b]) sc.order[pos++] = (uint16_t)it;
    }
    sc.start[ctas] = (uint16_t)pos;
    sc.n = 1;
}

// Grid of the limb GEMM (PG_PERSIST): 1 = one CTA per SM, each walking its
// share of the work items (its tiles' output stores overlap the next tile's
// copies and MMAs); 0 = one CTA per item.
static bool persistent_grid() {
    static const bool on = [] {
        const char *e = getenv("PG_PERSIST");
        return !(e && *e == '0');
    }();
    return on;
}

// whether PG_ORDER or PG_LAG fixes the limb schedule (the tuner then keeps out)
static bool schedule_from_env() {
    static const bool set = getenv("PG_ORDER") || getenv("PG_LAG");
    return set;
}

// CTAs of the persistent grid: one per SM, or fewer where PG_CTAS caps them
// (the tests use a small cap to make every CTA walk many items)
static int persistent_ctas(int sms) {
    static const int cap = [] {
        const char *e = getenv("PG_CTAS");
        return e && *e ? atoi(e) : 0;
    }();
    return cap > 0 && cap < sms ? cap : sms;
}

// MMA order within a group's stage (PG_ORDER: 1 interleaved, 0 by A plane;
// measured with issue_lag).
static int issue_order() {
    static const int order = [] {
        const char *e = getenv("PG_ORDER");
        return e && *e == '0' ? 0 : 1;
    }();
    return order;
}

// Output positions per image up to which a same convolution is tiled by
// position: 1024 (32 x 32 and smaller; measured on VGG16 at batch 128, the
// 2x2 to 8x8 layers gain 16-58 %, 16x16 3-7 %, 32x32 1 %) unless the
// environment variable PG_POSMAJOR gives another limit; PG_POSMAJOR=0 turns
// the position-major tiles off (every implicit convolution then uses
// rectangles).
static int posmajor_max_pixels() {
    static const int lim = [] {
        const char *e = getenv("PG_POSMAJOR");
        return e && *e ? atoi(e) : 1024;
    }();
    return lim;
}

int plan_conv(Ctx *c, Plan &p, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad,
              bool posmajor_ok) {
    memset(&p, 0, sizeof(p));
    if (batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Din <= 0 || Dout <= 0 || stride <= 0 || pad < 0 ||
        H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "convolution: bad geometry");
    const int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    p.M = batch * P * Q;
    p.N = Dout;
    p.tB_kn = 0;  // KRSC filters: b[n * f*f*Din + k]
    p.colmajor = 0;
    p.H = H; p.W = W; p.Din = Din; p.stride = stride;
    const int Cpad = (Din + BK - 1) / BK * BK;
    const bool padded = Din % BK != 0 && 5 * Cpad <= 8 * Din && cpad_enabled();
    if (stride == 1 && (Din % BK == 0 || padded) && Q <= BM && P <= H && Q <= W) {
        // implicit: the image is the activation tensor itself (channels zero-padded
        // to Cpad), taps are box shifts
        p.implicit = 1;
        p.Kreal = Din;
        p.C = Cpad;
        p.pixels = (long long)batch * H * W;
        p.src_mode = SRC_ROWS;
        p.ld = Din;
        p.f = f; p.pad = pad;
        p.Wimg = W; p.Himg = H; p.Nimg = batch;
        p.P = P; p.Q = Q;
        // Small "same" convolutions of a batch of whole 128-image tiles run by
        // output position: a rectangle tile of a 4x4 or 2x2 image spends most
        // of its taps on the zero padding (5/9 of them at 2x2), which a tile
        // of one output position over 128 images skips.
        p.posmajor = posmajor_ok && batch % BM == 0 && P == H && Q == W && 2 * pad + 1 == f &&
                     P * Q <= posmajor_max_pixels();
    } else {
        // explicit: the image holds the im2col rows (K = f*f*Din padded to 16)
        p.implicit = 0;
        p.Kreal = f * f * Din;
        p.C = (p.Kreal + BK - 1) / BK * BK;
        p.pixels = p.M;
        p.src_mode = SRC_IM2COL;
        p.f = 1; p.pad = 0;
        p.cf = f; p.cpad = pad; p.cP = P; p.cQ = Q;
        p.Wimg = 1; p.Himg = 1; p.Nimg = p.M;
        p.P = 1; p.Q = 1;
    }
    finish_plan(p);
    return PG_OK;
}

bool wgrad_implicit_applies(int batch, int stride) { return stride == 1 && batch % 16 == 0 && wgt_enabled(); }

int plan_dgrad_flip(Ctx *c, Plan &p, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad) {
    memset(&p, 0, sizeof(p));
    if (stride != 1 || pad < 0 || pad > f - 1 || H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_UNSUPPORTED, "flipped input gradient: stride %d, pad %d", stride, pad);
    const int P = H + 2 * pad - f + 1, Q = W + 2 * pad - f + 1;
    // dX[n][h][w][c] = sum over (r', s', k) of dY[n][h - (f-1-pad) + r'][w - (f-1-pad) + s'][k] W[k][f-1-r'][f-1-s'][c]
    int st = plan_conv(c, p, batch, P, Q, f, Dout, Din, 1, f - 1 - pad);
    if (st) return st;
    if (!p.implicit || p.P != H || p.Q != W) {
        memset(&p, 0, sizeof(p));
        return set_error(c, PG_ERR_UNSUPPORTED, "flipped input gradient: not an implicit convolution");
    }
    p.flip_f = f;
    return PG_OK;
}

int plan_wgrad(Ctx *c, Plan &p, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad,
               bool implicit_ok) {
    memset(&p, 0, sizeof(p));
    if (batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Din <= 0 || Dout <= 0 || stride <= 0 || pad < 0 ||
        H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "convolution: bad geometry");
    const int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    const long long K = (long long)batch * P * Q;
    if (K > (1ll << 30)) return set_error(c, PG_ERR_UNSUPPORTED, "weight gradient over %lld output pixels", K);
    if (implicit_ok && wgrad_implicit_applies(batch, stride)) {
        // implicit: rows (tap, c) from one image of the forward input, taps as
        // shifts of its pixel coordinate, K = valid output pixels x images
        p.wgt = 1;
        p.implicit = 0;
        p.M = f * f * Din;
        p.N = Dout;
        p.Kreal = (int)K;
        p.C = (int)K;  // K' per segment (a multiple of 16)
        p.src_mode = SRC_WGRAD_T;
        p.tB_kn = 1;
        p.colmajor = 1;
        p.H = H; p.W = W; p.Din = Din; p.stride = 1;
        p.f = f; p.pad = pad; p.P = P; p.Q = Q;
        p.Himg = H; p.Wimg = W; p.Nimg = batch;
        p.kblocks = (int)(K / BK);
        p.cblocks = 0;
        p.ntiles_n = (Dout + BN - 1) / BN;
        p.pixels = (long long)H * W * batch;
        p.pixels_alloc = p.pixels;
        // image channels: Din, or Din rounded up to 8 below one 128-row tile, so
        // that the tensor-map box (min(128, that) rows) stays inside the tensor
        p.C8 = Din >= BM ? Din : (Din + 7) / 8 * 8;
        p.image_bytes = 96ull * (size_t)p.pixels * (size_t)p.C8;
        p.packB_bytes = (size_t)6 * p.kblocks * p.ntiles_n * B_STAGE_BYTES;
        p.Wt = 1; p.Ht = 1; p.Nt = BM; p.R = p.C8 < BM ? p.C8 : BM;
        p.tiles_w = (Din + BM - 1) / BM;
        p.tiles_h = f * f;
        p.tiles_m = p.tiles_w * p.tiles_h;
        return PG_OK;
    }
    // rows (r, s, c) of the filter, K = output pixels (n, p, q): the image is the
    // transposed im2col gather of the forward input, the packed operand the
    // output gradient dY[pixel][Dout], the output dW[Dout][r][s][c] column-major
    p.implicit = 0;
    p.M = f * f * Din;
    p.N = Dout;
    p.Kreal = (int)K;
    p.C = (p.Kreal + BK - 1) / BK * BK;
    p.pixels = p.M;
    p.src_mode = SRC_WGRAD;
    p.tB_kn = 1;
    p.colmajor = 1;
    p.H = H; p.W = W; p.Din = Din; p.stride = stride;
    p.cf = f; p.cpad = pad; p.cP = P; p.cQ = Q;
    p.f = 1; p.pad = 0;
    p.Wimg = 1; p.Himg = 1; p.Nimg = p.M;
    p.P = 1; p.Q = 1;
    finish_plan(p);
    return PG_OK;
}

void choose_split(const Plan &p, int sms, int &split, int &cps) {
    const int total_stages = 6 * p.kblocks;
    const int chunks = (total_stages + CHUNK_STAGES - 1) / CHUNK_STAGES;
    const int tiles = p.tiles_m * p.ntiles_n;
    split = tiles >= sms ? 1 : sms / tiles;
    if (split > chunks) split = chunks;
    if (split < 1) split = 1;
    cps = (chunks + split - 1) / split;
    split = (chunks + cps - 1) / cps;
}

size_t partial_bytes(const Plan &p, int split) { return split > 1 ? (size_t)split * p.M * p.N * 8 : 0; }

// ---------------------------------------------------------- autotuner

// Split-K candidates of a plan: the heuristic split, 1-8, 10, 12, 14, 16,
// and doublings up to 4x the heuristic (at most 64), none above the number
// of K chunks; each normalised so that every split holds at least one chunk.
// The odd splits let a grid of tiles x split CTAs come closer to a whole
// number of waves (4x4 x 512 channels: 128 tiles, 6 -> 5.05 waves, 7 -> 5.9).
// Returns how many (at most MAX_SPLIT_CAND).
constexpr int MAX_SPLIT_CAND = 16;
static int split_candidates(const Plan &p, int sms, int (&sp)[MAX_SPLIT_CAND], int (&cp)[MAX_SPLIT_CAND]) {
    const int chunks = (6 * p.kblocks + CHUNK_STAGES - 1) / CHUNK_STAGES;
    int h, hc;
    choose_split(p, sms, h, hc);
    int n = 0;
    auto add = [&](int s) {
        if (s < 1 || s > chunks || n >= MAX_SPLIT_CAND) return;
        const int c = (chunks + s - 1) / s;
        const int s2 = (chunks + c - 1) / c;
        for (int i = 0; i < n; i++)
            if (sp[i] == s2) return;
        sp[n] = s2;
        cp[n] = c;
        n++;
    };
    add(h);
    for (int s : {1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 14, 16}) add(s);
    const int cap = 4 * h < 64 ? 4 * h : 64;
    for (int s = 32; s <= cap; s *= 2) add(s);
    return n;
}

size_t tune_partial_bytes(const Plan &p, int sms) {
    int sp[MAX_SPLIT_CAND], cp[MAX_SPLIT_CAND];
    const int n = split_candidates(p, sms, sp, cp);
    size_t b = 0;
    for (int i = 0; i < n; i++) b = partial_bytes(p, sp[i]) > b ? partial_bytes(p, sp[i]) : b;
    return b;
}

static std::string tune_key(const Plan &p);

std::string plan_key(const Plan &p) { return tune_key(p); }

// the context's tuned choice for this shape, if any
bool cached_split(Ctx *c, const Plan &p, int &split, int &cps) {
    auto it = c->split_cache.find(tune_key(p));
    if (it == c->split_cache.end()) return false;
    split = it->second.first;
    cps = it->second.second;
    return true;
}

static std::string tune_key(const Plan &p) {
    char k[256];
    snprintf(k, sizeof(k), "%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d%s", p.implicit, p.src_mode, p.M, p.N, p.C,
             p.kblocks, p.ntiles_n, p.tiles_m, p.Wt, p.Ht, p.Nt, p.f, p.colmajor,
             p.posmajor ? (p.flip_f ? "/pos/flip" : "/pos") : p.wgt ? "/wgt" : p.flip_f ? "/flip" : "");
    return k;
}

// Picks split / cps for the plan: the context's cached choice for this shape,
// else (autotuning on, no stream capture in progress) the fastest candidate
// by CUDA-event time (one warm-up and two timed runs each — more for runs
// under a quarter millisecond — on the context's
// stream, with the caller's operands and outputs: every candidate computes
// the same result; another split must beat the heuristic one by 3 %), else
// the heuristic. partial must hold
// tune_partial_bytes(p) when tuning can run.
int tune_split(Ctx *c, const Plan &p, const void *image, const void *packB, uint64_t *partial,
               uint64_t *const out[6], const uint64_t *const bias[6], int trunc, bool zeros_kept, uint64_t *raw,
               int &split, int &cps, bool shared) {
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    const std::string key = tune_key(p);
    auto it = c->split_cache.find(key);
    if (it != c->split_cache.end()) {
        split = it->second.first;
        cps = it->second.second;
        return PG_OK;
    }
    choose_split(p, sms, split, cps);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
    if (!c->autotune || cs != cudaStreamCaptureStatusNone) return PG_OK;
    int sp[MAX_SPLIT_CAND], cp[MAX_SPLIT_CAND];
    const int n = split_candidates(p, sms, sp, cp);
    if (n <= 1) {
        c->split_cache[key] = {split, cps};
        return PG_OK;
    }
    cudaEvent_t e0, e1;
    PG_CHECK_CUDA(c, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return set_error(c, PG_ERR_CUDA, "cudaEventCreate failed");
    }
    int st = PG_OK;
    // one warm-up run, then 2 timed runs; short runs are timed again over
    // enough repetitions to fill about half a millisecond
    auto time_one = [&](int sp_, int cp_, float &ms) {
        uint64_t *part = sp_ > 1 ? partial : nullptr;
        int reps = 2;
        for (int pass = 0; pass < 2 && st == PG_OK; pass++) {
            for (int r = pass ? 1 : 0; r <= reps && st == PG_OK; r++) {
                if (r == 1 && cudaEventRecord(e0, c->stream) != cudaSuccess)
                    st = set_error(c, PG_ERR_CUDA, "event record");
                if (!st) st = run_gemm(c, p, image, packB, part, sp_, cp_, out, bias, trunc, zeros_kept, raw, shared);
            }
            if (!st && cudaEventRecord(e1, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event record");
            if (!st && cudaEventSynchronize(e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event synchronize");
            if (!st && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event time");
            if (st) break;
            ms /= (float)reps;
            if (pass == 0) {
                if (ms * reps >= 0.3f) break;
                reps = (int)(0.5f / (ms > 1e-3f ? ms : 1e-3f)) + 1;
                if (reps > 64) reps = 64;
            }
        }
    };
    float best = 0.f, href = -1.f;
    for (int i = 0; i < n && st == PG_OK; i++) {
        float ms = 0.f;
        time_one(sp[i], cp[i], ms);
        // candidate 0 is the heuristic; another one must beat it by 3 %
        if (!st && (i == 0 || ms < best * (best == href ? 0.97f : 1.f))) {
            best = ms;
            split = sp[i];
            cps = cp[i];
        }
        if (i == 0) href = ms;
    }
    // The limb schedule at the chosen split: MMA order and issue lag (see
    // issue_order / issue_lag), the default (interleaved, lag 1) unless
    // another one is 2 % faster; not where the environment fixes them.
    if (!st && !schedule_from_env()) {
        const int orders[4] = {1, 0, 1, 0}, lags[4] = {1, 1, 2, 2};
        float s0 = 0.f, sbest = 0.f;
        int sbi = 0;
        for (int i = 0; i < 4 && !st; i++) {
            c->lsched_order = orders[i];
            c->lsched_lag = lags[i];
            float ms = 0.f;
            time_one(split, cps, ms);
            if (st) break;
            if (i == 0) s0 = sbest = ms;
            else if (ms < 0.98f * s0 && ms < sbest) {
                sbest = ms;
                sbi = i;
            }
        }
        c->lsched_order = c->lsched_lag = -1;
        if (!st) c->split_cache["lsched/" + key] = {orders[sbi], lags[sbi]};
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    c->split_cache[key] = {split, cps};
    return PG_OK;
}

bool relu_image_fits(const Plan &p, size_t n) {
    // the kernel's tile and pixel indices are 32-bit
    const long long tiles = (p.pixels + RI_PIX - 1) / RI_PIX * (p.C / 16);
    return p.implicit && p.src_mode == SRC_ROWS && p.C == p.Kreal && p.C % 16 == 0 && p.ld == p.C &&
           (size_t)p.pixels * p.C == n && p.pixels < (1ll << 31) && tiles < (1ll << 31);
}

int run_relu_image(Ctx *c, const Plan &p, const uint64_t *const in[6], size_t n, uint64_t *const out[6],
                   uint8_t *const dout[6], void *image, bool shared) {
    if (!relu_image_fits(p, n)) return set_error(c, PG_ERR_INVALID_ARG, "relu/image geometry mismatch");
    ReluImageArgs a;
    memset(&a, 0, sizeof(a));
    for (int k = 0; k < 6; k++) {
        if (!in[k] || (out && !out[k])) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
        a.in[k] = in[k];
        a.out[k] = out ? out[k] : nullptr;
        a.dout[k] = dout ? dout[k] : nullptr;
    }
    a.img = (uint4 *)image;
    a.pixels = p.pixels;
    a.pixels_alloc = p.pixels_alloc;
    a.C8 = p.C / 8;
    a.bi_n = p.posmajor ? p.Nimg : 0;
    a.bi_hw = (long long)p.Himg * p.Wimg;
    a.nseg = shared ? 3 : 6;
    a.zmid = c->in_zero_mid ? 1 : 0;
    const long long tiles = (long long)(a.C8 / 2) * ((p.pixels + RI_PIX - 1) / RI_PIX);
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    long long blocks = tiles < (long long)sms * 16 ? tiles : (long long)sms * 16;
    if (a.zmid) relu_image_kernel<true, true><<<(unsigned)blocks, 256, 0, c->stream>>>(a);
    else relu_image_kernel<false, true><<<(unsigned)blocks, 256, 0, c->stream>>>(a);
    c->launches++;
    return launch_status(c, "relu_image_kernel");
}

int run_image_decode(Ctx *c, const Plan &p, const void *image, size_t n, uint64_t *const out[6], bool shared) {
    if (!relu_image_fits(p, n) || !image) return set_error(c, PG_ERR_INVALID_ARG, "image decode: geometry mismatch");
    ImageDecodeArgs a;
    memset(&a, 0, sizeof(a));
    for (int k = 0; k < 6; k++) {
        if (!out[k]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
        a.out[k] = out[k];
    }
    a.img = (const uint4 *)image;
    a.pixels = p.pixels;
    a.pixels_alloc = p.pixels_alloc;
    a.C8 = p.C / 8;
    a.nseg = shared ? 3 : 6;
    a.bi_n = p.posmajor ? p.Nimg : 0;
    a.bi_hw = (long long)p.Himg * p.Wimg;
    const long long total = 6ll * (long long)n;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    long long blocks = (total + 255) / 256;
    if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
    image_decode_kernel<<<(unsigned)blocks, 256, 0, c->stream>>>(a);
    c->launches++;
    return launch_status(c, "image_decode_kernel");
}

int run_image(Ctx *c, const Plan &p, const uint64_t *const a[6], void *image, bool shared, const int *rep_flag) {
    if (p.wgt) {
        WgtImageArgs wa;
        memset(&wa, 0, sizeof(wa));
        for (int i = 0; i < 6; i++) {
            if (!a[i]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
            wa.a[i] = a[i];
        }
        wa.hw = (long long)p.Himg * p.Wimg;
        wa.nb8 = p.Nimg / 8;
        wa.cdim = p.C8;  // the image's channels
        wa.din = p.Din;
        wa.nseg = shared ? 3 : 6;
        wa.img = (uint4 *)image;
        const long long units = wa.nseg * wa.hw * wa.nb8 * wa.cdim;
        const int sms = c->sm_count > 0 ? c->sm_count : 148;
        long long blocks = (units + 255) / 256;
        if (blocks > (long long)sms * 32) blocks = (long long)sms * 32;
        wgt_image_kernel<<<(unsigned)blocks, 256, 0, c->stream>>>(wa);
        c->launches++;
        return launch_status(c, "wgt_image_kernel");
    }
    if (p.src_mode == SRC_ROWS && p.posmajor && !rep_flag && p.pixels_alloc == p.pixels &&
        relu_image_fits(p, (size_t)p.pixels * p.C)) {
        // a position-major image of whole rows: the staged kernel reads each
        // source row as whole lines (the generic one below reads 64 bytes of
        // rows one image apart per thread)
        ReluImageArgs ra;
        memset(&ra, 0, sizeof(ra));
        for (int k = 0; k < 6; k++) {
            if (!a[k]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
            ra.in[k] = a[k];
        }
        ra.img = (uint4 *)image;
        ra.pixels = p.pixels;
        ra.pixels_alloc = p.pixels_alloc;
        ra.C8 = p.C / 8;
        ra.bi_n = p.Nimg;
        ra.bi_hw = (long long)p.Himg * p.Wimg;
        ra.nseg = shared ? 3 : 6;
        const long long tiles = (long long)(ra.C8 / 2) * ((p.pixels + RI_PIX - 1) / RI_PIX);
        const int sms = c->sm_count > 0 ? c->sm_count : 148;
        const long long blocks = tiles < (long long)sms * 16 ? tiles : (long long)sms * 16;
        relu_image_kernel<false, false><<<(unsigned)blocks, 256, 0, c->stream>>>(ra);
        c->launches++;
        return launch_status(c, "relu_image_kernel");
    }
    ImageArgs ia;
    memset(&ia, 0, sizeof(ia));
    bool vec = p.src_mode == SRC_ROWS && p.ld % 2 == 0;
    for (int i = 0; i < 6; i++) {
        if (!a[i]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
        ia.a[i] = a[i];
        if (((uintptr_t)a[i] & 15) != 0) vec = false;
    }
    ia.mode = p.src_mode;
    ia.pixels = p.pixels_alloc;
    ia.pixels_src = p.pixels;
    ia.C8 = p.C / 8;
    ia.Kreal = p.Kreal;
    ia.ld = p.ld;
    ia.vec = vec && p.Kreal % 8 == 0;
    ia.H = p.H; ia.W = p.W; ia.Din = p.Din; ia.f = p.cf; ia.stride = p.stride; ia.pad = p.cpad;
    ia.P = p.cP; ia.Q = p.cQ;
    ia.bi_n = p.posmajor ? p.Nimg : 0;
    ia.bi_hw = (long long)p.Himg * p.Wimg;
    ia.nseg = shared ? 3 : 6;
    ia.rep_flag = shared ? nullptr : rep_flag;
    ia.img = (uint4 *)image;
    if (ia.C8 & 1) return set_error(c, PG_ERR_INVALID_ARG, "image channels %d are not a multiple of 16", p.C);
    const long long units = (long long)ia.nseg * (ia.C8 / 2) * p.pixels_alloc;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    long long blocks = (units + 255) / 256;
    if (blocks > (long long)sms * 32) blocks = (long long)sms * 32;
    image_kernel<<<(unsigned)blocks, 256, 0, c->stream>>>(ia);
    c->launches++;
    return launch_status(c, "image_kernel");
}

int run_pack(Ctx *c, const Plan &p, const uint64_t *const b[6], void *packB) {
    PackArgs pa;
    memset(&pa, 0, sizeof(pa));
    for (int i = 0; i < 6; i++) {
        if (!b[i]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
        pa.b[i] = b[i];
    }
    pa.N = p.N;
    pa.Kreal = p.implicit ? p.f * p.f * p.Din : p.Kreal;
    pa.kblocks = p.kblocks;
    pa.ntiles_n = p.ntiles_n;
    pa.kn = p.tB_kn;
    pa.wg_pq = p.wgt ? (long long)p.P * p.Q : 0;
    pa.wg_batch = p.Nimg;
    if (p.flip_f) {
        pa.flip_f = p.flip_f;
        pa.cpad = p.C;
        pa.creal = p.Din;
    } else if (p.implicit && !p.wgt && p.C != p.Din) {
        pa.cpad = p.C;
        pa.creal = p.Din;
    }
    pa.packB = (uint8_t *)packB;
    const long long units = 3ll * p.ntiles_n * BN * p.kblocks * 2;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    long long blocks = (units + 255) / 256;
    if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
    pack_kernel<<<(unsigned)blocks, 256, 0, c->stream>>>(pa);
    c->launches++;
    return launch_status(c, "pack_kernel");
}

int run_gemm(Ctx *c, const Plan &p, const void *image, const void *packB, uint64_t *partial, int split, int cps,
             uint64_t *const out[6], const uint64_t *const bias[6], int trunc, bool zeros_kept, uint64_t *raw,
             bool shared, const int *rep_flag) {
    {
        int st = prepare_device(c);
        if (st) return st;
    }
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    if (((uintptr_t)image & 15) || ((uintptr_t)packB & 15))
        return set_error(c, PG_ERR_INVALID_ARG, "limb buffers must be 16-byte aligned");
    if (p.tiles_m > 65535) return set_error(c, PG_ERR_UNSUPPORTED, "M = %d has too many row tiles", p.M);
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn(c);
    if (!enc) return PG_ERR_CUDA;
    // image dims (innermost first): a line of pixels x 8 channels, rows, images,
    // (segment, plane, channel group of 8)
    alignas(64) CUtensorMap tm;
    cuuint64_t dims[5];
    cuuint64_t strides[4];
    cuuint32_t box[5];
    const cuuint64_t plane_stride = (cuuint64_t)p.pixels_alloc * 16;  // bytes between channel groups
    const cuuint64_t C8 = (cuuint64_t)(p.C / 8);
    if (p.wgt) {
        // [seg*8 + plane][pixel][n / 8][c][n % 8]: 8 images, 128 channels, 2 image blocks, one pixel, 8 planes
        const cuuint64_t nb8 = (cuuint64_t)p.Nimg / 8, cd = (cuuint64_t)p.C8, hw = (cuuint64_t)p.Himg * p.Wimg;
        dims[0] = 8; dims[1] = cd; dims[2] = nb8; dims[3] = hw; dims[4] = 48;
        strides[0] = 16; strides[1] = cd * 16; strides[2] = nb8 * cd * 16; strides[3] = hw * nb8 * cd * 16;
        box[0] = 8; box[1] = (cuuint32_t)p.R; box[2] = 2; box[3] = 1; box[4] = 8;
    } else if (p.implicit && !p.posmajor) {
        dims[0] = 8 * (cuuint64_t)p.Wimg; dims[1] = p.Himg; dims[2] = p.Nimg;
        strides[0] = (cuuint64_t)p.Wimg * 16; strides[1] = (cuuint64_t)p.Himg * p.Wimg * 16; strides[2] = plane_stride;
        box[0] = 8 * p.Wt; box[1] = p.Ht; box[2] = p.Nt;
    } else {
        dims[0] = 256; dims[1] = p.pixels_alloc / 32; dims[2] = 1;
        strides[0] = 512; strides[1] = plane_stride; strides[2] = plane_stride;
        box[0] = 256; box[1] = p.Nt / 32; box[2] = 1;
    }
    // dims 3 and 4: the channel group of 8 (two per K block) and the (segment, digit plane) index;
    // one box covers the eight planes of a segment
    if (!p.wgt) {
        dims[3] = C8; dims[4] = 48;
        strides[3] = C8 * plane_stride;
        box[3] = 2; box[4] = 8;
    }
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = enc(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT16, 5, const_cast<void *>(image), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(c, PG_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    Args g;
    memset(&g, 0, sizeof(g));
    g.M = p.M; g.N = p.N;
    g.kblocks = p.kblocks; g.cblocks = p.cblocks; g.C8 = p.C / 8; g.f = p.f; g.pad = p.pad;
    g.Wt = p.Wt; g.Ht = p.Ht; g.Nt = p.Nt; g.R = p.R; g.tiles_w = p.tiles_w; g.tiles_h = p.tiles_h;
    g.rows_mode = !p.implicit;
    g.posmajor = p.posmajor;
    g.wgt = p.wgt;
    g.cdim = p.Din;
    g.nb16 = p.Nimg / 16;
    g.P = p.P; g.Q = p.Q; g.Nimg = p.Nimg;
    g.Himg = p.Himg; g.Wimg = p.Wimg;
    g.ntiles_n = p.ntiles_n;
    g.total_stages = 6 * p.kblocks;
    g.chunks_per_split = cps;
    g.direct = (split > 1 || raw) ? 0 : 1;
    g.colmajor = p.colmajor;
    g.zeros_kept = zeros_kept ? 1 : 0;
    g.a_box_bytes = 32u * (uint32_t)p.R;
    g.packB = (const uint8_t *)packB;
    g.partial = raw && split <= 1 ? raw : partial;
    g.raw = raw;
    for (int i = 0; i < 6; i++) {
        g.out[i] = raw ? nullptr : out[i];
        g.bias[i] = bias ? bias[i] : nullptr;
    }
    g.d = 1ull << trunc;
    g.dshift = pow2_shift<uint64_t>(g.d);
    g.err = device_error_word(c);
    g.wait_ns = c->wait_ns;
    g.withhold = c->withhold_stage;
    g.lag = issue_lag();
    g.order = issue_order();
    if (c->lsched_order >= 0) {  // a timing run of the schedule tuner
        g.order = c->lsched_order;
        g.lag = c->lsched_lag;
    } else if (!schedule_from_env()) {
        auto it = c->split_cache.find("lsched/" + tune_key(p));
        if (it != c->split_cache.end()) {
            g.order = it->second.first ? 1 : 0;
            g.lag = it->second.second < 0 ? 0 : it->second.second > STAGES - 1 ? STAGES - 1 : it->second.second;
        }
    }
    for (int s = 0; s < 6; s++) g.seg_block[s] = shared ? ((s + 1) >> 1) % 3 : s;
    g.rep_flag = (shared || p.wgt) ? nullptr : rep_flag;  // the weight-gradient image keeps six blocks
    if (split > 1 && !partial) return set_error(c, PG_ERR_INVALID_ARG, "split-K needs a partial buffer");
    // value shares by tensor-map stores: the network's convolutions (no bias,
    // zero shares kept, row-major output of an even width of at least one N tile)
    alignas(64) CUtensorMap tmo[2];
    memset(tmo, 0, sizeof(tmo));
    g.tma_out = 0;
    // (every box dimension within its tensor dimension, tile origins never negative)
    if (g.direct && !raw && !p.colmajor && zeros_kept && !bias && p.N >= BN && p.N % 2 == 0 &&
        (p.implicit || p.Nt <= p.M) && !((uintptr_t)out[0] & 15) && !((uintptr_t)out[5] & 15)) {
        cuuint64_t od[4], os[3];
        cuuint32_t ob[4];
        const cuuint64_t rowb = (cuuint64_t)p.N * 8;
        if (p.implicit) {
            od[0] = p.N; od[1] = p.Q; od[2] = p.P; od[3] = p.Nimg;
            os[0] = rowb; os[1] = rowb * p.Q; os[2] = rowb * p.Q * p.P;
            ob[0] = BN; ob[1] = p.Wt; ob[2] = p.Ht; ob[3] = p.Nt;
        } else {
            od[0] = p.N; od[1] = p.M; od[2] = 1; od[3] = 1;
            os[0] = rowb; os[1] = rowb * p.M; os[2] = rowb * p.M;
            ob[0] = BN; ob[1] = p.Nt; ob[2] = 1; ob[3] = 1;
        }
        const cuuint32_t oe[4] = {1, 1, 1, 1};
        bool ok = true;
        for (int k = 0; k < 2 && ok; k++)
            ok = enc(&tmo[k], CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, out[k ? 5 : 0], od, os, ob, oe,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        if (ok) g.tma_out = 1;
    }
    g.tiles_m = p.tiles_m;
    g.nsplit = split;
    const long long items = (long long)p.ntiles_n * p.tiles_m * split;
    if (items > INT_MAX) return set_error(c, PG_ERR_UNSUPPORTED, "%lld work items", items);
    g.n_items = (int)items;
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    const int ctas = persistent_ctas(sms);
    dim3 grid((unsigned)(persistent_grid() && items > ctas ? ctas : items));
    // the item lists depend only on the plan, the split and the grid: built once per
    // shape (the kernel parameter is copied at launch)
    static std::unordered_map<std::string, std::unique_ptr<Sched>> sc_cache;
    static std::mutex sc_mu;
    std::lock_guard<std::mutex> sc_lock(sc_mu);
    char sk[320];  // every field item_geometry reads, the split and the grid
    snprintf(sk, sizeof(sk), "%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d", g.ntiles_n,
             g.tiles_m, g.tiles_w, g.tiles_h, g.Wt, g.Ht, g.Nt, g.f, g.pad, g.Himg, g.Wimg, g.P, g.Q, g.cblocks, g.nb16,
             g.kblocks, g.total_stages, g.chunks_per_split, g.wgt, g.posmajor, g.nsplit, g.n_items, (int)grid.x,
             g.Nimg);
    std::unique_ptr<Sched> &sc = sc_cache[sk];
    if (!sc) {
        sc.reset(new Sched);
        build_schedule(g, (int)grid.x, *sc);
    }
    limb_tma_kernel<<<grid, NTHREADS, smem_bytes(), c->stream>>>(tm, tmo[0], tmo[1], g, *sc);
    c->launches++;
    int st = launch_status(c, "limb_tma_kernel");
    if (st) return st;
    if (split > 1) {
        const long long total = (long long)p.M * p.N;
        const int sms = c->sm_count > 0 ? c->sm_count : 148;
        long long blocks = (total + 255) / 256;
        if (blocks > (long long)sms * 8) blocks = (long long)sms * 8;
        reduce_kernel<<<(unsigned)blocks, 256, 0, c->stream>>>(g, split);
        c->launches++;
        st = launch_status(c, "reduce_kernel");
    }
    return st;
}

}  // namespace lt

// --------------------------------------------------- standalone entry points

// shared: a's six buffers hold a replicated sharing (Ctx::rep_a / rep_b)
static int run_with_scratch(Ctx *c, const lt::Plan &p, const uint64_t *const a[6], const uint64_t *const b[6],
                            uint64_t *const out[6], const uint64_t *const bias[6], int trunc, bool shared = false) {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    int split, cps;
    const size_t ib = al(p.image_bytes), pb = al(p.packB_bytes);
    const size_t qb = al(lt::tune_partial_bytes(p, c->sm_count > 0 ? c->sm_count : 148));
    uint8_t *scr = (uint8_t *)scratch(c, ib + pb + qb);
    if (!scr) return PG_ERR_NO_MEMORY;
    uint64_t *part = (uint64_t *)(scr + ib + pb);
    int st = lt::run_image(c, p, a, scr, shared);
    if (!st) st = lt::run_pack(c, p, b, scr + ib);
    if (!st) st = lt::tune_split(c, p, scr, scr + ib, part, out, bias, trunc, false, nullptr, split, cps, shared);
    if (!st)
        st = lt::run_gemm(c, p, scr, scr + ib, split > 1 ? part : nullptr, split, cps, out, bias, trunc, false,
                          nullptr, shared);
    if (st) return st;
    comm_msg(c, 2ull * p.M * p.N * 8, 2ull * p.M * p.N * 8);
    comm_round(c);
    return PG_OK;
}

static int limb3_rss_matmul_impl(Ctx *c, const uint64_t *const a[6], const uint64_t *const b[6],
                                 uint64_t *const out[6], const uint64_t *const bias[6], int M, int N, int K, int tA,
                                 int tB, int tC, int trunc) {
    CSh6<uint64_t> ca, cb;
    Sh6<uint64_t> co;
    if (!load6(ca, a) || !load6(cb, b) || !load6(co, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    lt::Plan p;
    int st = lt::plan_gemm(c, p, M, N, K, tA, tB, tC);
    if (st) return st;
    return run_with_scratch(c, p, a, b, out, bias, trunc, c->rep_a);
}

static int limb3_rss_conv_impl(Ctx *c, const uint64_t *const A[6], const uint64_t *const B[6], uint64_t *const C[6],
                               int op, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad,
                               int trunc, bool wgrad_implicit) {
    CSh6<uint64_t> ca, cb;
    Sh6<uint64_t> co;
    if (!load6(ca, A) || !load6(cb, B) || !load6(co, C)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    if (op < 0 || op > 2) return set_error(c, PG_ERR_INVALID_ARG, "bad conv operator %d", op);
    lt::Plan p;
    int st;
    if (op == PG_CONV_FPROP) {
        if ((st = lt::plan_conv(c, p, batch, H, W, f, Din, Dout, stride, pad))) return st;
        return run_with_scratch(c, p, A, B, C, nullptr, trunc, c->rep_a);
    }
    if (op == PG_CONV_WGRAD) {
        // dW[Dout][r][s][c] = sum over output pixels of dY x im2col(X): A is
        // dY, B the forward input; the GEMM takes the forward input as its row
        // operand (the sum over the three parties of x_p0 (y_p0 + y_p1) + x_p1
        // y_p0 does not change when x and y trade places)
        if ((st = lt::plan_wgrad(c, p, batch, H, W, f, Din, Dout, stride, pad, wgrad_implicit))) return st;
        return run_with_scratch(c, p, B, A, C, nullptr, trunc, c->rep_b);
    }
    // dX = col2im(dY x W): the per-tap products of every output pixel as one
    // GEMM (M = output pixels, N = f * f * Din, K = Dout), kept as untruncated
    // Z, then summed into the input pixels and truncated once
    if (batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Din <= 0 || Dout <= 0 || stride <= 0 || pad < 0 ||
        H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "convolution: bad geometry");
    const int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    const long long Mcols = (long long)batch * P * Q;
    if (Mcols > (1ll << 30) || (long long)f * f * Din > (1ll << 30))
        return set_error(c, PG_ERR_UNSUPPORTED, "input gradient of %lld output pixels", Mcols);
    if ((st = lt::plan_gemm(c, p, (int)Mcols, f * f * Din, Dout, 1, 1, 1))) return st;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    int split, cps;
    const size_t ib = al(p.image_bytes), pb = al(p.packB_bytes);
    const size_t qb = al(lt::tune_partial_bytes(p, c->sm_count > 0 ? c->sm_count : 148));
    const size_t cb_bytes = al((size_t)p.M * p.N * 8);
    uint8_t *scr = (uint8_t *)scratch(c, ib + pb + qb + cb_bytes);
    if (!scr) return PG_ERR_NO_MEMORY;
    uint64_t *part = (uint64_t *)(scr + ib + pb);
    uint64_t *cols = (uint64_t *)(scr + ib + pb + qb);
    if ((st = lt::run_image(c, p, A, scr, c->rep_a))) return st;
    if ((st = lt::run_pack(c, p, B, scr + ib))) return st;
    if ((st = lt::tune_split(c, p, scr, scr + ib, part, C, nullptr, trunc, false, cols, split, cps, c->rep_a)))
        return st;
    if ((st = lt::run_gemm(c, p, scr, scr + ib, split > 1 ? part : nullptr, split, cps, C, nullptr, trunc, false,
                           cols, c->rep_a)))
        return st;
    lt::Col2ImArgs a2;
    memset(&a2, 0, sizeof(a2));
    a2.cols = cols;
    for (int i = 0; i < 6; i++) a2.out[i] = C[i];
    a2.total = (long long)batch * H * W * Din;
    a2.H = H; a2.W = W; a2.Din = Din; a2.f = f; a2.stride = stride; a2.pad = pad; a2.P = P; a2.Q = Q;
    a2.d = 1ull << trunc;
    a2.dshift = pow2_shift<uint64_t>(a2.d);
    {
        const int sms = c->sm_count > 0 ? c->sm_count : 148;
        long long blocks = (a2.total + 255) / 256;
        if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
        lt::col2im_kernel<<<(unsigned)blocks, 256, 0, c->stream>>>(a2);
        c->launches++;
        if ((st = launch_status(c, "col2im_kernel"))) return st;
    }
    const uint64_t n_out = (uint64_t)a2.total;
    comm_msg(c, 2 * n_out * 8, 2 * n_out * 8);
    comm_round(c);
    return PG_OK;
}

template <typename T>
int rss_matmul(Ctx *, const T *const *, const T *const *, T *const *, const T *const *, int, int, int, int, int, int,
               int);
template <typename T>
int rss_conv(Ctx *, const T *const *, const T *const *, T *const *, int, int, int, int, int, int, int, int, int, int);

// The form of a standalone share-GEMM / convolution in the limb context: the
// context's cached choice for the shape, else (autotuning on, no capture in
// progress) the fastest of the candidates, timed on the call's own operands
// (one warm-up and three runs each; all give the same bits; counters
// restored), else the first candidate. Candidates: the limb form, the plain
// u64 form, and for a weight gradient the limb form with the explicit
// transposed-im2col image besides the implicit one. Small or narrow problems
// (a weight gradient with 25 x 20 outputs, say) can run faster on the CUDA
// cores, and the implicit weight gradient fills only Din of a tile's 128 rows.
// Cached as 1 + the candidate's index.
static int run_picked(Ctx *c, const std::string &key, const std::vector<std::function<int()>> &cand) {
    int choice = 0;
    auto it = c->split_cache.find(key);
    if (it != c->split_cache.end()) {
        choice = it->second.first - 1;
        if (choice < 0 || choice >= (int)cand.size()) choice = 0;
    } else if (c->autotune && cand.size() > 1) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
        if (cs == cudaStreamCaptureStatusNone) {
            uint64_t comm0[9];
            memcpy(comm0, c->comm, sizeof(comm0));
            const uint64_t launches0 = c->launches.load();
            cudaEvent_t e0, e1;
            PG_CHECK_CUDA(c, cudaEventCreate(&e0));
            if (cudaEventCreate(&e1) != cudaSuccess) {
                cudaEventDestroy(e0);
                return set_error(c, PG_ERR_CUDA, "cudaEventCreate failed");
            }
            std::vector<float> ms(cand.size(), 0.f);
            int st = PG_OK;
            for (size_t f = 0; f < cand.size() && !st; f++) {
                for (int r = 0; r < 4 && !st; r++) {
                    if (r == 1 && cudaEventRecord(e0, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
                    if (!st) st = cand[f]();
                }
                if (!st && cudaEventRecord(e1, c->stream) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
                if (!st && cudaEventSynchronize(e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
                if (!st && cudaEventElapsedTime(&ms[f], e0, e1) != cudaSuccess) st = set_error(c, PG_ERR_CUDA, "event");
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            memcpy(c->comm, comm0, sizeof(comm0));
            c->launches.store(launches0);
            if (st) return st;
            // another candidate must beat the first by 3 %
            float best = ms[0];
            for (size_t f = 1; f < cand.size(); f++)
                if (ms[f] < 0.97f * ms[0] && ms[f] < best) {
                    best = ms[f];
                    choice = (int)f;
                }
            c->split_cache[key] = {choice + 1, 1};
        }
    }
    return cand[choice]();
}

int limb3_rss_matmul_u64(Ctx *c, const uint64_t *const a[6], const uint64_t *const b[6], uint64_t *const out[6],
                         const uint64_t *const bias[6], int M, int N, int K, int tA, int tB, int tC, int trunc) {
    const std::string key = "sform/mm/" + std::to_string(M) + "/" + std::to_string(N) + "/" + std::to_string(K) +
                            "/" + std::to_string(tA) + std::to_string(tB) + std::to_string(tC) + (bias ? "b" : "");
    return run_picked(c, key,
                      {[&] { return limb3_rss_matmul_impl(c, a, b, out, bias, M, N, K, tA, tB, tC, trunc); },
                       [&] { return rss_matmul<uint64_t>(c, a, b, out, bias, M, N, K, tA, tB, tC, trunc); }});
}

int limb3_rss_conv_u64(Ctx *c, const uint64_t *const A[6], const uint64_t *const B[6], uint64_t *const C[6], int op,
                       int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    char k[160];
    snprintf(k, sizeof(k), "sform/conv/%d/%d/%d/%d/%d/%d/%d/%d/%d", op, batch, H, W, f, Din, Dout, stride, pad);
    std::vector<std::function<int()>> cand = {
        [&] { return limb3_rss_conv_impl(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc, true); },
        [&] { return rss_conv<uint64_t>(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc); }};
    if (op == PG_CONV_WGRAD && lt::wgrad_implicit_applies(batch, stride))
        cand.push_back(
            [&] { return limb3_rss_conv_impl(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc, false); });
    lt::Plan fp;
    const std::string err0 = c->err;  // a flipped plan that does not apply is not an error of this call
    const bool flip_ok = op == PG_CONV_DGRAD && lt::plan_dgrad_flip(c, fp, batch, H, W, f, Din, Dout, stride, pad) == PG_OK;
    c->err = err0;
    if (flip_ok) {
        // the input gradient as a convolution of dY with the flipped filter (third candidate, timed like the others)
        cand.push_back([&, fp] {
            CSh6<uint64_t> ca, cb;
            Sh6<uint64_t> co;
            if (!load6(ca, A) || !load6(cb, B) || !load6(co, C))
                return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
            if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
            return run_with_scratch(c, fp, A, B, C, nullptr, trunc, c->rep_a);
        });
    }
    return run_picked(c, k, cand);
}

int limb_prepare_current_device(Ctx *c, bool again) { return lt::prepare_device(c, again); }

// limb3_rss_matmul_u64 without a bias, with every scratch byte taken from
// [scr, scr + cap): the digit image of A, the packed weights, and the split-K
// partial sums (used only when they fit too). A problem whose unsplit need
// exceeds cap is refused with PG_ERR_SIZE. It allocates nothing.
int limb_rss_matmul_u64_fixed(Ctx *c, uint8_t *scr, size_t cap, const uint64_t *const a[6],
                              const uint64_t *const b[6], uint64_t *const out[6], int M, int N, int K, int tA, int tB,
                              int tC, int trunc) {
    CSh6<uint64_t> ca, cb;
    Sh6<uint64_t> co;
    if (!load6(ca, a) || !load6(cb, b) || !load6(co, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (trunc < 0 || trunc > 63) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    if (!scr || ((uintptr_t)scr & 255)) return set_error(c, PG_ERR_INVALID_ARG, "scratch must be 256-byte aligned");
    lt::Plan p;
    int st = lt::plan_gemm(c, p, M, N, K, tA, tB, tC);
    if (st) return st;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    int split, cps;
    if (!lt::cached_split(c, p, split, cps)) lt::choose_split(p, c->sm_count > 0 ? c->sm_count : 148, split, cps);
    const size_t ib = al(p.image_bytes), pb = al(p.packB_bytes);
    if (ib + pb + al(lt::partial_bytes(p, split)) > cap) {
        split = 1;
        cps = (6 * p.kblocks + lt::CHUNK_STAGES - 1) / lt::CHUNK_STAGES;
    }
    const size_t need = ib + pb + al(lt::partial_bytes(p, split));
    if (need > cap)
        return set_error(c, PG_ERR_SIZE,
                         "M=%d N=%d K=%d needs %zu bytes of scratch; the fixed scratch holds %zu (the operand image "
                         "takes 96 * K16 * M32 bytes and the packed weights 96 * K16 * N64, with K16, M32 and N64 "
                         "= K, M and N rounded up to 16, 32 and 64)",
                         M, N, K, need, cap);
    st = lt::run_image(c, p, a, scr);
    if (!st) st = lt::run_pack(c, p, b, scr + ib);
    if (!st)
        st = lt::run_gemm(c, p, scr, scr + ib, split > 1 ? (uint64_t *)(scr + ib + pb) : nullptr, split, cps, out,
                          nullptr, trunc);
    if (st) return st;
    comm_msg(c, 2ull * M * N * 8, 2ull * M * N * 8);
    comm_round(c);
    return PG_OK;
}

int limb_selftest(Ctx *c, const uint16_t *A, const uint16_t *B, float *D) {
    if (!A || !B || !D) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    lt::selftest_kernel<<<1, 128, 0, c->stream>>>(A, B, D, device_error_word(c));
    c->launches++;
    return launch_status(c, "selftest_kernel");
}

}  // namespace pg
