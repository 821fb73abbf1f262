/*
 * piranha_gb300.h — C ABI of the GB300-native implementation of Piranha's
 * party-local secret-share arithmetic (3-party RSS over Z_2^64 / Z_2^32).
 *
 * All three parties are simulated on one GPU. An RSS tensor of n elements is
 * passed as SIX device pointers, index [party * 2 + share] with party A=0,
 * B=1, C=2 and share 0 = the reference's "shareA", 1 = "shareB" (RSS.h:74-75).
 * Each pointer addresses n contiguous elements. Per-party public data (the
 * output of a reconstruct) is THREE device pointers, one per party.
 *
 * Every call is enqueued on the context's stream and returns an int status
 * (PG_OK = 0). Nothing here exits or asserts: size mismatches and unsupported
 * shapes return PG_ERR_*, and pg_last_error() gives a message. Calls do not
 * synchronize; pg_sync() does. Inter-party messages become reads of the
 * sender's buffer inside the fused kernels; the bytes and rounds a socket
 * would carry are added to the context's counters with the accounting of
 * DeviceData::transmit/receive (src/gpu/DeviceData.h:87-118) and
 * Profiler::add_comm_round (src/util/Profiler.cpp:95-99).
 *
 * A length n = 0 is valid for the elementwise protocol steps (reconstruct,
 * reshare, *=, &=, dividePublic, dReLU, ReLU, selectShare, maxpool, the local
 * operators): nothing is launched, the share pointers may be null (an empty
 * CUDA tensor has none), and the step's rounds are counted with empty
 * messages, as the reference counts the rounds of its empty vectors.
 * maxpool of no rows counts nothing (the reference divides by the row count).
 *
 * Citations point at the Piranha (ucbrise/piranha) source each entry point
 * replaces; paths are relative to that project.
 */
#ifndef PIRANHA_GB300_H
#define PIRANHA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
#define PG_OK 0
#define PG_ERR_INVALID_ARG 1   /* null pointer, negative size, bad enum */
#define PG_ERR_SIZE 2          /* sizes that do not describe a valid problem */
#define PG_ERR_CUDA 3          /* a CUDA runtime call failed */
#define PG_ERR_UNSUPPORTED 4   /* shape outside what a kernel implements */
#define PG_ERR_TIMEOUT 5       /* a bounded device-side wait gave up */
#define PG_ERR_NO_MEMORY 6     /* context scratch could not be allocated */

/* share-GEMM / conv implementation forms */
#define PG_FORM_U64 0          /* plain 64-bit integer CUDA-core kernels */
#define PG_FORM_LIMB_TC 1      /* 8-bit limbs on tcgen05 tensor cores, exact */

/* cutlass::conv::Operator (used by RSS.inl:706-803), redefined locally */
#define PG_CONV_FPROP 0
#define PG_CONV_DGRAD 1
#define PG_CONV_WGRAD 2
/* local RSS operators (pg_rss_local_u64) */
#define PG_OP_ADD 0
#define PG_OP_SUB 1
#define PG_OP_MUL 2
#define PG_OP_XOR 3
#define PG_OP_AND 4
#define PG_OP_SHR 5 /* arithmetic */
#define PG_OP_SHL 6
#define PG_OP_DIV 7 /* DeviceData operator/= only (through double, functors.cuh:33-45,94-105) */
#define PG_OP_SET 8 /* DeviceData fill only */
#define PG_RHS_SCALAR 0 /* one public value */
#define PG_RHS_PUBLIC 1 /* a public device vector of n (DeviceData) */
#define PG_RHS_SHARES 2 /* another share tensor (six buffers) */

typedef struct pg_ctx pg_ctx;

/* ------------------------------------------------------------------ context
 * Replaces the reference's process-global state (partyNum, PrecomputeObject,
 * comm_profiler/func_profiler; src/main.cu:34-38) with an explicit handle. */
int pg_ctx_create(pg_ctx **out, int device);
int pg_ctx_destroy(pg_ctx *ctx);
int pg_ctx_set_stream(pg_ctx *ctx, void *cuda_stream);
void *pg_ctx_get_stream(pg_ctx *ctx);
/* The form of the share-GEMMs and convolutions. A new context uses
 * PG_FORM_LIMB_TC, in which (with autotuning on) the first call of each
 * problem shape times both forms and keeps the faster one for that shape;
 * PG_FORM_U64 sends every call to the CUDA-core kernels. */
int pg_ctx_set_form(pg_ctx *ctx, int form);
int pg_ctx_get_form(pg_ctx *ctx);
/* split-K of the limb-form GEMMs picked by timing the candidates on first use
 * of each problem shape (default on; off = the heuristic, and the cache is
 * cleared). Never tunes inside a stream capture. */
int pg_ctx_set_autotune(pg_ctx *ctx, int on);
/* The tuned choices as a text file (first line "pg-tune <SM count>"; a file
 * from a GPU with another SM count is refused). With the environment variable
 * PG_TUNE_CACHE set to a path, every context loads it when created and
 * merges its own choices into it when destroyed. */
int pg_tune_load(pg_ctx *ctx, const char *path);
int pg_tune_save(pg_ctx *ctx, const char *path);
/* Device share buffers, as the reference's share classes own them (RSS<T>:
 * 6 buffers [party*2 + share], TPC<T>: 2, FPC<T>: 12 [party*3 + share];
 * DeviceData.h:51-85): nbuf zeroed buffers of n elements of elem_bytes (1, 4
 * or 8) each, 256-byte aligned, in one allocation that pg_free_shares(out[0])
 * releases. */
int pg_alloc_shares(pg_ctx *ctx, int nbuf, size_t n, int elem_bytes, void **out);
int pg_free_shares(pg_ctx *ctx, void *first);
const char *pg_last_error(pg_ctx *ctx);
int pg_sync(pg_ctx *ctx);
/* counters: out[0..3] = bytes sent by party 0..3, out[4..7] = bytes received,
 * out[8] = communication rounds (src/util/Profiler.cpp:95-128) */
int pg_comm_get(pg_ctx *ctx, uint64_t out[9]);
int pg_comm_reset(pg_ctx *ctx);
/* number of kernels this library launched through ctx (all streams) */
uint64_t pg_kernel_launches(pg_ctx *ctx);
/* synchronize, then report (and clear) the device error word that bounded
 * device-side waits set when they give up: PG_ERR_TIMEOUT with *code != 0 */
int pg_device_errors(pg_ctx *ctx, int *code);
/* Host only: the reference's weight initialisation (FCLayer::initialize,
 * src/nn/FCLayer.cu:31-47; CNNLayer::initialize, src/nn/CNNLayer.cu:36-50):
 * n draws of std::normal_distribution<double>(0, std_dev) from
 * std::default_random_engine(seed), the layer's seed being nn_seed + layer
 * index (src/nn/NeuralNetwork.cu:32-48) and std_dev = sqrt(2 / fan_in). */
int pg_reference_init_normal(double *out, size_t n, int seed, double std_dev);
/* Stream capture of any sequence of calls on ctx into one CUDA graph (the
 * reference launches every kernel eagerly; this is the replacement for its
 * per-op launch overhead). Run the same sequence eagerly once first: that
 * sizes the context's scratch, which cannot be allocated inside a capture.
 * Every pointer the calls received stays baked into the graph. Capture does no
 * work and adds nothing to the counters; each launch adds the communication
 * and kernel counts of the captured calls. A graph lives until
 * pg_graph_destroy and must not outlive its context. */
typedef struct pg_graph pg_graph;
int pg_graph_begin(pg_ctx *ctx);
int pg_graph_end(pg_ctx *ctx, pg_graph **out);
int pg_graph_launch(pg_ctx *ctx, pg_graph *graph);
int pg_graph_destroy(pg_graph *graph);
/* Failure detection, no counterpart in the reference (whose socket errors
 * print and whose error() exits, src/util/connect.h:44-55, util.cu:18-21).
 * wait_ns bounds every device-side wait of the limb tensor-core kernels
 * (default 2 s; 0 restores it): a wait that runs out makes the kernel set the
 * device error word, stop issuing, wait (bounded) for its own copies and MMAs,
 * free its tensor memory and return, and pg_device_errors then reports
 * PG_ERR_TIMEOUT; the context stays usable. withhold_stage >= 0 is a
 * diagnostic for testing that path: the limb GEMM's producer issues no copies
 * for that K stage of each CTA, so its consumers' waits run out (-1 is off). */
int pg_ctx_set_wait_limit(pg_ctx *ctx, uint64_t wait_ns, int withhold_stage);
/* diagnostic: one 128x64x16 tcgen05 MMA of fp16 operands (A 128x16 and B
 * 64x16 row-major halves), D = A * B^T as 128x64 fp32 row-major */
int pg_tc_selftest(pg_ctx *ctx, const uint16_t *A, const uint16_t *B, float *D);
/* Measurement, no counterpart in the reference (whose GEMMs are CUDA-core
 * SIMT): the sustained rate of one tensor-core instruction form on ctx's
 * device, from one launch over every SM after a shorter warm-up launch.
 * out[0] = tera-operations per second (2 per multiply-add), out[1] = SM
 * cycles per instruction per issuing CTA (tcgen05) or warp (mma.sync),
 * out[2] = the timed launch in ms. Synchronizes. tcgen05.mma kind::i8 does
 * not exist for sm_103a (ptxas rejects it), so the only INT8 tensor form on a
 * GB300 is the legacy mma.sync one. */
#define PG_RATE_TC_F16 0  /* tcgen05.mma kind::f16, M=128 N=256 K=16, fp32 in tensor memory */
#define PG_RATE_TC_F8 1   /* tcgen05.mma kind::f8f6f4 e4m3, M=128 N=256 K=32, fp32 */
#define PG_RATE_MMA_S8 2  /* mma.sync m16n8k32 s8 x s8 -> s32 */
#define PG_RATE_MMA_F16 3 /* mma.sync m16n8k16 f16 x f16 -> f32 */
int pg_tensor_rate(pg_ctx *ctx, int form, int iters, double out[3]);

/* -------------------------------------------- single-array ring kernels
 * gpu::gemm (src/gpu/gemm.cuh:102-112): C = A*B mod 2^w, A MxK, B KxN, C MxN;
 * an operand is row-major when its transpose flag is set, column-major
 * otherwise (gemm.cuh:64-100). */
int pg_gemm_u64(pg_ctx *ctx, int M, int N, int K, const uint64_t *A, int tA, const uint64_t *B, int tB,
                uint64_t *C, int tC);
int pg_gemm_u32(pg_ctx *ctx, int M, int N, int K, const uint32_t *A, int tA, const uint32_t *B, int tB,
                uint32_t *C, int tC);
/* gpu::conv_fprop / conv_dgrad / conv_wgrad (src/gpu/conv.cuh:359-490):
 * NHWC activations, KRSC filters, cross-correlation, symmetric padding.
 * fprop: a = X (N,H,W,C), b = F (K,R,S,C), out = Y (N,P,Q,K)
 * dgrad: a = dY (N,P,Q,K), b = F (K,R,S,C), out = dX (N,H,W,C)
 * wgrad: a = dY (N,P,Q,K), b = X (N,H,W,C), out = dF (K,R,S,C) */
int pg_conv_u64(pg_ctx *ctx, int op, int N, int H, int W, int C, int K, int R, int S, int pad, int stride,
                const uint64_t *a, const uint64_t *b, uint64_t *out);

/* --------------------------------------------------------- RSS protocol
 * matmul (src/mpc/RSS.inl:482-540 with localMatMul :1097-1110 and
 * dividePublic3out3 :1077-1094): per party z = A0*(B0+B1) + A1*B0 computed
 * as one contraction over the concatenated K of all three parties, revealed
 * 3-out-of-3 and truncated by 2^trunc in the epilogue. */
int pg_rss_matmul_u64(pg_ctx *ctx, const uint64_t *const a[6], const uint64_t *const b[6], uint64_t *const c[6],
                      int M, int N, int K, int tA, int tB, int tC, int trunc);
int pg_rss_matmul_u32(pg_ctx *ctx, const uint32_t *const a[6], const uint32_t *const b[6], uint32_t *const c[6],
                      int M, int N, int K, int tA, int tB, int tC, int trunc);
/* FCLayer::forward (src/nn/FCLayer.cu:78-130): matmul(tA=tB=tC=1, FP) followed
 * by elementVectorAdd of the bias shares, fused into one launch. bias may be
 * NULL (no bias). */
int pg_rss_fc_forward_u64(pg_ctx *ctx, const uint64_t *const x[6], const uint64_t *const w[6],
                          const uint64_t *const bias[6], uint64_t *const out[6], int batch, int din, int dout,
                          int fp);
/* convolution (src/mpc/RSS.inl:706-803): the three party-local convolutions
 * (localFprop/Dgrad/Wgrad :614-703) fused as one implicit GEMM over the
 * concatenated K, then the 3-out-of-3 truncation. Argument roles follow the
 * reference: fprop (im, filter), dgrad (delta, filter), wgrad (delta, input). */
int pg_rss_conv_u64(pg_ctx *ctx, const uint64_t *const A[6], const uint64_t *const B[6], uint64_t *const C[6],
                    int op, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc);
/* dividePublic(RSS&, T) and dividePublic(RSS&, DeviceData&) (RSS.inl:423-455) */
int pg_rss_divide_public_u64(pg_ctx *ctx, uint64_t *const a[6], size_t n, uint64_t d);
int pg_rss_divide_public_vec_u64(pg_ctx *ctx, uint64_t *const a[6], size_t n, const uint64_t *d);
int pg_rss_divide_public_u32(pg_ctx *ctx, uint32_t *const a[6], size_t n, uint32_t d);
/* reconstruct (RSS.inl:458-479): out[p] = a_p0 + a_p1 + a_{prev(p)}0 */
int pg_rss_reconstruct_u64(pg_ctx *ctx, const uint64_t *const a[6], size_t n, uint64_t *const out[3]);
int pg_rss_reconstruct_u8(pg_ctx *ctx, const uint8_t *const a[6], size_t n, uint8_t *const out[3]);
/* reshare (RSS.inl:1053-1074): out_p = (c_p, c_{next(p)}) */
/* Counter-mode AES generator of AESObject (src/mpc/AESObject.cpp:9-91):
 * block k = AES-256-ECB_key(LE64(k) || LE64(k)); out[j] = 64-bit lane (j & 1)
 * of block counter + j / 2, i.e. the uint64 stream of getRandom from that
 * counter. The key is the first 32 bytes of the reference's key file (its
 * text up to the first NUL, zero-padded). Device output. */
int pg_prg_fill_u64(pg_ctx *ctx, const uint8_t key[32], uint64_t counter, uint64_t *out, size_t n);
/* Live resharing masks (the reference leaves rndMask = c, RSS.inl:1053-1074):
 * keys = 3 x 32 bytes, key p shared by party p and party p+1; reshare, *= and
 * &= then add alpha_p = G(key p) - G(key p-1) to party p's value (XOR of the
 * low bits for u8 bit shares, full-width XOR for u64 &=), which sums to zero,
 * drawing from one context counter that starts at `counter` and advances by
 * ceil(n / 2) blocks per step. keys = NULL turns them off. The fused dReLU /
 * ReLU / maxpool kernels and the GEMM epilogues keep the reference's masks. */
int pg_prg_set_keys(pg_ctx *ctx, const uint8_t *keys, uint64_t counter);
int pg_prg_counter(pg_ctx *ctx, uint64_t *counter);
int pg_rss_reshare_u64(pg_ctx *ctx, const uint64_t *const c[3], size_t n, uint64_t *const out[6]);
/* The local (communication-free) operators of RSSBase (RSS.inl:168-345), in
 * place on a: `a op= rhs` for rhs a public scalar (+ - * >>), a public device
 * vector (+ - * ^ & >> <<) or another share tensor (+ - ^). Public + - ^ touch
 * party A's shareA and party C's shareB only; * & and shifts touch every share;
 * share-tensor + - ^ go share by share. >> is arithmetic (functors.cuh:48-70);
 * shift amounts of 64 or more give all sign bits (>>) or 0 (<<). Other
 * combinations return PG_ERR_UNSUPPORTED (RSS * RSS and & are pg_rss_mul_u64 /
 * pg_rss_and_u64). */
/* DeviceData<uint64_t>'s own elementwise operators on one device array
 * (src/gpu/DeviceData.h:131-277, src/gpu/functors.cuh:1-117): a op= rhs for
 * op in ADD SUB MUL DIV XOR AND SHR SHL with rhs a scalar (PG_RHS_SCALAR) or
 * a device vector of n (PG_RHS_PUBLIC), and fill (PG_OP_SET, scalar). DIV is
 * the reference's division through double; SHR is arithmetic. */
int pg_device_op_u64(pg_ctx *ctx, int op, uint64_t *a, size_t n, int rhs_kind, uint64_t scalar,
                     const uint64_t *rhs);
int pg_rss_local_u64(pg_ctx *ctx, int op, uint64_t *const a[6], size_t n, int rhs_kind, uint64_t scalar,
                     const uint64_t *pub, const uint64_t *const shares[6]);
/* the same local operators of TPCBase (TPC.inl:146-240; public values at
 * party A's share) and FPCBase (FPC.inl:187-300; public values in the x0
 * component: party B's shareC, party C's shareB, party D's shareA) */
int pg_tpc_local_u64(pg_ctx *ctx, int op, uint64_t *const a[2], size_t n, int rhs_kind, uint64_t scalar,
                     const uint64_t *pub, const uint64_t *const shares[2]);
int pg_fpc_local_u64(pg_ctx *ctx, int op, uint64_t *const a[12], size_t n, int rhs_kind, uint64_t scalar,
                     const uint64_t *pub, const uint64_t *const shares[12]);
/* RSS *= RSS and RSS &= RSS (RSS.inl:284-345), in place on a */
int pg_rss_mul_u64(pg_ctx *ctx, uint64_t *const a[6], const uint64_t *const b[6], size_t n);
int pg_rss_and_u64(pg_ctx *ctx, uint64_t *const a[6], const uint64_t *const b[6], size_t n);
int pg_rss_and_u8(pg_ctx *ctx, uint8_t *const a[6], const uint8_t *const b[6], size_t n);
/* dReLU (RSS.inl:807-852): result bit shares; carries of the bit-decomposition
 * circuit (carryOut :1113-1209) evaluated on bit-packed 64-bit words */
int pg_rss_drelu_u64_u8(pg_ctx *ctx, const uint64_t *const in[6], size_t n, uint8_t *const out[6]);
int pg_rss_drelu_u64_u64(pg_ctx *ctx, const uint64_t *const in[6], size_t n, uint64_t *const out[6]);
/* ReLU (RSS.inl:855-865) = dReLU + selectShare(0, x, d), one fused launch */
int pg_rss_relu_u64_u8(pg_ctx *ctx, const uint64_t *const in[6], size_t n, uint64_t *const out[6],
                       uint8_t *const dout[6]);
int pg_rss_relu_u64_u64(pg_ctx *ctx, const uint64_t *const in[6], size_t n, uint64_t *const out[6],
                        uint64_t *const dout[6]);
int pg_rss_relu_u32_u8(pg_ctx *ctx, const uint32_t *const in[6], size_t n, uint32_t *const out[6],
                       uint8_t *const dout[6]);
/* selectShare (RSS.inl:543-569): z = b ? y : x via the revealed bit */
int pg_rss_select_share_u64_u8(pg_ctx *ctx, const uint64_t *const x[6], const uint64_t *const y[6],
                               const uint8_t *const b[6], uint64_t *const z[6], size_t n);
int pg_rss_select_share_u64_u64(pg_ctx *ctx, const uint64_t *const x[6], const uint64_t *const y[6],
                                const uint64_t *const b[6], uint64_t *const z[6], size_t n);
/* maxpool (RSS.inl:868-1017) over rows of k contiguous values (k = 4 or 16);
 * in is n = rows * k values, out rows values, dout n bit shares */
int pg_rss_maxpool_u64_u8(pg_ctx *ctx, const uint64_t *const in[6], size_t n, int k, uint64_t *const out[6],
                          uint8_t *const dout[6]);
int pg_rss_maxpool_u64_u64(pg_ctx *ctx, const uint64_t *const in[6], size_t n, int k, uint64_t *const out[6],
                           uint64_t *const dout[6]);
/* MaxpoolLayer::forward (src/nn/MaxpoolLayer.cu:52-131): maxpool_im2row
 * windows (reference N,W,H,C indexing), power-of-two padding with
 * -10 * 2^fp, tournament, truncate_cols; one fused launch. out has
 * batch*P*Q*C values, maxprime batch*P*Q*C*pool*pool bit shares
 * (maxprime == NULL: the bit shares, which only the backward reads, are
 * not written). */
int pg_rss_maxpool_layer_u64_u8(pg_ctx *ctx, const uint64_t *const in[6], uint64_t *const out[6],
                                uint8_t *const maxprime[6], int H, int W, int C, int pool, int stride, int batch,
                                int fp);

/* AveragepoolLayer::forward (src/nn/AveragepoolLayer.cu:58-81): the sum of
 * each pool window (averagepool_im2row, src/gpu/convolution.cuh:340-374, with
 * its kernel's width/height swap) and dividePublic by pool^2; and ::backward
 * (:88-117): averagepool_expand_delta (convolution.cuh:195-208) then / pool^2.
 * in/deltas are batch x H x W x C, out/delta the pooled shape. The backward
 * needs non-overlapping pools (stride >= pool): the reference's expansion
 * writes past the gradient buffer otherwise, here PG_ERR_UNSUPPORTED. */
int pg_rss_avgpool_layer_u64(pg_ctx *ctx, const uint64_t *const in[6], uint64_t *const out[6], int H, int W, int C,
                             int pool, int stride, int batch);
int pg_rss_avgpool_backward_u64(pg_ctx *ctx, const uint64_t *const delta[6], uint64_t *const deltas[6], int H, int W,
                                int C, int pool, int stride, int batch);
/* ------------------------------------------------------- glue kernels
 * elementVectorAdd (src/gpu/matrix.cuh:75-84), reduceSum (:109-126),
 * truncate_cols (:141-154), bitexpand (src/gpu/bitwise.cuh:10-21),
 * expandCompare (:66-92), maxpool_im2row + stride_pad
 * (src/gpu/convolution.cuh:56-108,175-191,252-304) */
int pg_element_vector_add_u64(pg_ctx *ctx, uint64_t *a, const uint64_t *b, int rowwise, int rows, int cols);
int pg_reduce_sum_u64(pg_ctx *ctx, const uint64_t *a, uint64_t *b, int reduce_rows, int rows, int cols);
int pg_truncate_cols_u8(pg_ctx *ctx, const uint8_t *a, uint8_t *b, size_t rows, int start_cols, int end_cols);
int pg_bitexpand_u64(pg_ctx *ctx, const uint64_t *a, size_t n, uint64_t *bits);
int pg_expand_compare_u8(pg_ctx *ctx, const uint8_t *b, const uint8_t *nb, size_t n, uint8_t *out,
                         size_t out_n);
int pg_maxpool_im2row_u64(pg_ctx *ctx, const uint64_t *im, uint64_t *out, int H, int W, int f, int Din,
                          int batch, int stride, int pad, uint64_t pad_val);

/* --------------------------------------------------------- TPC (2PC) protocol
 * src/mpc/TPC.h, TPC.inl: two-party additive shares. A TPC tensor of n
 * elements is TWO device pointers, [party A, party B], each n elements; its
 * value is their sum. The reference's multiplications use constant Beaver
 * triples (src/mpc/Precompute.h), and its results land in party A's share
 * with party B's 0; these entry points produce the same shares bit for bit.
 * Counters add the bytes and rounds of every reveal the reference makes. */
/* matmul (TPC.inl:575-583, localMatMul :1060-1091): reveal a and b masked,
 * multiply, dividePublic by 2^trunc */
int pg_tpc_matmul_u64(pg_ctx *ctx, const uint64_t *const a[2], const uint64_t *const b[2], uint64_t *const c[2],
                      int M, int N, int K, int tA, int tB, int tC, int trunc);
int pg_tpc_matmul_u32(pg_ctx *ctx, const uint32_t *const a[2], const uint32_t *const b[2], uint32_t *const c[2],
                      int M, int N, int K, int tA, int tB, int tC, int trunc);
/* FCLayer::forward (src/nn/FCLayer.cu:78-130) for TPC: matmul(tA=tB=tC=1, FP)
 * then each party adds its bias share; bias may be NULL */
int pg_tpc_fc_forward_u64(pg_ctx *ctx, const uint64_t *const x[2], const uint64_t *const w[2],
                          const uint64_t *const bias[2], uint64_t *const out[2], int batch, int din, int dout, int fp);
int pg_tpc_fc_forward_u32(pg_ctx *ctx, const uint32_t *const x[2], const uint32_t *const w[2],
                          const uint32_t *const bias[2], uint32_t *const out[2], int batch, int din, int dout, int fp);
/* convolution (TPC.inl:789-827 with localFprop/Dgrad/Wgrad :645-787) */
int pg_tpc_conv_u64(pg_ctx *ctx, const uint64_t *const A[2], const uint64_t *const B[2], uint64_t *const C[2],
                    int op, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc);
/* dividePublic (TPC.inl:371-401), in place */
int pg_tpc_divide_public_u64(pg_ctx *ctx, uint64_t *const a[2], size_t n, uint64_t d);
int pg_tpc_divide_public_vec_u64(pg_ctx *ctx, uint64_t *const a[2], size_t n, const uint64_t *d);
int pg_tpc_divide_public_u32(pg_ctx *ctx, uint32_t *const a[2], size_t n, uint32_t d);
/* reconstruct (TPC.inl:552-572): out[p] = a_A + a_B for both parties */
int pg_tpc_reconstruct_u64(pg_ctx *ctx, const uint64_t *const a[2], size_t n, uint64_t *const out[2]);
int pg_tpc_reconstruct_u32(pg_ctx *ctx, const uint32_t *const a[2], size_t n, uint32_t *const out[2]);
int pg_tpc_reconstruct_u8(pg_ctx *ctx, const uint8_t *const a[2], size_t n, uint8_t *const out[2]);
/* TPC *= TPC (TPC.inl:242-272), in place on a */
int pg_tpc_mul_u64(pg_ctx *ctx, uint64_t *const a[2], const uint64_t *const b[2], size_t n);
/* dReLU (TPC.inl:829-868), ReLU (:871-884), selectShare (:586-610),
 * maxpool over rows of k = 2, 4, 8 or 16 values (:887-1058) */
int pg_tpc_drelu_u64_u8(pg_ctx *ctx, const uint64_t *const in[2], size_t n, uint8_t *const out[2]);
int pg_tpc_drelu_u32_u8(pg_ctx *ctx, const uint32_t *const in[2], size_t n, uint8_t *const out[2]);
int pg_tpc_relu_u64_u8(pg_ctx *ctx, const uint64_t *const in[2], size_t n, uint64_t *const out[2],
                       uint8_t *const dout[2]);
int pg_tpc_relu_u32_u8(pg_ctx *ctx, const uint32_t *const in[2], size_t n, uint32_t *const out[2],
                       uint8_t *const dout[2]);
int pg_tpc_select_share_u64_u8(pg_ctx *ctx, const uint64_t *const x[2], const uint64_t *const y[2],
                               const uint8_t *const b[2], uint64_t *const z[2], size_t n);
int pg_tpc_maxpool_u64_u8(pg_ctx *ctx, const uint64_t *const in[2], size_t n, int k, uint64_t *const out[2],
                          uint8_t *const dout[2]);

/* --------------------------------------------------------- FPC (4PC) protocol
 * src/mpc/FPC.h, FPC.inl: four-party replicated shares. An FPC tensor of n
 * elements is TWELVE device pointers, index party * 3 + share with parties
 * A..D = 0..3 and shares shareA/shareB/shareC = 0..2; party p's share k holds
 * component x_{(p+1+k) mod 4} of x = x0 + x1 + x2 + x3 (FPC.inl:948-953), and
 * public values live in x0 (B.shareC, C.shareB, D.shareA: FPC.inl:120-155).
 * Every party's arrays come out as the reference computes them at that party,
 * including the reshare's per-party cross terms (reshareFPC, FPC.inl:1184-1259).
 * Counters: reconstruct sends n elements from every party to the next (1
 * round); each of a product's six reshares sends n elements from party I to
 * party G (1 round each). */
/* matmul (FPC.inl:636-670): local products, six reshares, dividePublic */
int pg_fpc_matmul_u64(pg_ctx *ctx, const uint64_t *const a[12], const uint64_t *const b[12], uint64_t *const c[12],
                      int M, int N, int K, int tA, int tB, int tC, int trunc);
int pg_fpc_matmul_u32(pg_ctx *ctx, const uint32_t *const a[12], const uint32_t *const b[12], uint32_t *const c[12],
                      int M, int N, int K, int tA, int tB, int tC, int trunc);
/* FCLayer::forward (src/nn/FCLayer.cu:78-130) for FPC: matmul(tA=tB=tC=1, FP)
 * then every share adds its bias share; bias may be NULL */
int pg_fpc_fc_forward_u64(pg_ctx *ctx, const uint64_t *const x[12], const uint64_t *const w[12],
                          const uint64_t *const bias[12], uint64_t *const out[12], int batch, int din, int dout, int fp);
int pg_fpc_fc_forward_u32(pg_ctx *ctx, const uint32_t *const x[12], const uint32_t *const w[12],
                          const uint32_t *const bias[12], uint32_t *const out[12], int batch, int din, int dout, int fp);
/* convolution (FPC.inl:862-925 with localFprop/Dgrad/Wgrad :745-860) */
int pg_fpc_conv_u64(pg_ctx *ctx, const uint64_t *const A[12], const uint64_t *const B[12], uint64_t *const C[12],
                    int op, int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc);
/* dividePublic (FPC.inl:576-608), in place */
int pg_fpc_divide_public_u64(pg_ctx *ctx, uint64_t *const a[12], size_t n, uint64_t d);
int pg_fpc_divide_public_vec_u64(pg_ctx *ctx, uint64_t *const a[12], size_t n, const uint64_t *d);
int pg_fpc_divide_public_u32(pg_ctx *ctx, uint32_t *const a[12], size_t n, uint32_t d);
/* reconstruct (FPC.inl:611-634): out[p] = party p's three shares plus the
 * previous party's shareA, for the four parties */
int pg_fpc_reconstruct_u64(pg_ctx *ctx, const uint64_t *const a[12], size_t n, uint64_t *const out[4]);
int pg_fpc_reconstruct_u32(pg_ctx *ctx, const uint32_t *const a[12], size_t n, uint32_t *const out[4]);
int pg_fpc_reconstruct_u8(pg_ctx *ctx, const uint8_t *const a[12], size_t n, uint8_t *const out[4]);
/* FPC *= FPC (FPC.inl:322-364) and &= (:375-399), in place on a */
int pg_fpc_mul_u64(pg_ctx *ctx, uint64_t *const a[12], const uint64_t *const b[12], size_t n);
int pg_fpc_and_u8(pg_ctx *ctx, uint8_t *const a[12], const uint8_t *const b[12], size_t n);
/* dReLU (FPC.inl:930-990), ReLU (:992-1003), selectShare (:672-711),
 * maxpool over rows of k values, k a power of two (:1005-1177) */
int pg_fpc_drelu_u64_u8(pg_ctx *ctx, const uint64_t *const in[12], size_t n, uint8_t *const out[12]);
int pg_fpc_drelu_u32_u8(pg_ctx *ctx, const uint32_t *const in[12], size_t n, uint8_t *const out[12]);
int pg_fpc_relu_u64_u8(pg_ctx *ctx, const uint64_t *const in[12], size_t n, uint64_t *const out[12],
                       uint8_t *const dout[12]);
int pg_fpc_relu_u32_u8(pg_ctx *ctx, const uint32_t *const in[12], size_t n, uint32_t *const out[12],
                       uint8_t *const dout[12]);
int pg_fpc_select_share_u64_u8(pg_ctx *ctx, const uint64_t *const x[12], const uint64_t *const y[12],
                               const uint8_t *const b[12], uint64_t *const z[12], size_t n);
int pg_fpc_maxpool_u64_u8(pg_ctx *ctx, const uint64_t *const in[12], size_t n, int k, uint64_t *const out[12],
                          uint8_t *const dout[12]);

/* ---------------------------------------------- share-GEMM without allocation
 * No counterpart in the reference. The same result as pg_rss_matmul_u64, bit
 * for bit, computed by the limb tensor-core kernels, for callers that must not
 * allocate device memory while they run: a host that hands out all device
 * memory from its own pool, a serving loop that cannot stall its other
 * streams on cudaFree's device-wide wait, or one that must not fail with
 * out-of-memory halfway through a request. pg_rss_matmul_u64 grows the
 * context's scratch with cudaMalloc/cudaFree; this call allocates nothing and
 * takes its scratch from one fixed device array of PG_NOALLOC_SCRATCH_BYTES,
 * which the CUDA runtime reserves on a device when it loads the library module
 * that holds it: at the first call on that device under the default lazy
 * module loading, or for every device the process uses, called or not, under
 * CUDA_MODULE_LOADING=EAGER. It stays reserved until the process exits.
 *  - The first call on a device does set-up (finds the array's address, sets
 *    the kernel's shared-memory limit and looks up the tensor-map encoder)
 *    and needs the context's device current. Make it before any stream
 *    capture on that device. Later calls look the address up again (no
 *    allocation) and repeat the set-up if a device reset moved the array.
 *  - The scratch need is 96 * K16 * M32 bytes for the digit image of a plus
 *    96 * K16 * N64 bytes for the packed weights (K16, M32, N64 = K, M, N
 *    rounded up to 16, 32, 64); K = M = N = 1024 fits. A problem that does not
 *    fit returns PG_ERR_SIZE; pg_last_error gives the need and the limit.
 *    Split-K partial sums (8 * split * M * N bytes, rounded up to 256) are used
 *    only when they fit beside those; otherwise the call runs unsplit, which
 *    is slow for few output tiles and a long K.
 *  - All calls on a device, from every context and thread, share the one
 *    array. Calls that can run at the same time on the device (streams with
 *    no ordering between them) corrupt each other's results: order them on
 *    one stream or with events. */
#define PG_NOALLOC_SCRATCH_BYTES ((size_t)256 << 20)
int pg_rss_matmul_u64_noalloc(pg_ctx *ctx, const uint64_t *const a[6], const uint64_t *const b[6],
                              uint64_t *const c[6], int M, int N, int K, int tA, int tB, int tC, int trunc);

/* ------------------------------------------------------ network executor
 * NeuralNetwork::forward (src/nn/NeuralNetwork.cu:109-133) for FC / CNN /
 * ReLU / Maxpool stacks: layers run in order on preallocated share buffers
 * and the whole forward can be captured as one CUDA graph. */
#define PG_LAYER_FC 1      /* p = {din, dout} */
#define PG_LAYER_CNN 2     /* p = {H, W, Din, Dout, f, stride, pad} */
#define PG_LAYER_RELU 3    /* p = {n per image} */
#define PG_LAYER_MAXPOOL 4 /* p = {H, W, C, pool, stride} */
#define PG_LAYER_AVGPOOL 5 /* p = {H, W, C, pool, stride} */

typedef struct pg_net pg_net;
/* spec: nlayers records of 8 ints {type, p0..p6}. Weight/bias shares are
 * copied in later with pg_net_set_params. */
int pg_net_create(pg_ctx *ctx, pg_net **out, const int *spec, int nlayers, int batch, int fp);
int pg_net_destroy(pg_net *net);
/* layer i's weights (and FC bias, may be NULL) as six device pointers each;
 * copies on the context stream and waits for the copies to finish */
int pg_net_set_params(pg_net *net, int layer, const uint64_t *const w[6], const uint64_t *const bias[6]);
size_t pg_net_input_size(pg_net *net);   /* elements per share buffer */
size_t pg_net_output_size(pg_net *net);
/* forward on device-resident shares (six pointers each) */
int pg_net_forward(pg_net *net, const uint64_t *const in[6], uint64_t *const out[6]);
/* the same with host buffers: in_host/out_host are [6][n] contiguous
 * (pinned memory recommended). Asynchronous: the host buffers must stay valid
 * until the context stream is synchronised. Without a captured forward the
 * copies are on the context stream; after pg_net_capture the input goes to
 * one of two input buffer sets on a copy stream, each with its own graph, so
 * that calls queued back to back overlap a call's input copy with the
 * previous call's replay (the output copy follows each replay on the context
 * stream) */
int pg_net_forward_host(pg_net *net, const uint64_t *in_host, uint64_t *out_host);
/* capture the forward (on the network's own input/output buffers) as a CUDA
 * graph, recorded on a private stream; later forwards replay it on the
 * context stream (which may be the legacy default stream) */
int pg_net_capture(pg_net *net);
/* forward on the network's own input buffers (filled by the caller through
 * pg_net_input_shares), replaying the captured graph when there is one */
int pg_net_forward_resident(pg_net *net);
int pg_net_input_shares(pg_net *net, uint64_t *out[6]);
/* per-layer CUDA-event timing (events are recorded into a captured graph
 * too); pg_net_layer_times gives each layer's milliseconds of the last
 * completed forward */
int pg_net_enable_timing(pg_net *net, int on);
int pg_net_layer_times(pg_net *net, float *ms);
/* device pointers (owned by the network) of layer i's output shares.
 * A forward before the training buffers exist (pg_net_train_setup, or any
 * training call) is an inference forward: it writes no ReLU / maxpool bit
 * shares, and a ReLU whose output feeds a limb-form convolution keeps that
 * output only as the convolution's fp16 digit image (exact: the shares are
 * the image's digits). This call then rebuilds the six shares from the image
 * on the context stream and synchronises it before it returns. */
int pg_net_layer_output(pg_net *net, int layer, uint64_t *const out[6], size_t *n);
/* how FC / CNN layer i runs (no counterpart in the reference): out[0] = 1
 * limb tensor-core form, 2 plain u64 form; out[1] = 1 if its tiles are
 * position-major; out[2] = split-K; out[3] = tiles per split. Valid after the
 * first forward (which sets the network up); zeros for other layers. */
int pg_net_layer_plan(pg_net *net, int layer, int out[4]);

/* Training: one SGD iteration (src/main.cu:314-330) = forward, then
 * NeuralNetwork::backward (NeuralNetwork.cu:136-148): the revealed softmax
 * gradient (_reveal_softmax_grad :207-267: each party's logits revealed, the
 * softmax taken in double on the host as the reference does, here as a
 * stream-ordered host function), then every layer's backward from the last
 * (FCLayer.cu:132-217, CNNLayer.cu:114-193, ReLULayer.cu:90-124,
 * MaxpoolLayer.cu:133-185), each updating its weights with learning rate
 * 2^-log_lr. Labels are RSS shares of the one-hot targets, out_n elements
 * per share. Training buffers are allocated by the first training call,
 * which must be eager (not inside a stream capture); needs fp <= 30. */
int pg_net_train_setup(pg_net *net);
int pg_net_train_step(pg_net *net, const uint64_t *const in[6], const uint64_t *const labels[6], int log_lr);
/* backward only, after a forward on the shares in[] (layer 0's weight
 * gradient needs them) that ran after pg_net_train_setup (an inference
 * forward keeps no bit shares: PG_ERR_INVALID_ARG) */
int pg_net_backward(pg_net *net, const uint64_t *const in[6], const uint64_t *const labels[6], int log_lr);
/* the network's own label buffers ([6][out_n] contiguous) */
int pg_net_label_shares(pg_net *net, uint64_t *out[6]);
/* capture forward + backward on the network's own input and label buffers as
 * one CUDA graph (after one eager step whose parameter updates are undone) */
int pg_net_capture_train(pg_net *net, int log_lr);
int pg_net_train_resident(pg_net *net);
/* host buffers: in_host [6][in_n], labels_host [6][out_n]; out_host receives
 * the forward's output shares [6][out_n]; replays the captured step if any */
int pg_net_train_host(pg_net *net, const uint64_t *in_host, const uint64_t *labels_host, uint64_t *out_host,
                      int log_lr);
/* layer i's backward output (the gradient it passes on; layer -1 = the
 * softmax gradient entering the last layer), and its parameter buffers */
int pg_net_layer_delta(pg_net *net, int layer, uint64_t *out[6], size_t *n);
int pg_net_layer_params(pg_net *net, int layer, uint64_t *w[6], uint64_t *b[6], size_t *w_n, size_t *b_n);

/* ----------------------------------------------------- party mode (TCP)
 * One party per process, parties on separate hosts (or processes), messages
 * over TCP exactly as the reference sends them: per ordered pair of parties
 * three connections (NUMCONNECTIONS, src/util/basicSockets.h:35), the
 * receiving party listening on base_port + sender * num_parties + receiver
 * (initializeCommunication, src/util/connect.cu:109-123, base 32000 there),
 * set up in the reference's serial order (initializeCommunicationSerial,
 * :64-80), TCP_NODELAY, and every message the raw bytes of the vector on the
 * first connection, with no header (sendVector / receiveVector,
 * src/util/connect.h:41-55). A reference party process can be a peer.
 * Unlike the reference, which prints and carries on (or waits forever),
 * every call returns a status: a peer that does not connect, a receive that
 * stays short of its length (PG_ERR_TIMEOUT after timeout_ms), a peer that
 * closes its connection (PG_ERR_COMM). */
#define PG_ERR_COMM 7          /* a party message was lost, cut short or duplicated */
typedef struct pg_party pg_party;
int pg_party_create(pg_party **out, int party, int num_parties, const char *const *hosts, int base_port,
                    int timeout_ms);
int pg_party_destroy(pg_party *p);
/* the last error's text; pg_party_last_error(NULL) gives that of this
 * thread's last failed pg_party_create */
const char *pg_party_last_error(pg_party *p);
/* sendVector / receiveVector of bytes of host memory */
int pg_party_send(pg_party *p, int to, const void *data, size_t bytes);
int pg_party_recv(pg_party *p, int from, void *data, size_t bytes);
/* DeviceData::transmit + receive + join (src/gpu/DeviceData.h:87-129): bytes
 * of device memory sent to `to` while bytes_in are received from `from` (a
 * sending thread beside the receiving one, as the reference overlaps them),
 * through pinned host staging, ordered on ctx's stream; to or from may be -1 */
int pg_party_exchange(pg_party *p, pg_ctx *ctx, int to, const void *dev_out, size_t bytes_out, int from,
                      void *dev_in, size_t bytes_in);
/* the party's counters, with the reference's accounting (comm_profiler bytes
 * per transmit / receive, one round per protocol step): out[0..n-1] bytes
 * sent to each party, out[n..2n-1] bytes received from each, out[2n] rounds */
int pg_party_counters(pg_party *p, uint64_t *out);
/* End-of-step check (no counterpart in the reference): every pair of
 * parties swaps its byte counters on the second connection and compares
 * them, and no data may be left unread on the first; PG_ERR_COMM names the
 * peer and the numbers when a message was lost, duplicated or cut short. */
int pg_party_check(pg_party *p);
/* Host-side fault injection for testing the detection: the nth send from now
 * (n >= 1) is dropped (counted, not written), duplicated (written twice) or
 * truncated (half written); PG_FAULT_NONE clears it. */
#define PG_FAULT_NONE 0
#define PG_FAULT_DROP 1
#define PG_FAULT_DUPLICATE 2
#define PG_FAULT_TRUNCATE 3
int pg_party_inject(pg_party *p, int kind, int nth);
/* RSS protocol steps of this party alone, on its two device share buffers
 * sh[0] = shareA, sh[1] = shareB (RSS.h:74-75), with the reference's messages
 * and accounting:
 *  - reconstruct (RSS.inl:457-479): shareA to the next party, the previous
 *    party's shareA received, out = shareA + shareB + received;
 *  - reshare (RSS.inl:1052-1074): out[0] = c sent to the previous party,
 *    out[1] received from the next;
 *  - matmul (RSS.inl:481-540): localMatMul (three gpu::gemm, :1096-1110),
 *    dividePublic3out3 (:1076-1094: r' = 2^trunc taken off at party A,
 *    reconstruct3out3 :1019-1050 with the next and the previous party, the
 *    division through double, r = 1 and the quotient added at party A's
 *    shareA and party C's shareB). */
int pg_party_rss_reconstruct_u64(pg_party *p, pg_ctx *ctx, const uint64_t *const sh[2], size_t n, uint64_t *out);
int pg_party_rss_reshare_u64(pg_party *p, pg_ctx *ctx, const uint64_t *c, size_t n, uint64_t *const out[2]);
int pg_party_rss_matmul_u64(pg_party *p, pg_ctx *ctx, const uint64_t *const a[2], const uint64_t *const b[2],
                            uint64_t *const c[2], int M, int N, int K, int tA, int tB, int tC, int trunc);

#ifdef __cplusplus
}
#endif
#endif /* PIRANHA_GB300_H */
