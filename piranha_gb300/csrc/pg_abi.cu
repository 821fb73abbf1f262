// pg_abi.cu — the extern "C" surface declared in include/piranha_gb300.h:
// context lifetime, status/error reporting, communication counters, and thin
// wrappers that forward to the templated kernels of the other translation
// units.
#include <cstdlib>
#include <cstring>
#include <random>

#include "pg_common.cuh"

namespace pg {

int set_error(Ctx *c, int code, const char *fmt, ...) {
    if (!c) return code;
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
    return code;
}

int launch_status(Ctx *c, const char *what) {
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, PG_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    }
    return PG_OK;
}

int *device_error_word(Ctx *c) { return c->dev_err; }

// A grow-only device buffer of the context (grows with cudaMalloc, which a
// stream capture does not allow: capture after an eager run has sized it).
// An outgrown buffer is retired, not freed: graphs captured earlier may still
// read and write it.
static void *grow(Ctx *c, void *&buf, size_t &have, size_t bytes, const char *what) {
    if (bytes <= have) return buf;
    size_t want = bytes + (bytes >> 3);
    if (buf) {
        if (want < 2 * have) want = 2 * have;  // geometric: the retired buffers sum to less than the live one
        c->retired.push_back(buf);
        buf = nullptr;
        have = 0;
    }
    if (cudaMalloc(&buf, want) != cudaSuccess) {
        cudaGetLastError();
        buf = nullptr;
        set_error(c, PG_ERR_NO_MEMORY, "%s allocation of %zu bytes failed", what, want);
        return nullptr;
    }
    have = want;
    return buf;
}

void *scratch(Ctx *c, size_t bytes) { return grow(c, c->scratch, c->scratch_bytes, bytes, "scratch"); }
void *gemm_partial(Ctx *c, size_t bytes) { return grow(c, c->partial, c->partial_bytes, bytes, "split-K buffer"); }

// kernels in other translation units
int prg_fill_u64(Ctx *, const uint8_t *, uint64_t, uint64_t *, size_t);
int prg_set_keys(Ctx *, const uint8_t *, uint64_t);
int rss_local_u64(Ctx *, int, uint64_t *const *, size_t, int, uint64_t, const uint64_t *, const uint64_t *const *);
int local_u64(Ctx *, int, int, uint64_t *const *, size_t, int, uint64_t, const uint64_t *, const uint64_t *const *);
int device_op_u64(Ctx *, int, uint64_t *, size_t, int, uint64_t, const uint64_t *);
template <typename T>
int rss_matmul(Ctx *, const T *const *, const T *const *, T *const *, const T *const *, int, int, int, int, int, int,
               int);
template <typename T>
int rss_conv(Ctx *, const T *const *, const T *const *, T *const *, int, int, int, int, int, int, int, int, int, int);
template <typename T> int plain_gemm(Ctx *, int, int, int, const T *, int, const T *, int, T *, int);
int plain_conv_u64(Ctx *, int, int, int, int, int, int, int, int, int, int, const uint64_t *, const uint64_t *,
                   uint64_t *);
template <typename T, typename U> int rss_drelu(Ctx *, const T *const *, size_t, U *const *);
template <typename T, typename U> int rss_relu(Ctx *, const T *const *, size_t, T *const *, U *const *);
template <typename T, typename U>
int rss_select(Ctx *, const T *const *, const T *const *, const U *const *, T *const *, size_t);
template <typename T, typename U> int rss_maxpool(Ctx *, const T *const *, size_t, int, T *const *, U *const *);
template <typename T, typename U>
int rss_maxpool_layer(Ctx *, const T *const *, T *const *, U *const *, int, int, int, int, int, int, int);
template <typename T>
int rss_avgpool_layer(Ctx *, const T *const *, T *const *, int, int, int, int, int, int);
template <typename T>
int rss_avgpool_backward(Ctx *, const T *const *, T *const *, int, int, int, int, int, int);
template <typename T> int rss_reconstruct(Ctx *, const T *const *, size_t, T *const *);
template <typename T> int rss_reshare(Ctx *, const T *const *, size_t, T *const *);
template <typename T, bool AND> int rss_mul(Ctx *, T *const *, const T *const *, size_t);
template <typename T> int rss_divide_public(Ctx *, T *const *, size_t, T, const T *);
int element_vector_add_u64(Ctx *, uint64_t *, const uint64_t *, int, int, int);
int reduce_sum_u64(Ctx *, const uint64_t *, uint64_t *, int, int, int);
int truncate_cols_u8(Ctx *, const uint8_t *, uint8_t *, size_t, int, int);
int bitexpand_u64(Ctx *, const uint64_t *, size_t, uint64_t *);
int expand_compare_u8(Ctx *, const uint8_t *, const uint8_t *, size_t, uint8_t *, size_t);
int maxpool_im2row_u64(Ctx *, const uint64_t *, uint64_t *, int, int, int, int, int, int, int, uint64_t);
int limb3_rss_matmul_u64(Ctx *, const uint64_t *const *, const uint64_t *const *, uint64_t *const *,
                        const uint64_t *const *, int, int, int, int, int, int, int);
int limb3_rss_conv_u64(Ctx *, const uint64_t *const *, const uint64_t *const *, uint64_t *const *, int, int, int, int,
                      int, int, int, int, int, int);
int limb_selftest(Ctx *, const uint16_t *, const uint16_t *, float *);

}  // namespace pg

using namespace pg;

#define CTX_OR_FAIL(c) \
    if (!(c)) return PG_ERR_INVALID_ARG

extern "C" {

}  // extern "C"

// Tuning cache file: a header line "pg-tune <SM count>", then one
// "<shape key> <split> <chunks per split>" per line. A file written on a GPU
// with another SM count is ignored.
static int tune_load(pg::Ctx *c, const char *path, bool keep_own = false) {
    FILE *f = fopen(path, "r");
    if (!f) return PG_ERR_INVALID_ARG;
    int sms = -1;
    if (fscanf(f, "pg-tune %d", &sms) != 1 || sms != c->sm_count) {
        fclose(f);
        return PG_ERR_UNSUPPORTED;
    }
    char key[256];
    int sp, cp;
    while (fscanf(f, "%255s %d %d", key, &sp, &cp) == 3)
        if (sp >= 1 && cp >= 1 && !(keep_own && c->split_cache.count(key))) c->split_cache[key] = {sp, cp};
    fclose(f);
    return PG_OK;
}

static int tune_save(pg::Ctx *c, const char *path) {
    // merge with what the file already holds (another context may have written it)
    tune_load(c, path, true);
    FILE *f = fopen(path, "w");
    if (!f) return PG_ERR_INVALID_ARG;
    fprintf(f, "pg-tune %d\n", c->sm_count);
    for (const auto &e : c->split_cache) fprintf(f, "%s %d %d\n", e.first.c_str(), e.second.first, e.second.second);
    fclose(f);
    return PG_OK;
}

extern "C" {

int pg_tune_load(pg_ctx *c, const char *path) {
    CTX_OR_FAIL(c);
    if (!path) return set_error(c, PG_ERR_INVALID_ARG, "null path");
    const int st = tune_load(c, path);
    return st ? set_error(c, st, "cannot read a tuning cache for %d SMs from %s", c->sm_count, path) : PG_OK;
}

int pg_tune_save(pg_ctx *c, const char *path) {
    CTX_OR_FAIL(c);
    if (!path) return set_error(c, PG_ERR_INVALID_ARG, "null path");
    const int st = tune_save(c, path);
    return st ? set_error(c, st, "cannot write the tuning cache %s", path) : PG_OK;
}

int pg_ctx_create(pg_ctx **out, int device) {
    if (!out) return PG_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return PG_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return PG_ERR_CUDA;
    pg_ctx *c = new pg_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaMalloc(&c->dev_err, 256) != cudaSuccess || cudaMemset(c->dev_err, 0, 256) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return PG_ERR_CUDA;
    }
    if (const char *tc = getenv("PG_TUNE_CACHE")) tune_load(c, tc);
    *out = c;
    return PG_OK;
}

int pg_ctx_destroy(pg_ctx *c) {
    CTX_OR_FAIL(c);
    cudaStreamSynchronize(c->stream);
    if (const char *tc = getenv("PG_TUNE_CACHE"))
        if (!c->split_cache.empty()) tune_save(c, tc);
    if (c->scratch) cudaFree(c->scratch);
    if (c->partial) cudaFree(c->partial);
    for (void *p : c->retired) cudaFree(p);
    if (c->dev_err) cudaFree(c->dev_err);
    delete c;
    return PG_OK;
}

int pg_ctx_set_stream(pg_ctx *c, void *s) {
    CTX_OR_FAIL(c);
    c->stream = (cudaStream_t)s;
    return PG_OK;
}
void *pg_ctx_get_stream(pg_ctx *c) { return c ? (void *)c->stream : nullptr; }
int pg_ctx_set_form(pg_ctx *c, int form) {
    CTX_OR_FAIL(c);
    if (form != PG_FORM_U64 && form != PG_FORM_LIMB_TC) return set_error(c, PG_ERR_INVALID_ARG, "bad form %d", form);
    c->form = form;
    return PG_OK;
}
int pg_ctx_get_form(pg_ctx *c) { return c ? c->form : -1; }
int pg_ctx_set_wait_limit(pg_ctx *c, uint64_t wait_ns, int withhold_stage) {
    CTX_OR_FAIL(c);
    if (withhold_stage < -1) return set_error(c, PG_ERR_INVALID_ARG, "withhold stage %d", withhold_stage);
    c->wait_ns = wait_ns ? wait_ns : 2000000000ull;
    c->withhold_stage = withhold_stage;
    return PG_OK;
}
int pg_ctx_set_autotune(pg_ctx *c, int on) {
    CTX_OR_FAIL(c);
    c->autotune = on ? 1 : 0;
    if (!on) c->split_cache.clear();
    return PG_OK;
}

int pg_alloc_shares(pg_ctx *c, int nbuf, size_t n, int elem_bytes, void **out) {
    CTX_OR_FAIL(c);
    if (!out || nbuf <= 0 || nbuf > 64 || (elem_bytes != 1 && elem_bytes != 4 && elem_bytes != 8))
        return set_error(c, PG_ERR_INVALID_ARG, "alloc_shares: %d buffers of %d-byte elements", nbuf, elem_bytes);
    for (int i = 0; i < nbuf; i++) out[i] = nullptr;
    const size_t one = (n * (size_t)elem_bytes + 255) & ~(size_t)255;
    void *base = nullptr;
    if (cudaMalloc(&base, one * nbuf + (one == 0 ? 256 : 0)) != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, PG_ERR_NO_MEMORY, "alloc_shares of %zu bytes", one * nbuf);
    }
    PG_CHECK_CUDA(c, cudaMemsetAsync(base, 0, one * nbuf, c->stream));
    for (int i = 0; i < nbuf; i++) out[i] = (char *)base + one * i;
    return PG_OK;
}

int pg_free_shares(pg_ctx *c, void *first) {
    CTX_OR_FAIL(c);
    if (!first) return PG_OK;
    PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    PG_CHECK_CUDA(c, cudaFree(first));
    return PG_OK;
}
const char *pg_last_error(pg_ctx *c) { return c ? c->err.c_str() : "null context"; }
int pg_sync(pg_ctx *c) {
    CTX_OR_FAIL(c);
    PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}
int pg_comm_get(pg_ctx *c, uint64_t out[9]) {
    CTX_OR_FAIL(c);
    if (!out) return PG_ERR_INVALID_ARG;
    memcpy(out, c->comm, sizeof(c->comm));
    return PG_OK;
}
int pg_comm_reset(pg_ctx *c) {
    CTX_OR_FAIL(c);
    memset(c->comm, 0, sizeof(c->comm));
    return PG_OK;
}
uint64_t pg_kernel_launches(pg_ctx *c) { return c ? c->launches.load() : 0; }

}  // extern "C"

struct pg_graph {
    pg_ctx *owner = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t comm[9] = {0};  // counters added by one launch
    uint64_t launches = 0;
};

extern "C" {

int pg_graph_begin(pg_ctx *c) {
    CTX_OR_FAIL(c);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CHECK_CUDA(c, cudaStreamIsCapturing(c->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone || c->capturing)
        return set_error(c, PG_ERR_INVALID_ARG, "the context's stream is already capturing");
    if (c->stream == nullptr)
        return set_error(c, PG_ERR_INVALID_ARG, "capture needs a non-default stream (pg_ctx_set_stream)");
    memcpy(c->capture_comm, c->comm, sizeof(c->comm));
    c->capture_launches = c->launches.load();
    PG_CHECK_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    return PG_OK;
}

int pg_graph_end(pg_ctx *c, pg_graph **out) {
    CTX_OR_FAIL(c);
    if (!out) return set_error(c, PG_ERR_INVALID_ARG, "null graph pointer");
    *out = nullptr;
    if (!c->capturing) return set_error(c, PG_ERR_INVALID_ARG, "no capture in progress");
    c->capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    pg_graph *g = new pg_graph;
    g->owner = c;
    for (int i = 0; i < 9; i++) g->comm[i] = c->comm[i] - c->capture_comm[i];
    g->launches = c->launches.load() - c->capture_launches;
    memcpy(c->comm, c->capture_comm, sizeof(c->comm));
    c->launches.store(c->capture_launches);
    if (e != cudaSuccess || !graph) {
        cudaGetLastError();
        if (graph) cudaGraphDestroy(graph);
        delete g;
        return set_error(c, PG_ERR_CUDA, "stream capture failed: %s (a call inside it allocated, synchronized or "
                                         "failed; run the sequence eagerly once first)",
                         cudaGetErrorString(e));
    }
    const cudaError_t ei = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        cudaGetLastError();
        delete g;
        return set_error(c, PG_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ei));
    }
    *out = g;
    return PG_OK;
}

int pg_graph_launch(pg_ctx *c, pg_graph *g) {
    CTX_OR_FAIL(c);
    if (!g || g->owner != c) return set_error(c, PG_ERR_INVALID_ARG, "graph of another context");
    PG_CHECK_CUDA(c, cudaGraphLaunch(g->exec, c->stream));
    for (int i = 0; i < 9; i++) c->comm[i] += g->comm[i];
    c->launches += g->launches;
    return PG_OK;
}

int pg_graph_destroy(pg_graph *g) {
    if (!g) return PG_ERR_INVALID_ARG;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    delete g;
    return PG_OK;
}

int pg_device_errors(pg_ctx *c, int *out) {
    CTX_OR_FAIL(c);
    if (!out) return PG_ERR_INVALID_ARG;
    PG_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    PG_CHECK_CUDA(c, cudaMemcpy(out, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
    PG_CHECK_CUDA(c, cudaMemset(c->dev_err, 0, sizeof(int)));
    return *out ? set_error(c, PG_ERR_TIMEOUT, "device wait timed out (code 0x%x)", *out) : PG_OK;
}

int pg_reference_init_normal(double *out, size_t n, int seed, double std_dev) {
    if (!out && n) return PG_ERR_INVALID_ARG;
    if (!(std_dev >= 0.0)) return PG_ERR_INVALID_ARG;
    std::default_random_engine generator(seed);
    std::normal_distribution<double> distribution(0.0, std_dev);
    for (size_t i = 0; i < n; i++) out[i] = distribution(generator);
    return PG_OK;
}

int pg_tc_selftest(pg_ctx *c, const uint16_t *A, const uint16_t *B, float *D) {
    CTX_OR_FAIL(c);
    return limb_selftest(c, A, B, D);
}

int pg_gemm_u64(pg_ctx *c, int M, int N, int K, const uint64_t *A, int tA, const uint64_t *B, int tB, uint64_t *C,
                int tC) {
    CTX_OR_FAIL(c);
    return plain_gemm<uint64_t>(c, M, N, K, A, tA, B, tB, C, tC);
}
int pg_gemm_u32(pg_ctx *c, int M, int N, int K, const uint32_t *A, int tA, const uint32_t *B, int tB, uint32_t *C,
                int tC) {
    CTX_OR_FAIL(c);
    return plain_gemm<uint32_t>(c, M, N, K, A, tA, B, tB, C, tC);
}
int pg_conv_u64(pg_ctx *c, int op, int N, int H, int W, int C, int K, int R, int S, int pad, int stride,
                const uint64_t *a, const uint64_t *b, uint64_t *out) {
    CTX_OR_FAIL(c);
    return plain_conv_u64(c, op, N, H, W, C, K, R, S, pad, stride, a, b, out);
}

int pg_rss_matmul_u64(pg_ctx *c, const uint64_t *const a[6], const uint64_t *const b[6], uint64_t *const out[6],
                      int M, int N, int K, int tA, int tB, int tC, int trunc) {
    CTX_OR_FAIL(c);
    if (c->form == PG_FORM_LIMB_TC) return limb3_rss_matmul_u64(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
    return rss_matmul<uint64_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}
int pg_rss_matmul_u32(pg_ctx *c, const uint32_t *const a[6], const uint32_t *const b[6], uint32_t *const out[6],
                      int M, int N, int K, int tA, int tB, int tC, int trunc) {
    CTX_OR_FAIL(c);
    return rss_matmul<uint32_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}
int pg_rss_fc_forward_u64(pg_ctx *c, const uint64_t *const x[6], const uint64_t *const w[6],
                          const uint64_t *const bias[6], uint64_t *const out[6], int batch, int din, int dout, int fp) {
    CTX_OR_FAIL(c);
    if (bias)
        for (int i = 0; i < 6; i++)
            if (!bias[i]) return set_error(c, PG_ERR_INVALID_ARG, "null bias share");
    if (c->form == PG_FORM_LIMB_TC) return limb3_rss_matmul_u64(c, x, w, out, bias, batch, dout, din, 1, 1, 1, fp);
    return rss_matmul<uint64_t>(c, x, w, out, bias, batch, dout, din, 1, 1, 1, fp);
}
int pg_rss_conv_u64(pg_ctx *c, const uint64_t *const A[6], const uint64_t *const B[6], uint64_t *const C[6], int op,
                    int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    CTX_OR_FAIL(c);
    if (c->form == PG_FORM_LIMB_TC)
        return limb3_rss_conv_u64(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc);
    return rss_conv<uint64_t>(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc);
}
int pg_rss_divide_public_u64(pg_ctx *c, uint64_t *const a[6], size_t n, uint64_t d) {
    CTX_OR_FAIL(c);
    return rss_divide_public<uint64_t>(c, a, n, d, nullptr);
}
int pg_rss_divide_public_vec_u64(pg_ctx *c, uint64_t *const a[6], size_t n, const uint64_t *d) {
    CTX_OR_FAIL(c);
    if (!d && n) return set_error(c, PG_ERR_INVALID_ARG, "null denominators");
    return rss_divide_public<uint64_t>(c, a, n, 0, d);
}
int pg_rss_divide_public_u32(pg_ctx *c, uint32_t *const a[6], size_t n, uint32_t d) {
    CTX_OR_FAIL(c);
    return rss_divide_public<uint32_t>(c, a, n, d, nullptr);
}
int pg_rss_reconstruct_u64(pg_ctx *c, const uint64_t *const a[6], size_t n, uint64_t *const out[3]) {
    CTX_OR_FAIL(c);
    return rss_reconstruct<uint64_t>(c, a, n, out);
}
int pg_rss_reconstruct_u8(pg_ctx *c, const uint8_t *const a[6], size_t n, uint8_t *const out[3]) {
    CTX_OR_FAIL(c);
    return rss_reconstruct<uint8_t>(c, a, n, out);
}
int pg_prg_fill_u64(pg_ctx *c, const uint8_t key[32], uint64_t counter, uint64_t *out, size_t n) {
    CTX_OR_FAIL(c);
    return prg_fill_u64(c, key, counter, out, n);
}
int pg_prg_set_keys(pg_ctx *c, const uint8_t *keys, uint64_t counter) {
    CTX_OR_FAIL(c);
    return prg_set_keys(c, keys, counter);
}
int pg_prg_counter(pg_ctx *c, uint64_t *out) {
    CTX_OR_FAIL(c);
    if (!out) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    *out = c->prg_ctr;
    return PG_OK;
}
int pg_rss_local_u64(pg_ctx *c, int op, uint64_t *const a[6], size_t n, int kind, uint64_t scalar,
                     const uint64_t *pub, const uint64_t *const shares[6]) {
    CTX_OR_FAIL(c);
    return rss_local_u64(c, op, a, n, kind, scalar, pub, shares);
}
int pg_device_op_u64(pg_ctx *c, int op, uint64_t *a, size_t n, int kind, uint64_t scalar, const uint64_t *rhs) {
    CTX_OR_FAIL(c);
    return device_op_u64(c, op, a, n, kind, scalar, rhs);
}
int pg_tpc_local_u64(pg_ctx *c, int op, uint64_t *const a[2], size_t n, int kind, uint64_t scalar,
                     const uint64_t *pub, const uint64_t *const shares[2]) {
    CTX_OR_FAIL(c);
    return local_u64(c, 2, op, a, n, kind, scalar, pub, shares);
}
int pg_fpc_local_u64(pg_ctx *c, int op, uint64_t *const a[12], size_t n, int kind, uint64_t scalar,
                     const uint64_t *pub, const uint64_t *const shares[12]) {
    CTX_OR_FAIL(c);
    return local_u64(c, 12, op, a, n, kind, scalar, pub, shares);
}
int pg_rss_reshare_u64(pg_ctx *c, const uint64_t *const cin[3], size_t n, uint64_t *const out[6]) {
    CTX_OR_FAIL(c);
    return rss_reshare<uint64_t>(c, cin, n, out);
}
int pg_rss_mul_u64(pg_ctx *c, uint64_t *const a[6], const uint64_t *const b[6], size_t n) {
    CTX_OR_FAIL(c);
    return rss_mul<uint64_t, false>(c, a, b, n);
}
int pg_rss_and_u64(pg_ctx *c, uint64_t *const a[6], const uint64_t *const b[6], size_t n) {
    CTX_OR_FAIL(c);
    return rss_mul<uint64_t, true>(c, a, b, n);
}
int pg_rss_and_u8(pg_ctx *c, uint8_t *const a[6], const uint8_t *const b[6], size_t n) {
    CTX_OR_FAIL(c);
    return rss_mul<uint8_t, true>(c, a, b, n);
}
int pg_rss_drelu_u64_u8(pg_ctx *c, const uint64_t *const in[6], size_t n, uint8_t *const out[6]) {
    CTX_OR_FAIL(c);
    return rss_drelu<uint64_t, uint8_t>(c, in, n, out);
}
int pg_rss_drelu_u64_u64(pg_ctx *c, const uint64_t *const in[6], size_t n, uint64_t *const out[6]) {
    CTX_OR_FAIL(c);
    return rss_drelu<uint64_t, uint64_t>(c, in, n, out);
}
int pg_rss_relu_u64_u8(pg_ctx *c, const uint64_t *const in[6], size_t n, uint64_t *const out[6],
                       uint8_t *const dout[6]) {
    CTX_OR_FAIL(c);
    return rss_relu<uint64_t, uint8_t>(c, in, n, out, dout);
}
int pg_rss_relu_u64_u64(pg_ctx *c, const uint64_t *const in[6], size_t n, uint64_t *const out[6],
                        uint64_t *const dout[6]) {
    CTX_OR_FAIL(c);
    return rss_relu<uint64_t, uint64_t>(c, in, n, out, dout);
}
int pg_rss_relu_u32_u8(pg_ctx *c, const uint32_t *const in[6], size_t n, uint32_t *const out[6],
                       uint8_t *const dout[6]) {
    CTX_OR_FAIL(c);
    return rss_relu<uint32_t, uint8_t>(c, in, n, out, dout);
}
int pg_rss_select_share_u64_u8(pg_ctx *c, const uint64_t *const x[6], const uint64_t *const y[6],
                               const uint8_t *const b[6], uint64_t *const z[6], size_t n) {
    CTX_OR_FAIL(c);
    return rss_select<uint64_t, uint8_t>(c, x, y, b, z, n);
}
int pg_rss_select_share_u64_u64(pg_ctx *c, const uint64_t *const x[6], const uint64_t *const y[6],
                                const uint64_t *const b[6], uint64_t *const z[6], size_t n) {
    CTX_OR_FAIL(c);
    return rss_select<uint64_t, uint64_t>(c, x, y, b, z, n);
}
int pg_rss_maxpool_u64_u8(pg_ctx *c, const uint64_t *const in[6], size_t n, int k, uint64_t *const out[6],
                          uint8_t *const dout[6]) {
    CTX_OR_FAIL(c);
    return rss_maxpool<uint64_t, uint8_t>(c, in, n, k, out, dout);
}
int pg_rss_maxpool_u64_u64(pg_ctx *c, const uint64_t *const in[6], size_t n, int k, uint64_t *const out[6],
                           uint64_t *const dout[6]) {
    CTX_OR_FAIL(c);
    return rss_maxpool<uint64_t, uint64_t>(c, in, n, k, out, dout);
}
int pg_rss_maxpool_layer_u64_u8(pg_ctx *c, const uint64_t *const in[6], uint64_t *const out[6],
                                uint8_t *const maxprime[6], int H, int W, int C, int pool, int stride, int batch,
                                int fp) {
    CTX_OR_FAIL(c);
    return rss_maxpool_layer<uint64_t, uint8_t>(c, in, out, maxprime, H, W, C, pool, stride, batch, fp);
}
int pg_rss_avgpool_layer_u64(pg_ctx *c, const uint64_t *const in[6], uint64_t *const out[6], int H, int W, int C,
                             int pool, int stride, int batch) {
    CTX_OR_FAIL(c);
    return rss_avgpool_layer<uint64_t>(c, in, out, H, W, C, pool, stride, batch);
}
int pg_rss_avgpool_backward_u64(pg_ctx *c, const uint64_t *const delta[6], uint64_t *const deltas[6], int H, int W,
                                int C, int pool, int stride, int batch) {
    CTX_OR_FAIL(c);
    return rss_avgpool_backward<uint64_t>(c, delta, deltas, H, W, C, pool, stride, batch);
}
int pg_element_vector_add_u64(pg_ctx *c, uint64_t *a, const uint64_t *b, int rowwise, int rows, int cols) {
    CTX_OR_FAIL(c);
    return element_vector_add_u64(c, a, b, rowwise, rows, cols);
}
int pg_reduce_sum_u64(pg_ctx *c, const uint64_t *a, uint64_t *b, int reduce_rows, int rows, int cols) {
    CTX_OR_FAIL(c);
    return reduce_sum_u64(c, a, b, reduce_rows, rows, cols);
}
int pg_truncate_cols_u8(pg_ctx *c, const uint8_t *a, uint8_t *b, size_t rows, int start_cols, int end_cols) {
    CTX_OR_FAIL(c);
    return truncate_cols_u8(c, a, b, rows, start_cols, end_cols);
}
int pg_bitexpand_u64(pg_ctx *c, const uint64_t *a, size_t n, uint64_t *bits) {
    CTX_OR_FAIL(c);
    return bitexpand_u64(c, a, n, bits);
}
int pg_expand_compare_u8(pg_ctx *c, const uint8_t *b, const uint8_t *nb, size_t n, uint8_t *out, size_t out_n) {
    CTX_OR_FAIL(c);
    return expand_compare_u8(c, b, nb, n, out, out_n);
}
int pg_maxpool_im2row_u64(pg_ctx *c, const uint64_t *im, uint64_t *out, int H, int W, int f, int Din, int batch,
                          int stride, int pad, uint64_t pad_val) {
    CTX_OR_FAIL(c);
    return maxpool_im2row_u64(c, im, out, H, W, f, Din, batch, stride, pad, pad_val);
}

}  // extern "C"
