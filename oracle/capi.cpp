// capi.cpp — C entry points of the CPU oracle (test infrastructure only).
//
// Every RSS tensor crosses this boundary as one flat array laid out
// [party(3)][share(2)][n]; per-party public data as [party(3)][n]. The comm
// argument points at 9 uint64 counters {tx[4], rx[4], rounds} that each call
// adds to (DeviceData.h:87-118 byte accounting, one round per protocol step).
#include "aes.hpp"
#include "oracle.hpp"

using namespace oracle;

namespace {

template <typename T> void load(RSSV<T>& r, const T* flat, size_t n) {
    r.resize(n);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++) std::memcpy(r.v[p][s].data(), flat + ((size_t)p * 2 + s) * n, n * sizeof(T));
}
template <typename T> void store(const RSSV<T>& r, T* flat) {
    size_t n = r.n;
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++) std::memcpy(flat + ((size_t)p * 2 + s) * n, r.v[p][s].data(), n * sizeof(T));
}
struct CommIO {
    uint64_t* out;
    Comm c;
    explicit CommIO(uint64_t* o) : out(o) {}
    ~CommIO() {
        if (!out) return;
        for (int p = 0; p < 4; p++) { out[p] += c.tx[p]; out[4 + p] += c.rx[p]; }
        out[8] += c.rounds;
    }
};

}  // namespace

#define OR_RING(T, SUF)                                                                                      \
    extern "C" int or_rss_matmul_##SUF(const T* a, const T* b, T* c, int M, int N, int K, int tA, int tB,     \
                                       int tC, int trunc, uint64_t* comm) {                                  \
        RSSV<T> A, B, C;                                                                                     \
        load(A, a, (size_t)M * K);                                                                           \
        load(B, b, (size_t)K * N);                                                                           \
        CommIO io(comm);                                                                                     \
        rss_matmul<T>(A, B, C, M, N, K, tA, tB, tC, trunc, io.c);                                            \
        store(C, c);                                                                                         \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_conv_##SUF(const T* a, size_t na, const T* b, size_t nb, T* c, int op, int batch,   \
                                     int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc,  \
                                     uint64_t* comm) {                                                       \
        RSSV<T> A, B, C;                                                                                     \
        load(A, a, na);                                                                                      \
        load(B, b, nb);                                                                                      \
        CommIO io(comm);                                                                                     \
        rss_convolution<T>(A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc, io.c);                \
        store(C, c);                                                                                         \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_divide_public_##SUF(T* a, size_t n, const T* d, int vector_d, uint64_t* comm) {     \
        RSSV<T> A;                                                                                           \
        load(A, a, n);                                                                                       \
        CommIO io(comm);                                                                                     \
        rss_divide_public<T>(A, d, vector_d != 0, io.c);                                                     \
        store(A, a);                                                                                         \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_divide_3of3_##SUF(const T* z, size_t n, T d, T* out, uint64_t* comm) {             \
        std::vector<T> zz[3];                                                                                \
        for (int p = 0; p < 3; p++) zz[p].assign(z + (size_t)p * n, z + (size_t)(p + 1) * n);                \
        RSSV<T> O;                                                                                           \
        CommIO io(comm);                                                                                     \
        rss_divide_public_3of3<T>(zz, d, O, io.c);                                                           \
        store(O, out);                                                                                       \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_reconstruct_##SUF(const T* a, size_t n, T* out, uint64_t* comm) {                  \
        RSSV<T> A;                                                                                           \
        load(A, a, n);                                                                                       \
        std::vector<T> o[3];                                                                                 \
        CommIO io(comm);                                                                                     \
        rss_reconstruct<T>(A, whole(n), o, io.c);                                                            \
        for (int p = 0; p < 3; p++) std::memcpy(out + (size_t)p * n, o[p].data(), n * sizeof(T));            \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_reshare_##SUF(const T* c, size_t n, T* out, uint64_t* comm) {                      \
        std::vector<T> cc[3];                                                                                \
        for (int p = 0; p < 3; p++) cc[p].assign(c + (size_t)p * n, c + (size_t)(p + 1) * n);               \
        RSSV<T> O(n);                                                                                        \
        CommIO io(comm);                                                                                     \
        reshare_into<T>(cc, O, whole(n), io.c);                                                              \
        store(O, out);                                                                                       \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_mul_##SUF(T* a, const T* b, size_t n, uint64_t* comm) {                            \
        RSSV<T> A, B;                                                                                        \
        load(A, a, n);                                                                                       \
        load(B, b, n);                                                                                       \
        CommIO io(comm);                                                                                     \
        rss_mul_assign<T>(A, B, io.c);                                                                       \
        store(A, a);                                                                                         \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_and_##SUF(T* a, const T* b, size_t n, uint64_t* comm) {                            \
        RSSV<T> A, B;                                                                                        \
        load(A, a, n);                                                                                       \
        load(B, b, n);                                                                                       \
        CommIO io(comm);                                                                                     \
        rss_and_assign<T>(A, whole(n), B, whole(n), io.c);                                                   \
        store(A, a);                                                                                         \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_set_public_##SUF(const double* vals, size_t n, T* out, int fp, int ref_compat) {   \
        RSSV<T> A(n);                                                                                        \
        rss_set_public<T>(A, vals, fp, ref_compat != 0);                                                     \
        store(A, out);                                                                                       \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_from_list_##SUF(const double* vals, size_t n, T* out, int fp, int to_fixed) {      \
        RSSV<T> A(n);                                                                                        \
        rss_from_list<T>(A, vals, fp, to_fixed != 0);                                                        \
        store(A, out);                                                                                       \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" void or_encode_##SUF(const double* vals, size_t n, T* out, int fp) {                          \
        for (size_t i = 0; i < n; i++) out[i] = encode_fixed<T>(vals[i], fp);                                \
    }                                                                                                        \
    extern "C" void or_div_public_scalar_##SUF(const T* x, size_t n, const T* d, int vector_d, T* out) {     \
        for (size_t i = 0; i < n; i++) out[i] = div_public<T>(x[i], vector_d ? d[i] : d[0]);                 \
    }                                                                                                        \
    extern "C" int or_gemm_##SUF(int M, int N, int K, const T* A, int tA, const T* B, int tB, T* C, int tC) { \
        gemm<T>(M, N, K, A, tA, B, tB, C, tC);                                                               \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_conv_##SUF(int op, int N, int H, int W, int C, int K, int R, int S, int pad,           \
                                 int stride, const T* a, const T* b, T* out) {                               \
        ConvShape sh{N, H, W, C, K, R, S, pad, stride};                                                      \
        conv_any<T>(op, sh, a, b, out);                                                                      \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" size_t or_maxpool_im2row_##SUF(const T* im, T* out, size_t cap, int H, int W, int f, int Din, \
                                              int batch, int stride, int pad, T pad_val) {                   \
        std::vector<T> o;                                                                                    \
        maxpool_im2row<T>(im, o, H, W, f, Din, batch, stride, pad, pad_val);                                 \
        if (out && cap >= o.size()) std::memcpy(out, o.data(), o.size() * sizeof(T));                        \
        return o.size();                                                                                     \
    }                                                                                                        \
    extern "C" void or_element_vector_add_##SUF(T* a, const T* b, int rowwise, int rows, int cols) {         \
        element_vector_add<T>(a, b, rowwise != 0, rows, cols);                                               \
    }                                                                                                        \
    extern "C" void or_reduce_sum_##SUF(const T* a, T* b, int reduceRows, int rows, int cols) {              \
        reduce_sum<T>(a, b, reduceRows != 0, rows, cols);                                                    \
    }                                                                                                        \
    extern "C" void or_bitexpand_##SUF(const T* a, size_t n, T* bits) {                                      \
        std::vector<T> av(a, a + n), b;                                                                      \
        bitexpand<T, T>(av, b);                                                                              \
        std::memcpy(bits, b.data(), b.size() * sizeof(T));                                                   \
    }

OR_RING(uint64_t, u64)
OR_RING(uint32_t, u32)

#define OR_BITS(T, TS, U, US)                                                                                \
    extern "C" int or_rss_drelu_##TS##_##US(const T* in, size_t n, U* out, uint64_t* comm) {                 \
        RSSV<T> A;                                                                                           \
        load(A, in, n);                                                                                      \
        RSSV<U> R(n);                                                                                        \
        CommIO io(comm);                                                                                     \
        rss_drelu<T, U>(A, whole(n), R, io.c);                                                               \
        store(R, out);                                                                                       \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_relu_##TS##_##US(const T* in, size_t n, T* out, U* dout, uint64_t* comm) {         \
        RSSV<T> A, O;                                                                                        \
        load(A, in, n);                                                                                      \
        RSSV<U> D(n);                                                                                        \
        CommIO io(comm);                                                                                     \
        rss_relu<T, U>(A, O, D, io.c);                                                                       \
        store(O, out);                                                                                       \
        store(D, dout);                                                                                      \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_select_share_##TS##_##US(const T* x, const T* y, const U* b, T* z, size_t n,       \
                                                   uint64_t* comm) {                                         \
        RSSV<T> X, Y, Z(n);                                                                                  \
        RSSV<U> B;                                                                                           \
        load(X, x, n);                                                                                       \
        load(Y, y, n);                                                                                       \
        load(B, b, n);                                                                                       \
        CommIO io(comm);                                                                                     \
        rss_select_share<T, U>(X, whole(n), Y, whole(n), B, Z, whole(n), io.c);                              \
        store(Z, z);                                                                                         \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_rss_maxpool_##TS##_##US(const T* in, size_t n, T* out, U* dout, int k,                 \
                                              uint64_t* comm) {                                              \
        RSSV<T> A, O;                                                                                        \
        load(A, in, n);                                                                                      \
        RSSV<U> D(n);                                                                                        \
        CommIO io(comm);                                                                                     \
        rss_maxpool<T, U>(A, O, D, k, io.c);                                                                 \
        store(O, out);                                                                                       \
        store(D, dout);                                                                                      \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_maxpool_layer_##TS##_##US(const T* in, T* out, U* maxprime, int H, int W, int C,       \
                                                int pool, int stride, int batch, int fp, uint64_t* comm) {   \
        RSSV<T> A, O;                                                                                        \
        load(A, in, (size_t)batch * H * W * C);                                                              \
        RSSV<U> D;                                                                                           \
        CommIO io(comm);                                                                                     \
        maxpool_layer_forward<T, U>(A, O, D, H, W, C, pool, stride, batch, fp, io.c);                        \
        store(O, out);                                                                                       \
        store(D, maxprime);                                                                                  \
        return 0;                                                                                            \
    }

OR_BITS(uint64_t, u64, uint8_t, u8)
OR_BITS(uint64_t, u64, uint64_t, u64)
OR_BITS(uint32_t, u32, uint8_t, u8)
OR_BITS(uint32_t, u32, uint32_t, u32)

extern "C" void or_expand_compare_u8(const uint8_t* b, const uint8_t* nb, size_t n, uint8_t* out, size_t out_n) {
    std::vector<uint8_t> bv(b, b + n), nv(nb, nb + n), o(out_n);
    expand_compare<uint8_t>(bv, nv, o);
    std::memcpy(out, o.data(), out_n);
}

extern "C" void or_truncate_cols_u8(const uint8_t* a, uint8_t* b, size_t rows, int start_cols, int end_cols) {
    truncate_cols<uint8_t>(a, b, rows, start_cols, end_cols);
}

// ------------------------------------------------------- training step (RSS)

extern "C" void or_vector_expand_u64(const uint64_t* a, size_t n, uint64_t* b, size_t f) {
    vector_expand<uint64_t>(a, n, b, f);
}
extern "C" void or_maxpool_row2im_u64(const uint64_t* rows, uint64_t* out, int imageHeight, int imageWidth, int f,
                                      int Din, int batch, int stride) {
    maxpool_row2im<uint64_t>(rows, out, imageHeight, imageWidth, f, Din, batch, stride);
}
extern "C" int or_relu_layer_backward_u64_u8(const uint64_t* delta, size_t n, const uint8_t* relu_prime,
                                             uint64_t* deltas, uint64_t* comm) {
    RSSV<uint64_t> D, O;
    RSSV<uint8_t> B;
    load(D, delta, n);
    load(B, relu_prime, n);
    CommIO io(comm);
    relu_layer_backward<uint64_t, uint8_t>(D, B, O, io.c);
    store(O, deltas);
    return 0;
}
extern "C" int or_maxpool_layer_backward_u64_u8(const uint64_t* delta, size_t n, const uint8_t* max_prime,
                                                uint64_t* deltas, int H, int W, int C, int pool, int stride, int batch,
                                                uint64_t* comm) {
    RSSV<uint64_t> D, O;
    RSSV<uint8_t> B;
    load(D, delta, n);
    load(B, max_prime, n * (size_t)pool * pool);
    CommIO io(comm);
    maxpool_layer_backward<uint64_t, uint8_t>(D, B, O, H, W, C, pool, stride, batch, io.c);
    store(O, deltas);
    return 0;
}
extern "C" int or_avgpool_layer_forward_u64(const uint64_t* in, uint64_t* out, int H, int W, int C, int pool,
                                            int stride, int batch, uint64_t* comm) {
    RSSV<uint64_t> A, O;
    load(A, in, (size_t)batch * H * W * C);
    CommIO io(comm);
    avgpool_layer_forward<uint64_t>(A, O, H, W, C, pool, stride, batch, io.c);
    store(O, out);
    return 0;
}
extern "C" int or_avgpool_layer_backward_u64(const uint64_t* delta, size_t n, uint64_t* deltas, int H, int W, int C,
                                             int pool, int batch, uint64_t* comm) {
    // the expansion writes n * pool^2 slots of the batch * H * W * C input
    // gradient; overlapping pools (stride < pool) would write past it
    if (n * (size_t)pool * pool > (size_t)batch * H * W * C) return 1;
    RSSV<uint64_t> D, O;
    load(D, delta, n);
    CommIO io(comm);
    avgpool_layer_backward<uint64_t>(D, O, H, W, C, pool, batch, io.c);
    store(O, deltas);
    return 0;
}
extern "C" int or_fc_layer_backward_u64(const uint64_t* delta, const uint64_t* fwd_in, uint64_t* w, uint64_t* b,
                                        uint64_t* deltas, int batch, int din, int dout, int fp, int lr, uint64_t* comm) {
    RSSV<uint64_t> D, X, Wt, Bs, O;
    load(D, delta, (size_t)batch * dout);
    load(X, fwd_in, (size_t)batch * din);
    load(Wt, w, (size_t)din * dout);
    load(Bs, b, (size_t)dout);
    CommIO io(comm);
    fc_layer_backward<uint64_t>(D, X, Wt, Bs, O, batch, din, dout, fp, lr, io.c);
    store(Wt, w);
    store(Bs, b);
    store(O, deltas);
    return 0;
}
extern "C" int or_cnn_layer_backward_u64(const uint64_t* delta, const uint64_t* fwd_in, uint64_t* w, uint64_t* deltas,
                                         int batch, int H, int W, int Din, int Dout, int f, int stride, int pad, int fp,
                                         int lr, uint64_t* comm) {
    const int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    RSSV<uint64_t> D, X, Wt, O;
    load(D, delta, (size_t)batch * P * Q * Dout);
    load(X, fwd_in, (size_t)batch * H * W * Din);
    load(Wt, w, (size_t)Dout * f * f * Din);
    CommIO io(comm);
    cnn_layer_backward<uint64_t>(D, X, Wt, O, batch, H, W, Din, Dout, f, stride, pad, fp, lr, io.c);
    store(Wt, w);
    store(O, deltas);
    return 0;
}
extern "C" int or_reveal_softmax_grad_u64(const uint64_t* act, const uint64_t* labels, size_t n, int batch, int fp,
                                          uint64_t* deltas, uint64_t* comm) {
    RSSV<uint64_t> A, L, O;
    load(A, act, n);
    load(L, labels, n);
    CommIO io(comm);
    rss_reveal_softmax_grad<uint64_t>(A, L, batch, fp, O, io.c);
    store(O, deltas);
    return 0;
}

// ------------------------------------------------------------------- TPC
// A TPC tensor crosses as one flat array [party(2)][n].

namespace {
template <typename T> void tload(TPCV<T>& r, const T* flat, size_t n) {
    r.resize(n);
    for (int p = 0; p < 2; p++) std::memcpy(r.s[p].data(), flat + (size_t)p * n, n * sizeof(T));
}
template <typename T> void tstore(const TPCV<T>& r, T* flat) {
    for (int p = 0; p < 2; p++) std::memcpy(flat + (size_t)p * r.n, r.s[p].data(), r.n * sizeof(T));
}
}  // namespace

#define OR_TPC(T, SUF)                                                                                       \
    extern "C" int or_tpc_matmul_##SUF(const T* a, const T* b, T* c, int M, int N, int K, int tA, int tB,     \
                                       int tC, int trunc, uint64_t* comm) {                                  \
        TPCV<T> A, B, C;                                                                                     \
        tload(A, a, (size_t)M * K);                                                                          \
        tload(B, b, (size_t)K * N);                                                                          \
        CommIO io(comm);                                                                                     \
        tpc_matmul<T>(A, B, C, M, N, K, tA, tB, tC, trunc, io.c);                                            \
        tstore(C, c);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_conv_##SUF(const T* a, size_t na, const T* b, size_t nb, T* c, int op, int batch,   \
                                     int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc,  \
                                     uint64_t* comm) {                                                       \
        TPCV<T> A, B, C;                                                                                     \
        tload(A, a, na);                                                                                     \
        tload(B, b, nb);                                                                                     \
        CommIO io(comm);                                                                                     \
        tpc_convolution<T>(A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc, io.c);                \
        tstore(C, c);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_divide_public_##SUF(T* a, size_t n, const T* d, int vector_d, uint64_t* comm) {     \
        TPCV<T> A;                                                                                           \
        tload(A, a, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        tpc_divide_public<T>(A, d, vector_d != 0, io.c);                                                     \
        tstore(A, a);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_reconstruct_##SUF(const T* a, size_t n, T* out, uint64_t* comm) {                  \
        TPCV<T> A;                                                                                           \
        tload(A, a, n);                                                                                      \
        std::vector<T> o[2];                                                                                 \
        CommIO io(comm);                                                                                     \
        tpc_reconstruct<T>(A, whole(n), o, io.c);                                                            \
        for (int p = 0; p < 2; p++) std::memcpy(out + (size_t)p * n, o[p].data(), n * sizeof(T));            \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_mul_##SUF(T* a, const T* b, size_t n, uint64_t* comm) {                            \
        TPCV<T> A, B;                                                                                        \
        tload(A, a, n);                                                                                      \
        tload(B, b, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        tpc_mul_assign<T>(A, whole(n), B, whole(n), io.c);                                                   \
        tstore(A, a);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_from_list_##SUF(const double* v, size_t n, int fp, int to_fixed, T* out) {         \
        TPCV<T> A(n);                                                                                        \
        tpc_from_list<T>(A, v, fp, to_fixed != 0);                                                           \
        tstore(A, out);                                                                                      \
        return 0;                                                                                            \
    }

#define OR_TPC_BITS(T, U, SUF)                                                                               \
    extern "C" int or_tpc_drelu_##SUF(const T* in, size_t n, U* out, uint64_t* comm) {                       \
        TPCV<T> A;                                                                                           \
        tload(A, in, n);                                                                                     \
        TPCV<U> R;                                                                                           \
        CommIO io(comm);                                                                                     \
        tpc_drelu<T, U>(A, whole(n), R, io.c);                                                               \
        tstore(R, out);                                                                                      \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_relu_##SUF(const T* in, size_t n, T* out, U* dout, uint64_t* comm) {               \
        TPCV<T> A, O;                                                                                        \
        tload(A, in, n);                                                                                     \
        TPCV<U> D;                                                                                           \
        CommIO io(comm);                                                                                     \
        tpc_relu<T, U>(A, O, D, io.c);                                                                       \
        tstore(O, out);                                                                                      \
        tstore(D, dout);                                                                                     \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_select_share_##SUF(const T* x, const T* y, const U* b, size_t n, T* z,             \
                                             uint64_t* comm) {                                               \
        TPCV<T> X, Y, Z(n);                                                                                  \
        tload(X, x, n);                                                                                      \
        tload(Y, y, n);                                                                                      \
        TPCV<U> B;                                                                                           \
        tload(B, b, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        tpc_select_share<T, U>(X, whole(n), Y, whole(n), B, Z, whole(n), io.c);                              \
        tstore(Z, z);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_tpc_maxpool_##SUF(const T* in, size_t n, int k, T* out, U* dout, uint64_t* comm) {     \
        TPCV<T> A, O;                                                                                        \
        tload(A, in, n);                                                                                     \
        TPCV<U> D;                                                                                           \
        CommIO io(comm);                                                                                     \
        tpc_maxpool<T, U>(A, O, D, k, io.c);                                                                 \
        tstore(O, out);                                                                                      \
        tstore(D, dout);                                                                                     \
        return 0;                                                                                            \
    }

OR_TPC(uint64_t, u64)
OR_TPC(uint32_t, u32)
OR_TPC_BITS(uint64_t, uint8_t, u64_u8)
OR_TPC_BITS(uint64_t, uint64_t, u64_u64)
OR_TPC_BITS(uint32_t, uint8_t, u32_u8)

extern "C" int or_tpc_reconstruct_u8(const uint8_t* a, size_t n, uint8_t* out, uint64_t* comm) {
    TPCV<uint8_t> A;
    tload(A, a, n);
    std::vector<uint8_t> o[2];
    CommIO io(comm);
    tpc_reconstruct<uint8_t>(A, whole(n), o, io.c);
    for (int p = 0; p < 2; p++) std::memcpy(out + (size_t)p * n, o[p].data(), n);
    return 0;
}

// ------------------------------------------------------------------- FPC
// An FPC tensor crosses as one flat array [party(4)][share(3)][n].

namespace {
template <typename T> void fload(FPCV<T>& r, const T* flat, size_t n) {
    r.resize(n);
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++) std::memcpy(r.s[p][k].data(), flat + ((size_t)p * 3 + k) * n, n * sizeof(T));
}
template <typename T> void fstore(const FPCV<T>& r, T* flat) {
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++) std::memcpy(flat + ((size_t)p * 3 + k) * r.n, r.s[p][k].data(), r.n * sizeof(T));
}
}  // namespace

#define OR_FPC(T, SUF)                                                                                       \
    extern "C" int or_fpc_matmul_##SUF(const T* a, const T* b, T* c, int M, int N, int K, int tA, int tB,     \
                                       int tC, int trunc, uint64_t* comm) {                                  \
        FPCV<T> A, B, C;                                                                                     \
        fload(A, a, (size_t)M * K);                                                                          \
        fload(B, b, (size_t)K * N);                                                                          \
        CommIO io(comm);                                                                                     \
        fpc_matmul<T>(A, B, C, M, N, K, tA, tB, tC, trunc, io.c);                                            \
        fstore(C, c);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_conv_##SUF(const T* a, size_t na, const T* b, size_t nb, T* c, int op, int batch,   \
                                     int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc,  \
                                     uint64_t* comm) {                                                       \
        FPCV<T> A, B, C;                                                                                     \
        fload(A, a, na);                                                                                     \
        fload(B, b, nb);                                                                                     \
        CommIO io(comm);                                                                                     \
        fpc_convolution<T>(A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc, io.c);                \
        fstore(C, c);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_divide_public_##SUF(T* a, size_t n, const T* d, int vector_d, uint64_t* comm) {     \
        FPCV<T> A;                                                                                           \
        fload(A, a, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        fpc_divide_public<T>(A, d, vector_d != 0, io.c);                                                     \
        fstore(A, a);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_reconstruct_##SUF(const T* a, size_t n, T* out, uint64_t* comm) {                  \
        FPCV<T> A;                                                                                           \
        fload(A, a, n);                                                                                      \
        std::vector<T> o[4];                                                                                 \
        CommIO io(comm);                                                                                     \
        fpc_reconstruct<T>(A, whole(n), o, io.c);                                                            \
        for (int p = 0; p < 4; p++) std::memcpy(out + (size_t)p * n, o[p].data(), n * sizeof(T));            \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_mul_##SUF(T* a, const T* b, size_t n, uint64_t* comm) {                            \
        FPCV<T> A, B;                                                                                        \
        fload(A, a, n);                                                                                      \
        fload(B, b, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        fpc_mul_assign<T>(A, whole(n), B, whole(n), io.c);                                                   \
        fstore(A, a);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_and_##SUF(T* a, const T* b, size_t n, uint64_t* comm) {                            \
        FPCV<T> A, B;                                                                                        \
        fload(A, a, n);                                                                                      \
        fload(B, b, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        fpc_and_assign<T>(A, whole(n), B, whole(n), io.c);                                                   \
        fstore(A, a);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_from_list_##SUF(const double* v, size_t n, int fp, int to_fixed, T* out) {         \
        FPCV<T> A(n);                                                                                        \
        fpc_from_list<T>(A, v, fp, to_fixed != 0);                                                           \
        fstore(A, out);                                                                                      \
        return 0;                                                                                            \
    }

#define OR_FPC_BITS(T, U, SUF)                                                                               \
    extern "C" int or_fpc_drelu_##SUF(const T* in, size_t n, U* out, uint64_t* comm) {                       \
        FPCV<T> A;                                                                                           \
        fload(A, in, n);                                                                                     \
        FPCV<U> R;                                                                                           \
        CommIO io(comm);                                                                                     \
        fpc_drelu<T, U>(A, whole(n), R, io.c);                                                               \
        fstore(R, out);                                                                                      \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_relu_##SUF(const T* in, size_t n, T* out, U* dout, uint64_t* comm) {               \
        FPCV<T> A, O;                                                                                        \
        fload(A, in, n);                                                                                     \
        FPCV<U> D;                                                                                           \
        CommIO io(comm);                                                                                     \
        fpc_relu<T, U>(A, O, D, io.c);                                                                       \
        fstore(O, out);                                                                                      \
        fstore(D, dout);                                                                                     \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_select_share_##SUF(const T* x, const T* y, const U* b, size_t n, T* z,             \
                                             uint64_t* comm) {                                               \
        FPCV<T> X, Y, Z(n);                                                                                  \
        fload(X, x, n);                                                                                      \
        fload(Y, y, n);                                                                                      \
        FPCV<U> B;                                                                                           \
        fload(B, b, n);                                                                                      \
        CommIO io(comm);                                                                                     \
        fpc_select_share<T, U>(X, whole(n), Y, whole(n), B, Z, whole(n), io.c);                              \
        fstore(Z, z);                                                                                        \
        return 0;                                                                                            \
    }                                                                                                        \
    extern "C" int or_fpc_maxpool_##SUF(const T* in, size_t n, int k, T* out, U* dout, uint64_t* comm) {     \
        FPCV<T> A, O;                                                                                        \
        fload(A, in, n);                                                                                     \
        FPCV<U> D;                                                                                           \
        CommIO io(comm);                                                                                     \
        fpc_maxpool<T, U>(A, O, D, k, io.c);                                                                 \
        fstore(O, out);                                                                                      \
        fstore(D, dout);                                                                                     \
        return 0;                                                                                            \
    }

OR_FPC(uint64_t, u64)
OR_FPC(uint32_t, u32)
OR_FPC(uint8_t, u8)
OR_FPC_BITS(uint64_t, uint8_t, u64_u8)
OR_FPC_BITS(uint64_t, uint64_t, u64_u64)
OR_FPC_BITS(uint32_t, uint8_t, u32_u8)

// AESObject's counter-mode stream (aes.hpp) and one AES-256 block
extern "C" void or_prg_fill_u64(const uint8_t* key, uint64_t ctr, uint64_t* out, size_t n) {
    prg_fill_u64(key, ctr, out, n);
}
extern "C" void or_aes256_encrypt(const uint8_t* key, const uint8_t* in, uint8_t* out) {
    aes256_encrypt_block(key, in, out);
}
