// pg_tpc.cu — the 2-party protocol (TPC: src/mpc/TPC.h, TPC.inl) on one GPU.
//
// A TPC tensor of n elements is two device arrays [party A, party B]; the
// value is their sum. Piranha's TPC multiplications use constant Beaver
// triples (Precompute.h: elementwise x = y = z = 1, the matrix triple x = y = 1
// and z = K, convolution triples 0), and adding public data to a share only
// changes party A's (TPC.inl:175-189). Worked through, every operation here
// has a closed form in the revealed values, with the result held by party A
// and party B's share 0 unless an input share passes through unchanged:
//   reconstruct (TPC.inl:552-572)        out_p = a_A + a_B
//   dividePublic (TPC.inl:371-401)       (1 + (a - d) / d, 0)
//   matmul (TPC.inl:575-583, 1060-1091)  (1 + (ab - d) / d, 0), ab = (a_A+a_B)(b_A+b_B)
//   convolution (TPC.inl:789-827)        the same with conv(a, b)
//   x *= y (TPC.inl:242-272)             (x y, 0)
//   dReLU (TPC.inl:829-868)              (bit, 0); the carry circuit over the
//                                        revealed a = x + 1 and r = all ones
//                                        reduces to bit = 1 - ([a mod 2^(W-1) != 0] ^ 1 ^ msb(a))
//   selectShare (TPC.inl:586-610)        (d (y - x) + x_A, x_B), d = [b_A + b_B == 1]
//   ReLU (TPC.inl:871-884)               (bit x, 0) and dReLU's bit shares
// The message bytes and rounds are those the reference's reveals would send
// (each Beaver multiplication reveals its two masked operands).
#include <cstring>

#include "pg_common.cuh"

namespace pg {

template <typename T> int plain_gemm(Ctx *, int, int, int, const T *, int, const T *, int, T *, int);
int plain_conv_u64(Ctx *, int, int, int, int, int, int, int, int, int, int, const uint64_t *, const uint64_t *,
                   uint64_t *);

namespace tpc {

static unsigned grid_for(Ctx *c, size_t n, int per_sm = 16) {
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    size_t b = (n + 255) / 256;
    if (b > (size_t)sms * per_sm) b = (size_t)sms * per_sm;
    return (unsigned)(b ? b : 1);
}

// one reveal of n elements of `bytes` each by both parties: one round
static void reveal_comm(Ctx *c, uint64_t n, uint64_t bytes) {
    for (int p = 0; p < 2; p++) {
        c->comm[p] += n * bytes;
        c->comm[4 + p] += n * bytes;
    }
    c->comm[8] += 1;
}

template <typename T> __device__ __forceinline__ int dbit(T v) {
    constexpr int W = sizeof(T) * 8;
    const T a = (T)(v + 1);
    const T low = a & (((T)1 << (W - 1)) - 1);
    const int carry = low != 0;
    const int msb = (int)(a >> (W - 1));
    return 1 - (carry ^ 1 ^ msb);
}

template <typename T> __global__ void sum_kernel(const T *a0, const T *a1, T *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (T)(a0[i] + a1[i]);
}

template <typename T> __global__ void reconstruct_kernel(const T *a0, const T *a1, T *o0, T *o1, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const T v = (T)(a0[i] + a1[i]);
        o0[i] = v;
        o1[i] = v;
    }
}

// dividePublic on (a0, a1) in place; z1 == nullptr means the value is z0 alone.
// bias (per column n % ncols, or n / rows for column-major) is added per share.
template <typename T>
__global__ void divide_kernel(const T *z0, const T *z1, T *o0, T *o1, size_t n, T d, const T *dvec, int dshift,
                              const T *b0, const T *b1, int ncols, int rows, int colmajor) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const T dd = dvec ? dvec[i] : d;
        const T v = (T)(z0[i] + (z1 ? z1[i] : (T)0));
        T r0 = (T)(1 + div_public<T>((T)(v - dd), dd, dvec ? -1 : dshift));
        T r1 = 0;
        if (b0) {
            const size_t col = colmajor ? i / (size_t)rows : i % (size_t)ncols;
            r0 = (T)(r0 + b0[col]);
            r1 = b1[col];
        }
        o0[i] = r0;
        o1[i] = r1;
    }
}

template <typename T> __global__ void mul_kernel(T *a0, T *a1, const T *b0, const T *b1, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        a0[i] = (T)((T)(a0[i] + a1[i]) * (T)(b0[i] + b1[i]));
        a1[i] = 0;
    }
}

template <typename T, typename U> __global__ void drelu_kernel(const T *x0, const T *x1, U *o0, U *o1, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        o0[i] = (U)dbit<T>((T)(x0[i] + x1[i]));
        o1[i] = 0;
    }
}

template <typename T, typename U>
__global__ void relu_kernel(const T *x0, const T *x1, T *y0, T *y1, U *d0, U *d1, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const T v = (T)(x0[i] + x1[i]);
        const int b = dbit<T>(v);
        y0[i] = b ? v : (T)0;
        y1[i] = 0;
        d0[i] = (U)b;
        d1[i] = 0;
    }
}

template <typename T, typename U>
__global__ void select_kernel(const T *x0, const T *x1, const T *y0, const T *y1, const U *b0, const U *b1, T *z0,
                              T *z1, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const U e = (U)(b0[i] + b1[i]);
        const T xa = x0[i], xb = x1[i];
        const T diff = (T)((T)(y0[i] + y1[i]) - (T)(xa + xb));
        z0[i] = (T)((e == (U)1 ? diff : (T)0) + xa);
        z1[i] = xb;
    }
}

// Tournament over rows of k values (TPC.inl:887-1058): per level the pair
// (even, odd) of each slot gives b = dReLU(even - odd), even <- select(odd,
// even, b), and the row's derivative bits are ANDed with b expanded over the
// slots that pair covers (expandCompare, bitwise.cuh:66-92).
template <typename T, typename U, int K>
__global__ void maxpool_kernel(const T *in0, const T *in1, size_t rows, T *o0, T *o1, U *d0, U *d1) {
    for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < rows; r += (size_t)gridDim.x * blockDim.x) {
        T a[K], b[K];
        int d[K];
#pragma unroll
        for (int j = 0; j < K; j++) {
            a[j] = in0[r * K + j];
            b[j] = in1[r * K + j];
            d[j] = 1;
        }
#pragma unroll
        for (int s = 1; s < K; s *= 2) {
            // slots j = 0, 2s, 4s, ... compare with j + s
#pragma unroll
            for (int j = 0; j < K; j += 2 * s) {
                const T ev = (T)(a[j] + b[j]), ov = (T)(a[j + s] + b[j + s]);
                const int bit = dbit<T>((T)(ev - ov));
                // select(x = odd, y = even, b)
                a[j] = (T)((bit ? (T)(ev - ov) : (T)0) + a[j + s]);
                b[j] = b[j + s];
                // expandCompare: the first s slots of the pair's 2s get bit, the rest 1 - bit
#pragma unroll
                for (int e = 0; e < 2 * s; e++) d[j + e] &= (e < s ? bit : 1 - bit);
            }
        }
        o0[r] = a[0];
        o1[r] = b[0];
#pragma unroll
        for (int j = 0; j < K; j++) {
            d0[r * K + j] = (U)d[j];
            d1[r * K + j] = 0;
        }
    }
}

// ------------------------------------------------------------------- host

template <typename T> static bool ok2(const T *const *a) { return a && a[0] && a[1]; }

template <typename T> static int pow2_of(T d) {
    if (d == 0 || (d & (d - 1))) return -1;
    int t = 0;
    while (((T)1 << t) != d) t++;
    return t <= (int)(sizeof(T) * 8 - 2) ? t : -1;
}

template <typename T>
int matmul(Ctx *c, const T *const a[2], const T *const b[2], T *const out[2], const T *const bias[2], int M, int N,
           int K, int tA, int tB, int tC, int trunc) {
    if (!ok2(a) || !ok2(b) || !ok2(out) || (bias && !ok2(bias))) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    if (trunc < 0 || trunc > (int)sizeof(T) * 8 - 2) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t mk = (size_t)M * K, kn = (size_t)K * N, mn = (size_t)M * N;
    uint8_t *s = (uint8_t *)scratch(c, al(mk * sizeof(T)) + al(kn * sizeof(T)) + al(mn * sizeof(T)));
    if (!s) return PG_ERR_NO_MEMORY;
    T *ea = (T *)s, *eb = (T *)(s + al(mk * sizeof(T))), *z = (T *)(s + al(mk * sizeof(T)) + al(kn * sizeof(T)));
    // localMatMul reveals e = x + a and f = y + b; with x = y = 1 the product
    // the three GEMMs leave in party A's share is (a_A + a_B)(b_A + b_B)
    sum_kernel<T><<<grid_for(c, mk), 256, 0, c->stream>>>(a[0], a[1], ea, mk);
    sum_kernel<T><<<grid_for(c, kn), 256, 0, c->stream>>>(b[0], b[1], eb, kn);
    c->launches += 2;
    int st = launch_status(c, "tpc sum_kernel");
    if (st) return st;
    st = plain_gemm<T>(c, M, N, K, ea, tA, eb, tB, z, tC);
    if (st) return st;
    const T d = (T)((T)1 << trunc);
    divide_kernel<T><<<grid_for(c, mn), 256, 0, c->stream>>>(z, nullptr, out[0], out[1], mn, d, nullptr, trunc,
                                                             bias ? bias[0] : nullptr, bias ? bias[1] : nullptr, N,
                                                             M, tC ? 0 : 1);
    c->launches++;
    st = launch_status(c, "tpc divide_kernel");
    if (st) return st;
    reveal_comm(c, mk, sizeof(T));
    reveal_comm(c, kn, sizeof(T));
    reveal_comm(c, mn, sizeof(T));
    return PG_OK;
}

int conv_u64(Ctx *c, const uint64_t *const A[2], const uint64_t *const B[2], uint64_t *const C[2], int op, int batch,
             int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    if (!ok2(A) || !ok2(B) || !ok2(C)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Din <= 0 || Dout <= 0 || stride <= 0 || pad < 0 ||
        H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "convolution: bad geometry");
    if (op < PG_CONV_FPROP || op > PG_CONV_WGRAD) return set_error(c, PG_ERR_INVALID_ARG, "bad conv op %d", op);
    if (trunc < 0 || trunc > 62) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    const int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    const size_t nx = (size_t)batch * H * W * Din, nw = (size_t)Dout * f * f * Din, ny = (size_t)batch * P * Q * Dout;
    const size_t na = op == PG_CONV_FPROP ? nx : ny;
    const size_t nb = op == PG_CONV_WGRAD ? nx : nw;
    const size_t nc = op == PG_CONV_FPROP ? ny : op == PG_CONV_DGRAD ? nx : nw;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    uint8_t *s = (uint8_t *)scratch(c, al(na * 8) + al(nb * 8) + al(nc * 8));
    if (!s) return PG_ERR_NO_MEMORY;
    uint64_t *ea = (uint64_t *)s, *eb = (uint64_t *)(s + al(na * 8)), *z = (uint64_t *)(s + al(na * 8) + al(nb * 8));
    sum_kernel<uint64_t><<<grid_for(c, na), 256, 0, c->stream>>>(A[0], A[1], ea, na);
    sum_kernel<uint64_t><<<grid_for(c, nb), 256, 0, c->stream>>>(B[0], B[1], eb, nb);
    c->launches += 2;
    int st = launch_status(c, "tpc sum_kernel");
    if (st) return st;
    // pg_conv_u64 argument order: (op, N, H, W, C, K, R, S, pad, stride, a, b, out)
    st = plain_conv_u64(c, op, batch, H, W, Din, Dout, f, f, pad, stride, ea, eb, z);
    if (st) return st;
    divide_kernel<uint64_t><<<grid_for(c, nc), 256, 0, c->stream>>>(z, nullptr, C[0], C[1], nc, 1ull << trunc, nullptr,
                                                                    trunc, nullptr, nullptr, 1, 1, 0);
    c->launches++;
    st = launch_status(c, "tpc divide_kernel");
    if (st) return st;
    reveal_comm(c, na, 8);
    reveal_comm(c, nb, 8);
    reveal_comm(c, nc, 8);
    return PG_OK;
}

template <typename T> int divide_public(Ctx *c, T *const a[2], size_t n, T d, const T *dvec) {
    if (!dvec && d == 0) return set_error(c, PG_ERR_INVALID_ARG, "division by zero");
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        reveal_comm(c, 0, sizeof(T));
        return PG_OK;
    }
    if (!ok2(a)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    divide_kernel<T><<<grid_for(c, n), 256, 0, c->stream>>>(a[0], a[1], a[0], a[1], n, d, dvec, pow2_of<T>(d),
                                                            nullptr, nullptr, 1, 1, 0);
    c->launches++;
    int st = launch_status(c, "tpc divide_kernel");
    if (st) return st;
    reveal_comm(c, n, sizeof(T));
    return PG_OK;
}

template <typename T> int reconstruct(Ctx *c, const T *const a[2], size_t n, T *const out[2]) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        reveal_comm(c, 0, sizeof(T));
        return PG_OK;
    }
    if (!ok2(a) || !ok2(out)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    reconstruct_kernel<T><<<grid_for(c, n), 256, 0, c->stream>>>(a[0], a[1], out[0], out[1], n);
    c->launches++;
    int st = launch_status(c, "tpc reconstruct_kernel");
    if (st) return st;
    reveal_comm(c, n, sizeof(T));
    return PG_OK;
}

template <typename T> int mul(Ctx *c, T *const a[2], const T *const b[2], size_t n) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        reveal_comm(c, 0, sizeof(T));  // e = x + a
        reveal_comm(c, 0, sizeof(T));  // f = y + b
        return PG_OK;
    }
    if (!ok2(a) || !ok2(b)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    mul_kernel<T><<<grid_for(c, n), 256, 0, c->stream>>>(a[0], a[1], b[0], b[1], n);
    c->launches++;
    int st = launch_status(c, "tpc mul_kernel");
    if (st) return st;
    reveal_comm(c, n, sizeof(T));  // e = x + a
    reveal_comm(c, n, sizeof(T));  // f = y + b
    return PG_OK;
}

// bytes and rounds of dReLU (TPC.inl:829-868): the reveal of the input, then
// per carry level two ANDs on the level's half-size views, each revealing its
// two masked operands
template <typename T, typename U> static void drelu_comm(Ctx *c, uint64_t n) {
    reveal_comm(c, n, sizeof(T));
    for (int half = (int)sizeof(T) * 4; half >= 1; half /= 2)
        for (int r = 0; r < 4; r++) reveal_comm(c, n * half, sizeof(U));
}

template <typename T, typename U> int drelu(Ctx *c, const T *const in[2], size_t n, U *const out[2]) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        drelu_comm<T, U>(c, 0);
        return PG_OK;
    }
    if (!ok2(in) || !ok2(out)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    drelu_kernel<T, U><<<grid_for(c, n), 256, 0, c->stream>>>(in[0], in[1], out[0], out[1], n);
    c->launches++;
    int st = launch_status(c, "tpc drelu_kernel");
    if (st) return st;
    drelu_comm<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U> static void select_comm(Ctx *c, uint64_t n) {
    reveal_comm(c, n, sizeof(U));  // e = b
    reveal_comm(c, n, sizeof(T));  // the multiplication's two reveals
    reveal_comm(c, n, sizeof(T));
}

template <typename T, typename U>
int relu(Ctx *c, const T *const in[2], size_t n, T *const out[2], U *const dout[2]) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        drelu_comm<T, U>(c, 0);
        select_comm<T, U>(c, 0);
        return PG_OK;
    }
    if (!ok2(in) || !ok2(out) || !ok2(dout)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    relu_kernel<T, U><<<grid_for(c, n), 256, 0, c->stream>>>(in[0], in[1], out[0], out[1], dout[0], dout[1], n);
    c->launches++;
    int st = launch_status(c, "tpc relu_kernel");
    if (st) return st;
    drelu_comm<T, U>(c, n);
    select_comm<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int select_share(Ctx *c, const T *const x[2], const T *const y[2], const U *const b[2], T *const z[2], size_t n) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        select_comm<T, U>(c, 0);
        return PG_OK;
    }
    if (!ok2(x) || !ok2(y) || !ok2(b) || !ok2(z)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    select_kernel<T, U><<<grid_for(c, n), 256, 0, c->stream>>>(x[0], x[1], y[0], y[1], b[0], b[1], z[0], z[1], n);
    c->launches++;
    int st = launch_status(c, "tpc select_kernel");
    if (st) return st;
    select_comm<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int maxpool(Ctx *c, const T *const in[2], size_t n, int k, T *const out[2], U *const dout[2]) {
    if (n && (!ok2(in) || !ok2(out) || !ok2(dout))) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (k != 4 && k != 16 && k != 2 && k != 8)
        return set_error(c, PG_ERR_UNSUPPORTED, "maxpool rows of %d (2, 4, 8 or 16 supported)", k);
    if (n % (size_t)k) return set_error(c, PG_ERR_SIZE, "maxpool input %zu is not a multiple of %d", n, k);
    const size_t rows = n / k;
    if (rows == 0) return PG_OK;
    switch (k) {
        case 2: maxpool_kernel<T, U, 2><<<grid_for(c, rows), 256, 0, c->stream>>>(in[0], in[1], rows, out[0], out[1], dout[0], dout[1]); break;
        case 4: maxpool_kernel<T, U, 4><<<grid_for(c, rows), 256, 0, c->stream>>>(in[0], in[1], rows, out[0], out[1], dout[0], dout[1]); break;
        case 8: maxpool_kernel<T, U, 8><<<grid_for(c, rows), 256, 0, c->stream>>>(in[0], in[1], rows, out[0], out[1], dout[0], dout[1]); break;
        default: maxpool_kernel<T, U, 16><<<grid_for(c, rows), 128, 0, c->stream>>>(in[0], in[1], rows, out[0], out[1], dout[0], dout[1]); break;
    }
    c->launches++;
    int st = launch_status(c, "tpc maxpool_kernel");
    if (st) return st;
    // per level: dReLU and selectShare on the level's pairs, AND over all n derivative bits
    for (size_t m = n / 2; m >= rows && m > 0; m /= 2) {
        drelu_comm<T, U>(c, m);
        select_comm<T, U>(c, m);
        reveal_comm(c, n, sizeof(U));
        reveal_comm(c, n, sizeof(U));
        if (m == rows) break;
    }
    return PG_OK;
}

}  // namespace tpc
}  // namespace pg

using namespace pg;

#define TPC_CTX(c) \
    if (!(c)) return PG_ERR_INVALID_ARG

extern "C" {

int pg_tpc_matmul_u64(pg_ctx *c, const uint64_t *const a[2], const uint64_t *const b[2], uint64_t *const out[2],
                      int M, int N, int K, int tA, int tB, int tC, int trunc) {
    TPC_CTX(c);
    return tpc::matmul<uint64_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}
int pg_tpc_matmul_u32(pg_ctx *c, const uint32_t *const a[2], const uint32_t *const b[2], uint32_t *const out[2],
                      int M, int N, int K, int tA, int tB, int tC, int trunc) {
    TPC_CTX(c);
    return tpc::matmul<uint32_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}
int pg_tpc_fc_forward_u64(pg_ctx *c, const uint64_t *const x[2], const uint64_t *const w[2],
                          const uint64_t *const bias[2], uint64_t *const out[2], int batch, int din, int dout, int fp) {
    TPC_CTX(c);
    return tpc::matmul<uint64_t>(c, x, w, out, bias, batch, dout, din, 1, 1, 1, fp);
}
int pg_tpc_fc_forward_u32(pg_ctx *c, const uint32_t *const x[2], const uint32_t *const w[2],
                          const uint32_t *const bias[2], uint32_t *const out[2], int batch, int din, int dout, int fp) {
    TPC_CTX(c);
    return tpc::matmul<uint32_t>(c, x, w, out, bias, batch, dout, din, 1, 1, 1, fp);
}
int pg_tpc_conv_u64(pg_ctx *c, const uint64_t *const A[2], const uint64_t *const B[2], uint64_t *const C[2], int op,
                    int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    TPC_CTX(c);
    return tpc::conv_u64(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc);
}
int pg_tpc_divide_public_u64(pg_ctx *c, uint64_t *const a[2], size_t n, uint64_t d) {
    TPC_CTX(c);
    return tpc::divide_public<uint64_t>(c, a, n, d, nullptr);
}
int pg_tpc_divide_public_vec_u64(pg_ctx *c, uint64_t *const a[2], size_t n, const uint64_t *d) {
    TPC_CTX(c);
    if (!d && n) return set_error(c, PG_ERR_INVALID_ARG, "null denominators");
    return tpc::divide_public<uint64_t>(c, a, n, 0, d);
}
int pg_tpc_divide_public_u32(pg_ctx *c, uint32_t *const a[2], size_t n, uint32_t d) {
    TPC_CTX(c);
    return tpc::divide_public<uint32_t>(c, a, n, d, nullptr);
}
int pg_tpc_reconstruct_u64(pg_ctx *c, const uint64_t *const a[2], size_t n, uint64_t *const out[2]) {
    TPC_CTX(c);
    return tpc::reconstruct<uint64_t>(c, a, n, out);
}
int pg_tpc_reconstruct_u32(pg_ctx *c, const uint32_t *const a[2], size_t n, uint32_t *const out[2]) {
    TPC_CTX(c);
    return tpc::reconstruct<uint32_t>(c, a, n, out);
}
int pg_tpc_reconstruct_u8(pg_ctx *c, const uint8_t *const a[2], size_t n, uint8_t *const out[2]) {
    TPC_CTX(c);
    return tpc::reconstruct<uint8_t>(c, a, n, out);
}
int pg_tpc_mul_u64(pg_ctx *c, uint64_t *const a[2], const uint64_t *const b[2], size_t n) {
    TPC_CTX(c);
    return tpc::mul<uint64_t>(c, a, b, n);
}
int pg_tpc_drelu_u64_u8(pg_ctx *c, const uint64_t *const in[2], size_t n, uint8_t *const out[2]) {
    TPC_CTX(c);
    return tpc::drelu<uint64_t, uint8_t>(c, in, n, out);
}
int pg_tpc_drelu_u32_u8(pg_ctx *c, const uint32_t *const in[2], size_t n, uint8_t *const out[2]) {
    TPC_CTX(c);
    return tpc::drelu<uint32_t, uint8_t>(c, in, n, out);
}
int pg_tpc_relu_u64_u8(pg_ctx *c, const uint64_t *const in[2], size_t n, uint64_t *const out[2],
                       uint8_t *const dout[2]) {
    TPC_CTX(c);
    return tpc::relu<uint64_t, uint8_t>(c, in, n, out, dout);
}
int pg_tpc_relu_u32_u8(pg_ctx *c, const uint32_t *const in[2], size_t n, uint32_t *const out[2],
                       uint8_t *const dout[2]) {
    TPC_CTX(c);
    return tpc::relu<uint32_t, uint8_t>(c, in, n, out, dout);
}
int pg_tpc_select_share_u64_u8(pg_ctx *c, const uint64_t *const x[2], const uint64_t *const y[2],
                               const uint8_t *const b[2], uint64_t *const z[2], size_t n) {
    TPC_CTX(c);
    return tpc::select_share<uint64_t, uint8_t>(c, x, y, b, z, n);
}
int pg_tpc_maxpool_u64_u8(pg_ctx *c, const uint64_t *const in[2], size_t n, int k, uint64_t *const out[2],
                          uint8_t *const dout[2]) {
    TPC_CTX(c);
    return tpc::maxpool<uint64_t, uint8_t>(c, in, n, k, out, dout);
}

}  // extern "C"
