// pg_fpc.cu — the 4-party protocol (FPC: src/mpc/FPC.h, FPC.inl) on one GPU.
//
// An FPC tensor of n elements is twelve device arrays [party * 3 + share],
// parties A..D = 0..3. Party p's share k holds component x_{(p+1+k) mod 4} of
// x = x0 + x1 + x2 + x3 (FPC.inl:948-953); public values live in x0, which
// party A does not hold (FPC.inl:120-155, :184-260). Every simulated party's
// arrays are computed as the reference computes them at that party, so views
// that disagree between parties (reshareFPC adds different cross terms at
// parties I and J) come out the same as the reference's.
//
//   elementwise products (FPC *=, &=: FPC.inl:322-399) run the six reshares
//     per element in registers;
//   matmul / convolution (FPC.inl:636-670, :862-925) collapse through
//     dividePublic: party A ends with zeros, party p = B, C, D with
//     x0 = 1 + (R_p - d) / d and its other shares zero, where R_p is p's
//     reveal of the reshared products, a fixed sum of local GEMMs
//     a_{u,i} b_{u,j} that fpc_reveal_terms derives by running the reshare
//     schedule symbolically; one fused ring GEMM per party computes it;
//   dReLU (FPC.inl:930-990): the masks r are public-only (fill(1)) and every
//     carry-tree AND reshares zero cross terms, so party p >= 1 ends with
//     x0 = 1 - ([a mod 2^(W-1) != 0] ^ 1 ^ msb(a)) for its own reveal a = x + 1,
//     every other share 0;
//   selectShare / ReLU / maxpool follow FPC.inl:672-711, :992-1003, :1005-1177
//     with the products simulated per element.
// The byte and round counters follow reconstruct (every party sends n
// elements to the next, 1 round) and reshareFPC (party I sends n elements to
// party G, 1 round per call).
#include <cstring>

#include "pg_common.cuh"

namespace pg {

template <typename T>
int fpc_party_gemm(Ctx *, const SegList<T> &, int, int, int, int, int, int, T *const *, const T *const *, int, int);
int fpc_party_conv_u64(Ctx *, const SegList<uint64_t> &, int, int, int, int, int, int, int, int, int,
                       uint64_t *const *, int, int);

namespace fpc {

// reshareFPC pairs q = 0..5 in call order: (I, J) = (0,1) (0,2) (0,3) (1,2)
// (1,3) (2,3), with partyG / partyH (FPC.inl:452-496)
__host__ __device__ constexpr int pI(int q) { return q < 3 ? 0 : q < 5 ? 1 : 2; }
__host__ __device__ constexpr int pJ(int q) { return q == 0 ? 1 : q == 1 || q == 3 ? 2 : 3; }
__host__ __device__ constexpr int pG(int q) { return q == 0 ? 2 : q == 1 || q == 2 ? 1 : q == 3 ? 3 : q == 4 ? 2 : 0; }
__host__ __device__ constexpr int pH(int q) { return q < 2 ? 3 : q == 2 ? 2 : q < 5 ? 0 : 1; }

// the share index at which party p holds component c (shareH, FPC.inl:498-504)
__host__ __device__ constexpr int share_of(int p, int c) { return (3 - p + c) & 3; }
__host__ __device__ constexpr int x0_share(int p) { return p == 0 ? -1 : share_of(p, 0); }

template <typename T> struct F12 {
    T *p[12];
};
template <typename T> struct CF12 {
    const T *p[12];
};

static unsigned grid_for(Ctx *c, size_t n, int per_sm = 16) {
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    size_t b = (n + 255) / 256;
    if (b > (size_t)sms * per_sm) b = (size_t)sms * per_sm;
    return (unsigned)(b ? b : 1);
}

// reconstruct: every party sends n elements to the next one; 1 round
static void reveal_comm(Ctx *c, uint64_t n, uint64_t bytes) {
    for (int p = 0; p < 4; p++) {
        c->comm[p] += n * bytes;
        c->comm[4 + p] += n * bytes;
    }
    c->comm[8] += 1;
}
// the six reshareFPC calls of one product: I sends n elements to G, 1 round each
static void reshare_comm(Ctx *c, uint64_t n, uint64_t bytes) {
    for (int q = 0; q < 6; q++) {
        c->comm[pI(q)] += n * bytes;
        c->comm[4 + pG(q)] += n * bytes;
    }
    c->comm[8] += 6;
}
template <typename T, typename U> static void drelu_comm(Ctx *c, uint64_t n) {
    reveal_comm(c, n, sizeof(T));
    for (int half = (int)sizeof(T) * 4; half >= 1; half /= 2) {
        reshare_comm(c, n * half, sizeof(U));  // gEven &= pOdd
        reshare_comm(c, n * half, sizeof(U));  // pEven &= pOdd
    }
}
template <typename T, typename U> static void select_comm(Ctx *c, uint64_t n) {
    reveal_comm(c, n, sizeof(U));    // e = reveal(b ^ c), c = 0
    reshare_comm(c, n, sizeof(T));  // (y - x) *= d
}

// ------------------------------------------------------------ device helpers

template <typename T> __device__ __forceinline__ void load12(const CF12<T> &a, size_t i, T (&v)[4][3]) {
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) v[p][k] = a.p[p * 3 + k][i];
}
template <typename T> __device__ __forceinline__ void load12(const F12<T> &a, size_t i, T (&v)[4][3]) {
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) v[p][k] = a.p[p * 3 + k][i];
}
template <typename T> __device__ __forceinline__ void store12(const F12<T> &a, size_t i, const T (&v)[4][3]) {
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) a.p[p * 3 + k][i] = v[p][k];
}

// party p's reveal: its own three shares plus the previous party's shareA
template <typename T> __device__ __forceinline__ T reveal_at(const T (&v)[4][3], int p) {
    return (T)(v[p][0] + v[p][1] + v[p][2] + v[(p + 3) & 3][0]);
}

// FPC *= FPC (BOOL = false) or &= (BOOL = true) on one element, in place:
// the local cross terms z, z', the diagonal products, then reshareFPC for the
// six pairs, each adding z or z' (z' for opposite parties) to component H at
// I, J (their own term) and G (I's term). The reshare adds arithmetically in
// both cases (FPC.inl:1231-1249).
template <typename T, bool BOOL> __device__ __forceinline__ void mul12(T (&s)[4][3], const T (&r)[4][3]) {
    T z[4], zp[4];
#pragma unroll
    for (int p = 0; p < 4; p++) {
        if (BOOL) {
            z[p] = (T)((s[p][0] & r[p][1]) ^ (s[p][1] & r[p][0]));
            zp[p] = (T)((s[p][0] & r[p][2]) ^ (s[p][2] & r[p][0]));
        } else {
            z[p] = (T)(s[p][0] * r[p][1] + s[p][1] * r[p][0]);
            zp[p] = (T)(s[p][0] * r[p][2] + s[p][2] * r[p][0]);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) s[p][k] = BOOL ? (T)(s[p][k] & r[p][k]) : (T)(s[p][k] * r[p][k]);
    }
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const bool opp = pJ(q) - pI(q) == 2;
#pragma unroll
        for (int p = 0; p < 4; p++) {
            if (p == pH(q)) continue;
            const int src = p == pG(q) ? pI(q) : p;
            s[p][share_of(p, pH(q))] = (T)(s[p][share_of(p, pH(q))] + (opp ? zp[src] : z[src]));
        }
    }
}

template <typename T> __device__ __forceinline__ int dbit(T a_minus_one) {
    constexpr int W = sizeof(T) * 8;
    const T a = (T)(a_minus_one + 1);
    const int carry = (a & (((T)1 << (W - 1)) - 1)) != 0;
    const int msb = (int)(a >> (W - 1));
    return 1 - (carry ^ 1 ^ msb);
}

// dReLU of one element: party p >= 1 holds its bit in x0
template <typename T, typename U> __device__ __forceinline__ void drelu12(const T (&x)[4][3], U (&b)[4][3]) {
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const U bit = p ? (U)dbit<T>(reveal_at(x, p)) : (U)0;
#pragma unroll
        for (int k = 0; k < 3; k++) b[p][k] = k == x0_share(p) ? bit : (U)0;
    }
}

// selectShare of one element: z = (y - x) * d + x with d = [e_p == 1] in x0,
// e_p party p's reveal of b (convex_comb with c = 0, FPC.inl:31-66)
template <typename T, typename U>
__device__ __forceinline__ void select12(const T (&x)[4][3], const T (&y)[4][3], const U (&b)[4][3], T (&z)[4][3]) {
    T d[4][3];
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const T e1 = p && (U)reveal_at(b, p) == (U)1 ? (T)1 : (T)0;
#pragma unroll
        for (int k = 0; k < 3; k++) d[p][k] = k == x0_share(p) ? e1 : (T)0;
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) z[p][k] = (T)(y[p][k] - x[p][k]);
    mul12<T, false>(z, d);
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) z[p][k] = (T)(z[p][k] + x[p][k]);
}

// ------------------------------------------------------------------ kernels

#define FPC_LOOP(i, n) \
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

template <typename T> __global__ void reconstruct_kernel(const CF12<T> a, T *o0, T *o1, T *o2, T *o3, size_t n) {
    FPC_LOOP(i, n) {
        T v[4][3];
        load12(a, i, v);
        o0[i] = reveal_at(v, 0);
        o1[i] = reveal_at(v, 1);
        o2[i] = reveal_at(v, 2);
        o3[i] = reveal_at(v, 3);
    }
}

// dividePublic (FPC.inl:576-608): a -= r' (x0), reveal, divide, a = r + q (x0)
template <typename T> __global__ void divide_kernel(const CF12<T> a, const F12<T> o, size_t n, T d, const T *dvec, int dshift) {
    FPC_LOOP(i, n) {
        const T dd = dvec ? dvec[i] : d;
        T v[4][3];
        load12(a, i, v);
#pragma unroll
        for (int p = 1; p < 4; p++) v[p][x0_share(p)] = (T)(v[p][x0_share(p)] - dd);
        T r[4][3];
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const T q = p ? (T)(1 + div_public<T>(reveal_at(v, p), dd, dvec ? -1 : dshift)) : (T)0;
#pragma unroll
            for (int k = 0; k < 3; k++) r[p][k] = k == x0_share(p) ? q : (T)0;
        }
        store12(o, i, r);
    }
}

template <typename T, bool BOOL> __global__ void mul_kernel(const F12<T> a, const CF12<T> b, size_t n) {
    FPC_LOOP(i, n) {
        T s[4][3], r[4][3];
        load12(a, i, s);
        load12(b, i, r);
        mul12<T, BOOL>(s, r);
        store12(a, i, s);
    }
}

template <typename T, typename U> __global__ void drelu_kernel(const CF12<T> x, const F12<U> o, size_t n) {
    FPC_LOOP(i, n) {
        T v[4][3];
        U b[4][3];
        load12(x, i, v);
        drelu12<T, U>(v, b);
        store12(o, i, b);
    }
}

template <typename T, typename U>
__global__ void select_kernel(const CF12<T> x, const CF12<T> y, const CF12<U> b, const F12<T> z, size_t n) {
    FPC_LOOP(i, n) {
        T xv[4][3], yv[4][3], zv[4][3];
        U bv[4][3];
        load12(x, i, xv);
        load12(y, i, yv);
        load12(b, i, bv);
        select12<T, U>(xv, yv, bv, zv);
        store12(z, i, zv);
    }
}

// ReLU (FPC.inl:992-1003): dReLU, then selectShare(zeros, input, dresult)
template <typename T, typename U> __global__ void relu_kernel(const CF12<T> x, const F12<T> y, const F12<U> d, size_t n) {
    FPC_LOOP(i, n) {
        T xv[4][3], zero[4][3], out[4][3];
        U bv[4][3];
        load12(x, i, xv);
        drelu12<T, U>(xv, bv);
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int k = 0; k < 3; k++) zero[p][k] = 0;
        select12<T, U>(zero, xv, bv, out);
        store12(y, i, out);
        store12(d, i, bv);
    }
}

// One maxpool level at slot stride s (FPC.inl:1005-1177): for pair t the even
// slot e = t s and the odd slot e + s/2 give b = dReLU(even - odd) and
// even <- selectShare(odd, even, b). b is kept for the derivative step; the
// last level writes the row maxima to out instead of the work array.
template <typename T, typename U>
__global__ void maxpool_level_kernel(const CF12<T> src, const F12<T> work, const F12<U> bl, const F12<T> out,
                                     size_t pairs, size_t s, int last) {
    FPC_LOOP(t, pairs) {
        const size_t e = t * s, o = e + s / 2;
        T ev[4][3], ov[4][3], diff[4][3], r[4][3];
        U b[4][3];
        load12(src, e, ev);
        load12(src, o, ov);
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int k = 0; k < 3; k++) diff[p][k] = (T)(ev[p][k] - ov[p][k]);
        drelu12<T, U>(diff, b);
        select12<T, U>(ov, ev, b, r);
        if (last) store12(out, t, r);
        else store12(work, e, r);
        store12(bl, t, b);
    }
}

// dresult &= expandCompare(b, 1 - b) (bitwise.cuh:66-92): element j of the
// n inputs takes b of pair j / s where j mod s < s/2, else 1 - b (FPC fill(1)
// minus b: x0 gets 1 - b, the other shares -b). first: dresult = fill(1).
template <typename U> __global__ void maxpool_and_kernel(const F12<U> dres, const CF12<U> bl, size_t n, size_t s, int first) {
    FPC_LOOP(j, n) {
        const size_t t = j / s;
        const bool lo = (j - t * s) < s / 2;
        U b[4][3], cur[4][3];
        load12(bl, t, b);
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const U one = k == x0_share(p) ? (U)1 : (U)0;
                if (!lo) b[p][k] = (U)(one - b[p][k]);
                cur[p][k] = first ? one : dres.p[p * 3 + k][j];
            }
        mul12<U, true>(cur, b);
        store12(dres, j, cur);
    }
}

// party A's output of a matmul or convolution: zeros (plus the bias shares)
template <typename T>
__global__ void party_a_kernel(T *o0, T *o1, T *o2, const T *b0, const T *b1, const T *b2, size_t n, int ncols, int rows,
                               int colmajor) {
    FPC_LOOP(i, n) {
        const size_t col = colmajor ? i / (size_t)rows : i % (size_t)ncols;
        o0[i] = b0 ? b0[col] : (T)0;
        o1[i] = b1 ? b1[col] : (T)0;
        o2[i] = b2 ? b2[col] : (T)0;
    }
}

// --------------------------------------------------------------------- host

template <typename T> static bool ok12(const T *const *a) {
    if (!a) return false;
    for (int i = 0; i < 12; i++)
        if (!a[i]) return false;
    return true;
}
template <typename T> static CF12<T> cf(const T *const *a) {
    CF12<T> r;
    for (int i = 0; i < 12; i++) r.p[i] = a[i];
    return r;
}
template <typename T> static F12<T> mf(T *const *a) {
    F12<T> r;
    for (int i = 0; i < 12; i++) r.p[i] = a[i];
    return r;
}

// coef[u][i][j]: the multiplicity of the local product a_{u,i} b_{u,j} in a
// party's reveal after the six reshares of an FPC product (FPC.inl:636-670)
struct RevealTerms {
    int c[4][3][3];
};
static void add_terms(RevealTerms &d, const RevealTerms &s) {
    for (int u = 0; u < 4; u++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) d.c[u][i][j] += s.c[u][i][j];
}
static RevealTerms fpc_reveal_terms(int party) {
    RevealTerms C[4][3], z[4], zp[4];
    std::memset(C, 0, sizeof(C));
    std::memset(z, 0, sizeof(z));
    std::memset(zp, 0, sizeof(zp));
    for (int p = 0; p < 4; p++) {
        for (int k = 0; k < 3; k++) C[p][k].c[p][k][k] = 1;  // c_k = gemm(a_k, b_k)
        z[p].c[p][0][1] = z[p].c[p][1][0] = 1;                // z  = a0 b1 + a1 b0
        zp[p].c[p][0][2] = zp[p].c[p][2][0] = 1;              // z' = a0 b2 + a2 b0
    }
    for (int q = 0; q < 6; q++) {
        const bool opp = pJ(q) - pI(q) == 2;
        for (int p = 0; p < 4; p++) {
            if (p == pH(q)) continue;
            const int src = p == pG(q) ? pI(q) : p;
            add_terms(C[p][share_of(p, pH(q))], opp ? zp[src] : z[src]);
        }
    }
    RevealTerms r;
    std::memset(&r, 0, sizeof(r));
    for (int k = 0; k < 3; k++) add_terms(r, C[party][k]);
    add_terms(r, C[(party + 3) & 3][0]);
    return r;
}

// Pack a party's reveal into GEMM segments: per A operand a_{u,i}, its B
// operands with multiplicity, two per segment (b0 + b1; the same pointer twice
// for a doubled term).
template <typename T> static int reveal_segments(int party, const T *const a[12], const T *const b[12], SegList<T> &s) {
    const RevealTerms t = fpc_reveal_terms(party);
    s.nseg = 0;
    for (int u = 0; u < 4; u++)
        for (int i = 0; i < 3; i++) {
            const T *bs[16];
            int nb = 0;
            for (int j = 0; j < 3; j++)
                for (int m = 0; m < t.c[u][i][j] && nb < 16; m++) bs[nb++] = b[u * 3 + j];
            for (int q = 0; q < nb; q += 2) {
                if (s.nseg >= 12) return -1;
                s.a[s.nseg] = a[u * 3 + i];
                s.b0[s.nseg] = bs[q];
                s.b1[s.nseg] = q + 1 < nb ? bs[q + 1] : nullptr;
                s.nseg++;
            }
        }
    return 0;
}

template <typename T>
int matmul(Ctx *c, const T *const a[12], const T *const b[12], T *const out[12], const T *const bias[12], int M, int N,
           int K, int tA, int tB, int tC, int trunc) {
    if (!ok12(a) || !ok12(b) || !ok12(out) || (bias && !ok12(bias)))
        return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    if (trunc < 0 || trunc > (int)sizeof(T) * 8 - 2) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    const size_t mn = (size_t)M * N;
    for (int p = 1; p < 4; p++) {
        SegList<T> s;
        if (reveal_segments<T>(p, a, b, s)) return set_error(c, PG_ERR_UNSUPPORTED, "fpc: too many GEMM segments");
        int st = fpc_party_gemm<T>(c, s, M, N, K, tA, tB, tC, out + p * 3, bias ? bias + p * 3 : nullptr, x0_share(p),
                                   trunc);
        if (st) return st;
    }
    party_a_kernel<T><<<grid_for(c, mn), 256, 0, c->stream>>>(out[0], out[1], out[2], bias ? bias[0] : nullptr,
                                                              bias ? bias[1] : nullptr, bias ? bias[2] : nullptr, mn,
                                                              N, M, tC ? 0 : 1);
    c->launches++;
    int st = launch_status(c, "fpc party_a_kernel");
    if (st) return st;
    reshare_comm(c, mn, sizeof(T));
    reveal_comm(c, mn, sizeof(T));  // dividePublic
    return PG_OK;
}

int conv_u64(Ctx *c, const uint64_t *const A[12], const uint64_t *const B[12], uint64_t *const C[12], int op, int batch,
             int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    if (!ok12(A) || !ok12(B) || !ok12(C)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Din <= 0 || Dout <= 0 || stride <= 0 || pad < 0 ||
        H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "convolution: bad geometry");
    if (op < PG_CONV_FPROP || op > PG_CONV_WGRAD) return set_error(c, PG_ERR_INVALID_ARG, "bad conv op %d", op);
    const int P = (H + 2 * pad - f) / stride + 1, Q = (W + 2 * pad - f) / stride + 1;
    const size_t nc = op == PG_CONV_FPROP ? (size_t)batch * P * Q * Dout
                    : op == PG_CONV_DGRAD ? (size_t)batch * H * W * Din
                                          : (size_t)Dout * f * f * Din;
    for (int p = 1; p < 4; p++) {
        SegList<uint64_t> s;
        if (reveal_segments<uint64_t>(p, A, B, s)) return set_error(c, PG_ERR_UNSUPPORTED, "fpc: too many GEMM segments");
        int st = fpc_party_conv_u64(c, s, op, batch, H, W, f, Din, Dout, stride, pad, C + p * 3, x0_share(p), trunc);
        if (st) return st;
    }
    party_a_kernel<uint64_t><<<grid_for(c, nc), 256, 0, c->stream>>>(C[0], C[1], C[2], nullptr, nullptr, nullptr, nc, 1,
                                                                     1, 0);
    c->launches++;
    int st = launch_status(c, "fpc party_a_kernel");
    if (st) return st;
    reshare_comm(c, nc, 8);
    reveal_comm(c, nc, 8);
    return PG_OK;
}

template <typename T> int divide_public(Ctx *c, T *const a[12], size_t n, T d, const T *dvec) {
    if (!dvec && d == 0) return set_error(c, PG_ERR_INVALID_ARG, "division by zero");
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        reveal_comm(c, 0, sizeof(T));
        return PG_OK;
    }
    if (!ok12(a)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    divide_kernel<T><<<grid_for(c, n), 256, 0, c->stream>>>(cf<T>(a), mf<T>(a), n, d, dvec, pow2_shift<T>(d));
    c->launches++;
    int st = launch_status(c, "fpc divide_kernel");
    if (st) return st;
    reveal_comm(c, n, sizeof(T));
    return PG_OK;
}

template <typename T> int reconstruct(Ctx *c, const T *const a[12], size_t n, T *const out[4]) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        reveal_comm(c, 0, sizeof(T));
        return PG_OK;
    }
    if (!ok12(a) || !out || !out[0] || !out[1] || !out[2] || !out[3]) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    reconstruct_kernel<T><<<grid_for(c, n), 256, 0, c->stream>>>(cf<T>(a), out[0], out[1], out[2], out[3], n);
    c->launches++;
    int st = launch_status(c, "fpc reconstruct_kernel");
    if (st) return st;
    reveal_comm(c, n, sizeof(T));
    return PG_OK;
}

template <typename T, bool BOOL> int mul(Ctx *c, T *const a[12], const T *const b[12], size_t n) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        reshare_comm(c, 0, sizeof(T));
        return PG_OK;
    }
    if (!ok12(a) || !ok12(b)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    mul_kernel<T, BOOL><<<grid_for(c, n), 256, 0, c->stream>>>(mf<T>(a), cf<T>(b), n);
    c->launches++;
    int st = launch_status(c, "fpc mul_kernel");
    if (st) return st;
    reshare_comm(c, n, sizeof(T));
    return PG_OK;
}

template <typename T, typename U> int drelu(Ctx *c, const T *const in[12], size_t n, U *const out[12]) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        drelu_comm<T, U>(c, 0);
        return PG_OK;
    }
    if (!ok12(in) || !ok12(out)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    drelu_kernel<T, U><<<grid_for(c, n), 256, 0, c->stream>>>(cf<T>(in), mf<U>(out), n);
    c->launches++;
    int st = launch_status(c, "fpc drelu_kernel");
    if (st) return st;
    drelu_comm<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int relu(Ctx *c, const T *const in[12], size_t n, T *const out[12], U *const dout[12]) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        drelu_comm<T, U>(c, 0);
        select_comm<T, U>(c, 0);
        return PG_OK;
    }
    if (!ok12(in) || !ok12(out) || !ok12(dout)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    relu_kernel<T, U><<<grid_for(c, n), 256, 0, c->stream>>>(cf<T>(in), mf<T>(out), mf<U>(dout), n);
    c->launches++;
    int st = launch_status(c, "fpc relu_kernel");
    if (st) return st;
    drelu_comm<T, U>(c, n);
    select_comm<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int select_share(Ctx *c, const T *const x[12], const T *const y[12], const U *const b[12], T *const z[12], size_t n) {
    if (n == 0) {  // no values: empty messages, the protocol's rounds still counted
        select_comm<T, U>(c, 0);
        return PG_OK;
    }
    if (!ok12(x) || !ok12(y) || !ok12(b) || !ok12(z)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    select_kernel<T, U><<<grid_for(c, n), 256, 0, c->stream>>>(cf<T>(x), cf<T>(y), cf<U>(b), mf<T>(z), n);
    c->launches++;
    int st = launch_status(c, "fpc select_kernel");
    if (st) return st;
    select_comm<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int maxpool(Ctx *c, const T *const in[12], size_t n, int k, T *const out[12], U *const dout[12]) {
    if (n && (!ok12(in) || !ok12(out) || !ok12(dout))) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (k < 2 || (k & (k - 1))) return set_error(c, PG_ERR_UNSUPPORTED, "maxpool rows of %d (a power of two >= 2)", k);
    if (n % (size_t)k) return set_error(c, PG_ERR_SIZE, "maxpool input %zu is not a multiple of %d", n, k);
    if (n == 0) return PG_OK;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t work_b = al(n * sizeof(T)), bl_b = al((n / 2) * sizeof(U));
    uint8_t *s = (uint8_t *)scratch(c, 12 * (work_b + bl_b));
    if (!s) return PG_ERR_NO_MEMORY;
    F12<T> work;
    F12<U> bl;
    for (int i = 0; i < 12; i++) {
        work.p[i] = (T *)(s + i * work_b);
        bl.p[i] = (U *)(s + 12 * work_b + i * bl_b);
    }
    CF12<T> src = cf<T>(in);
    for (size_t st_ = 2; st_ <= (size_t)k; st_ *= 2) {
        const size_t pairs = n / st_;
        const int last = st_ == (size_t)k;
        maxpool_level_kernel<T, U><<<grid_for(c, pairs), 128, 0, c->stream>>>(src, work, bl, mf<T>(out), pairs, st_, last);
        maxpool_and_kernel<U><<<grid_for(c, n), 128, 0, c->stream>>>(mf<U>(dout), cf<U>(bl.p), n, st_, st_ == 2);
        c->launches += 2;
        int st = launch_status(c, "fpc maxpool kernels");
        if (st) return st;
        for (int i = 0; i < 12; i++) src.p[i] = work.p[i];
        drelu_comm<T, U>(c, pairs);
        select_comm<T, U>(c, pairs);
        reshare_comm(c, n, sizeof(U));  // dresult &= expandedB
    }
    return PG_OK;
}

}  // namespace fpc
}  // namespace pg

using namespace pg;

#define FPC_CTX(c) \
    if (!(c)) return PG_ERR_INVALID_ARG

extern "C" {

int pg_fpc_matmul_u64(pg_ctx *c, const uint64_t *const a[12], const uint64_t *const b[12], uint64_t *const out[12],
                      int M, int N, int K, int tA, int tB, int tC, int trunc) {
    FPC_CTX(c);
    return fpc::matmul<uint64_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}
int pg_fpc_matmul_u32(pg_ctx *c, const uint32_t *const a[12], const uint32_t *const b[12], uint32_t *const out[12],
                      int M, int N, int K, int tA, int tB, int tC, int trunc) {
    FPC_CTX(c);
    return fpc::matmul<uint32_t>(c, a, b, out, nullptr, M, N, K, tA, tB, tC, trunc);
}
int pg_fpc_fc_forward_u64(pg_ctx *c, const uint64_t *const x[12], const uint64_t *const w[12],
                          const uint64_t *const bias[12], uint64_t *const out[12], int batch, int din, int dout, int fp) {
    FPC_CTX(c);
    return fpc::matmul<uint64_t>(c, x, w, out, bias, batch, dout, din, 1, 1, 1, fp);
}
int pg_fpc_fc_forward_u32(pg_ctx *c, const uint32_t *const x[12], const uint32_t *const w[12],
                          const uint32_t *const bias[12], uint32_t *const out[12], int batch, int din, int dout, int fp) {
    FPC_CTX(c);
    return fpc::matmul<uint32_t>(c, x, w, out, bias, batch, dout, din, 1, 1, 1, fp);
}
int pg_fpc_conv_u64(pg_ctx *c, const uint64_t *const A[12], const uint64_t *const B[12], uint64_t *const C[12], int op,
                    int batch, int H, int W, int f, int Din, int Dout, int stride, int pad, int trunc) {
    FPC_CTX(c);
    return fpc::conv_u64(c, A, B, C, op, batch, H, W, f, Din, Dout, stride, pad, trunc);
}
int pg_fpc_divide_public_u64(pg_ctx *c, uint64_t *const a[12], size_t n, uint64_t d) {
    FPC_CTX(c);
    return fpc::divide_public<uint64_t>(c, a, n, d, nullptr);
}
int pg_fpc_divide_public_vec_u64(pg_ctx *c, uint64_t *const a[12], size_t n, const uint64_t *d) {
    FPC_CTX(c);
    if (!d && n) return set_error(c, PG_ERR_INVALID_ARG, "null denominators");
    return fpc::divide_public<uint64_t>(c, a, n, 0, d);
}
int pg_fpc_divide_public_u32(pg_ctx *c, uint32_t *const a[12], size_t n, uint32_t d) {
    FPC_CTX(c);
    return fpc::divide_public<uint32_t>(c, a, n, d, nullptr);
}
int pg_fpc_reconstruct_u64(pg_ctx *c, const uint64_t *const a[12], size_t n, uint64_t *const out[4]) {
    FPC_CTX(c);
    return fpc::reconstruct<uint64_t>(c, a, n, out);
}
int pg_fpc_reconstruct_u32(pg_ctx *c, const uint32_t *const a[12], size_t n, uint32_t *const out[4]) {
    FPC_CTX(c);
    return fpc::reconstruct<uint32_t>(c, a, n, out);
}
int pg_fpc_reconstruct_u8(pg_ctx *c, const uint8_t *const a[12], size_t n, uint8_t *const out[4]) {
    FPC_CTX(c);
    return fpc::reconstruct<uint8_t>(c, a, n, out);
}
int pg_fpc_mul_u64(pg_ctx *c, uint64_t *const a[12], const uint64_t *const b[12], size_t n) {
    FPC_CTX(c);
    return fpc::mul<uint64_t, false>(c, a, b, n);
}
int pg_fpc_and_u8(pg_ctx *c, uint8_t *const a[12], const uint8_t *const b[12], size_t n) {
    FPC_CTX(c);
    return fpc::mul<uint8_t, true>(c, a, b, n);
}
int pg_fpc_drelu_u64_u8(pg_ctx *c, const uint64_t *const in[12], size_t n, uint8_t *const out[12]) {
    FPC_CTX(c);
    return fpc::drelu<uint64_t, uint8_t>(c, in, n, out);
}
int pg_fpc_drelu_u32_u8(pg_ctx *c, const uint32_t *const in[12], size_t n, uint8_t *const out[12]) {
    FPC_CTX(c);
    return fpc::drelu<uint32_t, uint8_t>(c, in, n, out);
}
int pg_fpc_relu_u64_u8(pg_ctx *c, const uint64_t *const in[12], size_t n, uint64_t *const out[12],
                       uint8_t *const dout[12]) {
    FPC_CTX(c);
    return fpc::relu<uint64_t, uint8_t>(c, in, n, out, dout);
}
int pg_fpc_relu_u32_u8(pg_ctx *c, const uint32_t *const in[12], size_t n, uint32_t *const out[12],
                       uint8_t *const dout[12]) {
    FPC_CTX(c);
    return fpc::relu<uint32_t, uint8_t>(c, in, n, out, dout);
}
int pg_fpc_select_share_u64_u8(pg_ctx *c, const uint64_t *const x[12], const uint64_t *const y[12],
                               const uint8_t *const b[12], uint64_t *const z[12], size_t n) {
    FPC_CTX(c);
    return fpc::select_share<uint64_t, uint8_t>(c, x, y, b, z, n);
}
int pg_fpc_maxpool_u64_u8(pg_ctx *c, const uint64_t *const in[12], size_t n, int k, uint64_t *const out[12],
                          uint8_t *const dout[12]) {
    FPC_CTX(c);
    return fpc::maxpool<uint64_t, uint8_t>(c, in, n, k, out, dout);
}

}  // extern "C"
