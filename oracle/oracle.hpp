// oracle.hpp — CPU restatement of Piranha's party-local secret-share arithmetic.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: the pytest suite, the
// smoke check and the CPU-baseline leg of bench.py call it to produce the
// expected shares. Nothing in the piranha_gb300 product links or calls it.
//
// What it restates (paths relative to the Piranha source tree):
//   * src/mpc/RSS.inl      — the 3-party replicated-secret-sharing protocol,
//                            step by step, for every simulated party
//   * src/gpu/functors.cuh — ring operators, including division through double
//   * src/gpu/gemm.cuh     — the 8-layout ring GEMM (column-major default)
//   * src/gpu/conv.cuh     — CUTLASS fprop/dgrad/wgrad problem semantics
//   * src/gpu/bitwise.cuh, convolution.cuh, matrix.cuh — bit/maxpool/bias glue
//   * src/mpc/Precompute.h — the constant "randomness" (r = 1, r' = d)
//   * src/util/util.cuh    — fixed-point encode/decode
//
// Simulation model. Piranha runs one process per party; every DeviceData op
// runs at each party on that party's own view. Here the three parties live in
// one process: an RSS tensor of n elements is held as views[party][share][n]
// (party A=0, B=1, C=2; share 0 = "shareA", share 1 = "shareB"). Per-party
// public data (the result of a reconstruct, bit expansions) is pub[party][n].
// A message "sent" by one party is read directly from the sender's view; the
// bytes and rounds a socket would carry are added to a Comm counter with the
// accounting of DeviceData::transmit/receive (DeviceData.h:87-118) and
// Profiler::add_comm_round.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace oracle {

enum { PA = 0, PB = 1, PC = 2 };
static inline int next_party(int p) { return (p + 1) % 3; }  // RSS.inl:348-357
static inline int prev_party(int p) { return (p + 2) % 3; }  // RSS.inl:360-369

struct Comm {
    uint64_t tx[4] = {0, 0, 0, 0};
    uint64_t rx[4] = {0, 0, 0, 0};
    uint64_t rounds = 0;
    void msg(int nparties, uint64_t bytes_tx, uint64_t bytes_rx) {
        for (int p = 0; p < nparties; p++) { tx[p] += bytes_tx; rx[p] += bytes_rx; }
    }
};

// ---------------------------------------------------------------- ring ops --

template <typename T> using S_t = typename std::make_signed<T>::type;

// Saturating double -> signed conversion with PTX cvt.rzi semantics
// (truncate toward zero, clamp to range, NaN -> 0). The reference runs its
// division functor on the device, so these are the semantics it sees.
template <typename S> static inline S cvt_rzi_sat(double q) {
    if (std::isnan(q)) return 0;
    const double hi = std::ldexp(1.0, int(sizeof(S) * 8 - 1));
    if (q >= hi) return std::numeric_limits<S>::max();
    if (q <= -hi) return std::numeric_limits<S>::min();
    return (S)q;  // in range: C++ truncates toward zero
}

// functors.cuh:33-45 (scalar) and :94-105 (vector): (T)(S)((double)(S)x / (double)(S)d)
template <typename T> static inline T div_public(T x, T d) {
    using S = S_t<T>;
    double q = (double)(S)x / (double)(S)d;
    return (T)cvt_rzi_sat<S>(q);
}

// util.cuh:28-33 / RSS.inl:126: (T)(f * (1 << FP)). A negative double must go
// through a signed integer first: that is what x86-64 hosts did for the
// reference; aarch64's unsigned conversion would saturate to 0 instead.
template <typename T> static inline T encode_fixed(double f, int fp) {
    double v = f * (double)(1 << fp);
    return (T)(int64_t)v;
}
// util.cuh:46-53
template <typename T> static inline double decode_fixed(T v, int fp) {
    return (double)(S_t<T>)v / (double)(1 << fp);
}

// ------------------------------------------------------------ share views --

// views[p][s] is an n-element array; a strided view (StridedRange.cuh:11-52)
// is expressed by (offset, stride, size) over the parent array.
template <typename T> struct RSSV {
    size_t n = 0;
    std::vector<T> v[3][2];
    RSSV() {}
    explicit RSSV(size_t n_) { resize(n_); }
    void resize(size_t n_) {
        n = n_;
        for (int p = 0; p < 3; p++)
            for (int s = 0; s < 2; s++) v[p][s].assign(n, (T)0);
    }
    void zero() { for (int p = 0; p < 3; p++) for (int s = 0; s < 2; s++) std::fill(v[p][s].begin(), v[p][s].end(), (T)0); }
};

template <typename T> using Pub = std::vector<T>[3];

struct Strided {
    size_t offset, stride, size;
};
static inline Strided strided(size_t parent_n, size_t offset, size_t stride) {
    // StridedRange.cuh:44-46: size = ((last - first) + (stride - 1)) / stride
    size_t span = parent_n > offset ? parent_n - offset : 0;
    return Strided{offset, stride, (span + stride - 1) / stride};
}
static inline Strided whole(size_t n) { return Strided{0, 1, n}; }

// RSS.inl:117-120: fill puts val into party A's shareA and party C's shareB.
template <typename T> void rss_fill(RSSV<T>& a, T val) {
    for (int p = 0; p < 3; p++) {
        std::fill(a.v[p][0].begin(), a.v[p][0].end(), p == PA ? val : (T)0);
        std::fill(a.v[p][1].begin(), a.v[p][1].end(), p == PC ? val : (T)0);
    }
}

// RSS.inl:123-142. With ref_compat the missing `break` after case PARTY_B is
// reproduced: party B also receives the public values in its shareB.
template <typename T> void rss_set_public(RSSV<T>& a, const double* vals, int fp, bool ref_compat) {
    for (size_t i = 0; i < a.n; i++) {
        T x = encode_fixed<T>(vals[i], fp);
        a.v[PA][0][i] = x; a.v[PA][1][i] = 0;
        a.v[PB][0][i] = 0; a.v[PB][1][i] = ref_compat ? x : (T)0;
        a.v[PC][0][i] = 0; a.v[PC][1][i] = x;
    }
}

// RSS.inl:389-414: the initializer-list constructor (no fall-through).
template <typename T> void rss_from_list(RSSV<T>& a, const double* vals, int fp, bool to_fixed) {
    for (size_t i = 0; i < a.n; i++) {
        T x = to_fixed ? encode_fixed<T>(vals[i], fp) : (T)(int64_t)vals[i];
        a.v[PA][0][i] = x; a.v[PA][1][i] = 0;
        a.v[PB][0][i] = 0; a.v[PB][1][i] = 0;
        a.v[PC][0][i] = 0; a.v[PC][1][i] = x;
    }
}

// reshare (RSS.inl:1053-1074): out = (c_p, c_next). Applied to strided views.
template <typename T> void reshare_into(const std::vector<T> (&c)[3], RSSV<T>& out, Strided w, Comm& comm) {
    for (int p = 0; p < 3; p++)
        for (size_t i = 0; i < w.size; i++) {
            size_t j = w.offset + i * w.stride;
            out.v[p][0][j] = c[p][i];
            out.v[p][1][j] = c[next_party(p)][i];
        }
    comm.msg(3, w.size * sizeof(T), w.size * sizeof(T));
    comm.rounds++;
}

// RSS &= RSS on (strided) views (RSS.inl:331-345):
//   z = (a0 & (b0 ^ b1)) ^ (a1 & b0), then reshare.
template <typename T> void rss_and_assign(RSSV<T>& a, Strided wa, const RSSV<T>& b, Strided wb, Comm& comm) {
    std::vector<T> c[3];
    for (int p = 0; p < 3; p++) {
        c[p].resize(wa.size);
        for (size_t i = 0; i < wa.size; i++) {
            size_t ia = wa.offset + i * wa.stride, ib = wb.offset + i * wb.stride;
            T b0 = b.v[p][0][ib], b1 = b.v[p][1][ib];
            c[p][i] = (T)((a.v[p][0][ia] & (T)(b0 ^ b1)) ^ (a.v[p][1][ia] & b0));
        }
    }
    reshare_into(c, a, wa, comm);
}

// RSS *= RSS (RSS.inl:284-320): z = a0*(b0+b1) + a1*b0, then reshare.
template <typename T> void rss_mul_assign(RSSV<T>& a, const RSSV<T>& b, Comm& comm) {
    std::vector<T> c[3];
    for (int p = 0; p < 3; p++) {
        c[p].resize(a.n);
        for (size_t i = 0; i < a.n; i++) {
            T b0 = b.v[p][0][i], b1 = b.v[p][1][i];
            c[p][i] = (T)(a.v[p][0][i] * (T)(b0 + b1) + a.v[p][1][i] * b0);
        }
    }
    reshare_into(c, a, whole(a.n), comm);
}

// RSS ^= RSS (RSS.inl:324-328), on views.
template <typename T> void rss_xor_assign(RSSV<T>& a, Strided wa, const RSSV<T>& b, Strided wb) {
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            for (size_t i = 0; i < wa.size; i++)
                a.v[p][s][wa.offset + i * wa.stride] ^= b.v[p][s][wb.offset + i * wb.stride];
}

// reconstruct (RSS.inl:458-479): out_p = a_p0 + a_p1 + (prev party's a0).
template <typename T> void rss_reconstruct(const RSSV<T>& a, Strided w, std::vector<T> (&out)[3], Comm& comm) {
    for (int p = 0; p < 3; p++) {
        out[p].resize(w.size);
        int q = prev_party(p);
        for (size_t i = 0; i < w.size; i++) {
            size_t j = w.offset + i * w.stride;
            out[p][i] = (T)(a.v[p][0][j] + a.v[p][1][j] + a.v[q][0][j]);
        }
    }
    comm.msg(3, w.size * sizeof(T), w.size * sizeof(T));
    comm.rounds++;
}

// dividePublic(RSS, T) (RSS.inl:423-436) and the vector form (:439-455), with
// Precompute::getDividedShares r = fill(1), r' = fill(d) (Precompute.h:107-134).
template <typename T> void rss_divide_public(RSSV<T>& a, const T* d, bool vector_d, Comm& comm) {
    // a -= r'  (RSS -= RSS): r' holds d in A.shareA and C.shareB
    for (size_t i = 0; i < a.n; i++) {
        T di = vector_d ? d[i] : d[0];
        a.v[PA][0][i] -= di;
        a.v[PC][1][i] -= di;
    }
    std::vector<T> rec[3];
    rss_reconstruct(a, whole(a.n), rec, comm);
    for (int p = 0; p < 3; p++)
        for (size_t i = 0; i < a.n; i++) rec[p][i] = div_public<T>(rec[p][i], vector_d ? d[i] : d[0]);
    // a.zero(); a += r; a += reconstructed
    for (size_t i = 0; i < a.n; i++) {
        a.v[PA][0][i] = (T)(1 + rec[PA][i]); a.v[PA][1][i] = 0;
        a.v[PB][0][i] = 0;                    a.v[PB][1][i] = 0;
        a.v[PC][0][i] = 0;                    a.v[PC][1][i] = (T)(1 + rec[PC][i]);
    }
}

// dividePublic3out3 (RSS.inl:1077-1094) + reconstruct3out3 (:1020-1050).
// z[p] is party p's 3-out-of-3 share; output is an RSS tensor.
template <typename T> void rss_divide_public_3of3(std::vector<T> (&z)[3], T d, RSSV<T>& out, Comm& comm) {
    size_t n = z[0].size();
    for (size_t i = 0; i < n; i++) z[PA][i] -= d;  // a -= rPrime.shareA (only A holds d)
    out.resize(n);
    for (size_t i = 0; i < n; i++) {
        T rec[3];
        for (int p = 0; p < 3; p++) rec[p] = (T)(z[p][i] + z[prev_party(p)][i] + z[next_party(p)][i]);
        out.v[PA][0][i] = (T)(1 + div_public<T>(rec[PA], d));
        out.v[PC][1][i] = (T)(1 + div_public<T>(rec[PC], d));
    }
    comm.msg(3, 2 * n * sizeof(T), 2 * n * sizeof(T));
    comm.rounds++;
}

// ---------------------------------------------------------------- GEMM ----

// gpu::gemm (gemm.cuh:64-100): C(MxN) = A(MxK) * B(KxN) mod 2^w; each operand
// is row-major when its transpose flag is set, column-major otherwise.
template <typename T>
void gemm(int M, int N, int K, const T* A, bool tA, const T* B, bool tB, T* C, bool tC) {
    if (tB) {
        // B row-major: accumulate whole rows of C (unit-stride over B's rows);
        // the sums are the same mod 2^w in any order
        #pragma omp parallel
        {
            std::vector<T> acc((size_t)N);
            #pragma omp for schedule(static)
            for (int m = 0; m < M; m++) {
                std::fill(acc.begin(), acc.end(), (T)0);
                for (int k = 0; k < K; k++) {
                    const T a = tA ? A[(size_t)m * K + k] : A[m + (size_t)k * M];
                    const T* brow = B + (size_t)k * N;
                    for (int n = 0; n < N; n++) acc[n] = (T)(acc[n] + a * brow[n]);
                }
                for (int n = 0; n < N; n++) {
                    if (tC) C[(size_t)m * N + n] = acc[n]; else C[m + (size_t)n * M] = acc[n];
                }
            }
        }
        return;
    }
    #pragma omp parallel for schedule(static)
    for (int m = 0; m < M; m++) {
        for (int n = 0; n < N; n++) {
            T acc = 0;
            for (int k = 0; k < K; k++) {
                T a = tA ? A[(size_t)m * K + k] : A[m + (size_t)k * M];
                T b = tB ? B[(size_t)k * N + n] : B[k + (size_t)n * K];
                acc = (T)(acc + a * b);
            }
            if (tC) C[(size_t)m * N + n] = acc; else C[m + (size_t)n * M] = acc;
        }
    }
}

// localMatMul (RSS.inl:1097-1110): z_p = A_p0*B_p0 + A_p0*B_p1 + A_p1*B_p0.
// Computed in the fused form A_p0*(B_p0+B_p1) + A_p1*B_p0 (identical mod 2^w).
template <typename T>
void local_matmul(const RSSV<T>& a, const RSSV<T>& b, std::vector<T> (&z)[3], int M, int N, int K,
                  bool tA, bool tB, bool tC) {
    std::vector<T> bs((size_t)K * N), t1((size_t)M * N), t2((size_t)M * N);
    for (int p = 0; p < 3; p++) {
        for (size_t i = 0; i < bs.size(); i++) bs[i] = (T)(b.v[p][0][i] + b.v[p][1][i]);
        gemm<T>(M, N, K, a.v[p][0].data(), tA, bs.data(), tB, t1.data(), tC);
        gemm<T>(M, N, K, a.v[p][1].data(), tA, b.v[p][0].data(), tB, t2.data(), tC);
        z[p].resize((size_t)M * N);
        for (size_t i = 0; i < z[p].size(); i++) z[p][i] = (T)(t1[i] + t2[i]);
    }
}

// matmul (RSS.inl:482-540)
template <typename T>
void rss_matmul(const RSSV<T>& a, const RSSV<T>& b, RSSV<T>& c, int M, int N, int K, bool tA, bool tB,
                bool tC, int trunc, Comm& comm) {
    std::vector<T> z[3];
    local_matmul(a, b, z, M, N, K, tA, tB, tC);
    rss_divide_public_3of3(z, (T)((T)1 << trunc), c, comm);
}

// ---------------------------------------------------------------- conv ----

// CUTLASS Conv2d problem semantics as used by conv.cuh:84-91,359-490:
// NHWC activations, KRSC filters, cross-correlation, symmetric padding,
// P = (H + 2*pad - R)/stride + 1.
struct ConvShape {
    int N, H, W, C, K, R, S, pad, stride;
    int P() const { return (H + 2 * pad - R) / stride + 1; }
    int Q() const { return (W + 2 * pad - S) / stride + 1; }
};

// fprop: Y[n,p,q,k] = sum_{r,s,c} X[n, p*st-pad+r, q*st-pad+s, c] * F[k,r,s,c]
template <typename T> void conv_fprop(const ConvShape& sh, const T* X, const T* F, T* Y) {
    int P = sh.P(), Q = sh.Q();
    #pragma omp parallel for collapse(2) schedule(static)
    for (int n = 0; n < sh.N; n++)
        for (int p = 0; p < P; p++)
            for (int q = 0; q < Q; q++)
                for (int k = 0; k < sh.K; k++) {
                    T acc = 0;
                    for (int r = 0; r < sh.R; r++) {
                        int h = p * sh.stride - sh.pad + r;
                        if (h < 0 || h >= sh.H) continue;
                        for (int s = 0; s < sh.S; s++) {
                            int w = q * sh.stride - sh.pad + s;
                            if (w < 0 || w >= sh.W) continue;
                            const T* x = X + (((size_t)n * sh.H + h) * sh.W + w) * sh.C;
                            const T* f = F + (((size_t)k * sh.R + r) * sh.S + s) * sh.C;
                            for (int c = 0; c < sh.C; c++) acc = (T)(acc + x[c] * f[c]);
                        }
                    }
                    Y[(((size_t)n * P + p) * Q + q) * sh.K + k] = acc;
                }
}

// dgrad: dX[n,h,w,c] = sum_{k,r,s : h = p*st-pad+r, w = q*st-pad+s} dY[n,p,q,k] * F[k,r,s,c]
template <typename T> void conv_dgrad(const ConvShape& sh, const T* dY, const T* F, T* dX) {
    int P = sh.P(), Q = sh.Q();
    #pragma omp parallel for collapse(2) schedule(static)
    for (int n = 0; n < sh.N; n++)
        for (int h = 0; h < sh.H; h++)
            for (int w = 0; w < sh.W; w++)
                for (int c = 0; c < sh.C; c++) {
                    T acc = 0;
                    for (int r = 0; r < sh.R; r++) {
                        int ph = h + sh.pad - r;
                        if (ph < 0 || ph % sh.stride) continue;
                        int p = ph / sh.stride;
                        if (p >= P) continue;
                        for (int s = 0; s < sh.S; s++) {
                            int qw = w + sh.pad - s;
                            if (qw < 0 || qw % sh.stride) continue;
                            int q = qw / sh.stride;
                            if (q >= Q) continue;
                            const T* dy = dY + (((size_t)n * P + p) * Q + q) * sh.K;
                            for (int k = 0; k < sh.K; k++)
                                acc = (T)(acc + dy[k] * F[(((size_t)k * sh.R + r) * sh.S + s) * sh.C + c]);
                        }
                    }
                    dX[(((size_t)n * sh.H + h) * sh.W + w) * sh.C + c] = acc;
                }
}

// wgrad: dF[k,r,s,c] = sum_{n,p,q} dY[n,p,q,k] * X[n, p*st-pad+r, q*st-pad+s, c]
template <typename T> void conv_wgrad(const ConvShape& sh, const T* dY, const T* X, T* dF) {
    int P = sh.P(), Q = sh.Q();
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < sh.K; k++)
        for (int r = 0; r < sh.R; r++)
            for (int s = 0; s < sh.S; s++)
                for (int c = 0; c < sh.C; c++) {
                    T acc = 0;
                    for (int n = 0; n < sh.N; n++)
                        for (int p = 0; p < P; p++) {
                            int h = p * sh.stride - sh.pad + r;
                            if (h < 0 || h >= sh.H) continue;
                            for (int q = 0; q < Q; q++) {
                                int w = q * sh.stride - sh.pad + s;
                                if (w < 0 || w >= sh.W) continue;
                                acc = (T)(acc + dY[(((size_t)n * P + p) * Q + q) * sh.K + k] *
                                                    X[(((size_t)n * sh.H + h) * sh.W + w) * sh.C + c]);
                            }
                        }
                    dF[(((size_t)k * sh.R + r) * sh.S + s) * sh.C + c] = acc;
                }
}

enum ConvOp { CONV_FPROP = 0, CONV_DGRAD = 1, CONV_WGRAD = 2 };

// One party-local conv of the given kind between two single arrays.
template <typename T> void conv_any(int op, const ConvShape& sh, const T* a, const T* b, T* out) {
    if (op == CONV_FPROP) conv_fprop(sh, a, b, out);
    else if (op == CONV_DGRAD) conv_dgrad(sh, a, b, out);
    else conv_wgrad(sh, a, b, out);
}

// convolution (RSS.inl:706-803) with localFprop/Dgrad/Wgrad (:614-703):
// three convs summed per party, then dividePublic3out3.
// A and B follow the reference argument roles: fprop (im, filter), dgrad
// (delta, filter), wgrad (delta, forward input).
template <typename T>
void rss_convolution(const RSSV<T>& A, const RSSV<T>& B, RSSV<T>& C, int op, int batch, int H, int W,
                     int f, int Din, int Dout, int stride, int pad, int trunc, Comm& comm) {
    ConvShape sh{batch, H, W, Din, Dout, f, f, pad, stride};
    size_t out_n = op == CONV_FPROP ? (size_t)batch * sh.P() * sh.Q() * Dout
                 : op == CONV_DGRAD ? (size_t)batch * H * W * Din
                                    : (size_t)Dout * f * f * Din;
    std::vector<T> z[3], t(out_n);
    for (int p = 0; p < 3; p++) {
        z[p].assign(out_n, 0);
        const T* a0 = A.v[p][0].data(); const T* a1 = A.v[p][1].data();
        const T* b0 = B.v[p][0].data(); const T* b1 = B.v[p][1].data();
        const T* pairs[3][2] = {{a0, b0}, {a0, b1}, {a1, b0}};
        for (auto& pr : pairs) {
            // wgrad's first operand is the delta (NPQK) and second the input (NHWC)
            conv_any<T>(op, sh, pr[0], pr[1], t.data());
            for (size_t i = 0; i < out_n; i++) z[p][i] = (T)(z[p][i] + t[i]);
        }
    }
    rss_divide_public_3of3(z, (T)((T)1 << trunc), C, comm);
}

// --------------------------------------------------------- bit kernels ----

// bitexpand (bitwise.cuh:10-21): bits[v*W + b] = (a[v] >> b) & 1 (in-bounds part)
template <typename T, typename U> void bitexpand(const std::vector<T>& a, std::vector<U>& bits) {
    const int W = sizeof(T) * 8;
    bits.assign(a.size() * W, 0);
    for (size_t v = 0; v < a.size(); v++)
        for (int b = 0; b < W; b++) bits[v * W + b] = (U)((a[v] >> b) & 1);
}

// setCarryOutMSB (bitwise.cuh:41-64)
template <typename U>
void set_carry_out_msb(std::vector<U>& rbits, std::vector<U>& abits, std::vector<U>& msb, int W, bool xor_msb) {
    for (size_t i = 0; i < msb.size(); i++) {
        size_t bi = i * W + (W - 1);
        msb[i] = rbits[bi];
        if (xor_msb) msb[i] ^= abits[bi];
        abits[bi] = 1;
        rbits[bi] = 0;
    }
}

// carryOut (RSS.inl:1113-1209): log-depth generate/propagate tree over
// strided views of the bit arrays; 2 AND-reshares per level.
template <typename U> void carry_out(RSSV<U>& p, RSSV<U>& g, int k, RSSV<U>& out, Comm& comm) {
    size_t N = p.n;
    size_t stride = 2, offset = 1;
    Strided pEven = strided(N, 0, stride), pOdd = strided(N, offset, stride);
    Strided gEven = strided(N, 0, stride), gOdd = strided(N, offset, stride);
    while (k > 1) {
        rss_and_assign(g, gEven, p, pOdd, comm);
        rss_and_assign(p, pEven, p, pOdd, comm);
        rss_xor_assign(g, gOdd, g, gEven);
        gEven = strided(N, offset, stride * 2);
        offset += stride;
        gOdd = strided(N, offset, stride * 2);
        stride *= 2;
        pEven = strided(N, 0, stride);
        pOdd = strided(N, stride / 2, stride);
        k /= 2;
    }
    Strided oE = strided(out.n, 0, 2), oO = strided(out.n, 1, 2);
    for (int q = 0; q < 3; q++)
        for (int s = 0; s < 2; s++) {
            for (size_t i = 0; i < gEven.size && i < oE.size; i++)
                out.v[q][s][oE.offset + i * 2] = g.v[q][s][gEven.offset + i * gEven.stride];
            for (size_t i = 0; i < gOdd.size && i < oO.size; i++)
                out.v[q][s][oO.offset + i * 2] = g.v[q][s][gOdd.offset + i * gOdd.stride];
        }
}

// dReLU (RSS.inl:807-852) over a strided view of the input.
template <typename T, typename U>
void rss_drelu(const RSSV<T>& in, Strided w, RSSV<U>& result, Comm& comm) {
    const int W = sizeof(T) * 8;
    size_t n = w.size;
    RSSV<U> rbits(n * W);
    rss_fill<U>(rbits, 1);
    std::vector<T> a[3];
    rss_reconstruct(in, w, a, comm);  // r = input; reconstruct(r, a)
    std::vector<U> abits[3];
    for (int p = 0; p < 3; p++) {
        for (auto& x : a[p]) x = (T)(x + 1);
        bitexpand<T, U>(a[p], abits[p]);
    }
    RSSV<U> msb(n);
    for (int p = 0; p < 3; p++) {
        std::vector<U>& r0 = rbits.v[p][0];
        std::vector<U>& r1 = rbits.v[p][1];
        if (p != PC) {
            set_carry_out_msb<U>(r0, abits[p], msb.v[p][0], W, p == PA);
            set_carry_out_msb<U>(r1, abits[p], msb.v[p][1], W, p == PC);
        } else {
            set_carry_out_msb<U>(r1, abits[p], msb.v[p][1], W, p == PC);
            set_carry_out_msb<U>(r0, abits[p], msb.v[p][0], W, p == PA);
        }
    }
    RSSV<U> g(n * W), pp(n * W);
    for (int p = 0; p < 3; p++)
        for (size_t i = 0; i < n * W; i++) {
            // g = rbits & abits (RSS &= DeviceData: both shares)
            g.v[p][0][i] = rbits.v[p][0][i] & abits[p][i];
            g.v[p][1][i] = rbits.v[p][1][i] & abits[p][i];
            // p = rbits ^ abits (RSS ^= DeviceData: A.shareA, C.shareB)
            pp.v[p][0][i] = rbits.v[p][0][i] ^ (p == PA ? abits[p][i] : (U)0);
            pp.v[p][1][i] = rbits.v[p][1][i] ^ (p == PC ? abits[p][i] : (U)0);
        }
    RSSV<U> pre(result.n);
    carry_out(pp, g, W, pre, comm);
    rss_xor_assign(pre, whole(pre.n), msb, whole(msb.n));
    // result.fill(1); result -= preResult
    for (int p = 0; p < 3; p++)
        for (size_t i = 0; i < result.n; i++) {
            result.v[p][0][i] = (U)((p == PA ? 1 : 0) - pre.v[p][0][i]);
            result.v[p][1][i] = (U)((p == PC ? 1 : 0) - pre.v[p][1][i]);
        }
}

// convex_comb (RSS.inl:1322-1333 with rss_convex_comb_functor :33-61)
template <typename T, typename U>
void convex_comb(RSSV<T>& d, const RSSV<T>& c, const std::vector<U> (&e)[3]) {
    for (int p = 0; p < 3; p++)
        for (size_t i = 0; i < d.n; i++) {
            T c0 = c.v[p][0][i], c1 = c.v[p][1][i];
            if (e[p][i] == 1) {
                if (p == PA) { d.v[p][0][i] = (T)(1 - c0); d.v[p][1][i] = (T)(0 - c1); }
                else if (p == PB) { d.v[p][0][i] = (T)(0 - c0); d.v[p][1][i] = (T)(0 - c1); }
                else { d.v[p][0][i] = (T)(0 - c0); d.v[p][1][i] = (T)(1 - c1); }
            } else {
                d.v[p][0][i] = c0; d.v[p][1][i] = c1;
            }
        }
}

// selectShare (RSS.inl:543-569): z = (y - x) * d + x with d from the revealed b.
// x, y, z may be strided views of larger tensors (maxpool uses that).
template <typename T, typename U>
void rss_select_share(const RSSV<T>& x, Strided wx, const RSSV<T>& y, Strided wy, const RSSV<U>& b,
                      RSSV<T>& z, Strided wz, Comm& comm) {
    size_t n = wx.size;
    RSSV<T> c(n);
    std::vector<U> e[3];
    rss_reconstruct(b, whole(b.n), e, comm);  // cbits = 0 ^ b; reconstruct(cbits, e)
    RSSV<T> d(n);
    convex_comb(d, c, e);
    RSSV<T> res(n);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            for (size_t i = 0; i < n; i++)
                res.v[p][s][i] = (T)(y.v[p][s][wy.offset + i * wy.stride] - x.v[p][s][wx.offset + i * wx.stride]);
    rss_mul_assign(res, d, comm);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            for (size_t i = 0; i < n; i++)
                z.v[p][s][wz.offset + i * wz.stride] = (T)(res.v[p][s][i] + x.v[p][s][wx.offset + i * wx.stride]);
}

// ReLU (RSS.inl:855-865)
template <typename T, typename U> void rss_relu(const RSSV<T>& in, RSSV<T>& out, RSSV<U>& dout, Comm& comm) {
    rss_drelu<T, U>(in, whole(in.n), dout, comm);
    RSSV<T> zeros(in.n);
    out.resize(in.n);
    rss_select_share<T, U>(zeros, whole(in.n), in, whole(in.n), dout, out, whole(in.n), comm);
}

// expandCompare (bitwise.cuh:66-92), in-bounds part
template <typename U>
void expand_compare(const std::vector<U>& b, const std::vector<U>& nb, std::vector<U>& expanded) {
    if (b.empty()) return;  // bitwise.cuh:70 divides by b.size(): empty pool rows have nothing to expand
    size_t f = (expanded.size() / b.size()) / 2;
    for (size_t i = 0; i < b.size(); i++)
        for (size_t e = 0; e < 2 * f; e++) expanded[i * 2 * f + e] = e < f ? b[i] : nb[i];
}

// maxpool (RSS.inl:868-1017): tournament over strided even/odd views of the
// (padded) pool rows; dresult tracks the argmax one-hot.
template <typename T, typename U>
void rss_maxpool(RSSV<T>& input, RSSV<T>& result, RSSV<U>& dresult, int k, Comm& comm) {
    size_t N = input.n;
    rss_fill<U>(dresult, 1);
    size_t stride = 2;
    Strided even = strided(N, 0, stride), odd = strided(N, 1, stride);
    auto level = [&](bool last) {
        RSSV<T> diff(even.size);
        for (int p = 0; p < 3; p++)
            for (int s = 0; s < 2; s++)
                for (size_t i = 0; i < even.size; i++)
                    diff.v[p][s][i] = (T)(input.v[p][s][even.offset + i * even.stride] -
                                          input.v[p][s][odd.offset + i * odd.stride]);
        RSSV<U> b(even.size);
        rss_drelu<T, U>(diff, whole(diff.n), b, comm);
        rss_select_share<T, U>(input, odd, input, even, b, input, even, comm);
        if (!last) {
            stride *= 2;
            even = strided(N, 0, stride);
            odd = strided(N, stride / 2, stride);
        } else {
            result.resize(even.size);
            for (int p = 0; p < 3; p++)
                for (int s = 0; s < 2; s++)
                    for (size_t i = 0; i < even.size; i++)
                        result.v[p][s][i] = input.v[p][s][even.offset + i * even.stride];
        }
        RSSV<U> neg(b.n);
        rss_fill<U>(neg, 1);
        for (int p = 0; p < 3; p++)
            for (int s = 0; s < 2; s++)
                for (size_t i = 0; i < b.n; i++) neg.v[p][s][i] = (U)(neg.v[p][s][i] - b.v[p][s][i]);
        RSSV<U> expanded(N);
        for (int p = 0; p < 3; p++)
            for (int s = 0; s < 2; s++) expand_compare<U>(b.v[p][s], neg.v[p][s], expanded.v[p][s]);
        rss_and_assign(dresult, whole(N), expanded, whole(N), comm);
    };
    while (k > 2) {
        level(false);
        k /= 2;
    }
    level(true);
}

// maxpool_im2row + stride_pad (convolution.cuh:56-108,175-191,252-304).
// Input is read with the reference's (batch, x=col, y=row, channel) indexing.
template <typename T>
void maxpool_im2row(const T* im, std::vector<T>& out, int H, int W, int f, int Din, int batch, int stride,
                    int pad, T pad_val) {
    int wK = (W - f + 2 * pad) / stride + 1, hK = (H - f + 2 * pad) / stride + 1;
    int pool = f * f;
    std::vector<T> unpadded((size_t)pool * wK * hK * batch * Din, 0);
    for (int ic = 0; ic < batch * Din; ic++)
        for (int win = 0; win < wK * hK; win++) {
            int b = ic / Din, ch = ic % Din;
            int baseCol = (win / hK) * stride - pad, baseRow = (win % hK) * stride - pad;
            size_t o = (size_t)b * (wK * hK * Din * pool) + (size_t)win * (Din * pool) + (size_t)ch * pool;
            for (int c = 0; c < f; c++)
                for (int r = 0; r < f; r++) {
                    int y = baseRow + r, x = baseCol + c;
                    if (y < 0 || y >= H || x < 0 || x >= W) continue;  // slot left untouched
                    unpadded[o++] = im[(size_t)b * H * W * Din + (size_t)x * H * Din + (size_t)y * Din + ch];
                }
        }
    int padded = (int)std::pow(std::ceil(std::log2((double)pool)), 2);
    out.assign((size_t)padded * wK * hK * batch * Din, 0);
    if (padded == pool) {
        out = unpadded;
    } else {
        size_t npools = (size_t)wK * hK * batch * Din;
        for (size_t q = 0; q < npools; q++) {
            for (int j = 0; j < pool; j++) out[q * padded + j] = unpadded[q * pool + j];
            for (int j = pool; j < padded; j++) out[q * padded + j] = pad_val;
        }
    }
}

// truncate_cols (matrix.cuh:141-154)
template <typename T> void truncate_cols(const T* a, T* b, size_t rows, int start_cols, int end_cols) {
    for (size_t r = 0; r < rows; r++)
        for (int i = 0; i < end_cols; i++) b[r * end_cols + i] = a[r * start_cols + i];
}

// elementVectorAdd (matrix.cuh:75-84): a[col*rows + row] += b[rowwise ? col : row]
template <typename T> void element_vector_add(T* a, const T* b, bool rowwise, int rows, int cols) {
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) a[(size_t)c * rows + r] = (T)(a[(size_t)c * rows + r] + b[rowwise ? c : r]);
}

// reduceSum (matrix.cuh:109-126); b accumulates (+=) like the reference.
template <typename T> void reduce_sum(const T* a, T* b, bool reduceRows, int rows, int cols) {
    int outn = reduceRows ? cols : rows;
    for (int c = 0; c < outn; c++)
        for (int i = 0; i < (reduceRows ? rows : cols); i++)
            b[c] = (T)(b[c] + (reduceRows ? a[(size_t)cols * i + c] : a[(size_t)cols * c + i]));
}

// MaxpoolLayer::forward (MaxpoolLayer.cu:52-131) for RSS (numShares() == 2,
// so every share of every party is padded with -10 * 2^FP).
template <typename T, typename U>
void maxpool_layer_forward(const RSSV<T>& in, RSSV<T>& act, RSSV<U>& maxPrime, int H, int W, int C, int pool,
                           int stride, int batch, int fp, Comm& comm) {
    int padded = (int)std::pow(std::ceil(std::log2((double)(pool * pool))), 2);
    T pad_val = (T)(int64_t)(-10 * (1 << fp));
    RSSV<T> pools;
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++) {
            std::vector<T> o;
            maxpool_im2row<T>(in.v[p][s].data(), o, H, W, pool, C, batch, stride, 0, pad_val);
            if (p == 0 && s == 0) pools.resize(o.size());
            pools.v[p][s] = o;
        }
    RSSV<U> expMax(pools.n);
    rss_maxpool<T, U>(pools, act, expMax, padded, comm);
    size_t rows = pools.n / padded;
    maxPrime.resize(rows * pool * pool);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            truncate_cols<U>(expMax.v[p][s].data(), maxPrime.v[p][s].data(), rows, padded, pool * pool);
}


// ---------------------------------------------------------- training step

// vectorExpand (matrix.cuh:129-139): b[i * f + j] = a[i]
template <typename T> void vector_expand(const T* a, size_t n, T* b, size_t f) {
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < f; j++) b[i * f + j] = a[i];
}

// maxpool_row2im (convolution.cuh:111-152): every window value is added
// (atomicAdd) into its image position, with the (batch, x, y, channel)
// indexing of maxpool_im2row.
template <typename T>
void maxpool_row2im(const T* rows, T* out, int imageHeight, int imageWidth, int f, int Din, int batch, int stride) {
    const int wk = (imageWidth - f) / stride + 1, hk = (imageHeight - f) / stride + 1;
    const size_t windows = (size_t)batch * Din * wk * hk;
    for (size_t cw = 0; cw < windows; cw++)
        for (int v = 0; v < f * f; v++) {
            size_t b = cw / ((size_t)wk * hk * Din);
            size_t rem = cw % ((size_t)wk * hk * Din);
            int widx = (int)(rem / Din), ch = (int)(rem % Din);
            int wcol = widx / hk, wrow = widx % hk;
            int vcol = wcol * stride + v / f, vrow = wrow * stride + v % f;
            size_t o = b * (size_t)imageHeight * imageWidth * Din + (size_t)vcol * imageHeight * Din + (size_t)vrow * Din + ch;
            out[o] = (T)(out[o] + rows[cw * f * f + v]);
        }
}

// ReLULayer::backward (ReLULayer.cu:90-124): deltas = selectShare(0, delta, reluPrime)
template <typename T, typename U>
void relu_layer_backward(const RSSV<T>& delta, const RSSV<U>& reluPrime, RSSV<T>& deltas, Comm& comm) {
    RSSV<T> zeros(delta.n);
    deltas.resize(delta.n);
    rss_select_share<T, U>(zeros, whole(delta.n), delta, whole(delta.n), reluPrime, deltas, whole(delta.n), comm);
}

// MaxpoolLayer::backward (MaxpoolLayer.cu:133-185): expand the incoming delta
// over each pool, keep it where maxPrime selects, scatter back with row2im.
// The reference passes (imageWidth, imageHeight) into row2im's (imageHeight,
// imageWidth) parameters; the swap is kept (it only matters for non-square
// images).
template <typename T, typename U>
void maxpool_layer_backward(const RSSV<T>& delta, const RSSV<U>& maxPrime, RSSV<T>& deltas, int H, int W, int C,
                            int pool, int stride, int batch, Comm& comm) {
    const size_t f2 = (size_t)pool * pool;
    RSSV<T> pools(maxPrime.n), zeros(maxPrime.n);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++) vector_expand<T>(delta.v[p][s].data(), delta.n, pools.v[p][s].data(), f2);
    rss_select_share<T, U>(zeros, whole(pools.n), pools, whole(pools.n), maxPrime, pools, whole(pools.n), comm);
    deltas.resize((size_t)batch * H * W * C);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++) maxpool_row2im<T>(pools.v[p][s].data(), deltas.v[p][s].data(), W, H, pool, C, batch, stride);
}

// AveragepoolLayer::forward (AveragepoolLayer.cu:58-81): averagepool_im2row
// (convolution.cuh:340-374, which hands the kernel of :56-107 its width and
// height swapped), reduceSum of each window, dividePublic by pool^2. Window
// positions out of the image are skipped by that kernel; with padding 0 and
// whole windows there are none.
template <typename T>
void avgpool_layer_forward(const RSSV<T>& in, RSSV<T>& act, int H, int W, int C, int pool, int stride, int batch,
                           Comm& comm) {
    const int kW = H, kH = W;  // the kernel's imageWidth / imageHeight
    const int wk = (kW - pool) / stride + 1, hk = (kH - pool) / stride + 1;
    const size_t n_out = (size_t)batch * wk * hk * C;
    act.resize(n_out);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            for (size_t e = 0; e < n_out; e++) {
                const size_t b = e / ((size_t)wk * hk * C), rem = e % ((size_t)wk * hk * C);
                const int win = (int)(rem / C), ch = (int)(rem % C);
                const int base_col = (win / hk) * stride, base_row = (win % hk) * stride;
                T acc = 0;
                for (int c = 0; c < pool; c++)
                    for (int r = 0; r < pool; r++) {
                        const int y = base_row + r, x = base_col + c;
                        if (y < 0 || y >= kH || x < 0 || x >= kW) continue;
                        acc = (T)(acc + in.v[p][s][b * (size_t)kH * kW * C + (size_t)x * kH * C + (size_t)y * C + ch]);
                    }
                act.v[p][s][e] = acc;
            }
    T d = (T)(pool * pool);
    rss_divide_public<T>(act, &d, false, comm);
}

// AveragepoolLayer::backward (AveragepoolLayer.cu:88-117) with
// averagepool_expand_delta (convolution.cuh:195-208): delta element i is
// copied to slots (i / C) * C * pool^2 + i % C + k * C, k < pool^2, of the
// zeroed input gradient (the input layout for a global pool), then / pool^2.
// The slots stay inside the input gradient only when delta.n * pool^2 <=
// batch * H * W * C (pools that tile the image); the C entry point refuses
// overlapping pools, for which the reference's kernel writes past its
// buffer.
template <typename T>
void avgpool_layer_backward(const RSSV<T>& delta, RSSV<T>& deltas, int H, int W, int C, int pool, int batch,
                            Comm& comm) {
    const int f2 = pool * pool;
    deltas.resize((size_t)batch * H * W * C);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            for (size_t i = 0; i < delta.n; i++) {
                const size_t b = i / C, ch = i % C;
                for (size_t j = b * C * f2 + ch; j < (b + 1) * C * f2; j += C) deltas.v[p][s][j] = delta.v[p][s][i];
            }
    T d = (T)f2;
    rss_divide_public<T>(deltas, &d, false, comm);
}

template <typename T> static void rss_sub_assign(RSSV<T>& a, const RSSV<T>& b) {
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++)
            for (size_t i = 0; i < a.n; i++) a.v[p][s][i] = (T)(a.v[p][s][i] - b.v[p][s][i]);
}

// FCLayer::backward (FCLayer.cu:132-217): deltas with the weights before the
// update, dW truncated by FP + lr, db by the reference's reduceSum call
// (reduceRows = false, rows = outputDim, cols = batchSize) then / 2^lr.
template <typename T>
void fc_layer_backward(const RSSV<T>& delta, const RSSV<T>& fwdInput, RSSV<T>& W, RSSV<T>& b, RSSV<T>& deltas,
                       int batch, int din, int dout, int fp, int lr, Comm& comm) {
    rss_matmul<T>(delta, W, deltas, batch, din, dout, true, false, true, fp, comm);
    RSSV<T> dW;
    rss_matmul<T>(delta, fwdInput, dW, dout, din, batch, false, true, false, fp + lr, comm);
    rss_sub_assign(W, dW);
    RSSV<T> db(dout);
    for (int p = 0; p < 3; p++)
        for (int s = 0; s < 2; s++) reduce_sum<T>(delta.v[p][s].data(), db.v[p][s].data(), false, dout, batch);
    T d = (T)((T)1 << lr);
    rss_divide_public<T>(db, &d, false, comm);
    rss_sub_assign(b, db);
}

// CNNLayer::backward (CNNLayer.cu:114-193): dgrad and wgrad convolutions
// truncated by FP, dF / 2^lr, no bias.
template <typename T>
void cnn_layer_backward(const RSSV<T>& delta, const RSSV<T>& fwdInput, RSSV<T>& Wt, RSSV<T>& deltas, int batch, int H,
                        int W, int Din, int Dout, int f, int stride, int pad, int fp, int lr, Comm& comm) {
    rss_convolution<T>(delta, Wt, deltas, CONV_DGRAD, batch, H, W, f, Din, Dout, stride, pad, fp, comm);
    RSSV<T> dF;
    rss_convolution<T>(delta, fwdInput, dF, CONV_WGRAD, batch, H, W, f, Din, Dout, stride, pad, fp, comm);
    T d = (T)((T)1 << lr);
    rss_divide_public<T>(dF, &d, false, comm);
    rss_sub_assign(Wt, dF);
}

// to_fixed_functor (util/functors.h:117-123) runs on the device: PTX
// cvt.rzi.u64.f64 truncates toward zero and saturates, NaN -> 0.
template <typename T> static inline T to_fixed_device(double x) {
    if (std::isnan(x) || x <= 0.0) return (T)0;
    if (x >= std::ldexp(1.0, (int)sizeof(T) * 8)) return std::numeric_limits<T>::max();
    return (T)x;
}

// NeuralNetwork::_reveal_softmax_grad (NeuralNetwork.cu:207-267): each party
// reveals the logits, takes the softmax in double on the host (exp per value,
// row sums in index order), converts back to fixed point, and the deltas are
// softmax (added like public data: party A shareA, party C shareB) minus the
// labels, divided by the batch when LOG_MINI_BATCH = (int)log2(batch) > 1.
template <typename T>
void rss_reveal_softmax_grad(const RSSV<T>& act, const RSSV<T>& labels, int batch, int fp, RSSV<T>& deltas,
                             Comm& comm) {
    typedef typename std::make_signed<T>::type S;
    const size_t n = act.n;
    const size_t classes = n / (size_t)batch;
    std::vector<T> rev[3];
    rss_reconstruct(act, whole(n), rev, comm);
    std::vector<T> sm[3];
    for (int p = 0; p < 3; p++) {
        std::vector<double> fa(n), sums(n / classes, 0.0);
        for (size_t i = 0; i < n; i++) fa[i] = ((double)((S)rev[p][i])) / (double)(1 << fp);
        for (size_t i = 0; i < n; i++) {
            fa[i] = std::exp(fa[i]);
            sums[i / classes] += fa[i];
        }
        for (size_t i = 0; i < n; i++) fa[i] /= sums[i / classes];
        sm[p].resize(n);
        for (size_t i = 0; i < n; i++) sm[p][i] = to_fixed_device<T>(fa[i] * (double)(1 << fp));
    }
    deltas.resize(n);
    for (size_t i = 0; i < n; i++) {
        deltas.v[PA][0][i] = sm[PA][i];
        deltas.v[PC][1][i] = sm[PC][i];
    }
    rss_sub_assign(deltas, labels);
    const int log_mb = (int)std::log2((double)batch);
    if (log_mb > 1) {
        T d = (T)((T)1 << log_mb);
        rss_divide_public<T>(deltas, &d, false, comm);
    }
}


// ========================================================================
// TPC: 2-party additive sharing (src/mpc/TPC.h, TPC.inl). Each party holds
// one share; x = x_A + x_B. Multiplications use the Beaver triples of
// Precompute.h (constant: x = y = z = 1 elementwise, the matrix triple
// x = y = 1 with z = K, the convolution triples x = y = z = 0). Adding public
// DeviceData to a TPC share changes party A's share only (TPC.inl:175-189).
// ========================================================================

enum { TA = 0, TB = 1 };

template <typename T> struct TPCV {
    size_t n = 0;
    std::vector<T> s[2];
    TPCV() {}
    explicit TPCV(size_t n_) { resize(n_); }
    void resize(size_t n_) {
        n = n_;
        for (int p = 0; p < 2; p++) s[p].assign(n, (T)0);
    }
};

// TPC.inl:104-106
template <typename T> void tpc_fill(TPCV<T>& a, T val) {
    std::fill(a.s[TA].begin(), a.s[TA].end(), val);
    std::fill(a.s[TB].begin(), a.s[TB].end(), (T)0);
}

// TPC.inl:109-123 (setPublic) and :341-363 (initializer list): A holds the values
template <typename T> void tpc_from_list(TPCV<T>& a, const double* vals, int fp, bool to_fixed) {
    for (size_t i = 0; i < a.n; i++) {
        a.s[TA][i] = to_fixed ? encode_fixed<T>(vals[i], fp) : (T)(int64_t)vals[i];
        a.s[TB][i] = 0;
    }
}

// reconstruct (TPC.inl:552-572): each party sends its share to the other;
// out = own share + received share.
template <typename T> void tpc_reconstruct(const TPCV<T>& in, Strided w, std::vector<T> (&out)[2], Comm& comm) {
    for (int p = 0; p < 2; p++) {
        out[p].resize(w.size);
        for (size_t i = 0; i < w.size; i++) {
            size_t j = w.offset + i * w.stride;
            out[p][i] = (T)(in.s[p][j] + in.s[1 - p][j]);
        }
    }
    comm.msg(2, w.size * sizeof(T), w.size * sizeof(T));
    comm.rounds++;
}

template <typename T> static TPCV<T> tpc_gather(const TPCV<T>& a, Strided w) {
    TPCV<T> r(w.size);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < w.size; i++) r.s[p][i] = a.s[p][w.offset + i * w.stride];
    return r;
}
template <typename T> static void tpc_scatter(TPCV<T>& a, Strided w, const TPCV<T>& r) {
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < w.size; i++) a.s[p][w.offset + i * w.stride] = r.s[p][i];
}

// TPC *= TPC (TPC.inl:242-272) on the view wa of a, with b viewed by wb.
template <typename T> void tpc_mul_assign(TPCV<T>& a, Strided wa, const TPCV<T>& b, Strided wb, Comm& comm) {
    size_t n = wb.size;
    TPCV<T> self = tpc_gather(a, wa), rhs = tpc_gather(b, wb);
    TPCV<T> x(n), y(n), z(n);
    tpc_fill<T>(x, 1); tpc_fill<T>(y, 1); tpc_fill<T>(z, 1);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) {
            x.s[p][i] = (T)(x.s[p][i] + self.s[p][i]);
            y.s[p][i] = (T)(y.s[p][i] + rhs.s[p][i]);
        }
    std::vector<T> e[2], f[2];
    tpc_reconstruct(x, whole(n), e, comm);
    tpc_reconstruct(y, whole(n), f, comm);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) {
            x.s[p][i] = (T)(x.s[p][i] - self.s[p][i]);
            y.s[p][i] = (T)(y.s[p][i] - rhs.s[p][i]);
        }
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) {
            T v = z.s[p][i];                                                     // this = 0; this += z
            if (p == TA) v = (T)(v + (T)((T)(f[p][i] - y.s[p][i]) * e[p][i]));  // += (f - y) * e  (A only)
            if (p == TA) v = (T)(v + (T)((T)(0 - x.s[p][i]) * f[p][i]));        // += (-x) * f     (A only)
            self.s[p][i] = v;
        }
    tpc_scatter(a, wa, self);
}

// TPC &= TPC (TPC.inl:281-312): the boolean Beaver triple, with reconstruct
// still adding the two shares.
template <typename U> void tpc_and_assign(TPCV<U>& a, Strided wa, const TPCV<U>& b, Strided wb, Comm& comm) {
    size_t n = wb.size;
    TPCV<U> self = tpc_gather(a, wa), rhs = tpc_gather(b, wb);
    TPCV<U> x(n), y(n), z(n);
    tpc_fill<U>(x, 1); tpc_fill<U>(y, 1); tpc_fill<U>(z, 1);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) {
            x.s[p][i] ^= self.s[p][i];
            y.s[p][i] ^= rhs.s[p][i];
        }
    std::vector<U> e[2], f[2];
    tpc_reconstruct(x, whole(n), e, comm);
    tpc_reconstruct(y, whole(n), f, comm);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) {
            x.s[p][i] ^= self.s[p][i];
            y.s[p][i] ^= rhs.s[p][i];
        }
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) {
            U v = z.s[p][i];
            if (p == TA) v ^= (U)((U)(f[p][i] ^ y.s[p][i]) & e[p][i]);
            if (p == TA) v ^= (U)(x.s[p][i] & f[p][i]);
            self.s[p][i] = v;
        }
    tpc_scatter(a, wa, self);
}

// TPC ^= TPC: local (TPC.inl:276-279)
template <typename U> void tpc_xor_assign(TPCV<U>& a, Strided wa, const TPCV<U>& b, Strided wb) {
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < wb.size; i++) a.s[p][wa.offset + i * wa.stride] ^= b.s[p][wb.offset + i * wb.stride];
}

// dividePublic (TPC.inl:371-401) with getDividedShares (Precompute.h:112-134):
// r = 1 and r' = d (scalar) or r' = d_i (vector), both held by party A.
template <typename T> void tpc_divide_public(TPCV<T>& a, const T* d, bool vec, Comm& comm) {
    for (size_t i = 0; i < a.n; i++) a.s[TA][i] = (T)(a.s[TA][i] - (vec ? d[i] : d[0]));  // a -= r'
    std::vector<T> rec[2];
    tpc_reconstruct(a, whole(a.n), rec, comm);
    for (size_t i = 0; i < a.n; i++) {
        T q = div_public<T>(rec[TA][i], vec ? d[i] : d[0]);
        a.s[TA][i] = (T)(1 + q);  // a = 0; a += r (A: 1); a += reconstructed (A only)
        a.s[TB][i] = 0;
    }
}

// localMatMul (TPC.inl:1060-1091) with the matrix triple of Precompute.h:77-90,
// then dividePublic by 2^trunc (matmul, TPC.inl:575-583).
template <typename T>
void tpc_matmul(const TPCV<T>& a, const TPCV<T>& b, TPCV<T>& c, int M, int N, int K, bool tA, bool tB, bool tC,
                int trunc, Comm& comm) {
    TPCV<T> x(a.n), y(b.n);
    tpc_fill<T>(x, 1); tpc_fill<T>(y, 1);
    for (int p = 0; p < 2; p++) {
        for (size_t i = 0; i < a.n; i++) x.s[p][i] = (T)(x.s[p][i] + a.s[p][i]);
        for (size_t i = 0; i < b.n; i++) y.s[p][i] = (T)(y.s[p][i] + b.s[p][i]);
    }
    std::vector<T> e[2], f[2];
    tpc_reconstruct(x, whole(x.n), e, comm);
    tpc_reconstruct(y, whole(y.n), f, comm);
    for (int p = 0; p < 2; p++) {
        for (size_t i = 0; i < a.n; i++) x.s[p][i] = (T)(x.s[p][i] - a.s[p][i]);
        for (size_t i = 0; i < b.n; i++) y.s[p][i] = (T)(y.s[p][i] - b.s[p][i]);
    }
    size_t mn = (size_t)M * N;
    c.resize(mn);
    std::vector<T> t(mn);
    for (int p = 0; p < 2; p++) {
        for (size_t i = 0; i < mn; i++) c.s[p][i] = p == TA ? (T)K : (T)0;  // c = 0; c += z (z = K at A)
        if (p != TA) continue;  // TPC += DeviceData: party A only
        gemm<T>(M, N, K, e[p].data(), tA, f[p].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) c.s[p][i] = (T)(c.s[p][i] + t[i]);
        gemm<T>(M, N, K, e[p].data(), tA, y.s[p].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) c.s[p][i] = (T)(c.s[p][i] - t[i]);
        gemm<T>(M, N, K, x.s[p].data(), tA, f[p].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) c.s[p][i] = (T)(c.s[p][i] - t[i]);
    }
    T d = (T)((T)1 << trunc);
    tpc_divide_public(c, &d, false, comm);
}

// convolution (TPC.inl:789-827) with localFprop/Dgrad/Wgrad (:645-787): the
// convolution triples are all zero, so party A's share becomes conv(A, B) of
// the revealed operands and party B's 0; then dividePublic by 2^trunc.
template <typename T>
void tpc_convolution(const TPCV<T>& A, const TPCV<T>& B, TPCV<T>& C, int op, int batch, int H, int W, int f,
                     int Din, int Dout, int stride, int pad, int trunc, Comm& comm) {
    ConvShape sh{batch, H, W, Din, Dout, f, f, pad, stride};
    size_t out_n = op == CONV_FPROP ? (size_t)batch * sh.P() * sh.Q() * Dout
                 : op == CONV_DGRAD ? (size_t)batch * H * W * Din
                                    : (size_t)Dout * f * f * Din;
    std::vector<T> e[2], fr[2];
    tpc_reconstruct(A, whole(A.n), e, comm);  // x = 0 + A
    tpc_reconstruct(B, whole(B.n), fr, comm);
    C.resize(out_n);
    std::vector<T> t(out_n);
    conv_any<T>(op, sh, e[TA].data(), fr[TA].data(), t.data());  // the e*y and x*f terms are 0
    for (size_t i = 0; i < out_n; i++) C.s[TA][i] = t[i];
    T d = (T)((T)1 << trunc);
    tpc_divide_public(C, &d, false, comm);
}

// carryOut (TPC.inl:1093-1146): the RSS tree with TPC ANDs.
template <typename U> void tpc_carry_out(TPCV<U>& p, TPCV<U>& g, int k, TPCV<U>& out, Comm& comm) {
    size_t N = p.n;
    size_t stride = 2, offset = 1;
    Strided pEven = strided(N, 0, stride), pOdd = strided(N, offset, stride);
    Strided gEven = strided(N, 0, stride), gOdd = strided(N, offset, stride);
    while (k > 1) {
        tpc_and_assign(g, gEven, p, pOdd, comm);
        tpc_and_assign(p, pEven, p, pOdd, comm);
        tpc_xor_assign(g, gOdd, g, gEven);
        gEven = strided(N, offset, stride * 2);
        offset += stride;
        gOdd = strided(N, offset, stride * 2);
        stride *= 2;
        pEven = strided(N, 0, stride);
        pOdd = strided(N, stride / 2, stride);
        k /= 2;
    }
    Strided oE = strided(out.n, 0, 2), oO = strided(out.n, 1, 2);
    for (int q = 0; q < 2; q++) {
        for (size_t i = 0; i < gEven.size && i < oE.size; i++) out.s[q][oE.offset + i * 2] = g.s[q][gEven.offset + i * gEven.stride];
        for (size_t i = 0; i < gOdd.size && i < oO.size; i++) out.s[q][oO.offset + i * 2] = g.s[q][gOdd.offset + i * gOdd.stride];
    }
}

// dReLU (TPC.inl:829-868)
template <typename T, typename U> void tpc_drelu(const TPCV<T>& in, Strided w, TPCV<U>& result, Comm& comm) {
    const int W = sizeof(T) * 8;
    size_t n = w.size;
    TPCV<U> rbits(n * W);
    tpc_fill<U>(rbits, 1);
    std::vector<T> a[2];
    tpc_reconstruct(in, w, a, comm);  // r = 0; r += input; reconstruct(r, a)
    std::vector<U> abits[2];
    for (int p = 0; p < 2; p++) {
        for (auto& x : a[p]) x = (T)(x + 1);
        bitexpand<T, U>(a[p], abits[p]);
    }
    TPCV<U> msb(n);
    for (int p = 0; p < 2; p++) set_carry_out_msb<U>(rbits.s[p], abits[p], msb.s[p], W, p == TA);
    TPCV<U> g(n * W), pp(n * W);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n * W; i++) {
            g.s[p][i] = rbits.s[p][i] & abits[p][i];                           // &= DeviceData: every party
            pp.s[p][i] = rbits.s[p][i] ^ (p == TA ? abits[p][i] : (U)0);  // ^= DeviceData: party A
        }
    TPCV<U> pre(n);
    tpc_carry_out(pp, g, W, pre, comm);
    tpc_xor_assign(pre, whole(n), msb, whole(n));
    result.resize(n);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) result.s[p][i] = (U)((p == TA ? 1 : 0) - pre.s[p][i]);
}

// selectShare (TPC.inl:586-610) with convex_comb (:1282-1289, functor :31-53).
template <typename T, typename U>
void tpc_select_share(const TPCV<T>& x, Strided wx, const TPCV<T>& y, Strided wy, const TPCV<U>& b, TPCV<T>& z,
                      Strided wz, Comm& comm) {
    size_t n = wx.size;
    std::vector<U> e[2];
    tpc_reconstruct(b, whole(b.n), e, comm);  // cbits = 0 ^ b
    TPCV<T> d(n);                             // c = 0
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++) d.s[p][i] = e[p][i] == 1 ? (p == TA ? (T)1 : (T)0) : (T)0;
    TPCV<T> res(n);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++)
            res.s[p][i] = (T)(y.s[p][wy.offset + i * wy.stride] - x.s[p][wx.offset + i * wx.stride]);
    tpc_mul_assign(res, whole(n), d, whole(n), comm);
    for (int p = 0; p < 2; p++)
        for (size_t i = 0; i < n; i++)
            z.s[p][wz.offset + i * wz.stride] = (T)(res.s[p][i] + x.s[p][wx.offset + i * wx.stride]);
}

// ReLU (TPC.inl:871-884)
template <typename T, typename U> void tpc_relu(const TPCV<T>& in, TPCV<T>& out, TPCV<U>& dout, Comm& comm) {
    tpc_drelu<T, U>(in, whole(in.n), dout, comm);
    TPCV<T> zeros(in.n);
    out.resize(in.n);
    tpc_select_share<T, U>(zeros, whole(in.n), in, whole(in.n), dout, out, whole(in.n), comm);
}

// maxpool (TPC.inl:887-1058)
template <typename T, typename U>
void tpc_maxpool(TPCV<T>& input, TPCV<T>& result, TPCV<U>& dresult, int k, Comm& comm) {
    size_t N = input.n;
    dresult.resize(N);
    tpc_fill<U>(dresult, 1);
    size_t stride = 2;
    Strided even = strided(N, 0, stride), odd = strided(N, 1, stride);
    auto level = [&](bool last) {
        TPCV<T> diff(even.size);
        for (int p = 0; p < 2; p++)
            for (size_t i = 0; i < even.size; i++)
                diff.s[p][i] = (T)(input.s[p][even.offset + i * even.stride] - input.s[p][odd.offset + i * odd.stride]);
        TPCV<U> b(even.size);
        tpc_drelu<T, U>(diff, whole(diff.n), b, comm);
        tpc_select_share<T, U>(input, odd, input, even, b, input, even, comm);
        if (!last) {
            stride *= 2;
            even = strided(N, 0, stride);
            odd = strided(N, stride / 2, stride);
        } else {
            result.resize(even.size);
            for (int p = 0; p < 2; p++)
                for (size_t i = 0; i < even.size; i++) result.s[p][i] = input.s[p][even.offset + i * even.stride];
        }
        TPCV<U> neg(b.n);
        tpc_fill<U>(neg, 1);
        for (int p = 0; p < 2; p++)
            for (size_t i = 0; i < b.n; i++) neg.s[p][i] = (U)(neg.s[p][i] - b.s[p][i]);
        TPCV<U> expanded(N);
        for (int p = 0; p < 2; p++) expand_compare<U>(b.s[p], neg.s[p], expanded.s[p]);
        tpc_and_assign(dresult, whole(N), expanded, whole(N), comm);
    };
    while (k > 2) {
        level(false);
        k /= 2;
    }
    level(true);
}


// ========================================================================
// FPC: 4-party replicated sharing (src/mpc/FPC.h, FPC.inl). x = x0+x1+x2+x3;
// party p (A=0 .. D=3) holds the three components it is not named after,
// share k = component (p+1+k) mod 4 (FPC.inl:948-953). Public values and
// public DeviceData added, subtracted or XORed go into component x0 only,
// held by B as shareC, C as shareB and D as shareA (FPC.inl:120-125,
// :184-260); *=, &=, >>= and <<= by public data touch every share.
// Products reshare their cross terms with reshareFPC (FPC.inl:1184-1259),
// whose PRG masks are zero.
// ========================================================================

template <typename T> struct FPCV {
    size_t n = 0;
    std::vector<T> s[4][3];
    FPCV() {}
    explicit FPCV(size_t n_) { resize(n_); }
    void resize(size_t n_) {
        n = n_;
        for (int p = 0; p < 4; p++)
            for (int k = 0; k < 3; k++) s[p][k].assign(n, (T)0);
    }
};

// the share index at which party p holds component c (c != p): FPC.inl:498-504
static inline int fpc_share_of(int p, int c) { return (3 - p + c) % 4; }
static inline int fpc_x0_share(int p) { return p == 0 ? -1 : fpc_share_of(p, 0); }

// fill (FPC.inl:120-125)
template <typename T> void fpc_fill(FPCV<T>& a, T val) {
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++) std::fill(a.s[p][k].begin(), a.s[p][k].end(), k == fpc_x0_share(p) ? val : (T)0);
}

// setPublic (FPC.inl:127-155) and the initializer list (:528-565)
template <typename T> void fpc_from_list(FPCV<T>& a, const double* vals, int fp, bool to_fixed) {
    fpc_fill<T>(a, 0);
    for (int p = 1; p < 4; p++)
        for (size_t i = 0; i < a.n; i++)
            a.s[p][fpc_x0_share(p)][i] = to_fixed ? encode_fixed<T>(vals[i], fp) : (T)(int64_t)vals[i];
}

// reconstruct (FPC.inl:611-634): shareA goes to the next party; the result is
// the own three shares plus the previous party's shareA.
template <typename T> void fpc_reconstruct(const FPCV<T>& in, Strided w, std::vector<T> (&out)[4], Comm& comm) {
    for (int p = 0; p < 4; p++) {
        int prev = (p + 3) % 4;
        out[p].resize(w.size);
        for (size_t i = 0; i < w.size; i++) {
            size_t j = w.offset + i * w.stride;
            out[p][i] = (T)(in.s[p][0][j] + in.s[p][1][j] + in.s[p][2][j] + in.s[prev][0][j]);
        }
    }
    comm.msg(4, w.size * sizeof(T), w.size * sizeof(T));
    comm.rounds++;
}

template <typename T> static FPCV<T> fpc_gather(const FPCV<T>& a, Strided w) {
    FPCV<T> r(w.size);
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < w.size; i++) r.s[p][k][i] = a.s[p][k][w.offset + i * w.stride];
    return r;
}
template <typename T> static void fpc_scatter(FPCV<T>& a, Strided w, const FPCV<T>& r) {
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < w.size; i++) a.s[p][k][w.offset + i * w.stride] = r.s[p][k][i];
}

// partyG / partyH (FPC.inl:452-496)
static inline int fpc_party_g(int i, int j) {
    static const int g[4][4] = {{-1, 2, 1, 1}, {-1, -1, 3, 2}, {-1, -1, -1, 0}, {-1, -1, -1, -1}};
    return g[i][j];
}
static inline int fpc_party_h(int i, int j) {
    static const int h[4][4] = {{-1, 3, 3, 2}, {-1, -1, 0, 0}, {-1, -1, -1, 1}, {-1, -1, -1, -1}};
    return h[i][j];
}

// reshareFPC (FPC.inl:1184-1259) of the per-party cross terms z / zPrime
// (zPrime when I and J are opposites). Parties I and J add their own term to
// the share holding component H; G adds the term I sent it; H does nothing.
template <typename T>
void fpc_reshare(const std::vector<T> (&z)[4], const std::vector<T> (&zp)[4], int I, int J, FPCV<T>& out, Comm& comm) {
    int G = fpc_party_g(I, J), H = fpc_party_h(I, J);
    bool opp = (I - J == 2) || (J - I == 2);
    size_t n = out.n;
    for (int p = 0; p < 4; p++) {
        if (p == H) continue;
        int src = p == G ? I : p;
        const std::vector<T>& mask = opp ? zp[src] : z[src];
        std::vector<T>& dst = out.s[p][fpc_share_of(p, H)];
        for (size_t i = 0; i < n; i++) dst[i] = (T)(dst[i] + mask[i]);
    }
    comm.tx[I] += n * sizeof(T);
    comm.rx[G] += n * sizeof(T);
    comm.rounds++;
}

template <typename T> static void fpc_reshare_all(const std::vector<T> (&z)[4], const std::vector<T> (&zp)[4], FPCV<T>& out,
                                                  Comm& comm) {
    static const int pairs[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    for (auto& pr : pairs) fpc_reshare<T>(z, zp, pr[0], pr[1], out, comm);
}

// FPC *= FPC (FPC.inl:322-364) and FPC &= FPC (:375-399, XOR for + and AND
// for *; the reshare still adds) on the view wa of a, with b viewed by wb.
template <typename T, bool BOOL>
void fpc_mul_like(FPCV<T>& a, Strided wa, const FPCV<T>& b, Strided wb, Comm& comm) {
    size_t n = wb.size;
    FPCV<T> self = fpc_gather(a, wa), rhs = fpc_gather(b, wb);
    auto mul = [](T x, T y) { return BOOL ? (T)(x & y) : (T)(x * y); };
    auto add = [](T x, T y) { return BOOL ? (T)(x ^ y) : (T)(x + y); };
    std::vector<T> z[4], zp[4];
    for (int p = 0; p < 4; p++) {
        z[p].resize(n);
        zp[p].resize(n);
        const auto& s = self.s[p];
        const auto& r = rhs.s[p];
        for (size_t i = 0; i < n; i++) {
            z[p][i] = add(mul(s[0][i], r[1][i]), mul(s[1][i], r[0][i]));
            zp[p][i] = add(mul(s[0][i], r[2][i]), mul(s[2][i], r[0][i]));
        }
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < n; i++) self.s[p][k][i] = mul(self.s[p][k][i], r[k][i]);
    }
    fpc_reshare_all<T>(z, zp, self, comm);
    fpc_scatter(a, wa, self);
}
template <typename T> void fpc_mul_assign(FPCV<T>& a, Strided wa, const FPCV<T>& b, Strided wb, Comm& comm) {
    fpc_mul_like<T, false>(a, wa, b, wb, comm);
}
template <typename U> void fpc_and_assign(FPCV<U>& a, Strided wa, const FPCV<U>& b, Strided wb, Comm& comm) {
    fpc_mul_like<U, true>(a, wa, b, wb, comm);
}

// FPC ^= FPC: local (FPC.inl:366-372)
template <typename U> void fpc_xor_assign(FPCV<U>& a, Strided wa, const FPCV<U>& b, Strided wb) {
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < wb.size; i++) a.s[p][k][wa.offset + i * wa.stride] ^= b.s[p][k][wb.offset + i * wb.stride];
}

// dividePublic (FPC.inl:576-608) with getDividedShares (Precompute.h:107-133):
// r = fill(1) and r' = d (scalar or per element), both in component x0.
template <typename T> void fpc_divide_public(FPCV<T>& a, const T* d, bool vec, Comm& comm) {
    for (int p = 1; p < 4; p++) {
        auto& x0 = a.s[p][fpc_x0_share(p)];
        for (size_t i = 0; i < a.n; i++) x0[i] = (T)(x0[i] - (vec ? d[i] : d[0]));  // a -= r'
    }
    std::vector<T> rec[4];
    fpc_reconstruct(a, whole(a.n), rec, comm);
    for (int p = 0; p < 4; p++) {
        for (int k = 0; k < 3; k++) std::fill(a.s[p][k].begin(), a.s[p][k].end(), (T)0);  // a.zero()
        if (p == 0) continue;  // party A holds no x0: r and the quotient do not reach it
        auto& x0 = a.s[p][fpc_x0_share(p)];
        for (size_t i = 0; i < a.n; i++) x0[i] = (T)(1 + div_public<T>(rec[p][i], vec ? d[i] : d[0]));
    }
}

// matmul (FPC.inl:636-670): diagonal products per share, cross terms into
// z = a0 b1 + a1 b0 and z' = a0 b2 + a2 b0, six reshares, dividePublic.
template <typename T>
void fpc_matmul(const FPCV<T>& a, const FPCV<T>& b, FPCV<T>& c, int M, int N, int K, bool tA, bool tB, bool tC,
                int trunc, Comm& comm) {
    size_t mn = (size_t)M * N;
    c.resize(mn);
    std::vector<T> z[4], zp[4], t(mn);
    for (int p = 0; p < 4; p++) {
        const auto& A = a.s[p];
        const auto& B = b.s[p];
        for (int k = 0; k < 3; k++) gemm<T>(M, N, K, A[k].data(), tA, B[k].data(), tB, c.s[p][k].data(), tC);
        z[p].assign(mn, 0);
        zp[p].assign(mn, 0);
        gemm<T>(M, N, K, A[0].data(), tA, B[1].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) z[p][i] = (T)(z[p][i] + t[i]);
        gemm<T>(M, N, K, A[1].data(), tA, B[0].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) z[p][i] = (T)(z[p][i] + t[i]);
        gemm<T>(M, N, K, A[0].data(), tA, B[2].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) zp[p][i] = (T)(zp[p][i] + t[i]);
        gemm<T>(M, N, K, A[2].data(), tA, B[0].data(), tB, t.data(), tC);
        for (size_t i = 0; i < mn; i++) zp[p][i] = (T)(zp[p][i] + t[i]);
    }
    fpc_reshare_all<T>(z, zp, c, comm);
    T d = (T)((T)1 << trunc);
    fpc_divide_public(c, &d, false, comm);
}

// convolution (FPC.inl:862-925) with localFprop/Dgrad/Wgrad (:745-860).
template <typename T>
void fpc_convolution(const FPCV<T>& A, const FPCV<T>& B, FPCV<T>& C, int op, int batch, int H, int W, int f,
                     int Din, int Dout, int stride, int pad, int trunc, Comm& comm) {
    ConvShape sh{batch, H, W, Din, Dout, f, f, pad, stride};
    size_t out_n = op == CONV_FPROP ? (size_t)batch * sh.P() * sh.Q() * Dout
                 : op == CONV_DGRAD ? (size_t)batch * H * W * Din
                                    : (size_t)Dout * f * f * Din;
    C.resize(out_n);
    std::vector<T> z[4], zp[4], t(out_n);
    for (int p = 0; p < 4; p++) {
        const auto& a = A.s[p];
        const auto& b = B.s[p];
        for (int k = 0; k < 3; k++) conv_any<T>(op, sh, a[k].data(), b[k].data(), C.s[p][k].data());
        z[p].assign(out_n, 0);
        zp[p].assign(out_n, 0);
        conv_any<T>(op, sh, a[0].data(), b[1].data(), t.data());
        for (size_t i = 0; i < out_n; i++) z[p][i] = (T)(z[p][i] + t[i]);
        conv_any<T>(op, sh, a[1].data(), b[0].data(), t.data());
        for (size_t i = 0; i < out_n; i++) z[p][i] = (T)(z[p][i] + t[i]);
        conv_any<T>(op, sh, a[0].data(), b[2].data(), t.data());
        for (size_t i = 0; i < out_n; i++) zp[p][i] = (T)(zp[p][i] + t[i]);
        conv_any<T>(op, sh, a[2].data(), b[0].data(), t.data());
        for (size_t i = 0; i < out_n; i++) zp[p][i] = (T)(zp[p][i] + t[i]);
    }
    fpc_reshare_all<T>(z, zp, C, comm);
    T d = (T)((T)1 << trunc);
    fpc_divide_public(C, &d, false, comm);
}

// carryOut (FPC.inl:1297-1416): the same tree with FPC ANDs.
template <typename U> void fpc_carry_out(FPCV<U>& p, FPCV<U>& g, int k, FPCV<U>& out, Comm& comm) {
    size_t N = p.n;
    size_t stride = 2, offset = 1;
    Strided pEven = strided(N, 0, stride), pOdd = strided(N, offset, stride);
    Strided gEven = strided(N, 0, stride), gOdd = strided(N, offset, stride);
    while (k > 1) {
        fpc_and_assign(g, gEven, p, pOdd, comm);
        fpc_and_assign(p, pEven, p, pOdd, comm);
        fpc_xor_assign(g, gOdd, g, gEven);
        gEven = strided(N, offset, stride * 2);
        offset += stride;
        gOdd = strided(N, offset, stride * 2);
        stride *= 2;
        pEven = strided(N, 0, stride);
        pOdd = strided(N, stride / 2, stride);
        k /= 2;
    }
    Strided oE = strided(out.n, 0, 2), oO = strided(out.n, 1, 2);
    for (int q = 0; q < 4; q++)
        for (int s = 0; s < 3; s++) {
            for (size_t i = 0; i < gEven.size && i < oE.size; i++)
                out.s[q][s][oE.offset + i * 2] = g.s[q][s][gEven.offset + i * gEven.stride];
            for (size_t i = 0; i < gOdd.size && i < oO.size; i++)
                out.s[q][s][oO.offset + i * 2] = g.s[q][s][gOdd.offset + i * gOdd.stride];
        }
}

// dReLU (FPC.inl:930-990)
template <typename T, typename U> void fpc_drelu(const FPCV<T>& in, Strided w, FPCV<U>& result, Comm& comm) {
    const int W = sizeof(T) * 8;
    size_t n = w.size;
    FPCV<U> rbits(n * W);
    fpc_fill<U>(rbits, 1);
    std::vector<T> a[4];
    fpc_reconstruct(in, w, a, comm);  // r = 0; r += input; reconstruct(r, a)
    std::vector<U> abits[4];
    FPCV<U> msb(n);
    for (int p = 0; p < 4; p++) {
        for (auto& x : a[p]) x = (T)(x + 1);
        bitexpand<T, U>(a[p], abits[p]);
        int x0 = fpc_x0_share(p);
        for (size_t i = 0; i < n; i++) {
            size_t bi = i * W + (W - 1);
            for (int k = 0; k < 3; k++) {
                msb.s[p][k][i] = rbits.s[p][k][bi];                 // getMSBs of every share
                if (k == x0) msb.s[p][k][i] ^= abits[p][bi];        // msb ^= abits_msb: x0 only
                rbits.s[p][k][bi] = 0;                              // setMSBs(rbits, 0)
            }
            abits[p][bi] = 1;                                       // setMSBs(abits, 1)
        }
    }
    FPCV<U> g(n * W), pp(n * W);
    for (int p = 0; p < 4; p++) {
        int x0 = fpc_x0_share(p);
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < n * W; i++) {
                g.s[p][k][i] = rbits.s[p][k][i] & abits[p][i];                        // &= DeviceData: all shares
                pp.s[p][k][i] = rbits.s[p][k][i] ^ (k == x0 ? abits[p][i] : (U)0);  // ^= DeviceData: x0
            }
    }
    FPCV<U> pre(n);
    fpc_carry_out(pp, g, W, pre, comm);
    fpc_xor_assign(pre, whole(n), msb, whole(n));
    result.resize(n);
    fpc_fill<U>(result, 1);
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < n; i++) result.s[p][k][i] = (U)(result.s[p][k][i] - pre.s[p][k][i]);
}

// selectShare (FPC.inl:672-711) with convex_comb (:1528-1541, functor :31-66):
// c = 0, so d holds 1 in component x0 where the party's opened e is 1.
template <typename T, typename U>
void fpc_select_share(const FPCV<T>& x, Strided wx, const FPCV<T>& y, Strided wy, const FPCV<U>& b, FPCV<T>& z,
                      Strided wz, Comm& comm) {
    size_t n = wx.size;
    std::vector<U> e[4];
    fpc_reconstruct(b, whole(b.n), e, comm);  // cbits = 0 ^ b
    FPCV<T> d(n);
    for (int p = 1; p < 4; p++) {
        int x0 = fpc_x0_share(p);
        for (size_t i = 0; i < n; i++) d.s[p][x0][i] = e[p][i] == 1 ? (T)1 : (T)0;
    }
    FPCV<T> res(n);
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < n; i++)
                res.s[p][k][i] = (T)(y.s[p][k][wy.offset + i * wy.stride] - x.s[p][k][wx.offset + i * wx.stride]);
    fpc_mul_assign(res, whole(n), d, whole(n), comm);
    for (int p = 0; p < 4; p++)
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < n; i++)
                z.s[p][k][wz.offset + i * wz.stride] = (T)(res.s[p][k][i] + x.s[p][k][wx.offset + i * wx.stride]);
}

// ReLU (FPC.inl:992-1003)
template <typename T, typename U> void fpc_relu(const FPCV<T>& in, FPCV<T>& out, FPCV<U>& dout, Comm& comm) {
    fpc_drelu<T, U>(in, whole(in.n), dout, comm);
    FPCV<T> zeros(in.n);
    out.resize(in.n);
    fpc_select_share<T, U>(zeros, whole(in.n), in, whole(in.n), dout, out, whole(in.n), comm);
}

// maxpool (FPC.inl:1005-1177)
template <typename T, typename U>
void fpc_maxpool(FPCV<T>& input, FPCV<T>& result, FPCV<U>& dresult, int k, Comm& comm) {
    size_t N = input.n;
    dresult.resize(N);
    fpc_fill<U>(dresult, 1);
    size_t stride = 2;
    Strided even = strided(N, 0, stride), odd = strided(N, 1, stride);
    auto level = [&](bool last) {
        FPCV<T> diff(even.size);
        for (int p = 0; p < 4; p++)
            for (int s = 0; s < 3; s++)
                for (size_t i = 0; i < even.size; i++)
                    diff.s[p][s][i] = (T)(input.s[p][s][even.offset + i * even.stride] -
                                          input.s[p][s][odd.offset + i * odd.stride]);
        FPCV<U> b(even.size);
        fpc_drelu<T, U>(diff, whole(diff.n), b, comm);
        fpc_select_share<T, U>(input, odd, input, even, b, input, even, comm);
        if (!last) {
            stride *= 2;
            even = strided(N, 0, stride);
            odd = strided(N, stride / 2, stride);
        } else {
            result.resize(even.size);
            for (int p = 0; p < 4; p++)
                for (int s = 0; s < 3; s++)
                    for (size_t i = 0; i < even.size; i++) result.s[p][s][i] = input.s[p][s][even.offset + i * even.stride];
        }
        FPCV<U> neg(b.n);
        fpc_fill<U>(neg, 1);
        for (int p = 0; p < 4; p++)
            for (int s = 0; s < 3; s++)
                for (size_t i = 0; i < b.n; i++) neg.s[p][s][i] = (U)(neg.s[p][s][i] - b.s[p][s][i]);
        FPCV<U> expanded(N);
        for (int p = 0; p < 4; p++)
            for (int s = 0; s < 3; s++) expand_compare<U>(b.s[p][s], neg.s[p][s], expanded.s[p][s]);
        fpc_and_assign(dresult, whole(N), expanded, whole(N), comm);
    };
    while (k > 2) {
        level(false);
        k /= 2;
    }
    level(true);
}

}  // namespace oracle
