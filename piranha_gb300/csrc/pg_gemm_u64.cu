// pg_gemm_u64.cu — the plain 64/32-bit integer CUDA-core form of the ring
// GEMM and implicit-GEMM convolutions, with the RSS truncation epilogue.
//
// One kernel covers gpu::gemm (src/gpu/gemm.cuh:64-112), gpu::conv_fprop /
// conv_dgrad / conv_wgrad (src/gpu/conv.cuh:359-490) and, through K
// segments, RSS localMatMul (src/mpc/RSS.inl:1097-1110) and
// localFprop/Dgrad/Wgrad (:614-703): for the three simulated parties the six
// segments are [x_p0 | x_p1] x [y_p0 + y_p1 ; y_p0], so one contraction over
// the concatenated K accumulates sum_p z_p, which is exactly what
// reconstruct3out3 (:1020-1050) reveals. The epilogue then applies
// dividePublic3out3 (:1077-1094) and writes all six output shares (plus the
// FC bias shares of FCLayer.cu:110-116 when given).
#include <mutex>

#include "pg_common.cuh"

namespace pg {

enum GemmKind { K_GEMM = 0, K_FPROP = 1, K_DGRAD = 2, K_WGRAD = 3 };
enum Epi { EPI_RAW = 0, EPI_RSS = 1, EPI_FPC = 2 };

// unsigned 32-bit division by a runtime constant (round-up multiply-high)
struct FastDiv {
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

constexpr int kMaxSeg = 12;

template <typename T> struct GemmArgs {
    int M, N, K;  // K per segment
    int nseg;
    const T *a[kMaxSeg];
    const T *b0[kMaxSeg];
    const T *b1[kMaxSeg];  // added to b0 when not null (the same pointer twice doubles it)
    int tA, tB, tC;
    // conv geometry
    int cn, ch, cw, cc, ck, cr, cs, cp, cq, pad, stride;
    FastDiv dQ, dP, dW, dH, dC, dS, dK, dRSC;
    // epilogue
    int epi;
    T *c_raw;
    T *out[6];
    const T *bias[6];
    T d;
    int dshift;
    int x0;  // EPI_FPC: the output share that holds component x0 (-1: none)
    // split-K: CTA z runs k-steps [z * steps_per_split, (z + 1) * steps_per_split) of the
    // concatenated (segment, k) range and adds its sums into partial (mod 2^w, exact);
    // ring_epilogue_kernel then applies the epilogue. partial == nullptr: no split.
    T *partial;
    int steps_per_split;
};

constexpr int BK = 8, NT = 256;
constexpr int APAD = 2, BPAD = 2;

// CTA tile shapes: BM x BN outputs, TM x TN per thread, (BM/TM) x (BN/TN) = NT
// threads. Wide is the default; Thin serves narrow outputs (N <= 8: the input
// gradient of a convolution with few input channels), Small serves small
// M x N with a long K (weight gradients), where a 128 x 64 tile would be
// mostly idle. Col serves a single output column (the input gradient of a
// convolution over one-channel images), one output per thread.
template <int BM_, int BN_, int TM_, int TN_> struct Tile {
    static constexpr int BM = BM_, BN = BN_, TM = TM_, TN = TN_;
    static_assert((BM / TM) * (BN / TN) == NT, "one output block per thread");
};
using Wide = Tile<128, 64, 8, 4>;
using Thin = Tile<128, 8, 4, 1>;
using Small = Tile<32, 32, 2, 2>;
using Col = Tile<256, 1, 1, 1>;

// Which index of a loaded element varies fastest across threads.
template <int KIND> struct Layout {
    // A: true = m-fastest (M-contiguous operand), false = k-fastest
    static __device__ __forceinline__ bool a_mfast(const void *) { return KIND == K_WGRAD; }
};

template <typename T, int KIND> struct Loader {
    // A[m][k] of segment s
    static __device__ __forceinline__ T load_a(const GemmArgs<T> &g, const T *a, int m, int k) {
        if (m >= g.M || k >= g.K) return 0;
        if (KIND == K_GEMM) {
            return g.tA ? a[(size_t)m * g.K + k] : a[(size_t)m + (size_t)k * g.M];
        } else if (KIND == K_FPROP) {
            // m = (n, p, q); k = (r, s, c)
            uint32_t nq = g.dQ.div(m), q = m - nq * g.cq;
            uint32_t n = g.dP.div(nq), p = nq - n * g.cp;
            uint32_t rs = g.dC.div(k), c = k - rs * g.cc;
            uint32_t r = g.dS.div(rs), s = rs - r * g.cs;
            int h = (int)(p * g.stride) - g.pad + (int)r, w = (int)(q * g.stride) - g.pad + (int)s;
            if (h < 0 || h >= g.ch || w < 0 || w >= g.cw) return 0;
            return a[(((size_t)n * g.ch + h) * g.cw + w) * g.cc + c];
        } else if (KIND == K_DGRAD) {
            // m = (n, h, w); k = (r, s, kk); value dY[n][p][q][kk] with h = p*st - pad + r
            uint32_t nh = g.dW.div(m), w = m - nh * g.cw;
            uint32_t n = g.dH.div(nh), h = nh - n * g.ch;
            uint32_t rs = g.dK.div(k), kk = k - rs * g.ck;
            uint32_t r = g.dS.div(rs), s = rs - r * g.cs;
            int ph = (int)h + g.pad - (int)r, qw = (int)w + g.pad - (int)s;
            if (ph < 0 || qw < 0 || ph % g.stride || qw % g.stride) return 0;
            int p = ph / g.stride, q = qw / g.stride;
            if (p >= g.cp || q >= g.cq) return 0;
            return a[(((size_t)n * g.cp + p) * g.cq + q) * g.ck + kk];
        } else {  // K_WGRAD: m = kk, k = (n, p, q): dY[k][m]
            return a[(size_t)k * g.ck + m];
        }
    }
    static __device__ __forceinline__ T load_b1(const GemmArgs<T> &g, const T *b, int k, int n) {
        if (KIND == K_GEMM) {
            return g.tB ? b[(size_t)k * g.N + n] : b[(size_t)k + (size_t)n * g.K];
        } else if (KIND == K_FPROP) {
            return b[(size_t)n * g.K + k];  // F[co][r][s][c], k = (r,s,c)
        } else if (KIND == K_DGRAD) {
            uint32_t rs = g.dK.div(k), kk = k - rs * g.ck;  // k = (r, s, kk), n = c
            return b[((size_t)kk * g.cr * g.cs + rs) * g.cc + n];
        } else {  // K_WGRAD: k = (n, p, q), n_out = (r, s, c): X[n][p*st-pad+r][q*st-pad+s][c]
            uint32_t nq = g.dQ.div(k), q = k - nq * g.cq;
            uint32_t nn = g.dP.div(nq), p = nq - nn * g.cp;
            uint32_t rs = g.dC.div(n), c = n - rs * g.cc;
            uint32_t r = g.dS.div(rs), s = rs - r * g.cs;
            int h = (int)(p * g.stride) - g.pad + (int)r, w = (int)(q * g.stride) - g.pad + (int)s;
            if (h < 0 || h >= g.ch || w < 0 || w >= g.cw) return 0;
            return b[(((size_t)nn * g.ch + h) * g.cw + w) * g.cc + c];
        }
    }
    static __device__ __forceinline__ T load_b(const GemmArgs<T> &g, int seg, int k, int n) {
        if (k >= g.K || n >= g.N) return 0;
        T v = load_b1(g, g.b0[seg], k, n);
        if (g.b1[seg]) v = (T)(v + load_b1(g, g.b1[seg], k, n));
        return v;
    }
    // B k-fastest for K-contiguous B operands
    static constexpr bool b_kfast = (KIND == K_FPROP);
};

template <int KIND, typename T> __device__ __forceinline__ size_t out_index(const GemmArgs<T> &g, int m, int n) {
    return (KIND == K_GEMM && !g.tC) ? (size_t)m + (size_t)n * g.M : (size_t)m * g.N + n;
}

__device__ __forceinline__ void atomic_add_ring(uint64_t *p, uint64_t v) {
    atomicAdd((unsigned long long *)p, (unsigned long long)v);
}
__device__ __forceinline__ void atomic_add_ring(uint32_t *p, uint32_t v) { atomicAdd((unsigned int *)p, v); }

// Output of one ring element z of the contraction at output index idx, column n.
template <typename T> __device__ __forceinline__ void apply_epilogue(const GemmArgs<T> &g, size_t idx, int n, T z) {
    if (g.epi == EPI_RAW) {
        g.c_raw[idx] = z;
    } else if (g.epi == EPI_FPC) {
        // FPC dividePublic at one party: its reveal minus d, divided, plus r = 1 in x0
        T v = (T)(1 + div_public<T>((T)(z - g.d), g.d, g.dshift));
#pragma unroll
        for (int ps = 0; ps < 3; ps++) {
            T base = ps == g.x0 ? v : (T)0;
            if (g.bias[ps]) base = (T)(base + g.bias[ps][n]);
            g.out[ps][idx] = base;
        }
    } else {
        // dividePublic3out3: reveal sum_p z_p - d, divide, r = 1 at A.shareA / C.shareB
        T v = (T)(1 + div_public<T>((T)(z - g.d), g.d, g.dshift));
#pragma unroll
        for (int ps = 0; ps < 6; ps++) {
            T base = (ps == 0 || ps == 5) ? v : (T)0;
            if (g.bias[ps]) base = (T)(base + g.bias[ps][n]);
            g.out[ps][idx] = base;
        }
    }
}

template <typename T, int KIND, class TL>
__global__ void __launch_bounds__(NT, 2) ring_gemm_kernel(const GemmArgs<T> g) {
    constexpr int BM = TL::BM, BN = TL::BN, TM = TL::TM, TN = TL::TN;
    constexpr int NA = (BM * BK + NT - 1) / NT, NB = (BN * BK + NT - 1) / NT;  // loads per thread
    __shared__ T As[2][BK][BM + APAD];
    __shared__ T Bs[2][BK][BN + BPAD];
    using L = Loader<T, KIND>;
    const int tid = threadIdx.x;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const bool a_mfast = (KIND == K_WGRAD) || (KIND == K_GEMM && !g.tA);
    const bool b_kfast = (KIND == K_FPROP) || (KIND == K_GEMM && !g.tB);

    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = 0;

    T ra[NA], rb[NB];
    const int ksteps = (g.K + BK - 1) / BK;
    const int all_steps = ksteps * g.nseg;
    const int first = g.partial ? (int)blockIdx.z * g.steps_per_split : 0;
    const int last = g.partial ? min(all_steps, first + g.steps_per_split) : all_steps;
    const int total = last > first ? last - first : 0;

    auto gload = [&](int local_step) {
        const int step = first + local_step;
        int seg = step / ksteps, k0 = (step - seg * ksteps) * BK;
        const T *a = g.a[seg];
#pragma unroll
        for (int i = 0; i < NA; i++) {
            int e = tid + i * NT;
            if (NA * NT > BM * BK && e >= BM * BK) break;
            int mm = a_mfast ? (e % BM) : (e / BK), kk = a_mfast ? (e / BM) : (e % BK);
            ra[i] = L::load_a(g, a, m0 + mm, k0 + kk);
        }
#pragma unroll
        for (int i = 0; i < NB; i++) {
            int e = tid + i * NT;
            if (NB * NT > BN * BK && e >= BN * BK) break;
            int kk = b_kfast ? (e % BK) : (e / BN), nn = b_kfast ? (e / BK) : (e % BN);
            rb[i] = L::load_b(g, seg, k0 + kk, n0 + nn);
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int i = 0; i < NA; i++) {
            int e = tid + i * NT;
            if (NA * NT > BM * BK && e >= BM * BK) break;
            int mm = a_mfast ? (e % BM) : (e / BK), kk = a_mfast ? (e / BM) : (e % BK);
            As[buf][kk][mm] = ra[i];
        }
#pragma unroll
        for (int i = 0; i < NB; i++) {
            int e = tid + i * NT;
            if (NB * NT > BN * BK && e >= BN * BK) break;
            int kk = b_kfast ? (e % BK) : (e / BN), nn = b_kfast ? (e / BK) : (e % BN);
            Bs[buf][kk][nn] = rb[i];
        }
    };

    const int tm = tid / (BN / TN), tn = tid % (BN / TN);
    if (total > 0) {
        gload(0);
        sstore(0);
    }
    __syncthreads();
    for (int step = 0; step < total; step++) {
        int buf = step & 1;
        if (step + 1 < total) gload(step + 1);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            T av[TM], bv[TN];
#pragma unroll
            for (int i = 0; i < TM; i++) av[i] = As[buf][kk][tm * TM + i];
#pragma unroll
            for (int j = 0; j < TN; j++) bv[j] = Bs[buf][kk][tn * TN + j];
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = (T)(acc[i][j] + av[i] * bv[j]);
        }
        if (step + 1 < total) sstore(buf ^ 1);
        __syncthreads();
    }

    // epilogue
#pragma unroll
    for (int i = 0; i < TM; i++) {
        int m = m0 + tm * TM + i;
        if (m >= g.M) continue;
#pragma unroll
        for (int j = 0; j < TN; j++) {
            int n = n0 + tn * TN + j;
            if (n >= g.N) continue;
            const size_t idx = out_index<KIND>(g, m, n);
            if (g.partial) atomic_add_ring(&g.partial[idx], acc[i][j]);
            else apply_epilogue(g, idx, n, acc[i][j]);
        }
    }
}

// The epilogue of split-K GEMMs, after all splits have added into partial.
template <typename T, int KIND> __global__ void ring_epilogue_kernel(const GemmArgs<T> g) {
    const size_t mn = (size_t)g.M * g.N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < mn; e += (size_t)gridDim.x * blockDim.x) {
        const int m = (int)(e / g.N), n = (int)(e - (size_t)m * g.N);
        const size_t idx = out_index<KIND>(g, m, n);
        apply_epilogue(g, idx, n, g.partial[idx]);
    }
}

// Weight gradients with few outputs and a long K (LeNet's first
// convolution: 20 filters x 25 taps over 128 x 24 x 24 output pixels): each
// thread owns a 4 x 4 block of (filter, tap) outputs and one of `phases`
// interleaved slices of the CTA's (segment, pixel) range, with the input
// offsets of its four taps fixed for the whole run, so the gather costs one
// add and a bounds test per value. The CTA's phases are summed in shared
// memory and added into the split-K partial sums with one 64/32-bit atomic
// per output (exact mod 2^w); ring_epilogue_kernel then applies the
// epilogue. A = dY[k][m] (m = filter), B = X gathered at tap n = (r, s, c).
constexpr int WS_OB = 4, WS_TB = 4, WS_THREADS = 256;

template <typename T>
__global__ void __launch_bounds__(WS_THREADS, 2) wgrad_small_kernel(const GemmArgs<T> g, int phases, long long per_cta) {
    __shared__ T red[WS_THREADS][WS_OB * WS_TB + 1];
    const int ob_n = (g.M + WS_OB - 1) / WS_OB, tb_n = (g.N + WS_TB - 1) / WS_TB;
    const int lbs = ob_n * tb_n;
    const int tid = threadIdx.x;
    const int lb = tid % lbs, phase = tid / lbs;
    const int o0 = (lb / tb_n) * WS_OB, t0 = (lb % tb_n) * WS_TB;
    T acc[WS_OB][WS_TB];
#pragma unroll
    for (int i = 0; i < WS_OB; i++)
#pragma unroll
        for (int j = 0; j < WS_TB; j++) acc[i][j] = 0;
    if (phase < phases) {
        // this thread's taps: input offset relative to the output pixel's corner, and (r, s) for the bounds
        int toff[WS_TB];
        int tr[WS_TB], ts[WS_TB];
        bool tval[WS_TB];
#pragma unroll
        for (int j = 0; j < WS_TB; j++) {
            const int t = t0 + j;
            tval[j] = t < g.N;
            const int tt = tval[j] ? t : 0;
            const int rs = tt / g.cc, c = tt - rs * g.cc;
            tr[j] = rs / g.cs - g.pad;
            ts[j] = rs % g.cs - g.pad;
            toff[j] = (tr[j] * g.cw + ts[j]) * g.cc + c;
        }
        const long long ksz = g.K;
        const long long begin = (long long)blockIdx.x * per_cta;
        long long end = begin + per_cta;
        const long long all = ksz * g.nseg;
        if (end > all) end = all;
        for (int seg = (int)(begin / ksz); seg < g.nseg && (long long)seg * ksz < end; seg++) {
        const long long s0 = (long long)seg * ksz;
        const uint32_t klo = (uint32_t)((begin > s0 ? begin : s0) - s0);
        const uint32_t khi = (uint32_t)((end < s0 + ksz ? end : s0 + ksz) - s0);
        const T *a = g.a[seg], *b0 = g.b0[seg], *b1 = g.b1[seg];
        // the operands of output pixel k (dY row, gathered taps); two pixels per
        // iteration, all loads issued before either block of multiply-adds
        auto load = [&](uint32_t k, T (&av)[WS_OB], T (&bv)[WS_TB]) {
            const uint32_t nq = g.dQ.div(k), q = k - nq * g.cq;
            const uint32_t n = g.dP.div(nq), p = nq - n * g.cp;
            const int hb = (int)p * g.stride, wb = (int)q * g.stride;
            const long long base = (((long long)n * g.ch + hb) * g.cw + wb) * g.cc;
#pragma unroll
            for (int i = 0; i < WS_OB; i++) av[i] = o0 + i < g.M ? __ldg(a + (size_t)k * g.ck + o0 + i) : (T)0;
#pragma unroll
            for (int j = 0; j < WS_TB; j++) {
                const int h = hb + tr[j], w = wb + ts[j];
                T v = 0;
                if (tval[j] && h >= 0 && h < g.ch && w >= 0 && w < g.cw) {
                    v = __ldg(b0 + base + toff[j]);
                    if (b1) v = (T)(v + __ldg(b1 + base + toff[j]));
                }
                bv[j] = v;
            }
        };
        auto mac = [&](const T (&av)[WS_OB], const T (&bv)[WS_TB]) {
#pragma unroll
            for (int i = 0; i < WS_OB; i++)
#pragma unroll
                for (int j = 0; j < WS_TB; j++) acc[i][j] = (T)(acc[i][j] + av[i] * bv[j]);
        };
        uint32_t k = klo + (uint32_t)phase;
        for (; k + (uint32_t)phases < khi; k += 2u * (uint32_t)phases) {
            T av0[WS_OB], bv0[WS_TB], av1[WS_OB], bv1[WS_TB];
            load(k, av0, bv0);
            load(k + (uint32_t)phases, av1, bv1);
            mac(av0, bv0);
            mac(av1, bv1);
        }
        if (k < khi) {
            T av0[WS_OB], bv0[WS_TB];
            load(k, av0, bv0);
            mac(av0, bv0);
        }
        }
    }
#pragma unroll
    for (int i = 0; i < WS_OB; i++)
#pragma unroll
        for (int j = 0; j < WS_TB; j++) red[tid][i * WS_TB + j] = acc[i][j];
    __syncthreads();
    // thread e < lbs * 16 sums output e % 16 of lane block e / 16 over the phases
    for (int e = tid; e < lbs * WS_OB * WS_TB; e += WS_THREADS) {
        const int blk = e / (WS_OB * WS_TB), w = e - blk * (WS_OB * WS_TB);
        const int m = (blk / tb_n) * WS_OB + w / WS_TB, nn = (blk % tb_n) * WS_TB + w % WS_TB;
        if (m >= g.M || nn >= g.N) continue;
        T sum = 0;
        for (int ph = 0; ph < phases; ph++) sum = (T)(sum + red[ph * lbs + blk][w]);
        atomic_add_ring(&g.partial[out_index<K_WGRAD>(g, m, nn)], sum);
    }
}

// The same weight gradients, staged through shared memory by output row:
// each phase of the CTA takes one output row (segment, image n, row p) at a
// time and its threads copy the row's dY values (Q x Dout) and the f input
// rows it touches (zero-padded to W + 2 pad columns, b0 + b1 summed) into the
// phase's slice of shared memory; then every thread runs its 4 x 4 block of
// (filter, tap) outputs over the row's Q pixels with pointer increments only.
// Phases run their rows independently (one named barrier each).
template <typename T>
__global__ void __launch_bounds__(WS_THREADS, 2) wgrad_rows_kernel(const GemmArgs<T> g, int phases, int rows_per_cta, int rpr) {
    extern __shared__ __align__(16) unsigned char ws_smem[];
    T *sm = reinterpret_cast<T *>(ws_smem);
    const int ob_n = (g.M + WS_OB - 1) / WS_OB, tb_n = (g.N + WS_TB - 1) / WS_TB;
    const int lbs = ob_n * tb_n;
    const int tid = threadIdx.x;
    const int lb = tid % lbs, phase = tid / lbs;
    const int o0 = (lb / tb_n) * WS_OB, t0 = (lb % tb_n) * WS_TB;
    const int Wp = g.cw + 2 * g.pad;                 // staged input row length in pixels
    const int xrow = Wp * g.cc;                      // values per staged input row
    const int dy_vals = g.cq * g.ck, x_vals = g.cr * xrow;
    const int slice = dy_vals + x_vals;
    T acc[WS_OB][WS_TB];
#pragma unroll
    for (int i = 0; i < WS_OB; i++)
#pragma unroll
        for (int j = 0; j < WS_TB; j++) acc[i][j] = 0;
    const bool active = phase < phases;
    T *const slices = sm + (size_t)(active ? phase : 0) * rpr * slice;  // this phase's rpr row slices
    // this thread's taps inside the staged rows
    int toff[WS_TB];
#pragma unroll
    for (int j = 0; j < WS_TB; j++) {
        const int t = t0 + j < g.N ? t0 + j : 0;
        const int rs = t / g.cc, c = t - rs * g.cc;
        toff[j] = (rs / g.cs) * xrow + (rs % g.cs) * g.cc + c;
    }
    const int pt = phase * lbs;  // first thread of the phase
    const long long per_img = (long long)g.cn * g.cp;
    const long long rows = (long long)g.nseg * per_img;
    const long long r0 = (long long)blockIdx.x * rows_per_cta;
    // every thread runs the same number of rounds (rpr rows per phase each,
    // staged together so their loads overlap), so the two CTA-wide barriers of
    // a round are reached by all threads
    const int per_round = phases * rpr;
    const int rounds = (rows_per_cta + per_round - 1) / per_round;
    for (int rnd = 0; rnd < rounds; rnd++) {
      for (int ri = 0; ri < rpr; ri++) {
        const long long row = r0 + ((long long)rnd * phases + phase) * rpr + ri;
        const bool have = active && row < r0 + rows_per_cta && row < rows;
        T *dys = slices + (size_t)ri * slice, *xs = dys + dy_vals;
        const T *a = nullptr;
        if (have) {
            const int seg = (int)(row / per_img);
            const int np = (int)(row - (long long)seg * per_img);
            const int n = np / g.cp, p = np - n * g.cp;
            a = g.a[seg];
            const T *b0 = g.b0[seg], *b1 = g.b1[seg];
            // stage dY[n][p][*][*] and the input rows p*stride - pad + r, r < f
            const T *dyg = a + ((size_t)n * g.cp + p) * g.cq * g.ck;
#pragma unroll 4
            for (int e = tid - pt; e < dy_vals; e += lbs) dys[e] = dyg[e];
#pragma unroll 4
            for (int e = tid - pt; e < x_vals; e += lbs) {
                const int r = e / xrow, rem = e - r * xrow;
                const int wp = rem / g.cc, c = rem - wp * g.cc;
                const int h = p * g.stride - g.pad + r, w = wp - g.pad;
                T v = 0;
                if (h >= 0 && h < g.ch && w >= 0 && w < g.cw) {
                    const size_t idx = (((size_t)n * g.ch + h) * g.cw + w) * g.cc + c;
                    v = b0[idx];
                    if (b1) v = (T)(v + b1[idx]);
                }
                xs[e] = v;
            }
        }
      }
        __syncthreads();
      for (int ri = 0; ri < rpr; ri++) {
        const long long row = r0 + ((long long)rnd * phases + phase) * rpr + ri;
        const int q_n = active && row < r0 + rows_per_cta && row < rows ? g.cq : 0;
        const T *dys = slices + (size_t)ri * slice, *xs = dys + dy_vals;
        const T *dp = dys + o0, *xp = xs;
        const int xstep = g.stride * g.cc;
        for (int q = 0; q < q_n; q++, dp += g.ck, xp += xstep) {
            T av[WS_OB], bv[WS_TB];
#pragma unroll
            for (int i = 0; i < WS_OB; i++) av[i] = o0 + i < g.M ? dp[i] : (T)0;
#pragma unroll
            for (int j = 0; j < WS_TB; j++) bv[j] = t0 + j < g.N ? xp[toff[j]] : (T)0;
#pragma unroll
            for (int i = 0; i < WS_OB; i++)
#pragma unroll
                for (int j = 0; j < WS_TB; j++) acc[i][j] = (T)(acc[i][j] + av[i] * bv[j]);
        }
      }
        __syncthreads();
    }
    __syncthreads();
    T (*red)[WS_OB * WS_TB + 1] = reinterpret_cast<T (*)[WS_OB * WS_TB + 1]>(sm);
#pragma unroll
    for (int i = 0; i < WS_OB; i++)
#pragma unroll
        for (int j = 0; j < WS_TB; j++) red[tid][i * WS_TB + j] = acc[i][j];
    __syncthreads();
    for (int e = tid; e < lbs * WS_OB * WS_TB; e += WS_THREADS) {
        const int blk = e / (WS_OB * WS_TB), w = e - blk * (WS_OB * WS_TB);
        const int m = (blk / tb_n) * WS_OB + w / WS_TB, nn = (blk % tb_n) * WS_TB + w % WS_TB;
        if (m >= g.M || nn >= g.N) continue;
        T sum = 0;
        for (int ph = 0; ph < phases; ph++) sum = (T)(sum + red[ph * lbs + blk][w]);
        atomic_add_ring(&g.partial[out_index<K_WGRAD>(g, m, nn)], sum);
    }
}

// whether wgrad_small_kernel serves a weight gradient: at least two phases
// of lane blocks per CTA and a K long enough to spread over the GPU
template <typename T> static bool wgrad_small_applies(const GemmArgs<T> &g) {
    const long long lbs = (long long)((g.M + WS_OB - 1) / WS_OB) * ((g.N + WS_TB - 1) / WS_TB);
    return 2 * lbs <= WS_THREADS && (long long)g.K * g.nseg >= 16384 && g.K < (1LL << 31);
}

template <typename T> static void setup_conv(GemmArgs<T> &g, int op, int N, int H, int W, int C, int K, int R,
                                            int S, int pad, int stride) {
    int P = (H + 2 * pad - R) / stride + 1, Q = (W + 2 * pad - S) / stride + 1;
    g.cn = N; g.ch = H; g.cw = W; g.cc = C; g.ck = K; g.cr = R; g.cs = S; g.cp = P; g.cq = Q;
    g.pad = pad; g.stride = stride;
    g.dQ.init(Q); g.dP.init(P); g.dW.init(W); g.dH.init(H); g.dC.init(C); g.dS.init(S); g.dK.init(K);
    g.dRSC.init(R * S * C);
    if (op == PG_CONV_FPROP) { g.M = N * P * Q; g.N = K; g.K = R * S * C; }
    else if (op == PG_CONV_DGRAD) { g.M = N * H * W; g.N = C; g.K = R * S * K; }
    else { g.M = K; g.N = R * S * C; g.K = N * P * Q; }
}

template <typename T, int KIND, class TL> static void launch_kind(Ctx *c, dim3 grid, const GemmArgs<T> &g) {
    ring_gemm_kernel<T, KIND, TL><<<grid, NT, 0, c->stream>>>(g);
    if (g.partial) {
        const size_t mn = (size_t)g.M * g.N;
        const int sms = c->sm_count > 0 ? c->sm_count : 148;
        size_t blocks = (mn + 255) / 256;
        if (blocks > (size_t)sms * 8) blocks = (size_t)sms * 8;
        ring_epilogue_kernel<T, KIND><<<(unsigned)blocks, 256, 0, c->stream>>>(g);
    }
}

template <typename T, class TL> static void launch_tile(Ctx *c, dim3 grid, const GemmArgs<T> &g, int kind) {
    switch (kind) {
        case K_GEMM: launch_kind<T, K_GEMM, TL>(c, grid, g); break;
        case K_FPROP: launch_kind<T, K_FPROP, TL>(c, grid, g); break;
        case K_DGRAD: launch_kind<T, K_DGRAD, TL>(c, grid, g); break;
        default: launch_kind<T, K_WGRAD, TL>(c, grid, g); break;
    }
}

template <typename T> static int launch_gemm(Ctx *c, GemmArgs<T> &g, int kind) {
    if (g.M <= 0 || g.N <= 0 || g.K < 0) return set_error(c, PG_ERR_SIZE, "ring gemm: bad sizes M=%d N=%d K=%d", g.M, g.N, g.K);
    if (kind == K_WGRAD && wgrad_small_applies(g)) {
        const int sms = c->sm_count > 0 ? c->sm_count : 148;
        const int lbs = ((g.M + WS_OB - 1) / WS_OB) * ((g.N + WS_TB - 1) / WS_TB);
        // staged by output row when a phase's slice (one row of dY and the f
        // input rows it touches) fits: at most 96 KB per CTA, two CTAs per SM
        const long long slice = (long long)g.cq * g.ck + (long long)g.cr * (g.cw + 2 * g.pad) * g.cc;
        const long long red_bytes = (long long)WS_THREADS * (WS_OB * WS_TB + 1) * sizeof(T);
        int row_phases = WS_THREADS / lbs;
        while (row_phases > 0 && row_phases * slice * (long long)sizeof(T) > 96 * 1024) row_phases--;
        if (row_phases >= 1 && slice * sizeof(T) <= 96 * 1024) {
            // one output row per phase and round (two rows per round measured
            // 0.5 % slower on LeNet's training step)
            const int rpr = 1;
            const long long rows = (long long)g.nseg * g.cn * g.cp;
            const long long per_round = (long long)row_phases * rpr;
            // one wave of resident CTAs (two per SM), each a whole number of rounds
            const long long slots = 2LL * sms;
            long long per = (rows + slots - 1) / slots;
            per = (per + per_round - 1) / per_round * per_round;
            const long long ctas = (rows + per - 1) / per;
            const long long stage = per_round * slice * (long long)sizeof(T);
            const long long smem = stage > red_bytes ? stage : red_bytes;
            const size_t bytes = (size_t)g.M * g.N * sizeof(T);
            g.partial = (T *)gemm_partial(c, bytes);
            if (!g.partial) return PG_ERR_NO_MEMORY;
            g.steps_per_split = 0;
            if (smem > 48 * 1024) {
                // once per device: the kernel's shared-memory limit (never inside a stream capture)
                static std::mutex mu;
                static bool done[64];
                std::lock_guard<std::mutex> lock(mu);
                if (c->device < 0 || c->device >= 64) return set_error(c, PG_ERR_UNSUPPORTED, "device %d", c->device);
                if (!done[c->device]) {
                    PG_CHECK_CUDA(c, cudaFuncSetAttribute(wgrad_rows_kernel<T>,
                                                          cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
                    done[c->device] = true;
                }
            }
            PG_CHECK_CUDA(c, cudaMemsetAsync(g.partial, 0, bytes, c->stream));
            wgrad_rows_kernel<T><<<(unsigned)ctas, WS_THREADS, (size_t)smem, c->stream>>>(g, row_phases, (int)per, rpr);
            size_t blocks = (bytes / sizeof(T) + 255) / 256;
            if (blocks > (size_t)sms * 8) blocks = (size_t)sms * 8;
            ring_epilogue_kernel<T, K_WGRAD><<<(unsigned)blocks, 256, 0, c->stream>>>(g);
            c->launches += 2;
            return launch_status(c, "wgrad_rows_kernel");
        }
        const int phases = WS_THREADS / lbs;
        const long long all = (long long)g.K * g.nseg;
        long long ctas = 4LL * sms;
        const long long min_per = 64LL * phases;  // at least 64 pixels per phase
        if (ctas * min_per > all) ctas = (all + min_per - 1) / min_per;
        if (ctas < 1) ctas = 1;
        const long long per = (all + ctas - 1) / ctas;
        ctas = (all + per - 1) / per;
        const size_t bytes = (size_t)g.M * g.N * sizeof(T);
        g.partial = (T *)gemm_partial(c, bytes);
        if (!g.partial) return PG_ERR_NO_MEMORY;
        g.steps_per_split = 0;
        PG_CHECK_CUDA(c, cudaMemsetAsync(g.partial, 0, bytes, c->stream));
        wgrad_small_kernel<T><<<(unsigned)ctas, WS_THREADS, 0, c->stream>>>(g, phases, per);
        size_t blocks = (bytes / sizeof(T) + 255) / 256;
        if (blocks > (size_t)sms * 8) blocks = (size_t)sms * 8;
        ring_epilogue_kernel<T, K_WGRAD><<<(unsigned)blocks, 256, 0, c->stream>>>(g);
        c->launches += 2;
        return launch_status(c, "wgrad_small_kernel");
    }
    // tile shape: Col for N = 1, Thin for N <= 8, Small when a Wide tile would be less than half used
    int shape = 0, bm = Wide::BM, bn = Wide::BN;
    const double wide_use = (double)g.M * g.N /
                            ((double)((g.M + Wide::BM - 1) / Wide::BM) * Wide::BM * ((g.N + Wide::BN - 1) / Wide::BN) * Wide::BN);
    if (g.N == 1) { shape = 3; bm = Col::BM; bn = Col::BN; }
    else if (g.N <= Thin::BN) { shape = 1; bm = Thin::BM; bn = Thin::BN; }
    else if (wide_use < 0.5) { shape = 2; bm = Small::BM; bn = Small::BN; }
    dim3 grid((g.N + bn - 1) / bn, (g.M + bm - 1) / bm);
    if (grid.y > 65535) return set_error(c, PG_ERR_UNSUPPORTED, "ring gemm: M=%d too large", g.M);
    // Split K when the output tiles cannot fill the GPU (small M x N, long K:
    // weight gradients, narrow layers): about four CTAs per SM (two resident),
    // at least four k-steps each.
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    const long long tiles = (long long)grid.x * grid.y;
    const int all_steps = ((g.K + BK - 1) / BK) * g.nseg;
    g.partial = nullptr;
    g.steps_per_split = 0;
    if (tiles < sms && all_steps >= 8) {
        long long split = (4LL * sms + tiles - 1) / tiles;
        if (split > all_steps / 4) split = all_steps / 4;
        if (split > 65535) split = 65535;
        if (split >= 2) {
            const int per = (int)((all_steps + split - 1) / split);
            grid.z = (unsigned)((all_steps + per - 1) / per);
            const size_t bytes = (size_t)g.M * g.N * sizeof(T);
            g.partial = (T *)gemm_partial(c, bytes);
            if (!g.partial) return PG_ERR_NO_MEMORY;
            g.steps_per_split = per;
            PG_CHECK_CUDA(c, cudaMemsetAsync(g.partial, 0, bytes, c->stream));
        }
    }
    if (shape == 1) launch_tile<T, Thin>(c, grid, g, kind);
    else if (shape == 2) launch_tile<T, Small>(c, grid, g, kind);
    else if (shape == 3) launch_tile<T, Col>(c, grid, g, kind);
    else launch_tile<T, Wide>(c, grid, g, kind);
    c->launches += g.partial ? 2 : 1;
    return launch_status(c, "ring_gemm_kernel");
}

// --------------------------------------------------------------- entry glue

template <typename T> static void zero_args(GemmArgs<T> &g) { memset(&g, 0, sizeof(g)); }

// Fill the six RSS segments: seg 2p = (x_p0, y_p0 + y_p1), seg 2p+1 = (x_p1, y_p0).
template <typename T> static void rss_segments(GemmArgs<T> &g, const T *const *a, const T *const *b) {
    g.nseg = 6;
    for (int p = 0; p < 3; p++) {
        g.a[2 * p] = a[2 * p];
        g.b0[2 * p] = b[2 * p];
        g.b1[2 * p] = b[2 * p + 1];
        g.a[2 * p + 1] = a[2 * p + 1];
        g.b0[2 * p + 1] = b[2 * p];
        g.b1[2 * p + 1] = nullptr;
    }
}

template <typename T> static int rss_epilogue(Ctx *c, GemmArgs<T> &g, T *const *out, int trunc) {
    if (trunc < 0 || trunc >= (int)(sizeof(T) * 8)) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    g.epi = EPI_RSS;
    for (int i = 0; i < 6; i++) g.out[i] = out[i];
    g.d = (T)((T)1 << trunc);
    g.dshift = pow2_shift<T>(g.d);
    return PG_OK;
}

template <typename T>
int rss_matmul(Ctx *c, const T *const a[6], const T *const b[6], T *const out[6], const T *const bias[6], int M,
               int N, int K, int tA, int tB, int tC, int trunc) {
    CSh6<T> ca, cb;
    Sh6<T> co;
    if (!load6(ca, a) || !load6(cb, b) || !load6(co, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    GemmArgs<T> g;
    zero_args(g);
    g.M = M; g.N = N; g.K = K; g.tA = tA; g.tB = tB; g.tC = tC;
    rss_segments(g, a, b);
    int st = rss_epilogue(c, g, out, trunc);
    if (st) return st;
    if (bias)
        for (int i = 0; i < 6; i++) g.bias[i] = bias[i];
    st = launch_gemm(c, g, K_GEMM);
    if (st) return st;
    comm_msg(c, 2ull * M * N * sizeof(T), 2ull * M * N * sizeof(T));  // reconstruct3out3
    comm_round(c);
    return PG_OK;
}

template <typename T>
int rss_conv(Ctx *c, const T *const A[6], const T *const B[6], T *const C[6], int op, int batch, int H, int W, int f,
             int Din, int Dout, int stride, int pad, int trunc) {
    CSh6<T> ca, cb;
    Sh6<T> co;
    if (!load6(ca, A) || !load6(cb, B) || !load6(co, C)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (op < 0 || op > 2) return set_error(c, PG_ERR_INVALID_ARG, "bad conv operator %d", op);
    if (batch <= 0 || H <= 0 || W <= 0 || f <= 0 || Din <= 0 || Dout <= 0 || stride <= 0 || pad < 0 ||
        H + 2 * pad < f || W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "conv: bad geometry");
    GemmArgs<T> g;
    zero_args(g);
    setup_conv(g, op, batch, H, W, Din, Dout, f, f, pad, stride);
    rss_segments(g, A, B);
    int st = rss_epilogue(c, g, C, trunc);
    if (st) return st;
    st = launch_gemm(c, g, op == PG_CONV_FPROP ? K_FPROP : op == PG_CONV_DGRAD ? K_DGRAD : K_WGRAD);
    if (st) return st;
    uint64_t n_out = (uint64_t)g.M * g.N;
    comm_msg(c, 2 * n_out * sizeof(T), 2 * n_out * sizeof(T));
    comm_round(c);
    return PG_OK;
}

// One simulated FPC party's share-GEMM: the reveal of the party's product
// shares after the six reshares is a sum of local products a_{u,i} b_{u,j};
// the caller passes them as segments and the epilogue finishes dividePublic.
template <typename T>
int fpc_party_gemm(Ctx *c, const SegList<T> &s, int M, int N, int K, int tA, int tB, int tC, T *const out[3],
                   const T *const bias[3], int x0, int trunc) {
    if (s.nseg <= 0 || s.nseg > kMaxSeg) return set_error(c, PG_ERR_INVALID_ARG, "fpc gemm: %d segments", s.nseg);
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "matmul: bad sizes");
    if (trunc < 0 || trunc > (int)(sizeof(T) * 8 - 2)) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    GemmArgs<T> g;
    zero_args(g);
    g.M = M; g.N = N; g.K = K; g.tA = tA; g.tB = tB; g.tC = tC;
    g.nseg = s.nseg;
    for (int i = 0; i < s.nseg; i++) { g.a[i] = s.a[i]; g.b0[i] = s.b0[i]; g.b1[i] = s.b1[i]; }
    g.epi = EPI_FPC;
    for (int i = 0; i < 3; i++) { g.out[i] = out[i]; g.bias[i] = bias ? bias[i] : nullptr; }
    g.x0 = x0;
    g.d = (T)((T)1 << trunc);
    g.dshift = pow2_shift<T>(g.d);
    return launch_gemm(c, g, K_GEMM);
}

int fpc_party_conv_u64(Ctx *c, const SegList<uint64_t> &s, int op, int batch, int H, int W, int f, int Din,
                       int Dout, int stride, int pad, uint64_t *const out[3], int x0, int trunc) {
    if (s.nseg <= 0 || s.nseg > kMaxSeg) return set_error(c, PG_ERR_INVALID_ARG, "fpc conv: %d segments", s.nseg);
    if (op < 0 || op > 2) return set_error(c, PG_ERR_INVALID_ARG, "bad conv operator %d", op);
    if (trunc < 0 || trunc > 62) return set_error(c, PG_ERR_INVALID_ARG, "bad truncation %d", trunc);
    GemmArgs<uint64_t> g;
    zero_args(g);
    setup_conv(g, op, batch, H, W, Din, Dout, f, f, pad, stride);
    g.nseg = s.nseg;
    for (int i = 0; i < s.nseg; i++) { g.a[i] = s.a[i]; g.b0[i] = s.b0[i]; g.b1[i] = s.b1[i]; }
    g.epi = EPI_FPC;
    for (int i = 0; i < 3; i++) g.out[i] = out[i];
    g.x0 = x0;
    g.d = 1ull << trunc;
    g.dshift = trunc;
    return launch_gemm(c, g, op == PG_CONV_FPROP ? K_FPROP : op == PG_CONV_DGRAD ? K_DGRAD : K_WGRAD);
}

template <typename T>
int plain_gemm(Ctx *c, int M, int N, int K, const T *A, int tA, const T *B, int tB, T *C, int tC) {
    if (!A || !B || !C) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(c, PG_ERR_SIZE, "gemm: bad sizes");
    GemmArgs<T> g;
    zero_args(g);
    g.M = M; g.N = N; g.K = K; g.tA = tA; g.tB = tB; g.tC = tC;
    g.nseg = 1; g.a[0] = A; g.b0[0] = B; g.b1[0] = nullptr;
    g.epi = EPI_RAW; g.c_raw = C;
    return launch_gemm(c, g, K_GEMM);
}

int plain_conv_u64(Ctx *c, int op, int N, int H, int W, int C, int K, int R, int S, int pad, int stride,
                   const uint64_t *a, const uint64_t *b, uint64_t *out) {
    if (!a || !b || !out) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (op < 0 || op > 2 || N <= 0 || H <= 0 || W <= 0 || C <= 0 || K <= 0 || R <= 0 || S <= 0 || stride <= 0 ||
        pad < 0 || H + 2 * pad < R || W + 2 * pad < S)
        return set_error(c, PG_ERR_SIZE, "conv: bad geometry");
    GemmArgs<uint64_t> g;
    zero_args(g);
    setup_conv(g, op, N, H, W, C, K, R, S, pad, stride);
    g.nseg = 1; g.a[0] = a; g.b0[0] = b; g.b1[0] = nullptr;
    g.epi = EPI_RAW; g.c_raw = out;
    return launch_gemm(c, g, op == PG_CONV_FPROP ? K_FPROP : op == PG_CONV_DGRAD ? K_DGRAD : K_WGRAD);
}

template int rss_matmul<uint64_t>(Ctx *, const uint64_t *const *, const uint64_t *const *, uint64_t *const *,
                                  const uint64_t *const *, int, int, int, int, int, int, int);
template int rss_matmul<uint32_t>(Ctx *, const uint32_t *const *, const uint32_t *const *, uint32_t *const *,
                                  const uint32_t *const *, int, int, int, int, int, int, int);
template int rss_conv<uint64_t>(Ctx *, const uint64_t *const *, const uint64_t *const *, uint64_t *const *, int, int,
                                int, int, int, int, int, int, int, int);
template int fpc_party_gemm<uint64_t>(Ctx *, const SegList<uint64_t> &, int, int, int, int, int, int,
                                      uint64_t *const *, const uint64_t *const *, int, int);
template int fpc_party_gemm<uint32_t>(Ctx *, const SegList<uint32_t> &, int, int, int, int, int, int,
                                      uint32_t *const *, const uint32_t *const *, int, int);
template int plain_gemm<uint64_t>(Ctx *, int, int, int, const uint64_t *, int, const uint64_t *, int, uint64_t *, int);
template int plain_gemm<uint32_t>(Ctx *, int, int, int, const uint32_t *, int, const uint32_t *, int, uint32_t *, int);

}  // namespace pg
