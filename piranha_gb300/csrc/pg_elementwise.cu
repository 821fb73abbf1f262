// pg_elementwise.cu — the RSS protocol steps that are pure streaming work
// (reconstruct, reshare, *=, &=, dividePublic) and the reference's small glue
// kernels (src/gpu/matrix.cuh, bitwise.cuh, convolution.cuh). Each kernel
// reads every party's share slots once and writes every output slot once.
#include <cstring>

#include "pg_common.cuh"

namespace pg {

template <typename T> int rss_reshare_prg(Ctx *, const T *const *, size_t, T *const *);
template <typename T, bool AND> int rss_mul_prg(Ctx *, T *const *, const T *const *, size_t);

static unsigned grid1(Ctx *c, size_t n, int threads = 256) {
    size_t b = (n + threads - 1) / threads;
    size_t cap = (size_t)(c->sm_count > 0 ? c->sm_count : 148) * 32;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}
#define GRID_STRIDE(i, n) for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

// reconstruct (RSS.inl:458-479)
template <typename T> __global__ void reconstruct_kernel(CSh6<T> a, size_t n, Pub3<T> out) {
    GRID_STRIDE(i, n) {
#pragma unroll
        for (int p = 0; p < 3; p++) out.p[p][i] = (T)(a.p[2 * p][i] + a.p[2 * p + 1][i] + a.p[2 * prev_party(p)][i]);
    }
}

// reshare (RSS.inl:1053-1074)
template <typename T> __global__ void reshare_kernel(Pub3<T> cin, size_t n, Sh6<T> out) {
    GRID_STRIDE(i, n) {
        T c[3] = {cin.p[0][i], cin.p[1][i], cin.p[2][i]};
#pragma unroll
        for (int p = 0; p < 3; p++) {
            out.p[2 * p][i] = c[p];
            out.p[2 * p + 1][i] = c[next_party(p)];
        }
    }
}

// RSS *= (RSS.inl:284-320) and &= (:331-345), then reshare
template <typename T, bool AND> __global__ void mul_kernel(Sh6<T> a, CSh6<T> b, size_t n) {
    GRID_STRIDE(i, n) {
        T c[3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            T a0 = a.p[2 * p][i], a1 = a.p[2 * p + 1][i], b0 = b.p[2 * p][i], b1 = b.p[2 * p + 1][i];
            c[p] = AND ? (T)((a0 & (T)(b0 ^ b1)) ^ (a1 & b0)) : (T)(a0 * (T)(b0 + b1) + a1 * b0);
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
            a.p[2 * p][i] = c[p];
            a.p[2 * p + 1][i] = c[next_party(p)];
        }
    }
}

// dividePublic (RSS.inl:423-455) with r = 1, r' = d (Precompute.h:107-134):
// a -= r'; reveal; divide; a = r + revealed (A.shareA, C.shareB).
template <typename T> __global__ void divide_public_kernel(Sh6<T> a, size_t n, T d, int dshift, const T *dvec) {
    GRID_STRIDE(i, n) {
        T di = dvec ? dvec[i] : d;
        int t = dvec ? -2 : dshift;
        if (dvec) {
            // per-element power-of-two test (denominators are 1 << pows in practice)
            if (di != 0 && (di & (di - 1)) == 0 && di < ((T)1 << (sizeof(T) * 8 - 2)) * 2) t = __ffsll((long long)di) - 1;
            else t = -1;
        }
        T s[6];
#pragma unroll
        for (int k = 0; k < 6; k++) s[k] = a.p[k][i];
        s[0] = (T)(s[0] - di);  // party A shareA
        s[5] = (T)(s[5] - di);  // party C shareB
        T rA = (T)(s[0] + s[1] + s[4]);  // party A: own two + C's shareA
        T rC = (T)(s[4] + s[5] + s[2]);  // party C: own two + B's shareA
        a.p[0][i] = (T)(1 + div_public<T>(rA, di, t));
        a.p[1][i] = 0;
        a.p[2][i] = 0;
        a.p[3][i] = 0;
        a.p[4][i] = 0;
        a.p[5][i] = (T)(1 + div_public<T>(rC, di, t));
    }
}

// elementVectorAdd (matrix.cuh:75-84): a[col*rows + row] += b[rowwise ? col : row]
template <typename T> __global__ void eva_kernel(T *a, const T *b, int rowwise, int rows, int cols) {
    size_t n = (size_t)rows * cols;
    GRID_STRIDE(i, n) {
        int col = (int)(i / rows), row = (int)(i % rows);
        a[i] = (T)(a[i] + b[rowwise ? col : row]);
    }
}

// reduceSum (matrix.cuh:109-126): b[c] += sum over the reduced dimension
template <typename T> __global__ void reduce_sum_kernel(const T *a, T *b, int reduce_rows, int rows, int cols) {
    int outn = reduce_rows ? cols : rows;
    int len = reduce_rows ? rows : cols;
    for (int c = blockIdx.x; c < outn; c += gridDim.x) {
        T acc = 0;
        for (int i = threadIdx.x; i < len; i += blockDim.x)
            acc = (T)(acc + (reduce_rows ? a[(size_t)cols * i + c] : a[(size_t)cols * c + i]));
        __shared__ T red[256];
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) red[threadIdx.x] = (T)(red[threadIdx.x] + red[threadIdx.x + s]);
            __syncthreads();
        }
        if (threadIdx.x == 0) b[c] = (T)(b[c] + red[0]);
        __syncthreads();
    }
}

// truncate_cols (matrix.cuh:141-154)
__global__ void truncate_cols_kernel(const uint8_t *a, uint8_t *b, size_t rows, int start_cols, int end_cols) {
    size_t n = rows * end_cols;
    GRID_STRIDE(i, n) {
        size_t r = i / end_cols;
        int j = (int)(i % end_cols);
        b[i] = a[r * start_cols + j];
    }
}

// bitexpand (bitwise.cuh:10-21), in-bounds part
__global__ void bitexpand_kernel(const uint64_t *a, size_t n, uint64_t *bits) {
    GRID_STRIDE(i, n * 64) { bits[i] = (a[i >> 6] >> (i & 63)) & 1; }
}

// expandCompare (bitwise.cuh:66-92), in-bounds part
__global__ void expand_compare_kernel(const uint8_t *b, const uint8_t *nb, size_t n, size_t f, uint8_t *out) {
    GRID_STRIDE(i, n * 2 * f) {
        size_t j = i / (2 * f), e = i % (2 * f);
        out[i] = e < f ? b[j] : nb[j];
    }
}

// maxpool_im2row + stride_pad (convolution.cuh:56-108,175-191,252-304)
__global__ void maxpool_im2row_kernel(const uint64_t *im, uint64_t *out, int H, int W, int f, int Din, int batch,
                                      int stride, int pad, int wK, int hK, int padded, uint64_t pad_val) {
    size_t rows = (size_t)batch * Din * wK * hK;
    GRID_STRIDE(row, rows) {
        // row order (b, win, ch) as the reference's outputIdx
        int ch = (int)(row % Din);
        size_t t = row / Din;
        int win = (int)(t % ((size_t)wK * hK));
        int b = (int)(t / ((size_t)wK * hK));
        int baseCol = (win / hK) * stride - pad, baseRow = (win % hK) * stride - pad;
        uint64_t *o = out + row * padded;
        int k = 0;
        for (int c = 0; c < f; c++)
            for (int r = 0; r < f; r++) {
                int y = baseRow + r, x = baseCol + c;
                if (y < 0 || y >= H || x < 0 || x >= W) continue;  // reference leaves the slot as is
                o[k++] = im[(size_t)b * H * W * Din + (size_t)x * H * Din + (size_t)y * Din + ch];
            }
        for (; k < f * f; k++) o[k] = 0;
        for (int j = f * f; j < padded; j++) o[j] = pad_val;
    }
}

// ------------------------------------------------------------------ hosts

template <typename T> int rss_reconstruct(Ctx *c, const T *const a[6], size_t n, T *const out[3]) {
    CSh6<T> ca;
    if (n && (!load6(ca, a) || !out || !out[0] || !out[1] || !out[2]))
        return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    Pub3<T> o{{out[0], out[1], out[2]}};
    if (n) {
        reconstruct_kernel<T><<<grid1(c, n), 256, 0, c->stream>>>(ca, n, o);
        c->launches++;
        int st = launch_status(c, "reconstruct_kernel");
        if (st) return st;
    }
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    return PG_OK;
}

template <typename T> int rss_reshare(Ctx *c, const T *const cin[3], size_t n, T *const out[6]) {
    if (c->prg_on) return rss_reshare_prg<T>(c, cin, n, out);
    Sh6<T> o;
    if (n && (!cin || !cin[0] || !cin[1] || !cin[2] || !load6(o, out)))
        return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    Pub3<T> ci{};
    if (n) ci = Pub3<T>{{(T *)cin[0], (T *)cin[1], (T *)cin[2]}};
    if (n) {
        reshare_kernel<T><<<grid1(c, n), 256, 0, c->stream>>>(ci, n, o);
        c->launches++;
        int st = launch_status(c, "reshare_kernel");
        if (st) return st;
    }
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    return PG_OK;
}

template <typename T, bool AND> int rss_mul(Ctx *c, T *const a[6], const T *const b[6], size_t n) {
    if (c->prg_on) return rss_mul_prg<T, AND>(c, a, b, n);
    Sh6<T> ca;
    CSh6<T> cb;
    if (n && (!load6(ca, a) || !load6(cb, b))) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (n) {
        mul_kernel<T, AND><<<grid1(c, n), 256, 0, c->stream>>>(ca, cb, n);
        c->launches++;
        int st = launch_status(c, "mul_kernel");
        if (st) return st;
    }
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    return PG_OK;
}

template <typename T> int rss_divide_public(Ctx *c, T *const a[6], size_t n, T d, const T *dvec) {
    Sh6<T> ca;
    if (n && !load6(ca, a)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (n) {
        divide_public_kernel<T><<<grid1(c, n), 256, 0, c->stream>>>(ca, n, d, pow2_shift<T>(d), dvec);
        c->launches++;
        int st = launch_status(c, "divide_public_kernel");
        if (st) return st;
    }
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    return PG_OK;
}

int element_vector_add_u64(Ctx *c, uint64_t *a, const uint64_t *b, int rowwise, int rows, int cols) {
    if (!a || !b) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (rows <= 0 || cols <= 0) return set_error(c, PG_ERR_SIZE, "bad sizes");
    eva_kernel<uint64_t><<<grid1(c, (size_t)rows * cols), 256, 0, c->stream>>>(a, b, rowwise, rows, cols);
    c->launches++;
    return launch_status(c, "eva_kernel");
}

int reduce_sum_u64(Ctx *c, const uint64_t *a, uint64_t *b, int reduce_rows, int rows, int cols) {
    if (!a || !b) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (rows <= 0 || cols <= 0) return set_error(c, PG_ERR_SIZE, "bad sizes");
    int outn = reduce_rows ? cols : rows;
    reduce_sum_kernel<uint64_t><<<outn < 4096 ? outn : 4096, 256, 0, c->stream>>>(a, b, reduce_rows, rows, cols);
    c->launches++;
    return launch_status(c, "reduce_sum_kernel");
}

int truncate_cols_u8(Ctx *c, const uint8_t *a, uint8_t *b, size_t rows, int start_cols, int end_cols) {
    if (!a || !b) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (end_cols < 0 || start_cols < end_cols) return set_error(c, PG_ERR_SIZE, "bad columns");
    if (rows && end_cols) {
        truncate_cols_kernel<<<grid1(c, rows * end_cols), 256, 0, c->stream>>>(a, b, rows, start_cols, end_cols);
        c->launches++;
        return launch_status(c, "truncate_cols_kernel");
    }
    return PG_OK;
}

int bitexpand_u64(Ctx *c, const uint64_t *a, size_t n, uint64_t *bits) {
    if (!a || !bits) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (!n) return PG_OK;
    bitexpand_kernel<<<grid1(c, n * 64), 256, 0, c->stream>>>(a, n, bits);
    c->launches++;
    return launch_status(c, "bitexpand_kernel");
}

int expand_compare_u8(Ctx *c, const uint8_t *b, const uint8_t *nb, size_t n, uint8_t *out, size_t out_n) {
    if (!b || !nb || !out) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (!n) return PG_OK;
    size_t f = (out_n / n) / 2;
    if (f == 0) return set_error(c, PG_ERR_SIZE, "expandCompare: output smaller than 2n");
    expand_compare_kernel<<<grid1(c, n * 2 * f), 256, 0, c->stream>>>(b, nb, n, f, out);
    c->launches++;
    return launch_status(c, "expand_compare_kernel");
}

int maxpool_im2row_u64(Ctx *c, const uint64_t *im, uint64_t *out, int H, int W, int f, int Din, int batch, int stride,
                       int pad, uint64_t pad_val) {
    if (!im || !out) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (H <= 0 || W <= 0 || f <= 0 || Din <= 0 || batch <= 0 || stride <= 0 || pad < 0 || H + 2 * pad < f ||
        W + 2 * pad < f)
        return set_error(c, PG_ERR_SIZE, "maxpool_im2row: bad geometry");
    int wK = (W - f + 2 * pad) / stride + 1, hK = (H - f + 2 * pad) / stride + 1;
    int l2 = 0;
    while ((1 << l2) < f * f) l2++;
    int padded = l2 * l2;
    if (padded < f * f) return set_error(c, PG_ERR_UNSUPPORTED, "maxpool_im2row: pool %d", f);
    size_t rows = (size_t)batch * Din * wK * hK;
    maxpool_im2row_kernel<<<grid1(c, rows), 256, 0, c->stream>>>(im, out, H, W, f, Din, batch, stride, pad, wK, hK,
                                                                  padded, pad_val);
    c->launches++;
    return launch_status(c, "maxpool_im2row_kernel");
}

template int rss_reconstruct<uint64_t>(Ctx *, const uint64_t *const *, size_t, uint64_t *const *);
template int rss_reconstruct<uint8_t>(Ctx *, const uint8_t *const *, size_t, uint8_t *const *);
// The local (communication-free) RSS operators, RSS.inl:168-345: a public
// scalar or vector added / subtracted / XORed where the reference's setPublic
// puts public values (party A's shareA, party C's shareB: slots 0 and 5), and
// multiplied / ANDed / shifted into every share; a share tensor added,
// subtracted or XORed share by share. Shifts are arithmetic to the right
// (functors.cuh:48-70) and logical to the left, with amounts of 64 or more
// giving what the shift instructions give: all sign bits, or 0.
__device__ __forceinline__ uint64_t sar64(uint64_t x, uint64_t y) {
    return y >= 64 ? ((int64_t)x < 0 ? ~0ull : 0ull) : (uint64_t)((int64_t)x >> y);
}
__device__ __forceinline__ uint64_t shl64(uint64_t x, uint64_t y) { return y >= 64 ? 0ull : x << y; }

struct LocalArgs {
    uint64_t *a[12];
    const uint64_t *sh[12];
    int nbuf, pubmask;  // share buffers; bit k: buffer k holds the public component
    int op, kind;
    uint64_t scalar;
    const uint64_t *pub;
};

__global__ void local_kernel(const __grid_constant__ LocalArgs g, size_t n) {
    GRID_STRIDE(i, n) {
        const uint64_t pv = g.kind == PG_RHS_SCALAR ? g.scalar : g.kind == PG_RHS_PUBLIC ? g.pub[i] : 0;
        for (int k = 0; k < g.nbuf; k++) {
            const uint64_t r = g.kind == PG_RHS_SHARES ? g.sh[k][i] : pv;
            const bool pub_slot = (g.pubmask >> k) & 1;
            uint64_t x = g.a[k][i];
            switch (g.op) {
                case PG_OP_ADD: if (g.kind == PG_RHS_SHARES || pub_slot) x += r; break;
                case PG_OP_SUB: if (g.kind == PG_RHS_SHARES || pub_slot) x -= r; break;
                case PG_OP_XOR: if (g.kind == PG_RHS_SHARES || pub_slot) x ^= r; break;
                case PG_OP_MUL: x *= r; break;
                case PG_OP_AND: x &= r; break;
                case PG_OP_SHR: x = sar64(x, r); break;
                default: x = shl64(x, r); break;
            }
            g.a[k][i] = x;
        }
    }
}

// nbuf = 6 (RSS: public at party A's shareA and party C's shareB), 2 (TPC:
// party A's share, TPC.inl:146-214) or 12 (FPC: the x0 component, held as
// party B's shareC, party C's shareB and party D's shareA, FPC.inl:187-272)
int local_u64(Ctx *c, int nbuf, int op, uint64_t *const *a, size_t n, int kind, uint64_t scalar, const uint64_t *pub,
              const uint64_t *const *shares) {
    LocalArgs g;
    memset(&g, 0, sizeof(g));
    g.nbuf = nbuf;
    g.pubmask = nbuf == 6 ? (1 << 0) | (1 << 5) : nbuf == 2 ? 1 : (1 << 5) | (1 << 7) | (1 << 9);
    if (!a) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    for (int k = 0; k < nbuf; k++) {
        if (n && !a[k]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
        g.a[k] = a[k];
    }
    // the combinations the reference's share classes define
    static const bool ok[3][7] = {
        // ADD   SUB   MUL   XOR    AND    SHR   SHL
        {true, true, true, false, false, true, false},   // public scalar (operator op=(const T))
        {true, true, true, true, true, true, true},      // public vector (operator op=(const DeviceData &))
        {true, true, false, true, false, false, false},  // shares (operator op=(share class)); * & are protocol steps
    };
    if (kind < 0 || kind > 2 || op < 0 || op > 6 || !ok[kind][op])
        return set_error(c, PG_ERR_UNSUPPORTED, "no local operator %d with right-hand side kind %d", op, kind);
    if (kind == PG_RHS_PUBLIC && !pub && n) return set_error(c, PG_ERR_INVALID_ARG, "null public vector");
    if (kind == PG_RHS_SHARES) {
        if (!shares) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
        for (int k = 0; k < nbuf; k++) {
            if (n && !shares[k]) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
            g.sh[k] = shares[k];
        }
    }
    g.op = op;
    g.kind = kind;
    g.scalar = scalar;
    g.pub = pub;
    if (n) {
        local_kernel<<<grid1(c, n), 256, 0, c->stream>>>(g, n);
        c->launches++;
        return launch_status(c, "local_kernel");
    }
    return PG_OK;
}

int rss_local_u64(Ctx *c, int op, uint64_t *const a[6], size_t n, int kind, uint64_t scalar, const uint64_t *pub,
                  const uint64_t *const shares[6]) {
    return local_u64(c, 6, op, a, n, kind, scalar, pub, shares);
}

// DeviceData's own operators (src/gpu/DeviceData.h:131-277 with the functors
// of src/gpu/functors.cuh:1-117) on one array: a op= scalar or a op= vector
// for + - * / ^ & >> <<, and fill. Division is the reference's through double
// (div_public: exact integers for powers of two, device double otherwise).
template <typename T>
__global__ void device_op_kernel(T *a, size_t n, int op, T scalar, const T *vec, int shift) {
    GRID_STRIDE(i, n) {
        const T r = vec ? vec[i] : scalar;
        T x = a[i];
        switch (op) {
            case PG_OP_ADD: x += r; break;
            case PG_OP_SUB: x -= r; break;
            case PG_OP_MUL: x *= r; break;
            case PG_OP_XOR: x ^= r; break;
            case PG_OP_AND: x &= r; break;
            case PG_OP_SHR: x = sar64(x, r); break;
            case PG_OP_SHL: x = shl64(x, r); break;
            case PG_OP_DIV: x = div_public<T>(x, r, vec ? pow2_shift_dev(r) : shift); break;
            default: x = r; break;  // PG_OP_SET
        }
        a[i] = x;
    }
}

int device_op_u64(Ctx *c, int op, uint64_t *a, size_t n, int kind, uint64_t scalar, const uint64_t *vec) {
    if (op < 0 || op > PG_OP_SET) return set_error(c, PG_ERR_UNSUPPORTED, "no DeviceData operator %d", op);
    if (kind != PG_RHS_SCALAR && kind != PG_RHS_PUBLIC)
        return set_error(c, PG_ERR_UNSUPPORTED, "DeviceData operators take a scalar or a vector");
    if (n && (!a || (kind == PG_RHS_PUBLIC && !vec))) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (op == PG_OP_SET && kind != PG_RHS_SCALAR) return set_error(c, PG_ERR_UNSUPPORTED, "fill takes a scalar");
    if (!n) return PG_OK;
    device_op_kernel<uint64_t><<<grid1(c, n), 256, 0, c->stream>>>(a, n, op, scalar,
                                                                   kind == PG_RHS_PUBLIC ? vec : nullptr,
                                                                   pow2_shift<uint64_t>(scalar));
    c->launches++;
    return launch_status(c, "device_op_kernel");
}

template int rss_reshare<uint64_t>(Ctx *, const uint64_t *const *, size_t, uint64_t *const *);
template int rss_mul<uint64_t, false>(Ctx *, uint64_t *const *, const uint64_t *const *, size_t);
template int rss_mul<uint64_t, true>(Ctx *, uint64_t *const *, const uint64_t *const *, size_t);
template int rss_mul<uint8_t, true>(Ctx *, uint8_t *const *, const uint8_t *const *, size_t);
template int rss_divide_public<uint64_t>(Ctx *, uint64_t *const *, size_t, uint64_t, const uint64_t *);
template int rss_divide_public<uint32_t>(Ctx *, uint32_t *const *, size_t, uint32_t, const uint32_t *);

}  // namespace pg
