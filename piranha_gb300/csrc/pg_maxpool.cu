// pg_maxpool.cu — fused RSS maxpool: window gather + tournament + argmax bits.
//
// Restates MaxpoolLayer::forward (src/nn/MaxpoolLayer.cu:52-131) and maxpool
// (src/mpc/RSS.inl:868-1017). The reference materialises the pool rows with
// maxpool_im2row + stride_pad (src/gpu/convolution.cuh:56-108,175-191), then
// runs a tournament over strided even/odd views of the whole row array: per
// level a dReLU of even - odd, a selectShare that keeps the larger value in
// the even slot, and dresult &= expandCompare(b, 1 - b). Pairs never cross a
// pool row (the padded row length is a power of two), so one thread can own
// one pool row for all three parties and run every level in registers.
#include "pg_relu_value.cuh"

namespace pg {

template <typename T, typename U, int K>
__device__ __forceinline__ void tournament(T (&v)[K][3][2], U (&dr)[K][3][2]) {
#pragma unroll
    for (int i = 0; i < K; i++)
#pragma unroll
        for (int p = 0; p < 3; p++) {
            dr[i][p][0] = (p == 0) ? 1 : 0;  // dresult.fill(1)
            dr[i][p][1] = (p == 2) ? 1 : 0;
        }
#pragma unroll
    for (int s = 2; s <= K; s *= 2) {
        const int half = s / 2;
        U ex[K][3][2];
#pragma unroll
        for (int j = 0; j < K / s; j++) {
            const int e = s * j, o = s * j + half;
            T diff[3][2];
            U b[3][2];
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 2; q++) diff[p][q] = (T)(v[e][p][q] - v[o][p][q]);
            drelu_value<T, U>(diff, b);
            T z[3][2];
            select_value<T, U>(v[o], v[e], b, z);  // selectShare(odd, even, b, even)
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 2; q++) v[e][p][q] = z[p][q];
            // negated = fill(1) - b; expandCompare(b, negated)
#pragma unroll
            for (int i = 0; i < s; i++)
#pragma unroll
                for (int p = 0; p < 3; p++) {
                    if (i < half) {
                        ex[e + i][p][0] = b[p][0];
                        ex[e + i][p][1] = b[p][1];
                    } else {
                        ex[e + i][p][0] = (U)((p == 0 ? 1 : 0) - b[p][0]);
                        ex[e + i][p][1] = (U)((p == 2 ? 1 : 0) - b[p][1]);
                    }
                }
        }
        // dresult &= expandedB (RSS AND with reshare)
#pragma unroll
        for (int i = 0; i < K; i++) {
            U c[3];
#pragma unroll
            for (int p = 0; p < 3; p++)
                c[p] = (U)((dr[i][p][0] & (U)(ex[i][p][0] ^ ex[i][p][1])) ^ (dr[i][p][1] & ex[i][p][0]));
#pragma unroll
            for (int p = 0; p < 3; p++) {
                dr[i][p][0] = c[p];
                dr[i][p][1] = c[next_party(p)];
            }
        }
    }
}

template <typename T, typename U, int K>
__global__ void maxpool_rows_kernel(CSh6<T> in, size_t rows, Sh6<T> out, Sh6<U> dout) {
    for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < rows; r += (size_t)gridDim.x * blockDim.x) {
        T v[K][3][2];
        U dr[K][3][2];
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int k = 0; k < 6; k++) v[i][k >> 1][k & 1] = in.p[k][r * K + i];
        tournament<T, U, K>(v, dr);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            out.p[k][r] = v[0][k >> 1][k & 1];
#pragma unroll
            for (int i = 0; i < K; i++) dout.p[k][r * K + i] = dr[i][k >> 1][k & 1];
        }
    }
}

struct PoolGeom {
    int H, W, C, f, stride, batch, wK, hK;
    uint64_t pad_val;
};

// One thread per (image, window, channel) pool row in the reference's order:
// row = (b * (wK*hK) + win) * C + ch, window elements gathered with the
// (batch, x=col, y=row, channel) indexing of maxpool_im2row.
// ZM: shares 1-4 of the input are 0 (Ctx::in_zero_mid) and are not read.
// I: the row index type (uint32_t below 2^32 rows: its divisions are a few
// instructions where 64-bit ones are a long software sequence).
template <typename T, typename U, int K, bool ZM, typename I>
__global__ void maxpool_layer_kernel(CSh6<T> in, PoolGeom g, I rows, Sh6<T> out, Sh6<U> maxprime) {
    const int pool = g.f * g.f;
    const I C = (I)g.C, wins = (I)g.wK * (I)g.hK;
    auto load = [&](I row, T (&v)[K][3][2]) {
        const I t = row / C;
        const int ch = (int)(row - t * C);
        const I b_ = t / wins;
        const int win = (int)(t - b_ * wins), b = (int)b_;
        int baseCol = (win / g.hK) * g.stride, baseRow = (win % g.hK) * g.stride;
#pragma unroll
        for (int i = 0; i < K; i++) {
            if (i < pool) {
                int c = i / g.f, r = i - c * g.f;
                size_t src = (size_t)b * g.H * g.W * g.C + (size_t)(baseCol + c) * g.H * g.C +
                             (size_t)(baseRow + r) * g.C + ch;
#pragma unroll
                for (int k = 0; k < 6; k++)
                    v[i][k >> 1][k & 1] = (ZM && k > 0 && k < 5) ? (T)0 : in.p[k][src];
            } else {
#pragma unroll
                for (int k = 0; k < 6; k++) v[i][k >> 1][k & 1] = (T)g.pad_val;  // stride_pad value
            }
        }
    };
    for (I row = blockIdx.x * (I)blockDim.x + threadIdx.x; row < rows; row += (I)gridDim.x * blockDim.x) {
        T v[K][3][2];
        U dr[K][3][2];
        load(row, v);
        tournament<T, U, K>(v, dr);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            out.p[k][row] = v[0][k >> 1][k & 1];
            if (maxprime.p[k])
                for (int i = 0; i < pool; i++) maxprime.p[k][(size_t)row * pool + i] = dr[i][k >> 1][k & 1];
        }
    }
}

template <typename T, typename U> void count_drelu(Ctx *c, size_t n);
template <typename T, typename U> void count_select(Ctx *c, size_t n);

template <typename T, typename U> static void count_maxpool(Ctx *c, size_t n, int k) {
    for (int s = 2; s <= k; s *= 2) {
        size_t pairs = n / s;
        count_drelu<T, U>(c, pairs);
        count_select<T, U>(c, pairs);
        comm_msg(c, n * sizeof(U), n * sizeof(U));  // dresult &= expandedB
        comm_round(c);
    }
}

static unsigned pool_grid(Ctx *c, size_t n) {
    size_t b = (n + 127) / 128;
    size_t cap = (size_t)(c->sm_count > 0 ? c->sm_count : 148) * 16;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

template <typename T, typename U>
int rss_maxpool(Ctx *c, const T *const in[6], size_t n, int k, T *const out[6], U *const dout[6]) {
    CSh6<T> a;
    Sh6<T> o;
    Sh6<U> d;
    if (k != 4 && k != 16) return set_error(c, PG_ERR_UNSUPPORTED, "maxpool: k=%d (supported: 4, 16)", k);
    if (n % k) return set_error(c, PG_ERR_SIZE, "maxpool: n=%zu not a multiple of k=%d", n, k);
    size_t rows = n / k;
    if (rows == 0) return PG_OK;  // the reference divides by the row count here (bitwise.cuh:70)
    if (!load6(a, in) || !load6(o, out) || !load6(d, dout)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (k == 4) maxpool_rows_kernel<T, U, 4><<<pool_grid(c, rows), 128, 0, c->stream>>>(a, rows, o, d);
    else maxpool_rows_kernel<T, U, 16><<<pool_grid(c, rows), 128, 0, c->stream>>>(a, rows, o, d);
    c->launches++;
    int st = launch_status(c, "maxpool_rows_kernel");
    if (st) return st;
    count_maxpool<T, U>(c, n, k);
    return PG_OK;
}

template <typename T, typename U>
int rss_maxpool_layer(Ctx *c, const T *const in[6], T *const out[6], U *const maxprime[6], int H, int W, int C,
                      int pool, int stride, int batch, int fp) {
    CSh6<T> a;
    Sh6<T> o;
    Sh6<U> d;
    // maxprime == nullptr: no argmax bit shares (an inference forward needs none)
    if (!load6(a, in) || !load6(o, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (maxprime && !load6(d, maxprime)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (!maxprime)
        for (int k = 0; k < 6; k++) d.p[k] = nullptr;
    if (H <= 0 || W <= 0 || C <= 0 || pool <= 0 || stride <= 0 || batch <= 0 || pool > H || pool > W)
        return set_error(c, PG_ERR_SIZE, "maxpool layer: bad geometry");
    // padded pool size pow(ceil(log2(pool^2)), 2) (MaxpoolLayer.cu:69)
    int l2 = 0;
    while ((1 << l2) < pool * pool) l2++;
    int padded = l2 * l2;
    if (padded != 4 && padded != 16)
        return set_error(c, PG_ERR_UNSUPPORTED, "maxpool layer: pool %d pads to %d (supported: 4, 16)", pool, padded);
    PoolGeom g;
    g.H = H; g.W = W; g.C = C; g.f = pool; g.stride = stride; g.batch = batch;
    g.wK = (W - pool) / stride + 1;
    g.hK = (H - pool) / stride + 1;
    g.pad_val = (uint64_t)(T)(int64_t)(-10 * (1 << fp));
    size_t rows = (size_t)batch * g.wK * g.hK * C;
    // in_zero_mid: the caller knows shares 1-4 of the input are 0 (they are not read)
    const unsigned grid = pool_grid(c, rows);
    // 32-bit rows while the last row index and the grid stride past it fit
    const bool narrow = rows + (size_t)grid * 128 < (1ull << 32);
    const uint32_t rows32 = (uint32_t)rows;
#define PG_MAXPOOL_LAUNCH(KK, ZZ)                                                                      \
    (narrow ? maxpool_layer_kernel<T, U, KK, ZZ, uint32_t><<<grid, 128, 0, c->stream>>>(a, g, rows32, o, d) \
            : maxpool_layer_kernel<T, U, KK, ZZ, size_t><<<grid, 128, 0, c->stream>>>(a, g, rows, o, d))
    if (padded == 4) {
        if (c->in_zero_mid) PG_MAXPOOL_LAUNCH(4, true);
        else PG_MAXPOOL_LAUNCH(4, false);
    } else {
        if (c->in_zero_mid) PG_MAXPOOL_LAUNCH(16, true);
        else PG_MAXPOOL_LAUNCH(16, false);
    }
#undef PG_MAXPOOL_LAUNCH
    c->launches++;
    int st = launch_status(c, "maxpool_layer_kernel");
    if (st) return st;
    count_maxpool<T, U>(c, rows * padded, padded);
    return PG_OK;
}

// ------------------------------------------------------------ averagepool

template <typename T> int rss_divide_public(Ctx *, T *const *, size_t, T, const T *);

// AveragepoolLayer::forward (AveragepoolLayer.cu:58-81): each window summed
// per share, in the (batch, window, channel) order of averagepool_im2row
// (convolution.cuh:340-374), whose kernel (:56-107) gets the image's width and
// height swapped (kW = H, kH = W here); window positions outside the image are
// skipped, as that kernel skips them.
template <typename T>
__global__ void avgpool_sum_kernel(CSh6<T> in, Sh6<T> out, int kW, int kH, int C, int pool, int stride, int wk,
                                   int hk, size_t n_out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n_out; e += (size_t)gridDim.x * blockDim.x) {
        const size_t per_img = (size_t)wk * hk * C;
        const size_t b = e / per_img, rem = e - b * per_img;
        const int win = (int)(rem / C), ch = (int)(rem - (size_t)win * C);
        const int base_col = (win / hk) * stride, base_row = (win % hk) * stride;
        T acc[6] = {0, 0, 0, 0, 0, 0};
        for (int cc = 0; cc < pool; cc++)
            for (int r = 0; r < pool; r++) {
                const int y = base_row + r, x = base_col + cc;
                if (y < 0 || y >= kH || x < 0 || x >= kW) continue;
                const size_t src = b * (size_t)kH * kW * C + (size_t)x * kH * C + (size_t)y * C + ch;
#pragma unroll
                for (int k = 0; k < 6; k++) acc[k] = (T)(acc[k] + in.p[k][src]);
            }
#pragma unroll
        for (int k = 0; k < 6; k++) out.p[k][e] = acc[k];
    }
}

// averagepool_expand_delta (convolution.cuh:195-208): delta element i goes to
// slots (i / C) * C * f2 + i % C + j * C, j < f2, of the input gradient.
template <typename T> __global__ void avgpool_expand_kernel(CSh6<T> in, Sh6<T> out, size_t n, int C, int f2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t b = i / C, ch = i - b * C;
        const size_t first = b * (size_t)C * f2 + ch;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const T v = in.p[k][i];
            for (int j = 0; j < f2; j++) out.p[k][first + (size_t)j * C] = v;
        }
    }
}

template <typename T>
int rss_avgpool_layer(Ctx *c, const T *const in[6], T *const out[6], int H, int W, int C, int pool, int stride,
                      int batch) {
    CSh6<T> a;
    Sh6<T> o;
    if (!load6(a, in) || !load6(o, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (H <= 0 || W <= 0 || C <= 0 || pool <= 0 || stride <= 0 || batch <= 0 || pool > H || pool > W)
        return set_error(c, PG_ERR_SIZE, "averagepool layer: bad geometry");
    const int kW = H, kH = W;
    const int wk = (kW - pool) / stride + 1, hk = (kH - pool) / stride + 1;
    const size_t n_out = (size_t)batch * wk * hk * C;
    avgpool_sum_kernel<T><<<pool_grid(c, n_out), 128, 0, c->stream>>>(a, o, kW, kH, C, pool, stride, wk, hk, n_out);
    c->launches++;
    int st = launch_status(c, "avgpool_sum_kernel");
    if (st) return st;
    return rss_divide_public<T>(c, out, n_out, (T)(pool * pool), nullptr);
}

// AveragepoolLayer::backward (AveragepoolLayer.cu:88-117): deltas zeroed, the
// incoming gradient expanded, then dividePublic by pool^2. The expansion
// writes delta_n * pool^2 = batch * H * W * C slots when the pools tile the
// image (stride == pool), as the reference's layer sizes assume.
template <typename T>
int rss_avgpool_backward(Ctx *c, const T *const delta[6], T *const deltas[6], int H, int W, int C, int pool,
                         int stride, int batch) {
    CSh6<T> a;
    Sh6<T> o;
    if (!load6(a, delta) || !load6(o, deltas)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    if (H <= 0 || W <= 0 || C <= 0 || pool <= 0 || stride <= 0 || batch <= 0 || pool > H || pool > W)
        return set_error(c, PG_ERR_SIZE, "averagepool layer: bad geometry");
    const size_t n_in = (size_t)batch * H * W * C;
    const size_t n_delta = (size_t)batch * ((H - pool) / stride + 1) * ((W - pool) / stride + 1) * C;
    if (n_delta * (size_t)pool * pool > n_in)
        return set_error(c, PG_ERR_UNSUPPORTED, "averagepool backward: overlapping pools (stride %d < pool %d)", stride,
                         pool);
    for (int k = 0; k < 6; k++) PG_CHECK_CUDA(c, cudaMemsetAsync(deltas[k], 0, n_in * sizeof(T), c->stream));
    avgpool_expand_kernel<T><<<pool_grid(c, n_delta), 128, 0, c->stream>>>(a, o, n_delta, C, pool * pool);
    c->launches++;
    int st = launch_status(c, "avgpool_expand_kernel");
    if (st) return st;
    return rss_divide_public<T>(c, deltas, n_in, (T)(pool * pool), nullptr);
}

template int rss_avgpool_layer<uint64_t>(Ctx *, const uint64_t *const *, uint64_t *const *, int, int, int, int, int,
                                         int);
template int rss_avgpool_backward<uint64_t>(Ctx *, const uint64_t *const *, uint64_t *const *, int, int, int, int,
                                            int, int);

template int rss_maxpool<uint64_t, uint8_t>(Ctx *, const uint64_t *const *, size_t, int, uint64_t *const *,
                                            uint8_t *const *);
template int rss_maxpool<uint64_t, uint64_t>(Ctx *, const uint64_t *const *, size_t, int, uint64_t *const *,
                                             uint64_t *const *);
template int rss_maxpool_layer<uint64_t, uint8_t>(Ctx *, const uint64_t *const *, uint64_t *const *,
                                                  uint8_t *const *, int, int, int, int, int, int, int);

}  // namespace pg
