// pg_relu.cu — fused dReLU / ReLU / selectShare kernels for 3-party RSS
// (src/mpc/RSS.inl:543-569,807-865). The value-level arithmetic is in
// pg_relu_value.cuh; these kernels stream the six share buffers through it
// and count the bytes and rounds the reference would send.
#include "pg_relu_value.cuh"

namespace pg {

template <typename T, typename U>
__global__ void drelu_kernel(CSh6<T> in, size_t n, Sh6<U> out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        T x[3][2];
        U r[3][2];
#pragma unroll
        for (int k = 0; k < 6; k++) x[k >> 1][k & 1] = in.p[k][i];
        drelu_value<T, U>(x, r);
#pragma unroll
        for (int k = 0; k < 6; k++) out.p[k][i] = r[k >> 1][k & 1];
    }
}

template <typename T, typename U>
__global__ void relu_kernel(CSh6<T> in, size_t n, Sh6<T> out, Sh6<U> dout) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        T x[3][2], zero[3][2], z[3][2];
        U r[3][2];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            x[k >> 1][k & 1] = in.p[k][i];
            zero[k >> 1][k & 1] = 0;
        }
        drelu_value<T, U>(x, r);
        select_value<T, U>(zero, x, r, z);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            out.p[k][i] = z[k >> 1][k & 1];
            if (dout.p[k]) dout.p[k][i] = r[k >> 1][k & 1];
        }
    }
}

template <typename T, typename U>
__global__ void select_kernel(CSh6<T> x_, CSh6<T> y_, CSh6<U> b_, size_t n, Sh6<T> z_) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        T x[3][2], y[3][2], z[3][2];
        U b[3][2];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            x[k >> 1][k & 1] = x_.p[k][i];
            y[k >> 1][k & 1] = y_.p[k][i];
            b[k >> 1][k & 1] = b_.p[k][i];
        }
        select_value<T, U>(x, y, b, z);
#pragma unroll
        for (int k = 0; k < 6; k++) z_.p[k][i] = z[k >> 1][k & 1];
    }
}

static unsigned ew_grid(Ctx *c, size_t n) {
    size_t b = (n + 255) / 256;
    size_t cap = (size_t)(c->sm_count > 0 ? c->sm_count : 148) * 16;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

// Byte/round accounting of dReLU: reconstruct(T) + 2 AND-reshares per level
// over n*W/2^L bit slots of U each (RSS.inl:818,1151-1155).
template <typename T, typename U> void count_drelu(Ctx *c, size_t n) {
    constexpr int W = sizeof(T) * 8;
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    for (int L = 1; (1 << L) <= W; L++) {
        uint64_t slots = (uint64_t)n * W >> L;
        comm_msg(c, 2 * slots * sizeof(U), 2 * slots * sizeof(U));
        comm_round(c, 2);
    }
}
// selectShare: reconstruct of the bits (U) + one *= reshare (T)
template <typename T, typename U> void count_select(Ctx *c, size_t n) {
    comm_msg(c, n * sizeof(U), n * sizeof(U));
    comm_round(c);
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
}

template <typename T, typename U> int rss_drelu(Ctx *c, const T *const in[6], size_t n, U *const out[6]) {
    CSh6<T> a;
    Sh6<U> o;
    if (n == 0) {  // no values: the protocol's messages are empty, its rounds still counted
        count_drelu<T, U>(c, 0);
        return PG_OK;
    }
    if (!load6(a, in) || !load6(o, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    drelu_kernel<T, U><<<ew_grid(c, n), 256, 0, c->stream>>>(a, n, o);
    c->launches++;
    int st = launch_status(c, "drelu_kernel");
    if (st) return st;
    count_drelu<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int rss_relu(Ctx *c, const T *const in[6], size_t n, T *const out[6], U *const dout[6]) {
    CSh6<T> a;
    Sh6<T> o;
    Sh6<U> d;
    if (n == 0) {
        count_drelu<T, U>(c, 0);
        count_select<T, U>(c, 0);
        return PG_OK;
    }
    if (!load6(a, in) || !load6(o, out)) return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    for (int i = 0; i < 6; i++) d.p[i] = dout ? dout[i] : nullptr;
    relu_kernel<T, U><<<ew_grid(c, n), 256, 0, c->stream>>>(a, n, o, d);
    c->launches++;
    int st = launch_status(c, "relu_kernel");
    if (st) return st;
    count_drelu<T, U>(c, n);
    count_select<T, U>(c, n);
    return PG_OK;
}

template <typename T, typename U>
int rss_select(Ctx *c, const T *const x[6], const T *const y[6], const U *const b[6], T *const z[6], size_t n) {
    CSh6<T> cx, cy;
    CSh6<U> cb;
    Sh6<T> cz;
    if (n == 0) {
        count_select<T, U>(c, 0);
        return PG_OK;
    }
    if (!load6(cx, x) || !load6(cy, y) || !load6(cb, b) || !load6(cz, z))
        return set_error(c, PG_ERR_INVALID_ARG, "null share pointer");
    select_kernel<T, U><<<ew_grid(c, n), 256, 0, c->stream>>>(cx, cy, cb, n, cz);
    c->launches++;
    int st = launch_status(c, "select_kernel");
    if (st) return st;
    count_select<T, U>(c, n);
    return PG_OK;
}

template int rss_drelu<uint64_t, uint8_t>(Ctx *, const uint64_t *const *, size_t, uint8_t *const *);
template int rss_drelu<uint64_t, uint64_t>(Ctx *, const uint64_t *const *, size_t, uint64_t *const *);
// the messages of ReLU (dReLU + selectShare) on n uint64 values with uint8
// bit shares, for kernels that fuse the ReLU into other work
void count_relu_u64_u8(Ctx *c, size_t n) {
    count_drelu<uint64_t, uint8_t>(c, n);
    count_select<uint64_t, uint8_t>(c, n);
}

template int rss_relu<uint64_t, uint8_t>(Ctx *, const uint64_t *const *, size_t, uint64_t *const *, uint8_t *const *);
template int rss_relu<uint64_t, uint64_t>(Ctx *, const uint64_t *const *, size_t, uint64_t *const *, uint64_t *const *);
template int rss_relu<uint32_t, uint8_t>(Ctx *, const uint32_t *const *, size_t, uint32_t *const *, uint8_t *const *);
template int rss_select<uint64_t, uint8_t>(Ctx *, const uint64_t *const *, const uint64_t *const *,
                                           const uint8_t *const *, uint64_t *const *, size_t);
template int rss_select<uint64_t, uint64_t>(Ctx *, const uint64_t *const *, const uint64_t *const *,
                                            const uint64_t *const *, uint64_t *const *, size_t);
template void count_drelu<uint64_t, uint8_t>(Ctx *, size_t);
template void count_drelu<uint64_t, uint64_t>(Ctx *, size_t);
template void count_select<uint64_t, uint8_t>(Ctx *, size_t);
template void count_select<uint64_t, uint64_t>(Ctx *, size_t);

}  // namespace pg
