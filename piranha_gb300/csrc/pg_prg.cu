// pg_prg.cu — the counter-mode AES generator of the reference's AESObject
// (src/mpc/AESObject.cpp:9-91) on the device, and the zero-sharing masks it
// gives the RSS resharing steps when a context turns it on.
//
// Generator. AESObject encrypts counter blocks with AES-256-ECB under the
// key read from its key file; block k is the __m128i whose two 64-bit lanes
// both hold k (rCounter + i adds i to both lanes), so the stream is
//   block k = AES-256_key(LE64(k) || LE64(k)),  k = 0, 1, 2, ...
// and a run of uint64 draws takes lane 0 then lane 1 of each block
// (getRandom's memcpy of whole blocks). One thread encrypts one block with
// the FIPS-197 round structure in the 32-bit table form; the S-box and the
// tables are derived on the host from the field arithmetic (multiplicative
// inverse in GF(2^8) mod x^8 + x^4 + x^3 + x + 1, then the affine map), the
// round keys by the AES-256 key expansion.
//
// Masks. The reference's reshare (src/mpc/RSS.inl:1053-1074) sends z_p with
// a mask that is never filled (rndMask = c). With keys on, party p adds
//   alpha_p = G(k_p) - G(k_prev(p))   (XOR of the low bits for bit shares)
// where k_p is the key party p shares with party p+1, so the alpha_p sum to
// zero and every reconstruction is unchanged; one counter per context
// advances by the blocks each step uses.
#include <cstring>
#include <mutex>

#include "pg_common.cuh"

namespace pg {

namespace {

struct Tables {
    uint32_t t[4][256];
    uint8_t sbox[256];
};

uint8_t gmul(uint8_t a, uint8_t b) {
    uint8_t r = 0;
    while (b) {
        if (b & 1) r ^= a;
        a = (uint8_t)((a << 1) ^ ((a & 0x80) ? 0x1B : 0));
        b >>= 1;
    }
    return r;
}

// S(x) = affine(x^-1), x^-1 = x^254 (0 -> 0)
void make_tables(Tables &tb) {
    for (int x = 0; x < 256; x++) {
        uint8_t inv = 0;
        if (x) {
            uint8_t p = 1, b = (uint8_t)x;
            for (int e = 254; e; e >>= 1) {
                if (e & 1) p = gmul(p, b);
                b = gmul(b, b);
            }
            inv = p;
        }
        uint8_t s = inv;
        for (int r = 1; r <= 4; r++) s ^= (uint8_t)((inv << r) | (inv >> (8 - r)));
        tb.sbox[x] = (uint8_t)(s ^ 0x63);
    }
    for (int x = 0; x < 256; x++) {
        const uint8_t s = tb.sbox[x];
        const uint32_t w = ((uint32_t)gmul(s, 2) << 24) | ((uint32_t)s << 16) | ((uint32_t)s << 8) | gmul(s, 3);
        for (int k = 0; k < 4; k++) tb.t[k][x] = k ? (w >> (8 * k)) | (w << (32 - 8 * k)) : w;
    }
}

const Tables &tables() {
    static Tables tb;
    static std::once_flag once;
    std::call_once(once, [] { make_tables(tb); });
    return tb;
}

__device__ uint32_t d_tab[4][256];
__device__ uint8_t d_sbox[256];

}  // namespace

struct AesKeys {
    uint32_t rk[3][60];  // AES-256 round keys of up to three keys
};

// AES-256 key expansion (FIPS-197 5.2, Nk = 8, Nr = 14), words big-endian
void aes256_expand(const uint8_t key[32], uint32_t rk[60]) {
    const Tables &tb = tables();
    for (int i = 0; i < 8; i++)
        rk[i] = ((uint32_t)key[4 * i] << 24) | ((uint32_t)key[4 * i + 1] << 16) | ((uint32_t)key[4 * i + 2] << 8) |
                key[4 * i + 3];
    uint8_t rcon = 1;
    auto sub = [&](uint32_t w) {
        return ((uint32_t)tb.sbox[w >> 24] << 24) | ((uint32_t)tb.sbox[(w >> 16) & 255] << 16) |
               ((uint32_t)tb.sbox[(w >> 8) & 255] << 8) | tb.sbox[w & 255];
    };
    for (int i = 8; i < 60; i++) {
        uint32_t t = rk[i - 1];
        if (i % 8 == 0) {
            t = sub((t << 8) | (t >> 24)) ^ ((uint32_t)rcon << 24);
            rcon = gmul(rcon, 2);
        } else if (i % 8 == 4) {
            t = sub(t);
        }
        rk[i] = rk[i - 8] ^ t;
    }
}

// the device tables, once per device (with it current)
static int prg_prepare(Ctx *c) {
    static std::mutex mu;
    static bool done[64];
    std::lock_guard<std::mutex> lock(mu);
    if (c->device < 0 || c->device >= 64) return set_error(c, PG_ERR_UNSUPPORTED, "device ordinal %d", c->device);
    if (!done[c->device]) {
        const Tables &tb = tables();
        PG_CHECK_CUDA(c, cudaMemcpyToSymbol(d_tab, tb.t, sizeof(tb.t)));
        PG_CHECK_CUDA(c, cudaMemcpyToSymbol(d_sbox, tb.sbox, sizeof(tb.sbox)));
        done[c->device] = true;
    }
    return PG_OK;
}

namespace {

__device__ __forceinline__ uint32_t ld_be(const uint8_t *b) {
    return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | b[3];
}

// block k = AES(LE64(k) || LE64(k)); returns its two little-endian lanes
__device__ __forceinline__ void aes_block(const uint32_t (&T)[4][256], const uint8_t *S, const uint32_t *rk,
                                          uint64_t k, uint64_t &lo, uint64_t &hi) {
    uint8_t in[16];
#pragma unroll
    for (int i = 0; i < 8; i++) in[i] = in[8 + i] = (uint8_t)(k >> (8 * i));
    uint32_t s0 = ld_be(in) ^ rk[0], s1 = ld_be(in + 4) ^ rk[1], s2 = ld_be(in + 8) ^ rk[2],
             s3 = ld_be(in + 12) ^ rk[3];
#pragma unroll 1
    for (int r = 1; r < 14; r++) {
        const uint32_t *k4 = rk + 4 * r;
        const uint32_t t0 = T[0][s0 >> 24] ^ T[1][(s1 >> 16) & 255] ^ T[2][(s2 >> 8) & 255] ^ T[3][s3 & 255] ^ k4[0];
        const uint32_t t1 = T[0][s1 >> 24] ^ T[1][(s2 >> 16) & 255] ^ T[2][(s3 >> 8) & 255] ^ T[3][s0 & 255] ^ k4[1];
        const uint32_t t2 = T[0][s2 >> 24] ^ T[1][(s3 >> 16) & 255] ^ T[2][(s0 >> 8) & 255] ^ T[3][s1 & 255] ^ k4[2];
        const uint32_t t3 = T[0][s3 >> 24] ^ T[1][(s0 >> 16) & 255] ^ T[2][(s1 >> 8) & 255] ^ T[3][s2 & 255] ^ k4[3];
        s0 = t0; s1 = t1; s2 = t2; s3 = t3;
    }
    // final round: SubBytes, ShiftRows, AddRoundKey
    const uint32_t *k4 = rk + 56;
    const uint32_t u[4] = {s0, s1, s2, s3};
    uint8_t out[16];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const uint32_t w = ((uint32_t)S[u[c] >> 24] << 24) | ((uint32_t)S[(u[(c + 1) & 3] >> 16) & 255] << 16) |
                           ((uint32_t)S[(u[(c + 2) & 3] >> 8) & 255] << 8) | S[u[(c + 3) & 3] & 255];
        const uint32_t o = w ^ k4[c];
        out[4 * c] = (uint8_t)(o >> 24);
        out[4 * c + 1] = (uint8_t)(o >> 16);
        out[4 * c + 2] = (uint8_t)(o >> 8);
        out[4 * c + 3] = (uint8_t)o;
    }
    lo = hi = 0;
#pragma unroll
    for (int i = 7; i >= 0; i--) {
        lo = (lo << 8) | out[i];
        hi = (hi << 8) | out[8 + i];
    }
}

__device__ __forceinline__ void load_tables(uint32_t (&T)[4][256], uint8_t (&S)[256]) {
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) T[i >> 8][i & 255] = d_tab[i >> 8][i & 255];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) S[i] = d_sbox[i];
    __syncthreads();
}

// out[j] = lane (j & 1) of block ctr + j / 2
__global__ void prg_fill_kernel(const __grid_constant__ AesKeys keys, uint64_t ctr, uint64_t *out, size_t n) {
    __shared__ uint32_t T[4][256];
    __shared__ uint8_t S[256];
    load_tables(T, S);
    const size_t blocks = (n + 1) / 2;
    for (size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x; b < blocks; b += (size_t)gridDim.x * blockDim.x) {
        uint64_t lo, hi;
        aes_block(T, S, keys.rk[0], ctr + b, lo, hi);
        out[2 * b] = lo;
        if (2 * b + 1 < n) out[2 * b + 1] = hi;
    }
}

// the zero-sharing masks of element i: alpha_p = G_p(i) - G_prev(p)(i) (ring)
// or the XOR of their low bits (bit shares)
template <typename T, bool XOR> struct Masks {
    static __device__ __forceinline__ void of(const uint32_t (&Tt)[4][256], const uint8_t *S, const AesKeys &keys,
                                              uint64_t ctr, size_t i, T (&alpha)[3]) {
        uint64_t g[3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            uint64_t lo, hi;
            aes_block(Tt, S, keys.rk[p], ctr + i / 2, lo, hi);
            g[p] = (i & 1) ? hi : lo;
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const int q = prev_party(p);
            // bit shares (u8) take the low bit only, so they stay 0 / 1
            alpha[p] = XOR ? (T)((g[p] ^ g[q]) & (sizeof(T) == 1 ? 1u : ~0ull)) : (T)(g[p] - g[q]);
        }
    }
};

// reshare with masks: party p sends z_p + alpha_p to its previous party
template <typename T> __global__ void reshare_prg_kernel(const __grid_constant__ AesKeys keys, uint64_t ctr,
                                                         Pub3<T> cin, size_t n, Sh6<T> out) {
    __shared__ uint32_t Tt[4][256];
    __shared__ uint8_t S[256];
    load_tables(Tt, S);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        T alpha[3];
        Masks<T, false>::of(Tt, S, keys, ctr, i, alpha);
        T c[3];
#pragma unroll
        for (int p = 0; p < 3; p++) c[p] = (T)(cin.p[p][i] + alpha[p]);
#pragma unroll
        for (int p = 0; p < 3; p++) {
            out.p[2 * p][i] = c[p];
            out.p[2 * p + 1][i] = c[next_party(p)];
        }
    }
}

// RSS *= / &= (RSS.inl:284-345) with masked resharing
template <typename T, bool AND> __global__ void mul_prg_kernel(const __grid_constant__ AesKeys keys, uint64_t ctr,
                                                               Sh6<T> a, CSh6<T> b, size_t n) {
    __shared__ uint32_t Tt[4][256];
    __shared__ uint8_t S[256];
    load_tables(Tt, S);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        T alpha[3];
        Masks<T, AND>::of(Tt, S, keys, ctr, i, alpha);
        T c[3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const T a0 = a.p[2 * p][i], a1 = a.p[2 * p + 1][i], b0 = b.p[2 * p][i], b1 = b.p[2 * p + 1][i];
            c[p] = AND ? (T)(((a0 & (T)(b0 ^ b1)) ^ (a1 & b0)) ^ alpha[p]) : (T)(a0 * (T)(b0 + b1) + a1 * b0 + alpha[p]);
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
            a.p[2 * p][i] = c[p];
            a.p[2 * p + 1][i] = c[next_party(p)];
        }
    }
}

unsigned prg_grid(Ctx *c, size_t units) {
    size_t b = (units + 255) / 256;
    const size_t cap = (size_t)(c->sm_count > 0 ? c->sm_count : 148) * 8;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

}  // namespace

int prg_fill_u64(Ctx *c, const uint8_t key[32], uint64_t ctr, uint64_t *out, size_t n) {
    if (!key || (!out && n)) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    int st = prg_prepare(c);
    if (st) return st;
    if (!n) return PG_OK;
    AesKeys k;
    memset(&k, 0, sizeof(k));
    aes256_expand(key, k.rk[0]);
    prg_fill_kernel<<<prg_grid(c, (n + 1) / 2), 256, 0, c->stream>>>(k, ctr, out, n);
    c->launches++;
    return launch_status(c, "prg_fill_kernel");
}

int prg_set_keys(Ctx *c, const uint8_t *keys, uint64_t ctr) {
    if (!keys) {
        c->prg_on = false;
        return PG_OK;
    }
    int st = prg_prepare(c);
    if (st) return st;
    for (int p = 0; p < 3; p++) aes256_expand(keys + 32 * p, c->prg_rk[p]);
    c->prg_ctr = ctr;
    c->prg_on = true;
    return PG_OK;
}

template <typename T> int rss_reshare_prg(Ctx *c, const T *const cin[3], size_t n, T *const out[6]) {
    Sh6<T> o;
    if (n && (!cin || !cin[0] || !cin[1] || !cin[2] || !load6(o, out)))
        return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (n) {
        Pub3<T> ci{{(T *)cin[0], (T *)cin[1], (T *)cin[2]}};
        AesKeys k;
        memcpy(k.rk, c->prg_rk, sizeof(k.rk));
        reshare_prg_kernel<T><<<prg_grid(c, n), 256, 0, c->stream>>>(k, c->prg_ctr, ci, n, o);
        c->launches++;
        int st = launch_status(c, "reshare_prg_kernel");
        if (st) return st;
        c->prg_ctr += (n + 1) / 2;
    }
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    return PG_OK;
}

template <typename T, bool AND> int rss_mul_prg(Ctx *c, T *const a[6], const T *const b[6], size_t n) {
    Sh6<T> ca;
    CSh6<T> cb;
    if (n && (!load6(ca, a) || !load6(cb, b))) return set_error(c, PG_ERR_INVALID_ARG, "null pointer");
    if (n) {
        AesKeys k;
        memcpy(k.rk, c->prg_rk, sizeof(k.rk));
        mul_prg_kernel<T, AND><<<prg_grid(c, n), 256, 0, c->stream>>>(k, c->prg_ctr, ca, cb, n);
        c->launches++;
        int st = launch_status(c, "mul_prg_kernel");
        if (st) return st;
        c->prg_ctr += (n + 1) / 2;
    }
    comm_msg(c, n * sizeof(T), n * sizeof(T));
    comm_round(c);
    return PG_OK;
}

template int rss_reshare_prg<uint64_t>(Ctx *, const uint64_t *const *, size_t, uint64_t *const *);
template int rss_mul_prg<uint64_t, false>(Ctx *, uint64_t *const *, const uint64_t *const *, size_t);
template int rss_mul_prg<uint64_t, true>(Ctx *, uint64_t *const *, const uint64_t *const *, size_t);
template int rss_mul_prg<uint8_t, true>(Ctx *, uint8_t *const *, const uint8_t *const *, size_t);

}  // namespace pg
