// pg_relu_value.cuh — value-level dReLU and selectShare for all three
// simulated parties, shared by the ReLU and maxpool kernels.
//
// The reference evaluates dReLU (src/mpc/RSS.inl:807-852) on one byte per bit
// (bitexpand, src/gpu/bitwise.cuh:10-21) and walks the carry tree of carryOut
// (:1113-1209) over Thrust strided views, with a message round per AND. Here
// one thread owns one value for all three simulated parties: the 64 bit
// shares of each party's two share slots live in one 64-bit register each,
// every tree level is a handful of shifts and masks, and the "reshare" of an
// AND gate is the exchange of a register between the party slots.
//
// Bit-level restatement of the reference's tree (levels L = 1..6, s = 2^L,
// h = s/2; positions inside a value's 64-bit word):
//   g[s*j + h-1] = AND(g[s*j + h-1], p[s*j + h])     (gEven &= pOdd)
//   p[s*j]       = AND(p[s*j],       p[s*j + h])     (pEven &= pOdd)
//   g[s*j + s-1] ^= g[s*j + h-1]                     (gOdd ^= gEven)
// and the carry-out is g[63]. An RSS AND on XOR shares (RSS.inl:331-345) is
// c_p = (x_p0 & (y_p0 ^ y_p1)) ^ (x_p1 & y_p0), then x_p = (c_p, c_{p+1}).
#pragma once

#include "pg_common.cuh"

namespace pg {

template <int W> struct TreeMasks;
template <> struct TreeMasks<64> {
    // gE[L]: positions s*j + h-1; pE[L]: positions s*j; gO[L]: positions s*j + s-1
    static __device__ __forceinline__ uint64_t gE(int L) {
        const uint64_t m[6] = {0x5555555555555555ull, 0x2222222222222222ull, 0x0808080808080808ull,
                               0x0080008000800080ull, 0x0000800000008000ull, 0x0000000080000000ull};
        return m[L];
    }
    static __device__ __forceinline__ uint64_t pE(int L) {
        const uint64_t m[6] = {0x5555555555555555ull, 0x1111111111111111ull, 0x0101010101010101ull,
                               0x0001000100010001ull, 0x0000000100000001ull, 0x0000000000000001ull};
        return m[L];
    }
    static __device__ __forceinline__ uint64_t gO(int L) {
        const uint64_t m[6] = {0xAAAAAAAAAAAAAAAAull, 0x8888888888888888ull, 0x8080808080808080ull,
                               0x8000800080008000ull, 0x8000000080000000ull, 0x8000000000000000ull};
        return m[L];
    }
};
template <> struct TreeMasks<32> {
    static __device__ __forceinline__ uint64_t gE(int L) {
        const uint64_t m[5] = {0x55555555ull, 0x22222222ull, 0x08080808ull, 0x00800080ull, 0x00008000ull};
        return m[L];
    }
    static __device__ __forceinline__ uint64_t pE(int L) {
        const uint64_t m[5] = {0x55555555ull, 0x11111111ull, 0x01010101ull, 0x00010001ull, 0x00000001ull};
        return m[L];
    }
    static __device__ __forceinline__ uint64_t gO(int L) {
        const uint64_t m[5] = {0xAAAAAAAAull, 0x88888888ull, 0x80808080ull, 0x80008000ull, 0x80000000ull};
        return m[L];
    }
};

// dReLU of one value for all parties. x[p][s] are the input shares (T);
// returns the result bit shares res[p][s] in U arithmetic
// (result.fill(1); result -= (carry ^ msb), RSS.inl:848-851).
template <typename T, typename U>
__device__ __forceinline__ void drelu_value(const T (&x)[3][2], U (&res)[3][2]) {
    constexpr int W = sizeof(T) * 8;
    constexpr int LEVELS = W == 64 ? 6 : 5;
    const uint64_t top = 1ull << (W - 1);
    const uint64_t ones = W == 64 ? ~0ull : 0xFFFFFFFFull;
    uint64_t g[3][2], pp[3][2];
    U msb[3][2];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        // reconstruct (RSS.inl:458-479) and a += 1 (RSS.inl:819)
        T a = (T)(x[p][0] + x[p][1] + x[prev_party(p)][0] + (T)1);
        uint64_t ab = (uint64_t)a;
        // rbits.fill(1): party A shareA, party C shareB hold all-ones
        uint64_t r0 = p == 0 ? ones : 0, r1 = p == 2 ? ones : 0;
        // setCarryOutMSB (bitwise.cuh:41-64) in the reference's party order
        U m0 = (U)((r0 >> (W - 1)) & 1), m1 = (U)((r1 >> (W - 1)) & 1);
        if (p == 0) m0 ^= (U)((ab >> (W - 1)) & 1);
        if (p == 2) m1 ^= (U)((ab >> (W - 1)) & 1);
        msb[p][0] = m0;
        msb[p][1] = m1;
        ab |= top;
        r0 &= ~top;
        r1 &= ~top;
        g[p][0] = r0 & ab;
        g[p][1] = r1 & ab;
        pp[p][0] = r0 ^ (p == 0 ? ab : 0);
        pp[p][1] = r1 ^ (p == 2 ? ab : 0);
    }
#pragma unroll
    for (int L = 0; L < LEVELS; L++) {
        const int h = 1 << L;
        const uint64_t mgE = TreeMasks<W>::gE(L), mpE = TreeMasks<W>::pE(L), mgO = TreeMasks<W>::gO(L);
        // gEven &= pOdd: operand p at position +1 relative to target
        uint64_t c[3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            uint64_t y0 = pp[p][0] >> 1, y1 = pp[p][1] >> 1;
            c[p] = ((g[p][0] & (y0 ^ y1)) ^ (g[p][1] & y0)) & mgE;
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
            g[p][0] = (g[p][0] & ~mgE) | c[p];
            g[p][1] = (g[p][1] & ~mgE) | c[next_party(p)];
        }
        // pEven &= pOdd: operand at position +h
#pragma unroll
        for (int p = 0; p < 3; p++) {
            uint64_t y0 = pp[p][0] >> h, y1 = pp[p][1] >> h;
            c[p] = ((pp[p][0] & (y0 ^ y1)) ^ (pp[p][1] & y0)) & mpE;
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
            pp[p][0] = (pp[p][0] & ~mpE) | c[p];
            pp[p][1] = (pp[p][1] & ~mpE) | c[next_party(p)];
        }
        // gOdd ^= gEven: source at position -h
#pragma unroll
        for (int p = 0; p < 3; p++) {
            g[p][0] ^= (g[p][0] << h) & mgO;
            g[p][1] ^= (g[p][1] << h) & mgO;
        }
    }
#pragma unroll
    for (int p = 0; p < 3; p++) {
        U c0 = (U)((g[p][0] >> (W - 1)) & 1) ^ msb[p][0];
        U c1 = (U)((g[p][1] >> (W - 1)) & 1) ^ msb[p][1];
        res[p][0] = (U)((p == 0 ? 1 : 0) - c0);
        res[p][1] = (U)((p == 2 ? 1 : 0) - c1);
    }
}

// selectShare (RSS.inl:543-569) of one value: z = (y - x) * d + x with d from
// convex_comb (RSS.inl:33-61,1322-1333) of the revealed e = b (c = 0).
template <typename T, typename U>
__device__ __forceinline__ void select_value(const T (&x)[3][2], const T (&y)[3][2], const U (&b)[3][2],
                                             T (&z)[3][2]) {
    T zz[3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        U e = (U)(b[p][0] + b[p][1] + b[prev_party(p)][0]);
        bool one = e == (U)1;
        T d0 = (one && p == 0) ? (T)1 : (T)0;
        T d1 = (one && p == 2) ? (T)1 : (T)0;
        T r0 = (T)(y[p][0] - x[p][0]), r1 = (T)(y[p][1] - x[p][1]);
        zz[p] = (T)(r0 * (T)(d0 + d1) + r1 * d0);
    }
#pragma unroll
    for (int p = 0; p < 3; p++) {
        z[p][0] = (T)(zz[p] + x[p][0]);
        z[p][1] = (T)(zz[next_party(p)] + x[p][1]);
    }
}

}  // namespace pg
