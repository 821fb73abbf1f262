// oracle/aes.hpp — test infrastructure: AES-256 (FIPS-197) restated byte by
// byte, and the counter-mode stream of the reference's AESObject
// (src/mpc/AESObject.cpp:40-91): block k = AES-256-ECB_key(LE64(k) || LE64(k))
// (rCounter + i adds i to both 64-bit lanes of the __m128i counter), uint64
// draws taking lane 0 then lane 1 of each block. The S-box comes from
// log / antilog tables of the generator 3 and the bitwise affine map of
// FIPS-197 eq. 5.1; the cipher is SubBytes, ShiftRows, MixColumns (xtime),
// AddRoundKey on a 4 x 4 byte state. Pinned against the FIPS-197 C.3 example
// vector and, where the host has it, an independent AES implementation.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>

namespace oracle {

struct Aes256 {
    uint8_t sbox[256];
    uint8_t rk[15][16];  // round keys, bytes in state order (column-major)

    static uint8_t xtime(uint8_t a) { return (uint8_t)((a << 1) ^ ((a & 0x80) ? 0x1B : 0)); }

    void make_sbox() {
        uint8_t ex[256], lg[256];
        uint8_t v = 1;
        for (int i = 0; i < 255; i++) {
            ex[i] = v;
            lg[v] = (uint8_t)i;
            v = (uint8_t)(v ^ xtime(v));  // times 3
        }
        ex[255] = ex[0];
        for (int x = 0; x < 256; x++) {
            const uint8_t inv = x ? ex[(255 - lg[x]) % 255] : 0;
            uint8_t s = 0;
            for (int i = 0; i < 8; i++) {
                const int bit = ((inv >> i) ^ (inv >> ((i + 4) & 7)) ^ (inv >> ((i + 5) & 7)) ^ (inv >> ((i + 6) & 7)) ^
                                 (inv >> ((i + 7) & 7)) ^ (0x63 >> i)) &
                                1;
                s |= (uint8_t)(bit << i);
            }
            sbox[x] = s;
        }
    }

    explicit Aes256(const uint8_t key[32]) {
        make_sbox();
        uint8_t w[60][4];
        for (int i = 0; i < 8; i++)
            for (int j = 0; j < 4; j++) w[i][j] = key[4 * i + j];
        uint8_t rcon = 1;
        for (int i = 8; i < 60; i++) {
            uint8_t t[4] = {w[i - 1][0], w[i - 1][1], w[i - 1][2], w[i - 1][3]};
            if (i % 8 == 0) {
                const uint8_t t0 = t[0];
                t[0] = (uint8_t)(sbox[t[1]] ^ rcon);
                t[1] = sbox[t[2]];
                t[2] = sbox[t[3]];
                t[3] = sbox[t0];
                rcon = xtime(rcon);
            } else if (i % 8 == 4) {
                for (int j = 0; j < 4; j++) t[j] = sbox[t[j]];
            }
            for (int j = 0; j < 4; j++) w[i][j] = (uint8_t)(w[i - 8][j] ^ t[j]);
        }
        for (int r = 0; r < 15; r++)
            for (int c = 0; c < 4; c++)
                for (int j = 0; j < 4; j++) rk[r][4 * c + j] = w[4 * r + c][j];
    }

    void encrypt(const uint8_t in[16], uint8_t out[16]) const {
        uint8_t s[16];
        for (int i = 0; i < 16; i++) s[i] = (uint8_t)(in[i] ^ rk[0][i]);
        for (int r = 1; r <= 14; r++) {
            uint8_t t[16];
            // SubBytes + ShiftRows: state byte (row, col) = s[4 * col + row]
            for (int c = 0; c < 4; c++)
                for (int row = 0; row < 4; row++) t[4 * c + row] = sbox[s[4 * ((c + row) & 3) + row]];
            if (r < 14) {
                for (int c = 0; c < 4; c++) {
                    const uint8_t a0 = t[4 * c], a1 = t[4 * c + 1], a2 = t[4 * c + 2], a3 = t[4 * c + 3];
                    const uint8_t all = (uint8_t)(a0 ^ a1 ^ a2 ^ a3);
                    t[4 * c] = (uint8_t)(a0 ^ all ^ xtime((uint8_t)(a0 ^ a1)));
                    t[4 * c + 1] = (uint8_t)(a1 ^ all ^ xtime((uint8_t)(a1 ^ a2)));
                    t[4 * c + 2] = (uint8_t)(a2 ^ all ^ xtime((uint8_t)(a2 ^ a3)));
                    t[4 * c + 3] = (uint8_t)(a3 ^ all ^ xtime((uint8_t)(a3 ^ a0)));
                }
            }
            for (int i = 0; i < 16; i++) s[i] = (uint8_t)(t[i] ^ rk[r][i]);
        }
        memcpy(out, s, 16);
    }
};

// uint64 draws j = 0..n-1 from block counter ctr: lane (j & 1) of block ctr + j / 2
inline void prg_fill_u64(const uint8_t key[32], uint64_t ctr, uint64_t* out, size_t n) {
    const Aes256 aes(key);
    for (size_t b = 0; 2 * b < n; b++) {
        uint8_t in[16], o[16];
        const uint64_t k = ctr + b;
        for (int i = 0; i < 8; i++) in[i] = in[8 + i] = (uint8_t)(k >> (8 * i));
        aes.encrypt(in, o);
        uint64_t lo = 0, hi = 0;
        for (int i = 7; i >= 0; i--) {
            lo = (lo << 8) | o[i];
            hi = (hi << 8) | o[8 + i];
        }
        out[2 * b] = lo;
        if (2 * b + 1 < n) out[2 * b + 1] = hi;
    }
}

inline void aes256_encrypt_block(const uint8_t key[32], const uint8_t in[16], uint8_t out[16]) {
    const Aes256 aes(key);
    aes.encrypt(in, out);
}

}  // namespace oracle
