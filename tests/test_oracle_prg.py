"""The oracle's restatement of the reference's AES counter-mode generator
(src/mpc/AESObject.cpp) pinned on the CPU: the FIPS-197 AES-256 example
vector, an independent AES implementation where the host has one, the
counter-block layout, and the zero-sum of the resharing masks."""
import numpy as np
import pytest

import oracle as orc


def test_fips197_aes256_example():
    # FIPS-197 appendix C.3: key 00..1f, plaintext 00112233..ff
    key = bytes(range(32))
    pt = bytes.fromhex("00112233445566778899aabbccddeeff")
    assert orc.aes256_encrypt(key, pt).hex() == "8ea2b7ca516745bfeafc49904b496089"


@pytest.mark.parametrize("counter,n", [(0, 1), (0, 64), (12345, 101), (2**40 + 7, 33)])
def test_prg_stream_against_independent_aes(counter, n):
    crypto = pytest.importorskip("cryptography.hazmat.primitives.ciphers")
    rng = np.random.default_rng(counter + n)
    key = bytes(rng.integers(0, 256, 32, dtype=np.uint8))
    enc = crypto.Cipher(crypto.algorithms.AES(key), crypto.modes.ECB()).encryptor()
    nb = (n + 1) // 2
    blocks = b"".join(((counter + b) % 2**64).to_bytes(8, "little") * 2 for b in range(nb))
    want = np.frombuffer(enc.update(blocks) + enc.finalize(), dtype=np.uint64)[:n]
    assert np.array_equal(orc.prg_fill_u64(key, counter, n), want)


def test_prg_stream_is_blockwise():
    key = b"piranha key file contents\0\0\0\0\0\0\0"
    full = orc.prg_fill_u64(key, 10, 40)
    assert np.array_equal(full[8:], orc.prg_fill_u64(key, 14, 32))  # 2 draws per block


def test_masks_sum_to_zero():
    keys = [bytes([p]) * 32 for p in range(3)]
    m = orc.prg_masks(keys, 5, 1001)
    with np.errstate(over="ignore"):
        assert not (m[0] + m[1] + m[2]).any()
    x = orc.prg_masks(keys, 5, 1001, xor=True)
    assert not (x[0] ^ x[1] ^ x[2]).any()
    b = orc.prg_masks(keys, 5, 1001, xor=True, bits=True)
    assert set(np.unique(b)) <= {0, 1} and not (b[0] ^ b[1] ^ b[2]).any()

