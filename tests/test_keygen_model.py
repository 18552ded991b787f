"""CPU model of the key-generation kernels' control-bit algorithm (kg_cbits_kernel in
tensormceliece_gb300/csrc/keygen.cu) against the oracle's sort-based recursion.

The kernel runs the library's control-bit recursion (controlbits.c) level by level over all
sub-permutations at once and replaces each of the recursion's sorts by a scatter on the
packed word's key field, which is valid because every such key field is a permutation of the
segment's local indices. This model follows the kernel step for step in numpy; the oracle
(oracle/mceliece_oracle.c, pinned by libmceliece's KAT through keypair) computes the bits with
real sorts. Equality on random permutations of every size 2^4 .. 2^13 checks the argument.
"""
import numpy as np
import pytest

from oracle import pyoracle as O


def cbits_scatter(pi):
    """The kernel's algorithm: q = 2^W entries, depth d has 2^d segments of 2^(W-d)."""
    q = pi.size
    W = q.bit_length() - 1
    H = q // 2
    PI = pi.astype(np.uint32).copy()
    bits = np.zeros((2 * W - 1) * H, np.uint8)
    X = np.arange(q, dtype=np.uint32)
    for d in range(W):
        ww = W - d
        nn = 1 << ww
        x = X & np.uint32(nn - 1)
        base = X & np.uint32(~(nn - 1) & 0xFFFFFFFF)

        def offs(s):
            if d == 0:
                return np.zeros_like(s)
            r = np.zeros_like(s)
            for i in range(d):
                r |= ((s >> i) & 1) << (d - 1 - i)
            return r

        def scatter(arr, shift):
            out = np.empty_like(arr)
            out[base + ((arr >> np.uint32(shift)) & np.uint32(nn - 1))] = arr
            return out

        if ww == 1:
            s = np.arange(H, dtype=np.uint32)
            sel = (PI[0::2] & 1).astype(bool)
            bits[((W - 1) * H + offs(s))[sel]] = 1
            break
        A = ((PI ^ 1) << 16) | PI[X ^ 1]
        A = scatter(A, 16)
        px = A & 0xFFFF
        B = (px << 16) | np.minimum(px, x)
        A = (A << 16) | x
        A = scatter(A, 16)
        A = (A << 16) + (B >> 16)
        A = scatter(A, 16)
        if ww <= 10:
            B = ((A & 0xFFFF) << 10) | (B & 0x3FF)
            for _ in range(1, ww - 1):
                A = ((B & np.uint32(0xFFFFFC00)) << 6) | x
                A = scatter(A, 16)
                A = (A << 20) | B
                A = scatter(A, 20)
                ppcp = A & 0xFFFFF
                ppc = (A & 0xFFC00) | (B & 0x3FF)
                B = np.minimum(ppc, ppcp)
            B &= 0x3FF
        else:
            B = (A << 16) | (B & 0xFFFF)
            for i in range(1, ww - 1):
                A = (B & np.uint32(0xFFFF0000)) | x
                A = scatter(A, 16)
                A = (A << 16) | (B & 0xFFFF)
                if i < ww - 2:
                    B = (A & np.uint32(0xFFFF0000)) | (B >> 16)
                    B = scatter(B, 16)
                    B = (B << 16) | (A & 0xFFFF)
                A = scatter(A, 16)
                cp = (B & np.uint32(0xFFFF0000)) | (A & 0xFFFF)
                B = np.minimum(B, cp)
            B &= 0xFFFF
        A = (PI << 16) + x
        A = scatter(A, 16)
        even = X[0::2]
        z = even & np.uint32(nn - 1)
        s = even >> np.uint32(ww)
        fj = B[0::2] & 1
        Fz = z + fj
        bits[(d * H + offs(s) + ((z >> 1) << d))[fj.astype(bool)]] = 1
        B = np.empty_like(B)
        B[0::2] = (A[0::2] << 16) | Fz
        B[1::2] = (A[1::2] << 16) | (Fz ^ 1)
        B = scatter(B, 16)
        lk = B[0::2] & 1
        Ly = z + lk
        bits[((2 * W - 2 - d) * H + offs(s) + ((z >> 1) << d))[lk.astype(bool)]] = 1
        A2 = np.empty_like(A)
        A2[0::2] = (Ly << 16) | (B[0::2] & 0xFFFF)
        A2[1::2] = ((Ly ^ 1) << 16) | (B[1::2] & 0xFFFF)
        A = scatter(A2, 16)
        j = (even & np.uint32(nn - 1)) >> 1
        eb = even & np.uint32(~(nn - 1) & 0xFFFFFFFF)
        NP = np.empty_like(PI)
        NP[eb + j] = (A[0::2] & 0xFFFF) >> 1
        NP[eb + np.uint32(nn // 2) + j] = (A[1::2] & 0xFFFF) >> 1
        PI = NP
    return np.packbits(bits, bitorder="little")


@pytest.mark.parametrize("w", [4, 5, 6, 7, 10, 11, 12, 13])
def test_scatter_control_bits_equal_sorted_ones(w):
    rng = np.random.default_rng(1000 + w)
    for _ in range(3 if w >= 12 else 8):
        pi = rng.permutation(1 << w).astype(np.int16)
        assert np.array_equal(cbits_scatter(pi), O.controlbits(pi))


def test_identity_and_reversal():
    for w in (4, 12):
        for pi in (np.arange(1 << w), np.arange(1 << w)[::-1].copy()):
            assert np.array_equal(cbits_scatter(pi.astype(np.int16)), O.controlbits(pi.astype(np.int16)))
