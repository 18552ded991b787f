"""CPU model of the index transforms of the constant-time decapsulation kernels (kernels_dec.cu), checked against
their definitions without a GPU.

1. dec_root_kernel<SET, true> leaves, per request, the error vector in field-element order with bit-reversed index:
   word w holds y[32 w + i] = zero(alpha = bitrev_m(32 w + i)). Lane and register j hold the zero masks of one
   chunk slot over all 64 chunks; the kernel compacts every other bit and reverses the 5-bit index.
2. benes_ct_kernel applies the sk's control bits layer by layer on 32-bit words: strides below 32 with the 16
   control bits of a word deposited at the pairs' lower positions, larger strides as word pairs masked by one
   control word. The definition is the element-wise network that gives the support (applied to the identity it
   yields pi, and L_i = bitrev_m(pi(i))), as the engine's host key set-up computes it.
Test infrastructure only.
"""
import numpy as np
import pytest


def bitrev(a, m):
    r = 0
    for i in range(m):
        r |= ((a >> i) & 1) << (m - 1 - i)
    return r


def chunk_slot_final(d, lane, j):
    """The slot index lane and register j hold after the bottom-up pass (chunk_slot<D>(-1, lane, j))."""
    j0, j1 = j & 1, j >> 1
    if d == 7:
        return j0 | ((lane & 15) << 1) | (j1 << 5) | ((lane >> 4) << 6)
    return j0 | (lane << 1)


def comp_even16(x):
    x &= 0x55555555
    x = (x | (x >> 1)) & 0x33333333
    x = (x | (x >> 2)) & 0x0F0F0F0F
    x = (x | (x >> 4)) & 0x00FF00FF
    return (x | (x >> 8)) & 0x0000FFFF


def delta_swap(x, d, mask):
    t = ((x >> d) ^ x) & mask
    return (x ^ t ^ (t << d)) & 0xFFFFFFFF


def rev5_bits(x):
    return delta_swap(delta_swap(x, 15, 0x0000AAAA), 6, 0x00CC00CC)


def deposit(c16, s):
    """The 16 control bits of a word at the lower positions of its pairs of stride 2^s (bit s clear)."""
    masks = {3: 0xFF00FF00, 2: 0xF0F0F0F0, 1: 0xCCCCCCCC, 0: 0xAAAAAAAA}
    for pb in range(3, s - 1, -1):
        mp = masks[pb]
        c16 = ((c16 & ~mp) | ((c16 & mp) << (1 << pb))) & 0xFFFFFFFF
    return c16


@pytest.mark.parametrize("m,d", [(13, 7), (12, 6)])
def test_field_order_words(m, d):
    rng = np.random.default_rng(m)
    q = 1 << m
    zero = rng.integers(0, 2, q)
    words = np.zeros(q // 32, np.int64)
    for lane in range(32):
        for j in range((1 << d) // 32):
            sl = chunk_slot_final(d, lane, j)
            z = [sum(int(zero[((32 * h + k) << d) | sl]) << k for k in range(32)) for h in range(2)]
            for b0 in range(2):
                e32 = comp_even16(z[0] >> b0) | (comp_even16(z[1] >> b0) << 16)
                words[(bitrev(sl, d) << 1) | b0] = rev5_bits(e32)
    got = [(int(words[v >> 5]) >> (v & 31)) & 1 for v in range(q)]
    want = [int(zero[bitrev(v, m)]) for v in range(q)]
    assert got == want


@pytest.mark.parametrize("m", [13, 12])
def test_benes_words_match_element_network(m):
    rng = np.random.default_rng(100 + m)
    q = 1 << m
    order = list(range(m)) + list(range(m - 2, -1, -1))
    cond = rng.integers(0, 256, len(order) * (q // 16), dtype=np.uint8)
    cw = cond.view("<u4")
    x = rng.integers(0, 2, q)
    ref = x.copy()
    for li, s in enumerate(order):
        bits = cond[li * (q // 16):(li + 1) * (q // 16)]
        stride, idx = 1 << s, 0
        for i in range(0, q, 2 * stride):
            for j in range(stride):
                if (bits[idx >> 3] >> (idx & 7)) & 1:
                    ref[i + j], ref[i + j + stride] = ref[i + j + stride], ref[i + j]
                idx += 1
    words = [sum(int(x[32 * w + b]) << b for b in range(32)) for w in range(q // 32)]
    for li, s in enumerate(order):
        base = li * (q // 64)
        if s < 5:
            for w in range(q // 32):
                c = deposit((int(cw[base + (w >> 1)]) >> (16 * (w & 1))) & 0xFFFF, s)
                d = 1 << s
                t = ((words[w] >> d) ^ words[w]) & c
                words[w] = (words[w] ^ t ^ (t << d)) & 0xFFFFFFFF
        else:
            dd = 1 << (s - 5)
            for w in range(q // 32):
                if w & dd:
                    continue
                c = int(cw[base + (((w >> (s - 4)) << (s - 5)) | (w & (dd - 1)))])
                t = (words[w] ^ words[w + dd]) & c
                words[w] ^= t
                words[w + dd] ^= t
    got = np.array([(words[i >> 5] >> (i & 31)) & 1 for i in range(q)])
    assert (got == ref).all()
