"""Step-by-step CPU model of the decapsulation kernels, fed with the tables the
engine uploads (gmc_host_field_tables / gmc_host_sk_tables).

Checks the algorithm behind tensormceliece_gb300/csrc/kernels_dec.cu without a
GPU: front-end matrix F, the unpacking of the 2t syndromes, the BM update, the
additive FFT (twist + radix conversion + butterflies with the engine's
constants) and the error extraction at the support. Test infrastructure.
"""
import ctypes

import numpy as np

import tensormceliece_gb300 as gmc


def host_tables(set_id):
    L = gmc.lib()
    sz = gmc.set_sizes(set_id)
    m, t = sz["m"], sz["t"]
    q = 1 << m
    d = 6 if t <= 64 else 7
    gexp = np.zeros(2 * q - 1, np.uint16)
    glog = np.zeros(q, np.uint16)
    alog = np.zeros(q, np.uint16)
    tlog = np.zeros(2 << d, np.uint16)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    L.gmc_host_field_tables.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
    assert L.gmc_host_field_tables(set_id, p(gexp), p(glog), p(alog), p(tlog)) == 0
    return dict(m=m, t=t, q=q, d=d, n=sz["n"], mt=sz["mt"], gexp=gexp, glog=glog, alog=alog, tlog=tlog)


def sk_tables(set_id, sk):
    L = gmc.lib()
    sz = gmc.set_sizes(set_id)
    n = sz["n"]
    Ls = np.zeros(n, np.uint16)
    Lp = np.zeros(n, np.uint16)
    ldf = ctypes.c_int()
    L.gmc_host_sk_tables.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    skb = np.ascontiguousarray(sk, np.uint8)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    nwords = L.gmc_host_sk_tables(set_id, p(skb), None, None, None, 0, ctypes.byref(ldf))
    assert nwords > 0
    F = np.zeros(nwords, np.uint32)
    assert L.gmc_host_sk_tables(set_id, p(skb), p(Ls), p(Lp), p(F), nwords, ctypes.byref(ldf)) > 0
    return Ls, Lp, F.reshape(-1, ldf.value)


class Field:
    def __init__(self, tb):
        self.q = tb["q"]
        self.ZL = 2 * self.q - 2
        self.exp = tb["gexp"].astype(np.int64)
        self.log = tb["glog"].astype(np.int64)

    def mul_log(self, la, lb):
        return int(self.exp[min(la + lb, self.ZL)])

    def mul(self, a, b):
        return self.mul_log(int(self.log[a]), int(self.log[b]))


def front_end(F, ct, m, t):
    """s_j (j < 2t) = bits j*m..j*m+m-1 of F * c over GF(2)."""
    cw = F.shape[1]
    c = np.zeros(cw * 4, np.uint8)
    c[:len(ct)] = np.frombuffer(bytes(ct), np.uint8)
    cwords = c.view(np.uint32)
    rows = 2 * t * m
    par = np.zeros(rows, np.uint8)
    for r in range(rows):
        v = np.bitwise_and(F[r], cwords)
        par[r] = sum(bin(int(x)).count("1") for x in v) & 1
    s = [0] * (2 * t)
    for j in range(2 * t):
        for b in range(m):
            s[j] |= int(par[j * m + b]) << b
    return s


def bm(GF, s, t):
    C = [0] * (t + 1)
    B = [0] * (t + 1)
    C[0], B[1] = 1, 1
    L, b = 0, 1
    for n in range(2 * t):
        d = 0
        for i in range(min(n, t) + 1):
            d ^= GF.mul(C[i], s[n - i])
        T = list(C)
        if d:
            lf = int(GF.log[d]) - int(GF.log[b])
            if lf < 0:
                lf += GF.q - 1
            C = [C[i] ^ GF.mul_log(lf, int(GF.log[B[i]])) for i in range(t + 1)]
        if d and n >= 2 * L:
            L, b, B = n + 1 - L, d, T
        B = [0] + B[:t]
    return C  # locator: sigma(x) = sum_deg C[t-deg] x^deg


def fft(GF, tb, C):
    q, d, t = tb["q"], tb["d"], tb["t"]
    V = [0] * q
    for i in range(t + 1):
        deg = t - i
        if deg < (1 << d):
            V[deg] = C[i]
    for l in range(d):
        sz = 1 << (d - l)
        if l:
            off = (2 << d) - (2 << (d - l))
            for x in range(1 << d):
                V[x] = GF.mul_log(int(GF.log[V[x]]), int(tb["tlog"][off + (x >> l)]))
        s = sz
        while s >= 4:
            tau = s >> 2
            for it in range((1 << d) // 4):
                path, rest = it & ((1 << l) - 1), it >> l
                u, bl = rest % tau, rest // tau
                i2 = bl * s + 2 * tau + u
                V[path + (i2 << l)] ^= V[path + ((i2 + tau) << l)]
            for it in range((1 << d) // 4):
                path, rest = it & ((1 << l) - 1), it >> l
                u, bl = rest % tau, rest // tau
                i1 = bl * s + tau + u
                V[path + (i1 << l)] ^= V[path + ((i1 + tau) << l)]
            s >>= 1
    for x in range(1 << d, q):
        V[x] = V[x & ((1 << d) - 1)]
    for l in range(d - 1, -1, -1):
        off = q - (q >> l)
        h = 1 << l
        for u in range(q // 2):
            path, cp = u & (h - 1), u >> l
            x = path + (cp << (l + 1))
            a, bb = V[x], V[x + h]
            a ^= GF.mul_log(int(tb["alog"][off + cp]), int(GF.log[bb]))
            V[x], V[x + h] = a, a ^ bb
    return V


def decode(set_id, sk, ct, tb=None, skt=None):
    """Returns (s[2t], C[t+1] (BM order), e bytes [n/8], weight)."""
    tb = tb or host_tables(set_id)
    Ls, Lp, F = skt or sk_tables(set_id, sk)
    GF = Field(tb)
    m, t, n = tb["m"], tb["t"], tb["n"]
    s = front_end(F, ct, m, t)
    C = bm(GF, s, t)
    V = fft(GF, tb, C)
    lead = t == (1 << tb["d"])
    e = np.zeros(n // 8, np.uint8)
    w = 0
    for i in range(n):
        v = V[int(Ls[i])] ^ (int(Lp[i]) if lead else 0)
        if v == 0:
            e[i >> 3] |= 1 << (i & 7)
            w += 1
    return s, C, e, w
