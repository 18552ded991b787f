"""ctypes wrapper of the CPU oracle (oracle/_build/libmceliece_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, always as the checker or as the
timed CPU baseline, never by the engine.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libmceliece_oracle.so")
SETS = ("348864", "460896", "6688128", "6960119", "8192128")
# variants: id = set + 5 v, v = 0 plain, 1 pc (same keys), 2 f (semi-systematic keys), 3 pcf
VARIANTS = tuple(s + v for v in ("", "pc", "f", "pcf") for s in SETS)
_lib = None


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        L.gmo_sizes.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
        L.gmo_keypair.argtypes = [ctypes.c_int, vp, vp, vp]
        L.gmo_controlbits.argtypes = [vp, vp, ctypes.c_int]
        L.gmo_enc.argtypes = [ctypes.c_int, vp, vp, vp, vp]
        L.gmo_dec.argtypes = [ctypes.c_int, vp, vp, vp]
        L.gmo_gen_e.argtypes = [ctypes.c_int, vp, vp]
        L.gmo_syndrome.argtypes = [ctypes.c_int, vp, vp, vp]
        L.gmo_decrypt_stages.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp]
        L.gmo_support.argtypes = [ctypes.c_int, vp, vp, vp]
        L.gmo_enc_batch.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, vp, ctypes.c_int]
        L.gmo_dec_batch.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, ctypes.c_int]
        L.gmo_kat_checksum.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
        L.gmo_shake256.argtypes = [vp, ctypes.c_longlong, vp, ctypes.c_longlong]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def sid(s):
    return s if isinstance(s, int) else VARIANTS.index(str(s).replace("mceliece", ""))


def sizes(s):
    out = (ctypes.c_longlong * 8)()
    lib().gmo_sizes(sid(s), out)
    return dict(zip(("m", "n", "t", "mt", "k", "pk_bytes", "sk_bytes", "ct_bytes"), [int(v) for v in out]))


def keypair(s, seed32):
    z = sizes(s)
    pk = np.zeros(z["pk_bytes"], np.uint8)
    sk = np.zeros(z["sk_bytes"], np.uint8)
    seed = np.frombuffer(bytes(seed32), np.uint8).copy()
    rc = lib().gmo_keypair(sid(s), _p(pk), _p(sk), _p(seed))
    assert rc == 0, rc
    return pk, sk


def controlbits(pi):
    """Benes control bits of the permutation pi (2^w int entries), as key generation computes them."""
    pi = np.ascontiguousarray(pi, dtype=np.int16)
    w = int(pi.size).bit_length() - 1
    out = np.zeros(((2 * w - 1) * pi.size // 2 + 7) // 8, np.uint8)
    rc = lib().gmo_controlbits(_p(out), _p(pi), w)
    assert rc == 0, rc
    return out


def enc(s, pk, seed32):
    z = sizes(s)
    c = np.zeros(z["ct_bytes"], np.uint8)
    k = np.zeros(32, np.uint8)
    seed = np.frombuffer(bytes(seed32), np.uint8).copy()
    rc = lib().gmo_enc(sid(s), _p(c), _p(k), _p(np.ascontiguousarray(pk, np.uint8)), _p(seed))
    return rc, c, k


def dec(s, ct, sk):
    k = np.zeros(32, np.uint8)
    c = np.frombuffer(bytes(ct), np.uint8).copy() if isinstance(ct, (bytes, bytearray)) else np.ascontiguousarray(
        ct, np.uint8)
    rc = lib().gmo_dec(sid(s), _p(k), _p(c), _p(np.ascontiguousarray(sk, np.uint8)))
    return rc, k


def enc_batch(s, pk, seeds, threads=1):
    z = sizes(s)
    seeds = np.ascontiguousarray(seeds, np.uint8).reshape(-1, 32)
    n = seeds.shape[0]
    c = np.zeros((n, z["ct_bytes"]), np.uint8)
    k = np.zeros((n, 32), np.uint8)
    rc = np.zeros(n, np.int32)
    r = lib().gmo_enc_batch(sid(s), n, _p(c), _p(k), _p(np.ascontiguousarray(pk, np.uint8)), _p(seeds), _p(rc),
                            threads)
    assert r == 0
    return c, k, rc


def dec_batch(s, sk, cts, threads=1):
    z = sizes(s)
    cts = np.ascontiguousarray(cts, np.uint8).reshape(-1, z["ct_bytes"])
    n = cts.shape[0]
    k = np.zeros((n, 32), np.uint8)
    rc = np.zeros(n, np.int32)
    r = lib().gmo_dec_batch(sid(s), n, _p(k), _p(cts), _p(np.ascontiguousarray(sk, np.uint8)), _p(rc), threads)
    assert r == 0
    return k, rc


def gen_e(s, seed32):
    z = sizes(s)
    e = np.zeros(z["n"] // 8, np.uint8)
    seed = np.frombuffer(bytes(seed32), np.uint8).copy()
    attempts = lib().gmo_gen_e(sid(s), _p(e), _p(seed))
    return e, attempts


def syndrome(s, pk, e):
    z = sizes(s)
    out = np.zeros(z["ct_bytes"], np.uint8)
    lib().gmo_syndrome(sid(s), _p(out), _p(np.ascontiguousarray(pk, np.uint8)), _p(np.ascontiguousarray(e, np.uint8)))
    return out


def decrypt_stages(s, sk, ct):
    z = sizes(s)
    t = z["t"]
    sp = np.zeros(2 * t, np.uint16)
    loc = np.zeros(t + 1, np.uint16)
    e = np.zeros(z["n"] // 8, np.uint8)
    c = np.ascontiguousarray(np.frombuffer(bytes(ct), np.uint8) if isinstance(ct, (bytes, bytearray)) else ct,
                             np.uint8)
    rc = lib().gmo_decrypt_stages(sid(s), _p(np.ascontiguousarray(sk, np.uint8)), _p(c), _p(sp), _p(loc), _p(e))
    return rc, sp, loc, e


def kat_checksum(s, loops=8):
    buf = ctypes.create_string_buffer(65)
    rc = lib().gmo_kat_checksum(sid(s), loops, 0, buf)
    return rc, buf.value.decode()


def shake256(data, outlen):
    d = np.frombuffer(bytes(data), np.uint8).copy()
    out = np.zeros(outlen, np.uint8)
    lib().gmo_shake256(_p(out), outlen, _p(d), d.size)
    return out.tobytes()
