"""ctypes wrapper of oracle/_ref/libmcref.so: the reference's own CPU implementation of the KEM
(libmceliece-20250507, portable `vec` code, compiled by oracle/build_ref.py).

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: imported by tests/, by the cpu_baseline / --impl reference legs of
bench.py and by its parity check, never by the engine. Same call shapes as oracle/pyoracle.py.
"""
import ctypes
import os

import numpy as np

from . import build_ref

SETS = ("348864", "460896", "6688128", "6960119", "8192128")
VARIANTS = tuple(s + v for v in ("", "pc", "f", "pcf") for s in SETS)
_lib = None


def available():
    """True when the library is built, or its extracted sources (or the reference tarball) are here to build it."""
    return os.path.exists(build_ref.LIB) or build_ref.available() or os.path.exists(
        os.path.join(build_ref.reference_root(), build_ref.TARBALL))


def build():
    return build_ref.build()


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(build_ref.LIB)
        vp = ctypes.c_void_p
        L.mcref_sizes.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
        L.mcref_name.restype = ctypes.c_char_p
        L.mcref_name.argtypes = [ctypes.c_int]
        L.mcref_implementation.restype = ctypes.c_char_p
        L.mcref_keypair.argtypes = [ctypes.c_int, vp, vp, vp]
        L.mcref_enc.argtypes = [ctypes.c_int, vp, vp, vp, vp]
        L.mcref_dec.argtypes = [ctypes.c_int, vp, vp, vp]
        L.mcref_enc_batch.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, vp, ctypes.c_int]
        L.mcref_dec_batch.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, ctypes.c_int]
        L.mcref_kat_checksum.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
        L.mcref_shake256.argtypes = [vp, ctypes.c_longlong, vp, ctypes.c_longlong]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def sid(s):
    return s if isinstance(s, int) else VARIANTS.index(str(s).replace("mceliece", ""))


def implementation():
    return lib().mcref_implementation().decode()


def sizes(s):
    out = (ctypes.c_longlong * 8)()
    lib().mcref_sizes(sid(s), out)
    return dict(zip(("m", "n", "t", "mt", "k", "pk_bytes", "sk_bytes", "ct_bytes"), [int(v) for v in out]))


def keypair(s, seed32):
    z = sizes(s)
    pk = np.zeros(z["pk_bytes"], np.uint8)
    sk = np.zeros(z["sk_bytes"], np.uint8)
    seed = np.frombuffer(bytes(seed32), np.uint8).copy()
    assert lib().mcref_keypair(sid(s), _p(pk), _p(sk), _p(seed)) == 0
    return pk, sk


def enc(s, pk, seed32):
    z = sizes(s)
    c = np.zeros(z["ct_bytes"], np.uint8)
    k = np.zeros(32, np.uint8)
    seed = np.frombuffer(bytes(seed32), np.uint8).copy()
    rc = lib().mcref_enc(sid(s), _p(c), _p(k), _p(np.ascontiguousarray(pk, np.uint8)), _p(seed))
    return rc, c, k


def dec(s, ct, sk):
    k = np.zeros(32, np.uint8)
    c = np.ascontiguousarray(np.frombuffer(bytes(ct), np.uint8) if isinstance(ct, (bytes, bytearray)) else ct,
                             np.uint8)
    rc = lib().mcref_dec(sid(s), _p(k), _p(c), _p(np.ascontiguousarray(sk, np.uint8)))
    return rc, k


def enc_batch(s, pk, seeds, threads=1):
    z = sizes(s)
    seeds = np.ascontiguousarray(seeds, np.uint8).reshape(-1, 32)
    n = seeds.shape[0]
    c = np.zeros((n, z["ct_bytes"]), np.uint8)
    k = np.zeros((n, 32), np.uint8)
    rc = np.zeros(n, np.int32)
    r = lib().mcref_enc_batch(sid(s), n, _p(c), _p(k), _p(np.ascontiguousarray(pk, np.uint8)), _p(seeds), _p(rc),
                              threads)
    assert r == 0
    return c, k, rc


def dec_batch(s, sk, cts, threads=1):
    z = sizes(s)
    cts = np.ascontiguousarray(cts, np.uint8).reshape(-1, z["ct_bytes"])
    n = cts.shape[0]
    k = np.zeros((n, 32), np.uint8)
    rc = np.zeros(n, np.int32)
    r = lib().mcref_dec_batch(sid(s), n, _p(k), _p(cts), _p(np.ascontiguousarray(sk, np.uint8)), _p(rc), threads)
    assert r == 0
    return k, rc


def kat_checksum(s, loops=8, index_first=0):
    buf = ctypes.create_string_buffer(65)
    rc = lib().mcref_kat_checksum(sid(s), loops, index_first, buf)
    return rc, buf.value.decode()
