"""GB300 batched Classic McEliece KEM engine: Python mirror of the C ABI (include/gmc.h).

The engine is libgmc.so, built in-tree by tensormceliece_gb300.build. This module
loads it with ctypes and exposes the libmceliece-shaped calls
(``kem_enc``/``kem_dec`` per set) and the batched, resident-key calls
(``PublicKey``/``SecretKey`` with ``enc_batch``/``dec_batch``). There is no CPU
fallback: if the library or a GPU is missing the calls raise ``GmcError``.

Buffers: host calls take/return ``bytes``/numpy ``uint8`` arrays; the ``*_dev``
calls take raw device pointers (ints), e.g. ``torch.Tensor.data_ptr()``, and a
``cudaStream_t`` handle (``torch.cuda.current_stream().cuda_stream``).
"""
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = [
    "SETS", "VARIANTS", "GmcError", "lib", "set_id", "set_sizes", "keypair", "keypair_batch", "Plan", "Server", "PublicKey", "SecretKey", "kem_enc", "kem_dec",
    "set_gemm_engine", "get_gemm_engine", "set_randombytes", "autotune", "autotune_load", "tune_get",
    "tune_set", "GEMM_POPC", "GEMM_B1MMA", "GEMM_TC", "GEMM_SPARSE",
]

SETS = ("348864", "460896", "6688128", "6960119", "8192128")
# set id = set + 5 v: v = 0 the set, 1 "pc" (plaintext confirmation: same keys, ciphertexts 32 bytes longer),
# 2 "f" (semi-systematic keys, same enc/dec), 3 "pcf"
VARIANTS = tuple(s + v for v in ("", "pc", "f", "pcf") for s in SETS)
GEMM_POPC, GEMM_B1MMA, GEMM_TC, GEMM_SPARSE = 0, 1, 2, 3
_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of device memory", -4: "bad key"}

_lib = None


class GmcError(RuntimeError):
    pass


def lib():
    """Loads libgmc.so (building it first when the sources are newer)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path) or os.environ.get("GMC_AUTOBUILD", "1") == "1":
            path = _build.build()
        L = ctypes.CDLL(path)
        c_u8p = ctypes.c_void_p
        L.gmc_set_name.restype = ctypes.c_char_p
        L.gmc_last_error.restype = ctypes.c_char_p
        L.gmc_set_id.argtypes = [ctypes.c_char_p]
        L.gmc_set_sizes.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
        L.gmc_pk_load.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, c_u8p]
        L.gmc_sk_load.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, c_u8p]
        L.gmc_key_free.argtypes = [ctypes.c_void_p]
        L.gmc_key_free.restype = None
        for fn in ("gmc_enc_batch", "gmc_enc_batch_dev"):
            f = getattr(L, fn)
            f.argtypes = [ctypes.c_void_p, c_u8p, c_u8p, c_u8p, ctypes.c_longlong, ctypes.c_void_p] + (
                [ctypes.c_void_p] if fn.endswith("_dev") else [])
        for fn in ("gmc_dec_batch", "gmc_dec_batch_dev"):
            f = getattr(L, fn)
            f.argtypes = [ctypes.c_void_p, c_u8p, c_u8p, ctypes.c_longlong, ctypes.c_void_p] + (
                [ctypes.c_void_p] if fn.endswith("_dev") else [])
        L.gmc_dec_stages_dev.argtypes = [ctypes.c_void_p, c_u8p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.gmc_enc_stages_dev.argtypes = [ctypes.c_void_p, c_u8p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.gmc_gf2_gemm_dev.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p]
        for s in VARIANTS:
            for op in ("enc", "dec"):
                getattr(L, f"gmc_kem_{s}_{op}").argtypes = [c_u8p, c_u8p, c_u8p]
        L.gmc_keypair_seed.argtypes = [ctypes.c_int, c_u8p, c_u8p, c_u8p]
        L.gmc_keypair_batch.argtypes = [ctypes.c_int, c_u8p, c_u8p, c_u8p, ctypes.c_longlong]
        L.gmc_key_export.argtypes = [ctypes.c_void_p, c_u8p, ctypes.c_longlong]
        L.gmc_key_export.restype = ctypes.c_longlong
        L.gmc_key_import.argtypes = [ctypes.POINTER(ctypes.c_void_p), c_u8p, ctypes.c_longlong]
        for s in VARIANTS:
            getattr(L, f"gmc_kem_{s}_keypair").argtypes = [c_u8p, c_u8p]
            getattr(L, f"gmc_kem_{s}_keypair").restype = None
        L.gmc_plan_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_int]
        L.gmc_plan_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gmc_plan_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]
        L.gmc_plan_free.argtypes = [ctypes.c_void_p]
        L.gmc_plan_free.restype = None
        L.gmc_autotune.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_char_p]
        L.gmc_autotune_load.argtypes = [ctypes.c_char_p]
        L.gmc_tune_set.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.gmc_tune_get.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_int)]
        L.gmc_int32_peak.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.gmc_tc_f8_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
        L.gmc_b1mma_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
        L.gmc_server_latency_ms.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        L.gmc_server_worst_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gmc_tune_set_launch.argtypes = [ctypes.c_int] * 5
        L.gmc_tune_get_launch.argtypes = [ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 4
        vp = ctypes.c_void_p
        L.gmc_server_create.argtypes = [ctypes.POINTER(vp), ctypes.c_longlong, ctypes.c_int, ctypes.c_double]
        L.gmc_server_add_key.argtypes = [vp, vp]
        L.gmc_server_submit.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.gmc_server_drain.argtypes = [vp, ctypes.c_double]
        L.gmc_server_stats.argtypes = [vp, vp]
        L.gmc_server_reset_stats.argtypes = [vp]
        L.gmc_server_loadgen.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_ulonglong, vp]
        L.gmc_server_destroy.argtypes = [vp]
        L.gmc_server_destroy.restype = None
        L.gmc_server_error.argtypes = [vp]
        L.gmc_server_error.restype = ctypes.c_char_p
        L.gmc_set_randombytes.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gmc_set_randombytes.restype = None
        _lib = L
    return _lib


def _check(rc, what):
    if rc < 0:
        msg = lib().gmc_last_error().decode(errors="replace")
        raise GmcError(f"{what}: {_ERRORS.get(rc, rc)} ({msg})")
    return rc


def set_id(name):
    name = str(name)
    if name.startswith("mceliece"):
        name = name[len("mceliece"):]
    if name not in VARIANTS:
        raise GmcError(f"unknown parameter set {name!r}")
    return VARIANTS.index(name)


def set_sizes(s):
    """dict with m, n, t, mt, k, pk_bytes, sk_bytes, ct_bytes for a set (name or id)."""
    sid = s if isinstance(s, int) else set_id(s)
    out = (ctypes.c_longlong * 8)()
    _check(lib().gmc_set_sizes(sid, out), "gmc_set_sizes")
    keys = ("m", "n", "t", "mt", "k", "pk_bytes", "sk_bytes", "ct_bytes")
    return dict(zip(keys, [int(v) for v in out]))


def _u8(buf, n=None):
    a = np.frombuffer(buf, dtype=np.uint8) if isinstance(buf, (bytes, bytearray)) else np.ascontiguousarray(
        buf, dtype=np.uint8)
    if n is not None and a.size != n:
        raise GmcError(f"expected {n} bytes, got {a.size}")
    return a


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Key:
    _kind = None

    def __init__(self, set_name, key_bytes):
        self.set = set_id(set_name) if not isinstance(set_name, int) else set_name
        self.sizes = set_sizes(self.set)
        nbytes = self.sizes["pk_bytes" if self._kind == "pk" else "sk_bytes"]
        raw = _u8(key_bytes, nbytes)
        h = ctypes.c_void_p()
        loader = lib().gmc_pk_load if self._kind == "pk" else lib().gmc_sk_load
        _check(loader(ctypes.byref(h), self.set, _ptr(raw)), f"gmc_{self._kind}_load")
        self._h = h

    @property
    def handle(self):
        return self._h

    def export(self):
        """The key's device state as a self-checking byte string (gmc_key_export)."""
        n = _check(int(lib().gmc_key_export(self._h, None, 0)), "gmc_key_export")
        buf = np.zeros(n, np.uint8)
        _check(int(lib().gmc_key_export(self._h, _ptr(buf), n)), "gmc_key_export")
        return buf.tobytes()

    @classmethod
    def from_export(cls, blob):
        """Re-creates a resident key from gmc_key_export's string, without the host-side table build."""
        raw = _u8(blob)
        h = ctypes.c_void_p()
        _check(lib().gmc_key_import(ctypes.byref(h), _ptr(raw), raw.size), "gmc_key_import")
        self = cls.__new__(cls)
        self._h = h
        self.set = int(lib().gmc_key_set(h))
        self.sizes = set_sizes(self.set)
        return self

    def close(self):
        if getattr(self, "_h", None):
            lib().gmc_key_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PublicKey(_Key):
    """Device-resident public key: batched encapsulation."""
    _kind = "pk"

    def enc_batch(self, seeds):
        """seeds: n x 32 bytes -> (ct [n, ct_bytes] uint8, K [n, 32] uint8, rc [n] int32)."""
        s = _u8(seeds)
        n = s.size // 32
        if s.size != 32 * n:
            raise GmcError("seeds must be a multiple of 32 bytes")
        c = np.zeros((n, self.sizes["ct_bytes"]), np.uint8)
        k = np.zeros((n, 32), np.uint8)
        rc = np.zeros(n, np.int32)
        _check(lib().gmc_enc_batch(self._h, _ptr(c), _ptr(k), _ptr(s), n, _ptr(rc)), "gmc_enc_batch")
        return c, k, rc

    def enc_batch_dev(self, c_ptr, k_ptr, seeds_ptr, n, rc_ptr=0, stream=0):
        return _check(lib().gmc_enc_batch_dev(self._h, c_ptr, k_ptr, seeds_ptr, n, rc_ptr or None, stream or None),
                      "gmc_enc_batch_dev")


class SecretKey(_Key):
    """Device-resident secret key: batched decapsulation."""
    _kind = "sk"

    def dec_batch(self, cts):
        """cts: n x ct_bytes -> (K [n, 32] uint8, rc [n] int32)."""
        cb = self.sizes["ct_bytes"]
        c = _u8(cts)
        n = c.size // cb
        if c.size != cb * n:
            raise GmcError(f"ciphertexts must be a multiple of {cb} bytes")
        k = np.zeros((n, 32), np.uint8)
        rc = np.zeros(n, np.int32)
        _check(lib().gmc_dec_batch(self._h, _ptr(k), _ptr(c), n, _ptr(rc)), "gmc_dec_batch")
        return k, rc

    def dec_batch_dev(self, k_ptr, c_ptr, n, rc_ptr=0, stream=0):
        return _check(lib().gmc_dec_batch_dev(self._h, k_ptr, c_ptr, n, rc_ptr or None, stream or None),
                      "gmc_dec_batch_dev")


class _Group(ctypes.Structure):
    _fields_ = [("key", ctypes.c_void_p), ("n", ctypes.c_longlong), ("in_", ctypes.c_void_p),
                ("ct", ctypes.c_void_p), ("k", ctypes.c_void_p), ("rc", ctypes.c_void_p)]


class Plan:
    """A grouped launch over many keys (and parameter sets): one CUDA graph replay per launch().

    groups: iterable of (key, n, in_ptr, ct_ptr, k_ptr, rc_ptr) with device pointers; key is a PublicKey
    (encapsulation of n seeds) or SecretKey (decapsulation of n ciphertexts).
    """

    def __init__(self, groups):
        arr = (_Group * len(groups))()
        self._keys = []
        for i, (key, n, inp, ct, k, rc) in enumerate(groups):
            self._keys.append(key)
            arr[i] = _Group(key.handle, n, inp, ct or None, k, rc or None)
        h = ctypes.c_void_p()
        _check(lib().gmc_plan_create(ctypes.byref(h), ctypes.cast(arr, ctypes.c_void_p), len(groups)),
               "gmc_plan_create")
        self._h = h

    def launch(self, stream=0):
        _check(lib().gmc_plan_launch(self._h, stream or None), "gmc_plan_launch")

    def info(self):
        p, r = ctypes.c_int(), ctypes.c_longlong()
        _check(lib().gmc_plan_info(self._h, ctypes.byref(p), ctypes.byref(r)), "gmc_plan_info")
        return {"pipelines": p.value, "padded_rows": r.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().gmc_plan_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop (gmc_server_*): register keys, submit requests, read statistics."""

    STATS = ("completed", "batches", "mean_batch", "p50_ms", "p99_ms", "ops_s", "errors", "slots")
    LOADGEN = ("submitted", "completed", "ops_s", "p50_ms", "p99_ms", "mean_batch", "batches", "offered_rate")

    def __init__(self, max_batch=65536, slots=3, mem_fraction=0.5):
        h = ctypes.c_void_p()
        _check(lib().gmc_server_create(ctypes.byref(h), int(max_batch), int(slots), float(mem_fraction)),
               "gmc_server_create")
        self._h = h
        self._keys = []

    def add_key(self, key):
        _check(lib().gmc_server_add_key(self._h, key.handle), "gmc_server_add_key")
        self._keys.append(key)

    def submit(self, key, in_ptr, ct_ptr, k_ptr, rc_ptr=None, done_ptr=None):
        """Host pointers; returns at once. *done becomes 1 when outputs are written."""
        _check(lib().gmc_server_submit(self._h, key.handle, in_ptr, ct_ptr, k_ptr, rc_ptr, done_ptr),
               "gmc_server_submit")

    def drain(self, timeout_s=60.0):
        _check(lib().gmc_server_drain(self._h, float(timeout_s)), "gmc_server_drain")

    def stats(self):
        out = (ctypes.c_double * 8)()
        _check(lib().gmc_server_stats(self._h, out), "gmc_server_stats")
        d = dict(zip(self.STATS, list(out)))
        d["last_error"] = lib().gmc_server_error(self._h).decode(errors="replace")
        return d

    def reset_stats(self):
        _check(lib().gmc_server_reset_stats(self._h), "gmc_server_reset_stats")

    def loadgen(self, pairs, rate, seconds, enc_fraction=0.5, seed=1):
        """pairs: [(PublicKey, SecretKey)] registered with this server. Poisson arrivals at `rate`/s."""
        pk = (ctypes.c_void_p * len(pairs))(*[p.handle.value for p, _ in pairs])
        sk = (ctypes.c_void_p * len(pairs))(*[s.handle.value for _, s in pairs])
        out = (ctypes.c_double * 8)()
        _check(lib().gmc_server_loadgen(self._h, pk, sk, len(pairs), float(rate), float(seconds),
                                        float(enc_fraction), int(seed), out), "gmc_server_loadgen")
        res = dict(zip(self.LOADGEN, list(out)))
        res["p999_ms"] = self.latency_ms(0.999)
        res["max_ms"] = self.latency_ms(1.0)
        res["worst_batch"] = self.worst_batch()
        return res

    WORST = ("latency_ms", "queue_wait_ms", "take_ms", "group_ms", "stage_copy_ms", "issue_ms", "device_ms",
             "scatter_ms", "batches", "batches_over_5ms")

    def worst_batch(self):
        """The batch whose oldest request waited longest since the last reset, split by stage (ms)."""
        out = (ctypes.c_double * 10)()
        _check(lib().gmc_server_worst_batch(self._h, out), "gmc_server_worst_batch")
        return dict(zip(self.WORST, list(out)))

    def latency_ms(self, q):
        """q-quantile (0 < q <= 1) of the request latencies recorded since the last reset, in ms."""
        ms = ctypes.c_double()
        _check(lib().gmc_server_latency_ms(self._h, ctypes.c_double(q), ctypes.byref(ms)), "gmc_server_latency_ms")
        return ms.value

    def close(self):
        if getattr(self, "_h", None):
            lib().gmc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def keypair(set_name, seed32=None):
    """(pk, sk) as uint8 arrays; seed32 = the keypair's single randombytes draw (None: randombytes source)."""
    sid = set_name if isinstance(set_name, int) else set_id(set_name)
    sz = set_sizes(sid)
    pk = np.zeros(sz["pk_bytes"], np.uint8)
    sk = np.zeros(sz["sk_bytes"], np.uint8)
    if seed32 is None:
        getattr(lib(), f"gmc_kem_{VARIANTS[sid]}_keypair")(_ptr(pk), _ptr(sk))
    else:
        seed = _u8(bytes(seed32), 32)
        _check(lib().gmc_keypair_seed(sid, _ptr(pk), _ptr(sk), _ptr(seed)), "gmc_keypair_seed")
    return pk, sk


def keypair_batch(set_name, seeds):
    """Keys generated on the GPU, one per 32-byte seed: (pk, sk) uint8 arrays of shape
    (nkeys, pk_bytes) and (nkeys, sk_bytes), each row identical to keypair(set_name, seed)."""
    sid = set_name if isinstance(set_name, int) else set_id(set_name)
    sz = set_sizes(sid)
    seeds = np.ascontiguousarray(np.frombuffer(bytes(seeds), np.uint8) if not isinstance(seeds, np.ndarray) else seeds,
                                 dtype=np.uint8).reshape(-1, 32)
    n = seeds.shape[0]
    pk = np.zeros((n, sz["pk_bytes"]), np.uint8)
    sk = np.zeros((n, sz["sk_bytes"]), np.uint8)
    _check(lib().gmc_keypair_batch(sid, _ptr(pk), _ptr(sk), _ptr(seeds), n), "gmc_keypair_batch")
    return pk, sk


def kem_enc(set_name, pk):
    """libmceliece-shaped enc: returns (rc, ct, K); randomness from the randombytes source."""
    sz = set_sizes(set_name)
    c = np.zeros(sz["ct_bytes"], np.uint8)
    k = np.zeros(32, np.uint8)
    p = _u8(pk, sz["pk_bytes"])
    name = VARIANTS[set_name] if isinstance(set_name, int) else VARIANTS[set_id(set_name)]
    rc = getattr(lib(), f"gmc_kem_{name}_enc")(_ptr(c), _ptr(k), _ptr(p))
    if rc < -1:
        _check(rc, f"gmc_kem_{name}_enc")
    return rc, c.tobytes(), k.tobytes()


def kem_dec(set_name, ct, sk):
    """libmceliece-shaped dec: returns (rc, K)."""
    sz = set_sizes(set_name)
    c = _u8(ct, sz["ct_bytes"])
    s = _u8(sk, sz["sk_bytes"])
    k = np.zeros(32, np.uint8)
    name = VARIANTS[set_name] if isinstance(set_name, int) else VARIANTS[set_id(set_name)]
    rc = getattr(lib(), f"gmc_kem_{name}_dec")(_ptr(k), _ptr(c), _ptr(s))
    if rc < -1:
        _check(rc, f"gmc_kem_{name}_dec")
    return rc, k.tobytes()


def autotune(set_name, n=65536, cache_path=None):
    """Times the candidate configurations for a set on this GPU; returns the chosen configuration."""
    sid = set_name if isinstance(set_name, int) else set_id(set_name)
    _check(lib().gmc_autotune(sid, int(n), cache_path.encode() if cache_path else None), "gmc_autotune")
    return tune_get(sid)


def autotune_load(cache_path):
    return _check(lib().gmc_autotune_load(cache_path.encode()), "gmc_autotune_load")


def tune_get(set_name):
    sid = set_name if isinstance(set_name, int) else set_id(set_name)
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    tuned = _check(lib().gmc_tune_get(sid, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "gmc_tune_get")
    names = {GEMM_POPC: "popc", GEMM_B1MMA: "b1mma", GEMM_TC: "tc", GEMM_SPARSE: "sparse"}
    g, w1, w2, w3 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(lib().gmc_tune_get_launch(sid, ctypes.byref(g), ctypes.byref(w1), ctypes.byref(w2), ctypes.byref(w3)),
           "gmc_tune_get_launch")
    return {"enc_engine": names[a.value], "dec_engine": names[b.value], "sample_threads": c.value,
            "sample_sm_warps": w3.value, "gemm_stages": g.value, "bm_warps": w1.value, "root_warps": w2.value,
            "tuned": bool(tuned)}


def tune_set(set_name, enc_engine, dec_engine, sample_threads, gemm_stages=None, bm_warps=None, root_warps=None,
             sample_sm_warps=None):
    """Sets a parameter set's launch configuration; the launch-shape arguments
    left as None keep their current values."""
    sid = set_name if isinstance(set_name, int) else set_id(set_name)
    ids = {"popc": GEMM_POPC, "b1mma": GEMM_B1MMA, "tc": GEMM_TC, "sparse": GEMM_SPARSE}
    _check(lib().gmc_tune_set(sid, ids[enc_engine], ids[dec_engine], int(sample_threads)), "gmc_tune_set")
    shape = (gemm_stages, bm_warps, root_warps, sample_sm_warps)
    if any(v is not None for v in shape):
        cur = tune_get(sid)
        vals = [cur[k] if v is None else v
                for k, v in zip(("gemm_stages", "bm_warps", "root_warps", "sample_sm_warps"), shape)]
        _check(lib().gmc_tune_set_launch(sid, *[int(v) for v in vals]), "gmc_tune_set_launch")


def int32_peak():
    """Measured integer-pipe rates of the current GPU: {"lop3_per_s", "shf_per_s"} (lane-ops per second)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(lib().gmc_int32_peak(ctypes.byref(a), ctypes.byref(b)), "gmc_int32_peak")
    return {"lop3_per_s": a.value, "shf_per_s": b.value}


def set_dec_constant_time(on):
    """Constant-time decapsulation kernels (True) or the table forms (False); identical session keys."""
    _check(lib().gmc_set_dec_constant_time(1 if on else 0), "gmc_set_dec_constant_time")


def get_dec_constant_time():
    return bool(lib().gmc_get_dec_constant_time())


def b1mma_peak():
    """Measured bit-MACs per second of mma.sync m8n8k128 .b1 AND.POPC with register operands."""
    a = ctypes.c_double()
    _check(lib().gmc_b1mma_peak(ctypes.byref(a)), "gmc_b1mma_peak")
    return a.value


def tc_f8_peak():
    """Measured multiply-accumulates per second of the tcgen05 FP8 MMA the GF(2) GEMM engine issues."""
    a = ctypes.c_double()
    _check(lib().gmc_tc_f8_peak(ctypes.byref(a)), "gmc_tc_f8_peak")
    return a.value


def set_gemm_engine(engine):
    _check(lib().gmc_set_gemm_engine(int(engine)), "gmc_set_gemm_engine")


def get_gemm_engine():
    return lib().gmc_get_gemm_engine()


_RNG_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_ubyte), ctypes.c_longlong)
_rng_keepalive = None


def set_randombytes(fn):
    """fn(n) -> bytes of length n, or None for the OS generator (the one-request enc and keypair calls)."""
    global _rng_keepalive
    if fn is None:
        lib().gmc_set_randombytes(None, None)
        _rng_keepalive = None
        return

    def cb(_ctx, out, n):
        data = fn(int(n))
        ctypes.memmove(out, data, int(n))

    _rng_keepalive = _RNG_CB(cb)
    lib().gmc_set_randombytes(ctypes.cast(_rng_keepalive, ctypes.c_void_p), None)
