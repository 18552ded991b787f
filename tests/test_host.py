"""CPU-only tests of the engine's host side: the C ABI library loads and exports
every symbol include/gmc.h declares, argument checking, and the per-key /
per-field tables it would upload (checked against the oracle through a CPU
model of the decode kernel)."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import ROOT, SETS, request_seeds

HEADER = os.path.join(ROOT, "include", "gmc.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gmc_[a-z0-9_]+)\s*\(", text)
    return sorted(set(n for n in names if not n.endswith("_fn")))


def test_library_exports_every_declared_symbol():
    import tensormceliece_gb300 as gmc
    L = gmc.lib()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_set_table():
    import tensormceliece_gb300 as gmc
    for sid, name in enumerate(SETS):
        z, oz = gmc.set_sizes(sid), O.sizes(sid)
        assert z == oz
        assert gmc.lib().gmc_set_id(name.encode()) == sid
        assert gmc.lib().gmc_set_id(("mceliece" + name).encode()) == sid
    assert gmc.lib().gmc_set_id(b"nope") == -1
    # plaintext-confirmation variants: ids 5..9, same keys, 32 more ciphertext bytes
    for i, name in enumerate(SETS):
        sid = 5 + i
        assert gmc.lib().gmc_set_id((name + "pc").encode()) == sid
        assert gmc.lib().gmc_set_name(sid) == (name + "pc").encode()
        z = gmc.set_sizes(sid)
        assert z == O.sizes(sid) and z["ct_bytes"] == gmc.set_sizes(i)["ct_bytes"] + 32
    assert gmc.lib().gmc_set_name(20) is None
    for sid, name in enumerate(gmc.VARIANTS):
        assert gmc.lib().gmc_set_id(name.encode()) == sid and gmc.set_sizes(sid) == O.sizes(sid)


def test_no_gpu_fails_loudly():
    """Without a usable device the engine returns an error: there is no CPU path."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import tensormceliece_gb300 as gmc
    pk, _ = O.keypair(0, bytes(32))
    with pytest.raises(gmc.GmcError):
        gmc.PublicKey(0, pk)
    with pytest.raises(gmc.GmcError):
        gmc.kem_enc(0, pk)


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_support_and_front_end_tables(keys, sid):
    """Support L and front-end matrix F from the secret key agree with the oracle."""
    from tests import decode_model as DM
    pk, sk = keys(sid)
    L, Lp, F = DM.sk_tables(sid, sk)
    OL = np.zeros(O.sizes(sid)["n"], np.uint16)
    O.lib().gmo_support(sid, sk.ctypes.data_as(ctypes.c_void_p), OL.ctypes.data_as(ctypes.c_void_p), None)
    assert (L == OL).all()


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_decode_algorithm_model(keys, sid):
    """The decode kernel's algorithm (with the engine's tables) reproduces the oracle's stages."""
    from tests import decode_model as DM
    pk, sk = keys(sid)
    tb = DM.host_tables(sid)
    skt = DM.sk_tables(sid, sk)
    t = O.sizes(sid)["t"]
    seeds = request_seeds(sid, 2, b"model")
    for i in range(2):
        rc, c, k = O.enc(sid, pk, seeds[i].tobytes())
        for variant in (c, np.bitwise_xor(c, np.eye(1, len(c), 1 + i, dtype=np.uint8)[0] * (1 << i))):
            orc, sp, loc, e = O.decrypt_stages(sid, sk, variant)
            s, C, e2, w = DM.decode(sid, sk, variant, tb, skt)
            assert s == [int(x) for x in sp]
            assert [C[t - j] for j in range(t + 1)] == [int(x) for x in loc]
            if orc == 0:
                assert (e == e2).all() and w == t


def test_golden_fixtures_match_oracle(keys):
    import hashlib
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "kem_vectors.json")))
    for sid, name in enumerate(SETS):
        pk, sk = keys(sid)
        assert hashlib.sha256(pk.tobytes()).hexdigest() == g[name]["pk_sha256"]
        assert hashlib.sha256(sk.tobytes()).hexdigest() == g[name]["sk_sha256"]
        for v in g[name]["enc"]:
            rc, c, k = O.enc(sid, pk, bytes.fromhex(v["seed"]))
            assert c.tobytes().hex() == v["ct"] and k.tobytes().hex() == v["k"]
        for v in g[name]["flipped"] + ([g[name]["padding"]] if "padding" in g[name] else []):
            rc, k = O.dec(sid, bytes.fromhex(v["ct"]), sk)
            assert k.tobytes().hex() == v["k"] and rc == v["rc"]


def test_key_import_rejects_foreign_strings():
    """gmc_key_import checks magic, version, dimensions and checksum on the host, before any device work."""
    import ctypes
    import tensormceliece_gb300 as gmc
    L = gmc.lib()
    h = ctypes.c_void_p()
    junk = np.frombuffer(b"not a key string" * 16, np.uint8).copy()
    assert L.gmc_key_import(ctypes.byref(h), junk.ctypes.data_as(ctypes.c_void_p), junk.size) == -4  # GMC_EKEY
    assert L.gmc_key_import(ctypes.byref(h), junk.ctypes.data_as(ctypes.c_void_p), 8) == -1  # too short


def test_tune_cache_load_on_host(tmp_path):
    """gmc_autotune_load applies a JSON cache on the host (no device work):
    known fields are taken, out-of-range launch shapes fall back to their
    defaults, and sets absent from the file keep their configuration."""
    import tensormceliece_gb300 as gmc
    before = {s: gmc.tune_get(s) for s in ("460896", "6688128")}
    cache = {"gpu": "any", "sets": {
        "348864": {"enc_engine": "tc", "dec_engine": "popc", "sample_threads": 64, "sample_sm_warps": 8,
                   "gemm_stages": 3, "bm_warps": 4, "root_warps": 2, "n": 4096, "enc_ms": 0.1, "dec_ms": 0.2},
        "8192128": {"enc_engine": "sparse", "dec_engine": "sparse", "sample_threads": 100, "sample_sm_warps": 99,
                    "gemm_stages": 7, "bm_warps": 0, "root_warps": 12, "n": 1, "enc_ms": 1, "dec_ms": 1}}}
    path = tmp_path / "tune.json"
    path.write_text(json.dumps(cache, indent=2))
    try:
        assert gmc.autotune_load(str(path)) == 2
        a = gmc.tune_get("348864")
        assert a["tuned"] and (a["enc_engine"], a["dec_engine"], a["sample_threads"]) == ("tc", "popc", 64)
        assert (a["sample_sm_warps"], a["gemm_stages"], a["bm_warps"], a["root_warps"]) == (8, 3, 4, 2)
        b = gmc.tune_get("8192128")
        # no sparse front end for decapsulation; invalid shapes take the defaults
        assert b["dec_engine"] == "tc" and b["sample_threads"] == 128
        assert (b["sample_sm_warps"], b["gemm_stages"], b["bm_warps"], b["root_warps"]) == (0, 4, 14, 8)
        for s, t in before.items():
            assert gmc.tune_get(s) == t
    finally:
        for s in ("348864", "8192128"):
            gmc.tune_set(s, "sparse", "tc", 128, gemm_stages=4, bm_warps=14, root_warps=8, sample_sm_warps=0)
