"""The autotuner: measures, persists to a JSON cache, reloads, and the tuned
configuration still gives byte-exact results."""
import json

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def test_autotune_cache_roundtrip(gmc, keys, tmp_path):
    path = str(tmp_path / "tune.json")
    cfg = gmc.autotune(0, 4096, path)
    assert cfg["tuned"] and cfg["sample_threads"] in (32, 64, 128)
    data = json.load(open(path))
    entry = data["sets"]["348864"]
    assert entry["enc_engine"] == cfg["enc_engine"]
    assert entry["gemm_stages"] in (2, 3, 4) and entry["root_warps"] in (2, 4, 8) and entry["bm_warps"] == 14
    assert entry["sample_sm_warps"] in (0, 8, 16)
    gmc.tune_set(0, "popc", "popc", 32, gemm_stages=2, bm_warps=1, root_warps=1, sample_sm_warps=4)
    assert gmc.autotune_load(path) == 1
    got = gmc.tune_get(0)
    for f in ("enc_engine", "dec_engine", "sample_threads", "gemm_stages", "bm_warps", "root_warps",
              "sample_sm_warps"):
        assert got[f] == cfg[f], f
    pk, sk = keys(0)
    seeds = request_seeds(0, 200, b"tune")
    c, k, _ = gmc.PublicKey(0, pk).enc_batch(seeds)
    oc, ok_, _ = O.enc_batch(0, pk, seeds, threads=8)
    assert (c == oc).all() and (k == ok_).all()
    k2, _ = gmc.SecretKey(0, sk).dec_batch(c)
    assert (k2 == k).all()


@pytest.mark.parametrize("threads", [32, 128])
def test_sampler_block_sizes(gmc, keys, threads):
    sid = 4
    pk, _ = keys(sid)
    prev = gmc.tune_get(sid)
    gmc.tune_set(sid, prev["enc_engine"], prev["dec_engine"], threads)
    try:
        seeds = request_seeds(sid, 300, b"threads")
        c, k, _ = gmc.PublicKey(sid, pk).enc_batch(seeds)
        oc, ok_, _ = O.enc_batch(sid, pk, seeds, threads=8)
        assert (c == oc).all() and (k == ok_).all()
    finally:
        gmc.tune_set(sid, prev["enc_engine"], prev["dec_engine"], prev["sample_threads"])


@pytest.mark.parametrize("sid", [2, 4], ids=["6960119", "8192128"])
def test_launch_shapes(gmc, keys, sid):
    """Every GEMM pipeline depth and decoding block shape the tuner may pick
    gives the results of the default shape, on a batch large enough for the
    bit-sliced Berlekamp-Massey form, with invalid ciphertexts mixed in."""
    pk, sk = keys(sid)
    prev = gmc.tune_get(sid)
    n = 24576 + 77
    seeds = request_seeds(sid, n, b"shapes")
    try:
        gmc.tune_set(sid, "tc", "tc", prev["sample_threads"], gemm_stages=4, bm_warps=14, root_warps=8,
                     sample_sm_warps=0)
        P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
        c, k, rc = P.enc_batch(seeds)
        oc, ok_, _ = O.enc_batch(sid, pk, seeds[:64], threads=8)
        assert (c[:64] == oc).all() and (k[:64] == ok_).all()
        bad = c.copy()
        bad[::5, 3] ^= 0x21
        kd, rcd = S.dec_batch(bad)
        assert (kd[1::5] == k[1::5]).all()
        for stages, bw, rw, sw in ((2, 8, 2, 8), (3, 5, 4, 16), (4, 1, 1, 4)):
            gmc.tune_set(sid, "tc", "tc", prev["sample_threads"], gemm_stages=stages, bm_warps=bw, root_warps=rw,
                         sample_sm_warps=sw)
            c2, k2, rc2 = P.enc_batch(seeds)
            assert (c2 == c).all() and (k2 == k).all() and (rc2 == rc).all(), (stages, bw, rw)
            kd2, rcd2 = S.dec_batch(bad)
            assert (kd2 == kd).all() and (rcd2 == rcd).all(), (stages, bw, rw)
        assert gmc.lib().gmc_tc_status() == 0
    finally:
        gmc.tune_set(sid, prev["enc_engine"], prev["dec_engine"], prev["sample_threads"],
                     gemm_stages=prev["gemm_stages"], bm_warps=prev["bm_warps"], root_warps=prev["root_warps"],
                     sample_sm_warps=prev["sample_sm_warps"])


def test_int32_peak(gmc):
    """The integer-pipe microbenchmark behind the Keccak ceiling gives rates
    between 1 and 1000 T lane-ops/s for both instruction kinds."""
    pk = gmc.int32_peak()
    for k in ("lop3_per_s", "shf_per_s"):
        assert 1e12 < pk[k] < 1e15, pk
