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
    assert data["sets"]["348864"]["enc_engine"] == cfg["enc_engine"]
    gmc.tune_set(0, "popc", "popc", 32)
    assert gmc.autotune_load(path) == 1
    assert gmc.tune_get(0)["enc_engine"] == cfg["enc_engine"]
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
