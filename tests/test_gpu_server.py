"""Serving loop (gmc_server_*): requests submitted from several host threads,
in random order, over all five parameter sets and two plaintext-confirmation
(pc) forms, enc and dec mixed; each result
must be the one the request gets alone (one-request batch), bit for bit; the
dispatcher must have formed multi-request batches; the open-loop Poisson load
generator completes every request it submits."""
import ctypes
import threading

import numpy as np
import pytest

from tests.conftest import SETS, key_seed, request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


@pytest.fixture(scope="module")
def pairs(gmc):
    out = []
    for sid in range(5):
        pk, sk = gmc.keypair(sid, key_seed(sid))
        out.append((sid, pk, sk, gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)))
    # plaintext-confirmation forms of two sets (same key bytes, 32-byte-longer ciphertexts)
    for sid in (0, 4):
        _, pk, sk, _, _ = out[sid]
        out.append((sid + 5, pk, sk, gmc.PublicKey(sid + 5, pk), gmc.SecretKey(sid + 5, sk)))
    return out


def test_results_in_the_mix_equal_results_alone(gmc, pairs):
    srv = gmc.Server(max_batch=1024, slots=3, mem_fraction=0.2)
    for _, _, _, P, S in pairs:
        srv.add_key(P)
        srv.add_key(S)
    rng = np.random.default_rng(5)
    reqs = []
    for sid, pk, sk, P, S in pairs:
        z = gmc.set_sizes(sid)
        seeds = request_seeds(sid % 5, 150, b"srv" + bytes([sid]))
        cts, _, _ = P.enc_batch(request_seeds(sid % 5, 150, b"srvd" + bytes([sid])))
        flip = rng.choice(150, 15, replace=False)
        for i in flip:
            b = int(rng.integers(0, z["mt"]))
            cts[i, b // 8] ^= np.uint8(1 << (b % 8))
        for i in range(150):
            reqs.append(("enc", sid, P, seeds[i].copy(), np.zeros(z["ct_bytes"], np.uint8)))
            reqs.append(("dec", sid, S, cts[i].copy(), None))
    order = rng.permutation(len(reqs))
    n = len(reqs)
    k_out = np.zeros((n, 32), np.uint8)
    rc_out = np.full(n, 7, np.int32)
    done = np.zeros(n, np.int32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)

    def submitter(idx):
        for j in idx:
            j = int(j)
            op, sid, key, inp, ct = reqs[j]
            srv.submit(key, p(inp), p(ct) if ct is not None else None,
                       k_out[j].ctypes.data_as(ctypes.c_void_p),
                       ctypes.c_void_p(rc_out.ctypes.data + 4 * j),
                       ctypes.c_void_p(done.ctypes.data + 4 * j))

    threads = [threading.Thread(target=submitter, args=(order[t::3],)) for t in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    srv.drain(120)
    st = srv.stats()
    assert (done == 1).all(), (st["last_error"], st["errors"], st["completed"], int((done == -1).sum()))
    assert st["completed"] == n and st["errors"] == 0
    assert st["batches"] < n and st["mean_batch"] > 1.0, st
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    # every request alone
    for j, (op, sid, key, inp, ct) in enumerate(reqs):
        if op == "enc":
            c1, k1, r1 = key.enc_batch(inp.reshape(1, 32))
            assert (ct == c1[0]).all() and (k_out[j] == k1[0]).all() and rc_out[j] == r1[0], j
        else:
            k1, r1 = key.dec_batch(inp.reshape(1, -1))
            assert (k_out[j] == k1[0]).all() and rc_out[j] == r1[0], j
    srv.close()


def test_poisson_loadgen(gmc, pairs):
    srv = gmc.Server(max_batch=8192, slots=3, mem_fraction=0.2)
    plist = []
    for _, _, _, P, S in pairs:
        srv.add_key(P)
        srv.add_key(S)
        plist.append((P, S))
    r = srv.loadgen(plist, rate=20000.0, seconds=1.0, seed=9)
    assert r["submitted"] > 10000 and r["completed"] == r["submitted"]
    assert 0 < r["p50_ms"] <= r["p99_ms"] <= r["p999_ms"] <= r["max_ms"]
    w = r["worst_batch"]  # the slowest batch and its stages (all non-negative, summing to its latency)
    parts = ("queue_wait_ms", "take_ms", "group_ms", "stage_copy_ms", "issue_ms", "device_ms", "scatter_ms")
    assert w["batches"] > 0 and all(w[p_] >= 0 for p_ in parts)
    assert abs(sum(w[p_] for p_ in parts) - w["latency_ms"]) < 0.05 * w["latency_ms"] + 0.01
    srv.close()
