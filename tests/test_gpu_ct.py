"""Constant-time decapsulation (gmc_set_dec_constant_time): the inversion-free, table-free Berlekamp-Massey with
slot counts fixed by the iteration, the root finder's table-free twist, the error vector taken to code positions
by the key's Benes network and checked by a dense product with the key's first-t syndrome matrix (no gather at an
error position anywhere). Session keys and return codes must be the oracle's and the table forms' on valid,
one-bit-flipped and random ciphertexts, for every set, a pc variant, batches on either side of the table form's
bit-sliced threshold, an imported key and a grouped plan; the per-request error vectors and decode flags must be
the oracle's decrypt stages."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import SETS, request_seeds
from tests.test_gpu_kem import flipped_and_random

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
THREADS = os.cpu_count() or 8


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    yield g
    g.set_dec_constant_time(False)


def dec_both(gmc, sid, sk, cts):
    key = gmc.SecretKey(sid, sk)
    gmc.set_dec_constant_time(True)
    try:
        k_ct, rc_ct = key.dec_batch(cts)
    finally:
        gmc.set_dec_constant_time(False)
    k_tab, rc_tab = key.dec_batch(cts)
    return k_ct, rc_ct, k_tab, rc_tab


@pytest.mark.parametrize("sid", [0, 1, 2, 3, 4, 9], ids=list(SETS) + ["8192128pc"])
def test_ct_decapsulation_matches_oracle(gmc, keys, sid):
    pk, sk = keys(sid % 5)
    oc, _, _ = O.enc_batch(sid, pk, request_seeds(sid % 5, 300, b"ct"), threads=THREADS)
    cts, _ = flipped_and_random(sid, oc, frac=0.2, nrand=16, seed=21)
    k_ct, rc_ct, k_tab, rc_tab = dec_both(gmc, sid, sk, cts)
    ok_, orc = O.dec_batch(sid, sk, cts, threads=THREADS)
    assert (k_ct == ok_).all() and (rc_ct == orc).all(), "constant-time keys differ from the oracle"
    assert (k_ct == k_tab).all() and (rc_ct == rc_tab).all()


@pytest.mark.parametrize("sid", [0, 4], ids=["348864", "8192128"])
def test_ct_large_batch_matches_table_form(gmc, keys, sid):
    """32768 rows (the table form's bit-sliced Berlekamp-Massey) against the constant-time form, plus an oracle
    sample of valid, flipped and random ciphertexts."""
    pk, sk = keys(sid)
    n = 32768
    rng = np.random.default_rng(31 + sid)
    c, _, _ = gmc.PublicKey(sid, pk).enc_batch(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    cts, flipped = flipped_and_random(sid, c, frac=0.1, nrand=64, seed=13)
    k_ct, rc_ct, k_tab, rc_tab = dec_both(gmc, sid, sk, cts)
    assert (k_ct == k_tab).all() and (rc_ct == rc_tab).all()
    sample = np.concatenate([rng.choice(n, 16, replace=False), flipped[:16], np.arange(n, n + 16)])
    ok_, orc = O.dec_batch(sid, sk, cts[sample], threads=THREADS)
    assert (k_ct[sample] == ok_).all() and (rc_ct[sample] == orc).all()


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_ct_error_vectors_match_oracle_stages(gmc, keys, sid):
    pk, sk = keys(sid)
    z = O.sizes(sid)
    oc, _, _ = O.enc_batch(sid, pk, request_seeds(sid, 64, b"ct-stages"), threads=THREADS)
    cts, _ = flipped_and_random(sid, oc, frac=0.25, nrand=4)
    n = len(cts)
    lde = max((1 << z["m"]) // 32, ((z["n"] + 31) // 32 + 7) // 8 * 8)  # the constant-time row stride
    lds2 = (((2 * z["t"] * z["m"] + 31) // 32) + 3) // 4 * 4
    dev = torch.device("cuda")
    d_c = torch.from_numpy(cts).to(dev)
    d_s = torch.zeros((n, lds2), dtype=torch.int32, device=dev)
    d_e = torch.zeros((n, lde), dtype=torch.int32, device=dev)
    d_ok = torch.zeros(n, dtype=torch.int32, device=dev)
    key = gmc.SecretKey(sid, sk)
    gmc.set_dec_constant_time(True)
    try:
        assert gmc.lib().gmc_dec_stages_dev(key.handle, d_c.data_ptr(), n, d_s.data_ptr(), lds2, d_e.data_ptr(),
                                            lde, d_ok.data_ptr(), None) == 0
        torch.cuda.synchronize()
    finally:
        gmc.set_dec_constant_time(False)
    E = d_e.cpu().numpy().view(np.uint32)
    OK = d_ok.cpu().numpy()
    for i in range(n):
        orc, _, _, e = O.decrypt_stages(sid, sk, cts[i])
        assert OK[i] == (1 if orc == 0 else 0), f"request {i}: decode flag"
        if orc == 0:
            assert (E[i].view(np.uint8)[: z["n"] // 8] == e).all(), f"request {i}: error vector differs"


def test_ct_imported_key_and_grouped_plan(gmc, keys):
    """A secret key re-created from its exported string (which carries the Benes control bits), and a grouped plan
    created under the switch, give the table forms' keys."""
    dev = torch.device("cuda")
    sids = [4, 3]
    bufs, groups, refs = [], [], []
    for sid in sids:
        pk, sk = keys(sid)
        oc, _, _ = O.enc_batch(sid, pk, request_seeds(sid, 200, b"ct-plan"), threads=THREADS)
        cts, _ = flipped_and_random(sid, oc, frac=0.2, nrand=8, seed=5)
        S = gmc.SecretKey(sid, sk)
        k_tab, rc_tab = S.dec_batch(cts)
        S2 = gmc.SecretKey.from_export(S.export())
        gmc.set_dec_constant_time(True)
        try:
            k_imp, rc_imp = S2.dec_batch(cts)
        finally:
            gmc.set_dec_constant_time(False)
        assert (k_imp == k_tab).all() and (rc_imp == rc_tab).all()
        d_c = torch.from_numpy(cts).to(dev)
        d_k = torch.zeros((len(cts), 32), dtype=torch.uint8, device=dev)
        d_rc = torch.zeros(len(cts), dtype=torch.int32, device=dev)
        bufs.append((S, d_c, d_k, d_rc))
        groups.append((S, len(cts), d_c.data_ptr(), 0, d_k.data_ptr(), d_rc.data_ptr()))
        refs.append((k_tab, rc_tab))
    gmc.set_dec_constant_time(True)
    try:
        plan = gmc.Plan(groups)
    finally:
        gmc.set_dec_constant_time(False)
    plan.launch(torch.cuda.current_stream().cuda_stream)  # the form is fixed when the plan is created
    torch.cuda.synchronize()
    plan.close()
    for (S, d_c, d_k, d_rc), (k_tab, rc_tab) in zip(bufs, refs):
        assert (d_k.cpu().numpy() == k_tab).all() and (d_rc.cpu().numpy() == rc_tab).all()


def test_ct_switch(gmc):
    assert gmc.get_dec_constant_time() is False
    gmc.set_dec_constant_time(True)
    assert gmc.get_dec_constant_time() is True
    gmc.set_dec_constant_time(False)
    assert gmc.lib().gmc_set_dec_constant_time(2) == -1


def test_ct_serving_loop(gmc, keys):
    """Decapsulations served under the switch (several keys and sets in one batch, the keys' first-t syndrome
    matrices built on their first constant-time batch) equal the table form's results."""
    import ctypes
    srv = gmc.Server(max_batch=4096, slots=2, mem_fraction=0.1)
    items = []
    for sid in (0, 3, 4, 9):
        pk, sk = keys(sid % 5)
        S = gmc.SecretKey(sid, sk)
        srv.add_key(S)
        oc, _, _ = O.enc_batch(sid, pk, request_seeds(sid % 5, 40, b"ct-srv"), threads=THREADS)
        cts, _ = flipped_and_random(sid, oc, frac=0.2, nrand=4, seed=9)
        k_tab, rc_tab = S.dec_batch(cts)
        items += [(S, cts[i].copy(), k_tab[i], rc_tab[i]) for i in range(len(cts))]
    n = len(items)
    k_out = np.zeros((n, 32), np.uint8)
    rc_out = np.full(n, 7, np.int32)
    done = np.zeros(n, np.int32)
    gmc.set_dec_constant_time(True)
    try:
        for j, (S, c, _, _) in enumerate(items):
            srv.submit(S, c.ctypes.data_as(ctypes.c_void_p), None, ctypes.c_void_p(k_out.ctypes.data + 32 * j),
                       ctypes.c_void_p(rc_out.ctypes.data + 4 * j), ctypes.c_void_p(done.ctypes.data + 4 * j))
        srv.drain(120)
    finally:
        gmc.set_dec_constant_time(False)
    st = srv.stats()
    srv.close()
    assert (done == 1).all(), st["last_error"]
    for j, (_, _, k_tab, rc_tab) in enumerate(items):
        assert (k_out[j] == k_tab).all() and rc_out[j] == rc_tab, j
