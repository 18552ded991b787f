"""GPU parity for the plaintext-confirmation ("pc") variants, set ids 5..9
(mc:crypto_kem/<set>pc): the same keys as the base set, ciphertexts C0 || C1
with C1 = SHAKE256(2 || e, 32), the session key over C0 || C1, and
decapsulation rejecting when C1 does not match the decoded e. Every byte is
compared with the oracle, whose pc restatement is pinned by libmceliece's
pc known-answer checksums (tests/test_oracle_kat.py).
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import SETS, request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
THREADS = min(16, os.cpu_count() or 1)
PC = {s: 5 + i for i, s in enumerate(SETS)}


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def corrupted(sid, cts, seed=0):
    """Valid ciphertexts, 10% with one bit of C0 flipped, 10% with one bit of C1 flipped (pc ids only), plus
    random ones."""
    rng = np.random.default_rng(seed + 31 * sid)
    z = O.sizes(sid)
    out = cts.copy()
    n = len(cts)
    idx = rng.permutation(n)
    c0, c1 = idx[: n // 10], idx[n // 10: n // 5]
    for i in c0:
        bit = int(rng.integers(0, z["mt"]))
        out[i, bit // 8] ^= np.uint8(1 << (bit % 8))
    sb = (z["mt"] + 7) // 8
    for i in (c1 if (sid // 5) & 1 else []):
        bit = int(rng.integers(0, 256))
        out[i, sb + bit // 8] ^= np.uint8(1 << (bit % 8))
    rnd = rng.integers(0, 256, size=(8, z["ct_bytes"]), dtype=np.uint8)
    if z["mt"] % 8:
        rnd[:4, sb - 1] &= np.uint8((1 << (z["mt"] % 8)) - 1)
    return np.concatenate([out, rnd])


def test_pc_ids_and_sizes(gmc):
    for s, sid in PC.items():
        assert gmc.set_id(s + "pc") == sid and gmc.set_id("mceliece" + s + "pc") == sid
        base, pc = gmc.set_sizes(SETS.index(s)), gmc.set_sizes(sid)
        assert pc["ct_bytes"] == base["ct_bytes"] + 32
        assert pc["pk_bytes"] == base["pk_bytes"] and pc["sk_bytes"] == base["sk_bytes"]
        assert pc == O.sizes(sid)


@pytest.mark.parametrize("base", range(5), ids=SETS)
def test_pc_enc_dec_parity(gmc, keys, base):
    sid = base + 5
    pk, sk = keys(base)  # pc keys are the base set's keys
    n = 200
    seeds = request_seeds(base, n, b"pc")
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
    oc, ok_, orc = O.enc_batch(sid, pk, seeds, threads=THREADS)
    assert (rc == orc).all()
    assert (c == oc).all(), f"{int((c != oc).any(1).sum())} ciphertexts differ"
    assert (k == ok_).all(), f"{int((k != ok_).any(1).sum())} session keys differ"
    cts = corrupted(sid, c)
    kd, rcd = gmc.SecretKey(sid, sk).dec_batch(cts)
    okd, orcd = O.dec_batch(sid, sk, cts, threads=THREADS)
    assert (rcd == orcd).all()
    assert (kd == okd).all(), f"{int((kd != okd).any(1).sum())} decapsulated keys differ"
    # the valid ones round-trip; a flipped C1 bit is rejected (implicit rejection key != encapsulated key)
    assert (kd[: n] == k).all(1).sum() == n - n // 5


def test_pc_and_base_keys_differ_only_in_ciphertext_form(gmc, keys):
    base = 0
    pk, sk = keys(base)
    seeds = request_seeds(base, 16, b"pc-vs-base")
    c0, k0, _ = gmc.PublicKey(base, pk).enc_batch(seeds)
    c1, k1, _ = gmc.PublicKey(base + 5, pk).enc_batch(seeds)
    assert (c1[:, : c0.shape[1]] == c0).all()  # the same e: the same C0
    assert not (k1 == k0).all(1).any()         # the session key covers C1 too


def test_pc_single_calls(gmc, keys):
    base = 1
    sid = base + 5
    pk, sk = keys(base)
    rc, ct, k = gmc.kem_enc(sid, pk)
    assert rc == 0 and len(ct) == O.sizes(sid)["ct_bytes"]
    rc2, k2 = gmc.kem_dec(sid, ct, sk)
    assert rc2 == 0 and k2 == k
    okey = np.zeros(32, np.uint8)
    assert O.lib().gmo_dec(sid, O._p(okey), O._p(np.frombuffer(ct, np.uint8).copy()), O._p(sk)) == 0
    assert okey.tobytes() == k2


def test_pc_grouped_plan_matches_per_key_calls(gmc, keys):
    """A plan holding base and pc keys of the same set runs them as separate pipelines."""
    dev = torch.device("cuda", 0)
    groups, refs = [], []
    for base in (0, 4):
        pk, sk = keys(base)
        for sid in (base, base + 5):
            n = 96 + 17 * sid
            seeds = torch.from_numpy(request_seeds(base, n, b"pc-plan%d" % sid)).to(dev)
            z = gmc.set_sizes(sid)
            P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
            c_ref, k_ref, _ = P.enc_batch(seeds.cpu().numpy())
            cts = torch.from_numpy(corrupted(sid, c_ref, seed=sid)).to(dev)
            kd_ref, rcd_ref = S.dec_batch(cts.cpu().numpy())
            c = torch.zeros((n, z["ct_bytes"]), dtype=torch.uint8, device=dev)
            k = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
            kd = torch.zeros((cts.shape[0], 32), dtype=torch.uint8, device=dev)
            rcd = torch.zeros(cts.shape[0], dtype=torch.int32, device=dev)
            groups.append((P, n, seeds.data_ptr(), c.data_ptr(), k.data_ptr(), 0))
            groups.append((S, cts.shape[0], cts.data_ptr(), 0, kd.data_ptr(), rcd.data_ptr()))
            refs.append((seeds, cts, c, k, kd, rcd, c_ref, k_ref, kd_ref, rcd_ref))
    plan = gmc.Plan(groups)
    assert plan.info()["pipelines"] == 8
    plan.launch()
    torch.cuda.synchronize()
    for (_, _, c, k, kd, rcd, c_ref, k_ref, kd_ref, rcd_ref) in refs:
        assert (c.cpu().numpy() == c_ref).all() and (k.cpu().numpy() == k_ref).all()
        assert (kd.cpu().numpy() == kd_ref).all() and (rcd.cpu().numpy() == rcd_ref).all()
    plan.close()


def test_pc_full_size_round_trip(gmc, keys):
    base = 4
    sid = base + 5
    pk, sk = keys(base)
    n = 16384
    seeds = request_seeds(base, n, b"pc-full")
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
    kd, rcd = gmc.SecretKey(sid, sk).dec_batch(c)
    assert (rc == 0).all() and (rcd == 0).all() and (kd == k).all()
    oc, ok_, _ = O.enc_batch(sid, pk, seeds[:256], threads=THREADS)
    assert (c[:256] == oc).all() and (k[:256] == ok_).all()


@pytest.mark.parametrize("sid", [13, 17, 19], ids=["6960119f", "6688128pcf", "8192128pcf"])
def test_semi_systematic_keys_enc_dec_parity(gmc, sid):
    """f / pcf variants: semi-systematic keys through the set's (or its pc form's) enc and dec."""
    import hashlib
    base = sid % 5
    pk, sk = O.keypair(sid, hashlib.sha256(b"semi-enc" + bytes([sid])).digest())
    seeds = request_seeds(base, 120, b"semi%d" % sid)
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
    oc, ok_, orc = O.enc_batch(sid, pk, seeds, threads=THREADS)
    assert (rc == orc).all() and (c == oc).all() and (k == ok_).all()
    cts = corrupted(sid, c)
    kd, rcd = gmc.SecretKey(sid, sk).dec_batch(cts)
    okd, orcd = O.dec_batch(sid, sk, cts, threads=THREADS)
    assert (rcd == orcd).all() and (kd == okd).all()


def test_pc_keys_in_the_serving_loop(gmc, keys):
    """pc keys are served next to plain keys of the same set (separate
    pipelines): results equal the batch calls, ciphertexts 32 bytes longer."""
    import ctypes
    pk, sk = keys(0)
    P, S, Pp, Sp = gmc.PublicKey(0, pk), gmc.SecretKey(0, sk), gmc.PublicKey(5, pk), gmc.SecretKey(5, sk)
    srv = gmc.Server(max_batch=1024, slots=2, mem_fraction=0.05)
    for key in (P, S, Pp, Sp):
        srv.add_key(key)
    seeds = request_seeds(0, 40, b"pcsrv")
    ref_c, ref_k, _ = Pp.enc_batch(seeds)
    plain_c, plain_k, _ = P.enc_batch(seeds)
    z = gmc.set_sizes(5)
    c_out = np.zeros((40, z["ct_bytes"]), np.uint8)
    k_out = np.zeros((40, 32), np.uint8)
    c2_out = np.zeros((40, gmc.set_sizes(0)["ct_bytes"]), np.uint8)
    k2_out = np.zeros((40, 32), np.uint8)
    kd_out = np.zeros((40, 32), np.uint8)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for i in range(40):
        srv.submit(Pp, p(seeds[i]), p(c_out[i]), p(k_out[i]))
        srv.submit(P, p(seeds[i]), p(c2_out[i]), p(k2_out[i]))
        srv.submit(Sp, p(ref_c[i]), None, p(kd_out[i]))
    srv.drain(60)
    assert srv.stats()["errors"] == 0
    assert (c_out == ref_c).all() and (k_out == ref_k).all() and (kd_out == ref_k).all()
    assert (c2_out == plain_c).all() and (k2_out == plain_k).all()
    srv.close()
