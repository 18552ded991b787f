"""GPU parity tests: every ciphertext and session key byte-exact against the oracle.

Calls go through the C ABI (include/gmc.h) via the ctypes mirror. Every
request of every batch is checked, including the full-size case (65536
requests), which is compared with libmceliece itself on all host threads.
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import SETS, key_seed, request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kem_vectors.json")))
THREADS = min(16, os.cpu_count() or 1)


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def flipped_and_random(sid, cts, frac=0.1, nrand=8, seed=0):
    """10% of the ciphertexts with one uniformly random bit flipped in the mt syndrome bits, plus random ones."""
    rng = np.random.default_rng(seed + 17 * sid)
    z = O.sizes(sid)
    out = cts.copy()
    idx = rng.choice(len(cts), size=max(1, int(frac * len(cts))), replace=False)
    for i in idx:
        bit = int(rng.integers(0, z["mt"]))
        out[i, bit // 8] ^= np.uint8(1 << (bit % 8))
    rnd = rng.integers(0, 256, size=(nrand, z["ct_bytes"]), dtype=np.uint8)
    if z["mt"] % 8:
        rnd[: nrand // 2, -1] &= np.uint8((1 << (z["mt"] % 8)) - 1)  # half with clean padding
    return np.concatenate([out, rnd]), idx


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_enc_parity(gmc, keys, sid):
    pk, _ = keys(sid)
    n = 300
    seeds = request_seeds(sid, n)
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
    oc, okey, orc = O.enc_batch(sid, pk, seeds, threads=THREADS)
    assert (rc == orc).all()
    assert (c == oc).all(), f"{int((c != oc).any(1).sum())} ciphertexts differ"
    assert (k == okey).all(), f"{int((k != okey).any(1).sum())} session keys differ"


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_dec_parity(gmc, keys, sid):
    pk, sk = keys(sid)
    n = 256
    seeds = request_seeds(sid, n, b"dec")
    oc, okey, _ = O.enc_batch(sid, pk, seeds, threads=THREADS)
    cts, flipped = flipped_and_random(sid, oc)
    k, rc = gmc.SecretKey(sid, sk).dec_batch(cts)
    ok2, orc = O.dec_batch(sid, sk, cts, threads=THREADS)
    assert (rc == orc).all()
    assert (k == ok2).all(), f"{int((k != ok2).any(1).sum())} session keys differ"
    valid = np.setdiff1d(np.arange(n), flipped)
    assert (k[valid] == okey[valid]).all()          # valid ciphertexts decapsulate to the enc key
    assert (k[flipped] != okey[flipped]).any(1).all()  # flipped ones take the rejection branch


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_golden_vectors(gmc, keys, sid):
    g = GOLDEN[SETS[sid]]
    pk, sk = keys(sid)
    assert hashlib.sha256(pk.tobytes()).hexdigest() == g["pk_sha256"]
    assert hashlib.sha256(sk.tobytes()).hexdigest() == g["sk_sha256"]
    seeds = np.array([np.frombuffer(bytes.fromhex(v["seed"]), np.uint8) for v in g["enc"]])
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
    for i, v in enumerate(g["enc"]):
        assert c[i].tobytes().hex() == v["ct"] and k[i].tobytes().hex() == v["k"] and rc[i] == v["rc"]
    cases = g["flipped"] + ([g["padding"]] if "padding" in g else [])
    cts = np.array([np.frombuffer(bytes.fromhex(v["ct"]), np.uint8) for v in cases])
    k2, rc2 = gmc.SecretKey(sid, sk).dec_batch(cts)
    for i, v in enumerate(cases):
        assert k2[i].tobytes().hex() == v["k"] and rc2[i] == v["rc"]


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_decode_stages(gmc, keys, sid):
    """Error vector and decode flag of every request against the oracle's decrypt stages."""
    pk, sk = keys(sid)
    z = O.sizes(sid)
    n = 96
    oc, _, _ = O.enc_batch(sid, pk, request_seeds(sid, n, b"stages"), threads=THREADS)
    cts, _ = flipped_and_random(sid, oc, frac=0.25, nrand=4)
    n = len(cts)
    lde = (((z["n"] + 31) // 32) + 3) // 4 * 4
    lds2 = (((2 * z["t"] * z["m"] + 31) // 32) + 3) // 4 * 4
    dev = torch.device("cuda")
    d_c = torch.from_numpy(cts).to(dev)
    d_s = torch.zeros((n, lds2), dtype=torch.int32, device=dev)
    d_e = torch.zeros((n, lde), dtype=torch.int32, device=dev)
    d_ok = torch.zeros(n, dtype=torch.int32, device=dev)
    key = gmc.SecretKey(sid, sk)
    rc = gmc.lib().gmc_dec_stages_dev(key.handle, d_c.data_ptr(), n, d_s.data_ptr(), lds2, d_e.data_ptr(), lde,
                                      d_ok.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    S = d_s.cpu().numpy().view(np.uint32)
    E = d_e.cpu().numpy().view(np.uint32)
    OK = d_ok.cpu().numpy()
    m, t = z["m"], z["t"]
    for i in range(n):
        orc, sp, loc, e = O.decrypt_stages(sid, sk, cts[i])
        bits = np.unpackbits(S[i].view(np.uint8), bitorder="little")
        s = [int(sum(int(bits[j * m + b]) << b for b in range(m))) for j in range(2 * t)]
        assert s == [int(x) for x in sp], f"request {i}: syndromes differ"
        ge = E[i].view(np.uint8)[: z["n"] // 8]
        assert OK[i] == (1 if orc == 0 else 0), f"request {i}: decode flag"
        if orc == 0:
            assert (ge == e).all(), f"request {i}: error vector differs"


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_libmceliece_calling_convention(gmc, keys, sid):
    """One-request enc/dec with libmceliece's signatures; deterministic randombytes; aliasing of dec."""
    pk, sk = keys(sid)
    seed = hashlib.sha256(b"one-request" + bytes([sid])).digest()
    gmc.set_randombytes(lambda n: seed[:n])
    try:
        rc, c, k = gmc.kem_enc(sid, pk)
    finally:
        gmc.set_randombytes(None)
    orc, oc, okey = O.enc(sid, pk, seed)
    assert rc == orc == 0 and c == oc.tobytes() and k == okey.tobytes()
    rc, k2 = gmc.kem_dec(sid, c, sk)
    assert rc == 0 and k2 == k
    # k == c aliasing (libmceliece test: dec(c2, c2, s))
    L = gmc.lib()
    buf = np.zeros(max(32, len(c)), np.uint8)
    buf[: len(c)] = np.frombuffer(c, np.uint8)
    name = SETS[sid]
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert getattr(L, f"gmc_kem_{name}_dec")(p(buf), p(buf), p(np.ascontiguousarray(sk))) == 0
    assert buf[:32].tobytes() == k
    # k == sk aliasing (dec(s2, c, s2))
    skc = np.ascontiguousarray(sk).copy()
    assert getattr(L, f"gmc_kem_{name}_dec")(p(skc), p(np.frombuffer(c, np.uint8).copy()), p(skc)) == 0
    assert skc[:32].tobytes() == k


def test_6960119_padding_rules(gmc, keys):
    sid = 3
    pk, sk = keys(sid)
    z = O.sizes(sid)
    bad_pk = pk.copy()
    row = 5
    bad_pk[row * ((z["k"] + 7) // 8) + (z["k"] + 7) // 8 - 1] |= 0x80  # padding bit of one row
    seeds = request_seeds(sid, 4, b"pad")
    c, k, rc = gmc.PublicKey(sid, bad_pk).enc_batch(seeds)
    assert (rc == -1).all() and not c.any() and not k.any()
    orc, oc, okey = O.enc(sid, bad_pk, seeds[0].tobytes())
    assert orc == -1 and not oc.any() and not okey.any()
    oc, _, _ = O.enc_batch(sid, pk, seeds, threads=THREADS)
    oc[:, -1] |= np.uint8(0x08)
    k2, rc2 = gmc.SecretKey(sid, sk).dec_batch(oc)
    assert (rc2 == -1).all() and (k2 == 0xFF).all()


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 129])
def test_batch_edges(gmc, keys, n):
    sid = 0
    pk, sk = keys(sid)
    seeds = request_seeds(sid, n, b"edge")
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds.reshape(-1))
    assert c.shape == (n, O.sizes(sid)["ct_bytes"])
    if n:
        oc, okey, _ = O.enc_batch(sid, pk, seeds, threads=THREADS)
        assert (c == oc).all() and (k == okey).all()
        k2, _ = gmc.SecretKey(sid, sk).dec_batch(c)
        assert (k2 == k).all()


def test_bad_arguments(gmc, keys):
    pk, sk = keys(0)
    with pytest.raises(gmc.GmcError):
        gmc.PublicKey(7, pk)
    P = gmc.PublicKey(0, pk)
    S = gmc.SecretKey(0, sk)
    L = gmc.lib()
    assert L.gmc_dec_batch(P.handle, None, None, 1, None) in (-4, -1)
    assert L.gmc_enc_batch(S.handle, None, None, None, 1, None) in (-4, -1)
    assert L.gmc_enc_batch(P.handle, None, None, None, -1, None) == -1


def _cpu_checker():
    """libmceliece itself (oracle/_ref, built from the reference's sources by build()) when present, else the
    oracle restatement; both are pinned to libmceliece's known-answer checksums."""
    from oracle import pyref
    if pyref.available():
        pyref.lib()
        return pyref
    return O


@pytest.mark.parametrize("sid", [0, 4], ids=["348864", "8192128"])
def test_full_size_every_request(gmc, keys, sid):
    """The headline batch size, 65536 requests, every output checked: all ciphertexts and session keys of the
    encapsulation, and all session keys and return codes of a decapsulation of those ciphertexts with 10%
    carrying one flipped bit, against the CPU implementation on all host threads; decapsulating the valid
    ciphertexts returns their encapsulated keys."""
    pk, sk = keys(sid)
    n = 65536
    R = _cpu_checker()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(99 + sid)
    seeds = rng.integers(0, 256, size=(n, 32), dtype=np.uint8)
    c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
    assert (rc == 0).all()
    oc, okey, orc = R.enc_batch(sid, pk, seeds, threads=threads)
    assert (rc == orc).all()
    assert (c == oc).all(), f"{int((c != oc).any(1).sum())} of {n} ciphertexts differ"
    assert (k == okey).all(), f"{int((k != okey).any(1).sum())} of {n} session keys differ"
    cts, flipped = flipped_and_random(sid, c, frac=0.1, nrand=0, seed=11)
    k2, rc2 = gmc.SecretKey(sid, sk).dec_batch(cts)
    ok2, orc2 = R.dec_batch(sid, sk, cts, threads=threads)
    assert (rc2 == orc2).all()
    assert (k2 == ok2).all(), f"{int((k2 != ok2).any(1).sum())} of {n} decapsulated keys differ"
    valid = np.ones(n, bool)
    valid[flipped] = False
    assert (k2[valid] == k[valid]).all() and not (k2[~valid] == k[~valid]).all(1).any()


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_bm_forms_agree_on_corrupted_batches(gmc, keys, sid):
    """A batch large enough for the bit-sliced Berlekamp-Massey (>= 24576 rows) and the same ciphertexts in
    small batches (warp-per-request form) give identical keys and return codes, on valid, single-bit-flipped
    and random ciphertexts; an oracle sample of each kind agrees. The small batches take every block shape of
    the warp-per-request launch: 1 warp per block, a few, one round of up to 28 warps, several rounds."""
    pk, sk = keys(sid)
    n = 32768
    rng = np.random.default_rng(7 + sid)
    seeds = rng.integers(0, 256, size=(n, 32), dtype=np.uint8)
    c, _, _ = gmc.PublicKey(sid, pk).enc_batch(seeds)
    cts, flipped = flipped_and_random(sid, c, frac=0.1, nrand=256, seed=3)
    key = gmc.SecretKey(sid, sk)
    k_big, rc_big = key.dec_batch(cts)
    cuts = np.cumsum([0, 1, 300, 4096, 9000])
    bounds = list(zip(cuts, list(cuts[1:]) + [len(cts)]))
    parts = [key.dec_batch(cts[a:b]) for a, b in bounds]
    k_small = np.concatenate([p[0] for p in parts])
    rc_small = np.concatenate([p[1] for p in parts])
    assert (k_big == k_small).all() and (rc_big == rc_small).all()
    sample = np.concatenate([rng.choice(n, 16, replace=False), flipped[:16], np.arange(n, n + 16)])
    ok2, orc2 = O.dec_batch(sid, sk, cts[sample], threads=THREADS)
    assert (k_big[sample] == ok2).all() and (rc_big[sample] == orc2).all()


@pytest.mark.parametrize("engine", ["tc", "b1mma", "popc", "sparse"])
@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_kem_parity_per_gemm_engine(gmc, keys, sid, engine):
    """Encapsulation and decapsulation byte-exact with every syndrome engine (sparse: encapsulation only)."""
    pk, sk = keys(sid)
    eng = {"tc": gmc.GEMM_TC, "b1mma": gmc.GEMM_B1MMA, "popc": gmc.GEMM_POPC, "sparse": gmc.GEMM_SPARSE}[engine]
    prev = gmc.get_gemm_engine()  # -1: no override
    gmc.set_gemm_engine(eng)
    try:
        n = 300
        seeds = request_seeds(sid, n, b"engine")
        c, k, rc = gmc.PublicKey(sid, pk).enc_batch(seeds)
        oc, okey, _ = O.enc_batch(sid, pk, seeds, threads=THREADS)
        assert (c == oc).all() and (k == okey).all()
        cts, _ = flipped_and_random(sid, oc, seed=5)
        k2, rc2 = gmc.SecretKey(sid, sk).dec_batch(cts)
        ok2, orc2 = O.dec_batch(sid, sk, cts, threads=THREADS)
        assert (k2 == ok2).all() and (rc2 == orc2).all()
        if eng == gmc.GEMM_TC:
            assert gmc.lib().gmc_tc_status() == 0
    finally:
        gmc.set_gemm_engine(prev)
