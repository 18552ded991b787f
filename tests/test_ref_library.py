"""libmceliece-20250507 itself (its portable `vec` code, compiled from the reference's bundled tarball by
oracle/build_ref.py) against its own known-answer checksums and against the oracle restatement.

This pins the oracle to the real library on seeded inputs (key generation, encapsulation through the seed chain,
decapsulation of valid, bit-flipped and random ciphertexts) in addition to the checksum replay of
tests/test_oracle_kat.py, and it checks that the library built here is the one bench.py times as the CPU baseline.
Skipped where neither the extracted sources nor the reference tarball are present.
"""
import hashlib

import numpy as np
import pytest

from oracle import pyoracle as O
from oracle import pyref as R
from tests.test_oracle_kat import KAT

pytestmark = pytest.mark.skipif(not R.available(), reason="libmceliece sources not present (oracle/build_ref.py)")


@pytest.mark.parametrize("name", ["348864", "460896", "6688128", "6960119", "8192128", "8192128pc", "6960119f"])
def test_library_kat_checksum(name):
    rc, h = R.kat_checksum(name, loops=8)
    assert rc == 0
    assert h == KAT[name][0]


@pytest.mark.parametrize("vid", range(20))
def test_library_matches_oracle(vid):
    seed = hashlib.sha256(b"ref-vs-oracle" + bytes([vid])).digest()
    pk, sk = O.keypair(vid, seed)
    rpk, rsk = R.keypair(vid, seed)
    assert np.array_equal(pk, rpk) and np.array_equal(sk, rsk), "keypair differs"
    n = 24
    seeds = np.frombuffer(hashlib.shake_256(b"ref-seeds" + bytes([vid])).digest(32 * n), np.uint8).reshape(n, 32)
    c, k, rc = R.enc_batch(vid, pk, seeds, threads=4)
    oc, ok_, orc = O.enc_batch(vid, pk, seeds, threads=4)
    assert np.array_equal(c, oc) and np.array_equal(k, ok_) and np.array_equal(rc, orc), "enc differs"
    rng = np.random.default_rng(vid)
    bad = c.copy()
    for i in range(0, n, 3):  # one flipped bit anywhere in the ciphertext
        b = int(rng.integers(0, 8 * bad.shape[1]))
        bad[i, b // 8] ^= np.uint8(1 << (b % 8))
    bad[n - 2:] = rng.integers(0, 256, (2, bad.shape[1]), dtype=np.uint8)  # random ciphertexts
    kd, rcd = R.dec_batch(vid, sk, bad, threads=4)
    okd, orcd = O.dec_batch(vid, sk, bad, threads=4)
    assert np.array_equal(kd, okd) and np.array_equal(rcd, orcd), "dec differs"
    assert np.array_equal(kd[1::3][: (n - 2) // 3], k[1::3][: (n - 2) // 3])


def test_golden_fixtures_match_library():
    """The committed golden vectors (made from the oracle) hold for the library too."""
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kem_vectors.json")))
    assert set(g) == {"348864", "460896", "6688128", "6960119", "8192128"}
    for name, rec in g.items():
        vid = R.sid(name)
        pk, sk = R.keypair(vid, bytes.fromhex(rec["key_seed"]))
        assert hashlib.sha256(pk.tobytes()).hexdigest() == rec["pk_sha256"]
        assert hashlib.sha256(sk.tobytes()).hexdigest() == rec["sk_sha256"]
        for e in rec["enc"]:
            rc, c, k = R.enc(vid, pk, bytes.fromhex(e["seed"]))
            assert (c.tobytes().hex(), k.tobytes().hex(), rc) == (e["ct"], e["k"], e["rc"])
        for e in rec["flipped"] + ([rec["padding"]] if "padding" in rec else []):
            rc, k = R.dec(vid, bytes.fromhex(e["ct"]), sk)
            assert (k.tobytes().hex(), rc) == (e["k"], e["rc"])
