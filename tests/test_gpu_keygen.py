"""GPU key generation (gmc_keypair_batch): every pk and sk byte-exact against the
oracle's keypair for the same 32-byte seed, over seeds whose seed chains need
one or several attempts, and a batch large enough for several rounds of
speculative attempts. A mismatch is reported per sk field (seed of the winning
attempt, Goppa polynomial, control bits, s) and for pk."""
import hashlib
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import SETS, key_seed

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
THREADS = min(16, os.cpu_count() or 1)


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def seeds_for(sid, n, tag=b"kg"):
    return np.frombuffer(b"".join(hashlib.sha256(tag + bytes([sid]) + i.to_bytes(4, "little")).digest()
                                  for i in range(n)), np.uint8).reshape(n, 32)


def oracle_keys(sid, seeds):
    with ThreadPoolExecutor(THREADS) as ex:
        return list(ex.map(lambda s: O.keypair(sid, bytes(s)), seeds))


def sk_fields(sid):
    z = O.sizes(sid % 5)
    t, m = z["t"], z["m"]
    cond = (1 << (m - 4)) * (2 * m - 1)
    return [("seed", 0, 32), ("pivots", 32, 40), ("g", 40, 40 + 2 * t), ("cond", 40 + 2 * t, 40 + 2 * t + cond),
            ("s", 40 + 2 * t + cond, z["sk_bytes"])]


def check(sid, seeds, pk, sk, ref):
    bad = []
    for i, (opk, osk) in enumerate(ref):
        fields = [name for name, a, b in sk_fields(sid) if not np.array_equal(sk[i, a:b], np.asarray(osk)[a:b])]
        if not np.array_equal(pk[i], np.asarray(opk)):
            fields.append("pk")
        if fields:
            bad.append((i, fields))
    assert not bad, f"{len(bad)}/{len(ref)} keys differ: {bad[:8]}"


@pytest.mark.parametrize("sid", range(5), ids=SETS)
def test_keygen_parity(gmc, sid):
    seeds = np.concatenate([np.frombuffer(key_seed(sid), np.uint8)[None], seeds_for(sid, 3)])
    pk, sk = gmc.keypair_batch(sid, seeds)
    check(sid, seeds, pk, sk, oracle_keys(sid, seeds))


@pytest.mark.parametrize("sid", range(10, 15), ids=[s + "f" for s in SETS])
def test_keygen_semi_systematic_parity(gmc, sid):
    """f variants (ids 10..14): the last 32 pivots from the 64-column window, the support swapped
    accordingly, pivots in sk[32:40]."""
    seeds = seeds_for(sid, 4, tag=b"kg-f")
    pk, sk = gmc.keypair_batch(sid, seeds)
    ref = oracle_keys(sid, seeds)
    check(sid, seeds, pk, sk, ref)
    pk2, sk2 = gmc.keypair_batch(sid + 5, seeds[:1])  # pcf: the same keys
    assert np.array_equal(pk2[0], pk[0]) and np.array_equal(sk2[0], sk[0])


def test_keygen_many_rounds(gmc):
    """More keys than one round's attempts for the small set: several rounds, with
    1 and more speculative attempts per key."""
    sid = 0
    cap = 4 * torch.cuda.get_device_properties(0).multi_processor_count  # attempts per round
    seeds = seeds_for(sid, cap + 37, tag=b"kg-many")
    pk, sk = gmc.keypair_batch(sid, seeds)
    check(sid, seeds, pk, sk, oracle_keys(sid, seeds))


def test_keygen_chunks_and_extension_blocks(gmc, monkeypatch):
    """Staging chunks of 7 keys and 2 links expanded ahead: several chunks per call, and most chains carried
    by extension blocks (an f set, so the window step runs in the same call)."""
    monkeypatch.setenv("GMC_KG_CHUNK_KEYS", "7")
    monkeypatch.setenv("GMC_KG_AHEAD_LINKS", "2")
    for sid in (0, 10):
        seeds = seeds_for(sid, 23, tag=b"kg-chunks")
        pk, sk = gmc.keypair_batch(sid, seeds)
        check(sid, seeds, pk, sk, oracle_keys(sid, seeds))


@pytest.mark.parametrize("sid", [1, 6, 11, 16], ids=["460896", "460896pc", "460896f", "460896pcf"])
def test_single_key_entry_points(gmc, sid):
    """gmc_keypair_seed and libmceliece's calling convention gmc_kem_<set>_keypair (randomness from the
    randombytes source, overridden here) run the GPU key generation with one key: the oracle's keys for plain,
    pc, f and pcf ids (pc keys are the plain set's, pcf keys the f set's), equal to the batched keys."""
    seeds = seeds_for(sid, 2, tag=b"kg-single")
    pk, sk = gmc.keypair_batch(sid, seeds)
    ref = oracle_keys(sid, seeds)
    check(sid, seeds, pk, sk, ref)
    for i in range(2):
        hpk, hsk = gmc.keypair(sid, bytes(seeds[i]))
        assert np.array_equal(pk[i], hpk) and np.array_equal(sk[i], hsk)
    draws = []
    gmc.set_randombytes(lambda n: (draws.append(n), bytes(seeds[1]))[1])
    try:
        kpk, ksk = gmc.keypair(sid)  # gmc_kem_<set>_keypair: one 32-byte draw
    finally:
        gmc.set_randombytes(None)
    assert draws == [32]
    assert np.array_equal(kpk, pk[1]) and np.array_equal(ksk, sk[1])


def test_keygen_keys_serve(gmc):
    """A GPU-generated key pair encapsulates and decapsulates through the engine."""
    sid = 4
    seeds = seeds_for(sid, 1, tag=b"kg-serve")
    pk, sk = gmc.keypair_batch(sid, seeds)
    rs = seeds_for(sid, 64, tag=b"kg-serve-req")
    c, k, rc = gmc.PublicKey(sid, pk[0]).enc_batch(rs)
    k2, rc2 = gmc.SecretKey(sid, sk[0]).dec_batch(c)
    assert (rc == 0).all() and (rc2 == 0).all()
    assert np.array_equal(k, k2)


def test_keygen_empty_and_bad_args(gmc):
    pk, sk = gmc.keypair_batch(0, np.zeros((0, 32), np.uint8))
    assert pk.shape[0] == 0 and sk.shape[0] == 0
    assert gmc.lib().gmc_keypair_batch(7, None, None, None, 1) == -1  # GMC_EINVAL
    assert gmc.lib().gmc_keypair_batch(0, None, None, None, 1) == -1
