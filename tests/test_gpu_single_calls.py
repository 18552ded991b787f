"""The libmceliece-convention entry points (gmc_kem_<set>_{enc,dec}) keep the
keys they were given resident: alternating keys, more keys than the cache
holds, and a secret key that aliases the output buffer all give the oracle's
results, and repeated calls with one key do not reload it."""
import time

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def test_alternating_and_evicted_keys(gmc):
    sid = 0
    pairs = [O.keypair(sid, bytes([i]) * 32) for i in range(10)]  # more than the 8 cached keys
    for rnd in range(2):
        for i in (0, 9, 1, 8, 2, 7, 3, 6, 4, 5, 0, 9):
            pk, sk = pairs[i]
            rc, ct, k = gmc.kem_enc(sid, pk)
            assert rc == 0
            rc2, k2 = gmc.kem_dec(sid, ct, sk)
            assert rc2 == 0 and k2 == k
            okey = np.zeros(32, np.uint8)
            assert O.lib().gmo_dec(sid, O._p(okey), O._p(np.frombuffer(ct, np.uint8).copy()), O._p(sk)) == 0
            assert okey.tobytes() == k


def test_dec_with_key_aliasing_the_secret_key(gmc):
    sid = 4
    pk, sk = O.keypair(sid, bytes([0x77]) * 32)
    rc, ct, k = gmc.kem_enc(sid, pk)
    L = gmc.lib()
    buf = np.array(sk, np.uint8)  # k == sk: the output overwrites the key's first 32 bytes
    c = np.frombuffer(ct, np.uint8).copy()
    assert L.gmc_kem_8192128_dec(gmc._ptr(buf), gmc._ptr(c), gmc._ptr(buf)) == 0
    assert buf[:32].tobytes() == k


def test_repeated_calls_do_not_reload(gmc):
    sid = 4
    pk, sk = O.keypair(sid, bytes([0x78]) * 32)
    gmc.kem_enc(sid, pk)
    t0 = time.perf_counter()
    for _ in range(20):
        rc, ct, k = gmc.kem_enc(sid, pk)
    per_call = (time.perf_counter() - t0) / 20
    # a reload (host tables, allocation, 1.3 MB copy, transpose) costs milliseconds; a cached call well below
    assert per_call < 2e-3, per_call
