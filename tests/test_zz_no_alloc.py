"""gmc_dec_batch_noalloc: decapsulation for callers that cannot allocate device
memory (their device memory belongs to another allocator with a fixed budget,
or cudaMalloc's device-wide synchronization is not acceptable on their path).

Its results must be the existing entry point's (gmc_dec_batch_dev) and the
oracle's, bit for bit, on calls in a row; it must allocate nothing (free
device memory is unchanged across the calls) and must reject batches above its
fixed limit.
This file is collected last, and also passes alone in a fresh process."""
import ctypes
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import SETS, key_seed, request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
THREADS = os.cpu_count() or 8


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    L = g.lib()
    L.gmc_dec_batch_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                        ctypes.c_void_p, ctypes.c_void_p]
    return g


def _cts(sid, pk, n, tag):
    z = O.sizes(sid)
    oc, _, _ = O.enc_batch(sid, pk, request_seeds(sid % 5, n, tag), threads=THREADS)
    rng = np.random.default_rng(n)
    for i in rng.choice(n, max(1, n // 10), replace=False):  # 10% one flipped bit
        b = int(rng.integers(0, z["mt"]))
        oc[i, b // 8] ^= np.uint8(1 << (b % 8))
    return oc


@pytest.mark.parametrize("sid", [0, 1, 2, 3, 4, 8], ids=list(SETS) + [SETS[3] + "pc"])
def test_noalloc_matches_existing_entry_point_and_oracle(gmc, sid):
    L = gmc.lib()
    pk, sk = gmc.keypair(sid % 5, key_seed(sid % 5))  # a pc variant (ids 5..9) has its base set's keys
    key = gmc.SecretKey(sid, sk)
    dev = torch.device("cuda")
    st = torch.cuda.current_stream()
    for call, n in enumerate((1, 777, 4096)):
        cts_h = _cts(sid, pk, n, b"noalloc%d" % call)
        cts = torch.from_numpy(cts_h).to(dev)
        k_ref = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
        rc_ref = torch.zeros(n, dtype=torch.int32, device=dev)
        assert L.gmc_dec_batch_dev(key.handle, k_ref.data_ptr(), cts.data_ptr(), n, rc_ref.data_ptr(),
                                   st.cuda_stream) == 0
        k_na = torch.full((n, 32), 0xAB, dtype=torch.uint8, device=dev)
        rc_na = torch.full((n,), 7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        assert L.gmc_dec_batch_noalloc(key.handle, k_na.data_ptr(), cts.data_ptr(), n, rc_na.data_ptr(),
                                       st.cuda_stream) == 0, L.gmc_last_error()
        torch.cuda.synchronize()
        assert torch.equal(k_na, k_ref), f"call {call}: session keys differ from gmc_dec_batch_dev"
        assert torch.equal(rc_na, rc_ref), f"call {call}: return codes differ from gmc_dec_batch_dev"
        ok_, orc = O.dec_batch(sid, sk, cts_h, threads=THREADS)
        assert np.array_equal(k_na.cpu().numpy(), ok_), f"call {call}: session keys differ from the oracle"
        assert np.array_equal(rc_na.cpu().numpy(), orc), f"call {call}: return codes differ from the oracle"
        # the first call on a device loads the module that holds the fixed array
        # (the library's static footprint); from then on nothing is allocated
        if call > 0:
            assert torch.cuda.mem_get_info()[0] == free_before, "free device memory changed"


def test_noalloc_rejects_oversized_batches(gmc):
    L = gmc.lib()
    pk, sk = gmc.keypair(0, key_seed(0))
    key = gmc.SecretKey(0, sk)
    big = 4097
    dev = torch.device("cuda")
    cts = torch.zeros((big, 96), dtype=torch.uint8, device=dev)
    k = torch.zeros((big, 32), dtype=torch.uint8, device=dev)
    assert L.gmc_dec_batch_noalloc(key.handle, k.data_ptr(), cts.data_ptr(), big, None, None) == -1
    assert b"GMC_NOALLOC_MAX_REQUESTS" in L.gmc_last_error()
