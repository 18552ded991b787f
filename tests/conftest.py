import hashlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SETS = ("348864", "460896", "6688128", "6960119", "8192128")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def key_seed(sid):
    """Fixed 32-byte keygen seed per parameter set (the single randombytes draw of keypair)."""
    return hashlib.sha256(b"gmc-keyseed-" + SETS[sid].encode()).digest()


def request_seeds(sid, n, tag=b""):
    """Per-request seeds: SHAKE256("gmc-seed" || set || tag || i)[0:32]."""
    out = np.zeros((n, 32), np.uint8)
    for i in range(n):
        h = hashlib.shake_256(b"gmc-seed" + SETS[sid].encode() + tag + int(i).to_bytes(8, "little"))
        out[i] = np.frombuffer(h.digest(32), np.uint8)
    return out


_KEYS = {}


@pytest.fixture(scope="session")
def keys():
    """keys(sid) -> (pk, sk) from the oracle's keygen with key_seed(sid)."""
    from oracle import pyoracle as O

    def get(sid):
        if sid not in _KEYS:
            _KEYS[sid] = O.keypair(sid, key_seed(sid))
        return _KEYS[sid]

    return get
