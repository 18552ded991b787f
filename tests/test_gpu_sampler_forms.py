"""The two sampler forms (pipelined lane groups, the default; lane per request,
GMC_SAMPLE_PIPELINE=0) give identical ciphertexts and session keys, for sets
with 2, 3 and 4 Keccak-f blocks per attempt, on batches smaller and larger
than the resident lane groups, and both match the oracle."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = [(0, 300), (1, 700), (2, 30000), (3, 5000), (4, 25000)]

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import tensormceliece_gb300 as g
from oracle import pyoracle as O
from tests.conftest import request_seeds
out = {}
for sid, n in %r:
    pk, _ = O.keypair(sid, bytes([0x31 + sid]) * 32)
    c, k, rc = g.PublicKey(sid, pk).enc_batch(request_seeds(sid, n, b"forms"))
    out["c%%d" %% sid], out["k%%d" %% sid] = c, k
np.savez(sys.argv[2], **out)
"""


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def test_sampler_forms_agree(gmc, tmp_path):
    path = str(tmp_path / "lane_form.npz")
    env = dict(os.environ, GMC_SAMPLE_PIPELINE="0")
    subprocess.run([sys.executable, "-c", CHILD % (CASES,), ROOT, path], env=env, check=True, cwd=ROOT, timeout=600)
    lane = np.load(path)
    for sid, n in CASES:
        pk, _ = O.keypair(sid, bytes([0x31 + sid]) * 32)
        seeds = request_seeds(sid, n, b"forms")
        c, k, _ = gmc.PublicKey(sid, pk).enc_batch(seeds)
        assert (c == lane["c%d" % sid]).all() and (k == lane["k%d" % sid]).all(), sid
        oc, ok_, _ = O.enc_batch(sid, pk, seeds[:48], threads=8)
        assert (c[:48] == oc).all() and (k[:48] == ok_).all(), sid
