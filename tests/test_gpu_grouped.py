"""Grouped launches (gmc_plan_*): 8 key pairs over all five parameter sets,
Zipf(1.2)-skewed request counts, 50/50 encapsulation/decapsulation, one CUDA
graph replay. Every output equals the per-key batched calls bit for bit, and a
sample is checked against the oracle."""
import hashlib

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import SETS, request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MIX = [0, 0, 1, 1, 2, 3, 4, 4]  # 8 keys over the five sets


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def zipf_counts(total, k, s=1.2, seed=3):
    w = 1.0 / np.arange(1, k + 1) ** s
    rng = np.random.default_rng(seed)
    w = w[rng.permutation(k)]
    c = np.floor(total * w / w.sum()).astype(int)
    c[0] += total - c.sum()
    return c


def test_grouped_plan_matches_per_key_calls(gmc):
    dev = torch.device("cuda")
    keys = []
    for i, sid in enumerate(MIX):
        pk, sk = gmc.keypair(sid, hashlib.sha256(b"grouped-key-%d" % i).digest())
        keys.append((sid, pk, sk, gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)))
    counts = zipf_counts(6000, 2 * len(MIX))
    groups, bufs = [], []
    for i, (sid, pk, sk, P, S) in enumerate(keys):
        z = gmc.set_sizes(sid)
        ne, nd = int(counts[2 * i]), int(counts[2 * i + 1])
        seeds = torch.from_numpy(request_seeds(sid, ne, b"grp%d" % i)).to(dev)
        c_out = torch.zeros((ne, z["ct_bytes"]), dtype=torch.uint8, device=dev)
        k_out = torch.zeros((ne, 32), dtype=torch.uint8, device=dev)
        rc_e = torch.full((ne,), 9, dtype=torch.int32, device=dev)
        cts_np, _, _ = O.enc_batch(sid, pk, request_seeds(sid, nd, b"grpd%d" % i), threads=8)
        rng = np.random.default_rng(i)
        for j in rng.choice(nd, nd // 10, replace=False):
            b = int(rng.integers(0, z["mt"]))
            cts_np[j, b // 8] ^= np.uint8(1 << (b % 8))
        cts = torch.from_numpy(cts_np).to(dev)
        k_dec = torch.zeros((nd, 32), dtype=torch.uint8, device=dev)
        rc_d = torch.full((nd,), 9, dtype=torch.int32, device=dev)
        bufs.append((seeds, c_out, k_out, rc_e, cts, k_dec, rc_d))
        groups.append((P, ne, seeds.data_ptr(), c_out.data_ptr(), k_out.data_ptr(), rc_e.data_ptr()))
        groups.append((S, nd, cts.data_ptr(), 0, k_dec.data_ptr(), rc_d.data_ptr()))
    plan = gmc.Plan(groups)
    info = plan.info()
    assert info["pipelines"] == 10  # five sets x {enc, dec}
    st = torch.cuda.current_stream()
    for rep in range(2):  # the graph replays to the same outputs
        for b in bufs:
            b[1].zero_(); b[2].zero_(); b[5].zero_()
        plan.launch(st.cuda_stream)
        torch.cuda.synchronize()
        for i, (sid, pk, sk, P, S) in enumerate(keys):
            seeds, c_out, k_out, rc_e, cts, k_dec, rc_d = bufs[i]
            ne, nd = seeds.shape[0], cts.shape[0]
            c_ref = torch.zeros_like(c_out); k_ref = torch.zeros_like(k_out)
            P.enc_batch_dev(c_ref.data_ptr(), k_ref.data_ptr(), seeds.data_ptr(), ne, 0, st.cuda_stream)
            kd_ref = torch.zeros_like(k_dec); rcd_ref = torch.zeros_like(rc_d)
            S.dec_batch_dev(kd_ref.data_ptr(), cts.data_ptr(), nd, rcd_ref.data_ptr(), st.cuda_stream)
            torch.cuda.synchronize()
            assert torch.equal(c_out, c_ref) and torch.equal(k_out, k_ref), f"key {i} enc differs"
            assert torch.equal(k_dec, kd_ref) and torch.equal(rc_d, rcd_ref), f"key {i} dec differs"
            assert int(rc_e.abs().sum()) == 0
    # oracle spot check on two keys
    for i in (0, 7):
        sid, pk, sk, P, S = keys[i]
        seeds, c_out, k_out, rc_e, cts, k_dec, rc_d = bufs[i]
        m = min(64, seeds.shape[0])
        oc, ok_, _ = O.enc_batch(sid, pk, seeds[:m].cpu().numpy(), threads=8)
        assert (c_out[:m].cpu().numpy() == oc).all() and (k_out[:m].cpu().numpy() == ok_).all()
        md = min(64, cts.shape[0])
        okd, _ = O.dec_batch(sid, sk, cts[:md].cpu().numpy(), threads=8)
        assert (k_dec[:md].cpu().numpy() == okd).all()
    plan.close()
