"""The three GF(2) GEMM engines (CUDA-core popcount, legacy b1 mma.sync, tcgen05
FP8 with TMEM accumulators) against a numpy GF(2) product, through the C ABI.
Exactness of the FP32 tensor-core accumulation is probed with all-ones rows
(the largest possible count, K) and rows of every weight 0..K."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


def gf2_reference(A, X, rows):
    """bit r of out[i] = parity(popcount(A[r] & X[i]))."""
    a = np.unpackbits(A.view(np.uint8), bitorder="little").reshape(A.shape[0], -1)[:rows].astype(np.int64)
    x = np.unpackbits(X.view(np.uint8), bitorder="little").reshape(X.shape[0], -1).astype(np.int64)
    par = (x @ a.T) & 1  # [n, rows]
    words = (rows + 31) // 32
    pad = np.zeros((x.shape[0], words * 32), np.uint8)
    pad[:, :rows] = par
    return np.packbits(pad, axis=1, bitorder="little").view(np.uint32)


def run_engine(gmc, engine, A, X, rows, n):
    dev = torch.device("cuda")
    rows_pad, lda = A.shape
    n_pad, ldx = X.shape
    kw_pad = lda
    words = (rows + 31) // 32
    ldo = (words + 3) // 4 * 4
    dA = torch.from_numpy(A.view(np.int32)).to(dev)
    dX = torch.from_numpy(X.view(np.int32)).to(dev)
    dO = torch.full((n, ldo), -1, dtype=torch.int32, device=dev)
    rc = gmc.lib().gmc_gf2_gemm_dev(engine, dA.data_ptr(), lda, rows_pad, dX.data_ptr(), ldx, n_pad, kw_pad,
                                     dO.data_ptr(), ldo, words, n, None)
    assert rc == 0, gmc.lib().gmc_last_error()
    torch.cuda.synchronize()
    if engine == gmc.GEMM_TC:
        assert gmc.lib().gmc_tc_status() == 0, "tensor-core CTA gave up on a bounded wait"
    return dO.cpu().numpy().view(np.uint32)[:, :words]


@pytest.mark.parametrize("engine", ["popc", "b1mma", "tc"])
@pytest.mark.parametrize("shape", [(256, 16, 300), (1664, 208, 513), (3328, 56, 256)])
def test_engine_matches_numpy(gmc, engine, shape):
    rows, kw_pad, n = shape
    rows_pad = (rows + 127) // 128 * 128
    n_pad = (n + 255) // 256 * 256
    rng = np.random.default_rng(rows + kw_pad + n)
    A = rng.integers(0, 2**32, size=(rows_pad, kw_pad), dtype=np.uint32)
    A[rows:] = 0
    X = rng.integers(0, 2**32, size=(n_pad, kw_pad), dtype=np.uint32)
    eng = {"popc": gmc.GEMM_POPC, "b1mma": gmc.GEMM_B1MMA, "tc": gmc.GEMM_TC}[engine]
    out = run_engine(gmc, eng, A, X, rows, n)
    ref = gf2_reference(A, X[:n], rows)
    assert (out == ref).all(), f"{int((out != ref).sum())} words differ"


def test_tc_exact_at_every_count(gmc):
    """Row r has its first r bits set; X all ones: the count for row r is r (up to K = 6656)."""
    kw_pad = 208
    K = kw_pad * 32
    rows_pad = 6656 + 128
    A = np.zeros((rows_pad, kw_pad), np.uint32)
    bits = np.zeros((rows_pad, K), np.uint8)
    for r in range(K + 1):
        bits[r, :r] = 1
    A[:] = np.packbits(bits, axis=1, bitorder="little").view(np.uint32)
    X = np.full((256, kw_pad), 0xFFFFFFFF, np.uint32)
    rows = K + 1
    out = run_engine(gmc, gmc.GEMM_TC, A, X, rows, 256)
    expect = np.zeros(((rows + 31) // 32) * 32, np.uint8)
    expect[:rows] = np.arange(rows) & 1
    expect_words = np.packbits(expect, bitorder="little").view(np.uint32)
    assert (out == expect_words[None, :]).all()
