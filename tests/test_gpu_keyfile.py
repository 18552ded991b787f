"""Resident-key persistence (gmc_key_export / gmc_key_import): a key re-created
from its exported string gives the same ciphertexts and session keys as the key
it came from, for public and secret keys of every set and of a pc variant, and
the import rejects altered or truncated strings."""
import numpy as np
import pytest

from tests.conftest import SETS, request_seeds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gmc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import tensormceliece_gb300 as g
    g.lib()
    return g


@pytest.mark.parametrize("sid", [0, 1, 2, 3, 4, 9], ids=list(SETS) + ["8192128pc"])
def test_export_import_round_trip(gmc, keys, sid):
    pk, sk = keys(sid % 5)
    P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
    P2, S2 = gmc.PublicKey.from_export(P.export()), gmc.SecretKey.from_export(S.export())
    assert P2.set == sid and S2.set == sid
    seeds = request_seeds(sid % 5, 96, b"keyfile")
    c, k, rc = P.enc_batch(seeds)
    c2, k2, rc2 = P2.enc_batch(seeds)
    assert (c == c2).all() and (k == k2).all() and (rc == rc2).all()
    bad = c.copy()
    bad[::3, 0] ^= 1
    kd, rcd = S.dec_batch(bad)
    kd2, rcd2 = S2.dec_batch(bad)
    assert (kd == kd2).all() and (rcd == rcd2).all()


def test_import_rejects_altered_strings(gmc, keys):
    pk, sk = keys(0)
    blob = bytearray(gmc.SecretKey(0, sk).export())
    for where in (0, 40, len(blob) // 2, len(blob) - 1):
        b = bytearray(blob)
        b[where] ^= 0x10
        with pytest.raises(gmc.GmcError):
            gmc.SecretKey.from_export(bytes(b))
    with pytest.raises(gmc.GmcError):
        gmc.SecretKey.from_export(bytes(blob[:-8]))


def _reseal(blob):
    """Recomputes the string's checksum (SHAKE256 over the string with the checksum field zeroed), as a crafted
    string would carry it: the checksum guards against corruption, not against a chosen header."""
    import hashlib
    b = bytearray(blob)
    b[104:136] = bytes(32)
    b[104:136] = hashlib.shake_256(bytes(b)).digest(32)
    return bytes(b)


def test_import_rejects_layouts_the_kernels_do_not_use(gmc, keys):
    """Header fields at their offsets: kw_pad 32, pad_bad 36 (public); cw_pad 52 (secret); checksum 104..136."""
    import struct
    pk, sk = keys(4)
    sblob = gmc.SecretKey(4, sk).export()
    pblob = gmc.PublicKey(4, pk).export()
    gmc.SecretKey.from_export(_reseal(sblob))  # resealing an unchanged string keeps it valid
    gmc.PublicKey.from_export(_reseal(pblob))
    for blob, off, value in ((sblob, 52, struct.unpack_from("<i", sblob, 52)[0] - 8),
                             (pblob, 32, struct.unpack_from("<i", pblob, 32)[0] - 8),
                             (pblob, 36, 2)):
        b = bytearray(blob)
        struct.pack_into("<i", b, off, value)
        with pytest.raises(gmc.GmcError):
            (gmc.SecretKey if blob is sblob else gmc.PublicKey).from_export(_reseal(b))
