"""The oracle against libmceliece-20250507's own known-answer checksums.

The expected values are the checksum table of libmceliece's test program
(deps/libmceliece-20250507.tar.gz: command/mceliece-test.c, kem_<set>_checksums,
e.g. :4567 for 348864 and :2751 for 8192128); oracle/kat.c replays the same
procedure (keypair, enc, dec, three corrupted-ciphertext decs per loop).
"""
import pytest

from oracle import pyoracle as O

KAT = {
    "348864": ("2f36e1825115c5accc9a6ea609dec708f83be85e7fe448637bd502de50a1dd91",
               "df7965299cab8d4669eb29ebe87a2f61a539aa016a8dcda268a8cd595bf6d8da"),
    "460896": ("006c110df7fd3ff1852c9096a6514855ef3e715469ecc21d5b6ba14d31057417",
               "604d5d0be1ec220a2a914735fa5469622cd1f66737cf7e0709b7eaaa1e382f66"),
    "6688128": ("a3446acecf9aff0e757dfafc5402e365eb3ba485dd1f7b052f3ca6eabfdcb6c4",
                "b2ee78aaa23c0612155239b1d92e9e1af589cb810bdb9d8c44eb85dbfd2e46d4"),
    "6960119": ("008c0538526a1c037e64f0543628b312a71e879c1f882f65493fd0d3a225d5d8",
                "15c6727d4f4867487a54bbb208c06c1142a56a7937d7b598c05f63801cbdd277"),
    "8192128": ("debad73db5027e8239b7e97d04c5a98b7521caba8ea4e58581c90efb50dd4b9e",
                "5e64e0aeb5ab566a1efbb2b1127dcbf909ee1b395945f066cd5f097a85f2e135"),
}


@pytest.mark.parametrize("name", list(KAT))
def test_kat_small(name):
    rc, h = O.kat_checksum(name, loops=8)
    assert rc == 0
    assert h == KAT[name][0]


@pytest.mark.parametrize("name", list(KAT))
def test_kat_large(name):
    rc, h = O.kat_checksum(name, loops=64)
    assert rc == 0
    assert h == KAT[name][1]


def test_shake256_vectors():
    import hashlib
    for msg in (b"", b"abc", bytes(range(200)), bytes(1000)):
        for n in (32, 136, 300):
            assert O.shake256(msg, n) == hashlib.shake_256(msg).digest(n)
