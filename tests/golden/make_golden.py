"""Generates tests/golden/kem_vectors.json from the oracle.

The oracle is pinned to libmceliece-20250507's known-answer checksums
(tests/test_oracle_kat.py); these fixtures freeze, per parameter set, the key
hashes for a fixed keygen seed and seed-chain encapsulations (ciphertext and
session key), plus decapsulations of bit-flipped ciphertexts (implicit
rejection) and, for 6960119, ciphertexts with padding bits set.
Run from the repository root: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pyoracle as O  # noqa: E402
from tests.conftest import SETS, key_seed, request_seeds  # noqa: E402

N_ENC = 6
N_FLIP = 3


def main():
    out = {}
    for sid, name in enumerate(SETS):
        pk, sk = O.keypair(sid, key_seed(sid))
        seeds = request_seeds(sid, N_ENC, b"golden")
        vec = []
        for i in range(N_ENC):
            rc, c, k = O.enc(sid, pk, seeds[i].tobytes())
            vec.append({"seed": seeds[i].tobytes().hex(), "ct": c.tobytes().hex(), "k": k.tobytes().hex(), "rc": rc})
        flips = []
        rng = np.random.default_rng(1234 + sid)
        mt = O.sizes(sid)["mt"]
        for i in range(N_FLIP):
            c = bytearray(bytes.fromhex(vec[i]["ct"]))
            bit = int(rng.integers(0, mt))
            c[bit // 8] ^= 1 << (bit % 8)
            rc, k = O.dec(sid, bytes(c), sk)
            flips.append({"ct": bytes(c).hex(), "k": k.tobytes().hex(), "rc": rc})
        entry = {
            "key_seed": key_seed(sid).hex(),
            "pk_sha256": hashlib.sha256(pk.tobytes()).hexdigest(),
            "sk_sha256": hashlib.sha256(sk.tobytes()).hexdigest(),
            "enc": vec,
            "flipped": flips,
        }
        if mt % 8:
            c = bytearray(bytes.fromhex(vec[0]["ct"]))
            c[-1] |= 0x80
            rc, k = O.dec(sid, bytes(c), sk)
            entry["padding"] = {"ct": bytes(c).hex(), "k": k.tobytes().hex(), "rc": rc}
        out[name] = entry
        print(name, "done", flush=True)
    with open(os.path.join(ROOT, "tests", "golden", "kem_vectors.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
