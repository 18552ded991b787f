"""Builds the reference's own CPU implementation of the KEM -- libmceliece-20250507's portable `vec` code, the
library the reference bundles as its oracle (deps/libmceliece-20250507.tar.gz) -- into oracle/_ref/libmcref.so.

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: the tests use it to pin the oracle restatement to the real library,
bench.py times it as the CPU baseline and checks GPU outputs against it; the engine never links it.

Two steps, so the build also runs where the reference tree is absent:

1. extract (needs the reference tree, GMC_REFERENCE or /root/reference): the files that the `vec` implementation
   of all 20 KEM variants compiles from are read out of the reference's tarball into oracle/_ref/src/ (git-ignored;
   nothing of the library enters the repository). The library's own configure script, a Python build system that
   generates namespacing headers, is not run: the small headers in oracle/ref_include/ give the same names.
2. compile (anywhere oracle/_ref/src/ exists, x86_64 or aarch64): every source with the library's default flags
   (gcc -Wall -fPIC -fwrapv -O2), each set's symbols under mcref_<set>_, linked with oracle/ref_harness.c and a
   second build of oracle/kat.c into oracle/_ref/libmcref.so.

Usage: python oracle/build_ref.py [--extract-only] [--force]
"""
import concurrent.futures as cf
import hashlib
import os
import posixpath
import shutil
import subprocess
import sys
import tarfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(REF_DIR, "src")
OBJ = os.path.join(REF_DIR, "obj")
LIB = os.path.join(REF_DIR, "libmcref.so")
STAMP = os.path.join(SRC, ".extracted")
TARBALL = "deps/libmceliece-20250507.tar.gz"
PREFIX = "libmceliece-20250507/"
BASE = ("348864", "460896", "6688128", "6960119", "8192128")
VARIANTS = tuple(s + v for v in ("", "pc", "f", "pcf") for s in BASE)
CFLAGS = ["-Wall", "-fPIC", "-fwrapv", "-O2"]  # libmceliece-20250507 compilers/default
INTS = ("int8", "int16", "int32", "int64", "uint8", "uint16", "uint32", "uint64")


def reference_root():
    return os.environ.get("GMC_REFERENCE", "/root/reference")


def _wanted(name):
    if not name.startswith(PREFIX):
        return False
    rel = name[len(PREFIX):]
    for v in VARIANTS:
        if rel.startswith(f"crypto_kem/{v}/vec/"):
            return True
    return (rel.startswith("cryptoint/") and (rel.endswith(".h") or rel.endswith("_optblocker.c"))) or rel in (
        "crypto_sort/int16/portable4/sort.c", "crypto_sort/int32/portable4/sort.c",
        "crypto_sort/int64/portable4/sort.c", "crypto_xof/shake256/unrollround/shake256.c",
        "crypto_xof/shake256/unrollround/keccak.inc", "crypto_xof/bitwrite16/64/write.c",
        "include-build/crypto_declassify.h", "LICENSE", "README.md")


def extract(force=False):
    """Reads the needed members of the reference's libmceliece tarball into oracle/_ref/src/."""
    tb = os.path.join(reference_root(), TARBALL)
    if os.path.exists(STAMP) and not force:
        return SRC
    if not os.path.exists(tb):
        raise FileNotFoundError(f"reference tarball not found: {tb}")
    digest = hashlib.sha256(open(tb, "rb").read()).hexdigest()
    if os.path.exists(SRC):
        shutil.rmtree(SRC)
    os.makedirs(SRC)
    with tarfile.open(tb) as tf:
        members = {m.name: m for m in tf.getmembers()}

        def resolve(m, depth=0):
            # the variant directories link their files into the base set's directories
            while m is not None and m.issym() and depth < 16:
                m = members.get(posixpath.normpath(posixpath.join(posixpath.dirname(m.name), m.linkname)))
                depth += 1
            return m if m is not None and m.isfile() else None

        for name, m in members.items():
            if not _wanted(name):
                continue
            rel = name[len(PREFIX):]
            if ".." in rel.split("/"):
                continue
            real = resolve(m)
            if real is None:
                continue
            dst = os.path.join(SRC, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            with tf.extractfile(real) as f, open(dst, "wb") as g:
                g.write(f.read())
    with open(STAMP, "w") as f:
        f.write(f"{TARBALL} sha256 {digest}\n")
    return SRC


def _jobs():
    """(source, object, extra flags) for every translation unit."""
    inc = ["-I", os.path.join(HERE, "ref_include"), "-I", os.path.join(SRC, "cryptoint"),
           "-I", os.path.join(SRC, "include-build")]
    jobs = []
    for v in VARIANTS:
        d = os.path.join(SRC, "crypto_kem", v, "vec")
        ns = [f"-DCRYPTO_NAMESPACE(x)=mcref_{v}_##x", f"-DCRYPTO_SHARED_NAMESPACE(x)=mcref_{v}_shared_##x"]
        for fn in sorted(os.listdir(d)):
            if fn.endswith(".c"):
                jobs.append((os.path.join(d, fn), os.path.join(OBJ, v, fn[:-2] + ".o"), ["-I", d, *inc, *ns]))
    for t in ("int16", "int32", "int64"):
        jobs.append((os.path.join(SRC, "crypto_sort", t, "portable4", "sort.c"), os.path.join(OBJ, f"sort_{t}.o"),
                     [*inc, f"-Dcrypto_sort=mcref_sort_{t}"]))
    jobs.append((os.path.join(SRC, "crypto_xof", "shake256", "unrollround", "shake256.c"),
                 os.path.join(OBJ, "shake256.o"),
                 ["-I", os.path.join(SRC, "crypto_xof", "shake256", "unrollround"), *inc,
                  "-Dcrypto_xof=mcref_xof_shake256"]))
    jobs.append((os.path.join(SRC, "crypto_xof", "bitwrite16", "64", "write.c"), os.path.join(OBJ, "bitwrite16.o"),
                 [*inc, "-Dcrypto_xof=mcref_xof_bitwrite16"]))
    for t in INTS:
        jobs.append((os.path.join(SRC, "cryptoint", f"{t}_optblocker.c"), os.path.join(OBJ, f"{t}_optblocker.o"),
                     inc))
    jobs.append((os.path.join(HERE, "ref_harness.c"), os.path.join(OBJ, "ref_harness.o"), ["-I", HERE]))
    jobs.append((os.path.join(HERE, "kat.c"), os.path.join(OBJ, "kat_ref.o"), ["-I", HERE, "-DKAT_FOR_REFERENCE"]))
    return jobs


def _cc():
    return os.environ.get("CC", "gcc")


def _compile(job):
    src, obj, extra = job
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    r = subprocess.run([_cc(), *CFLAGS, *extra, "-c", src, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stderr}")
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(HERE, f) for f in ("ref_harness.c", "ref_harness.h", "kat.c", "build_ref.py")]
    deps += [os.path.join(HERE, "ref_include", f) for f in os.listdir(os.path.join(HERE, "ref_include"))]
    return any(os.path.getmtime(d) > t for d in deps) or os.path.getmtime(STAMP) > t


def available():
    """True when the extracted sources are present (the library can be compiled here)."""
    return os.path.exists(STAMP)


def build(force=False):
    """Extracts (when the reference tree is present and nothing was extracted yet) and compiles; returns the
    library path. Raises when neither the extracted sources nor the reference tarball exist."""
    if not os.path.exists(STAMP):
        extract()
    if not force and not _stale():
        return LIB
    jobs = _jobs()
    with cf.ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(_compile, jobs))
    tmp = LIB + ".tmp"
    r = subprocess.run([_cc(), "-shared", "-o", tmp, *objs, "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    shutil.rmtree(OBJ, ignore_errors=True)  # objects are not reused; keep the tree small
    return LIB


if __name__ == "__main__":
    if "--extract-only" in sys.argv:
        print(extract(force="--force" in sys.argv))
    else:
        if "--force" in sys.argv and os.path.exists(os.path.join(reference_root(), TARBALL)):
            extract(force=True)
        print(build(force="--force" in sys.argv))
