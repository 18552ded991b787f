"""Builds and runs the reference's own GPU benchmark harness (mceliece-gpu-params/main.cu: CUDA-core, 1-bit BMMA
and INT8 tensor-core encapsulation, CUDA-core and 1-bit tensor-core decapsulation, each checked against
libmceliece), unmodified, on this machine's GPU.

REFERENCE MEASUREMENT ONLY: it records what the reference's kernels do on a GB300; nothing of it is linked into
the engine, and no test depends on it.

Three steps, so that the build also runs where the reference tree is absent:

1. extract (needs the reference tree, GMC_REFERENCE or /root/reference): the harness sources
   (mceliece-gpu-params/{main.cu, *.cuh, *.h, ref/<set>.cuh} and common/bench_common.h) are copied into
   oracle/_ref/gpu_src/ (git-ignored; nothing of them enters the repository).
2. build (anywhere oracle/_ref/gpu_src/ exists, with nvcc and a GPU architecture): the reference Makefile's own
   compile line for one set (-DPARAM_ID=<set>, -include ref/<set>.cuh, the HAS_FFT_* probes of the Makefile,
   -arch=sm_103a, -O3, -DN_TRIALS), linked against oracle/_ref/libmcref.so (libmceliece-20250507 `vec`, built
   by oracle/build_ref.py) through oracle/ref_gpu/shim.c, which provides libmceliece's public keypair / enc / dec
   names; the binary goes to oracle/_ref/gpu/mceliece-gpu-params-<set>.
3. run: executes the binary (it sweeps N = 256 .. 65536 itself) and copies its report to the given file.

Usage: python oracle/build_ref_gpu.py [--extract-only] [--set 8192128] [--trials 10] [--run OUT.txt]
"""
import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
GSRC = os.path.join(REF_DIR, "gpu_src")
GBIN = os.path.join(REF_DIR, "gpu")
SETS = ("348864", "460896", "6688128", "6960119", "8192128")
HARNESS = ("main.cu", "cc_kernels.cuh", "tc_kernels.cuh", "ref_prelude.cuh", "shake256.h", "crypto_sort.h")


def reference_root():
    return os.environ.get("GMC_REFERENCE", "/root/reference")


def available():
    return os.path.exists(os.path.join(GSRC, "main.cu"))


def extract():
    """Copies the harness sources of the reference into oracle/_ref/gpu_src/."""
    src = os.path.join(reference_root(), "mceliece-gpu-params")
    if not os.path.isdir(src):
        raise FileNotFoundError(f"reference harness not found: {src}")
    if os.path.exists(GSRC):
        shutil.rmtree(GSRC)
    os.makedirs(os.path.join(GSRC, "ref"))
    os.makedirs(os.path.join(GSRC, "common"))
    for f in HARNESS:
        shutil.copy(os.path.join(src, f), os.path.join(GSRC, f))
    for s in SETS:
        shutil.copy(os.path.join(src, "ref", f"{s}.cuh"), os.path.join(GSRC, "ref", f"{s}.cuh"))
    shutil.copy(os.path.join(reference_root(), "common", "bench_common.h"), os.path.join(GSRC, "common"))
    return GSRC


def build(set_name, trials=10, arch="sm_103a"):
    """Compiles the harness for one set; returns the binary's path."""
    if not available():
        extract()
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import pyref
    lib = pyref.build()  # oracle/_ref/libmcref.so
    os.makedirs(GBIN, exist_ok=True)
    shim_o = os.path.join(GBIN, "shim.o")
    r = subprocess.run(["gcc", "-O2", "-fPIC", "-c", os.path.join(HERE, "ref_gpu", "shim.c"), "-o", shim_o],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"shim compile failed:\n{r.stderr}")
    cuh = open(os.path.join(GSRC, "ref", f"{set_name}.cuh")).read()
    has_powers = 1 if "fft_powers" in cuh else 0
    has_post = 1 if "void postprocess(vec out" in cuh else 0
    out = os.path.join(GBIN, f"mceliece-gpu-params-{set_name}")
    libdir = os.path.dirname(os.path.abspath(lib))
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    # the reference Makefile's line: config.mk's NVCCFLAGS, then its per-set flags
    cmd = [nvcc, "-O3", f"-arch={arch}", "-I.", "-I" + os.path.join(GSRC, "common"),
           "-I" + os.path.join(HERE, "ref_gpu"), f"-DN_TRIALS={trials}", "-diag-suppress", "177",
           "-std=c++17", "-diag-suppress", "550", f"-DPARAM_ID={set_name}", f"-DHAS_FFT_POWERS={has_powers}",
           f"-DHAS_FFT_TR_POSTPROCESS={has_post}", "-include", f"ref/{set_name}.cuh", "main.cu", shim_o,
           "-o", out, "-L" + libdir, "-lmcref", "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, cwd=GSRC, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness compile failed for {set_name}:\n{r.stdout}\n{r.stderr}")
    return out


def run(binary, out_txt, timeout=1200):
    r = subprocess.run([binary], capture_output=True, text=True, timeout=timeout)
    with open(out_txt, "w") as f:
        f.write(f"$ {os.path.basename(binary)}  (exit {r.returncode})\n")
        f.write(r.stdout)
        if r.stderr:
            f.write("\n--- stderr ---\n" + r.stderr)
    return r.returncode


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--extract-only", action="store_true")
    ap.add_argument("--set", default="8192128", choices=SETS)
    ap.add_argument("--trials", type=int, default=10)
    ap.add_argument("--run", default=None, help="run the binary and write its report here")
    a = ap.parse_args()
    if a.extract_only:
        print(extract())
        sys.exit(0)
    b = build(a.set, a.trials)
    print(b)
    if a.run:
        sys.exit(run(b, a.run))
