#!/usr/bin/env python
"""Benchmark: batched Classic McEliece KEM, encapsulations + decapsulations per second on GB300.

Workload (default): mceliece8192128 full KEM. One step = one batched
encapsulation of N=65536 requests (seeded seed-chain randomness) plus one
batched decapsulation of N=65536 resident ciphertexts, 10% of them with one
uniformly random flipped bit (implicit-rejection path). Both against one
device-resident key pair. The metric counts each encapsulation and each
decapsulation as one operation: value = 2N / step time.

value: device time of the step (CUDA events on the launching stream), inputs
already in HBM, L2 flushed (256 MiB write) between timed steps.
e2e: the same step through the host-pointer C ABI calls (gmc_enc_batch /
gmc_dec_batch) from pinned host buffers, host<->device copies included.
roofline: the dominant kernel of the step, from the engine's own per-kernel
event timing (gmc_prof_*). The decoding kernels are bounded by the integer ALU
pipe: their algorithmic 32-bit lane operations (alu_lane_ops) over the launch
time, against the measured LOP3 rate of the GPU; the HBM figure rides along.
cpu_baseline: the reference's own CPU implementation (libmceliece-20250507,
portable vec code, built by oracle/build_ref.py; the oracle port only where
its sources are absent), threaded over the host cores, timed on the whole e2e
batch, every output of which is also checked against it (parity_check).

--impl reference: times that CPU implementation with all host threads on a
bounded sample of the workload, rank 0 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

SET_DEFAULT = "8192128"
N_DEFAULT = 65536


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gmc", choices=["gmc", "reference"])
    ap.add_argument("--set", default=SET_DEFAULT)
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--flip", type=float, default=0.10)
    ap.add_argument("--engine", default="auto", choices=["auto", "popc", "b1mma", "tc", "sparse"],
                    help="auto: per-set configuration (autotuned when --tune, else defaults)")
    ap.add_argument("--tune", action="store_true", help="autotune every set used before measuring")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-grouped", action="store_true", help="skip the mixed-key grouped-launch measurement")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="seconds per serving load level (60 = the "
                    "full serving configuration)")
    ap.add_argument("--no-sweep", action="store_true", help="skip the N = 256..65536 throughput sweep")
    ap.add_argument("--no-per-set", action="store_true", help="skip the per-set enc/s and dec/s at N = 65536")
    ap.add_argument("--no-engines", action="store_true", help="skip the syndrome-engine comparison")
    ap.add_argument("--no-keygen", action="store_true", help="skip the batched key-generation measurement")
    ap.add_argument("--no-ct", action="store_true", help="skip the constant-time decapsulation measurement")
    ap.add_argument("--keygen-keys", type=int, default=608, help="keys per batched key-generation call")
    ap.add_argument("--keygen-only", action="store_true",
                    help="measure only batched key generation (--keygen-sets, default all five) and print its JSON")
    ap.add_argument("--keygen-sets", default=None, help="comma-separated sets for the key-generation section")
    ap.add_argument("--keygen-calls", type=int, default=2, help="timed key-generation calls per set (best is kept)")
    ap.add_argument("--no-keygen-warmup", action="store_true", help="no 8-key warm-up call before the timed ones")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def ncu_traffic(set_name, n):
    """DRAM bytes per launch per kernel from a committed ncu summary for this workload ({} if none)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                        f"dram_traffic_kem{set_name}_n{n}.txt")
    out = {}
    if os.path.exists(path):
        for ln in open(path):
            ln = ln.strip()
            if ln and not ln.startswith("#"):
                k, v = ln.split()
                out[k] = int(v)
    return out


def algorithmic_bytes(kernel, z, n):
    """Bytes a kernel must move per launch of n requests (inputs read once, outputs written once)."""
    ew = (z["n"] + 31) // 32 * 4
    kw = (z["k"] + 31) // 32 * 4
    mw = (z["mt"] + 31) // 32 * 4
    ct = z["ct_bytes"]
    s2 = (2 * z["t"] * z["m"] + 31) // 32 * 4
    per = {
        "enc_sample": 32 + ew + kw,
        "enc_sample_syndrome": 32 + ew + mw,
        "enc_syndrome_gemm": kw + mw,
        "enc_finalize_hash": ew + mw + ct + 32,
        "dec_pack_ct": ct + (ct + 3) // 4 * 4,
        "dec_front_gemm": (ct + 3) // 4 * 4 + s2,
        "dec_bm": s2 + 2 * (1 << (6 if z["t"] <= 64 else 7)),
        "dec_fft_roots_reenc": 2 * (1 << (6 if z["t"] <= 64 else 7)) + s2 + ew + 4,
        "dec_tail_hash": ew + 4 + ct + 32 + 4,
    }[kernel]
    fixed = {"enc_syndrome_gemm": z["mt"] * kw, "enc_sample_syndrome": z["k"] * mw,
             "dec_front_gemm": 2 * z["t"] * z["m"] * ((ct + 3) // 4 * 4)}
    return per * n + fixed.get(kernel, 0)


def gf_mul_lane_ops(m):
    """32-bit lane operations of one bit-sliced GF(2^m) product (32 products at once): m^2 fused AND-XOR steps
    (one LOP3 each) and the reduction by the field polynomial, 4 (m = 13: x^13 + x^4 + x^3 + x + 1) or 2
    (m = 12: x^12 + x^3 + 1) XORs per high plane."""
    return m * m + (4 if m == 13 else 2) * (m - 1)


def alu_lane_ops(kernel, z):
    """Algorithmic 32-bit lane operations per request of the bit-sliced decoding kernels (None for the others).

    dec_bm: Berlekamp-Massey over 2t iterations; iteration n needs the discrepancy over coefficients
    i <= min(L, t) and the update C_i += f B_i over i <= min(max(L, n+1-L), t), one GF(2^m) product each, with
    the length profile L = ceil(n/2) of a full-rank syndrome sequence; 32 requests per lane operation.
    dec_fft_roots_reenc: the additive FFT's bottom-up pass, d = log2(2^d >= t) levels of 2^(m-1) butterflies,
    each one product and two m-plane additions, 32 chunks per lane operation (the top-down pass, the root
    extraction and the syndrome check are not counted)."""
    m, t = z["m"], z["t"]
    if kernel == "dec_bm":
        prods = 0
        for n in range(2 * t):
            L = min((n + 1) // 2, t)
            prods += min(L, t) + 1 + min(max(L, n + 1 - L), t) + 1
        return prods * gf_mul_lane_ops(m) / 32.0
    if kernel == "dec_fft_roots_reenc":
        d = max(1, (t - 1).bit_length())
        return d * 2 ** (m - 1) * (gf_mul_lane_ops(m) + 2 * m) / 32.0
    return None


def host_cpu():
    """Model name of the host CPU (lscpu), for the baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_impl():
    """The CPU implementation of the path: libmceliece-20250507 itself (its portable `vec` code, built by
    oracle/build_ref.py from the reference's tarball; the implementation libmceliece runs on arm64) when its
    sources are here, else the oracle port. Returns (module, kind, description)."""
    from oracle import pyref
    note = None
    if pyref.available():
        try:
            pyref.lib()
            return pyref, "reference", pyref.implementation()
        except Exception as e:  # a failed build is reported, and the port stands in
            note = f"libmceliece build failed: {str(e).splitlines()[0][:120]}"
    from oracle import pyoracle as O
    O.lib()
    return O, "port", "oracle/mceliece_oracle.c (plain C restatement of libmceliece-20250507)" + (
        f"; {note}" if note else "; libmceliece sources absent")


def cpu_baseline(sid, pk, sk, cts_host, seeds_host, c_gpu, k_gpu, kdec_gpu, threads):
    """The CPU implementation timed on the host cores, and every GPU output of the e2e batch checked against it.
    With libmceliece itself the whole batch (N encapsulations + N decapsulations) is both the timed sample and
    the parity check; with the slower oracle port a bounded sample of a few seconds is timed and checked."""
    M, kind, impl = cpu_impl()
    n = len(seeds_host)
    if kind == "port":
        t0 = time.perf_counter()
        M.dec_batch(sid, sk, cts_host[:threads], threads=threads)
        t_dec1 = (time.perf_counter() - t0) / threads
        n_dec = int(min(n, max(threads, 6.0 / max(t_dec1, 1e-9))))
        t0 = time.perf_counter()
        M.enc_batch(sid, pk, seeds_host[:threads], threads=threads)
        t_enc1 = (time.perf_counter() - t0) / threads
        n_enc = int(min(n, max(threads, 3.0 / max(t_enc1, 1e-9))))
    else:
        n_enc = n_dec = n
    t0 = time.perf_counter()
    oc, ok_, _ = M.enc_batch(sid, pk, seeds_host[:n_enc], threads=threads)
    t_enc = time.perf_counter() - t0
    t0 = time.perf_counter()
    okd, _ = M.dec_batch(sid, sk, cts_host[:n_dec], threads=threads)
    t_dec = time.perf_counter() - t0
    enc_rate, dec_rate = n_enc / t_enc, n_dec / t_dec
    value = (n_enc + n_dec) / (n_enc / enc_rate + n_dec / dec_rate)
    bad_c = int((oc != c_gpu[:n_enc]).any(1).sum())
    bad_k = int((ok_ != k_gpu[:n_enc]).any(1).sum())
    bad_kd = int((okd != kdec_gpu[:n_dec]).any(1).sum())
    what = "the whole e2e batch" if (n_enc, n_dec) == (n, n) else "a bounded sample of the same workload"
    return {
        "value": value, "unit": "KEM ops/s (enc+dec, 50/50)", "cores": threads, "kind": kind,
        "implementation": impl, "host_cpu": host_cpu(),
        "sample": f"{what}: {n_enc} encapsulations + {n_dec} decapsulations (10% bit-flipped), {threads} threads; "
                  f"enc {enc_rate:.0f}/s, dec {dec_rate:.0f}/s",
        "enc_ops_s": enc_rate, "dec_ops_s": dec_rate,
    }, {"checked_against": kind, "checked_enc": n_enc, "checked_dec": n_dec, "of": n,
        "mismatched_ct": bad_c, "mismatched_enc_key": bad_k, "mismatched_dec_key": bad_kd,
        "mismatches": bad_c + bad_k + bad_kd}


def metric_name(set_name):
    """The metric string both arms print (the reference arm measures the same workload on the host cores)."""
    return f"mceliece{set_name} KEM enc+dec ops/s (batched, bit-exact)"


def workload(set_name, n, flip):
    return (f"mceliece{set_name} full KEM: {n} batched encapsulations + {n} batched decapsulations "
            f"({int(flip * 100)}% with one flipped bit) per step, one resident key pair")


def run_reference(args, rank):
    """The reference's CPU implementation of the path on all host threads: libmceliece-20250507 itself (its
    portable `vec` code, built from the reference's bundled sources; the oracle port stands in only when those are
    absent). Each step is a bounded sample of the workload: 512 encapsulations and 512 decapsulations (10% with
    one flipped bit) per host thread, the same key pair, seeds and flips as the GPU arm's kind of input."""
    if rank != 0:
        return
    M, kind, impl = cpu_impl()
    sid = M.sid(args.set)
    z = M.sizes(sid)
    threads = os.cpu_count() or 1
    pk, sk = M.keypair(sid, bytes([0x5A]) * 32)
    rng = np.random.default_rng(7)
    sample = min(args.n, (512 if kind == "reference" else 16) * threads)
    seeds = rng.integers(0, 256, (sample, 32), dtype=np.uint8)
    cts, _, _ = M.enc_batch(sid, pk, rng.integers(0, 256, (sample, 32), dtype=np.uint8), threads=threads)
    flip = rng.choice(sample, int(args.flip * sample), replace=False)
    for i in flip:
        b = int(rng.integers(0, z["mt"]))
        cts[i, b // 8] ^= np.uint8(1 << (b % 8))

    def step():
        M.enc_batch(sid, pk, seeds, threads=threads)
        M.dec_batch(sid, sk, cts, threads=threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    value = 2 * sample / dt
    line = {
        "impl": "reference", "metric": metric_name(args.set), "value": value,
        "unit": "KEM ops/s (enc+dec, 50/50)", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded keys, seeds and flips)",
        "config": {"workload": workload(args.set, args.n, args.flip), "set": args.set, "n_per_gpu": args.n},
        "cpu_baseline": {"value": value, "unit": "KEM ops/s (enc+dec, 50/50)", "cores": threads, "kind": kind,
                         "implementation": impl, "host_cpu": host_cpu(),
                         "sample": f"{sample} enc + {sample} dec (10% bit-flipped) per step, {threads} threads"},
        "e2e": {"value": value, "unit": "KEM ops/s (enc+dec, 50/50)", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def constant_time_cost(gmc, torch, dev, L, set_name, n, steps, flip=0.10):
    """Decapsulation of n ciphertexts (10% one-bit-flipped) with the table forms and with the constant-time
    kernels (gmc_set_dec_constant_time): device ms per batch (CUDA events, L2 flushed), the per-kernel split of
    both, and whether every session key and return code agrees."""
    import ctypes
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    sid = gmc.set_id(set_name)
    z = gmc.set_sizes(sid)
    pk, sk = gmc.keypair(sid, bytes([0x6B]) * 32)
    P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
    gen = torch.Generator(device=dev)
    gen.manual_seed(71)
    seeds = torch.randint(0, 256, (n, 32), dtype=torch.uint8, device=dev, generator=gen)
    cts = torch.empty((n, z["ct_bytes"]), dtype=torch.uint8, device=dev)
    k = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    P.enc_batch_dev(cts.data_ptr(), k.data_ptr(), seeds.data_ptr(), n, 0, st)
    rng = np.random.default_rng(17)
    nflip = int(flip * n)
    idx = torch.from_numpy(rng.choice(n, nflip, replace=False)).to(dev)
    bits = torch.from_numpy(rng.integers(0, z["mt"], nflip)).to(dev)
    cts[idx, bits // 8] ^= (1 << (bits % 8)).to(torch.uint8)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device=dev)
    out = {"set": set_name, "n": n}
    keys_rc = {}
    for name, on in (("table", False), ("constant_time", True)):
        gmc.set_dec_constant_time(on)
        kd = torch.empty((n, 32), dtype=torch.uint8, device=dev)
        rc = torch.empty(n, dtype=torch.int32, device=dev)
        for _ in range(3):
            S.dec_batch_dev(kd.data_ptr(), cts.data_ptr(), n, rc.data_ptr(), st)
        torch.cuda.synchronize()
        L.gmc_prof_enable(1)
        ms = []
        for i in range(steps):
            flush.fill_(i)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            S.dec_batch_dev(kd.data_ptr(), cts.data_ptr(), n, rc.data_ptr(), st)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        buf = ctypes.create_string_buffer(4096)
        L.gmc_prof_report(buf, 4096)
        L.gmc_prof_enable(0)
        ks = {}
        for ln in buf.value.decode().strip().splitlines():
            nm, cnt, t = ln.split()
            ks[nm] = float(t) / steps
        out[name] = {"ms_per_batch": sum(ms) / len(ms), "dec_ops_s": n / (sum(ms) / len(ms) / 1e3), "kernels_ms": ks}
        keys_rc[name] = (kd.clone(), rc.clone())
    gmc.set_dec_constant_time(False)
    out["outputs_identical"] = bool(torch.equal(keys_rc["table"][0], keys_rc["constant_time"][0]) and
                                    torch.equal(keys_rc["table"][1], keys_rc["constant_time"][1]))
    out["slowdown"] = out["constant_time"]["ms_per_batch"] / out["table"]["ms_per_batch"]
    return out


MIX_SETS = [0, 0, 1, 1, 2, 3, 4, 4]  # 2x348864, 2x460896, 6688128, 6960119, 2x8192128


def zipf_counts(total, k, s=1.2, seed=11):
    w = 1.0 / np.arange(1, k + 1) ** s
    w = w[np.random.default_rng(seed).permutation(k)]
    c = np.floor(total * w / w.sum()).astype(int)
    c[0] += total - c.sum()
    return c


def grouped_mix(gmc, torch, dev, total, steps, warmup):
    """8 keys over the five sets, Zipf(1.2) request counts summing to `total`, each key's requests
    split 50/50 enc/dec: one plain batched call per (key, op) vs one grouped CUDA-graph launch."""
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    gen = torch.Generator(device=dev)
    gen.manual_seed(77)
    counts = zipf_counts(total, len(MIX_SETS))
    keys, bufs, groups = [], [], []
    for i, sid in enumerate(MIX_SETS):
        z = gmc.set_sizes(sid)
        pk, sk = gmc.keypair(sid, bytes([i + 1]) * 32)
        P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
        ne = int(counts[i]) // 2
        nd = int(counts[i]) - ne
        seeds = torch.randint(0, 256, (max(ne, 1), 32), dtype=torch.uint8, device=dev, generator=gen)
        c = torch.empty((max(ne, 1), z["ct_bytes"]), dtype=torch.uint8, device=dev)
        k = torch.empty((max(ne, 1), 32), dtype=torch.uint8, device=dev)
        s2 = torch.randint(0, 256, (max(nd, 1), 32), dtype=torch.uint8, device=dev, generator=gen)
        cts = torch.empty((max(nd, 1), z["ct_bytes"]), dtype=torch.uint8, device=dev)
        kd = torch.empty((max(nd, 1), 32), dtype=torch.uint8, device=dev)
        kt = torch.empty((max(nd, 1), 32), dtype=torch.uint8, device=dev)
        P.enc_batch_dev(cts.data_ptr(), kt.data_ptr(), s2.data_ptr(), nd, 0, st)  # valid ciphertexts
        keys.append((P, S))
        bufs.append((seeds, c, k, cts, kd, ne, nd))
        groups.append((P, ne, seeds.data_ptr(), c.data_ptr(), k.data_ptr(), 0))
        groups.append((S, nd, cts.data_ptr(), 0, kd.data_ptr(), 0))
    torch.cuda.synchronize()

    def plain():
        for (P, S), (seeds, c, k, cts, kd, ne, nd) in zip(keys, bufs):
            P.enc_batch_dev(c.data_ptr(), k.data_ptr(), seeds.data_ptr(), ne, 0, st)
            S.dec_batch_dev(kd.data_ptr(), cts.data_ptr(), nd, 0, st)

    plan = gmc.Plan(groups)

    def timed(fn):
        for _ in range(max(3, warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_plain = timed(plain)
    k_plain = [b[2].clone() for b in bufs] + [b[4].clone() for b in bufs]
    ms_group = timed(lambda: plan.launch(st))
    k_group = [b[2] for b in bufs] + [b[4] for b in bufs]
    same = all(torch.equal(a, b) for a, b in zip(k_plain, k_group))
    info = plan.info()
    plan.close()
    live = int(sum(counts))
    return {
        "workload": f"{len(MIX_SETS)} keys over the five sets (2x348864, 2x460896, 6688128, 6960119, 2x8192128), "
                    f"Zipf(1.2) request counts summing to {total}, 50/50 enc/dec",
        "counts": [int(x) for x in counts],
        "plain_ms": ms_plain, "plain_ops_s": total / (ms_plain / 1e3),
        "grouped_ms": ms_group, "grouped_ops_s": total / (ms_group / 1e3),
        "speedup": ms_plain / ms_group, "pipelines": info["pipelines"], "outputs_identical": same,
        "padded_rows": info["padded_rows"], "live_rows": live,
        "padding_share": (info["padded_rows"] - live) / max(1, info["padded_rows"]),
    }


def n_sweep(gmc, torch, dev, set_name, ns, steps, flip=0.10):
    """KEM ops/s (enc + dec of N requests, device-timed, L2 flushed between steps) for each batch size N."""
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    sid = gmc.set_id(set_name)
    z = gmc.set_sizes(sid)
    pk, sk = gmc.keypair(sid, bytes([0x5A]) * 32)
    P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
    gen = torch.Generator(device=dev)
    gen.manual_seed(99)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device=dev)
    out = {}
    for n in ns:
        seeds = torch.randint(0, 256, (n, 32), dtype=torch.uint8, device=dev, generator=gen)
        seeds2 = torch.randint(0, 256, (n, 32), dtype=torch.uint8, device=dev, generator=gen)
        c = torch.empty((n, z["ct_bytes"]), dtype=torch.uint8, device=dev)
        k = torch.empty((n, 32), dtype=torch.uint8, device=dev)
        cts = torch.empty((n, z["ct_bytes"]), dtype=torch.uint8, device=dev)
        kd = torch.empty((n, 32), dtype=torch.uint8, device=dev)
        P.enc_batch_dev(cts.data_ptr(), kd.data_ptr(), seeds2.data_ptr(), n, 0, st)
        nflip = int(flip * n)
        if nflip:
            rng = np.random.default_rng(n)
            idx = torch.from_numpy(rng.choice(n, nflip, replace=False)).to(dev)
            bits = torch.from_numpy(rng.integers(0, z["mt"], nflip)).to(dev)
            cts[idx, bits // 8] ^= (1 << (bits % 8)).to(torch.uint8)

        def step():
            P.enc_batch_dev(c.data_ptr(), k.data_ptr(), seeds.data_ptr(), n, 0, st)
            S.dec_batch_dev(kd.data_ptr(), cts.data_ptr(), n, 0, st)

        for _ in range(3):
            step()
        ms = []
        for i in range(steps):
            flush.fill_(i)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        m = sum(ms) / len(ms)
        out[str(n)] = {"ops_s": 2 * n / (m / 1e3), "ms_per_step": m}
    return out


def per_set(gmc, torch, dev, n, steps, flip=0.10):
    """Encapsulations/s and decapsulations/s of every parameter set at N requests, each operation timed on its own
    (device-resident inputs, L2 flushed between launches, CUDA events), the form in which the reference's GPU harness
    reports its engines (N / mean launch time)."""
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device=dev)
    out = {}
    for set_name in gmc.SETS:
        sid = gmc.set_id(set_name)
        z = gmc.set_sizes(sid)
        pk, sk = gmc.keypair(sid, bytes([0x3C]) * 32)
        P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
        gen = torch.Generator(device=dev)
        gen.manual_seed(7)
        seeds = torch.randint(0, 256, (n, 32), dtype=torch.uint8, device=dev, generator=gen)
        c = torch.empty((n, z["ct_bytes"]), dtype=torch.uint8, device=dev)
        k = torch.empty((n, 32), dtype=torch.uint8, device=dev)
        kd = torch.empty((n, 32), dtype=torch.uint8, device=dev)
        P.enc_batch_dev(c.data_ptr(), k.data_ptr(), seeds.data_ptr(), n, 0, st)
        cts = c.clone()
        nflip = int(flip * n)
        if nflip:
            rng = np.random.default_rng(n)
            idx = torch.from_numpy(rng.choice(n, nflip, replace=False)).to(dev)
            bits = torch.from_numpy(rng.integers(0, z["mt"], nflip)).to(dev)
            cts[idx, bits // 8] ^= (1 << (bits % 8)).to(torch.uint8)

        def timed(fn):
            for _ in range(3):
                fn()
            ms = []
            for i in range(steps):
                flush.fill_(i)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            return sum(ms) / len(ms)

        enc_ms = timed(lambda: P.enc_batch_dev(c.data_ptr(), k.data_ptr(), seeds.data_ptr(), n, 0, st))
        dec_ms = timed(lambda: S.dec_batch_dev(kd.data_ptr(), cts.data_ptr(), n, 0, st))
        out[set_name] = {"enc_ops_s": n / (enc_ms / 1e3), "dec_ops_s": n / (dec_ms / 1e3), "enc_ms": enc_ms,
                         "dec_ms": dec_ms}
        del P, S, seeds, c, k, kd, cts
    return out


def syndrome_engines(gmc, torch, dev, L, set_name, n, steps, tc_peak_tflops, fp8_mac_peak, b1_mac_peak=None):
    """The encapsulation syndrome c[0:mt] = e[0:mt] ^ T e[mt:n] of n requests with each engine, from the
    engine's per-kernel events: the GF(2) GEMM (mt x k bits times k x n) for the CUDA-core, legacy b1 mma and
    tcgen05 engines, and for the sparse engine the sampler time it adds over the sampler alone.
    Work = mt*k bit-MACs per request; the tcgen05 figure as a fraction of the measured rate of its own MMA
    instruction (gmc_tc_f8_peak: FP8 E4M3, M = 128, N = 256, K = 32, operands resident in shared memory), and
    for context of the measured dense bf16 cuBLAS peak."""
    import ctypes
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    sid = gmc.set_id(set_name)
    z = gmc.set_sizes(sid)
    pk, _ = gmc.keypair(sid, bytes([0x33]) * 32)
    P = gmc.PublicKey(sid, pk)
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    seeds = torch.randint(0, 256, (n, 32), dtype=torch.uint8, device=dev, generator=gen)
    c = torch.empty((n, z["ct_bytes"]), dtype=torch.uint8, device=dev)
    k = torch.empty((n, 32), dtype=torch.uint8, device=dev)
    macs = z["mt"] * z["k"] * n
    prev = gmc.get_gemm_engine()
    times = {}
    for name, eng in (("popc", gmc.GEMM_POPC), ("b1mma", gmc.GEMM_B1MMA), ("tc", gmc.GEMM_TC),
                      ("sparse", gmc.GEMM_SPARSE)):
        gmc.set_gemm_engine(eng)
        for _ in range(2):
            P.enc_batch_dev(c.data_ptr(), k.data_ptr(), seeds.data_ptr(), n, 0, st)
        torch.cuda.synchronize()
        L.gmc_prof_enable(1)
        reps = 2 if name == "b1mma" else steps
        for _ in range(reps):
            P.enc_batch_dev(c.data_ptr(), k.data_ptr(), seeds.data_ptr(), n, 0, st)
        torch.cuda.synchronize()
        buf = ctypes.create_string_buffer(4096)
        L.gmc_prof_report(buf, 4096)
        L.gmc_prof_enable(0)
        ks = {}
        for ln in buf.value.decode().strip().splitlines():
            nm, cnt, ms = ln.split()
            ks[nm] = float(ms) / reps
        times[name] = ks
    gmc.set_gemm_engine(prev)
    sample_only = times["tc"].get("enc_sample", 0.0)
    out = {"set": set_name, "n": n, "bit_macs": macs, "engines": {},
           "fp8_mma_peak_tflops": 2.0 * fp8_mac_peak / 1e12}
    for name in ("popc", "b1mma", "tc"):
        ms = times[name]["enc_syndrome_gemm"]
        e = {"ms": ms, "bit_macs_per_s": macs / (ms / 1e3)}
        if name == "b1mma" and b1_mac_peak:
            e["b1mma_peak_bit_macs_per_s"] = b1_mac_peak
            e["frac_of_measured_b1mma_peak"] = macs / (ms / 1e3) / b1_mac_peak
        if name == "tc":
            tf = 2.0 * macs / (ms / 1e3) / 1e12
            e["fp8_equivalent_tflops"] = tf
            e["frac_of_measured_fp8_mma_peak"] = macs / (ms / 1e3) / fp8_mac_peak
            e["frac_of_measured_bf16_peak"] = tf / tc_peak_tflops
        out["engines"][name] = e
    sp = times["sparse"]["enc_sample_syndrome"]
    out["engines"]["sparse"] = {"ms_sampler_with_syndrome": sp, "ms_added_over_sampler": sp - sample_only,
                                "note": "XOR of <= t public-key columns per request inside the sampler"}
    return out


# 32-bit instruction count of one Keccak-f[1600] permutation on 32-bit halves, fully fused (a lower bound):
# per round theta 20 lop3 (5-way column XORs) + 10 shf (rot 1) + 50 lop3 (A ^ C[x-1] ^ rot C[x+1]),
# rho 48 shf (24 rotations, none by 0 or 32), chi 50 lop3 (b ^ (~c & d)), iota 2 lop3.
KECCAK_LOP3_PER_PERM = 24 * (20 + 50 + 50 + 2)
KECCAK_SHF_PER_PERM = 24 * (10 + 48)


def keccak_rates(z, n, kernels, pk=None):
    """Keccak-f[1600] permutations per second of the two session-key hash kernels (each request hashes the
    1 + n/8 + ct-byte preimage: ceil((len + 1) / 136) permutations), beside the integer-op ceiling: the
    permutation's op count over the GPU's measured lop3 and funnel-shift rates."""
    perms = (1 + z["n"] // 8 + z["ct_bytes"] + 1 + 135) // 136
    out = {"perms_per_hash": perms}
    ceiling = None
    if pk is not None:
        ceiling = 1.0 / (KECCAK_LOP3_PER_PERM / pk["lop3_per_s"] + KECCAK_SHF_PER_PERM / pk["shf_per_s"])
        out["int32_peak"] = {"lop3_per_s": pk["lop3_per_s"], "shf_per_s": pk["shf_per_s"],
                             "ops_per_perm": {"lop3": KECCAK_LOP3_PER_PERM, "shf": KECCAK_SHF_PER_PERM},
                             "ceiling_perms_per_s": ceiling}
    for kname in ("enc_finalize_hash", "dec_tail_hash"):
        if kname in kernels:
            r = n * perms / (kernels[kname]["ms"] / 1e3)
            out[kname] = {"perms_per_s": r}
            if ceiling:
                out[kname]["frac_of_ceiling"] = r / ceiling
    return out


def keygen_rates(gmc, torch, nkeys, cpu_threads, with_cpu=True, sets=None, calls=2, warmup=True):
    """Batched key generation (gmc_keypair_batch, host buffers in and out) per parameter set: keys/s
    over nkeys seeds, beside the CPU implementation's keypair (libmceliece itself, else the oracle port) on the
    host threads: a bounded sample whose keys are also compared byte for byte with the GPU's."""
    import hashlib
    out = {"nkeys": nkeys, "sets": {}}
    if with_cpu:
        from concurrent.futures import ThreadPoolExecutor
        O, kind, impl = cpu_impl()
    for name in (sets or gmc.SETS):
        sid = gmc.set_id(name)
        seeds = np.frombuffer(b"".join(hashlib.sha256(b"bench-kg" + bytes([sid]) + i.to_bytes(4, "little")).digest()
                                       for i in range(nkeys)), np.uint8).reshape(nkeys, 32)
        if warmup:
            gmc.keypair_batch(sid, seeds[:8])  # warm-up (tables, pool)
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(1, calls)):
            t0 = time.perf_counter()
            pk, sk = gmc.keypair_batch(sid, seeds)
            ts.append(time.perf_counter() - t0)
        e = {"keys_s": nkeys / min(ts), "s_per_call": min(ts)}
        if with_cpu:
            ns = cpu_threads
            t0 = time.perf_counter()
            with ThreadPoolExecutor(cpu_threads) as ex:
                ref = list(ex.map(lambda s_: O.keypair(sid, bytes(s_)), seeds[:ns]))
            t_cpu = time.perf_counter() - t0
            bad = sum(int(not (np.array_equal(pk[i], np.asarray(ref[i][0])) and
                               np.array_equal(sk[i], np.asarray(ref[i][1])))) for i in range(ns))
            e["cpu_baseline"] = {"value": ns / t_cpu, "unit": "keys/s", "cores": cpu_threads, "kind": kind,
                                 "implementation": impl,
                                 "sample": f"{ns} keypairs of the same seeds, {cpu_threads} threads"}
            e["checked_keys"] = ns
            e["mismatches"] = bad
        out["sets"][name] = e
    return out


def serving(gmc, torch, seconds):
    """16 device-resident key pairs over the five sets, 50/50 enc/dec, Poisson arrivals at 10, 25, 50, 75, 90 and
    100% of the measured peak; p50/p99/p99.9/max latency (arrival to completion) against sequential one-request
    calls."""
    pairs = []
    for i in range(16):
        sid = i % 5
        pk, sk = gmc.keypair(sid, bytes([0x40 + i]) * 32)
        pairs.append((gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)))
    srv = gmc.Server(max_batch=65536, slots=3, mem_fraction=0.4)
    for P, S in pairs:
        srv.add_key(P)
        srv.add_key(S)
    peak = srv.loadgen(pairs, rate=2e8, seconds=max(1.0, seconds / 2), seed=1)  # overload: saturated throughput
    # untimed warm-up at the lowest level: the first small batches of a process paid one-time costs (a stall of
    # tens of ms in the first level of some runs, never in later ones)
    srv.loadgen(pairs, rate=0.1 * peak["ops_s"], seconds=1.0, seed=7)
    levels = {}
    for frac in (0.1, 0.25, 0.5, 0.75, 0.9, 1.0):
        r = srv.loadgen(pairs, rate=frac * peak["ops_s"], seconds=seconds, seed=int(frac * 100))
        levels[f"{int(frac * 100)}%"] = {k: r[k] for k in ("offered_rate", "ops_s", "p50_ms", "p99_ms", "p999_ms",
                                                             "max_ms", "mean_batch", "completed", "submitted",
                                                             "worst_batch")}
    srv.close()
    # sequential one-request calls (libmceliece calling convention, resident keys, host buffers)
    lat = []
    rng = np.random.default_rng(3)
    for i in range(100):
        P, S = pairs[i % 16]
        z = P.sizes
        seed = rng.integers(0, 256, (1, 32), dtype=np.uint8)
        t0 = time.perf_counter()
        if i % 2 == 0:
            P.enc_batch(seed)
        else:
            c, _, _ = pairs[i % 16][0].enc_batch(seed)  # untimed ciphertext for this dec
            t0 = time.perf_counter()
            S.dec_batch(c)
        lat.append((time.perf_counter() - t0) * 1e3)
    lat = np.array(lat)
    return {
        "workload": "16 key pairs (sets uniform over the five), 50/50 enc/dec, Poisson arrivals, "
                    f"{seconds:.0f} s per load level, latency = arrival to completion",
        "peak_ops_s": peak["ops_s"], "peak_mean_batch": peak["mean_batch"], "levels": levels,
        "sequential_one_request": {"ops_s": 1e3 / lat.mean(), "p50_ms": float(np.percentile(lat, 50)),
                                   "p99_ms": float(np.percentile(lat, 99))},
    }


def main():
    args = parse()
    rank, local_rank, world = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch
    import tensormceliece_gb300 as gmc
    import ctypes

    torch.cuda.set_device(local_rank)
    if args.keygen_only:
        if rank == 0:
            sets = args.keygen_sets.split(",") if args.keygen_sets else None
            print(json.dumps({"keygen": keygen_rates(gmc, torch, args.keygen_keys, os.cpu_count() or 1,
                                                     with_cpu=not args.no_cpu, sets=sets, calls=args.keygen_calls,
                                                     warmup=not args.no_keygen_warmup)}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank)
    L = gmc.lib()
    L.gmc_prof_report.argtypes = [ctypes.c_char_p, ctypes.c_int]
    gmc.set_gemm_engine({"auto": -1, "popc": gmc.GEMM_POPC, "b1mma": gmc.GEMM_B1MMA, "tc": gmc.GEMM_TC,
                         "sparse": gmc.GEMM_SPARSE}[args.engine])
    tuning = {}
    if args.tune:
        for sname in sorted({args.set} | ({gmc.SETS[s] for s in MIX_SETS} if not args.no_grouped else set())):
            t0 = time.perf_counter()
            tuning[sname] = gmc.autotune(sname, args.n)
            tuning[sname]["seconds"] = round(time.perf_counter() - t0, 2)
    sid = gmc.set_id(args.set)
    z = gmc.set_sizes(sid)
    N = args.n
    # resident key pair (product key generation; untimed setup)
    pk, sk = gmc.keypair(sid, bytes([0x5A]) * 32)
    P, S = gmc.PublicKey(sid, pk), gmc.SecretKey(sid, sk)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    seeds = torch.randint(0, 256, (N, 32), dtype=torch.uint8, device=dev, generator=gen)
    c_out = torch.empty((N, z["ct_bytes"]), dtype=torch.uint8, device=dev)
    k_out = torch.empty((N, 32), dtype=torch.uint8, device=dev)
    k_dec = torch.empty((N, 32), dtype=torch.uint8, device=dev)
    cts_in = torch.empty((N, z["ct_bytes"]), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    # decapsulation inputs: valid ciphertexts from a separate seeded batch, 10% with one flipped bit
    seeds2 = torch.randint(0, 256, (N, 32), dtype=torch.uint8, device=dev, generator=gen)
    P.enc_batch_dev(cts_in.data_ptr(), k_dec.data_ptr(), seeds2.data_ptr(), N, 0, st)
    rng = np.random.default_rng(4321 + rank)
    nflip = int(args.flip * N)
    idx = torch.from_numpy(rng.choice(N, nflip, replace=False)).to(dev)
    bits = torch.from_numpy(rng.integers(0, z["mt"], nflip)).to(dev)
    cts_in[idx, bits // 8] ^= (1 << (bits % 8)).to(torch.uint8)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device=dev)  # 256 MiB > L2

    def step():
        P.enc_batch_dev(c_out.data_ptr(), k_out.data_ptr(), seeds.data_ptr(), N, 0, st)
        S.dec_batch_dev(k_dec.data_ptr(), cts_in.data_ptr(), N, 0, st)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local_rank) if rank == 0 else None
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    # per-kernel events on the launching stream throughout the timed steps (the engine's profiler)
    L.gmc_prof_enable(1)
    wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(i)
        evs[i][0].record(stream)
        step()
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop() if clocks else None
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        torch.distributed.barrier()
    ms_per_step = total_ms / args.steps
    value = world * 2 * N / (ms_per_step / 1e3)

    # per-kernel breakdown: average duration per step over the timed steps
    buf = ctypes.create_string_buffer(4096)
    nk = L.gmc_prof_report(buf, 4096)
    L.gmc_prof_enable(0)
    kernels = {}
    for line in buf.value.decode().strip().splitlines():
        name, cnt, ms = line.split()
        kernels[name] = {"launches": int(cnt) // args.steps, "ms": float(ms) / args.steps}
    launches_per_step = sum(v["launches"] for v in kernels.values())
    tot = sum(v["ms"] for v in kernels.values()) or 1.0
    hbm_peak, tc_peak, peak_kind = measured_peaks()
    ipk = gmc.int32_peak()  # measured LOP3 / funnel-shift lane-op rates of this GPU
    for name, v in kernels.items():
        v["share"] = v["ms"] / tot
        v["gbs"] = algorithmic_bytes(name, z, N) / (v["ms"] / 1e3) / 1e9
        ops = alu_lane_ops(name, z)
        if ops is not None:
            v["alu_lane_ops_per_request"] = ops
            v["alu_frac"] = ops * N / (v["ms"] / 1e3) / ipk["lop3_per_s"]
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    dom_bytes = algorithmic_bytes(dom, z, N)
    achieved_gbs = dom_bytes / (kernels[dom]["ms"] / 1e3) / 1e9
    traffic = ncu_traffic(args.set, N).get(dom)
    hbm = {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
           "algorithmic_bytes_per_launch": dom_bytes, "peak_source": peak_kind}
    dom_ops = alu_lane_ops(dom, z)
    if dom_ops is not None:
        # the decoding kernels are bounded by the integer ALU pipe: algorithmic lane operations of one launch
        # over its duration, against the measured LOP3 rate of this GPU
        achieved = dom_ops * N / (kernels[dom]["ms"] / 1e3)
        roofline = {
            "bound": "int-alu", "kernel": dom, "achieved": achieved / 1e12, "peak": ipk["lop3_per_s"] / 1e12,
            "unit": "T lane-ops/s", "frac": achieved / ipk["lop3_per_s"], "traffic": traffic,
            "algorithmic_lane_ops_per_launch": dom_ops * N, "algorithmic_lane_ops_per_request": dom_ops,
            "peak_source": "measured on this GPU (gmc_int32_peak: dependent-free LOP3 stream)",
            "traffic_source": ("one ncu capture of the same command (dram__bytes_read.sum + "
                               "dram__bytes_write.sum)" if traffic else None),
            "hbm": hbm,
        }
    else:
        roofline = dict(hbm, bound="hbm", kernel=dom, traffic=traffic)

    line = {
        "metric": metric_name(args.set),
        "value": value, "unit": "KEM ops/s (enc+dec, 50/50)", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8",
        "data": "synthetic: seeded key pair, random 32-byte request seeds, 10% bit-flipped ciphertexts",
        "config": {"workload": workload(args.set, N, args.flip), "set": args.set, "n_per_gpu": N,
                   "parallelism": f"replicas x{world}", "l2": "flushed (256 MiB write) between timed steps",
                   "gemm_engine": args.engine,
                   "tuning": {k: gmc.tune_get(k) for k in gmc.SETS} if not tuning else tuning},
        "gpu_launches": launches_per_step * args.steps,
        "kernels": kernels,
        "roofline": roofline,
        "clocks": clk,
        "wall_s_timed_loop": wall,
    }

    line["keccak"] = keccak_rates(z, N, kernels, ipk)
    if rank == 0 and not args.no_sweep:
        line["n_sweep"] = {"set": args.set, "flip": args.flip,
                           "ops_s": n_sweep(gmc, torch, dev, args.set, [256, 1024, 4096, 16384, 65536], 5, args.flip)}
        # config 1: mceliece348864, one key, 256 encapsulations + 256 decapsulations per step
        line["config1"] = {"set": "348864", "n": 256, "flip": args.flip,
                           "ops_s": n_sweep(gmc, torch, dev, "348864", [256], 20, args.flip)["256"]}
    if rank == 0 and not args.no_per_set:
        # every parameter set at 65536 requests, enc and dec timed separately (the reference GPU harness's form)
        line["per_set_n65536"] = per_set(gmc, torch, dev, 65536, 5, args.flip)
    if rank == 0 and not args.no_engines:
        fp8_peak = gmc.tc_f8_peak()
        b1_peak = gmc.b1mma_peak()
        line["syndrome_engines"] = [syndrome_engines(gmc, torch, dev, L, s_, 65536, 5, tc_peak, fp8_peak, b1_peak)
                                    for s_ in dict.fromkeys(("348864", args.set))]
        # the decapsulation front end on the tcgen05 engine (the step's GEMM) against the same measured peak
        fe = kernels.get("dec_front_gemm")
        if fe:
            fmacs = 2 * z["t"] * z["m"] * z["mt"] * N
            line["front_end_gemm_tensor"] = {
                "bit_macs": fmacs, "ms": fe["ms"], "tflops_fp8_equivalent": 2.0 * fmacs / (fe["ms"] / 1e3) / 1e12,
                "fp8_mma_peak_tflops": 2.0 * fp8_peak / 1e12, "frac_of_measured_fp8_mma_peak":
                    fmacs / (fe["ms"] / 1e3) / fp8_peak}
    if rank == 0 and not args.no_ct:
        line["constant_time"] = constant_time_cost(gmc, torch, dev, L, args.set, N, 5, args.flip)
    if rank == 0 and not args.no_grouped:
        line["grouped"] = grouped_mix(gmc, torch, dev, N, max(5, args.steps // 2), args.warmup)
    if rank == 0 and not args.no_serving:
        line["serving"] = serving(gmc, torch, args.serve_seconds)
    if rank == 0 and not args.no_keygen:
        line["keygen"] = keygen_rates(gmc, torch, args.keygen_keys, os.cpu_count() or 1,
                                      with_cpu=not args.no_cpu and world == 1,
                                      sets=args.keygen_sets.split(",") if args.keygen_sets else None)

    if rank == 0 and not args.no_e2e:
        # end to end through the host-pointer C ABI (pinned host buffers)
        seeds_h = torch.empty((N, 32), dtype=torch.uint8, pin_memory=True)
        seeds_h.copy_(seeds.cpu())
        cts_h = torch.empty((N, z["ct_bytes"]), dtype=torch.uint8, pin_memory=True)
        cts_h.copy_(cts_in.cpu())
        c_h = torch.empty((N, z["ct_bytes"]), dtype=torch.uint8, pin_memory=True)
        k_h = torch.empty((N, 32), dtype=torch.uint8, pin_memory=True)
        kd_h = torch.empty((N, 32), dtype=torch.uint8, pin_memory=True)

        def e2e_step():
            r1 = L.gmc_enc_batch(P.handle, c_h.data_ptr(), k_h.data_ptr(), seeds_h.data_ptr(), N, None)
            r2 = L.gmc_dec_batch(S.handle, kd_h.data_ptr(), cts_h.data_ptr(), N, None)
            assert r1 == 0 and r2 == 0

        for _ in range(2):
            e2e_step()
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            e2e_step()
            ts.append(time.perf_counter() - t0)
        e2e_ms = 1e3 * sum(ts) / len(ts)
        line["e2e"] = {"value": 2 * N / (e2e_ms / 1e3), "unit": "KEM ops/s (enc+dec, 50/50)",
                       "h2d_bytes_per_step": N * 32 + N * z["ct_bytes"],
                       "d2h_bytes_per_step": N * (z["ct_bytes"] + 32) + N * 32, "ms_per_step": e2e_ms}
        if not args.no_cpu and world == 1:
            threads = os.cpu_count() or 1
            cb, check = cpu_baseline(sid, pk, sk, cts_h.numpy(), seeds_h.numpy(), c_h.numpy(), k_h.numpy(),
                                     kd_h.numpy(), threads)
            line["cpu_baseline"] = cb
            line["parity_check"] = check
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
