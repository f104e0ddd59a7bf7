#!/usr/bin/env python3
"""Damascus Fold commit+prove benchmark on GB300.

Workloads (seeded ChaCha20 random files; no public dataset is involved):
  serve   (default) the serving stream: Poisson arrivals at 200 requests/s, sizes
          50% log-uniform 50 KB-1 MiB, 40% 1-8 MiB, 10% 16 MiB (d = 6..11), per-file
          seeds, 150 GB HBM budget.  A step replays the whole stream.
  batched 64 files, log-uniform 50 KB-4 MiB (d = 6..10), one engine batch per step.
  d6/d9/d11  the plain single-proof full flows (53,248 B / 1 MiB / 16 MiB).
  serve_seed  the serving stream with every file under the default system seed and
          the provers' generator cache on (each shape expanded and transformed once).
  verify  the serving stream's files proven under the default system seed, then
          verified by the streaming verifier service; a step verifies every proof.

Reported, for the serve and batched workloads:
  value   MiB/s of the continuous-batching engine with every request arriving at
          t = 0 (saturating replay), files resident in HBM
  e2e     the same through the C ABI from pinned host memory (H2D of every file and
          D2H of every proof inside the timed region; the engine's copies read the
          caller's pinned buffers, and e2e.staged_value gives the copying submission)
  plain_mib_s   the plain one-request-at-a-time GPU path on the same files
  latency_ms    p50/p99 of the real-time Poisson replay (arrival -> proof ready)
For the plain workloads a step is one commit+prove of one file.  The verify
workload reports proofs verified per second (service, service without the
generator cache, and the one-at-a-time verifier) and p50/p99 latency.

``--impl reference`` times the CPU restatement of the reference's algorithm (the
oracle; the Rust reference cannot be built on this machine) on a bounded sample
of the same workload, on all host threads.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "commit+prove MiB/s"
UNIT = "MiB/s"
MIB = float(1 << 20)
MASTER_SEED = 0xDA3A5C05
EPOCH = bytes([11]) * 32
SERVE_BUDGET = 150 * 10 ** 9

WORKLOADS = {
    "serve": dict(kind="serve", requests=96, rate=200.0,
                  desc="serving stream: Poisson 200 req/s, 50% 50KB-1MiB / 40% 1-8MiB / 10% 16MiB, "
                       "150 GB HBM budget"),
    "batched": dict(kind="batched", files=64, lo=50_000, hi=4 << 20,
                    desc="batched: 64 files log-uniform 50KB-4MiB (d 6-10), one engine batch"),
    "d6": dict(kind="plain", file_bytes=53_248, desc="plain full flow d=6: 53,248 random bytes, 64x64 witness"),
    "d9": dict(kind="plain", file_bytes=1 << 20, desc="plain full flow d=9: 1 MiB random file, 512x512 witness"),
    "d10": dict(kind="plain", file_bytes=4 << 20, desc="plain full flow d=10: 4 MiB random file, 1024x1024 witness"),
    "d11": dict(kind="plain", file_bytes=16 << 20, desc="plain full flow d=11: 16 MiB random file, 2048x2048 witness"),
    "ringmul": dict(kind="ringmul", pairs=4096, n=512,
                    desc="ring-mult microbench: 4,096 random degree-512 R_q pairs per step"),
    "verify": dict(kind="verify", requests=96, rate=200.0, cache_bytes=16 << 30,
                   desc="verifier stream: proofs of the serving stream's 96 files (d 6-11) under the default "
                        "system seed, verified by the streaming verifier service (16 GiB generator cache)"),
}
WORKLOADS["serve_seed"] = dict(kind="serve", requests=96, rate=200.0, system_seed=True, generator_cache=16 << 30,
                               desc="serving stream under one system seed (SystemParams default) with the provers' "
                                    "generator cache (16 GiB): Poisson 200 req/s, 50% 50KB-1MiB / 40% 1-8MiB / "
                                    "10% 16MiB, 150 GB HBM budget")
WORKLOADS["verify16m"] = dict(kind="verify", requests=32, file_bytes=16 << 20, rate=200.0, cache_bytes=16 << 30,
                              desc="verifier stream of large proofs: 32 proofs of 16 MiB files (d = 11, 2048 x "
                                   "2048 witness) under the default system seed, streaming verifier service "
                                   "(16 GiB generator cache)")
SYSTEM_SEED = bytes([7]) * 32  # SystemParams::default seed_generators
KERNELS = ["file_hash", "unpack_witness", "gen_generators", "fold", "ntt_fwd", "mac", "mac_split", "finish"]
VERIFY_KERNELS = ["gen_generators", "fold_gen"]


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class Ranks:
    """The replicas' only coordination: a barrier around the timed region and the
    max of each rank's elapsed time.  Every rank proves its own files (no data
    exchange), so N>1 is N independent replicas with weak scaling."""

    def __init__(self, world: int, backend: str = "nccl", device=None):
        self.world, self.backend, self.device = world, backend, device
        if world > 1:
            import torch
            import torch.distributed as dist
            if not dist.is_initialized():
                kw = {"device_id": device} if backend == "nccl" else {}
                dist.init_process_group(backend, **kw)

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64, device=self.device if self.backend == "nccl" else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            import torch.distributed as dist
            if dist.is_initialized():
                dist.destroy_process_group()


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def workload_files(wl, rank: int = 0):
    """[(bytes, seed, arrival_s)] for the workload (per rank for replicas)."""
    from damascus000_gb300 import synth
    base = MASTER_SEED + 7919 * rank
    if wl["kind"] == "verify" and "file_bytes" in wl:
        return [(synth.random_file(base, wl["file_bytes"], 40_000 + i)[0], SYSTEM_SEED, i / wl["rate"])
                for i in range(wl["requests"])]
    if wl["kind"] in ("serve", "verify"):
        # one seed for every file in the verify and system-seed forms, as SystemParams::default
        one_seed = SYSTEM_SEED if wl["kind"] == "verify" or wl.get("system_seed") else None
        return synth.serving_files(base, wl["requests"], wl["rate"], one_seed)
    if wl["kind"] == "batched":
        return synth.batched_files(base, wl["files"], wl["lo"], wl["hi"])
    return None


def ring_pairs(wl, rank: int = 0):
    """Two byte strings of pairs * n random Z_q elements (16-byte LE, below 2^112)."""
    import numpy as np
    from damascus000_gb300 import synth
    nbytes = wl["pairs"] * wl["n"] * 16
    out = []
    for which in range(2):
        raw, _ = synth.random_file(MASTER_SEED + 7919 * rank, nbytes, 30_000 + which)
        w = np.frombuffer(raw, dtype=np.uint32).reshape(-1, 4).copy()
        w[:, 3] &= 0xFFFF
        out.append(w.tobytes())
    return out[0], out[1]


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu, self.proc, self.lines, self.thread = gpu_index, None, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=lambda: [self.lines.append(l.strip()) for l in self.proc.stdout],
                                       daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        if not self.lines:  # timed region shorter than one sampling period: one reading right after it
            try:
                out = subprocess.run(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                      "-i", str(self.gpu)], capture_output=True, text=True, timeout=10).stdout
                self.lines = [l.strip() for l in out.splitlines() if l.strip()]
            except Exception:
                pass
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline (oracle)
def cpu_baseline(wl, budget_s: float = 15.0, threads: int = 0, proofs=None):
    """The oracle (CPU restatement of the reference algorithm) on a bounded sample."""
    import oracle as O
    from damascus000_gb300 import synth
    O.build()
    threads = threads or (os.cpu_count() or 1)
    if wl["kind"] == "ringmul":
        import concurrent.futures as cf
        a, b = ring_pairs(wl, 0)
        sz = wl["n"] * 16
        done = 0
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            while time.perf_counter() - t0 < budget_s and done < wl["pairs"]:
                k = min(threads * 4, wl["pairs"] - done)
                list(ex.map(lambda i: O.negacyclic_multiply_bytes(a[i * sz:(i + 1) * sz], b[i * sz:(i + 1) * sz],
                                                                  wl["n"]), range(done, done + k)))
                done += k
        el = time.perf_counter() - t0
        return {"value": done / el, "unit": "products/s", "cores": threads, "kind": "port",
                "sample": f"{done} degree-{wl['n']} negacyclic products by the oracle restatement (2n-point NTT "
                          f"over 8 CRT primes + Garner CRT per product) on {threads} threads in {el:.1f} s"}
    if wl["kind"] == "verify":
        import concurrent.futures as cf
        if proofs is None:
            # inputs: oracle-made proofs of the stream's files up to 300 KB (untimed)
            small = [d for d, _, _ in workload_files(wl) if len(d) <= 300_000][:24]
            if not small:
                return {"value": None, "unit": "proofs/s", "cores": threads, "kind": "port",
                        "sample": "none: the workload's proofs come from the GPU arm (16 MiB files take the oracle "
                                  "prover minutes each)"}
            proofs = [O.prove(d, SYSTEM_SEED, EPOCH, use_ntt=True, threads=threads) for d in small]
            what = f"oracle-made proofs of the stream's first {len(small)} files up to 300 KB (d 6-8)"
        else:
            what = "the workload's own proofs in stream order"
        submitted = 0
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            pending = set()
            while True:
                while len(pending) < threads and time.perf_counter() - t0 < budget_s:
                    pending.add(ex.submit(O.verify, proofs[submitted % len(proofs)], EPOCH))
                    submitted += 1
                if not pending:
                    break
                finished, pending = cf.wait(pending, return_when=cf.FIRST_COMPLETED)
                if any(f.result() for f in finished):
                    raise SystemExit("oracle verifier rejected an honest proof")
        el = time.perf_counter() - t0
        return {"value": submitted / el, "unit": "proofs/s", "cores": threads, "kind": "port",
                "sample": f"{submitted} verifications by the oracle restatement (generator expansion, transcript replay, "
                          f"module folds) of {what}, {threads} at a time on {threads} threads, in {el:.1f} s"}
    if wl["kind"] != "plain":
        r = StratifiedOracle(wl, threads).step(0, max_full_depth=10)
        return {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port", "sample": r["sample"],
                "per_depth": r["per_depth"]}
    items = ((synth.random_file(MASTER_SEED, wl["file_bytes"], 1000 + i)) for i in range(64))
    what = f"full commit+prove of {wl['file_bytes']}-byte files"
    done = nbytes = 0
    t0 = time.perf_counter()
    for data, seed in items:
        O.prove(data, seed, EPOCH, use_ntt=True, threads=threads)
        done += 1
        nbytes += len(data)
        if time.perf_counter() - t0 >= budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": nbytes / MIB / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} {what}; oracle restatement (per-product 2n-point NTT over 8 CRT primes + Garner "
                      f"CRT, commitment columns over {threads} threads); {nbytes} bytes in {el:.1f} s"}


class StratifiedOracle:
    """The oracle's MiB/s on a workload of mixed depths, stratified by depth.

    Every depth present is timed on a full commit+prove of one of the workload's
    own files.  The oracle, like the reference, transforms every column of the
    square witness, zero padding included, so a proof's CPU time depends on its
    depth and not on how full the file is: the workload's time is the sum over
    depths of its proofs of that depth times the seconds measured there, and its
    rate its bytes over that time.  Depths up to 9 take seconds and are
    re-sampled every step on the next file of that depth; deeper ones (d = 10:
    tens of seconds, d = 11: minutes) are timed once, on the first file of that
    depth, and reused."""

    def __init__(self, wl, threads):
        import oracle as O
        O.build()
        self.O, self.threads = O, threads
        self.by_depth = {}
        for d, s, _ in workload_files(wl):
            self.by_depth.setdefault(O.layout_for_byte_len(len(d))[0], []).append((d, s))
        self.once = {}

    def _time(self, data, seed):
        t0 = time.perf_counter()
        self.O.prove(data, seed, EPOCH, use_ntt=True, threads=self.threads)
        return time.perf_counter() - t0

    def step(self, k, max_full_depth=11, resample_depth=9):
        per, proj_s, total, sampled = {}, 0.0, 0, 0
        for depth in sorted(self.by_depth):
            files = self.by_depth[depth]
            dbytes = sum(len(d) for d, _ in files)
            total += dbytes
            if depth > max_full_depth:
                continue
            if depth <= resample_depth:
                data, seed = files[k % len(files)]
                n, secs = len(data), self._time(data, seed)
            else:
                if depth not in self.once:
                    data, seed = files[0]
                    self.once[depth] = (len(data), self._time(data, seed))
                n, secs = self.once[depth]
            per[depth] = {"files_in_workload": len(files), "workload_bytes": dbytes, "sampled_bytes": n,
                          "seconds_per_proof": round(secs, 3)}
            proj_s += len(files) * secs
            sampled += dbytes
        value = sampled / MIB / proj_s
        skipped = [d for d in self.by_depth if d > max_full_depth]
        sample = (f"oracle restatement (per-product 2n-point NTT over 8 CRT primes + Garner CRT, commitment columns "
                  f"over {self.threads} threads), one full commit+prove per depth of the workload's own files "
                  f"(d <= {resample_depth}: the next file of that depth each step; deeper: the first, timed once); "
                  "value = the workload's bytes / sum over depths of (its proofs there x the measured seconds "
                  "per proof); per depth: " + "; ".join(f"d{d}: {v['files_in_workload']} proofs, one of "
                                                        f"{v['sampled_bytes']} B in {v['seconds_per_proof']} s"
                                                        for d, v in per.items()))
        if skipped:
            sample += (f"; depths {skipped} ({total - sampled} of {total} bytes) not sampled in this bounded leg, "
                       "the value covers the rest of the workload")
        return {"value": value, "per_depth": per, "sample": sample}


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    vals, base, per_depth = [], None, None
    if wl["kind"] in ("serve", "batched"):
        strat = StratifiedOracle(wl, threads)
        import oracle as O
        d6 = min(strat.by_depth)
        for i in range(args.warmup):  # warm-up: one proof of the shallowest depth
            O.prove(*strat.by_depth[d6][i % len(strat.by_depth[d6])], EPOCH, use_ntt=True, threads=threads)
        for k in range(args.steps):
            r = strat.step(k)
            vals.append(r["value"])
            base, per_depth = base or r, r["per_depth"]
        base = {"value": base["value"], "cores": threads, "sample": base["sample"]}
    else:
        for i in range(args.warmup + args.steps):
            r = cpu_baseline(wl, budget_s=4.0 if i else 10.0)
            if r["value"] is None:
                print(json.dumps({"impl": "reference", "unavailable": r["sample"]}))
                return 0
            base = base or r
            if i >= args.warmup:
                vals.append(r["value"])
    value = statistics.median(vals) if vals else base["value"]
    # one step of the GPU arm's workload at the sampled rate (the sample itself is bounded)
    if wl["kind"] == "ringmul":
        step_ms = wl["pairs"] / value * 1000.0
    elif wl["kind"] == "verify":
        step_ms = wl["requests"] / value * 1000.0
    elif wl["kind"] == "plain":
        step_ms = wl["file_bytes"] / MIB / value * 1000.0
    else:
        step_ms = sum(len(d) for d, _, _ in workload_files(wl)) / MIB / value * 1000.0
    metric, unit = {"ringmul": ("ring-mults/s", "products/s"),
                    "verify": ("proofs verified/s", "proofs/s")}.get(wl["kind"], (METRIC, UNIT))
    line = {"impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "ms_per_step_note": "one step of the workload at the sampled rate (each timed step is a bounded sample)",
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32/u128 integer", "data": "synthetic",
            "config": {"workload": wl["desc"], "impl_note": "CPU restatement of the reference algorithm; the Rust "
                       "reference cannot be built here (no cargo/rustc on either machine)",
                       "step_values": vals},
            "cpu_baseline": {"value": value, "unit": unit, "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if per_depth:
        line["cpu_baseline"]["per_depth_last_step"] = per_depth
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU
# DRAM bytes per algorithmic byte of a kernel, from ncu captures of small cases
# (dram__bytes_read.sum + dram__bytes_write.sum over the captured launches ÷ the
# same launches' algorithmic bytes).  Used to state `traffic` per launch of this
# run; the capture, not this run, measured it.
DRAM_PER_ALGO_BYTE = {
    "ntt_fwd": (0.93, "ncu of the transform at ring 2^11, the ring most of its bytes run at (0.90-0.95; rings "
                      "of 2^7-2^9 stay in L2 at 0.31-0.34: an upper estimate for a mixed workload), "
                      "profiles/ntt_fwd_traffic_by_ring.txt"),
}
# The transform is bound by the integer multiplier, not by HBM.  Its multiplies,
# counted from the kernel's code (dm_ntt.cuh, dm_field.cuh): a butterfly is one
# Shoup product (one mul.hi, two mul.lo); the input residue of a 112-bit
# coefficient under one prime is three 32x32->64 multiply-adds and a Shoup
# product (residue_fwd), and the output's reduction a mul.hi and a mul.lo
# (shoup_one).  Each form is weighted by its issue cost relative to mul.lo, and
# the peak is mul.lo's rate: all three rates measured on this device in this run
# (damascus_measure_int_multiply).
N_PRIMES = 9
NTT_MULS = {"butterfly": {"mul.hi": 1, "mul.lo": 2},
            "residue": {"mad.wide": 3, "mul.hi": 2, "mul.lo": 3}}  # per coefficient and prime


def int_pipe(dom, n, ms, byts, ops, rates):
    """Integer-multiplier fraction of the transform from counted multiplies."""
    if dom != "ntt_fwd" or not rates or not all(rates.values()):
        return None
    weight = {k: rates["mul.lo"] / v for k, v in rates.items()}  # mul.lo issue slots per instruction
    per = {u: sum(c * weight[k] for k, c in f.items()) for u, f in NTT_MULS.items()}
    coeffs = byts / (16 + 4 * N_PRIMES)  # each coefficient: 16 B read, nine 4-byte residues written
    slots = ops * per["butterfly"] + coeffs * N_PRIMES * per["residue"]
    rate = slots / (ms / 1000.0)
    return {"pipe": "integer multiplier (FMA-heavy)", "achieved": rate, "peak": rates["mul.lo"],
            "unit": "mul.lo-equivalent multiplies/s", "frac": rate / rates["mul.lo"],
            "counted_per_launch": slots / n, "multiplies": NTT_MULS,
            "measured_rates_ops_per_s": rates, "issue_weight_vs_mul_lo": weight,
            "butterflies_per_s": ops / (ms / 1000.0),
            "note": "peak and weights measured in this run on this GPU (independent chains of each form); counts "
                    "only the arithmetic's multiplies, while ncu's FMA-heavy busy % also includes the compiler's "
                    "integer moves and address arithmetic on that pipe"}


def roofline(stats, measured_on, rates=None):
    peak, src = read_peaks()
    live = {k: v for k, v in stats.items() if v}
    if not live:
        return None
    dom = max(live, key=lambda k: live[k][1])
    n, ms, byts, ops = live[dom]
    achieved = byts / n / (ms / n / 1000.0) / 1e9
    total_ms = sum(v[1] for v in live.values())
    ratio = DRAM_PER_ALGO_BYTE.get(dom)
    out = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured"
           else src, "traffic": byts / n * ratio[0] if ratio else None,
           "traffic_source": (f"not measured in this run: algorithmic bytes per launch x {ratio[0]} DRAM bytes "
                              f"per algorithmic byte from {ratio[1]}") if ratio else None,
           "algo_bytes_per_launch": byts / n, "avg_launch_ms": ms / n, "share_of_kernel_time": ms / total_ms,
           "measured_on": measured_on,
           "kernels": {k: {"launches": v[0], "ms": round(v[1], 4), "algo_bytes": v[2], "algo_ops": v[3],
                           "achieved_gbs": v[2] / (v[1] / 1000.0) / 1e9}
                       for k, v in live.items()}}
    ip = int_pipe(dom, n, ms, byts, ops, rates)
    if ip:
        out["int_pipe"] = ip
        out["note"] = ("integer-bound kernel: frac is its share of the HBM copy peak; its own limit is the "
                       "integer multiplier, int_pipe.frac")
    return out


def workload_digests(name, rank):
    """The oracle's proof digests for this workload's files (rank 0's files only)."""
    sets = {"serve": "serving", "serve_seed": "serving_system_seed", "batched": "batched", "d9": "d9",
            "d11": "d11"}
    p = ROOT / "tests" / "golden" / "workload_digests.json"
    if rank != 0 or name not in sets or not p.exists():
        return None
    d = json.loads(p.read_text())
    if d.get("master_seed") != MASTER_SEED or sets[name] not in d:
        return None
    return d[sets[name]]


def check_digests(entries, proofs, lengths, indices=None):
    """(proofs equal to the oracle's, proofs checked) by SHA-256."""
    import hashlib
    by_index = {e["index"]: e for e in entries}
    ok = checked = 0
    for k, (p, ln) in enumerate(zip(proofs, lengths)):
        e = by_index.get(indices[k] if indices else k)
        if e is None or e["file_len"] != ln:
            continue
        checked += 1
        ok += hashlib.sha256(p).hexdigest() == e["proof_sha256"]
    return ok, checked


def host_hash_rate(D, nbytes: int = 64 << 20, reps: int = 5):
    """GB/s of the host BLAKE3 on one core (the keyed entry point hashes on the
    calling thread; its chunks run in vector lanes), the transcript's hash."""
    import ctypes
    L = D.load()
    data = bytes(range(256)) * (nbytes // 256)
    out = ctypes.create_string_buffer(32)
    L.damascus_blake3_keyed(b"\x07" * 32, data, len(data), out)
    t0 = time.perf_counter()
    for _ in range(reps):
        L.damascus_blake3_keyed(b"\x07" * 32, data, len(data), out)
    return reps * len(data) / (time.perf_counter() - t0) / 1e9


def collect(eng, tickets):
    """[(proof, latency ms)] in ticket order, each proof taken as soon as its
    request finishes (Engine.as_completed), not in submission order."""
    got = {t: (p, lat) for t, p, lat in eng.as_completed(tickets)}
    return [got[t] for t in tickets]


def measure_batched(ctx, D, torch, args, rank, world, ranks):
    """The 64-file batched set (log-uniform 50 KB - 4 MiB, d 6-10): one engine batch
    per step against the plain one-at-a-time path, every proof checked against the
    oracle's digests.  Reported beside the serving stream's line."""
    wl = dict(WORKLOADS["batched"], name="batched")
    files = workload_files(wl, rank)
    total = sum(len(d) for d, _, _ in files)
    dev = [torch.frombuffer(bytearray(d), dtype=torch.uint8).cuda() for d, _, _ in files]
    torch.cuda.synchronize()
    with D.Engine(ctx) as eng:
        def batch():
            ts = [eng.submit_device(t.data_ptr(), len(d), s, EPOCH) for t, (d, s, _) in zip(dev, files)]
            return [r[0] for r in collect(eng, ts)]
        for _ in range(args.warmup):
            batch()
        ranks.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            proofs = batch()
        torch.cuda.synchronize()
        step_s = ranks.max(time.perf_counter() - t0) / args.steps
    ranks.barrier()
    t0 = time.perf_counter()
    for t, (d, s, _) in zip(dev, files):
        ctx.prove_device(t.data_ptr(), len(d), s, EPOCH)
    torch.cuda.synchronize()
    plain_s = ranks.max(time.perf_counter() - t0)
    digests = workload_digests("batched", rank)
    exact = check_digests(digests, proofs, [len(d) for d, _, _ in files]) if digests else None
    return {"workload": wl["desc"], "value": world * total / MIB / step_s, "unit": UNIT,
            "ms_per_step": step_s * 1000.0, "total_bytes": total, "steps": args.steps,
            "plain_mib_s": world * total / MIB / plain_s, "batched_vs_plain": plain_s / step_s,
            "bit_exact_vs_oracle": f"{exact[0]}/{exact[1]}" if exact else None,
            "note": "files resident in HBM; wall time of the whole batch (host challenges included)"}


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    f = math.floor(k)
    c = min(f + 1, len(xs) - 1)
    return xs[f] + (xs[c] - xs[f]) * (k - f)


def run_gpu(args, wl):
    import ctypes

    import torch

    import damascus000_gb300 as D

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    ranks = Ranks(world, "nccl", torch.device("cuda", local))
    barrier, max_over_ranks = ranks.barrier, ranks.max

    ctx = D.Context(local, hbm_budget_bytes=SERVE_BUDGET if wl["kind"] != "plain" else 0)
    int_rates = ctx.measure_int_multiply()  # the integer-multiplier peaks of the transform's roofline
    if wl.get("generator_cache"):
        ctx.set_generator_cache(wl["generator_cache"])
    cpu_inputs = None  # the verify workloads time the oracle verifier on their own proofs
    line = {"metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32/u128 integer",
            "data": "synthetic (seeded ChaCha20 files)"}

    if wl["kind"] == "ringmul":
        n, pairs = wl["n"], wl["pairs"]
        a, b = ring_pairs(wl, rank)
        da = torch.frombuffer(bytearray(a), dtype=torch.uint8).cuda()
        db = torch.frombuffer(bytearray(b), dtype=torch.uint8).cuda()
        dout = torch.empty_like(da)
        pa = torch.frombuffer(bytearray(a), dtype=torch.uint8).pin_memory()
        pb = torch.frombuffer(bytearray(b), dtype=torch.uint8).pin_memory()
        po = torch.empty(len(a), dtype=torch.uint8).pin_memory()
        torch.cuda.synchronize()
        for _ in range(args.warmup):
            ctx.ring_mul_batch_device(da.data_ptr(), db.data_ptr(), dout.data_ptr(), n, pairs)
        ctx.set_profiling(True)
        ctx.reset_stats()
        clocks = ClockSampler(local)
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        ev0.record()
        for _ in range(args.steps):
            ctx.flush_l2()
            ctx.ring_mul_batch_device(da.data_ptr(), db.data_ptr(), dout.data_ptr(), n, pairs)
        ev1.record()
        torch.cuda.synchronize()
        clk = clocks.stop()
        stats = {k: ctx.kernel_stat(k) for k in KERNELS + ["ring_mul"]}
        ctx.set_profiling(False)
        # device time of the products themselves (the per-step L2 flush excluded)
        dev_ms = sum(v[1] for k, v in stats.items() if v and k in ("ntt_fwd", "ring_mul"))
        total_ms = max_over_ranks(dev_ms)
        value = world * args.steps * pairs / (total_ms / 1000.0)
        lib = D.load()

        def host_call():
            ctx.check(lib.damascus_ring_mul_batch(ctx.handle, ctypes.cast(pa.data_ptr(), ctypes.c_char_p),
                                                  ctypes.cast(pb.data_ptr(), ctypes.c_char_p),
                                                  ctypes.c_void_p(po.data_ptr()), n, pairs), "ring_mul_batch")

        for _ in range(args.warmup):  # the host path's own buffers enter the device pool here
            host_call()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            host_call()
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        ok = bytes(po.numpy()) == bytes(dout.cpu().numpy())
        line.update({"metric": "ring-mults/s", "unit": "products/s", "value": value,
                     "ms_per_step": total_ms / args.steps,
                     "config": {"workload": wl["desc"], "pairs": pairs, "ring_degree": n,
                                "parallelism": f"replicas x{world}",
                                "l2": "flushed (256 MiB write) between timed steps", "host_and_device_agree": ok},
                     "e2e": {"value": world * args.steps * pairs / e2e_s, "unit": "products/s",
                             "h2d_bytes_per_step": 2 * len(a), "d2h_bytes_per_step": len(a)},
                     "gpu_launches": int(sum(s[0] for s in stats.values() if s)),
                     "roofline": roofline({k: v for k, v in stats.items() if k != "ring_mul"},
                                          "the timed steps (one launch at a time on the context stream, per-kernel "
                                          "CUDA events)", int_rates), "clocks": clk})
    elif wl["kind"] == "plain":
        file_bytes = wl["file_bytes"]
        nsteps = args.warmup + args.steps
        from damascus000_gb300 import synth
        files = [synth.random_file(MASTER_SEED, file_bytes, rank * 100_000 + i) for i in range(nsteps)]
        dev = [torch.frombuffer(bytearray(f), dtype=torch.uint8).cuda() for f, _ in files]
        pinned = [torch.frombuffer(bytearray(f), dtype=torch.uint8).pin_memory() for f, _ in files]
        torch.cuda.synchronize()
        cap = D.proof_size(file_bytes)
        out = ctypes.create_string_buffer(cap)
        for i in range(args.warmup):
            ctx.prove_device_timed(dev[i].data_ptr(), file_bytes, files[i][1], EPOCH, out)
        clocks = ClockSampler(local)
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        step_ms = []
        for i in range(args.warmup, nsteps):
            ctx.flush_l2()
            _, ms = ctx.prove_device_timed(dev[i].data_ptr(), file_bytes, files[i][1], EPOCH, out)
            step_ms.append(ms)
        torch.cuda.synchronize()
        clk = clocks.stop()
        # kernel breakdown: the same steps again with per-kernel CUDA events
        ctx.set_profiling(True)
        ctx.reset_stats()
        for i in range(args.warmup, nsteps):
            ctx.flush_l2()
            ctx.prove_device_timed(dev[i].data_ptr(), file_bytes, files[i][1], EPOCH, out)
        torch.cuda.synchronize()
        stats = {k: ctx.kernel_stat(k) for k in KERNELS}
        ctx.set_profiling(False)
        total_ms = max_over_ranks(sum(step_ms))
        value = world * args.steps * file_bytes / MIB / (total_ms / 1000.0)
        lib = D.load()
        n_out = ctypes.c_size_t()
        for i in range(args.warmup):  # the host path's staging buffers enter the pools here
            ctx.check(lib.damascus_prove(ctx.handle, ctypes.c_char_p(pinned[i].data_ptr()), file_bytes,
                                         files[i][1], EPOCH, out, cap, ctypes.byref(n_out)), "prove")
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        t0 = time.perf_counter()
        for i in range(args.warmup, nsteps):
            ctx.check(lib.damascus_prove(ctx.handle, ctypes.c_char_p(pinned[i].data_ptr()), file_bytes,
                                         files[i][1], EPOCH, out, cap, ctypes.byref(n_out)), "prove")
        ev1.record()
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(max(ev0.elapsed_time(ev1) / 1000.0, time.perf_counter() - t0))
        ok = ctx.verify(out.raw[:n_out.value], EPOCH)
        # the files the oracle's digests cover, proven again through the same path
        digests = workload_digests(wl["name"], rank)
        exact = None
        if digests:
            idx = [e["index"] for e in digests if e["index"] < nsteps]
            exact = check_digests(digests, [ctx.prove(files[i][0], files[i][1], EPOCH) for i in idx],
                                  [file_bytes] * len(idx), idx)
        line.update({"value": value, "ms_per_step": total_ms / args.steps,
                     "config": {"workload": wl["desc"], "file_bytes": file_bytes, "parallelism": f"replicas x{world}",
                                "l2": "flushed (256 MiB write) between timed steps", "verified": bool(ok),
                                "bit_exact_vs_oracle": f"{exact[0]}/{exact[1]} proofs of this workload's files equal "
                                                       "the CPU oracle's (SHA-256)" if exact else None},
                     "e2e": {"value": world * args.steps * file_bytes / MIB / e2e_s, "unit": UNIT,
                             "h2d_bytes_per_step": file_bytes, "d2h_bytes_per_step": n_out.value},
                     "gpu_launches": int(sum(s[0] for s in stats.values() if s)),
                     "roofline": roofline(stats, "the same K steps rerun with per-kernel CUDA events (one proof at a "
                                                 "time: launches serialised on the prover's stream)",
                                          int_rates),
                     "clocks": clk})
    elif wl["kind"] == "verify":
        files = workload_files(wl, rank)
        with D.Engine(ctx) as eng:
            proofs = eng.prove_batch([(d, s, EPOCH) for d, s, _ in files])
        nproofs = len(proofs)
        cpu_inputs = proofs
        svc = D.VerifyService(ctx, cache_bytes=wl["cache_bytes"])

        def one_pass(service):
            ts = [service.submit(p, EPOCH) for p in proofs]
            return [service.wait(t) for t in ts]

        for _ in range(args.warmup):
            res = one_pass(svc)
        if any(code for code, _ in res):
            raise SystemExit("the verifier service rejected an honest proof")
        st0 = svc.stats()
        clocks = ClockSampler(local)
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = one_pass(svc)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        st1 = svc.stats()
        accepted = sum(1 for code, _ in res if code == 0)
        step_s = max_over_ranks(wall) / args.steps
        value = world * nproofs / step_s

        # launches per pass: the same passes again with per-kernel CUDA events (their
        # durations overlap across the workers' streams, so they give counts only)
        ctx.set_profiling(True)
        ctx.reset_stats()
        for _ in range(args.steps):
            one_pass(svc)
        torch.cuda.synchronize()
        service_stats = {k: ctx.kernel_stat(k) for k in VERIFY_KERNELS}
        # per-kernel durations with each kernel alone on the GPU: the one-shot
        # verifier over the same proofs, L2 flushed before each
        ctx.reset_stats()
        for p in proofs:
            ctx.flush_l2()
            ctx.verify(p, EPOCH)
        torch.cuda.synchronize()
        alone_stats = {k: ctx.kernel_stat(k) for k in VERIFY_KERNELS}
        ctx.set_profiling(False)

        # real-time replay at the stream's arrival times for latency
        barrier()
        t0 = time.perf_counter()
        ts = []
        for p, (_, _, arr) in zip(proofs, files):
            delay = arr - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ts.append(svc.submit(p, EPOCH))
        lats = [svc.wait(t)[1] for t in ts]
        svc.close()

        # the service without the generator cache (every proof expands its g_0)
        with D.VerifyService(ctx, cache_bytes=0) as s0:
            one_pass(s0)
            barrier()
            t0 = time.perf_counter()
            one_pass(s0)
            nocache = world * nproofs / max_over_ranks(time.perf_counter() - t0)
        # the one-shot verifier, one proof at a time
        barrier()
        t0 = time.perf_counter()
        plain_ok = all(ctx.verify(p, EPOCH) for p in proofs)
        plain = world * nproofs / max_over_ranks(time.perf_counter() - t0)

        launches = int(sum(v[0] for v in service_stats.values() if v)) // args.steps
        rl = roofline({"fold_gen": alone_stats.get("fold_gen")},
                      "the one-shot verifier over the same proofs, each kernel alone on the GPU, L2 flushed "
                      "before each proof")
        if rl:
            rl["kernels_alone"] = {k: {"launches": v[0], "ms": round(v[1], 4), "algo_bytes": v[2]}
                                   for k, v in alone_stats.items() if v}
            rl["note"] = ("fold_gen is the only kernel of a service pass with a warm generator cache; the "
                          "expansion (gen_generators) runs once per shape")
        line.update({"metric": "proofs verified/s", "unit": "proofs/s", "value": value,
                     "ms_per_step": step_s * 1000.0,
                     "config": {"workload": wl["desc"], "proofs": nproofs,
                                "file_bytes": sum(len(d) for d, _, _ in files),
                                "proof_bytes": sum(map(len, proofs)), "parallelism": f"replicas x{world}",
                                "workers": "one per host core (at most 16)",
                                "l2": "families of the d 9-11 proofs (34-537 MB) exceed the 129 MB L2",
                                "accepted": accepted, "plain_path_accepts": bool(plain_ok),
                                "cache_hits_per_step": (st1["cache_hits"] - st0["cache_hits"]) / args.steps,
                                "cache_misses_per_step": (st1["cache_misses"] - st0["cache_misses"]) / args.steps},
                     "e2e": {"value": value, "unit": "proofs/s", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": nproofs * 128,
                             "note": "the timed value is already end to end: host proof bytes in, verdicts out "
                                     "through the C ABI; the device receives only scalars (challenges are kernel "
                                     "arguments) and returns each terminal generator (128 B)"},
                     "plain_per_s": plain, "service_vs_plain": value / plain,
                     "no_cache_per_s": nocache,
                     "latency_ms": {"p50_ms": percentile(lats, 0.5), "p99_ms": percentile(lats, 0.99),
                                    "max_ms": max(lats), "rate_per_s": wl["rate"], "requests": len(lats)},
                     "gpu_launches": launches,
                     "roofline": rl,
                     "clocks": clk})
    else:
        files = workload_files(wl, rank)
        total = sum(len(d) for d, _, _ in files)
        dev = [torch.frombuffer(bytearray(d), dtype=torch.uint8).cuda() for d, _, _ in files]
        pinned = [torch.frombuffer(bytearray(d), dtype=torch.uint8).pin_memory() for d, _, _ in files]
        torch.cuda.synchronize()
        eng = D.Engine(ctx, max_waves=args.waves)

        def replay_device():
            ts = [eng.submit_device(t.data_ptr(), len(d), s, EPOCH) for t, (d, s, _) in zip(dev, files)]
            return collect(eng, ts)

        # warm-up (also checks the engine against the plain path on a few files)
        for _ in range(args.warmup):
            res = replay_device()
        for i in range(0, len(files), max(1, len(files) // 6)):
            d, s, _ = files[i]
            if res[i][0] != ctx.prove(d, s, EPOCH):
                raise SystemExit(f"engine proof {i} differs from the plain path")
        # timed region: K replays without per-kernel events (they cost ~5 % throughput)
        st0 = eng.stats()
        clocks = ClockSampler(local)
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = replay_device()
        ev1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        st1 = eng.stats()
        step_s = max_over_ranks(max(ev0.elapsed_time(ev1) / 1000.0, wall)) / args.steps
        value = world * total / MIB / step_s
        # every proof of the last timed replay against the oracle's digests
        digests = workload_digests(wl["name"], rank)
        exact = check_digests(digests, [r[0] for r in res], [len(d) for d, _, _ in files]) if digests else None

        # kernel rates: one more replay with a single wave in flight, so the launches
        # run one after another on one stream and each kernel's CUDA events time it
        # alone (the timed replays overlap up to 16 waves)
        ctx.set_profiling(True)
        ctx.reset_stats()
        with D.Engine(ctx, max_waves=1) as eng1:
            # every request admitted before the first launch, so each wave carries one
            # stage of all the requests at it (the launches the kernels are rated on)
            eng1.set_admission_batch(0)
            t_serial = time.perf_counter()
            serial = [eng1.wait(t)[0] for t in
                      [eng1.submit_device(t.data_ptr(), len(d), s, EPOCH) for t, (d, s, _) in zip(dev, files)]]
            serial_s = time.perf_counter() - t_serial
        torch.cuda.synchronize()
        stats = {k: ctx.kernel_stat(k) for k in KERNELS}
        ctx.set_profiling(False)
        serial_same = sum(a == b[0] for a, b in zip(serial, res))

        # end to end from pinned host memory: the engine's host-to-device copies
        # read the caller's pinned buffers (submit_borrowed)
        lib = D.load()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d2h = 0
        for _ in range(args.steps):
            ts = [eng.submit_borrowed(p.data_ptr(), len(d), s, EPOCH) for p, (d, s, _) in zip(pinned, files)]
            outs = collect(eng, ts)
            d2h = sum(len(o[0]) for o in outs)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0) / args.steps
        # the same with the copying submission (each file copied into the engine's
        # staging buffer before submit returns), for comparison
        staged_steps = min(args.steps, 5)
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(staged_steps):
            ts = [eng.submit_ptr(p.data_ptr(), len(d), s, EPOCH) for p, (d, s, _) in zip(pinned, files)]
            staged = collect(eng, ts)
        torch.cuda.synchronize()
        staged_s = max_over_ranks(time.perf_counter() - t0) / staged_steps
        staged_same = sum(a[0] == b[0] for a, b in zip(staged, outs))
        verified = all(ctx.verify(o[0], EPOCH) for o in outs[:: max(1, len(outs) // 4)])
        e2e_exact = check_digests(digests, [o[0] for o in outs], [len(d) for d, _, _ in files]) if digests else None

        # plain one-request-at-a-time GPU path on the same files
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for t, (d, s, _) in zip(dev, files):
            ctx.prove_device(t.data_ptr(), len(d), s, EPOCH)
        torch.cuda.synchronize()
        plain_s = max_over_ranks(time.perf_counter() - t0)
        plain = world * total / MIB / plain_s

        lat = None
        if wl["kind"] == "serve":
            # real-time Poisson replay for latency
            barrier()
            t0 = time.perf_counter()
            ts = []
            for t, (d, s, arr) in zip(pinned, files):
                delay = arr - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ts.append(eng.submit_ptr(t.data_ptr(), len(d), s, EPOCH))
            lats = [eng.wait(t)[1] for t in ts]
            lat = {"p50_ms": percentile(lats, 0.5), "p99_ms": percentile(lats, 0.99), "max_ms": max(lats),
                   "rate_per_s": wl["rate"], "requests": len(lats),
                   "offered_mib_s": total / MIB / files[-1][2]}
        eng.close()
        if wl["name"] == "serve" and not args.no_batched:
            line["batched"] = measure_batched(ctx, D, torch, args, rank, world, ranks)
        line["host_blake3_gbs_per_core"] = host_hash_rate(D)
        line.update({"value": value, "ms_per_step": step_s * 1000.0,
                     "config": {"workload": wl["desc"], "requests": len(files), "total_bytes": total,
                                "parallelism": f"replicas x{world}", "hbm_budget_bytes": SERVE_BUDGET,
                                "l2": "working set (>= 1 GiB per step) exceeds the 129 MB L2",
                                "verified": bool(verified),
                                "bit_exact_vs_oracle": (f"{exact[0]}/{exact[1]} proofs of the last timed replay and "
                                                        f"{e2e_exact[0]}/{e2e_exact[1]} of the last e2e replay equal "
                                                        "the CPU oracle's (SHA-256, tests/golden/"
                                                        "workload_digests.json)") if exact else
                                "no oracle digests for this rank's files",
                                "proofs_exact": exact[0] if exact else None,
                                "proofs_checked": exact[1] if exact else None,
                                "waves_per_step": (st1["waves"] - st0["waves"]) / args.steps,
                                "launches_per_step": (st1["launches"] - st0["launches"]) / args.steps,
                                "gpu_idle_ms_per_step": (st1["gpu_idle_ms"] - st0["gpu_idle_ms"]) / args.steps,
                                "host_stage_ms_per_step": (st1["host_stage_ms"] - st0["host_stage_ms"]) / args.steps,
                                "scheduler_ms_per_step": {
                                    "admit": (st1["admit_ms"] - st0["admit_ms"]) / args.steps,
                                    "plan_and_launch": (st1["launch_ms"] - st0["launch_ms"]) / args.steps},
                                "generator_cache": ctx.generator_cache_stats() if wl.get("generator_cache") else None},
                     "e2e": {"value": world * total / MIB / e2e_s, "unit": UNIT, "h2d_bytes_per_step": total,
                             "d2h_bytes_per_step": d2h,
                             "submission": "files in the caller's pinned host buffers, read by the engine's "
                                           "host-to-device copies (damascus_engine_submit_borrowed); proofs copied "
                                           "out once each (damascus_engine_result)",
                             "staged_value": world * total / MIB / staged_s,
                             "staged_note": f"the copying submission (damascus_engine_submit: each file copied into "
                                            f"the engine's pinned staging first), {staged_steps} steps; "
                                            f"{staged_same}/{len(files)} proofs identical"},
                     "plain_mib_s": plain, "serving_vs_plain": value / plain,
                     "single_wave_replay": {"mib_s": total / MIB / serial_s,
                                            "kernel_ms": sum(v[1] for v in stats.values() if v),
                                            "note": "one stage wave in flight, per-kernel events on: the kernels "
                                                    "one after another, host stages not overlapped"},
                     "gpu_launches": int(st1["launches"] - st0["launches"]),
                     "roofline": roofline(stats, "one more replay of the workload with a single stage wave in "
                                                 "flight: launches serialised on one stream, per-kernel CUDA "
                                                 f"events ({serial_same}/{len(files)} proofs identical to the "
                                                 "timed replay's)", int_rates),
                     "clocks": clk})
        if lat:
            line["latency_ms"] = lat
    ranks.close()
    if rank != 0:
        return 0
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, proofs=cpu_inputs)
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="serve", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched set measured beside the serving "
                    "stream")
    ap.add_argument("--waves", type=int, default=0, help="engine stage waves in flight (0: library default)")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload], name=args.workload)
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
