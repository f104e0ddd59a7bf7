"""Autotuner of the kernels' launch shapes.

Measures, on the GPU at hand, each knob of `damascus_tuning_*` (include/damascus.h)
over its candidate values for every ring size the prover launches, with the
work sizes a proof of that depth gives the kernel, keeps the fastest value, and
writes a table that `apply()` loads into a context:

* `NTT_GROUP`  — threads per block of the forward transform for rings below 2^10
  (32 or 64: how many small polynomials share a block);
* `NTT_RADIX` — residues per thread of the forward transform for rings of 2^5 and
  up (16 or 32: radix-16 or radix-32 register passes; radix 32 needs one
  shared-memory exchange fewer at 2^9 and 2^10 but holds twice the registers).
  It is tuned jointly with `NTT_GROUP`;
* `MAC_TRIPLE`, `MAC_SPLIT`, `MAC_PLAIN` — the resident blocks per SM that a
  multiply-accumulate's column split fills (its part count; more parts mean more
  blocks in flight but more partial sums for the finish to add);
* `SPLIT_COORDS` — commitment coordinates per thread of the split MAC (1, 2, 4
  or 8: each witness slot pair loaded once for that many generator rows, at the
  cost of registers).  It is tuned jointly with `MAC_SPLIT`: every pair is timed;
* `TRIPLE_COORDS` — the same for the triple MAC (1, 2 or 4), tuned jointly with
  `MAC_TRIPLE`;
* `engine_waves` — stage waves the serving engine keeps in flight (one stream
  each), timed end to end on a replay of a serving-stream mix; `Engine(ctx)`
  takes it when no count is given.

Results never depend on the table; only launch shapes do.  The table committed
beside this file (`tuning_gb300.json`) came from `python -m damascus000_gb300.autotune`
on a GB300.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path
from typing import Dict, List, Optional

NTT_GROUP, MAC_TRIPLE, MAC_SPLIT, MAC_PLAIN, SPLIT_COORDS, TRIPLE_COORDS, NTT_RADIX = 0, 1, 2, 3, 4, 5, 6
KNOB_NAMES = {NTT_GROUP: "ntt_group", MAC_TRIPLE: "mac_triple", MAC_SPLIT: "mac_split", MAC_PLAIN: "mac_plain",
              SPLIT_COORDS: "split_coords", TRIPLE_COORDS: "triple_coords", NTT_RADIX: "ntt_radix"}
CANDIDATES = {
    NTT_GROUP: [32, 64],
    MAC_TRIPLE: [2, 4, 8, 12, 16, 24],
    MAC_SPLIT: [2, 4, 8, 12, 16, 24],
    MAC_PLAIN: [2, 4, 8, 16],
    SPLIT_COORDS: [1, 2, 4, 8],
    TRIPLE_COORDS: [1, 2, 4],
    NTT_RADIX: [16, 32],
}
DEFAULT_TABLE = Path(__file__).resolve().parent / "tuning_gb300.json"


def work_size(knob: int, L: int) -> int:
    """The kernel's work at ring 2^L in a proof of depth L (its commitment stage):
    witness + generator polynomials for the transform, column pairs for the triple
    MAC, columns for the split and single-sum MACs."""
    n = 1 << L
    if knob in (NTT_GROUP, NTT_RADIX):
        return 9 * n
    if knob == MAC_TRIPLE:
        return max(1, n // 2)
    return n


def ring_sizes(knob: int) -> List[int]:
    if knob == NTT_GROUP:
        return list(range(4, 10))  # larger rings fill their blocks either way
    if knob == NTT_RADIX:
        return list(range(5, 14))
    return list(range(4, 13))


# the library's built-in values (the split's coordinates per thread: 8 from rings of 2^9 on); the autotuner
# reads them from a context made without a table
DEFAULTS = {NTT_GROUP: 64, MAC_TRIPLE: 8, MAC_SPLIT: 8, MAC_PLAIN: 8, SPLIT_COORDS: 1, TRIPLE_COORDS: 1,
            NTT_RADIX: 16}
ENGINE_WAVES = "engine_waves"
WAVE_CANDIDATES = [4, 8, 12, 16, 24, 32]
DEFAULT_WAVES = 16


def choose(times: Dict[int, float], default: int, margin: float = 0.03, min_gain_ms: float = 0.001) -> int:
    """The fastest candidate, but the built-in value unless the fastest beats it by
    more than `margin` and by more than `min_gain_ms` (shapes at the launch-latency
    floor, a few microseconds, time within noise of each other)."""
    best = min(times, key=times.get)
    if default in times and (times[best] > (1.0 - margin) * times[default] or
                             times[default] - times[best] < min_gain_ms):
        return default
    return best


def tune(ctx, knobs: Optional[List[int]] = None, reps: int = 5, max_L: int = 12, margin: float = 0.03,
         log=print) -> Dict:
    """Measures every candidate and sets the chosen value on `ctx`; returns the table."""
    entries = []
    for knob in knobs if knobs is not None else list(CANDIDATES):
        if knob in (SPLIT_COORDS, TRIPLE_COORDS, NTT_GROUP):
            continue  # tuned with MAC_SPLIT / MAC_TRIPLE / NTT_RADIX
        for L in ring_sizes(knob):
            if L > max_L:
                continue
            count = work_size(knob, L)
            if knob in (MAC_SPLIT, MAC_TRIPLE):
                entries += tune_coords(ctx, knob, L, count, reps, margin, log)
                continue
            if knob == NTT_RADIX:
                entries += tune_transform(ctx, L, count, reps, margin, log)
                continue
            default = ctx.tuning_get(knob, L)  # the library's built-in value
            times = {}
            for v in CANDIDATES[knob]:
                times[v] = ctx.tuning_measure(knob, L, v, count, reps)
            best = choose(times, default, margin)
            ctx.tuning_set(knob, L, best)
            entries.append({"knob": KNOB_NAMES[knob], "log_ring": L, "value": best, "count": count,
                            "ms": {str(k): round(t, 5) for k, t in times.items()}})
            log(f"{KNOB_NAMES[knob]:10s} L={L:2d} count={count:6d} best={best:3d} "
                + " ".join(f"{k}:{t:.4f}" for k, t in times.items()))
    return {"device": "GB300", "generated": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "reps": reps,
            "margin": margin, "min_gain_ms": 0.001, "entries": entries}


def tune_transform(ctx, L: int, count: int, reps: int, margin: float, log=print) -> List[Dict]:
    """The forward transform's (residues per thread, threads per block) pair at
    ring 2^L; the block size is a choice below 2^10 only."""
    groups = CANDIDATES[NTT_GROUP] if L < 10 else [ctx.tuning_get(NTT_GROUP, L)]
    default = (ctx.tuning_get(NTT_RADIX, L), ctx.tuning_get(NTT_GROUP, L))
    times = {}
    for g in groups:
        ctx.tuning_set(NTT_GROUP, L, g)
        for e in CANDIDATES[NTT_RADIX]:
            times[(e, g)] = ctx.tuning_measure(NTT_RADIX, L, e, count, reps)
    e, g = choose(times, default, margin)
    ctx.tuning_set(NTT_RADIX, L, e)
    ctx.tuning_set(NTT_GROUP, L, g)
    ms = {f"{a}x{b}": round(t, 5) for (a, b), t in times.items()}
    log(f"ntt        L={L:2d} count={count:6d} best={e}x{g} " + " ".join(f"{k}:{t:.4f}" for k, t in ms.items()))
    out = [{"knob": KNOB_NAMES[NTT_RADIX], "log_ring": L, "value": e, "count": count, "ms": ms}]
    if L < 10:
        out.append({"knob": KNOB_NAMES[NTT_GROUP], "log_ring": L, "value": g, "count": count})
    return out


def tune_coords(ctx, knob: int, L: int, count: int, reps: int, margin: float, log=print) -> List[Dict]:
    """A MAC's (coordinates per thread, blocks per SM) pair at ring 2^L (knob is
    MAC_SPLIT or MAC_TRIPLE): every pair timed, the built-in pair kept unless
    beaten as `choose` requires."""
    coords = SPLIT_COORDS if knob == MAC_SPLIT else TRIPLE_COORDS
    default = (ctx.tuning_get(coords, L), ctx.tuning_get(knob, L))  # the library's built-in pair
    times = {}
    for kc in CANDIDATES[coords]:
        ctx.tuning_set(coords, L, kc)
        for v in CANDIDATES[knob]:
            times[(kc, v)] = ctx.tuning_measure(knob, L, v, count, reps)
    kc, v = choose(times, default, margin)
    ctx.tuning_set(coords, L, kc)
    ctx.tuning_set(knob, L, v)
    ms = {f"{a}x{b}": round(t, 5) for (a, b), t in times.items()}
    log(f"{KNOB_NAMES[knob]:10s} L={L:2d} count={count:6d} best={kc}x{v} "
        + " ".join(f"{k}:{t:.4f}" for k, t in ms.items()))
    return [{"knob": KNOB_NAMES[knob], "log_ring": L, "value": v, "count": count, "ms": ms},
            {"knob": KNOB_NAMES[coords], "log_ring": L, "value": kc, "count": count}]


def tune_waves(ctx, requests: int = 48, reps: int = 3, margin: float = 0.03, log=print) -> Dict:
    """Stage waves in flight of the serving engine: end-to-end MiB/s of `reps`
    replays (after one warm-up) of a serving-stream mix of `requests` files
    (host buffers, copies included), per candidate."""
    import damascus000_gb300 as D
    from damascus000_gb300 import synth
    files = synth.serving_files(0x7E57, requests, 200.0)
    total = sum(len(d) for d, _, _ in files)
    epoch = D.DEFAULT_EPOCH_SEED
    rates = {}
    for w in WAVE_CANDIDATES:
        with D.Engine(ctx, max_waves=w) as eng:
            eng.prove_batch([(d, s, epoch) for d, s, _ in files])
            t0 = time.perf_counter()
            for _ in range(reps):
                eng.prove_batch([(d, s, epoch) for d, s, _ in files])
            rates[w] = reps * total / (1 << 20) / (time.perf_counter() - t0)
    best = max(rates, key=rates.get)
    if rates[best] < (1.0 + margin) * rates[DEFAULT_WAVES]:
        best = DEFAULT_WAVES
    ctx.engine_waves = best
    log(f"engine_waves best={best} " + " ".join(f"{w}:{r:.0f}MiB/s" for w, r in rates.items()))
    return {"knob": ENGINE_WAVES, "value": best, "requests": requests, "total_bytes": total,
            "mib_s": {str(w): round(r, 1) for w, r in rates.items()}}


def apply(ctx, table: Optional[Dict] = None, path: Optional[Path] = None) -> int:
    """Sets a table's values on `ctx` (the packaged GB300 table by default); returns how many."""
    if table is None:
        p = Path(path) if path else DEFAULT_TABLE
        if not p.exists():
            return 0
        table = json.loads(p.read_text())
    names = {v: k for k, v in KNOB_NAMES.items()}
    n = 0
    for e in table.get("entries", []):
        if e["knob"] == ENGINE_WAVES:
            ctx.engine_waves = int(e["value"])
        else:
            ctx.tuning_set(names[e["knob"]], int(e["log_ring"]), int(e["value"]))
        n += 1
    return n


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=str(DEFAULT_TABLE))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--max-L", type=int, default=12)
    ap.add_argument("--no-waves", action="store_true", help="skip the engine's waves-in-flight sweep")
    args = ap.parse_args()
    import damascus000_gb300 as D
    ctx = D.Context(0, tuning=None)
    table = tune(ctx, reps=args.reps, max_L=args.max_L)
    if not args.no_waves:
        table["entries"].append(tune_waves(ctx))
    Path(args.out).write_text(json.dumps(table, indent=1) + "\n")
    print(f"wrote {args.out} ({len(table['entries'])} entries)")


if __name__ == "__main__":
    main()
