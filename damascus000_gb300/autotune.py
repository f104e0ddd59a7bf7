"""Autotuner of the kernels' launch shapes.

Measures, on the GPU at hand, each knob of `damascus_tuning_*` (include/damascus.h)
over its candidate values for every ring size the prover launches, with the
work sizes a proof of that depth gives the kernel, keeps the fastest value, and
writes a table that `apply()` loads into a context:

* `NTT_GROUP`  — threads per block of the forward transform for rings below 2^10
  (32 or 64: how many small polynomials share a block);
* `MAC_TRIPLE`, `MAC_SPLIT`, `MAC_PLAIN` — the resident blocks per SM that a
  multiply-accumulate's column split fills (its part count; more parts mean more
  blocks in flight but more partial sums for the finish to add).

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

NTT_GROUP, MAC_TRIPLE, MAC_SPLIT, MAC_PLAIN = 0, 1, 2, 3
KNOB_NAMES = {NTT_GROUP: "ntt_group", MAC_TRIPLE: "mac_triple", MAC_SPLIT: "mac_split", MAC_PLAIN: "mac_plain"}
CANDIDATES = {
    NTT_GROUP: [32, 64],
    MAC_TRIPLE: [2, 4, 8, 12, 16, 24],
    MAC_SPLIT: [2, 4, 8, 12, 16, 24],
    MAC_PLAIN: [2, 4, 8, 16],
}
DEFAULT_TABLE = Path(__file__).resolve().parent / "tuning_gb300.json"


def work_size(knob: int, L: int) -> int:
    """The kernel's work at ring 2^L in a proof of depth L (its commitment stage):
    witness + generator polynomials for the transform, column pairs for the triple
    MAC, columns for the split and single-sum MACs."""
    n = 1 << L
    if knob == NTT_GROUP:
        return 9 * n
    if knob == MAC_TRIPLE:
        return max(1, n // 2)
    return n


def ring_sizes(knob: int) -> List[int]:
    if knob == NTT_GROUP:
        return list(range(4, 10))  # larger rings fill their blocks either way
    return list(range(4, 13))


DEFAULTS = {NTT_GROUP: 64, MAC_TRIPLE: 8, MAC_SPLIT: 8, MAC_PLAIN: 8}  # the library's built-in values


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
        for L in ring_sizes(knob):
            if L > max_L:
                continue
            count = work_size(knob, L)
            times = {}
            for v in CANDIDATES[knob]:
                times[v] = ctx.tuning_measure(knob, L, v, count, reps)
            best = choose(times, DEFAULTS[knob], margin)
            ctx.tuning_set(knob, L, best)
            entries.append({"knob": KNOB_NAMES[knob], "log_ring": L, "value": best, "count": count,
                            "ms": {str(k): round(t, 5) for k, t in times.items()}})
            log(f"{KNOB_NAMES[knob]:10s} L={L:2d} count={count:6d} best={best:3d} "
                + " ".join(f"{k}:{t:.4f}" for k, t in times.items()))
    return {"device": "GB300", "generated": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "reps": reps,
            "margin": margin, "min_gain_ms": 0.001, "entries": entries}


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
        ctx.tuning_set(names[e["knob"]], int(e["log_ring"]), int(e["value"]))
        n += 1
    return n


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=str(DEFAULT_TABLE))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--max-L", type=int, default=12)
    args = ap.parse_args()
    import damascus000_gb300 as D
    ctx = D.Context(0)
    table = tune(ctx, reps=args.reps, max_L=args.max_L)
    Path(args.out).write_text(json.dumps(table, indent=1) + "\n")
    print(f"wrote {args.out} ({len(table['entries'])} entries)")


if __name__ == "__main__":
    main()
