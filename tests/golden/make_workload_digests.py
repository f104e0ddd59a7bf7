"""Writes tests/golden/workload_digests.json: the oracle's proof digests for the
benchmark workloads, so that the GPU tests and bench.py can check every proof
of those workloads bit-exact without running the oracle (minutes per 16 MiB
file) at test time.

    python tests/golden/make_workload_digests.py [--sets d9,batched,...]

Sets (files from damascus000_gb300.synth, master seed 0xDA3A5C05 as bench.py):
  d9       1 MiB files 0 and 1 of the plain d = 9 workload (512 x 512 witness)
  d11      16 MiB file 0 of the plain d = 11 workload (2048 x 2048 witness)
  batched  the 64-file batched set (log-uniform 50 KB - 4 MiB, d 6-10)
  serving  the 96-request serving stream (d 6-11), per-file seeds
  serving_system_seed  the same 96 files under the default system seed
  d12      the statement (com_0) and round-0 record of a 58.7 MB file (d = 12,
           4096 x 4096 witness, rings of 2^12): the nine-prime CRT range of the
           GPU path against the reference's per-product CRT
  d13      the same for a 218 MB file (d = 13, 8192 x 8192 witness, rings of
           2^13, the deepest the library proves; 30 min of the oracle on 8 cores)

Resumable: entries already in the JSON with the same file length are kept.
Every entry records the SHA-256 of the whole proof
(bincode((Statement, Vec<RoundRecord>, Fp))) and of its statement prefix.
"""
import argparse
import hashlib
import json
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from damascus000_gb300 import synth  # noqa: E402

OUT = HERE / "workload_digests.json"
MASTER_SEED = 0xDA3A5C05
EPOCH = bytes([11]) * 32
SYSTEM_SEED = bytes([7]) * 32
D12_FILE = dict(master_seed=12, length=2048 * 2048 * 13 + 4096 * 1024, index=0)
D13_FILE = dict(master_seed=13, length=4096 * 4096 * 13 + 1, index=0)


def statement_len(vector_len: int, ring_len: int) -> int:
    # Statement = [u8;32] file_id + u64 + u64 + ModuleElement (72 + 128 n) + [u8;32]
    return 32 + 8 + 8 + 72 + 128 * ring_len + 32


def entry(data: bytes, seed: bytes, threads: int, **extra):
    t0 = time.time()
    proof = O.prove(data, seed, EPOCH, use_ntt=True, threads=threads)
    d, dim = O.layout_for_byte_len(len(data))
    sl = statement_len(dim, dim)
    return dict(extra, file_len=len(data), depth=d, seed_generators=seed.hex(), proof_len=len(proof),
                proof_sha256=hashlib.sha256(proof).hexdigest(),
                statement_sha256=hashlib.sha256(proof[:sl]).hexdigest(),
                opening=proof[-16:].hex(), oracle_s=round(time.time() - t0, 1))


def file_set(name: str):
    """[((file bytes, seed_generators), extra fields)] of one set."""
    if name == "d9":
        return [(synth.random_file(MASTER_SEED, 1 << 20, i), {"index": i}) for i in range(2)]
    if name == "d11":
        return [(synth.random_file(MASTER_SEED, 16 << 20, 0), {"index": 0})]
    if name == "batched":
        files = synth.batched_files(MASTER_SEED, 64, 50_000, 4 << 20)
    elif name == "serving":
        files = synth.serving_files(MASTER_SEED, 96, 200.0)
    elif name == "serving_system_seed":
        files = synth.serving_files(MASTER_SEED, 96, 200.0, SYSTEM_SEED)
    else:
        raise ValueError(name)
    return [((d, s), {"index": i}) for i, (d, s, _) in enumerate(files)]


def deep_entry(spec, depth: int, threads: int):
    """Statement, round-0 record and the commitment after round 0 of one deep file."""
    data, seed = synth.random_file(spec["master_seed"], spec["length"], spec["index"])
    t0 = time.time()
    p = O.Prover(data, seed, EPOCH, max_preprocess=1 << 40, use_ntt=True, threads=threads)
    stmt = p.statement()
    rec0 = p.fold_round(0)
    com1 = p.current_commitment()
    N, n = p.dims()
    return dict(spec, depth=depth, seed_generators=seed.hex(),
                statement_sha256=hashlib.sha256(stmt).hexdigest(), statement_len=len(stmt),
                round0_record_sha256=hashlib.sha256(rec0).hexdigest(), round0_record_len=len(rec0),
                commitment_after_round0_sha256=hashlib.sha256(com1).hexdigest(), dims_after_round0=[N, n],
                oracle_s=round(time.time() - t0, 1))


def save(out):
    tmp = OUT.with_suffix(".json.tmp")
    tmp.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    os.replace(tmp, OUT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sets", default="d9,batched,d11,d12,serving,serving_system_seed")
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    threads = args.threads or os.cpu_count() or 1
    O.build()
    out = json.loads(OUT.read_text()) if OUT.exists() else {}
    out.update({"master_seed": MASTER_SEED, "epoch_seed": EPOCH.hex(), "system_seed": SYSTEM_SEED.hex(),
                "generator": "tests/golden/make_workload_digests.py (CPU oracle, oracle/damascus_oracle.c)"})
    for name in args.sets.split(","):
        if name in ("d12", "d13"):
            if name not in out:
                out[name] = deep_entry(D12_FILE if name == "d12" else D13_FILE, int(name[1:]), threads)
                save(out)
                print(name, out[name]["oracle_s"], "s", flush=True)
            continue
        have = out.setdefault(name, [])
        for k, ((data, seed), extra) in enumerate(file_set(name)):
            if k < len(have) and have[k].get("file_len") == len(data):
                continue
            e = entry(data, seed, threads, **extra)
            if k < len(have):
                have[k] = e
            else:
                have.append(e)
            save(out)
            print(name, k, e["depth"], e["file_len"], e["oracle_s"], "s", flush=True)
    save(out)


if __name__ == "__main__":
    main()
