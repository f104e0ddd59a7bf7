"""Bit-exact parity of the benchmark workloads at their full sizes.

The CPU oracle's proofs of these files take seconds (d = 9) to minutes (d = 11)
each, so tests/golden/make_workload_digests.py ran it once and committed the
SHA-256 of every proof (bincode((Statement, Vec<RoundRecord>, Fp))) and of its
statement.  Each test regenerates the same seeded files and compares the GPU
path's proofs with those digests:

* d = 9: 1 MiB files, 512 x 512 witness (plain path);
* d = 11: a 16 MiB file, 2048 x 2048 witness (plain path);
* the 64-file batched set, d 6-10, through the engine in one batch;
* the 96-request serving stream, d 6-11, through the engine, with per-file
  seeds and under one system seed with the provers' generator cache;
* d = 12 and d = 13: the statement (com_0), the round-0 record and the
  commitment after round 0 of a 58.7 MB and a 218 MB file, rings of 2^12 and
  2^13: the GPU path sums each commitment coordinate in the NTT domain over nine
  28-bit primes and reconstructs it once, where the reference reconstructs
  every product separately (src/algebra/ntt.rs:372-427).
"""
import hashlib
import json
from pathlib import Path

import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu
DIGESTS = json.loads((Path(__file__).resolve().parent / "golden" / "workload_digests.json").read_text())
MASTER = DIGESTS["master_seed"]
EPOCH = bytes.fromhex(DIGESTS["epoch_seed"])
SYSTEM_SEED = bytes.fromhex(DIGESTS["system_seed"])


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def check(entries, proofs, files):
    assert len(entries) == len(proofs) == len(files)
    bad = []
    for e, p, (data, seed) in zip(entries, proofs, files):
        assert e["file_len"] == len(data) and e["seed_generators"] == seed.hex()
        if sha(p) != e["proof_sha256"]:
            part = "statement" if sha(p[:_stmt_len(e)]) != e["statement_sha256"] else "rounds"
            bad.append((e["index"], e["depth"], part))
    assert not bad, f"proofs differing from the oracle (index, depth, first differing part): {bad}"


def _stmt_len(e):
    n = 1 << e["depth"]
    return 32 + 8 + 8 + 72 + 128 * n + 32


def test_d9_plain_proofs_match_oracle(ctx):
    files = [synth.random_file(MASTER, 1 << 20, e["index"]) for e in DIGESTS["d9"]]
    check(DIGESTS["d9"], [ctx.prove(d, s, EPOCH) for d, s in files], files)


def test_d11_plain_proof_matches_oracle(ctx):
    files = [synth.random_file(MASTER, 16 << 20, e["index"]) for e in DIGESTS["d11"]]
    check(DIGESTS["d11"], [ctx.prove(d, s, EPOCH) for d, s in files], files)


def test_batched_set_matches_oracle(ctx):
    files = [(d, s) for d, s, _ in synth.batched_files(MASTER, 64, 50_000, 4 << 20)]
    with D.Engine(ctx) as eng:
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
    check(DIGESTS["batched"], proofs, files)


def test_serving_stream_matches_oracle(ctx):
    files = [(d, s) for d, s, _ in synth.serving_files(MASTER, 96, 200.0)]
    with D.Engine(ctx) as eng:
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
    check(DIGESTS["serving"], proofs, files)
    # the plain one-at-a-time path on the deepest files as well
    deep = [i for i, e in enumerate(DIGESTS["serving"]) if e["depth"] == 11][:2]
    check([DIGESTS["serving"][i] for i in deep], [ctx.prove(*files[i], EPOCH) for i in deep],
          [files[i] for i in deep])


def test_serving_stream_system_seed_with_generator_cache_matches_oracle():
    files = [(d, s) for d, s, _ in synth.serving_files(MASTER, 96, 200.0, SYSTEM_SEED)]
    c = D.Context(0)
    try:
        c.set_generator_cache(16 << 30)
        with D.Engine(c) as eng:
            first = eng.prove_batch([(d, s, EPOCH) for d, s in files])
            second = eng.prove_batch([(d, s, EPOCH) for d, s in files])  # every shape cached by now
        st = c.generator_cache_stats()
    finally:
        c.close()
    assert st["fills"] >= 1 and st["hits"] >= len(files)
    check(DIGESTS["serving_system_seed"], first, files)
    check(DIGESTS["serving_system_seed"], second, files)


@pytest.mark.parametrize("depth", [12, 13])
def test_deep_statement_and_round0_match_oracle(ctx, depth):
    """d = 12 (58.7 MB, rings of 2^12) and d = 13 (218 MB, rings of 2^13, the
    deepest supported: its 2 GiB expansion needs the limit raised)."""
    e = DIGESTS[f"d{depth}"]
    data, seed = synth.random_file(e["master_seed"], e["length"], e["index"])
    assert D.layout_for_byte_len(len(data))[0] == depth and seed.hex() == e["seed_generators"]
    p = D.DamascusProver(ctx, data, seed, EPOCH, max_preprocess_bytes=4 << 30)
    try:
        stmt = p.statement()
        assert len(stmt) == e["statement_len"] and sha(stmt) == e["statement_sha256"]
        rec = p.fold_round(0)
        assert len(rec) == e["round0_record_len"] and sha(rec) == e["round0_record_sha256"]
        assert list(p.current_dimensions()) == e["dims_after_round0"]
        assert sha(p.current_commitment()) == e["commitment_after_round0_sha256"]
    finally:
        p.close()
