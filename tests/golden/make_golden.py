"""Regenerates the golden fixtures in tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

Inputs come from the seeded ChaCha20 workload generator; outputs are the
oracle's.  The fixtures pin the GPU path (and any later change of the oracle)
to fixed byte strings: a full d=6 proof of the 53,248-byte workload, ring
products, generator coefficients and BLAKE3 file ids.
"""
import hashlib
import json
import random
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from damascus000_gb300 import synth  # noqa: E402

MASTER_SEED = 20260101
EPOCH = bytes([11]) * 32


def main():
    O.build()
    out = {"master_seed": MASTER_SEED, "epoch_seed": EPOCH.hex()}
    # d=6 full flow: 53,248 random bytes (4,096 coefficients, 64 x 64 witness).
    data, seed = synth.random_file(MASTER_SEED, 53_248, 0)
    proof = O.prove(data, seed, EPOCH)
    (HERE / "d6_proof.bin").write_bytes(proof)
    out["d6"] = {"file_len": len(data), "file_index": 0, "seed_generators": seed.hex(),
                 "proof_sha256": hashlib.sha256(proof).hexdigest(), "proof_len": len(proof),
                 "file_id": O.blake3(data).hex(), "opening": proof[-16:].hex()}
    # d=7 pattern file from the reference's tests (prover.rs:473-487 helpers).
    d7 = bytes(((i & 0xFF) * 17 + 9) & 0xFF for i in range(((1 << 12) + 1) * 13))
    p7 = O.prove(d7, bytes([7]) * 32, EPOCH)
    out["d7_pattern"] = {"file_len": len(d7), "tweak": 9, "proof_sha256": hashlib.sha256(p7).hexdigest(),
                         "proof_len": len(p7)}
    # ring products
    rng = random.Random(MASTER_SEED)
    rm = []
    for n in [1, 2, 64, 512]:
        a = [rng.randrange(O.Q) for _ in range(n)]
        b = [rng.randrange(O.Q) for _ in range(n)]
        rm.append({"n": n, "a": O.fe_vec(a).hex(), "b": O.fe_vec(b).hex(),
                   "out": O.fe_vec(O.negacyclic_multiply(a, b)).hex()})
    out["ring_mul"] = rm
    # generators
    g_seed = O.derive_subseed(bytes([7]) * 32, b"g0")
    g = O.derive_generators(g_seed, 2, 64)
    out["generators"] = {"g_seed": g_seed.hex(), "vector_len": 2, "ring_len": 64,
                         "sha256": hashlib.sha256(g).hexdigest(), "first": g[:64].hex()}
    # file ids
    fids = []
    for n in [0, 1, 1023, 1024, 1025, 4096, 100_000]:
        d, _ = synth.random_file(MASTER_SEED, n, 100 + n)
        fids.append({"len": n, "index": 100 + n, "blake3": O.blake3(d).hex()})
    out["file_ids"] = fids
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "golden.json", HERE / "d6_proof.bin")


if __name__ == "__main__":
    main()
