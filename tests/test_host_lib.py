"""CPU tests of the shipped library: it loads, exports every symbol the C header
declares, and its host-side logic (field, BLAKE3, transcript, layout and bincode
sizes) matches the oracle.  No compute call needs a GPU here."""
import json
import random
import re
from pathlib import Path

import pytest

import damascus000_gb300 as D

ROOT = Path(__file__).resolve().parent.parent
Q = D.Q


def header_symbols():
    text = (ROOT / "include" / "damascus.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(damascus_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    lib = D.load()
    syms = header_symbols()
    assert len(syms) >= 50
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(D.EXPORTED_SYMBOLS) == syms


def test_field_matches_python(oracle_lib):
    rng = random.Random(1)
    for _ in range(5000):
        a, b = rng.randrange(Q), rng.randrange(Q)
        assert D.fp_mul(a, b) == a * b % Q
        assert D.fp_add(a, b) == (a + b) % Q
        assert D.fp_sub(a, b) == (a - b) % Q
    for a in [0, 1, Q - 1, 2 ** 111, 75]:
        for b in [0, 1, Q - 1, 2 ** 111]:
            assert D.fp_mul(a, b) == a * b % Q
            assert D.fp_sub(a, b) == (a - b) % Q
    assert D.fp_inv(9) * 9 % Q == 1
    assert D.fp_mul(2 ** 128 - 1, 1) == (2 ** 128 - 1) % Q  # deserialisation reduces mod q


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 32, 64, 100])
def test_from_le_bytes_mod_order(oracle_lib, n):
    b = bytes(random.Random(n).getrandbits(8) for _ in range(n))
    assert D.fp_from_le_bytes_mod_order(b) == oracle_lib.fp_from_le_bytes_mod_order(b) == \
        int.from_bytes(b, "little") % Q


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 1023, 1024, 1025, 2048, 3073, 4096, 4097, 5 * 1024, 8 * 1024 - 1,
                               8 * 1024, 9 * 1024 + 3, 16385, 33 * 1024, 70000, 1 << 20, (1 << 20) + 4 * 1024 + 1])
def test_host_blake3_matches_oracle(oracle_lib, n):
    """Lengths around the host hash's lane groups (four whole chunks at a time),
    its parent levels in lanes (four pairs at a time) and the parallel split."""
    data = bytes((i * 131 + n) & 0xFF for i in range(n))
    key = bytes(range(32))
    assert D.blake3(data) == oracle_lib.blake3(data)
    assert D.blake3_keyed(key, data) == oracle_lib.blake3_keyed(key, data)


@pytest.mark.parametrize("n", [1, 2, 64, 512])
def test_transcript_challenge_matches_oracle(oracle_lib, n):
    rng = random.Random(n)
    ep, fid = bytes([11]) * 32, bytes(range(32))
    c, l, r = (D.fe_vec(rng.randrange(Q) for _ in range(8 * n)) for _ in range(3))
    for label in ("vec", "poly"):
        assert D.transcript_challenge(ep, fid, label, 5, c, n, l, n, r, n) == \
            oracle_lib.challenge(ep, fid, label.encode(), 5, c, n, l, n, r, n)
    # mixed ring lengths (zero cross terms of a scalar stage)
    z = bytes(16 * 8)
    assert D.transcript_challenge(ep, fid, "poly", 0, c, n, z, 1, z, 1) == \
        oracle_lib.challenge(ep, fid, b"poly", 0, c, n, z, 1, z, 1)


@pytest.mark.parametrize("nbytes", [0, 1, 13, 14, 53_248, 1 << 20, 16 << 20, 128 << 20])
def test_layout_and_sizes(oracle_lib, nbytes):
    d, dim = D.layout_for_byte_len(nbytes)
    assert (d, dim) == oracle_lib.layout_for_byte_len(nbytes)
    assert D.coeff_count_for_byte_len(nbytes) == oracle_lib.lib().orc_coeff_count_for_byte_len(nbytes)
    assert D.proof_size(nbytes) == oracle_lib.proof_size_for_depth(d)


def test_record_and_statement_sizes(oracle_lib):
    assert D.record_size(64, 32) == 24_872 == oracle_lib.lib().orc_record_size(64, 32)
    assert D.statement_size(64) == 32 + 8 + 8 + 8 + 8 * (8 + 16 * 64) + 32
    assert D.depth_j(11, 3) == (256, 256)


def test_footprint_scales_with_depth():
    f9, f11 = D.prover_footprint(1 << 20), D.prover_footprint(16 << 20)
    assert 100 << 20 < f9 < 200 << 20
    assert 1 << 30 < f11 < 3 << 30


def test_context_without_gpu_fails_loudly():
    """No CPU fallback: on a machine without a usable GB300 the context refuses."""
    try:
        ctx = D.Context(0)
    except D.DamascusError as e:
        assert e.code in (D.ECUDA, D.EUNSUPPORTED, D.EINVAL)
        return
    ctx.close()
    pytest.skip("a GPU is present; the no-GPU failure path is not reachable here")


def test_parallel_hashing_from_many_threads(oracle_lib):
    """The host hashing pool is shared by every prover and engine worker: many
    concurrent large hashes must all complete with the right digest."""
    import threading
    data = [bytes((i * 7 + k) & 0xFF for i in range(300_000 + 1024 * k)) for k in range(4)]
    want = [oracle_lib.blake3(d) for d in data]
    errors = []

    def run(k):
        for it in range(60):
            j = (k + it) % 4
            if D.blake3(data[j]) != want[j]:
                errors.append((k, it))

    threads = [threading.Thread(target=run, args=(k,)) for k in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors


def test_autotune_table_apply_and_candidates():
    """The autotuner's table round trip on a stand-in context (no GPU): every entry
    is set through tuning_set with the knob ids of include/damascus.h."""
    from damascus000_gb300 import autotune as A

    class FakeCtx:
        def __init__(self):
            self.calls = []

        def tuning_set(self, knob, L, v):
            self.calls.append((knob, L, v))

    table = {"entries": [{"knob": "ntt_group", "log_ring": 6, "value": 32},
                         {"knob": "mac_triple", "log_ring": 11, "value": 12},
                         {"knob": "mac_split", "log_ring": 9, "value": 4},
                         {"knob": "mac_plain", "log_ring": 5, "value": 2}]}
    c = FakeCtx()
    assert A.apply(c, table=table) == 4
    assert c.calls == [(0, 6, 32), (1, 11, 12), (2, 9, 4), (3, 5, 2)]
    assert set(A.CANDIDATES[A.NTT_GROUP]) == {32, 64}
    assert all(1 <= v <= 32 for k in (A.MAC_TRIPLE, A.MAC_SPLIT, A.MAC_PLAIN) for v in A.CANDIDATES[k])
    assert A.work_size(A.NTT_GROUP, 9) == 9 * 512 and A.work_size(A.MAC_TRIPLE, 11) == 1024
    if A.DEFAULT_TABLE.exists():  # the packaged table only names valid knobs and values
        t = json.loads(A.DEFAULT_TABLE.read_text())
        c = FakeCtx()
        assert A.apply(c, table=t) == len(t["entries"]) > 0
        for knob, L, v in c.calls:
            assert 0 <= L <= 13 and (v in (32, 64) if knob == 0 else 1 <= v <= 32)
