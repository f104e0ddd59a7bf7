"""GPU parity: every kernel-level and protocol-level output of the sm_103a
library against the CPU oracle, bit-exact (integer work has no tolerance).
Calls go through the C ABI (ctypes)."""
import ctypes
import hashlib
import json
import random
from pathlib import Path

import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth
from conftest import byte_len_for_depth, write_pattern

pytestmark = pytest.mark.gpu
Q = D.Q
GOLDEN = Path(__file__).resolve().parent / "golden"
EPOCH = bytes([11]) * 32
SEED7 = bytes([7]) * 32


# ------------------------------------------------------------------ ring products
@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
def test_ring_mul_batch_matches_oracle(ctx, oracle_lib, n):
    rng = random.Random(n)
    count = 3 if n >= 1024 else 5
    a = [rng.randrange(Q) for _ in range(count * n)]
    b = [rng.randrange(Q) for _ in range(count * n)]
    out = D.unfe_vec(ctx.ring_mul_batch(D.fe_vec(a), D.fe_vec(b), n, count))
    for i in range(count):
        exp = oracle_lib.negacyclic_multiply(a[i * n:(i + 1) * n], b[i * n:(i + 1) * n])
        assert out[i * n:(i + 1) * n] == exp, (n, i)


@pytest.mark.parametrize("n", [64, 512, 2048, 4096])
def test_ring_mul_worst_case_all_q_minus_one(ctx, n):
    a = D.fe_vec([Q - 1] * n)
    out = D.unfe_vec(ctx.ring_mul_batch(a, a, n, 1))
    assert out == [(2 * i + 2 - n) % Q for i in range(n)]


def test_ring_mul_reference_known_answers(ctx):
    # 3 X^(n-1) * 5 X = -15 (src/algebra/ntt.rs:509-521)
    for n in [64, 128, 256, 512, 1024, 2048]:
        a = [0] * n
        b = [0] * n
        a[n - 1], b[1] = 3, 5
        out = D.unfe_vec(ctx.ring_mul_batch(D.fe_vec(a), D.fe_vec(b), n, 1))
        assert out == [Q - 15] + [0] * (n - 1)


def test_ring_mul_microbench_shape_sampled(ctx, oracle_lib):
    """4,096 random degree-512 pairs; 24 sampled products checked against the oracle."""
    n, count = 512, 4096
    raw = synth.chacha20_stream(b"ringmul".ljust(32, b"\0"), 2 * count * n * 16)
    vals = [int.from_bytes(raw[i:i + 16], "little") % Q for i in range(0, len(raw), 16)]
    a, b = vals[:count * n], vals[count * n:]
    out = ctx.ring_mul_batch(D.fe_vec(a), D.fe_vec(b), n, count)
    for i in random.Random(1).sample(range(count), 24):
        exp = oracle_lib.negacyclic_multiply(a[i * n:(i + 1) * n], b[i * n:(i + 1) * n])
        assert D.unfe_vec(out[i * n * 16:(i + 1) * n * 16]) == exp, i


def test_ring_mul_golden(ctx):
    g = json.loads((GOLDEN / "golden.json").read_text())
    for case in g["ring_mul"]:
        n = case["n"]
        out = ctx.ring_mul_batch(bytes.fromhex(case["a"]), bytes.fromhex(case["b"]), n, 1)
        assert out.hex() == case["out"]


def test_ring_mul_reduces_noncanonical_inputs(ctx, oracle_lib):
    n = 64
    rng = random.Random(5)
    a = [rng.randrange(2 ** 128) for _ in range(n)]
    b = [rng.randrange(2 ** 128) for _ in range(n)]
    out = D.unfe_vec(ctx.ring_mul_batch(D.fe_vec(a), D.fe_vec(b), n, 1))
    assert out == oracle_lib.negacyclic_multiply([x % Q for x in a], [x % Q for x in b])


# ------------------------------------------------------------------ hashing / expansion
@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 1023, 1024, 1025, 2048, 2049, 5000, 1 << 16, (1 << 20) + 7])
def test_file_id_matches_oracle(ctx, oracle_lib, n):
    data, _ = synth.random_file(3, n, n)
    assert ctx.file_id(data) == oracle_lib.blake3(data)


def test_file_id_golden(ctx):
    g = json.loads((GOLDEN / "golden.json").read_text())
    for case in g["file_ids"]:
        data, _ = synth.random_file(g["master_seed"], case["len"], case["index"])
        assert ctx.file_id(data).hex() == case["blake3"]


@pytest.mark.parametrize("N,n", [(1, 1), (2, 64), (4, 2), (3, 256), (1, 2048)])
def test_derive_generators_matches_oracle(ctx, oracle_lib, N, n):
    seed = oracle_lib.derive_subseed(bytes([N]) * 32, b"g0")
    assert ctx.derive_generators(seed, N, n) == oracle_lib.derive_generators(seed, N, n)


def test_generators_golden(ctx):
    g = json.loads((GOLDEN / "golden.json").read_text())["generators"]
    out = ctx.derive_generators(bytes.fromhex(g["g_seed"]), g["vector_len"], g["ring_len"])
    assert hashlib.sha256(out).hexdigest() == g["sha256"]


# ------------------------------------------------------------------ commitment
@pytest.mark.parametrize("N,n", [(1, 1), (1, 64), (8, 8), (64, 64), (16, 256), (2, 2048)])
def test_commit_with_generators_matches_oracle(ctx, oracle_lib, N, n):
    rng = random.Random(N * 7 + n)
    w = D.fe_vec(rng.randrange(Q) for _ in range(N * n))
    g = oracle_lib.derive_generators(bytes(range(32)), N, n)
    assert ctx.commit_with_generators(w, g, N, n) == oracle_lib.commit_with_generators(w, g, N, n, threads=8)


@pytest.mark.parametrize("N,n", [(1, 1), (8, 8), (64, 64), (3, 256), (2, 2048)])
def test_commit_witness_matches_oracle(ctx, oracle_lib, N, n):
    """commit_with_ntt with the committer's own generators (derived on the device)."""
    rng = random.Random(N * 13 + n)
    w = D.fe_vec(rng.randrange(Q) for _ in range(N * n))
    seed = bytes([N % 256]) * 32
    g = oracle_lib.derive_generators(oracle_lib.derive_subseed(seed, b"g0"), N, n)
    assert ctx.commit_witness(w, N, n, seed) == oracle_lib.commit_with_generators(w, g, N, n, threads=8)


def test_commit_witness_empty_is_zero_module(ctx):
    assert ctx.commit_witness(b"", 0, 64) == bytes(8 * 16)  # ModuleElement::zero(1), sis.rs:120-122


@pytest.mark.parametrize("N,n", [(64, 64), (512, 512), (2048, 2048), (4096, 4096),
                                 pytest.param(8192, 8192, marks=pytest.mark.slow)])
def test_commit_worst_case_crt_headroom(ctx, N, n):
    """All coefficients q-1: sum_i (-1)(-1) products = N * (2j + 2 - n) (mod q) per slot j.
    The exact sum at slot n-1 is N * n * (q-1)^2: 2^246 at 2048, 2^248 at 4096 and
    2^250 at 8192 (d = 13, 8 GiB of generators), against P / 2 > 2^250.98 of the
    nine CRT primes."""
    w = D.fe_vec([Q - 1]) * (N * n)
    g = D.fe_vec([Q - 1]) * (N * 8 * n)
    out = D.unfe_vec(ctx.commit_with_generators(w, g, N, n))
    exp = [(N * (2 * j + 2 - n)) % Q for j in range(n)]
    for k in range(8):
        assert out[k * n:(k + 1) * n] == exp


@pytest.mark.parametrize("nbytes", [53_248, 8192, 1])
def test_commit_statement_matches_oracle(ctx, oracle_lib, nbytes):
    data, seed = synth.random_file(11, nbytes, 0)
    p = oracle_lib.Prover(data, seed, EPOCH)
    assert ctx.commit(data, seed) == p.statement()


# ------------------------------------------------------------------ protocol
def _gpu_rounds(ctx, data, seed):
    p = D.DamascusProver(ctx, data, seed, EPOCH)
    st = p.statement()
    recs = [p.fold_round(r) for r in range(p.rounds_total())]
    return st, recs, p.final_opening()


@pytest.mark.parametrize("nbytes,tweak", [(8192, 9), (53_248, 1), (byte_len_for_depth(7), 3)])
def test_prover_rounds_bit_exact_with_oracle(ctx, oracle_lib, nbytes, tweak):
    data = write_pattern(nbytes, tweak)
    seed = bytes([tweak]) * 32
    op = oracle_lib.Prover(data, seed, EPOCH)
    gp = D.DamascusProver(ctx, data, seed, EPOCH)
    assert gp.statement() == op.statement()
    assert gp.rounds_total() == op.rounds_total
    for r in range(op.rounds_total):
        assert gp.current_dimensions() == op.dims()
        assert gp.current_commitment() == op.current_commitment()
        assert gp.fold_round(r) == op.fold_round(r), r
    assert gp.current_dimensions() == (1, 1)
    assert gp.final_opening() == op.final_opening()


# File sizes around the witness fill boundaries: the padding columns are zero and
# the device skips their transforms and the generator columns that only meet
# them (fill <= 1/2 of a stage's columns, exactly 1/2, just above, one column,
# the empty file), so every round must still match the oracle bit for bit.
@pytest.mark.parametrize("nbytes", [0, 832, 6656, 13_317, 26_624, 26_625, 106_496])
def test_zero_witness_columns_bit_exact_with_oracle(ctx, oracle_lib, nbytes):
    data, seed = synth.random_file(23, nbytes, 0)
    op = oracle_lib.Prover(data, seed, EPOCH)
    gp = D.DamascusProver(ctx, data, seed, EPOCH)
    assert gp.statement() == op.statement()
    for r in range(op.rounds_total):
        assert gp.fold_round(r) == op.fold_round(r), r
    assert gp.final_opening() == op.final_opening()


def test_full_proof_golden_d6(ctx):
    g = json.loads((GOLDEN / "golden.json").read_text())
    c = g["d6"]
    data, seed = synth.random_file(g["master_seed"], c["file_len"], c["file_index"])
    assert seed.hex() == c["seed_generators"]
    proof = ctx.prove(data, seed, bytes.fromhex(g["epoch_seed"]))
    assert proof == (GOLDEN / "d6_proof.bin").read_bytes()
    assert hashlib.sha256(proof).hexdigest() == c["proof_sha256"]


def test_full_proof_golden_d7_pattern(ctx):
    c = json.loads((GOLDEN / "golden.json").read_text())["d7_pattern"]
    data = write_pattern(c["file_len"], c["tweak"])
    proof = ctx.prove(data, SEED7, EPOCH)
    assert hashlib.sha256(proof).hexdigest() == c["proof_sha256"]


def test_gpu_verifier_accepts_and_oracle_accepts_gpu_proof(ctx, oracle_lib):
    data, seed = synth.random_file(5, 30_000, 0)
    proof = ctx.prove(data, seed, EPOCH)
    assert ctx.verify(proof, EPOCH)
    assert oracle_lib.verify(proof, EPOCH) == 0
    assert not ctx.verify(proof, bytes([12]) * 32)


def test_round_by_round_gpu_verifier(ctx):
    data = write_pattern(8192, 9)
    st, recs, opening = _gpu_rounds(ctx, data, SEED7)
    v = D.DamascusVerifier(ctx, st, EPOCH)
    for i, r in enumerate(recs):
        assert v.current_dimensions() == D.depth_j(6, i)
        assert v.update_commitment(r) == 0
    assert v.current_dimensions() == (1, 1)
    assert v.verify_final_opening(opening) == 0
    bad = bytes([opening[0] ^ 1]) + opening[1:]
    assert v.verify_final_opening(bad) == D.EVERIFY


def test_byte_flips_rejected_like_oracle(ctx, oracle_lib):
    """Sampled byte flips of every record: GPU and oracle verifiers both reject."""
    data = write_pattern(8192, 41)
    st, recs, opening = _gpu_rounds(ctx, data, SEED7)
    rng = random.Random(41)
    for idx, enc in enumerate(recs):
        positions = sorted(set([0, 8, 16, 24, 40, len(enc) - 1] + rng.sample(range(len(enc)), 6)))
        for pos in positions:
            t = bytearray(enc)
            t[pos] ^= 1
            for make in (lambda: D.DamascusVerifier(ctx, st, EPOCH), lambda: oracle_lib.Verifier(st, EPOCH)):
                v = make()
                upd = v.update_commitment if hasattr(v, "update_commitment") else v.update
                fin = v.verify_final_opening if hasattr(v, "verify_final_opening") else v.final
                rejected = False
                for j, r in enumerate(recs):
                    if upd(bytes(t) if j == idx else r) != 0:
                        rejected = True
                        break
                if not rejected:
                    rejected = fin(opening) != 0
                assert rejected, (idx, pos)


def test_round_index_mismatch_and_early_opening(ctx):
    p = D.DamascusProver(ctx, write_pattern(1000, 1), SEED7, EPOCH)
    assert p.final_opening() is None
    with pytest.raises(D.DamascusError) as e:
        p.fold_round(1)
    assert e.value.code == D.ESTATE


def test_timed_round_and_small_record_buffer(ctx, oracle_lib):
    """fold_round_timed returns the same records as the oracle plus RoundOutput's
    three timings (src/protocol/prover.rs:26-31); a record buffer one byte short
    fails with ESIZE before the round runs, so the same round can be retried."""
    data, seed = synth.random_file(31, byte_len_for_depth(7), 0)
    op = oracle_lib.Prover(data, seed, EPOCH)
    gp = D.DamascusProver(ctx, data, seed, EPOCH)
    try:
        assert gp.statement() == op.statement()
        lib = gp._lib
        for r in range(op.rounds_total):
            want = op.fold_round(r)
            short = ctypes.create_string_buffer(len(want) - 1)
            need = ctypes.c_size_t()
            assert lib.damascus_prover_fold_round(gp._h, r, short, len(want) - 1, ctypes.byref(need)) == D.ESIZE
            assert need.value == len(want)
            rec, t = gp.fold_round_timed(r)
            assert rec == want, r
            assert t["vector_fold_ms"] > 0 and t["poly_fold_ms"] > 0
            assert t["total_round_ms"] >= t["vector_fold_ms"] + t["poly_fold_ms"] - 1e-6
        assert gp.final_opening() == op.final_opening()
    finally:
        gp.close()


def test_default_memory_limit_rejects_depth13_on_every_file_path(ctx):
    """RuntimeConfig::default's 512 MiB expansion limit (src/utils/config.rs:21,
    src/utils/io.rs:42-49): a depth-13 file (2 GiB estimate) fails with EINVAL and
    the reference's message through the one-shot prover, the commitment, the
    engine and DamascusProver; a depth-12 file (exactly 512 MiB) passes."""
    assert ctx.max_preprocess_bytes == D.DEFAULT_MEMORY_LIMIT_BYTES
    d13 = b"\x5a" * (4096 * 4096 * 13 + 1)
    assert D.layout_for_byte_len(len(d13))[0] == 13
    calls = [lambda: ctx.prove(d13, SEED7, EPOCH), lambda: ctx.commit(d13, SEED7),
             lambda: D.DamascusProver(ctx, d13, SEED7, EPOCH)]
    for call in calls:
        with pytest.raises(D.DamascusError) as e:
            call()
        assert e.value.code == D.EINVAL and "above max_preprocess_bytes=536870912" in str(e.value)
    with D.Engine(ctx, host_threads=2) as eng:
        small = synth.random_file(31, 60_000, 0)[0]
        t_bad, t_ok = eng.submit(d13, SEED7, EPOCH), eng.submit(small, SEED7, EPOCH)
        with pytest.raises(D.DamascusError) as e:
            eng.wait(t_bad)
        assert e.value.code == D.EINVAL and "split the file" in str(e.value)
        assert eng.wait(t_ok)[0] == ctx.prove(small, SEED7, EPOCH)
    d12 = b"\x5a" * (2048 * 2048 * 13 + 1)
    assert D.layout_for_byte_len(len(d12))[0] == 12
    stmt = ctx.commit(d12, SEED7)
    assert len(stmt) == D.load().damascus_statement_size(4096)
    ctx.set_max_preprocess_bytes(256 << 20)
    try:
        with pytest.raises(D.DamascusError) as e:
            ctx.commit(d12, SEED7)
        assert e.value.code == D.EINVAL
    finally:
        ctx.set_max_preprocess_bytes(0)
    assert ctx.max_preprocess_bytes == D.DEFAULT_MEMORY_LIMIT_BYTES


def test_memory_limit_error_path(ctx):
    with pytest.raises(D.DamascusError) as e:
        D.DamascusProver(ctx, write_pattern(1 << 20, 7), SEED7, EPOCH, max_preprocess_bytes=1024)
    assert e.value.code == D.EINVAL and "split the file" in str(e.value)


def test_hbm_budget_exhaustion_is_an_error():
    small = D.Context(0, hbm_budget_bytes=1 << 20)
    try:
        with pytest.raises(D.DamascusError) as e:
            small.prove(write_pattern(1 << 20, 3), SEED7, EPOCH)
        assert e.value.code == D.ENOMEM_BUDGET
        assert small.reserved == 0
    finally:
        small.close()


def test_d9_prove_verifies_on_gpu_and_oracle(ctx, oracle_lib):
    data, seed = synth.random_file(9, 1 << 20, 0)
    proof = ctx.prove(data, seed, EPOCH)
    assert len(proof) == D.proof_size(1 << 20)
    assert ctx.verify(proof, EPOCH)
    assert oracle_lib.verify(proof, EPOCH) == 0


@pytest.mark.parametrize("nbytes,seed", [(5_689_247, 5), (14_000_000, 5), (3_500_000, 5)])
def test_deep_proofs_verify_and_match_engine(ctx, nbytes, seed):
    """Depths 10 and 11 on files whose transforms meet products with a zero
    Montgomery quotient (v * w * p^-1 = 0 mod 2^32): the prover's recompute
    checks pass, the proof verifies, and the engine gives the same bytes."""
    data, fseed = synth.random_file(seed, nbytes, 1)
    proof = ctx.prove(data, fseed, EPOCH)
    assert ctx.verify(proof, EPOCH)
    with D.Engine(ctx, max_waves=2) as eng:
        assert eng.wait(eng.submit(data, fseed, EPOCH))[0] == proof


@pytest.mark.slow
def test_d11_prove_verifies_on_gpu(ctx):
    data, seed = synth.random_file(11, 16 << 20, 0)
    proof = ctx.prove(data, seed, EPOCH)
    assert ctx.verify(proof, EPOCH)
    bad = bytearray(proof)
    bad[len(bad) // 2] ^= 4
    assert not ctx.verify(bytes(bad), EPOCH)


@pytest.mark.slow
def test_d13_prove_verifies_on_gpu(ctx):
    """Depth 13 (8192 x 8192 witness, rings of 2^13, the deepest the nine-prime CRT
    range holds: sums up to 2^250 < P / 2).  The reference accepts it once its
    memory limit is raised (the estimate is 2 GiB); the engine has no such limit."""
    nbytes = 4096 * 4096 * 13 + 1  # just above the depth-12 capacity
    data, seed = synth.random_file(13, nbytes, 0)
    assert D.layout_for_byte_len(nbytes)[0] == 13
    ctx.set_max_preprocess_bytes(4 << 30)  # the expansion needs 2 GiB
    try:
        with D.Engine(ctx, host_threads=4) as eng:
            proof = eng.prove_batch([(data, seed, EPOCH)])[0]
    finally:
        ctx.set_max_preprocess_bytes(0)
    assert len(proof) == D.proof_size(nbytes)
    assert ctx.verify(proof, EPOCH)
    bad = bytearray(proof)
    bad[len(bad) - 5] ^= 1  # the opening
    assert not ctx.verify(bytes(bad), EPOCH)
    p = D.DamascusProver(ctx, data, seed, EPOCH, max_preprocess_bytes=4 << 30)
    assert p.statement() == proof[:len(p.statement())]


@pytest.mark.slow
def test_d12_prove_verifies_on_gpu(ctx):
    """Depth 12 (4096 x 4096 witness): the commitment sums reach 2^248 in magnitude,
    inside the nine-prime CRT range."""
    nbytes = 2048 * 2048 * 13 + 4096 * 1024  # just above the depth-11 capacity
    data, seed = synth.random_file(12, nbytes, 0)
    assert D.layout_for_byte_len(nbytes)[0] == 12
    proof = ctx.prove(data, seed, EPOCH)
    assert len(proof) == D.proof_size(nbytes)
    assert ctx.verify(proof, EPOCH)


# ------------------------------------------------------------------ reference FFI drop-ins
def test_cuda_fold_batch_dropin():
    rng = random.Random(3)
    n = 5000
    left = [rng.randrange(Q) for _ in range(n)]
    right = [rng.randrange(Q) for _ in range(n)]
    x = rng.randrange(Q)
    assert D.cuda_fold_batch(left, right, x) == [(a + b * x) % Q for a, b in zip(left, right)]


@pytest.mark.parametrize("n", [2, 128, 1024, 4096])
def test_cuda_ntt_batch_dropin_cyclic_convolution(n):
    rng = random.Random(n)
    a = [[rng.randrange(p) for _ in range(n)] for p in D.CRT_PRIMES]
    b = [[rng.randrange(p) for _ in range(n)] for p in D.CRT_PRIMES]
    out = D.cuda_ntt_batch(a, b, n)
    idx = range(n) if n <= 128 else sorted(rng.sample(range(n), 12))
    for pi, p in enumerate(D.CRT_PRIMES):
        for k in idx:
            exp = sum(a[pi][i] * b[pi][(k - i) % n] for i in range(n)) % p
            assert out[pi][k] == exp, (pi, k)


@pytest.mark.parametrize("n", [32, 64, 256, 512, 1024, 2048, 4096])
def test_ring_mul_radix32_passes_match_oracle(oracle_lib, n):
    """The forward transform's radix-32 register passes (DAMASCUS_TUNE_NTT_RADIX = 32)
    give the same products as the oracle, including the all-(q-1) worst case."""
    L = n.bit_length() - 1
    rng = random.Random(1000 + n)
    a = [rng.randrange(Q) for _ in range(2 * n)] + [Q - 1] * n
    b = [rng.randrange(Q) for _ in range(2 * n)] + [Q - 1] * n
    with D.Context(0, tuning=None) as c:
        c.tuning_set(6, L, 32)
        out = D.unfe_vec(c.ring_mul_batch(D.fe_vec(a), D.fe_vec(b), n, 3))
    for i in range(3):
        exp = oracle_lib.negacyclic_multiply(a[i * n:(i + 1) * n], b[i * n:(i + 1) * n])
        assert out[i * n:(i + 1) * n] == exp, (n, i)
