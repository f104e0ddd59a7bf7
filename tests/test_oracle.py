"""Pins the CPU oracle against the reference's own known-answer and property tests.

Each test names the reference test it ports (paths relative to the reference
project root).  Random inputs use Python's seeded PRNG in place of the
reference's StdRng, so the properties, not the random values, carry over.
"""
import random

import pytest

from conftest import byte_len_for_depth, write_pattern

Q = (1 << 112) - 75
SEED7 = bytes([7]) * 32
EPOCH = bytes([11]) * 32


# ---- src/algebra/field.rs:268-311 ------------------------------------------------
def test_field_arithmetic_round_trip(oracle_lib):
    O = oracle_lib
    c = O.fp_mul(17, 9)
    assert c == 153
    assert O.fp_mul(c, O.fp_inv(9)) == 17


def test_arithmetic_matches_reference_modulus(oracle_lib):
    O = oracle_lib
    rng = random.Random(7)
    for _ in range(20_000):
        a, b = rng.randrange(Q), rng.randrange(Q)
        assert O.fp_add(a, b) == (a + b) % Q
        assert O.fp_mul(a, b) == a * b % Q


def test_challenge_bytes_reduce_into_field(oracle_lib):
    v = oracle_lib.fp_from_le_bytes_mod_order(b"\xff" * 64)
    assert v < Q and v == (2 ** 512 - 1) % Q


# ---- BLAKE3 (blake3 crate; spec restatement) ---------------------------------------
def test_blake3_empty_input_published_digest(oracle_lib):
    # The published BLAKE3 digest of the empty input.
    assert oracle_lib.blake3(b"").hex() == "af1349b9f5f9a1a6a0404dea36dcc9499bcb25c9adc112b7cc9a93cae41f3262"


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 1023, 1024, 1025, 2048, 2049, 3072, 3073, 7 * 1024 + 5, 65536 + 1])
def test_blake3_tree_formulations_agree(oracle_lib, n):
    data = bytes(random.Random(n).getrandbits(8) for _ in range(n))
    assert oracle_lib.blake3(data) == oracle_lib.blake3_recursive(data)


# ---- src/algebra/ntt.rs:437-521 ----------------------------------------------------
def test_ntt_round_trip(oracle_lib):
    import ctypes
    for n in [128, 64, 256, 512, 1024, 2048]:
        vals = [(i * 17 + 3) % oracle_lib.CRT_PRIMES[0] for i in range(n)]
        arr = (ctypes.c_uint64 * n)(*vals)
        assert oracle_lib.lib().orc_ntt_roundtrip(arr, n, oracle_lib.CRT_PRIMES[0]) == 0
        assert list(arr) == vals


def test_generic_convolution_matches_reference(oracle_lib):
    import ctypes
    O = oracle_lib
    out = ctypes.create_string_buffer(7 * 16)
    O.lib().orc_convolution(O.fe_vec([1, 2, 3, 4]), 4, O.fe_vec([4, 5, 6, 7]), 4, out)
    c = O.unfe_vec(out.raw)
    assert len(c) == 7 and c[0] == 4 and c[3] == 50


def test_negacyclic_multiply_matches_naive(oracle_lib):
    O = oracle_lib
    n = 64
    lhs = [i + 1 for i in range(n)]
    rhs = [i * 3 + 5 for i in range(n)]
    assert O.negacyclic_multiply(lhs, rhs) == O.negacyclic_multiply(lhs, rhs, naive=True)


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64])
def test_negacyclic_multiply_matches_naive_across_power_of_two_sizes(oracle_lib, n):
    O = oracle_lib
    lhs = [i * 5 + 1 for i in range(n)]
    rhs = [i * 7 + 3 for i in range(n)]
    assert O.negacyclic_multiply(lhs, rhs) == O.negacyclic_multiply(lhs, rhs, naive=True)


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048])
def test_negacyclic_multiply_across_runtime_sizes(oracle_lib, n):
    lhs = [0] * n
    rhs = [0] * n
    lhs[n - 1] = 3
    rhs[1] = 5
    expected = [0] * n
    expected[0] = Q - 15
    assert oracle_lib.negacyclic_multiply(lhs, rhs) == expected


def test_negacyclic_random_against_python(oracle_lib):
    rng = random.Random(11)
    for n in [1, 2, 8, 32, 128]:
        a = [rng.randrange(Q) for _ in range(n)]
        b = [rng.randrange(Q) for _ in range(n)]
        exp = [0] * n
        for i in range(n):
            for j in range(n):
                if i + j < n:
                    exp[i + j] += a[i] * b[j]
                else:
                    exp[i + j - n] -= a[i] * b[j]
        assert oracle_lib.negacyclic_multiply(a, b) == [e % Q for e in exp]


def test_crt_worst_case_all_q_minus_one(oracle_lib):
    n = 256
    a = [Q - 1] * n
    assert oracle_lib.negacyclic_multiply(a, a) == [(2 * i + 2 - n) % Q for i in range(n)]


# ---- src/algebra/poly.rs:184-241 ---------------------------------------------------
def test_odd_even_split_and_fold():
    p = list(range(1, 9))
    even, odd = p[0::2], p[1::2]
    assert even == [1, 3, 5, 7] and odd == [2, 4, 6, 8]
    assert even[0] + odd[0] * 2 == 5


def test_x_n_plus_one_vanishes(oracle_lib):
    import ctypes
    O = oracle_lib
    n = 64
    acc = [1] + [0] * (n - 1)
    for _ in range(n):
        out = ctypes.create_string_buffer(16 * n)
        O.lib().orc_mul_by_x(O.fe_vec(acc), n, out)
        acc = O.unfe_vec(out.raw)
    assert [(c + (1 if i == 0 else 0)) % Q for i, c in enumerate(acc)] == [0] * n


def test_scalar_unit_inverse_restores_ring_element(oracle_lib):
    O = oracle_lib
    rng = random.Random(9)
    n = 64
    for _ in range(8):
        a = [rng.randrange(Q) for _ in range(n)]
        s = rng.randrange(1, Q)
        b = [s] + [0] * (n - 1)
        binv = [O.fp_inv(s)] + [0] * (n - 1)
        assert O.negacyclic_multiply(O.negacyclic_multiply(a, b), binv) == a


# ---- src/commitment/sis.rs:276-326 --------------------------------------------------
def test_commitment_is_deterministic(oracle_lib):
    O = oracle_lib
    g_seed = O.derive_subseed(bytes([42]) * 32, b"g0")
    g = O.derive_generators(g_seed, 2, 64)
    w = bytes(2 * 64 * 16)
    assert O.commit_with_generators(w, g, 2, 64) == O.commit_with_generators(w, g, 2, 64)


def test_commitment_preserves_ring_linearity(oracle_lib):
    O = oracle_lib
    rng = random.Random(12)
    n, N = 64, 4
    g = O.derive_generators(O.derive_subseed(bytes([9]) * 32, b"g0"), N, n)
    wa = [[rng.randrange(Q) for _ in range(n)] for _ in range(N)]
    wb = [[rng.randrange(Q) for _ in range(n)] for _ in range(N)]
    ra = [rng.randrange(Q) for _ in range(n)]
    rb = [rng.randrange(Q) for _ in range(n)]
    ca = O.unfe_vec(O.commit_with_generators(O.fe_vec(sum(wa, [])), g, N, n))
    cb = O.unfe_vec(O.commit_with_generators(O.fe_vec(sum(wb, [])), g, N, n))
    lin = []
    for i in range(N):
        x = O.negacyclic_multiply(wa[i], ra)
        y = O.negacyclic_multiply(wb[i], rb)
        lin.append([(u + v) % Q for u, v in zip(x, y)])
    clin = O.unfe_vec(O.commit_with_generators(O.fe_vec(sum(lin, [])), g, N, n))
    for k in range(8):
        x = O.negacyclic_multiply(ca[k * n:(k + 1) * n], ra)
        y = O.negacyclic_multiply(cb[k * n:(k + 1) * n], rb)
        assert clin[k * n:(k + 1) * n] == [(u + v) % Q for u, v in zip(x, y)]


def test_commit_ntt_and_naive_agree(oracle_lib):
    O = oracle_lib
    rng = random.Random(4)
    n, N = 32, 8
    g = O.derive_generators(bytes(range(32)), N, n)
    w = O.fe_vec(rng.randrange(Q) for _ in range(N * n))
    assert O.commit_with_generators(w, g, N, n, use_ntt=True) == O.commit_with_generators(w, g, N, n, use_ntt=False)


def test_generator_family_is_module_valued(oracle_lib):
    g = oracle_lib.derive_generators(oracle_lib.derive_subseed(bytes([1]) * 32, b"g0"), 2, 64)
    assert len(g) == 2 * 8 * 64 * 16
    assert all(v < Q for v in oracle_lib.unfe_vec(g))


# ---- src/protocol/transcript.rs:116-142 ---------------------------------------------
def test_vec_and_poly_challenges_are_domain_separated(oracle_lib):
    O = oracle_lib
    n = 64

    def tagged(t):
        v = [0] * (8 * n)
        v[0] = t
        v[n + 1] = t + 1
        return O.fe_vec(v)

    args = (tagged(11), n, tagged(17), n, tagged(23), n)
    a = O.challenge(EPOCH, bytes([3]) * 32, b"vec", 0, *args)
    b = O.challenge(EPOCH, bytes([3]) * 32, b"poly", 0, *args)
    assert a != b and a != 0 and b != 0


# ---- src/utils/io.rs:128-166 --------------------------------------------------------
def test_expand_preserves_injective_chunks(oracle_lib):
    payload = bytes([0xA5]) * (13 * 3 + 5)
    fid, d, w = oracle_lib.expand_file(payload)
    assert d == 6 and len(w) == 64 * 64 * 16
    vals = oracle_lib.unfe_vec(w)
    assert vals[0] == int.from_bytes(bytes([0xA5]) * 13, "little")
    assert vals[3] == int.from_bytes(bytes([0xA5]) * 5, "little")
    assert all(v == 0 for v in vals[4:])
    assert fid == oracle_lib.blake3(payload)


@pytest.mark.parametrize("nbytes", [128 * 1024 * 1024, 1024 * 1024 * 1024])
def test_square_layout_expands_both_dimensions_for_large_inputs(oracle_lib, nbytes):
    d, dim = oracle_lib.layout_for_byte_len(nbytes)
    assert dim == 1 << d and d >= 6
    assert dim * dim >= oracle_lib.lib().orc_coeff_count_for_byte_len(nbytes)
    assert dim * dim * 13 >= nbytes


def test_expand_rejects_memory_overcommit(oracle_lib):
    with pytest.raises(ValueError):
        oracle_lib.expand_file(bytes([0x55]) * 4096, max_preprocess=64)


@pytest.mark.parametrize("d", [6, 7, 8, 9, 10, 11])
def test_byte_len_for_depth_lands_on_depth(oracle_lib, d):
    assert oracle_lib.layout_for_byte_len(byte_len_for_depth(d))[0] == d


# ---- src/protocol/prover.rs:511-877 --------------------------------------------------
def test_distinct_files_produce_distinct_initial_commitments(oracle_lib):
    O = oracle_lib
    a = O.Prover(write_pattern(8192, 3), SEED7, EPOCH)
    b = O.Prover(write_pattern(8192, 4), SEED7, EPOCH)
    assert a.current_commitment() != b.current_commitment()
    assert a.statement()[:32] != b.statement()[:32]


def test_initialize_errors_when_full_expansion_exceeds_memory_limit(oracle_lib):
    with pytest.raises(ValueError):
        oracle_lib.Prover(write_pattern(1 << 20, 7), SEED7, EPOCH, max_preprocess=1024)


def _prove_rounds(O, data):
    p = O.Prover(data, SEED7, EPOCH)
    st = p.statement()
    recs = [p.fold_round(r) for r in range(p.rounds_total)]
    return st, recs, p.final_opening()


def test_honest_transcript_replays_and_tampering_is_rejected(oracle_lib):
    O = oracle_lib
    st, recs, opening = _prove_rounds(O, write_pattern(8192, 9))
    v = O.Verifier(st, EPOCH)
    for r in recs:
        assert v.update(r) == 0
    assert v.final(opening) == 0
    bad = bytearray(recs[0])
    # l_vec coord 0 coeff 0 += 1  (u64 round | u64 8 | u64 n | coeff...)
    off = 8 + 8 + 8
    val = (int.from_bytes(bad[off:off + 16], "little") + 1) % Q
    bad[off:off + 16] = val.to_bytes(16, "little")
    v = O.Verifier(st, EPOCH)
    assert v.update(bytes(bad)) == 0
    for r in recs[1:]:
        assert v.update(r) == 0
    assert v.final(opening) != 0


def test_round_record_serialization_matches_module_payload_scale(oracle_lib):
    O = oracle_lib
    p = O.Prover(write_pattern(8192, 13), SEED7, EPOCH)
    rec = p.fold_round(0)
    coeffs = 2 * 8 * 64 + 2 * 8 * 32
    assert len(rec) >= coeffs * 16
    assert len(rec) >= 4 * 8 * 32 * 16
    assert len(rec) == 296 + 384 * 64  # 24,872 bytes at d=6, round 0


def test_single_round_preserves_commitment_through_vector_and_poly_stages(oracle_lib):
    """prover.rs:627-692, checked through the oracle verifier's replay of round 0."""
    O = oracle_lib
    p = O.Prover(write_pattern(8192, 31), SEED7, EPOCH)
    st = p.statement()
    rec = p.fold_round(0)  # the oracle prover asserts both recompute invariants
    v = O.Verifier(st, EPOCH)
    assert v.update(rec) == 0
    assert v.dims() == p.dims()


def test_serialized_round_record_byte_flip_is_rejected(oracle_lib):
    O = oracle_lib
    st, recs, opening = _prove_rounds(O, write_pattern(8192, 21))
    enc = bytearray(recs[0])
    enc[len(enc) - 8] ^= 1
    v = O.Verifier(st, EPOCH)
    rejected = v.update(bytes(enc)) != 0
    if not rejected:
        for r in recs[1:]:
            if v.update(r) != 0:
                rejected = True
                break
    if not rejected:
        rejected = v.final(opening) != 0
    assert rejected


def _zero_statement(d):
    n = 1 << d
    module = (8).to_bytes(8, "little") + b"".join(n.to_bytes(8, "little") + bytes(16 * n) for _ in range(8))
    return bytes([d]) * 32 + byte_len_for_depth(d).to_bytes(8, "little") + d.to_bytes(8, "little") + module + \
        bytes([17]) * 32


def _zero_record(d, rnd):
    def module(n):
        return (8).to_bytes(8, "little") + b"".join(n.to_bytes(8, "little") + bytes(16 * n) for _ in range(8))
    nv = 1 << (d - rnd)
    return rnd.to_bytes(8, "little") + module(nv) + module(nv) + module(nv // 2) + module(nv // 2)


@pytest.mark.parametrize("d", [6, 8, 10])
def test_dual_dimension_fold_halves_each_round(oracle_lib, d):
    O = oracle_lib
    v = O.Verifier(_zero_statement(d), EPOCH)
    total = (1 << d) ** 2
    for rnd in range(d):
        assert v.dims() == (1 << (d - rnd), 1 << (d - rnd))
        rec = _zero_record(d, rnd)
        assert len(rec) >= 2 * 8 * (1 << (d - rnd)) * 16
        assert v.update(rec) == 0
        N, n = v.dims()
        assert N * n * 4 == total
        total = N * n
    assert v.dims() == (1, 1)
    assert v.final(bytes(16)) == 0


@pytest.mark.parametrize("d", [6, 7, 8, 9])
def test_e2e_zero_record_replay_across_depths(oracle_lib, d):
    O = oracle_lib
    v = O.Verifier(_zero_statement(d), EPOCH)
    for rnd in range(d):
        assert v.update(_zero_record(d, rnd)) == 0
    assert v.final(bytes(16)) == 0


def test_serialized_micro_block_byte_flips_are_rejected(oracle_lib):
    """prover.rs:810-877 on a deterministic sample of byte positions of every record."""
    O = oracle_lib
    st, recs, opening = _prove_rounds(O, write_pattern(8192, 41))
    prefixes = []
    v = O.Verifier(st, EPOCH)
    for r in recs:
        prefixes.append(v.clone())
        assert v.update(r) == 0
    rng = random.Random(41)
    for idx, enc in enumerate(recs):
        positions = sorted(set(list(range(0, 48)) + [len(enc) - 1 - i for i in range(24)] +
                               rng.sample(range(len(enc)), min(40, len(enc)))))
        for pos in positions:
            t = bytearray(enc)
            t[pos] ^= 1
            vv = prefixes[idx].clone()
            rejected = vv.update(bytes(t)) != 0
            if not rejected:
                for r in recs[idx + 1:]:
                    if vv.update(r) != 0:
                        rejected = True
                        break
            if not rejected:
                rejected = vv.final(opening) != 0
            assert rejected, (idx, pos)


def test_full_prove_verify_one_shot(oracle_lib):
    O = oracle_lib
    data = write_pattern(53_248, 5)
    proof = O.prove(data, SEED7, EPOCH)
    assert len(proof) == O.proof_size_for_depth(6)
    assert O.verify(proof, EPOCH) == 0
    assert O.verify(proof, bytes([12]) * 32) != 0
