"""Streaming verifier service: every verdict equals the one-shot verifier's
(damascus_verify) on the same bytes, for honest proofs, tampered, truncated and
undecodable ones, whether the generator cache is on, off or too small, under a
tight HBM budget and with submissions from several threads."""
import random
import threading

import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu
EPOCH = bytes([11]) * 32
SYSTEM_SEED = bytes([7]) * 32  # SystemParams::default seed_generators


def _one_shot(ctx, proof: bytes, epoch: bytes = EPOCH) -> int:
    return ctx._lib.damascus_verify(ctx.handle, proof, len(proof), epoch)


def _proofs(ctx, sizes, seed=None, tag=0):
    out = []
    for i, n in enumerate(sizes):
        data, s = synth.random_file(1234 + tag, n, i)
        out.append(ctx.prove(data, seed if seed is not None else s, EPOCH))
    return out


def _tampered(proofs, rng):
    """Bit flips in the statement, a round record and the opening; truncations;
    garbage; an empty proof; trailing bytes."""
    bad = []
    for p in proofs:
        for pos in (40, len(p) // 2, len(p) - 3):
            b = bytearray(p)
            b[pos] ^= 1 << rng.randrange(8)
            bad.append(bytes(b))
        bad.append(p[: len(p) - 5])
        bad.append(p[: len(p) // 3])
        bad.append(p + b"\x00")
    bad.append(b"")
    bad.append(bytes(rng.randrange(256) for _ in range(300)))
    return bad


@pytest.mark.parametrize("cache_bytes", [16 << 30, 0, 1 << 20])
def test_service_verdicts_equal_one_shot(ctx, cache_bytes):
    rng = random.Random(cache_bytes)
    honest = _proofs(ctx, [1, 8192, 53_248, 200_000, 900_000], seed=SYSTEM_SEED)
    honest += _proofs(ctx, [60_000, 300_000], tag=1)  # per-file seeds
    cases = honest + _tampered(honest[::2], rng)
    rng.shuffle(cases)
    expected = [_one_shot(ctx, p) for p in cases]
    with D.VerifyService(ctx, workers=8, cache_bytes=cache_bytes) as svc:
        tickets = [svc.submit(p, EPOCH) for p in cases]
        got = [svc.wait(t)[0] for t in tickets]
        st = svc.stats()
    assert got == expected
    assert sum(1 for e in expected if e == 0) >= len(honest)
    assert st["completed"] == len(cases)
    assert st["accepted"] == sum(1 for e in expected if e == 0)
    if cache_bytes == 0:
        assert st["cache_hits"] == 0 and st["cache_misses"] == 0


def test_service_wrong_epoch_rejects(ctx):
    p = _proofs(ctx, [53_248], seed=SYSTEM_SEED)[0]
    other = bytes([12]) * 32
    with D.VerifyService(ctx, workers=2) as svc:
        code, _ = svc.wait(svc.submit(p, other))
        ok, _ = svc.wait(svc.submit(p, EPOCH))
    assert code == _one_shot(ctx, p, other) == D.EVERIFY
    assert ok == 0


def test_service_cache_shares_generators(ctx):
    """Same shape and system seed: a private expansion at the first sighting, one
    cached expansion at the second, hits afterwards."""
    proofs = _proofs(ctx, [200_000] * 6, seed=SYSTEM_SEED, tag=2)
    with D.VerifyService(ctx, workers=1, cache_bytes=1 << 30) as svc:
        assert svc.verify_batch(proofs, EPOCH) == [True] * 6
        st = svc.stats()
        # a second pass over the same shapes expands nothing
        assert svc.verify_batch(proofs, EPOCH) == [True] * 6
        st2 = svc.stats()
    assert st["cache_misses"] == 2 and st["cache_hits"] == 4
    assert st2["cache_misses"] == 2 and st2["cache_hits"] == 10


def test_service_per_file_seeds_never_cache(ctx):
    """Every proof under its own seed: no family is kept, verdicts are unchanged."""
    proofs = _proofs(ctx, [8192, 60_000, 200_000] * 2, tag=11)
    with D.VerifyService(ctx, workers=3, cache_bytes=1 << 30) as svc:
        assert svc.verify_batch(proofs, EPOCH) == [True] * 6
        st = svc.stats()
    assert st["cache_hits"] == 0 and st["cache_misses"] == 6


def test_service_cache_evicts_least_recently_used(ctx):
    """A cap holding one family: shapes alternate, every one verifies."""
    a = _proofs(ctx, [200_000] * 2, seed=SYSTEM_SEED, tag=3)
    b = _proofs(ctx, [900_000] * 2, seed=SYSTEM_SEED, tag=4)
    fam_b = 512 * 8 * 512 * 16  # d = 9 family, the larger of the two
    with D.VerifyService(ctx, workers=1, cache_bytes=fam_b + (1 << 20)) as svc:
        verdicts = svc.verify_batch([a[0], b[0], a[1], b[1], a[0]], EPOCH)
        st = svc.stats()
    assert verdicts == [True] * 5
    assert st["cache_misses"] == 5 and st["cache_hits"] == 0


def test_service_under_tight_budget(ctx):
    """A budget holding about one d = 9 verification: proofs queue for memory,
    all verify, and the reservation never exceeds the budget."""
    one = 512 * 8 * 512 * 16 * 3 // 2 + 4096
    c = D.Context(0, hbm_budget_bytes=int(one * 1.3))
    try:
        proofs = _proofs(ctx, [900_000] * 4 + [30_000] * 4, seed=SYSTEM_SEED, tag=5)
        with D.VerifyService(c, workers=8, cache_bytes=0) as svc:
            assert svc.verify_batch(proofs, EPOCH) == [True] * 8
            st = svc.stats()
        assert 0 < st["peak_reserved"] <= c.budget
        assert c.reserved == 0
    finally:
        c.close()


def test_service_budget_with_cache_falls_back_and_matches(ctx):
    """Budget too small for a cached family beside the private buffers: the
    verifier drops the cache entry and uses its own copy; verdicts unchanged."""
    one = 512 * 8 * 512 * 16 * 3 // 2 + 4096
    c = D.Context(0, hbm_budget_bytes=one + (1 << 20))
    try:
        proofs = _proofs(ctx, [900_000] * 3, seed=SYSTEM_SEED, tag=6)
        bad = bytearray(proofs[1])
        bad[len(bad) // 2] ^= 4
        cases = proofs + [bytes(bad)]
        with D.VerifyService(c, workers=4, cache_bytes=8 << 30) as svc:
            got = [svc.wait(svc.submit(p, EPOCH))[0] for p in cases]
        assert got == [_one_shot(c, p) for p in cases]
        assert got[:3] == [0, 0, 0] and got[3] != 0
        assert c.reserved == 0
    finally:
        c.close()


def test_service_concurrent_submitters(ctx):
    proofs = _proofs(ctx, [1, 53_248, 200_000, 300_000], seed=SYSTEM_SEED, tag=7)
    bad = [p[:-1] for p in proofs]
    results = {}
    with D.VerifyService(ctx, workers=6) as svc:
        def run(k):
            items = (proofs + bad) * 3
            random.Random(k).shuffle(items)
            ts = [(svc.submit(p, EPOCH), p) for p in items]
            results[k] = [(svc.wait(t)[0], p) for t, p in ts]

        threads = [threading.Thread(target=run, args=(k,)) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        st = svc.stats()
    expected = {p: _one_shot(ctx, p) for p in proofs + bad}
    for k in range(4):
        assert len(results[k]) == 24
        for code, p in results[k]:
            assert code == expected[p]
    assert st["completed"] == 96


def test_service_poll_and_unknown_ticket(ctx):
    p = _proofs(ctx, [53_248], seed=SYSTEM_SEED, tag=8)[0]
    with D.VerifyService(ctx, workers=1) as svc:
        t = svc.submit(p, EPOCH)
        svc.drain()
        code, lat = svc.poll(t)
        assert code == 0 and lat > 0
        with pytest.raises(D.DamascusError):
            svc.poll(t)  # reported once, then forgotten
        with pytest.raises(D.DamascusError):
            svc.wait(987654321)


def test_service_matches_oracle_verifier(ctx, oracle_lib):
    """Oracle-made proofs (and tampered copies): the service's verdicts agree
    with the oracle's own verifier."""
    cases = []
    for i, n in enumerate([1, 8192, 53_248]):
        data, _ = synth.random_file(4321, n, i)
        p = oracle_lib.prove(data, SYSTEM_SEED, EPOCH)
        b = bytearray(p)
        b[len(b) // 2] ^= 0x10
        cases += [p, bytes(b)]
    with D.VerifyService(ctx, workers=4) as svc:
        got = [svc.wait(svc.submit(p, EPOCH))[0] for p in cases]
    assert [g == 0 for g in got] == [oracle_lib.verify(p, EPOCH) == 0 for p in cases]
    assert got[0::2] == [0, 0, 0]


def test_service_cached_family_gives_way_to_a_job(ctx):
    """A budget just above one d = 10 verification: the d = 9 family cached by
    an earlier proof is evicted when the d = 10 job needs the room; both verify."""
    fam10 = 1024 * 8 * 1024 * 16
    private10 = fam10 + fam10 // 2 + 4096
    c = D.Context(0, hbm_budget_bytes=private10 + (8 << 20))
    try:
        p9 = _proofs(ctx, [900_000], seed=SYSTEM_SEED, tag=9)[0]
        p10 = _proofs(ctx, [4 << 20], seed=SYSTEM_SEED, tag=10)[0]
        with D.VerifyService(c, workers=2, cache_bytes=8 << 30) as svc:
            assert svc.verify_batch([p9], EPOCH) == [True]  # first sighting: private copy
            assert svc.verify_batch([p9], EPOCH) == [True]  # second: the family stays cached
            assert svc.stats()["cache_misses"] == 2
            assert svc.verify_batch([p10, p9], EPOCH) == [True, True]
        assert c.reserved == 0
    finally:
        c.close()
