"""Provers' generator cache: proofs are byte-identical with the cache on and off,
through the plain path and the engine, when an entry is filled, hit, shared by
the requests of the plan that fills it, evicted, or dropped for budget; per-file
seeds never fill; turning it off returns its memory."""
import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu
EPOCH = bytes([11]) * 32
SYSTEM_SEED = bytes([7]) * 32


def _files(tag, sizes):
    return [synth.random_file(777 + tag, n, i)[0] for i, n in enumerate(sizes)]


@pytest.fixture(scope="module")
def reference_proofs(ctx):
    """Proofs from the session context, which has no generator cache."""
    cache = {}

    def get(data, seed=SYSTEM_SEED):
        key = (data, seed)
        if key not in cache:
            cache[key] = ctx.prove(data, seed, EPOCH)
        return cache[key]
    return get


def test_plain_path_fill_hit_identical(reference_proofs):
    c = D.Context(0, tuning=None)
    try:
        c.set_generator_cache(4 << 30)
        files = _files(1, [1, 8192, 53_248, 60_000, 200_000, 250_000, 900_000, 1_000_000])
        for rep in range(3):  # first sighting, fill, hits
            for d in files:
                assert c.prove(d, SYSTEM_SEED, EPOCH) == reference_proofs(d), (rep, len(d))
        st = c.generator_cache_stats()
        # shapes d = 6, 7, 8 (60 KB) ... : every shape fills once and hits afterwards
        assert st["fills"] >= 4 and st["hits"] >= st["fills"]
        assert st["bytes"] > 0
        assert all(c.verify(c.prove(d, SYSTEM_SEED, EPOCH), EPOCH) for d in files[:3])
        c.set_generator_cache(0)
        assert c.reserved == 0
    finally:
        c.close()


def test_per_file_seeds_never_fill(reference_proofs):
    c = D.Context(0, tuning=None)
    try:
        c.set_generator_cache(4 << 30)
        items = [synth.random_file(55, n, i) for i, n in enumerate([8192, 60_000, 200_000] * 2)]
        for d, s in items:
            assert c.prove(d, s, EPOCH) == reference_proofs(d, s)
        st = c.generator_cache_stats()
        assert st["fills"] == 0 and st["hits"] == 0 and st["bytes"] == 0
    finally:
        c.close()


def test_engine_shares_fill_within_and_across_waves(reference_proofs):
    c = D.Context(0, tuning=None)
    try:
        c.set_generator_cache(8 << 30)
        files = _files(2, [60_000, 70_000, 80_000, 200_000, 210_000, 900_000, 950_000, 1 << 20] * 3)
        with D.Engine(c) as eng:
            first = eng.prove_batch([(d, SYSTEM_SEED, EPOCH) for d in files])
            st1 = c.generator_cache_stats()
            second = eng.prove_batch([(d, SYSTEM_SEED, EPOCH) for d in files])
            st2 = c.generator_cache_stats()
        for d, p, q in zip(files, first, second):
            assert p == q == reference_proofs(d)
        assert st1["fills"] >= 1
        # the second batch finds every shape cached
        assert st2["hits"] - st1["hits"] == len(files)
        assert st2["fills"] == st1["fills"]
    finally:
        c.close()


def test_small_cap_evicts_and_proofs_identical(reference_proofs):
    c = D.Context(0, tuning=None)
    try:
        # room for one d = 9 family but not for a d = 7 one beside it
        c.set_generator_cache(_entry_bytes(9) + (1 << 20))
        a = _files(3, [200_000, 210_000])
        b = _files(4, [900_000, 950_000])
        order = [a[0], a[1], b[0], b[1], a[0], b[0], a[1], b[1], a[0]]
        for d in order:
            assert c.prove(d, SYSTEM_SEED, EPOCH) == reference_proofs(d)
        st = c.generator_cache_stats()
        assert st["fills"] >= 2
    finally:
        c.close()


def _entry_bytes(d):
    return (1 << (2 * d)) * 8 * (16 + 9 * 4)


def test_tight_budget_drops_cached_families(reference_proofs):
    """A budget that holds one d = 10 prover: a cached d = 9 family fills beside
    a d = 9 prover, then gives way to the d = 10 request (plain path and engine);
    every proof completes and matches."""
    big9, big10 = D.prover_footprint(1 << 20), D.prover_footprint(4 << 20)
    assert big9 + _entry_bytes(9) < big10
    c = D.Context(0, hbm_budget_bytes=big10 + (1 << 20), tuning=None)
    try:
        c.set_generator_cache(64 << 30)
        d9 = _files(5, [900_000, 1 << 20, 950_000])
        d10 = _files(6, [4 << 20])[0]
        for d in d9[:2]:  # first sighting, then a fill that stays cached
            assert c.prove(d, SYSTEM_SEED, EPOCH) == reference_proofs(d)
        assert c.generator_cache_stats()["bytes"] == _entry_bytes(9)
        assert c.prove(d10, SYSTEM_SEED, EPOCH) == reference_proofs(d10)  # trims the d = 9 family
        assert c.generator_cache_stats()["bytes"] == 0
        for d in d9:  # refill
            assert c.prove(d, SYSTEM_SEED, EPOCH) == reference_proofs(d)
        assert c.generator_cache_stats()["bytes"] == _entry_bytes(9)
        with D.Engine(c) as eng:  # admission trims for the d = 10 request
            items = [d9[0], d10, d9[1]]
            proofs = eng.prove_batch([(d, SYSTEM_SEED, EPOCH) for d in items])
            st = eng.stats()
        assert proofs == [reference_proofs(d) for d in items]
        assert st["failed"] == 0 and st["peak_reserved"] <= c.budget
    finally:
        c.close()


def test_turning_off_while_idle_frees_memory():
    c = D.Context(0, tuning=None)
    try:
        c.set_generator_cache(1 << 30)
        d = _files(6, [53_248])[0]
        for _ in range(3):
            c.prove(d, SYSTEM_SEED, EPOCH)
        assert c.generator_cache_stats()["bytes"] > 0
        assert c.reserved > 0
        c.set_generator_cache(0)
        assert c.reserved == 0
        assert c.generator_cache_stats() == {"hits": 0, "fills": 0, "misses": 0, "bytes": 0}
    finally:
        c.close()


def test_engine_plain_provers_and_verifier_share_one_context(reference_proofs):
    """Everything at once on one context with the cache on: the engine, two
    threads of plain provers and the verifier service.  Proofs match the
    uncached ones, honest proofs verify, tampered ones do not, and the cache's
    memory comes back when it is turned off.  (The budget is the default: a
    plain prover does not wait for memory the engine holds, it fails.)"""
    import threading
    c = D.Context(0, tuning=None)
    try:
        c.set_generator_cache(8 << 30)
        files = _files(7, [60_000, 200_000, 900_000, 1 << 20, 53_248, 250_000] * 3)
        out, errors = {}, []

        def plain(k):
            try:
                for i, d in enumerate(files[k::3]):
                    out[("plain", k, i)] = (d, c.prove(d, SYSTEM_SEED, EPOCH))
            except Exception as e:  # surfaced below
                errors.append(e)

        threads = [threading.Thread(target=plain, args=(k,)) for k in range(2)]
        for t in threads:
            t.start()
        with D.Engine(c) as eng, D.VerifyService(c, workers=4, cache_bytes=1 << 30) as svc:
            proofs = eng.prove_batch([(d, SYSTEM_SEED, EPOCH) for d in files])
            bad = [p[:-1] for p in proofs[:4]] + [bytes(p[:100]) + bytes([p[100] ^ 1]) + p[101:] for p in proofs[4:8]]
            verdicts = svc.verify_batch(proofs + bad, EPOCH)
        for t in threads:
            t.join()
        assert not errors, errors
        assert proofs == [reference_proofs(d) for d in files]
        for d, p in out.values():
            assert p == reference_proofs(d)
        assert verdicts == [True] * len(proofs) + [False] * len(bad)
        assert c.reserved <= c.budget
        c.set_generator_cache(0)
        assert c.reserved == 0
    finally:
        c.close()


def test_verifiers_read_generators_from_prover_cache():
    """A context that proves and verifies under one seed: the verifiers (one-shot
    and service) take g_0 from the provers' cache; verdicts are unchanged."""
    c = D.Context(0, tuning=None)
    try:
        c.set_generator_cache(4 << 30)
        files = _files(8, [200_000, 205_000, 210_000])  # all d = 7 (at most 128^2 coefficients)
        proofs = [c.prove(d, SYSTEM_SEED, EPOCH) for d in files]  # first sighting, fill, hit
        bad = bytearray(proofs[0])
        bad[len(bad) // 2] ^= 2
        bad = bytes(bad)
        hits0 = c.generator_cache_stats()["hits"]
        assert all(c.verify(p, EPOCH) for p in proofs)
        assert not c.verify(bad, EPOCH)
        assert c.generator_cache_stats()["hits"] == hits0 + 4
        with D.VerifyService(c, workers=2, cache_bytes=0) as svc:
            assert svc.verify_batch(proofs + [bad], EPOCH) == [True, True, True, False]
        assert c.generator_cache_stats()["hits"] == hits0 + 8
        c.set_generator_cache(0)
        assert c.reserved == 0
    finally:
        c.close()


def test_engine_trims_cached_family_while_waves_in_flight(reference_proofs):
    """An unreferenced cached d = 9 family must give way to a request while a
    different request's waves run.  The eviction frees device memory, which waits
    for the device; the engine therefore trims outside its scheduler lock, so the
    running waves' completion callbacks are not blocked behind it."""
    f10 = D.prover_footprint(4 << 20)
    f8 = D.prover_footprint(600_000)
    assert f8 < _entry_bytes(9)
    c = D.Context(0, hbm_budget_bytes=f10 + _entry_bytes(9) + (1 << 20), tuning=None)
    try:
        c.set_generator_cache(64 << 30)
        d9 = _files(7, [900_000, 950_000])
        for d in d9:  # first sighting, then a fill that stays cached and unreferenced
            assert c.prove(d, SYSTEM_SEED, EPOCH) == reference_proofs(d)
        assert c.generator_cache_stats()["bytes"] == _entry_bytes(9)
        a10, s10 = synth.random_file(808, 4 << 20, 0)  # per-file seeds: neither request uses the cache
        b8, s8 = synth.random_file(808, 600_000, 1)
        with D.Engine(c) as eng:
            ta = eng.submit(a10, s10, EPOCH)
            for _ in range(20000):  # until the d = 10 request's first wave is on the GPU
                if eng.stats()["waves"] >= 1:
                    break
            tb = eng.submit(b8, s8, EPOCH)  # does not fit beside the cached family: trimmed
            pa, pb = eng.wait(ta)[0], eng.wait(tb)[0]
            st = eng.stats()
        assert pa == reference_proofs(a10, s10) and pb == reference_proofs(b8, s8)
        assert st["failed"] == 0 and st["peak_reserved"] <= c.budget
        assert c.generator_cache_stats()["bytes"] == 0
    finally:
        c.close()


def test_engine_cancels_during_admission_and_trims(reference_proofs):
    """Cancels racing the admission of a tight engine: queued requests under a
    budget that holds about two d = 9 provers, cached families that must give way
    (the scheduler trims them outside its lock), and a thread cancelling every
    third request while the engine admits.  Every request ends (no ticket is lost
    or admitted twice), the others' proofs equal the cache-free path's, and the
    memory comes back."""
    import random
    import threading
    f9 = D.prover_footprint(900_000)
    c = D.Context(0, hbm_budget_bytes=2 * f9 + _entry_bytes(9) + (8 << 20), tuning=None)
    try:
        c.set_generator_cache(64 << 30)
        sizes = [900_000, 250_000, 60_000, 700_000, 30_000, 400_000] * 4
        rng = random.Random(11)
        files = []
        for i, n in enumerate(sizes):
            data = _files(20 + i, [n])[0]
            files.append((data, SYSTEM_SEED if i % 2 == 0 else bytes([i]) * 32))
        with D.Engine(c, max_waves=4) as eng:
            tickets = [eng.submit(d, s, EPOCH) for d, s in files]
            victims = tickets[1::3]

            def canceller():
                for t in victims:
                    for _ in range(rng.randrange(0, 3000)):
                        pass
                    try:
                        eng.cancel(t)
                    except D.DamascusError as e:  # already finished, or finished and taken
                        assert e.code in (D.ESTATE, D.EINVAL)

            th = threading.Thread(target=canceller)
            th.start()
            outcomes = {}
            for t in tickets:
                try:
                    res = eng.wait(t, timeout_ms=120_000)
                    assert res is not None, "a request never finished"
                    outcomes[t] = res[0]
                except D.DamascusError as e:
                    assert e.code == D.ECANCELED and t in victims
                    outcomes[t] = None
            th.join()
            assert eng.health()["unfinished"] == 0
        for t, (d, s) in zip(tickets, files):
            if outcomes[t] is not None:
                assert outcomes[t] == reference_proofs(d, s), len(d)
        assert sum(p is not None for p in outcomes.values()) >= len(tickets) - len(victims)
        c.set_generator_cache(0)
        assert c.reserved == 0
    finally:
        c.close()
