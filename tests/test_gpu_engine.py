"""Continuous-batching engine: every proof is byte-identical to the plain
one-at-a-time path (and to the oracle for small files), whether the request ran
alone or mixed with others of different depths; admission respects the HBM
budget; a failing request does not disturb the others."""
import ctypes
import random

import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu
EPOCH = bytes([11]) * 32


def _files(seed, sizes):
    return [synth.random_file(seed, n, i) for i, n in enumerate(sizes)]


def test_engine_proofs_match_plain_path_and_oracle(ctx, oracle_lib):
    sizes = [1, 8192, 53_248, 60_000, 200_000, 300_000, 900_000]
    files = _files(31, sizes)
    with D.Engine(ctx) as eng:
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
    for (d, s), p in zip(files, proofs):
        assert p == ctx.prove(d, s, EPOCH), len(d)
    for (d, s), p in list(zip(files, proofs))[:3]:
        assert p == oracle_lib.prove(d, s, EPOCH)
    assert ctx.verify(proofs[-1], EPOCH)


def test_engine_result_same_alone_and_in_mix(ctx):
    target = synth.random_file(77, 150_000, 0)
    with D.Engine(ctx) as eng:
        alone = eng.wait(eng.submit(*target, EPOCH))[0]
    rng = random.Random(5)
    others = _files(78, [rng.choice([2_000, 60_000, 400_000, 1 << 20, 3 << 20]) for _ in range(24)])
    with D.Engine(ctx, host_threads=4, max_waves=3) as eng:
        tickets = [eng.submit(d, s, EPOCH) for d, s in others[:12]]
        t = eng.submit(*target, EPOCH)
        tickets += [eng.submit(d, s, EPOCH) for d, s in others[12:]]
        mixed = eng.wait(t)[0]
        rest = [eng.wait(x)[0] for x in tickets]
        st = eng.stats()
    assert mixed == alone
    assert st["completed"] == 25 and st["failed"] == 0
    # coalescing: far fewer waves than the per-request stage count
    assert st["waves"] < 25 * 2 * 9
    for (d, s), p in list(zip(others, rest))[::6]:
        assert p == ctx.prove(d, s, EPOCH)


def test_engine_admission_respects_budget():
    big = D.prover_footprint(1 << 20)
    c = D.Context(0, hbm_budget_bytes=int(big * 2.5))
    try:
        files = _files(91, [1 << 20] * 6 + [30_000] * 4)
        with D.Engine(c) as eng:
            proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
            st = eng.stats()
        assert st["completed"] == 10
        assert st["peak_reserved"] <= c.budget
        assert c.reserved == 0
        for (d, s), p in list(zip(files, proofs))[::4]:
            assert c.verify(p, EPOCH)
    finally:
        c.close()


@pytest.mark.parametrize("limit,code", [(0, D.EINVAL), (1 << 40, D.EUNSUPPORTED)])
def test_engine_failure_is_isolated(ctx, limit, code):
    """872 MB + 1 byte lands on depth 14: above the reference's default expansion
    limit (EINVAL, as src/utils/io.rs:42-49), and with the limit raised above the
    supported maximum depth (13: the CRT range).  The requests around it finish."""
    good = _files(92, [40_000, 70_000])
    ctx.set_max_preprocess_bytes(limit)
    try:
        with D.Engine(ctx) as eng:
            t0 = eng.submit(*good[0], EPOCH)
            bad = eng.submit(bytes(8192 * 8192 * 13 + 1), bytes(32), EPOCH)
            t1 = eng.submit(*good[1], EPOCH)
            p0 = eng.wait(t0)[0]
            with pytest.raises(D.DamascusError) as e:
                eng.wait(bad)
            p1 = eng.wait(t1)[0]
    finally:
        ctx.set_max_preprocess_bytes(0)
    assert e.value.code == code
    assert p0 == ctx.prove(*good[0], EPOCH)
    assert p1 == ctx.prove(*good[1], EPOCH)


def test_engine_device_resident_submission(ctx):
    torch = pytest.importorskip("torch")
    files = _files(93, [50_000, 500_000])
    dev = [torch.frombuffer(bytearray(d), dtype=torch.uint8).cuda() for d, _ in files]
    torch.cuda.synchronize()
    with D.Engine(ctx) as eng:
        ts = [eng.submit_device(t.data_ptr(), len(d), s, EPOCH) for t, (d, s) in zip(dev, files)]
        proofs = [eng.wait(t)[0] for t in ts]
    for (d, s), p in zip(files, proofs):
        assert p == ctx.prove(d, s, EPOCH)


def test_engine_many_small_requests_and_profile(ctx):
    """Many small requests (depths 6-8) in flight at once: every proof verifies,
    sampled ones equal the plain path, and the engine accounts its time."""
    rng = random.Random(17)
    files = _files(94, [rng.randrange(1, 200_000) for _ in range(120)])
    with D.Engine(ctx, max_waves=6) as eng:
        tickets = [eng.submit(d, s, EPOCH) for d, s in files]
        proofs = [eng.wait(t)[0] for t in tickets]
        st = eng.stats()
    assert st["completed"] == 120 and st["failed"] == 0
    assert st["host_stage_ms"] > 0 and st["gpu_idle_ms"] >= 0
    assert st["admit_ms"] > 0 and st["launch_ms"] > 0  # the scheduler thread admitted and launched
    assert st["launches"] > st["waves"] > 0
    for p in proofs:
        assert ctx.verify(p, EPOCH)
    for (d, s), p in list(zip(files, proofs))[::17]:
        assert p == ctx.prove(d, s, EPOCH)


@pytest.mark.slow
def test_engine_soak_streamed_submissions_under_budget():
    """A long stream (400 requests, 1 KB - 2 MiB, log-uniform) submitted while earlier
    ones are still running, under a budget that holds only a few large proofs at
    once: every request completes, sampled proofs verify and equal the plain path,
    and the budget is fully released at the end."""
    rng = random.Random(2026)
    sizes = [int(10 ** rng.uniform(3, 6.32)) for _ in range(400)]
    files = _files(95, sizes)
    budget = 3 * D.prover_footprint(2 << 20)
    c = D.Context(0, hbm_budget_bytes=budget)
    try:
        with D.Engine(c, host_threads=8) as eng:
            tickets, proofs = [], {}
            for i, (d, s) in enumerate(files):
                tickets.append(eng.submit(d, s, EPOCH))
                if i % 50 == 49:  # collect the oldest half while the rest keeps running
                    for t in tickets[: len(tickets) // 2]:
                        if t not in proofs:
                            proofs[t] = eng.wait(t)[0]
            for t in tickets:
                if t not in proofs:
                    proofs[t] = eng.wait(t)[0]
            st = eng.stats()
        assert st["completed"] == 400 and st["failed"] == 0
        assert st["peak_reserved"] <= budget
        assert c.reserved == 0
        for i in range(0, 400, 23):
            p = proofs[tickets[i]]
            assert len(p) == D.proof_size(sizes[i])
            assert c.verify(p, EPOCH)
            assert p == c.prove(*files[i], EPOCH)
    finally:
        c.close()


def test_engine_empty_and_one_byte_files(ctx, oracle_lib):
    """The smallest inputs (an empty file: one zero coefficient; one byte) prove through
    the engine exactly as through the plain path and the oracle."""
    items = [(b"", bytes(range(32))), (b"\x07", bytes(32))]
    with D.Engine(ctx, host_threads=2) as eng:
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in items])
    for (d, s), p in zip(items, proofs):
        assert p == ctx.prove(d, s, EPOCH)
        assert p == oracle_lib.prove(d, s, EPOCH)
        assert ctx.verify(p, EPOCH)


@pytest.mark.parametrize("priority_depth", ["11", "0"])
def test_engine_priority_split_keeps_proofs(ctx, monkeypatch, priority_depth):
    """Stages of d = 11 requests run in their own waves on high-priority streams
    (the default) or with everything else (0): the proofs are the same bytes as
    the plain path's either way."""
    monkeypatch.setenv("DM_ENGINE_PRIORITY_DEPTH", priority_depth)
    files = _files(93, [16 << 20, 60_000, 1 << 20, 300_000, 16 << 20, 8192])
    with D.Engine(ctx) as eng:
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
        st = eng.stats()
    assert st["failed"] == 0
    for (d, s), p in zip(files, proofs):
        assert p == ctx.prove(d, s, EPOCH), len(d)


def test_engine_cancel_queued_and_admitted_requests(ctx):
    """Two 16 MiB requests under a budget that admits one: the second waits in the
    queue and is cancelled there, the first is cancelled between two of its
    stages.  Both end with ECANCELED and leave no memory behind, and the small
    request queued behind them finishes with the plain path's bytes."""
    a = synth.random_file(95, 16 << 20, 0)
    b = synth.random_file(95, 16 << 20, 1)
    small = _files(96, [60_000])[0]
    budget = D.prover_footprint(16 << 20) + D.prover_footprint(60_000) + (64 << 20)
    c = D.Context(0, hbm_budget_bytes=budget, tuning=None)
    try:
        with D.Engine(c) as eng:
            ta = eng.submit(*a, EPOCH)
            for _ in range(200000):  # until the first request's first stage is on the GPU
                if eng.stats()["waves"] >= 1:
                    break
            tb = eng.submit(*b, EPOCH)  # cannot be admitted beside the first
            ts = eng.submit(*small, EPOCH)  # behind it in arrival order
            eng.cancel(tb)
            eng.cancel(ta)
            for t in (ta, tb):
                with pytest.raises(D.DamascusError) as e:
                    eng.wait(t)
                assert e.value.code == D.ECANCELED
            proof = eng.wait(ts)[0]  # finished and taken: the ticket is forgotten
            with pytest.raises(D.DamascusError) as e:
                eng.cancel(ts)
            assert e.value.code == D.EINVAL
            # finished but not yet taken: too late to cancel
            lib = D.load()
            t2 = eng.submit(*small, EPOCH)
            n, lat = ctypes.c_size_t(), ctypes.c_double()
            assert lib.damascus_engine_wait(eng._h, t2, ctypes.byref(n), ctypes.byref(lat)) == 1
            assert lib.damascus_engine_cancel(eng._h, t2) == D.ESTATE
            assert eng.wait(t2)[0] == proof
            assert eng.health()["unfinished"] == 0
        assert c.reserved == 0
    finally:
        c.close()
    assert proof == ctx.prove(*small, EPOCH)


def test_engine_request_timeout_and_bounded_wait(ctx):
    big = synth.random_file(97, 16 << 20, 0)
    small = _files(98, [80_000])[0]
    with D.Engine(ctx) as eng:
        eng.set_request_timeout(0.5)  # a 16 MiB proof takes milliseconds
        t = eng.submit(*big, EPOCH)
        with pytest.raises(D.DamascusError) as e:
            eng.wait(t)
        assert e.value.code == D.ETIMEOUT
        eng.set_request_timeout(0)
        t = eng.submit(*big, EPOCH)
        assert eng.wait(t, timeout_ms=0.01) is None  # still running: the ticket stays valid
        h = eng.health()
        assert h["unfinished"] >= 1 and h["ms_since_progress"] >= 0.0
        proof = eng.wait(t)[0]
        assert eng.wait(eng.submit(*small, EPOCH), timeout_ms=60_000)[0] == ctx.prove(*small, EPOCH)
        assert eng.health() == {"unfinished": 0, "ms_since_progress": 0.0}
        st = eng.stats()
    assert proof == ctx.prove(*big, EPOCH)
    assert st["failed"] == 1


def test_launch_trace_covers_every_kernel_kind(ctx):
    """The launch trace: every timed group of an engine batch, with its stream,
    a start no later than its end, and the kinds of a proof's stages."""
    files = _files(95, [60_000, 300_000, 1_200_000])
    with D.Engine(ctx, max_waves=4) as eng:
        ctx.trace_start()
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
        rows = ctx.trace_read(stop=True)
    ctx.set_profiling(False)
    host_kinds = {"sched_wave", "sched_wave_deep", "wave_done", "fiat_shamir", "req_wait", "req_gpu", "req_host"}
    gpu = [r for r in rows if r[0] not in host_kinds]
    host = [r for r in rows if r[0] in host_kinds]
    kinds = {r[0] for r in gpu}
    assert {"file_hash", "unpack_witness", "gen_generators", "ntt_fwd", "fold", "finish"} <= kinds
    assert all(0 <= r[2] <= r[3] for r in gpu) and all(r[5] >= 1 for r in gpu)
    assert max(r[1] for r in gpu) < 5  # the admission stream and up to four wave streams
    # host rows: every wave's planning and launching (its stream, requests and
    # launches), its completion callback, and one Fiat-Shamir step per stage
    waves = [r for r in host if r[0].startswith("sched_wave")]
    assert waves and all(0 <= r[1] < 4 and r[4] >= 1 and r[5] >= 1 and 0 <= r[2] <= r[3] for r in waves)
    assert len([r for r in host if r[0] == "wave_done"]) == len(waves)
    # every request's stages: Init plus two per round (60 KB, 300 KB and 1.2 MB
    # files: d = 7, 8 and 9)
    steps = sum(2 * d + 1 for d in (7, 8, 9))
    assert len([r for r in host if r[0] == "fiat_shamir"]) == steps
    # and each step's path (ticket in the count field): ready -> launched ->
    # landed -> host step done, in order
    for kind in ("req_wait", "req_gpu", "req_host"):
        path = [r for r in host if r[0] == kind]
        assert len(path) == steps and all(0 <= r[2] <= r[3] for r in path)
    assert len({r[4] for r in host if r[0] == "req_gpu"}) == len(files)
    assert ctx.trace_read() == []  # stopped: nothing more is kept
    for (d, s), p in zip(files, proofs):
        assert p == ctx.prove(d, s, EPOCH)


@pytest.mark.parametrize("env", [{"DM_ENGINE_POLL": "0"}, {"DM_ENGINE_SPIN_US": "0"},
                                 {"DM_ENGINE_POLL": "1", "DM_ENGINE_SPIN_US": "1000"}])
def test_engine_completion_modes_give_identical_proofs(ctx, monkeypatch, env):
    """Wave completion by host callback or by the polling thread, with or without
    the short awake waits: the hand-overs change, the proofs do not (the engine
    reads these settings when it is created)."""
    files = _files(96, [40_000, 250_000, 700_000, 2_000_000])
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with D.Engine(ctx, max_waves=6) as eng:
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
        st = eng.stats()
    assert st["completed"] == len(files) and st["failed"] == 0
    for (d, s), p in zip(files, proofs):
        assert p == ctx.prove(d, s, EPOCH), len(d)


@pytest.mark.parametrize("batch", [0, 3])
def test_engine_admission_batch_gives_identical_proofs(ctx, batch):
    """Admitting every queued request before launching (0) or a few per pass:
    the waves' composition changes, the proofs do not."""
    files = _files(97, [30_000, 120_000, 500_000, 1_500_000, 70_000])
    with D.Engine(ctx, max_waves=4) as eng:
        eng.set_admission_batch(batch)
        proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
    for (d, s), p in zip(files, proofs):
        assert p == ctx.prove(d, s, EPOCH), len(d)
    with D.Engine(ctx) as eng:
        with pytest.raises(D.DamascusError):
            eng.set_admission_batch(-1)


def test_engine_options_give_identical_proofs(ctx):
    """Every engine setting through damascus_engine_create_with_options (callbacks,
    no awake waits, admitting all first, no priority split, few waves): the
    proofs are the plain path's."""
    files = _files(98, [45_000, 180_000, 650_000, 2_500_000])
    for kw in [dict(polling=False, spin_us=0), dict(admission_batch=0, priority_depth=0),
               dict(max_waves=2, host_threads=2, spin_us=1000, admission_batch=2)]:
        with D.Engine(ctx, **kw) as eng:
            proofs = eng.prove_batch([(d, s, EPOCH) for d, s in files])
        for (d, s), p in zip(files, proofs):
            assert p == ctx.prove(d, s, EPOCH), (kw, len(d))


def test_engine_result_view_and_release(ctx):
    """damascus_engine_result points at the finished proof without copying it
    (the same bytes the copying take gives), release forgets it, and a released
    or already taken ticket answers ESTATE."""
    lib = D.load()
    files = _files(91, [60_000, 300_000, 1 << 20])
    with D.Engine(ctx) as eng:
        tickets = [eng.submit(d, s, EPOCH) for d, s in files]
        n, lat = ctypes.c_size_t(), ctypes.c_double()
        ptr, size = ctypes.c_void_p(), ctypes.c_size_t()
        for t, (d, s) in zip(tickets, files):
            assert lib.damascus_engine_wait(eng._h, t, ctypes.byref(n), ctypes.byref(lat)) == 1
            assert lib.damascus_engine_result(eng._h, t, ctypes.byref(ptr), ctypes.byref(size)) == D.OK
            assert size.value == n.value == D.proof_size(len(d))
            viewed = ctypes.string_at(ptr.value, size.value)
            assert viewed == ctx.prove(d, s, EPOCH)
            if t == tickets[0]:
                buf = ctypes.create_string_buffer(n.value)
                assert lib.damascus_engine_take(eng._h, t, buf, n.value) == D.OK
                assert buf.raw == viewed
            else:
                assert lib.damascus_engine_release(eng._h, t) == D.OK
            assert lib.damascus_engine_result(eng._h, t, ctypes.byref(ptr), ctypes.byref(size)) == D.ESTATE
            assert lib.damascus_engine_release(eng._h, t) == D.ESTATE
        # the binding's wait copies once from the same view
        t = eng.submit(*files[1], EPOCH)
        assert eng.wait(t)[0] == ctx.prove(*files[1], EPOCH)


def test_engine_borrowed_host_submission(ctx):
    """Files submitted from the caller's own host memory (pinned, and pageable)
    without a staging copy give the proofs of the copying submission."""
    torch = pytest.importorskip("torch")
    files = _files(93, [0, 1, 60_000, 700_000, 3 << 20])
    pinned = [torch.frombuffer(bytearray(d or b"\0"), dtype=torch.uint8).pin_memory() for d, _ in files]
    pageable = [ctypes.create_string_buffer(d, len(d) or 1) for d, _ in files]
    with D.Engine(ctx) as eng:
        want = [eng.wait(eng.submit(d, s, EPOCH))[0] for d, s in files]
        got_pinned = [eng.wait(t)[0] for t in [eng.submit_borrowed(p.data_ptr(), len(d), s, EPOCH)
                                              for p, (d, s) in zip(pinned, files)]]
        got_pageable = [eng.wait(t)[0] for t in [eng.submit_borrowed(ctypes.addressof(b), len(d), s, EPOCH)
                                                for b, (d, s) in zip(pageable, files)]]
    assert got_pinned == want and got_pageable == want
    assert want[-1] == ctx.prove(*files[-1], EPOCH)


def test_engine_as_completed_yields_every_request_once(ctx):
    """wait_any / as_completed hand back every ticket once, each with the proof
    the ticket-order wait gives, the small requests ahead of the large one."""
    files = _files(95, [3 << 20, 2_000, 60_000, 8_000, 300_000])
    with D.Engine(ctx) as eng:
        tickets = [eng.submit(d, s, EPOCH) for d, s in files]
        got = list(eng.as_completed(tickets))
        assert sorted(t for t, _, _ in got) == sorted(tickets)
        by_ticket = {t: p for t, p, _ in got}
        for t, (d, s) in zip(tickets, files):
            assert by_ticket[t] == ctx.prove(d, s, EPOCH)
        assert got[-1][0] == tickets[0]  # the 3 MiB file (depth 10) finishes last
        lib = D.load()
        arr = (ctypes.c_uint64 * 2)(987654321, 987654322)
        which = ctypes.c_size_t()
        assert lib.damascus_engine_wait_any(eng._h, arr, 2, ctypes.byref(which)) == D.EINVAL


def test_engine_concurrent_collectors(ctx):
    """Several threads wait on the same tickets while others take them: every
    ticket is collected, and a waiter whose ticket another thread took gets an
    answer (its result, kept by the C layer, or EINVAL) instead of waiting on a
    freed request."""
    import threading
    lib = D.load()
    files = _files(99, [2_000, 60_000, 200_000, 8_000, 700_000, 30_000])
    with D.Engine(ctx) as eng:
        tickets = [eng.submit(d, s, EPOCH) for d, s in files]
        answers, errors = [], []

        def waiter():
            try:
                n, lat = ctypes.c_size_t(), ctypes.c_double()
                for t in tickets:
                    answers.append((t, lib.damascus_engine_wait(eng._h, t, ctypes.byref(n), ctypes.byref(lat))))
            except Exception as e:  # pragma: no cover - reported below
                errors.append(e)

        def any_waiter():
            try:
                arr = (ctypes.c_uint64 * len(tickets))(*tickets)
                which = ctypes.c_size_t()
                for _ in range(len(tickets)):
                    rc = lib.damascus_engine_wait_any(eng._h, arr, len(tickets), ctypes.byref(which))
                    answers.append(("any", rc))
            except Exception as e:  # pragma: no cover
                errors.append(e)

        threads = [threading.Thread(target=f) for f in (waiter, waiter, any_waiter, any_waiter)]
        for th in threads:
            th.start()
        for th in threads:
            th.join(timeout=120)
        assert not any(th.is_alive() for th in threads) and not errors
        assert all(rc in (1, D.EINVAL) for t, rc in answers if t != "any")
        assert all(rc in (D.OK, D.EINVAL) for t, rc in answers if t == "any")
        for t, (d, s) in zip(tickets, files):
            n, lat = ctypes.c_size_t(), ctypes.c_double()
            assert lib.damascus_engine_poll(eng._h, t, ctypes.byref(n), ctypes.byref(lat)) == 1
            buf = ctypes.create_string_buffer(n.value)
            assert lib.damascus_engine_take(eng._h, t, buf, n.value) == D.OK
            assert buf.raw == ctx.prove(d, s, EPOCH)
