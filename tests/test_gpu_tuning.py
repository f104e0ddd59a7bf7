"""Launch-shape tuning (damascus_tuning_*): knobs round-trip and are validated,
the measurement entry runs every knob's kernel, and proofs stay byte-identical
under extreme launch shapes (the results never depend on the tuning)."""
import pytest

import damascus000_gb300 as D
from damascus000_gb300 import autotune as A
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu
EPOCH = bytes([11]) * 32


def test_tuning_set_get_and_validation():
    with D.Context(0, tuning=None) as c:
        assert c.tuning_get(A.NTT_GROUP, 6) == 64
        assert c.tuning_get(A.MAC_TRIPLE, 11) == 8
        c.tuning_set(A.NTT_GROUP, 6, 32)
        c.tuning_set(A.MAC_SPLIT, 9, 24)
        assert c.tuning_get(A.NTT_GROUP, 6) == 32 and c.tuning_get(A.MAC_SPLIT, 9) == 24
        for knob, L, v in [(A.NTT_GROUP, 6, 48), (A.MAC_TRIPLE, 6, 0), (A.MAC_PLAIN, 6, 33), (7, 6, 8),
                           (A.MAC_SPLIT, 14, 8)]:
            with pytest.raises(D.DamascusError):
                c.tuning_set(knob, L, v)


def test_tuning_measure_runs_every_knob():
    with D.Context(0, tuning=None) as c:
        for knob in (A.NTT_GROUP, A.MAC_TRIPLE, A.MAC_SPLIT, A.MAC_PLAIN):
            for v in A.CANDIDATES[knob][:2]:
                ms = c.tuning_measure(knob, 6, v, A.work_size(knob, 6), reps=2)
                assert 0.0 < ms < 1000.0
        with pytest.raises(D.DamascusError):
            c.tuning_measure(A.NTT_GROUP, 6, 40, 16, 1)


@pytest.mark.parametrize("shape", ["small", "large"])
def test_proofs_identical_under_extreme_shapes(shape, oracle_lib):
    files = [synth.random_file(41, n, i) for i, n in enumerate([1, 26_625, 106_496, 300_000])]
    with D.Context(0, tuning=None) as base:
        want = [base.prove(f, s, EPOCH) for f, s in files]
    with D.Context(0, tuning=None) as c:
        for L in range(0, 14):
            if L >= 4:
                c.tuning_set(A.NTT_GROUP, L, 32 if shape == "small" else 64)
            for knob in (A.MAC_TRIPLE, A.MAC_SPLIT, A.MAC_PLAIN):
                c.tuning_set(knob, L, 1 if shape == "small" else 32)
        got = [c.prove(f, s, EPOCH) for f, s in files]
        with D.Engine(c, host_threads=4) as eng:
            via_engine = eng.prove_batch([(f, s, EPOCH) for f, s in files])
    assert got == want and via_engine == want
    assert got[1] == oracle_lib.prove(files[1][0], files[1][1], EPOCH)
