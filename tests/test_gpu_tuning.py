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
        assert c.tuning_get(A.SPLIT_COORDS, 8) == 1 and c.tuning_get(A.SPLIT_COORDS, 9) == 8
        c.tuning_set(A.SPLIT_COORDS, 9, 2)
        assert c.tuning_get(A.SPLIT_COORDS, 9) == 2
        for knob, L, v in [(A.NTT_GROUP, 6, 48), (A.MAC_TRIPLE, 6, 0), (A.MAC_PLAIN, 6, 33), (7, 6, 8),
                           (A.MAC_SPLIT, 14, 8), (A.SPLIT_COORDS, 9, 3), (A.SPLIT_COORDS, 9, 16),
                           (A.TRIPLE_COORDS, 9, 8), (A.TRIPLE_COORDS, 9, 3), (A.NTT_RADIX, 9, 64),
                           (A.NTT_RADIX, 9, 8)]:
            with pytest.raises(D.DamascusError):
                c.tuning_set(knob, L, v)


def test_tuning_measure_runs_every_knob():
    with D.Context(0, tuning=None) as c:
        for knob in (A.NTT_GROUP, A.MAC_TRIPLE, A.MAC_SPLIT, A.MAC_PLAIN, A.SPLIT_COORDS, A.TRIPLE_COORDS,
                     A.NTT_RADIX):
            for v in A.CANDIDATES[knob][:2] + A.CANDIDATES[knob][-1:]:
                ms = c.tuning_measure(knob, 6, v, A.work_size(knob, 6), reps=2)
                assert 0.0 < ms < 1000.0
        with pytest.raises(D.DamascusError):
            c.tuning_measure(A.NTT_GROUP, 6, 40, 16, 1)


@pytest.mark.parametrize("shape,coords", [("small", 2), ("large", 8), ("large", 4), ("mixed", 0)])
def test_proofs_identical_under_extreme_shapes(shape, coords, oracle_lib):
    """coords: the split MAC's coordinates per thread at every ring size; 0 takes
    1, 2, 4 and 8 in turn by ring size, so jobs of one launch differ in it."""
    files = [synth.random_file(41, n, i) for i, n in enumerate([1, 26_625, 106_496, 300_000, 1_500_000])]
    with D.Context(0, tuning=None) as base:
        want = [base.prove(f, s, EPOCH) for f, s in files]
    with D.Context(0, tuning=None) as c:
        for L in range(0, 14):
            if L >= 4:
                c.tuning_set(A.NTT_GROUP, L, 32 if shape == "small" else 64)
            for knob in (A.MAC_TRIPLE, A.MAC_SPLIT, A.MAC_PLAIN):
                c.tuning_set(knob, L, {"small": 1, "large": 32, "mixed": 4}[shape])
            c.tuning_set(A.SPLIT_COORDS, L, coords or (1, 2, 4, 8)[L % 4])
            c.tuning_set(A.TRIPLE_COORDS, L, min(coords, 4) if coords else (1, 2, 4)[L % 3])
            c.tuning_set(A.NTT_RADIX, L, 32 if shape != "mixed" else (16, 32)[L % 2])
        got = [c.prove(f, s, EPOCH) for f, s in files]
        with D.Engine(c, host_threads=4) as eng:
            via_engine = eng.prove_batch([(f, s, EPOCH) for f, s in files])
    assert got == want and via_engine == want
    assert got[1] == oracle_lib.prove(files[1][0], files[1][1], EPOCH)
