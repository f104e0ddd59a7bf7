import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the sm_103a library (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running case")


def write_pattern(size: int, tweak: int) -> bytes:
    """(idx * 17 + tweak) mod 256, the reference's write_pattern_file (src/protocol/prover.rs:473-478)."""
    return bytes(((i & 0xFF) * 17 + tweak) & 0xFF for i in range(size))


def byte_len_for_depth(d: int) -> int:
    """Smallest-ish length landing exactly on depth d (src/protocol/prover.rs:480-487)."""
    assert d >= 6
    return 1 if d == 6 else ((1 << (2 * (d - 1))) + 1) * 13


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx():
    import damascus000_gb300 as D
    c = D.Context(0)
    yield c
    c.close()
