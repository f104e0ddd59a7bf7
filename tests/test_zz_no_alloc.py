"""The allocation-free file-id entry point, for callers that cannot allocate
device memory (graph capture, fixed-budget serving loops, foreign allocators).

Checks damascus_file_id_noalloc through the C ABI against the allocating
damascus_file_id, bit-exact, on two calls in a row per input (the static
scratch keeps the previous call's contents).  Collected last on purpose."""
import ctypes

import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_BYTES = 64 << 20


def test_file_id_noalloc_matches_allocating_entry_point(ctx):
    torch = pytest.importorskip("torch")
    lib = D.load()
    stream = torch.cuda.current_stream()
    out = torch.zeros(32, dtype=torch.uint8, device="cuda")
    for n in [0, 1, 1024, 1025, 4099, 1 << 20, (16 << 20) + 5, MAX_BYTES]:
        data, _ = synth.random_file(77, n, n)
        want = ctx.file_id(data)
        dev = torch.frombuffer(bytearray(data if n else b"\0"), dtype=torch.uint8).cuda()
        for _ in range(2):
            out.fill_(0xEE)
            rc = lib.damascus_file_id_noalloc(ctypes.c_void_p(dev.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                              ctypes.c_void_p(stream.cuda_stream))
            assert rc == D.OK
            stream.synchronize()
            assert bytes(out.cpu().tolist()) == want, n


def test_file_id_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    lib = D.load()
    dev = torch.zeros(16, dtype=torch.uint8, device="cuda")
    out = torch.zeros(32, dtype=torch.uint8, device="cuda")
    rc = lib.damascus_file_id_noalloc(ctypes.c_void_p(dev.data_ptr()), MAX_BYTES + 1,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert rc == D.ESIZE
