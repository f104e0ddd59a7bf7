"""The allocation-free file-id entry point, for callers that cannot allocate
device memory: serving loops confined to a fixed, pre-reserved budget, and hosts
whose device allocator belongs to another framework.

Checks damascus_file_id_noalloc through the C ABI against the allocating
damascus_file_id, bit-exact, on two calls in a row per input (the static
scratch keeps the previous call's contents), that a call leaves the device's
free memory unchanged, that it captures into a CUDA graph and replays there,
and the size limit.  Collected last on purpose."""
import ctypes

import pytest

import damascus000_gb300 as D
from damascus000_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_BYTES = 64 << 20


def _call(lib, dev, n, out, stream):
    return lib.damascus_file_id_noalloc(ctypes.c_void_p(dev.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream))


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
            assert _call(lib, dev, n, out, stream) == D.OK
            stream.synchronize()
            assert bytes(out.cpu().tolist()) == want, n


def test_file_id_noalloc_leaves_free_memory_unchanged(ctx):
    torch = pytest.importorskip("torch")
    lib = D.load()
    stream = torch.cuda.current_stream()
    data, _ = synth.random_file(78, 3 << 20, 0)
    dev = torch.frombuffer(bytearray(data), dtype=torch.uint8).cuda()
    out = torch.zeros(32, dtype=torch.uint8, device="cuda")
    assert _call(lib, dev, len(data), out, stream) == D.OK  # the array exists once the module is loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, dev, len(data), out, stream) == D.OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert bytes(out.cpu().tolist()) == ctx.file_id(data)


def test_file_id_noalloc_replays_from_a_cuda_graph(ctx):
    """The call captured into a CUDA graph once (after a first call outside
    capture resolved the array's address), then replayed over new contents of
    the same input buffer: each replay gives that content's file id."""
    torch = pytest.importorskip("torch")
    lib = D.load()
    n = (2 << 20) + 77
    first, _ = synth.random_file(79, n, 0)
    second, _ = synth.random_file(80, n, 0)
    dev = torch.frombuffer(bytearray(first), dtype=torch.uint8).cuda()
    out = torch.zeros(32, dtype=torch.uint8, device="cuda")
    assert _call(lib, dev, n, out, torch.cuda.current_stream()) == D.OK
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, capture_error_mode="thread_local"):
        rc = _call(lib, dev, n, out, torch.cuda.current_stream())
    assert rc == D.OK
    for data in (second, first, second):
        dev.copy_(torch.frombuffer(bytearray(data), dtype=torch.uint8))
        out.fill_(0xEE)
        graph.replay()
        torch.cuda.synchronize()
        assert bytes(out.cpu().tolist()) == ctx.file_id(data)


def test_file_id_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    lib = D.load()
    dev = torch.zeros(16, dtype=torch.uint8, device="cuda")
    out = torch.zeros(32, dtype=torch.uint8, device="cuda")
    rc = lib.damascus_file_id_noalloc(ctypes.c_void_p(dev.data_ptr()), MAX_BYTES + 1,
                                      ctypes.c_void_p(out.data_ptr()), None)
    assert rc == D.ESIZE
