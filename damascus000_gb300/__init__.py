"""GB300 (sm_103a) Damascus Fold prover/verifier -- Python binding of the C ABI.

The compute path is ``libdamascus_gb300.so`` (hand-written CUDA for sm_103a plus
the C++ host runtime) built in-tree by :mod:`damascus000_gb300.build` and
loaded here through ctypes.  The classes mirror the reference crate's public API
(``DamascusProver``, ``DamascusVerifier``, ``ModuleSisCommitter``,
``negacyclic_multiply``), with field elements as Python ints and serialized
objects as bincode bytes identical to the reference's.

There is no CPU fallback: creating a :class:`Context` without a GB300 raises
:class:`DamascusError`.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Iterable, List, Optional, Sequence, Tuple

from . import build as _build

Q = (1 << 112) - 75
MODULE_RANK = 8
MIN_FOLD_DEPTH = 6
BYTES_PER_COEFF = 13
CRT_PRIMES = (3892314113, 2281701377, 2013265921, 2885681153,
              2483027969, 1811939329, 469762049, 4194304001)
DEFAULT_GENERATOR_SEED = bytes([7]) * 32
DEFAULT_EPOCH_SEED = bytes([11]) * 32
DEFAULT_MEMORY_LIMIT_BYTES = 512 * 1024 * 1024

OK = 0
EINVAL, ENOMEM_BUDGET, ECUDA, ETIMEOUT, EVERIFY, EINVARIANT, ESTATE, ESIZE, EDESERIALIZE, EUNSUPPORTED = \
    -1, -2, -3, -4, -5, -6, -7, -8, -9, -10
ECANCELED = -11
_CODE_NAMES = {EINVAL: "EINVAL", ENOMEM_BUDGET: "ENOMEM_BUDGET", ECUDA: "ECUDA", ETIMEOUT: "ETIMEOUT",
               EVERIFY: "EVERIFY", EINVARIANT: "EINVARIANT", ESTATE: "ESTATE", ESIZE: "ESIZE",
               EDESERIALIZE: "EDESERIALIZE", EUNSUPPORTED: "EUNSUPPORTED", ECANCELED: "ECANCELED"}

#: every symbol include/damascus.h declares
EXPORTED_SYMBOLS = (
    "damascus_ctx_create", "damascus_ctx_destroy", "damascus_last_error", "damascus_create_error",
    "damascus_ctx_budget", "damascus_ctx_reserved",
    "damascus_ctx_set_max_preprocess_bytes", "damascus_ctx_max_preprocess_bytes", "damascus_measure_int_multiply",
    "damascus_fp_add", "damascus_fp_sub", "damascus_fp_mul", "damascus_fp_inv",
    "damascus_fp_from_le_bytes_mod_order", "damascus_blake3", "damascus_blake3_keyed",
    "damascus_transcript_challenge", "damascus_coeff_count_for_byte_len", "damascus_layout_for_byte_len",
    "damascus_proof_size", "damascus_record_size", "damascus_statement_size", "damascus_prover_footprint",
    "damascus_file_id", "damascus_derive_generators", "damascus_commit_with_generators", "damascus_commit",
    "damascus_ring_mul_batch", "damascus_ring_mul_batch_device", "damascus_engine_profile",
    "damascus_engine_scheduler_profile", "damascus_ctx_trace_start", "damascus_ctx_trace_read",
    "damascus_prover_new", "damascus_prover_free", "damascus_prover_rounds_total",
    "damascus_prover_current_round", "damascus_prover_dimensions", "damascus_prover_statement",
    "damascus_prover_current_commitment", "damascus_prover_fold_round", "damascus_prover_final_opening",
    "damascus_prover_fold_round_timed",
    "damascus_prove", "damascus_prove_device", "damascus_prove_device_timed", "damascus_ctx_flush_l2",
    "damascus_verifier_new", "damascus_verifier_free", "damascus_verifier_update_commitment",
    "damascus_verifier_verify_final_opening", "damascus_verifier_round", "damascus_verifier_dimensions",
    "damascus_verify", "damascus_cuda_fold_batch", "damascus_cuda_ntt_batch",
    "damascus_ctx_set_profiling", "damascus_ctx_reset_stats", "damascus_ctx_kernel_stat",
    "damascus_ctx_synchronize", "damascus_file_id_noalloc",
    "damascus_engine_create", "damascus_engine_destroy", "damascus_engine_submit", "damascus_engine_submit_device",
    "damascus_engine_submit_borrowed", "damascus_engine_wait_any",
    "damascus_engine_poll",
    "damascus_engine_wait", "damascus_engine_take", "damascus_engine_drain", "damascus_engine_stats",
    "damascus_engine_wait_timeout", "damascus_engine_cancel", "damascus_engine_set_request_timeout",
    "damascus_engine_set_admission_batch", "damascus_engine_create_with_options",
    "damascus_engine_health", "damascus_engine_result", "damascus_engine_release",
    "damascus_tuning_set", "damascus_tuning_get", "damascus_tuning_measure",
    "damascus_verify_service_create", "damascus_verify_service_destroy", "damascus_verify_service_submit",
    "damascus_verify_service_poll", "damascus_verify_service_wait", "damascus_verify_service_drain",
    "damascus_verify_service_stats", "damascus_ctx_set_generator_cache", "damascus_ctx_generator_cache_stats",
    "damascus_commit_witness",
)


class EngineOptions(ctypes.Structure):
    """damascus_engine_options: a negative value keeps the default (which the
    DM_ENGINE_* environment variable overrides); host_threads and max_waves keep
    theirs at 0."""
    _fields_ = [("host_threads", ctypes.c_int), ("max_waves", ctypes.c_int), ("priority_depth", ctypes.c_int),
                ("polling", ctypes.c_int), ("spin_us", ctypes.c_int), ("admission_batch", ctypes.c_int)]


class DamascusError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        self.code = code
        super().__init__(f"{_CODE_NAMES.get(code, code)}: {message}")


_lib: Optional[ctypes.CDLL] = None


def library_path() -> Path:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libdamascus_gb300.so (building it in-tree when missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    path = library_path()
    if not path.exists():
        raise DamascusError(ECUDA, f"{path} is missing; run damascus000_gb300.build.build()")
    L = ctypes.CDLL(str(path))
    _declare(L)
    _lib = L
    return L


def _declare(L: ctypes.CDLL) -> None:
    vp, sz, u64, u32, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
    cp = ctypes.c_char_p
    P = ctypes.POINTER

    def sig(name, res, *args):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = list(args)

    sig("damascus_ctx_create", i32, i32, u64, P(vp))
    sig("damascus_ctx_destroy", None, vp)
    sig("damascus_last_error", cp, vp)
    sig("damascus_create_error", cp)
    sig("damascus_ctx_budget", u64, vp)
    sig("damascus_ctx_reserved", u64, vp)
    for n in ("damascus_fp_add", "damascus_fp_sub", "damascus_fp_mul"):
        sig(n, None, cp, cp, vp)
    sig("damascus_fp_inv", None, cp, vp)
    sig("damascus_fp_from_le_bytes_mod_order", None, cp, sz, vp)
    sig("damascus_blake3", None, cp, sz, vp)
    sig("damascus_blake3_keyed", None, cp, cp, sz, vp)
    sig("damascus_transcript_challenge", i32, cp, cp, cp, u64, cp, u64, cp, u64, cp, u64, vp)
    sig("damascus_coeff_count_for_byte_len", u64, u64)
    sig("damascus_layout_for_byte_len", i32, u64, P(u32), P(u64))
    sig("damascus_proof_size", sz, u64)
    sig("damascus_record_size", sz, u64, u64)
    sig("damascus_statement_size", sz, u64)
    sig("damascus_prover_footprint", u64, u64)
    sig("damascus_file_id", i32, vp, cp, sz, vp)
    sig("damascus_derive_generators", i32, vp, cp, u64, u64, vp)
    sig("damascus_commit_with_generators", i32, vp, cp, cp, u64, u64, vp)
    sig("damascus_commit", i32, vp, cp, sz, cp, vp, sz, P(sz))
    sig("damascus_ring_mul_batch", i32, vp, cp, cp, vp, u64, u64)
    sig("damascus_ring_mul_batch_device", i32, vp, vp, vp, vp, u64, u64, i32)
    sig("damascus_prover_new", i32, vp, cp, sz, cp, cp, u64, P(vp))
    sig("damascus_prover_free", None, vp)
    sig("damascus_prover_rounds_total", u32, vp)
    sig("damascus_prover_current_round", u64, vp)
    sig("damascus_prover_dimensions", None, vp, P(u64), P(u64))
    sig("damascus_prover_statement", i32, vp, vp, sz, P(sz))
    sig("damascus_prover_current_commitment", i32, vp, vp, sz, P(sz))
    sig("damascus_prover_fold_round", i32, vp, u64, vp, sz, P(sz))
    sig("damascus_prover_fold_round_timed", i32, vp, u64, vp, sz, P(sz), P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double))
    sig("damascus_prover_final_opening", i32, vp, vp)
    sig("damascus_prove", i32, vp, cp, sz, cp, cp, vp, sz, P(sz))
    sig("damascus_prove_device", i32, vp, vp, sz, cp, cp, vp, sz, P(sz))
    sig("damascus_prove_device_timed", i32, vp, vp, sz, cp, cp, vp, sz, P(sz), P(ctypes.c_double))
    sig("damascus_ctx_flush_l2", i32, vp)
    sig("damascus_verifier_new", i32, vp, cp, sz, cp, P(vp))
    sig("damascus_verifier_free", None, vp)
    sig("damascus_verifier_update_commitment", i32, vp, cp, sz)
    sig("damascus_verifier_verify_final_opening", i32, vp, cp)
    sig("damascus_verifier_round", u64, vp)
    sig("damascus_verifier_dimensions", None, vp, P(u64), P(u64))
    sig("damascus_verify", i32, vp, cp, sz, cp)
    sig("damascus_cuda_fold_batch", i32, vp, vp, vp, vp, vp, vp, sz, u64, u64)
    sig("damascus_cuda_ntt_batch", i32, vp, vp, vp, sz, vp, vp, vp, vp)
    sig("damascus_ctx_set_profiling", i32, vp, i32)
    sig("damascus_ctx_reset_stats", None, vp)
    sig("damascus_ctx_kernel_stat", i32, vp, cp, P(u64), P(ctypes.c_double), P(ctypes.c_double),
        P(ctypes.c_double))
    sig("damascus_ctx_synchronize", i32, vp)
    sig("damascus_file_id_noalloc", i32, vp, sz, vp, vp)
    sig("damascus_engine_create", i32, vp, i32, i32, P(vp))
    sig("damascus_engine_create_with_options", i32, vp, P(EngineOptions), P(vp))
    sig("damascus_engine_destroy", None, vp)
    sig("damascus_engine_submit", i32, vp, cp, sz, cp, cp, P(u64))
    sig("damascus_engine_submit_device", i32, vp, vp, sz, cp, cp, P(u64))
    sig("damascus_engine_submit_borrowed", i32, vp, vp, sz, cp, cp, P(u64))
    sig("damascus_engine_wait_any", i32, vp, P(u64), sz, P(sz))
    sig("damascus_engine_poll", i32, vp, u64, P(sz), P(ctypes.c_double))
    sig("damascus_engine_wait", i32, vp, u64, P(sz), P(ctypes.c_double))
    sig("damascus_engine_take", i32, vp, u64, vp, sz)
    sig("damascus_engine_result", i32, vp, u64, P(vp), P(sz))
    sig("damascus_engine_release", i32, vp, u64)
    sig("damascus_engine_wait_timeout", i32, vp, u64, ctypes.c_double, P(sz), P(ctypes.c_double))
    sig("damascus_engine_cancel", i32, vp, u64)
    sig("damascus_engine_set_request_timeout", i32, vp, ctypes.c_double)
    sig("damascus_engine_set_admission_batch", i32, vp, i32)
    sig("damascus_engine_health", i32, vp, P(u64), P(ctypes.c_double))
    sig("damascus_engine_drain", i32, vp)
    sig("damascus_engine_stats", i32, vp, P(u64), P(u64), P(u64), P(u64), P(u64))
    sig("damascus_engine_profile", i32, vp, P(ctypes.c_double), P(ctypes.c_double))
    sig("damascus_engine_scheduler_profile", i32, vp, P(ctypes.c_double), P(ctypes.c_double))
    sig("damascus_ctx_trace_start", i32, vp)
    sig("damascus_ctx_trace_read", i32, vp, vp, sz, P(sz), i32)
    sig("damascus_tuning_set", i32, vp, i32, u32, i32)
    sig("damascus_tuning_get", i32, vp, i32, u32, P(i32))
    sig("damascus_tuning_measure", i32, vp, i32, u32, i32, u32, i32, P(ctypes.c_double))
    sig("damascus_commit_witness", i32, vp, cp, u64, u64, cp, vp)
    sig("damascus_ctx_set_generator_cache", i32, vp, u64)
    sig("damascus_ctx_set_max_preprocess_bytes", i32, vp, u64)
    sig("damascus_ctx_max_preprocess_bytes", u64, vp)
    sig("damascus_measure_int_multiply", i32, vp, P(ctypes.c_double))
    sig("damascus_ctx_generator_cache_stats", i32, vp, P(u64), P(u64), P(u64), P(u64))
    sig("damascus_verify_service_create", i32, vp, i32, u64, P(vp))
    sig("damascus_verify_service_destroy", None, vp)
    sig("damascus_verify_service_submit", i32, vp, cp, sz, cp, P(u64))
    sig("damascus_verify_service_poll", i32, vp, u64, P(i32), P(ctypes.c_double))
    sig("damascus_verify_service_wait", i32, vp, u64, P(i32), P(ctypes.c_double))
    sig("damascus_verify_service_drain", i32, vp)
    sig("damascus_verify_service_stats", i32, vp, P(u64), P(u64), P(u64), P(u64), P(u64), P(u64))


# ------------------------------------------------------------------ encoding helpers
def fe(v: int) -> bytes:
    return int(v).to_bytes(16, "little")


def fe_vec(vals: Iterable[int]) -> bytes:
    return b"".join(int(v).to_bytes(16, "little") for v in vals)


def unfe_vec(b: bytes) -> List[int]:
    return [int.from_bytes(b[i:i + 16], "little") for i in range(0, len(b), 16)]


# ------------------------------------------------------------------ host-side API (no GPU needed)
def fp_mul(a: int, b: int) -> int:
    out = ctypes.create_string_buffer(16)
    load().damascus_fp_mul(fe(a), fe(b), out)
    return int.from_bytes(out.raw, "little")


def fp_add(a: int, b: int) -> int:
    out = ctypes.create_string_buffer(16)
    load().damascus_fp_add(fe(a), fe(b), out)
    return int.from_bytes(out.raw, "little")


def fp_sub(a: int, b: int) -> int:
    out = ctypes.create_string_buffer(16)
    load().damascus_fp_sub(fe(a), fe(b), out)
    return int.from_bytes(out.raw, "little")


def fp_inv(a: int) -> int:
    out = ctypes.create_string_buffer(16)
    load().damascus_fp_inv(fe(a), out)
    return int.from_bytes(out.raw, "little")


def fp_from_le_bytes_mod_order(b: bytes) -> int:
    out = ctypes.create_string_buffer(16)
    load().damascus_fp_from_le_bytes_mod_order(b, len(b), out)
    return int.from_bytes(out.raw, "little")


def blake3(data: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    load().damascus_blake3(data, len(data), out)
    return out.raw


def blake3_keyed(key: bytes, data: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    load().damascus_blake3_keyed(key, data, len(data), out)
    return out.raw


def transcript_challenge(epoch_seed: bytes, file_id: bytes, label: str, rnd: int,
                         c: bytes, n_c: int, l: bytes, n_l: int, r: bytes, n_r: int) -> int:
    out = ctypes.create_string_buffer(16)
    rc = load().damascus_transcript_challenge(epoch_seed, file_id, label.encode(), rnd, c, n_c, l, n_l, r, n_r,
                                              out)
    if rc:
        raise DamascusError(rc, "transcript challenge")
    return int.from_bytes(out.raw, "little")


def coeff_count_for_byte_len(n: int) -> int:
    return load().damascus_coeff_count_for_byte_len(n)


def layout_for_byte_len(n: int) -> Tuple[int, int]:
    d, dim = ctypes.c_uint32(), ctypes.c_uint64()
    rc = load().damascus_layout_for_byte_len(n, ctypes.byref(d), ctypes.byref(dim))
    if rc:
        raise DamascusError(rc, "layout")
    return d.value, dim.value


def proof_size(file_len: int) -> int:
    return load().damascus_proof_size(file_len)


def record_size(ring_len_vec: int, ring_len_poly: int) -> int:
    return load().damascus_record_size(ring_len_vec, ring_len_poly)


def statement_size(ring_len: int) -> int:
    return load().damascus_statement_size(ring_len)


def prover_footprint(file_len: int) -> int:
    return load().damascus_prover_footprint(file_len)


def depth_j(d: int, j: int) -> Tuple[int, int]:
    """(N_j, n_j) after j rounds (src/protocol/prover.rs:316-320)."""
    assert j <= d, "round index exceeds fold depth"
    dim = 1 << (d - j)
    return dim, dim


# ------------------------------------------------------------------ device API
class Context:
    """A GPU context: device, stream, twiddle/CRT tables and an HBM budget."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, tuning="auto"):
        """tuning: "auto" applies the packaged autotuner table (tuning_gb300.json) when
        present, None keeps the built-in launch shapes, a dict applies that table."""
        L = load()
        h = ctypes.c_void_p()
        rc = L.damascus_ctx_create(device, hbm_budget_bytes, ctypes.byref(h))
        if rc:
            raise DamascusError(rc, L.damascus_create_error().decode())
        self._h = h
        self._lib = L
        self.engine_waves = 0  # stage waves an Engine keeps in flight when none is given (0: the library's 16)
        if tuning is not None:
            from . import autotune
            autotune.apply(self, table=None if tuning == "auto" else tuning)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.damascus_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def last_error(self) -> str:
        return self._lib.damascus_last_error(self._h).decode()

    def check(self, rc: int, what: str = "") -> None:
        if rc:
            raise DamascusError(rc, f"{what}: {self.last_error()}")

    @property
    def budget(self) -> int:
        return self._lib.damascus_ctx_budget(self._h)

    @property
    def reserved(self) -> int:
        return self._lib.damascus_ctx_reserved(self._h)

    # -- RuntimeConfig.max_preprocess_bytes of prove / commit / engine submissions
    @property
    def max_preprocess_bytes(self) -> int:
        return self._lib.damascus_ctx_max_preprocess_bytes(self._h)

    def set_max_preprocess_bytes(self, nbytes: int) -> None:
        """Witness-expansion limit of prove, commit and engine submissions
        (src/utils/io.rs:42-49); 0 restores the reference default of 512 MiB."""
        self.check(self._lib.damascus_ctx_set_max_preprocess_bytes(self._h, nbytes), "set_max_preprocess_bytes")

    # -- provers' generator cache (damascus_ctx_set_generator_cache)
    def set_generator_cache(self, cap_bytes: int) -> None:
        """Keep provers' initial generator families and their transforms in HBM
        (a key is cached on its second sighting); 0 turns the cache off."""
        self.check(self._lib.damascus_ctx_set_generator_cache(self._h, cap_bytes), "set_generator_cache")

    def generator_cache_stats(self) -> dict:
        v = [ctypes.c_uint64() for _ in range(4)]
        self.check(self._lib.damascus_ctx_generator_cache_stats(self._h, *[ctypes.byref(x) for x in v]),
                   "generator_cache_stats")
        return dict(zip(("hits", "fills", "misses", "bytes"), (x.value for x in v)))

    # -- launch-shape tuning (damascus_tuning_*; autotune.py measures and sets them)
    def tuning_set(self, knob: int, log_ring: int, value: int) -> None:
        self.check(self._lib.damascus_tuning_set(self._h, knob, log_ring, value), "tuning_set")

    def tuning_get(self, knob: int, log_ring: int) -> int:
        v = ctypes.c_int()
        self.check(self._lib.damascus_tuning_get(self._h, knob, log_ring, ctypes.byref(v)), "tuning_get")
        return v.value

    def tuning_measure(self, knob: int, log_ring: int, value: int, count: int, reps: int = 5) -> float:
        """Mean ms per launch of the knob's kernel with `value` on synthetic device data."""
        ms = ctypes.c_double()
        self.check(self._lib.damascus_tuning_measure(self._h, knob, log_ring, value, count, reps, ctypes.byref(ms)),
                   "tuning_measure")
        return ms.value

    # -- profiling
    def measure_int_multiply(self) -> dict:
        """Measured ops/s of 32-bit multiply-add, mul.hi and 32x32->64 multiply-add."""
        v = (ctypes.c_double * 3)()
        self.check(self._lib.damascus_measure_int_multiply(self._h, v), "measure_int_multiply")
        return {"mul.lo": v[0], "mul.hi": v[1], "mad.wide": v[2]}

    def set_profiling(self, on: bool) -> None:
        self.check(self._lib.damascus_ctx_set_profiling(self._h, int(on)), "set_profiling")

    def reset_stats(self) -> None:
        self._lib.damascus_ctx_reset_stats(self._h)

    def trace_start(self) -> None:
        """Keeps every timed launch group from here on (turns profiling on)."""
        self.check(self._lib.damascus_ctx_trace_start(self._h), "trace_start")

    def trace_read(self, stop: bool = True):
        """[(kind, stream, start_ms, end_ms, algorithmic_bytes, kernels)] since
        trace_start() or the last read; stop ends the trace.  Engines add host
        rows on the same time base: ("sched_wave" | "sched_wave_deep", stream,
        start, end, requests, launches), ("wave_done", stream, t, t, requests, 0)
        and ("fiat_shamir", depth, start, end, 1, 0); per request stage, with the
        request's ticket in the fifth field, ("req_wait", depth, ready, launched,
        ticket, 0), ("req_gpu", depth, launched, landed, ticket, 0) and
        ("req_host", depth, landed, host step done, ticket, 0)."""
        ln = ctypes.c_size_t()
        rc = self._lib.damascus_ctx_trace_read(self._h, None, 0, ctypes.byref(ln), int(stop))
        if rc not in (0, ESIZE):
            self.check(rc, "trace_read")
        buf = ctypes.create_string_buffer(ln.value + 1)
        self.check(self._lib.damascus_ctx_trace_read(self._h, buf, ln.value + 1, ctypes.byref(ln), int(stop)),
                   "trace_read")
        out = []
        for line in buf.raw[:ln.value].decode().splitlines():
            k, s, t0, t1, b, n = line.split(",")
            out.append((k, int(s), float(t0), float(t1), float(b), int(n)))
        return out

    def kernel_stat(self, name: str):
        """(launches, total_ms, algorithmic_bytes, algorithmic_ops) or None."""
        n, ms, b, o = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = self._lib.damascus_ctx_kernel_stat(self._h, name.encode(), ctypes.byref(n), ctypes.byref(ms),
                                                ctypes.byref(b), ctypes.byref(o))
        if rc:
            return None
        return n.value, ms.value, b.value, o.value

    def synchronize(self) -> None:
        self.check(self._lib.damascus_ctx_synchronize(self._h), "synchronize")

    # -- commitment layer
    def file_id(self, data: bytes) -> bytes:
        out = ctypes.create_string_buffer(32)
        self.check(self._lib.damascus_file_id(self._h, data, len(data), out), "file_id")
        return out.raw

    def derive_generators(self, g_seed: bytes, vector_len: int, ring_len: int) -> bytes:
        out = ctypes.create_string_buffer(vector_len * MODULE_RANK * ring_len * 16)
        self.check(self._lib.damascus_derive_generators(self._h, g_seed, vector_len, ring_len, out),
                   "derive_generators")
        return out.raw

    def commit_with_generators(self, witness: bytes, generators: bytes, vector_len: int, ring_len: int) -> bytes:
        out = ctypes.create_string_buffer(MODULE_RANK * ring_len * 16)
        self.check(self._lib.damascus_commit_with_generators(self._h, witness, generators, vector_len, ring_len,
                                                             out), "commit_with_generators")
        return out.raw

    def commit_witness(self, witness: bytes, vector_len: int, ring_len: int,
                       seed_generators: bytes = DEFAULT_GENERATOR_SEED) -> bytes:
        """ModuleSisCommitter::new(seed).commit_with_ntt(witness) (src/commitment/sis.rs:115-131):
        generators derived on the device; an empty witness gives the zero module of ring length 1."""
        out = ctypes.create_string_buffer(MODULE_RANK * (ring_len if vector_len else 1) * 16)
        self.check(self._lib.damascus_commit_witness(self._h, witness, vector_len, ring_len, seed_generators, out),
                   "commit_witness")
        return out.raw

    def commit(self, data: bytes, seed_generators: bytes = DEFAULT_GENERATOR_SEED) -> bytes:
        d, dim = layout_for_byte_len(len(data))
        cap = statement_size(dim)
        out = ctypes.create_string_buffer(cap)
        n = ctypes.c_size_t()
        self.check(self._lib.damascus_commit(self._h, data, len(data), seed_generators, out, cap, ctypes.byref(n)),
                   "commit")
        return ctypes.string_at(out, n.value)

    def ring_mul_batch(self, a: bytes, b: bytes, n: int, count: int) -> bytes:
        out = ctypes.create_string_buffer(count * n * 16)
        self.check(self._lib.damascus_ring_mul_batch(self._h, a, b, out, n, count), "ring_mul_batch")
        return out.raw

    def ring_mul_batch_device(self, d_a: int, d_b: int, d_out: int, n: int, count: int, sync: bool = True) -> None:
        self.check(self._lib.damascus_ring_mul_batch_device(self._h, ctypes.c_void_p(d_a), ctypes.c_void_p(d_b),
                                                            ctypes.c_void_p(d_out), n, count, int(sync)),
                   "ring_mul_batch_device")

    # -- protocol
    def prove(self, data: bytes, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
              epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> bytes:
        cap = proof_size(len(data))
        out = ctypes.create_string_buffer(cap)
        n = ctypes.c_size_t()
        self.check(self._lib.damascus_prove(self._h, data, len(data), seed_generators, epoch_seed, out, cap,
                                            ctypes.byref(n)), "prove")
        return ctypes.string_at(out, n.value)

    def prove_device(self, d_file: int, length: int, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
                     epoch_seed: bytes = DEFAULT_EPOCH_SEED, out=None) -> bytes:
        cap = proof_size(length)
        if out is None:
            out = ctypes.create_string_buffer(cap)
        n = ctypes.c_size_t()
        self.check(self._lib.damascus_prove_device(self._h, ctypes.c_void_p(d_file), length, seed_generators,
                                                   epoch_seed, out, cap, ctypes.byref(n)), "prove_device")
        return ctypes.string_at(out, n.value)

    def prove_device_timed(self, d_file: int, length: int, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
                           epoch_seed: bytes = DEFAULT_EPOCH_SEED, out=None):
        """(proof bytes, device milliseconds) for a file already in device memory."""
        cap = proof_size(length)
        if out is None:
            out = ctypes.create_string_buffer(cap)
        n = ctypes.c_size_t()
        ms = ctypes.c_double()
        self.check(self._lib.damascus_prove_device_timed(self._h, ctypes.c_void_p(d_file), length, seed_generators,
                                                         epoch_seed, out, cap, ctypes.byref(n), ctypes.byref(ms)),
                   "prove_device_timed")
        return ctypes.string_at(out, n.value), ms.value

    def flush_l2(self) -> None:
        self.check(self._lib.damascus_ctx_flush_l2(self._h), "flush_l2")

    def verify(self, proof: bytes, epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> bool:
        rc = self._lib.damascus_verify(self._h, proof, len(proof), epoch_seed)
        if rc == EVERIFY or rc == EDESERIALIZE:
            return False
        self.check(rc, "verify")
        return True


class DamascusProver:
    """Mirror of DamascusProver (src/protocol/prover.rs:56-313) on the GPU."""

    def __init__(self, ctx: Context, data: bytes, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
                 epoch_seed: bytes = DEFAULT_EPOCH_SEED, max_preprocess_bytes: int = DEFAULT_MEMORY_LIMIT_BYTES):
        self._ctx = ctx
        self._lib = ctx._lib
        h = ctypes.c_void_p()
        ctx.check(self._lib.damascus_prover_new(ctx.handle, data, len(data), seed_generators, epoch_seed,
                                                max_preprocess_bytes, ctypes.byref(h)), "initialize")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.damascus_prover_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rounds_total(self) -> int:
        return self._lib.damascus_prover_rounds_total(self._h)

    def current_round(self) -> int:
        return self._lib.damascus_prover_current_round(self._h)

    def current_dimensions(self) -> Tuple[int, int]:
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._lib.damascus_prover_dimensions(self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def statement(self) -> bytes:
        n = ctypes.c_size_t()
        self._lib.damascus_prover_statement(self._h, None, 0, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value)
        self._ctx.check(self._lib.damascus_prover_statement(self._h, buf, n.value, ctypes.byref(n)), "statement")
        return buf.raw

    def current_commitment(self) -> bytes:
        n = ctypes.c_size_t()
        self._lib.damascus_prover_current_commitment(self._h, None, 0, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value)
        self._ctx.check(self._lib.damascus_prover_current_commitment(self._h, buf, n.value, ctypes.byref(n)),
                        "current_commitment")
        return buf.raw

    def fold_round(self, rnd: int) -> bytes:
        N, n = self.current_dimensions()
        cap = record_size(N, max(n // 2, 1))
        buf = ctypes.create_string_buffer(cap)
        ln = ctypes.c_size_t()
        self._ctx.check(self._lib.damascus_prover_fold_round(self._h, rnd, buf, cap, ctypes.byref(ln)),
                        f"fold_round({rnd})")
        return ctypes.string_at(buf, ln.value)

    def fold_round_timed(self, rnd: int):
        """fold_round plus the reference's RoundOutput timings
        (src/protocol/prover.rs:26-31): (record, {"vector_fold_ms",
        "poly_fold_ms", "total_round_ms"})."""
        N, n = self.current_dimensions()
        cap = record_size(N, max(n // 2, 1))
        buf = ctypes.create_string_buffer(cap)
        ln = ctypes.c_size_t()
        t = [ctypes.c_double() for _ in range(3)]
        self._ctx.check(self._lib.damascus_prover_fold_round_timed(
            self._h, rnd, buf, cap, ctypes.byref(ln), *(ctypes.byref(x) for x in t)), f"fold_round({rnd})")
        return ctypes.string_at(buf, ln.value), {"vector_fold_ms": t[0].value, "poly_fold_ms": t[1].value,
                                                 "total_round_ms": t[2].value}

    def final_opening(self) -> Optional[bytes]:
        out = ctypes.create_string_buffer(16)
        if self._lib.damascus_prover_final_opening(self._h, out):
            return None
        return out.raw


class DamascusVerifier:
    """Mirror of DamascusVerifier (src/protocol/verifier.rs:11-134) on the GPU."""

    def __init__(self, ctx: Context, statement: bytes, epoch_seed: bytes = DEFAULT_EPOCH_SEED):
        self._ctx = ctx
        self._lib = ctx._lib
        h = ctypes.c_void_p()
        ctx.check(self._lib.damascus_verifier_new(ctx.handle, statement, len(statement), epoch_seed,
                                                  ctypes.byref(h)), "verifier new")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.damascus_verifier_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update_commitment(self, record: bytes) -> int:
        """0 when the round replays; a negative DAMASCUS_E* code when rejected."""
        return self._lib.damascus_verifier_update_commitment(self._h, record, len(record))

    def verify_final_opening(self, opening: bytes) -> int:
        return self._lib.damascus_verifier_verify_final_opening(self._h, opening)

    def round(self) -> int:
        return self._lib.damascus_verifier_round(self._h)

    def current_dimensions(self) -> Tuple[int, int]:
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._lib.damascus_verifier_dimensions(self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value


class Engine:
    """Continuous-batching prover: submit files, collect proofs (identical bytes to Context.prove)."""

    def __init__(self, ctx: Context, host_threads: int = 0, max_waves: int = 0, *,
                 priority_depth: Optional[int] = None, polling: Optional[bool] = None,
                 spin_us: Optional[int] = None, admission_batch: Optional[int] = None):
        """Settings left at None keep the library's defaults (or the DM_ENGINE_*
        environment variables): see damascus_engine_options."""
        self._ctx = ctx
        self._lib = ctx._lib
        max_waves = max_waves or getattr(ctx, "engine_waves", 0)
        opt = lambda v: -1 if v is None else int(v)
        o = EngineOptions(host_threads, max_waves, opt(priority_depth), opt(polling), opt(spin_us),
                          opt(admission_batch))
        h = ctypes.c_void_p()
        ctx.check(self._lib.damascus_engine_create_with_options(ctx.handle, ctypes.byref(o), ctypes.byref(h)),
                  "engine create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.damascus_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, data: bytes, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
               epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> int:
        t = ctypes.c_uint64()
        self._ctx.check(self._lib.damascus_engine_submit(self._h, data, len(data), seed_generators, epoch_seed,
                                                         ctypes.byref(t)), "engine submit")
        return t.value

    def submit_device(self, d_file: int, length: int, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
                      epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> int:
        """Submit a file already in device memory (kept valid by the caller until done)."""
        t = ctypes.c_uint64()
        self._ctx.check(self._lib.damascus_engine_submit_device(self._h, ctypes.c_void_p(d_file), length,
                                                                seed_generators, epoch_seed, ctypes.byref(t)),
                        "engine submit_device")
        return t.value

    def submit_borrowed(self, ptr: int, length: int, seed_generators: bytes = DEFAULT_GENERATOR_SEED,
                        epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> int:
        """Submit from a raw host address that stays valid and unchanged until the
        request finishes (pinned memory: an asynchronous copy): the engine's
        host-to-device copy reads it directly, with no staging copy."""
        t = ctypes.c_uint64()
        self._ctx.check(self._lib.damascus_engine_submit_borrowed(self._h, ctypes.c_void_p(ptr), length,
                                                                  seed_generators, epoch_seed, ctypes.byref(t)),
                        "engine submit_borrowed")
        return t.value

    def submit_ptr(self, ptr: int, length: int, seed_generators: bytes, epoch_seed: bytes) -> int:
        """Submit from a raw host address (e.g. pinned memory), copied before return."""
        t = ctypes.c_uint64()
        self._ctx.check(self._lib.damascus_engine_submit(self._h, ctypes.c_char_p(ptr), length, seed_generators,
                                                         epoch_seed, ctypes.byref(t)), "engine submit")
        return t.value

    def _result(self, ticket: int, block: bool, timeout_ms: Optional[float] = None):
        n = ctypes.c_size_t()
        lat = ctypes.c_double()
        if timeout_ms is not None:
            rc = self._lib.damascus_engine_wait_timeout(self._h, ticket, float(timeout_ms), ctypes.byref(n),
                                                        ctypes.byref(lat))
            if rc == ETIMEOUT:
                return None
        else:
            fn = self._lib.damascus_engine_wait if block else self._lib.damascus_engine_poll
            rc = fn(self._h, ticket, ctypes.byref(n), ctypes.byref(lat))
        if rc == 0:
            return None
        if rc < 0:
            msg = self._ctx.last_error()
            self._lib.damascus_engine_release(self._h, ticket)  # the failure is reported once, here
            raise DamascusError(rc, f"engine request {ticket}: {msg}")
        # one copy, straight from the engine's buffer into the returned bytes
        ptr, size = ctypes.c_void_p(), ctypes.c_size_t()
        self._ctx.check(self._lib.damascus_engine_result(self._h, ticket, ctypes.byref(ptr), ctypes.byref(size)),
                        "engine result")
        proof = ctypes.string_at(ptr.value, size.value) if size.value else b""
        self._ctx.check(self._lib.damascus_engine_release(self._h, ticket), "engine release")
        return proof, lat.value

    def wait(self, ticket: int, timeout_ms: Optional[float] = None):
        """(proof bytes, latency ms) once the request finished; with timeout_ms,
        None when it has not finished by then (it keeps running)."""
        return self._result(ticket, True, timeout_ms)

    def as_completed(self, tickets):
        """Yields (ticket, proof bytes, latency ms) for every ticket, in the order
        the requests finish; a failed request raises when its turn comes."""
        pending = list(tickets)
        which = ctypes.c_size_t()
        while pending:
            arr = (ctypes.c_uint64 * len(pending))(*pending)
            self._ctx.check(self._lib.damascus_engine_wait_any(self._h, arr, len(pending), ctypes.byref(which)),
                            "engine wait_any")
            t = pending.pop(which.value)
            proof, lat = self._result(t, True)
            yield t, proof, lat

    def cancel(self, ticket: int) -> None:
        """Ends the request early (queued: at once; admitted: at its next stage
        boundary); its wait then raises ECANCELED."""
        self._ctx.check(self._lib.damascus_engine_cancel(self._h, ticket), "engine cancel")

    def set_request_timeout(self, timeout_ms: float) -> None:
        """Requests submitted from now on fail with ETIMEOUT when unfinished after
        timeout_ms (0: no limit)."""
        self._ctx.check(self._lib.damascus_engine_set_request_timeout(self._h, float(timeout_ms)),
                        "engine set_request_timeout")

    def set_admission_batch(self, requests_per_pass: int) -> None:
        """Admissions per scheduling pass while an admitted request is ready
        (default 1; 0 admits every queued request that fits before launching)."""
        self._ctx.check(self._lib.damascus_engine_set_admission_batch(self._h, int(requests_per_pass)),
                        "engine set_admission_batch")

    def health(self) -> dict:
        """Unfinished requests and milliseconds since any stage finished."""
        u, ms = ctypes.c_uint64(), ctypes.c_double()
        self._ctx.check(self._lib.damascus_engine_health(self._h, ctypes.byref(u), ctypes.byref(ms)), "engine health")
        return {"unfinished": u.value, "ms_since_progress": ms.value}

    def poll(self, ticket: int):
        """(proof bytes, latency ms), or None while running."""
        return self._result(ticket, False)

    def drain(self) -> None:
        self._ctx.check(self._lib.damascus_engine_drain(self._h), "engine drain")

    def stats(self) -> dict:
        v = [ctypes.c_uint64() for _ in range(5)]
        self._ctx.check(self._lib.damascus_engine_stats(self._h, *[ctypes.byref(x) for x in v]), "engine stats")
        out = dict(zip(("completed", "failed", "waves", "launches", "peak_reserved"), (x.value for x in v)))
        h, i = ctypes.c_double(), ctypes.c_double()
        self._ctx.check(self._lib.damascus_engine_profile(self._h, ctypes.byref(h), ctypes.byref(i)), "engine profile")
        out.update(host_stage_ms=h.value, gpu_idle_ms=i.value)
        self._ctx.check(self._lib.damascus_engine_scheduler_profile(self._h, ctypes.byref(h), ctypes.byref(i)),
                        "engine scheduler profile")
        out.update(admit_ms=h.value, launch_ms=i.value)
        return out

    def prove_batch(self, items) -> list:
        """items: iterable of (data, seed_generators, epoch_seed); returns the proofs in order."""
        tickets = [self.submit(d, s, e) for d, s, e in items]
        return [self.wait(t)[0] for t in tickets]


class VerifyService:
    """Streaming verifier: proofs submitted from any thread are verified by worker
    threads on their own streams, admitted against the context's HBM budget, with
    initial generator families shared through an HBM cache (``cache_bytes``, 0
    disables).  Each verdict equals ``Context.verify``'s on the same bytes."""

    def __init__(self, ctx: Context, workers: int = 0, cache_bytes: int = 16 << 30):
        self._ctx = ctx
        self._lib = ctx._lib
        h = ctypes.c_void_p()
        ctx.check(self._lib.damascus_verify_service_create(ctx.handle, workers, cache_bytes, ctypes.byref(h)),
                  "verify service create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.damascus_verify_service_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, proof: bytes, epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> int:
        t = ctypes.c_uint64()
        self._ctx.check(self._lib.damascus_verify_service_submit(self._h, proof, len(proof), epoch_seed,
                                                                 ctypes.byref(t)), "verify service submit")
        return t.value

    def _result(self, ticket: int, block: bool):
        v = ctypes.c_int32()
        lat = ctypes.c_double()
        fn = self._lib.damascus_verify_service_wait if block else self._lib.damascus_verify_service_poll
        rc = fn(self._h, ticket, ctypes.byref(v), ctypes.byref(lat))
        if rc == 0:
            return None
        if rc < 0:
            raise DamascusError(rc, f"verify service ticket {ticket}")
        return v.value, lat.value

    def wait(self, ticket: int):
        """(verdict code, latency ms): 0 accepts, else the code ``damascus_verify`` returns."""
        return self._result(ticket, True)

    def poll(self, ticket: int):
        """(verdict code, latency ms), or None while running."""
        return self._result(ticket, False)

    def drain(self) -> None:
        self._ctx.check(self._lib.damascus_verify_service_drain(self._h), "verify service drain")

    def stats(self) -> dict:
        v = [ctypes.c_uint64() for _ in range(6)]
        self._ctx.check(self._lib.damascus_verify_service_stats(self._h, *[ctypes.byref(x) for x in v]),
                        "verify service stats")
        return dict(zip(("completed", "accepted", "rejected", "cache_hits", "cache_misses", "peak_reserved"),
                        (x.value for x in v)))

    def verify_batch(self, proofs, epoch_seed: bytes = DEFAULT_EPOCH_SEED) -> list:
        """Verdicts as ``Context.verify`` gives them (False for a rejected or
        undecodable proof; other failures raise)."""
        tickets = [self.submit(p, epoch_seed) for p in proofs]
        out = []
        for t in tickets:
            code, _ = self.wait(t)
            if code in (EVERIFY, EDESERIALIZE):
                out.append(False)
            elif code:
                raise DamascusError(code, f"verify service ticket {t}: {self._ctx.last_error()}")
            else:
                out.append(True)
        return out


# ------------------------------------------------------------------ reference FFI drop-ins
def cuda_fold_batch(left: Sequence[int], right: Sequence[int], challenge: int) -> List[int]:
    """damascus_cuda_fold_batch with the reference's split lo/hi layout (src/utils/gpu.rs:95-138)."""
    n = len(left)
    A = ctypes.c_uint64 * n
    ll, lh = A(*[v & (2**64 - 1) for v in left]), A(*[v >> 64 for v in left])
    rl, rh = A(*[v & (2**64 - 1) for v in right]), A(*[v >> 64 for v in right])
    ol, oh = A(), A()
    rc = load().damascus_cuda_fold_batch(ll, lh, rl, rh, ol, oh, n, challenge & (2**64 - 1), challenge >> 64)
    if rc:
        raise DamascusError(rc, "cuda_fold_batch")
    return [ol[i] | (oh[i] << 64) for i in range(n)]


def cuda_ntt_batch(a: Sequence[Sequence[int]], b: Sequence[Sequence[int]], n: int) -> List[List[int]]:
    """damascus_cuda_ntt_batch (src/utils/gpu.rs:140-207): per-prime cyclic convolution of length n."""
    A = ctypes.c_uint64 * (8 * n)
    ha = A(*[v for row in a for v in row])
    hb = A(*[v for row in b for v in row])
    out = A()
    primes = (ctypes.c_uint64 * 8)(*CRT_PRIMES)
    log_n = n.bit_length() - 1
    roots = (ctypes.c_uint64 * max(1, 8 * log_n))()
    inv_sizes = (ctypes.c_uint64 * 8)()
    rc = load().damascus_cuda_ntt_batch(ha, hb, out, n, primes, roots, roots, inv_sizes)
    if rc:
        raise DamascusError(rc, "cuda_ntt_batch")
    return [[out[p * n + i] for i in range(n)] for p in range(8)]
