"""CPU oracle for the Damascus Fold path -- TEST INFRASTRUCTURE ONLY.

A plain-C restatement of the reference crate (damascus-core) compiled with gcc
into ``oracle/_build/libdamascus_oracle.so`` and driven through ctypes.  Only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / reference
leg of ``bench.py`` use it, and only as the checker or the timed CPU baseline;
the shipped library never calls it.

Parity status: pinned on the reference's known-answer and property tests and on
the published BLAKE3 digest of the empty input; BLAKE3 trees, transcripts,
commitments and records are "parity unpinned" beyond self-consistency, since
the reference (Rust) cannot be built here and ships no golden vectors.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB_PATH = BUILD_DIR / "libdamascus_oracle.so"
SOURCES = [ORACLE_DIR / "damascus_oracle.c"]

Q = (1 << 112) - 75
CRT_PRIMES = [3892314113, 2281701377, 2013265921, 2885681153,
              2483027969, 1811939329, 469762049, 4194304001]


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (no -march flags: builds on x86_64 and aarch64)."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    newest = max(s.stat().st_mtime for s in SOURCES + [ORACLE_DIR / "damascus_oracle.h"])
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= newest:
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-pthread", "-Wall",
           "-o", str(tmp)] + [str(s) for s in SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        c_u8p = ctypes.c_char_p
        sz = ctypes.c_size_t
        u64 = ctypes.c_uint64
        vp = ctypes.c_void_p
        L.orc_prover_new.restype = vp
        L.orc_prover_new.argtypes = [c_u8p, sz, c_u8p, c_u8p, u64, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int)]
        L.orc_prover_free.argtypes = [vp]
        L.orc_prover_rounds_total.argtypes = [vp]
        L.orc_prover_rounds_total.restype = ctypes.c_uint32
        L.orc_prover_statement.argtypes = [vp, vp, sz]
        L.orc_prover_statement.restype = sz
        L.orc_prover_fold_round.argtypes = [vp, u64, vp, sz, ctypes.POINTER(sz)]
        L.orc_prover_final_opening.argtypes = [vp, vp]
        L.orc_prover_dims.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.orc_prover_current_commitment.argtypes = [vp, vp]
        L.orc_prover_state.argtypes = [vp, vp, vp]
        L.orc_verifier_new.restype = vp
        L.orc_verifier_new.argtypes = [c_u8p, sz, c_u8p, ctypes.POINTER(ctypes.c_int)]
        L.orc_verifier_clone.restype = vp
        L.orc_verifier_clone.argtypes = [vp]
        L.orc_verifier_free.argtypes = [vp]
        L.orc_verifier_update.argtypes = [vp, c_u8p, sz]
        L.orc_verifier_final.argtypes = [vp, c_u8p]
        L.orc_verifier_dims.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.orc_verify.argtypes = [c_u8p, sz, c_u8p]
        L.orc_prove.argtypes = [c_u8p, sz, c_u8p, c_u8p, ctypes.c_int, ctypes.c_int, vp, sz,
                                ctypes.POINTER(sz)]
        L.orc_proof_size_for_depth.argtypes = [ctypes.c_uint32]
        L.orc_proof_size_for_depth.restype = sz
        L.orc_record_size.argtypes = [u64, u64]
        L.orc_record_size.restype = sz
        L.orc_coeff_count_for_byte_len.argtypes = [u64]
        L.orc_coeff_count_for_byte_len.restype = u64
        L.orc_layout_for_byte_len.argtypes = [u64, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(u64)]
        L.orc_expand_file.argtypes = [c_u8p, sz, u64, vp, ctypes.POINTER(ctypes.c_uint32), vp, sz]
        L.orc_derive_generators.argtypes = [c_u8p, sz, sz, vp]
        L.orc_derive_subseed.argtypes = [c_u8p, c_u8p, sz, vp]
        L.orc_commit_with_generators.argtypes = [c_u8p, c_u8p, sz, sz, ctypes.c_int, ctypes.c_int, vp]
        L.orc_negacyclic_multiply.argtypes = [c_u8p, c_u8p, sz, vp]
        L.orc_naive_negacyclic.argtypes = [c_u8p, c_u8p, sz, vp]
        L.orc_convolution.argtypes = [c_u8p, sz, c_u8p, sz, vp]
        L.orc_mul_by_x.argtypes = [c_u8p, sz, vp]
        L.orc_ntt_roundtrip.argtypes = [vp, sz, u64]
        L.orc_forward_ntt.argtypes = [vp, sz, u64]
        L.orc_inverse_ntt.argtypes = [vp, sz, u64]
        L.orc_blake3_hash.argtypes = [c_u8p, sz, vp]
        L.orc_blake3_hash_recursive.argtypes = [c_u8p, sz, vp]
        L.orc_blake3_keyed_hash.argtypes = [c_u8p, c_u8p, sz, vp]
        L.orc_challenge.argtypes = [c_u8p, c_u8p, c_u8p, u64, c_u8p, sz, c_u8p, sz, c_u8p, sz, vp]
        for fn in ("orc_fp_add", "orc_fp_sub", "orc_fp_mul"):
            getattr(L, fn).argtypes = [c_u8p, c_u8p, vp]
        L.orc_fp_inv.argtypes = [c_u8p, vp]
        L.orc_fp_from_le_bytes_mod_order.argtypes = [c_u8p, sz, vp]
        _lib = L
    return _lib


# ---------------------------------------------------------------- helpers
def fe(v: int) -> bytes:
    return int(v).to_bytes(16, "little")


def fe_vec(vals) -> bytes:
    return b"".join(int(v).to_bytes(16, "little") for v in vals)


def unfe_vec(b: bytes):
    return [int.from_bytes(b[i:i + 16], "little") for i in range(0, len(b), 16)]


def fp_mul(a: int, b: int) -> int:
    out = ctypes.create_string_buffer(16)
    lib().orc_fp_mul(fe(a), fe(b), out)
    return int.from_bytes(out.raw, "little")


def fp_add(a: int, b: int) -> int:
    out = ctypes.create_string_buffer(16)
    lib().orc_fp_add(fe(a), fe(b), out)
    return int.from_bytes(out.raw, "little")


def fp_inv(a: int) -> int:
    out = ctypes.create_string_buffer(16)
    lib().orc_fp_inv(fe(a), out)
    return int.from_bytes(out.raw, "little")


def fp_from_le_bytes_mod_order(b: bytes) -> int:
    out = ctypes.create_string_buffer(16)
    lib().orc_fp_from_le_bytes_mod_order(b, len(b), out)
    return int.from_bytes(out.raw, "little")


def blake3(data: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    lib().orc_blake3_hash(data, len(data), out)
    return out.raw


def blake3_recursive(data: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    lib().orc_blake3_hash_recursive(data, len(data), out)
    return out.raw


def blake3_keyed(key: bytes, data: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    lib().orc_blake3_keyed_hash(key, data, len(data), out)
    return out.raw


def negacyclic_multiply(a, b, naive: bool = False):
    n = len(a)
    out = ctypes.create_string_buffer(16 * n)
    if naive:
        lib().orc_naive_negacyclic(fe_vec(a), fe_vec(b), n, out)
    else:
        rc = lib().orc_negacyclic_multiply(fe_vec(a), fe_vec(b), n, out)
        assert rc == 0
    return unfe_vec(out.raw)


def negacyclic_multiply_bytes(a: bytes, b: bytes, n: int) -> bytes:
    out = ctypes.create_string_buffer(16 * n)
    rc = lib().orc_negacyclic_multiply(a, b, n, out)
    assert rc == 0
    return out.raw


def layout_for_byte_len(byte_len: int):
    d = ctypes.c_uint32()
    dim = ctypes.c_uint64()
    rc = lib().orc_layout_for_byte_len(byte_len, ctypes.byref(d), ctypes.byref(dim))
    assert rc == 0
    return d.value, dim.value


def expand_file(data: bytes, max_preprocess: int = (1 << 64) - 1):
    d, dim = layout_for_byte_len(len(data))
    fid = ctypes.create_string_buffer(32)
    dd = ctypes.c_uint32()
    w = ctypes.create_string_buffer(dim * dim * 16)
    rc = lib().orc_expand_file(data, len(data), max_preprocess, fid, ctypes.byref(dd), w, dim * dim * 16)
    if rc:
        raise ValueError(f"expand_file failed rc={rc}")
    return fid.raw, dd.value, w.raw


def derive_subseed(seed: bytes, label: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    lib().orc_derive_subseed(seed, label, len(label), out)
    return out.raw


def derive_generators(g_seed: bytes, vector_len: int, ring_len: int) -> bytes:
    out = ctypes.create_string_buffer(vector_len * 8 * ring_len * 16)
    lib().orc_derive_generators(g_seed, vector_len, ring_len, out)
    return out.raw


def commit_with_generators(witness: bytes, g: bytes, vector_len: int, ring_len: int,
                           use_ntt: bool = True, threads: int = 1) -> bytes:
    out = ctypes.create_string_buffer(8 * ring_len * 16)
    rc = lib().orc_commit_with_generators(witness, g, vector_len, ring_len, int(use_ntt), threads, out)
    assert rc == 0
    return out.raw


def challenge(epoch_seed: bytes, file_id: bytes, label: bytes, rnd: int,
              c: bytes, n_c: int, l: bytes, n_l: int, r: bytes, n_r: int) -> int:
    out = ctypes.create_string_buffer(16)
    lib().orc_challenge(epoch_seed, file_id, label, rnd, c, n_c, l, n_l, r, n_r, out)
    return int.from_bytes(out.raw, "little")


def proof_size_for_depth(d: int) -> int:
    return lib().orc_proof_size_for_depth(d)


def prove(data: bytes, seed_generators: bytes, epoch_seed: bytes, use_ntt: bool = False,
          threads: int = 0) -> bytes:
    """Full prove; returns bincode((Statement, Vec<RoundRecord>, Fp)).

    ``use_ntt=False`` takes the reference's naive product (identical results,
    faster for small rings); ``threads=0`` uses every host core.
    """
    if threads <= 0:
        threads = os.cpu_count() or 1
    d, _ = layout_for_byte_len(len(data))
    cap = proof_size_for_depth(d)
    out = ctypes.create_string_buffer(cap)
    n = ctypes.c_size_t()
    rc = lib().orc_prove(data, len(data), seed_generators, epoch_seed, int(use_ntt), threads, out, cap,
                         ctypes.byref(n))
    if rc:
        raise RuntimeError(f"oracle prove failed rc={rc}")
    return out.raw[:n.value]


def verify(proof: bytes, epoch_seed: bytes) -> int:
    return lib().orc_verify(proof, len(proof), epoch_seed)


class Prover:
    """Round-by-round oracle prover mirroring DamascusProver (prover.rs:56-313)."""

    def __init__(self, data: bytes, seed_generators: bytes, epoch_seed: bytes,
                 max_preprocess: int = (1 << 64) - 1, use_ntt: bool = False, threads: int = 0):
        if threads <= 0:
            threads = os.cpu_count() or 1
        err = ctypes.c_int()
        self._h = lib().orc_prover_new(data, len(data), seed_generators, epoch_seed, max_preprocess,
                                       int(use_ntt), threads, ctypes.byref(err))
        if not self._h:
            raise ValueError(f"oracle prover init failed rc={err.value}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_prover_free(h)
            self._h = None

    @property
    def rounds_total(self) -> int:
        return lib().orc_prover_rounds_total(self._h)

    def dims(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        lib().orc_prover_dims(self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def statement(self) -> bytes:
        need = lib().orc_prover_statement(self._h, None, 0)
        buf = ctypes.create_string_buffer(need)
        lib().orc_prover_statement(self._h, buf, need)
        return buf.raw

    def current_commitment(self) -> bytes:
        _, n = self.dims()
        buf = ctypes.create_string_buffer(8 * n * 16)
        lib().orc_prover_current_commitment(self._h, buf)
        return buf.raw

    def state(self):
        N, n = self.dims()
        w = ctypes.create_string_buffer(N * n * 16)
        g = ctypes.create_string_buffer(N * 8 * n * 16)
        lib().orc_prover_state(self._h, w, g)
        return w.raw, g.raw

    def fold_round(self, rnd: int) -> bytes:
        N, n = self.dims()
        cap = lib().orc_record_size(N, max(n // 2, 1))
        buf = ctypes.create_string_buffer(cap)
        ln = ctypes.c_size_t()
        rc = lib().orc_prover_fold_round(self._h, rnd, buf, cap, ctypes.byref(ln))
        if rc:
            raise RuntimeError(f"oracle fold_round failed rc={rc}")
        return buf.raw[:ln.value]

    def final_opening(self):
        out = ctypes.create_string_buffer(16)
        if lib().orc_prover_final_opening(self._h, out):
            return None
        return out.raw


class Verifier:
    """Round-by-round oracle verifier mirroring DamascusVerifier (verifier.rs:11-134)."""

    def __init__(self, statement: bytes, epoch_seed: bytes, _handle=None):
        if _handle is not None:
            self._h = _handle
            return
        err = ctypes.c_int()
        self._h = lib().orc_verifier_new(statement, len(statement), epoch_seed, ctypes.byref(err))
        if not self._h:
            raise ValueError(f"oracle verifier init failed rc={err.value}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_verifier_free(h)
            self._h = None

    def clone(self) -> "Verifier":
        return Verifier(b"", b"", _handle=lib().orc_verifier_clone(self._h))

    def dims(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        lib().orc_verifier_dims(self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def update(self, record: bytes) -> int:
        return lib().orc_verifier_update(self._h, record, len(record))

    def final(self, opening: bytes) -> int:
        return lib().orc_verifier_final(self._h, opening)
