"""Loader for the CPU oracles -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module,
to check results and as the timed CPU baseline.  The product path (libmhsw.so and mhm2_staging_gb300) never imports it.

  liboracle.so   C restatement of the reference SSW result contract (sw_oracle.c);
                 pinned against the reference's own SSW and test/ssw-test.cpp's
                 known answers (tests/golden/).
  libssw_ref.so  the reference SSW itself (src/ssw/ssw.cpp + ssw_core.cpp), compiled by
                 oracle/Makefile: on x86_64 from the reference checkout with SSE2; on
                 aarch64 from the unmodified sources staged in oracle/_ref/ssw_src/
                 (git-ignored) through oracle/sse2_shim/ (NEON).
  libssw_ref_shim.so  (x86_64) the same sources through the shim's portable vector form,
                 checked bit for bit against the SSE2 build.

The reference checkout is found through the MHSW_REFERENCE environment variable.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liboracle.so"
GEN_SO = HERE / "_build" / "libmhsw_gen.so"
REF_SO = HERE / "_ref" / "libssw_ref.so"
REF_SHIM_SO = HERE / "_ref" / "libssw_ref_shim.so"
STAGED_SSW = HERE / "_ref" / "ssw_src"
REFERENCE_ROOT = Path(os.environ.get("MHSW_REFERENCE", "/root/reference"))

_P = C.c_void_p
_ORACLE = None
_REF: dict = {}


def build(with_reference: bool | None = None) -> None:
    """Builds liboracle.so.  Where the reference checkout is present (the x86_64 build
    container): libssw_ref.so (SSE2), its shim twin libssw_ref_shim.so, the staged copy of
    the SSW sources for the aarch64 host, and the ADEPT comparator cubin.  On aarch64 with
    the staged sources: libssw_ref.so through the NEON shim."""
    subprocess.run(["make", "-s", "-C", str(HERE), "_build/liboracle.so", "_build/libmhsw_gen.so"], check=True)
    if with_reference is False:
        return
    ref = f"REF={REFERENCE_ROOT}"
    if (REFERENCE_ROOT / "src" / "ssw" / "ssw.cpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "stage", ref], check=True)
        if platform.machine() == "x86_64":
            subprocess.run(["make", "-s", "-C", str(HERE), "ref", "ref-shim", ref], check=True)
    if platform.machine() != "x86_64" and (STAGED_SSW / "ssw_core.cpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)
    if (REFERENCE_ROOT / "src" / "adept-sw" / "kernel.cpp").exists() and shutil.which("nvcc"):
        subprocess.run(["make", "-s", "-C", str(HERE), "adept", ref], check=True)


def _bind(lib: C.CDLL, name: str) -> None:
    fn = getattr(lib, name)
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, _P, _P, C.c_char_p, _P, _P, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                   C.c_int, _P]


def _bind_cigar(lib: C.CDLL, name: str) -> None:
    fn = getattr(lib, name)
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, _P, _P, C.c_char_p, _P, _P, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                   C.c_int, _P, _P, _P, C.c_int]


def oracle_lib() -> C.CDLL:
    global _ORACLE
    if _ORACLE is None:
        if not ORACLE_SO.exists():
            build(with_reference=False)
        lib = C.CDLL(str(ORACLE_SO))
        _bind(lib, "sw_oracle_align_batch")
        _bind(lib, "sw_oracle_align_batch7")
        _bind(lib, "sw_oracle_align_batch_lanes")
        _bind_cigar(lib, "sw_oracle_cigar_batch")
        lib.sw_oracle_protein_batch.restype = C.c_int
        lib.sw_oracle_protein_batch.argtypes = [C.c_char_p, _P, _P, C.c_char_p, _P, _P, C.c_int64, _P, _P, C.c_int,
                                                C.c_int, C.c_int, _P]
        lib.sw_oracle_align_codes.restype = C.c_int64
        lib.sw_oracle_align_codes.argtypes = [_P, C.c_int, _P, C.c_int, _P, C.c_int, C.c_int, _P]
        _ORACLE = lib
    return _ORACLE


def reference_available() -> bool:
    return REF_SO.exists()


def reference_build_kind() -> str:
    """How libssw_ref.so was built here: "sse2" (x86_64, the reference's own vector code)
    or "sse2-shim-neon" (aarch64, through oracle/sse2_shim)."""
    return "sse2" if platform.machine() == "x86_64" else "sse2-shim-neon"


def ref_lib(path: Path | None = None) -> C.CDLL:
    path = Path(path or REF_SO)
    if path not in _REF:
        if not path.exists():
            raise RuntimeError(f"reference SSW not built ({path})")
        lib = C.CDLL(str(path))
        _bind(lib, "ssw_ref_align_batch")
        _bind(lib, "ssw_ref_align_batch7")
        _bind_cigar(lib, "ssw_ref_cigar_batch")
        lib.ssw_ref_protein_batch.restype = C.c_int
        lib.ssw_ref_protein_batch.argtypes = [C.c_char_p, _P, _P, C.c_char_p, _P, _P, C.c_int64, _P, _P, C.c_int,
                                              C.c_int, _P]
        lib.ssw_ref_align.restype = C.c_int
        lib.ssw_ref_align.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int, C.c_int, _P]
        _REF[path] = lib
    return _REF[path]


def _run(lib, fn, pairs, scoring, threads, width=5):
    n = pairs.n
    out = np.zeros((n, width), dtype=np.int32)
    if n == 0:
        return out
    m, x, go, ge, amb = scoring
    rc = getattr(lib, fn)(pairs.a_seq.ctypes.data_as(C.c_char_p), pairs.a_off.ctypes.data, pairs.a_len.ctypes.data,
                          pairs.b_seq.ctypes.data_as(C.c_char_p), pairs.b_off.ctypes.data, pairs.b_len.ctypes.data,
                          n, m, x, go, ge, amb, threads, out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"{fn} failed")
    return out


def align_batch(pairs, scoring=(1, 3, 5, 2, 2), threads: int | None = None, score2: bool = False) -> np.ndarray:
    """Oracle results n x 5 (score, a_begin, a_end, b_begin, b_end), or n x 7 with score2
    and a_end2 (SSW's second-best score, maskLen = max(len(A)/2, 15)); scoring =
    (match, mismatch, gap_open, gap_extend, ambiguity) as positive magnitudes."""
    if score2:
        return _run(oracle_lib(), "sw_oracle_align_batch7", pairs, scoring, threads or (os.cpu_count() or 1), 7)
    return _run(oracle_lib(), "sw_oracle_align_batch", pairs, scoring, threads or (os.cpu_count() or 1))


def align_batch_lanes(pairs, scoring=(1, 3, 5, 2, 2), threads: int | None = None) -> np.ndarray:
    """align_batch's results (n x 5) from the across-pairs vectorised restatement
    (sw_lanes.cpp): eight pairs per 128-bit vector, the CPU baseline's implementation."""
    return _run(oracle_lib(), "sw_oracle_align_batch_lanes", pairs, scoring, threads or (os.cpu_count() or 1))


def ref_align_batch(pairs, scoring=(1, 3, 5, 2, 2), threads: int | None = None, score2: bool = False,
                    lib: Path | None = None) -> np.ndarray:
    """The reference SSW, called as klign calls it (src/klign.cpp:257); n x 7 with
    sw_score_next_best and ref_end_next_best when score2.  lib selects another build of
    it (REF_SHIM_SO)."""
    if score2:
        return _run(ref_lib(lib), "ssw_ref_align_batch7", pairs, scoring, threads or (os.cpu_count() or 1), 7)
    return _run(ref_lib(lib), "ssw_ref_align_batch", pairs, scoring, threads or (os.cpu_count() or 1))


def _run_cigar(lib, fn, pairs, scoring, threads, ops_cap):
    n = pairs.n
    out = np.zeros((n, 6), dtype=np.int32)
    ops = np.zeros((n, ops_cap), dtype=np.uint32)
    nops = np.zeros(n, dtype=np.int32)
    if n == 0:
        return out, ops, nops
    m, x, go, ge, amb = scoring
    rc = getattr(lib, fn)(pairs.a_seq.ctypes.data_as(C.c_char_p), pairs.a_off.ctypes.data, pairs.a_len.ctypes.data,
                          pairs.b_seq.ctypes.data_as(C.c_char_p), pairs.b_off.ctypes.data, pairs.b_len.ctypes.data,
                          n, m, x, go, ge, amb, threads, out.ctypes.data, ops.ctypes.data, nops.ctypes.data, ops_cap)
    if rc != 0:
        raise RuntimeError(f"{fn} failed")
    return out, ops, nops


def cigar_batch(pairs, scoring=(1, 3, 5, 2, 2), threads: int | None = None, ops_cap: int = 256):
    """Oracle alignments with CIGARs (SSW's Filter(true, true, 0, 32767)): returns
    (out n x 6 = score, a_begin, a_end, b_begin, b_end, mismatches; ops n x ops_cap
    BAM-encoded ops; nops n = op count, 0 for none, -1 when over ops_cap)."""
    return _run_cigar(oracle_lib(), "sw_oracle_cigar_batch", pairs, scoring, threads or (os.cpu_count() or 1), ops_cap)


def ref_cigar_batch(pairs, scoring=(1, 3, 5, 2, 2), threads: int | None = None, ops_cap: int = 256):
    """The reference SSW with report_cigar, same layout as cigar_batch."""
    return _run_cigar(ref_lib(), "ssw_ref_cigar_batch", pairs, scoring, threads or (os.cpu_count() or 1), ops_cap)


PROTEIN_LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*"


def protein_encoding() -> np.ndarray:
    """A 91-entry ASCII encoding (the form the reference's protein kernels take): the 24
    letters above to 0..23, every other byte to 22 ('X')."""
    enc = np.full(91, PROTEIN_LETTERS.index("X"), dtype=np.int16)
    for k, ch in enumerate(PROTEIN_LETTERS):
        enc[ord(ch)] = k
    return enc


def protein_batch(pairs, mat24: np.ndarray, enc91: np.ndarray, gap_open: int, gap_extend: int,
                  threads: int | None = None) -> np.ndarray:
    """Oracle protein alignments n x 5 (bytes must be below 91)."""
    n = pairs.n
    out = np.zeros((n, 5), dtype=np.int32)
    if n == 0:
        return out
    mat = np.ascontiguousarray(mat24, dtype=np.int16)
    enc = np.ascontiguousarray(enc91, dtype=np.int16)
    oracle_lib().sw_oracle_protein_batch(pairs.a_seq.ctypes.data_as(C.c_char_p), pairs.a_off.ctypes.data,
                                         pairs.a_len.ctypes.data, pairs.b_seq.ctypes.data_as(C.c_char_p),
                                         pairs.b_off.ctypes.data, pairs.b_len.ctypes.data, n, mat.ctypes.data,
                                         enc.ctypes.data, gap_open, gap_extend, threads or (os.cpu_count() or 1),
                                         out.ctypes.data)
    return out


def ref_protein_batch(pairs, mat24: np.ndarray, enc91: np.ndarray, gap_open: int, gap_extend: int) -> np.ndarray:
    """The reference SSW with the same matrix and encoding (scores must fit int8)."""
    n = pairs.n
    out = np.zeros((n, 5), dtype=np.int32)
    if n == 0:
        return out
    mat = np.ascontiguousarray(mat24, dtype=np.int8)
    trans = np.zeros(128, dtype=np.int8)
    trans[:91] = enc91
    ref_lib().ssw_ref_protein_batch(pairs.a_seq.ctypes.data_as(C.c_char_p), pairs.a_off.ctypes.data,
                                    pairs.a_len.ctypes.data, pairs.b_seq.ctypes.data_as(C.c_char_p),
                                    pairs.b_off.ctypes.data, pairs.b_len.ctypes.data, n, mat.ctypes.data,
                                    trans.ctypes.data, gap_open, gap_extend, out.ctypes.data)
    return out


CIGAR_OPS = "MIDNSHP=X"


def cigar_string(ops_row, n: int) -> str:
    """SAM text of n BAM-encoded ops."""
    return "".join(f"{int(c) >> 4}{CIGAR_OPS[int(c) & 15]}" for c in ops_row[:n])


def ref_align_one(query: bytes, ref: bytes, scoring=(1, 3, 5, 2, 2), mask_len: int = -1) -> list[int]:
    """One reference SSW call: returns [score, ref_begin, ref_end, query_begin, query_end,
    score2, ref_end2, mismatches]."""
    out = (C.c_int32 * 8)()
    m, x, go, ge, amb = scoring
    ref_lib().ssw_ref_align(query, len(query), ref, len(ref), m, x, go, ge, amb, mask_len, C.cast(out, _P))
    return list(out)
