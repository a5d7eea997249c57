"""Python mirror of the reference's GPU aligner surface, bound to libmhsw.so via ctypes.

`GPUDriver` mirrors adept_sw::GPUDriver (reference src/adept-sw/driver.hpp:37-55):
init / run_kernel_forwards / run_kernel_backwards / kernel_is_done / kernel_block /
get_aln_results, with the same argument meaning (scores passed negated, reads then
contigs) and the same error behaviour (a failed call raises RuntimeError, as the
reference's cudaErrchk throws std::runtime_error, driver.cpp:17-26).

There is no CPU fallback: if libmhsw.so is missing or no GPU is present the calls
raise.  The CPU oracle lives in oracle/ and is only used by tests and benchmarks.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

from . import build as _build

ORIENT_KLIGN = 0
ORIENT_REF_IS_A = 1
FORM_PLAIN = 0
FORM_BATCHED = 1

_P = C.c_void_p


class _AlnResults(C.Structure):
    _fields_ = [
        ("ref_begin", C.POINTER(C.c_int16)),
        ("query_begin", C.POINTER(C.c_int16)),
        ("ref_end", C.POINTER(C.c_int16)),
        ("query_end", C.POINTER(C.c_int16)),
        ("top_scores", C.POINTER(C.c_int16)),
        ("ref_begin32", C.POINTER(C.c_int32)),
        ("query_begin32", C.POINTER(C.c_int32)),
        ("ref_end32", C.POINTER(C.c_int32)),
        ("query_end32", C.POINTER(C.c_int32)),
        ("top_scores32", C.POINTER(C.c_int32)),
        ("n", C.c_int32),
        ("score2_32", C.POINTER(C.c_int32)),
        ("a_end2_32", C.POINTER(C.c_int32)),
    ]


class Timing(C.Structure):
    _fields_ = [
        ("fwd_ms", C.c_double),
        ("rev_ms", C.c_double),
        ("total_ms", C.c_double),
        ("fwd_cells", C.c_double),
        ("n_pairs", C.c_int64),
        ("n_overflow16", C.c_int64),
        ("n_rev_wide", C.c_int64),
        ("launches", C.c_int64),
        ("graph_replays", C.c_int64),
        ("cigar_ms", C.c_double),
        ("n_cigar_generic", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class CallRecord(C.Structure):
    _fields_ = [(k, C.c_uint64 if k == "seq" else (C.c_int64 if k == "n_pairs" else C.c_double))
                for k in ("seq", "n_pairs", "copy_in_start", "copy_in_end", "stream_ready", "translated",
                          "forward_done", "begin_done", "done")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [
        ("threads_per_block", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("lane_rows", C.c_int32),
        ("wide_try16", C.c_int32),
        ("last_call_tuned", C.c_int32),
        ("trials", C.c_int32),
        ("sample_pairs", C.c_int64),
        ("tunings", C.c_int64),
        ("tune_wall_ms", C.c_double),
        ("trial_ms", C.c_float * 16),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "trial_ms"}
        d["trial_ms"] = [float(x) for x in self.trial_ms[:min(self.trials, 16)]]
        return d


class Limits(C.Structure):
    _fields_ = [("max_b_len", C.c_int32), ("max_coord", C.c_int32), ("int16_ceiling", C.c_int32)]


class PairsT(C.Structure):
    _fields_ = [
        ("a_seq", _P),
        ("a_off", _P),
        ("a_len", _P),
        ("b_seq", _P),
        ("b_off", _P),
        ("b_len", _P),
        ("n", C.c_int64),
        ("max_a_len", C.c_int32),
        ("max_b_len", C.c_int32),
        ("cells", C.c_double),
        ("a_bytes", C.c_int64),
        ("b_bytes", C.c_int64),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int),
        ("slots", C.c_int),
        ("max_pairs_per_batch", C.c_int32),
        ("flank", C.c_int32),
        ("hbm_budget", C.c_size_t),
        ("queue_budget", C.c_size_t),
        ("match_score", C.c_short),
        ("mismatch_score", C.c_short),
        ("gap_opening_score", C.c_short),
        ("gap_extending_score", C.c_short),
        ("ambiguity_score", C.c_short),
        ("form", C.c_int),
    ]


class RequestsT(C.Structure):
    _fields_ = [
        ("read_seq", _P),
        ("read_off", _P),
        ("read_len", _P),
        ("contig_id", _P),
        ("contig_pos", _P),
        ("n", C.c_int32),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64),
        ("completed", C.c_int64),
        ("pairs_done", C.c_int64),
        ("cells_done", C.c_double),
        ("micro_batches", C.c_int64),
        ("queued_pairs", C.c_int64),
        ("admitted_bytes", C.c_size_t),
        ("slots", C.c_int),
        ("busy_slots", C.c_int),
        ("slot_pairs", C.c_int32),
        ("device_bytes", C.c_size_t),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol include/mhsw.h declares, with its ctypes signature.
class CandidatesT(C.Structure):
    _fields_ = [("read_seq", _P), ("read_off", _P), ("read_len", _P), ("contig_id", _P), ("pos_in_ctg", _P),
                ("pos_in_read", _P), ("strand", _P), ("n", C.c_int64), ("kmer_len", C.c_int32)]


class AlnsT(C.Structure):
    _fields_ = [("rstart", _P), ("rstop", _P), ("cstart", _P), ("cstop", _P), ("score1", _P), ("score2", _P),
                ("identity", _P), ("orient", _P), ("perfect", _P), ("cigar_slot", _P)]


SIGNATURES: dict[str, tuple] = {
    "mhsw_get_num_node_gpus": (C.c_int, [C.POINTER(C.c_int)]),
    "mhsw_get_tot_gpu_mem": (C.c_int, [C.POINTER(C.c_size_t)]),
    "mhsw_get_avail_gpu_mem_per_rank": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_size_t)]),
    "mhsw_get_device_name": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t]),
    "mhsw_initialize_gpu": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
    "mhsw_limits": (C.c_int, [C.POINTER(Limits)]),
    "mhsw_driver_create": (C.c_int, [C.POINTER(_P)]),
    "mhsw_driver_destroy": (None, [_P]),
    "mhsw_driver_last_error": (C.c_char_p, [_P]),
    "mhsw_driver_init": (
        C.c_int,
        [_P, C.c_int, C.c_int, C.c_short, C.c_short, C.c_short, C.c_short, C.c_int, C.POINTER(C.c_double)],
    ),
    "mhsw_driver_set_ambiguity": (C.c_int, [_P, C.c_short]),
    "mhsw_driver_set_orientation": (C.c_int, [_P, C.c_int]),
    "mhsw_driver_set_form": (C.c_int, [_P, C.c_int]),
    "mhsw_driver_set_int16_ceiling": (C.c_int, [_P, C.c_int]),
    "mhsw_driver_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "mhsw_driver_set_score2": (C.c_int, [_P, C.c_int]),
    "mhsw_last_score2": (C.c_int, [_P, _P, _P, C.c_int]),
    "mhsw_driver_set_cigar": (C.c_int, [_P, C.c_int]),
    "mhsw_last_cigar": (C.c_int, [_P, _P, _P, _P, _P, C.c_int64, C.POINTER(C.c_int64), C.c_int]),
    "mhsw_cigar_format": (C.c_int64, [_P, C.c_int32, C.c_char_p, C.c_int64]),
    "mhsw_run_kernel_forwards": (C.c_int, [_P, _P, _P, _P, _P, C.c_int32, C.c_uint32, C.c_uint32]),
    "mhsw_run_kernel_backwards": (C.c_int, [_P, _P, _P, _P, _P, C.c_int32, C.c_uint32, C.c_uint32]),
    "mhsw_kernel_is_done": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "mhsw_kernel_block": (C.c_int, [_P]),
    "mhsw_get_aln_results": (C.c_int, [_P, C.POINTER(_AlnResults)]),
    "mhsw_align_pairs": (C.c_int, [_P, C.POINTER(PairsT), _P, C.c_int, C.c_int]),
    "mhsw_align_pairs_async": (C.c_int, [_P, C.POINTER(PairsT), _P, C.c_int, C.c_int]),
    "mhsw_align_wait": (C.c_int, [_P]),
    "mhsw_last_timing": (C.c_int, [_P, C.POINTER(Timing)]),
    "mhsw_last_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "mhsw_call_history": (C.c_int, [_P, C.POINTER(CallRecord), C.c_int, C.POINTER(C.c_int)]),
    "mhsw_driver_fix_batch_config": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int]),
    "mhsw_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P), C.c_char_p, C.c_size_t]),
    "mhsw_server_destroy": (None, [_P]),
    "mhsw_server_last_error": (C.c_char_p, [_P]),
    "mhsw_server_load_contigs": (C.c_int, [_P, _P, _P, _P, C.c_int64]),
    "mhsw_server_submit": (C.c_int, [_P, C.POINTER(RequestsT), _P, _P, C.c_int, C.POINTER(C.c_uint64)]),
    "mhsw_server_test": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_int)]),
    "mhsw_server_wait": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_double)]),
    "mhsw_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "mhsw_forward_noalloc": (
        C.c_int,
        [C.POINTER(PairsT), C.c_short, C.c_short, C.c_short, C.c_short, C.c_short, _P, _P, C.c_char_p, C.c_size_t],
    ),
    "mhsw_align_protein": (C.c_int, [_P, C.POINTER(PairsT), _P, _P, _P, C.c_int]),
    "mhsw_contigs_create": (C.c_int, [C.c_int, _P, _P, _P, C.c_int64, C.POINTER(_P)]),
    "mhsw_contigs_destroy": (None, [_P]),
    "mhsw_klign_align": (C.c_int, [_P, _P, C.POINTER(CandidatesT), C.POINTER(AlnsT), C.POINTER(C.c_int64)]),
    "mhsw_probe_dpx_rate": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mhsw_probe_op_rate": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
}

_LIB: C.CDLL | None = None


def load_library(path: str | Path | None = None) -> C.CDLL:
    """Loads libmhsw.so (built in-tree by build.build()); raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else _build.lib_path()
    if not p.exists():
        raise RuntimeError(f"libmhsw.so not found at {p}: run mhm2_staging_gb300.build.build() first")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def _check(lib: C.CDLL, rc: int, handle=None, what: str = "") -> None:
    if rc != 0:
        msg = lib.mhsw_driver_last_error(handle).decode() if handle else ""
        raise RuntimeError(f"{what} failed (status {rc}): {msg}")


# ---- free functions (src/adept-sw/driver.hpp:25-35) --------------------------------
def get_num_node_gpus() -> int:
    lib = load_library()
    c = C.c_int(0)
    lib.mhsw_get_num_node_gpus(C.byref(c))
    return c.value


def get_tot_gpu_mem() -> int:
    lib = load_library()
    v = C.c_size_t(0)
    _check(lib, lib.mhsw_get_tot_gpu_mem(C.byref(v)), what="get_tot_gpu_mem")
    return v.value


def get_avail_gpu_mem_per_rank(tot_ranks: int, num_devices: int = 0) -> int:
    lib = load_library()
    v = C.c_size_t(0)
    _check(lib, lib.mhsw_get_avail_gpu_mem_per_rank(tot_ranks, num_devices, C.byref(v)), what="get_avail_gpu_mem")
    return v.value


def get_device_name(device_id: int) -> str:
    lib = load_library()
    buf = C.create_string_buffer(256)
    _check(lib, lib.mhsw_get_device_name(device_id, buf, 256), what="get_device_name")
    return buf.value.decode()


def initialize_gpu() -> tuple[bool, float, int, int]:
    """Returns (ok, seconds, device_count, total_mem) like initialize_gpu(double&, int&, size_t&)."""
    lib = load_library()
    t, c, m = C.c_double(0), C.c_int(0), C.c_size_t(0)
    rc = lib.mhsw_initialize_gpu(C.byref(t), C.byref(c), C.byref(m))
    return rc == 0, t.value, c.value, m.value


def probe_dpx_rate(device: int = 0) -> tuple[float, float]:
    """(packed int16 DPX add-max instructions per second, SM cycles per second) measured on the device."""
    lib = load_library()
    ops, hz = C.c_double(0), C.c_double(0)
    _check(lib, lib.mhsw_probe_dpx_rate(device, C.byref(ops), C.byref(hz)), what="probe_dpx_rate")
    return ops.value, hz.value


def probe_op_rate(op: int, device: int = 0) -> float:
    """Lane operations per second of one instruction form (see include/mhsw.h)."""
    lib = load_library()
    v = C.c_double(0)
    _check(lib, lib.mhsw_probe_op_rate(device, op, C.byref(v)), what="probe_op_rate")
    return v.value


def limits() -> Limits:
    lib = load_library()
    out = Limits()
    lib.mhsw_limits(C.byref(out))
    return out


def forward_noalloc(dev: "DevicePairs", out3_dev_ptr: int, scores=(1, -3, -5, -2, -2), stream: int = 0) -> None:
    """Forward pass (score, a_end, b_end per pair into the device buffer out3_dev_ptr,
    n x 3 int32) through mhsw_forward_noalloc, which allocates no device memory; dev
    must carry max_a_len and max_b_len.  scores = (match, mismatch, gap open, gap extend,
    ambiguity), penalties negated.  Asynchronous on `stream` (a cudaStream_t value)."""
    lib = load_library()
    pt = dev.c_struct()
    err = C.create_string_buffer(256)
    rc = lib.mhsw_forward_noalloc(C.byref(pt), *scores, _P(out3_dev_ptr), _P(stream or None), err, len(err))
    if rc != 0:
        raise RuntimeError(f"forward_noalloc failed (status {rc}): {err.value.decode()}")


@dataclass
class AlignmentResults:
    """adept_sw::AlignmentResults (driver.hpp:17-23) as numpy copies, plus int32 views."""

    ref_begin: np.ndarray
    query_begin: np.ndarray
    ref_end: np.ndarray
    query_end: np.ndarray
    top_scores: np.ndarray
    ref_begin32: np.ndarray
    query_begin32: np.ndarray
    ref_end32: np.ndarray
    query_end32: np.ndarray
    top_scores32: np.ndarray
    score2: np.ndarray | None = None  # score2 mode: SSW's second-best score
    a_end2: np.ndarray | None = None  # and its A row (the read row in klign's orientation)


def _as_bytes_list(seqs: Sequence[str | bytes]) -> list[bytes]:
    return [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]


CIGAR_OPS = "MIDNSHP=X"


@dataclass
class Cigars:
    """CIGARs of a batch in pair order: pair i has nops[i] BAM-encoded ops (length << 4 |
    op) at ops[op_off[i] : op_off[i] + nops[i]]; 0 ops: none (score 0, or a span beyond
    SSW's distance filter); -1: not computed.  mismatches as SSW's Alignment::mismatches."""
    nops: np.ndarray
    mismatches: np.ndarray
    op_off: np.ndarray
    ops: np.ndarray

    def of(self, i: int) -> np.ndarray:
        k = max(int(self.nops[i]), 0)
        return self.ops[self.op_off[i]:self.op_off[i] + k]

    def string(self, i: int) -> str:
        """SAM CIGAR text of pair i (SSW's cigar_string)."""
        return "".join(f"{int(c) >> 4}{CIGAR_OPS[int(c) & 15]}" for c in self.of(i))


class GPUDriver:
    """Mirror of adept_sw::GPUDriver (reference src/adept-sw/driver.hpp:37-55)."""

    def __init__(self) -> None:
        self._lib = load_library()
        h = _P()
        _check(self._lib, self._lib.mhsw_driver_create(C.byref(h)), what="driver create")
        self._h = h
        self._keep: list = []

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            self._lib.mhsw_driver_destroy(h)
            self._h = None

    def _ck(self, rc: int, what: str) -> None:
        _check(self._lib, rc, self._h, what)

    # GPUDriver::init (driver.cpp:198-247); returns seconds like the reference.
    def init(self, upcxx_rank_me: int, upcxx_rank_n: int, match_score: int, mismatch_score: int,
             gap_opening_score: int, gap_extending_score: int, rlen_limit: int) -> float:
        t = C.c_double(0)
        self._ck(self._lib.mhsw_driver_init(self._h, upcxx_rank_me, upcxx_rank_n, match_score, mismatch_score,
                                            gap_opening_score, gap_extending_score, rlen_limit, C.byref(t)), "init")
        return t.value

    def set_ambiguity(self, ambiguity_score: int) -> None:
        self._ck(self._lib.mhsw_driver_set_ambiguity(self._h, ambiguity_score), "set_ambiguity")

    def set_orientation(self, orientation: int) -> None:
        self._ck(self._lib.mhsw_driver_set_orientation(self._h, orientation), "set_orientation")

    def set_form(self, form: int) -> None:
        self._ck(self._lib.mhsw_driver_set_form(self._h, form), "set_form")

    def set_int16_ceiling(self, ceiling: int) -> None:
        self._ck(self._lib.mhsw_driver_set_int16_ceiling(self._h, ceiling), "set_int16_ceiling")

    def set_score2(self, on: bool) -> None:
        """Score2 mode: also compute SSW's second-best score (klign's aln.score2)."""
        self._ck(self._lib.mhsw_driver_set_score2(self._h, 1 if on else 0), "set_score2")

    def last_score2(self, n: int) -> np.ndarray:
        """n x 2 int32 (score2, its A row) of the last batch aligned in score2 mode."""
        s2 = np.zeros(n, dtype=np.int32)
        a2 = np.zeros(n, dtype=np.int32)
        self._ck(self._lib.mhsw_last_score2(self._h, s2.ctypes.data if n else None, a2.ctypes.data if n else None, 1),
                 "last_score2")
        return np.stack([s2, a2], axis=1)

    def set_cigar(self, on: bool) -> None:
        """CIGAR mode: also compute SSW's report_cigar output (klign's post-assembly SAM)."""
        self._ck(self._lib.mhsw_driver_set_cigar(self._h, 1 if on else 0), "set_cigar")

    def last_cigar(self, n: int) -> Cigars:
        """CIGARs of the last batch aligned in CIGAR mode (n pairs), in pair order."""
        nops = np.zeros(n, dtype=np.int32)
        mism = np.zeros(n, dtype=np.int32)
        off = np.zeros(n + 1, dtype=np.int64)
        total = C.c_int64(0)
        self._ck(self._lib.mhsw_last_cigar(self._h, nops.ctypes.data if n else None, mism.ctypes.data if n else None,
                                           off.ctypes.data, None, 0, C.byref(total), 1), "last_cigar")
        ops = np.zeros(max(int(total.value), 1), dtype=np.uint32)
        self._ck(self._lib.mhsw_last_cigar(self._h, None, None, None, ops.ctypes.data, ops.shape[0], C.byref(total),
                                           1), "last_cigar")
        return Cigars(nops, mism, off, ops[:int(total.value)])

    def stream(self) -> int:
        s = _P()
        self._ck(self._lib.mhsw_driver_stream(self._h, C.byref(s)), "stream")
        return s.value or 0

    def _marshal(self, reads: Sequence[str | bytes], contigs: Sequence[str | bytes]):
        rb, cb = _as_bytes_list(reads), _as_bytes_list(contigs)
        if len(rb) != len(cb):
            raise RuntimeError("reads and contigs must have the same length")
        n = len(cb)
        rbufs = [C.create_string_buffer(b, len(b) + 1) for b in rb]
        cbufs = [C.create_string_buffer(b, len(b) + 1) for b in cb]
        rp = (C.c_char_p * max(n, 1))(*[C.cast(x, C.c_char_p) for x in rbufs])
        cp = (C.c_char_p * max(n, 1))(*[C.cast(x, C.c_char_p) for x in cbufs])
        rl = (C.c_int32 * max(n, 1))(*[len(b) for b in rb])
        cl = (C.c_int32 * max(n, 1))(*[len(b) for b in cb])
        keep = (rbufs, cbufs, rp, cp, rl, cl)
        return n, keep

    # run_kernel_forwards(reads, contigs, maxReadSize, maxContigSize) (driver.cpp:281-375)
    def run_kernel_forwards(self, reads, contigs, max_read_size: int, max_contig_size: int) -> None:
        n, keep = self._marshal(reads, contigs)
        self._keep = list(keep)
        rbufs, cbufs, rp, cp, rl, cl = keep
        self._ck(self._lib.mhsw_run_kernel_forwards(self._h, C.cast(rp, _P), C.cast(rl, _P), C.cast(cp, _P),
                                                    C.cast(cl, _P), n, max_read_size, max_contig_size),
                 "run_kernel_forwards")

    # run_kernel_backwards(...) (driver.cpp:377-417)
    def run_kernel_backwards(self, reads, contigs, max_read_size: int, max_contig_size: int) -> None:
        n, keep = self._marshal(reads, contigs)
        rbufs, cbufs, rp, cp, rl, cl = keep
        self._ck(self._lib.mhsw_run_kernel_backwards(self._h, C.cast(rp, _P), C.cast(rl, _P), C.cast(cp, _P),
                                                     C.cast(cl, _P), n, max_read_size, max_contig_size),
                 "run_kernel_backwards")

    def kernel_is_done(self) -> bool:
        d = C.c_int(0)
        self._ck(self._lib.mhsw_kernel_is_done(self._h, C.byref(d)), "kernel_is_done")
        return bool(d.value)

    def kernel_block(self) -> None:
        self._ck(self._lib.mhsw_kernel_block(self._h), "kernel_block")

    def get_aln_results(self) -> AlignmentResults:
        r = _AlnResults()
        self._ck(self._lib.mhsw_get_aln_results(self._h, C.byref(r)), "get_aln_results")
        n = r.n

        def arr(ptr, dt):
            if n == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)

        return AlignmentResults(
            arr(r.ref_begin, np.int16), arr(r.query_begin, np.int16), arr(r.ref_end, np.int16),
            arr(r.query_end, np.int16), arr(r.top_scores, np.int16), arr(r.ref_begin32, np.int32),
            arr(r.query_begin32, np.int32), arr(r.ref_end32, np.int32), arr(r.query_end32, np.int32),
            arr(r.top_scores32, np.int32),
            arr(r.score2_32, np.int32) if r.score2_32 else None, arr(r.a_end2_32, np.int32) if r.a_end2_32 else None)

    # ---- batch entry point ---------------------------------------------------------
    def align_pairs(self, pairs: "Pairs", form: int = FORM_PLAIN, out: np.ndarray | None = None,
                    hints: bool = False) -> np.ndarray:
        """Aligns host-resident pairs (A = SSW ref, B = SSW query); returns n x 5 int32
        (score, a_begin, a_end, b_begin, b_end).  hints=True passes the batch's extents
        (from Pairs.extents(), computed once per batch) so the call skips its host scan."""
        n = pairs.n
        if out is None:
            out = np.zeros((n, 5), dtype=np.int32)
        pt = pairs.c_struct()
        if hints:
            pt.max_a_len, pt.max_b_len, pt.cells, pt.a_bytes, pt.b_bytes = pairs.extents()
        self._ck(self._lib.mhsw_align_pairs(self._h, C.byref(pt), out.ctypes.data_as(_P) if n else None, 1, form),
                 "align_pairs")
        return out

    def align_pairs_async(self, pairs: "Pairs", form: int = FORM_PLAIN, out: np.ndarray | None = None,
                          hints: bool = False) -> np.ndarray:
        """align_pairs enqueued without waiting (mhsw_align_pairs_async): returns the output
        array, valid after wait().  pairs and out are kept referenced until then; pinned
        host arrays let the copies overlap other work."""
        n = pairs.n
        if out is None:
            out = np.zeros((n, 5), dtype=np.int32)
        pt = pairs.c_struct()
        if hints:
            pt.max_a_len, pt.max_b_len, pt.cells, pt.a_bytes, pt.b_bytes = pairs.extents()
        # the handle keeps up to four calls in flight (this call completes the one four back
        # first): their arrays stay referenced here
        self._pending = (list(getattr(self, "_pending", None) or []) + [(pairs, out, pt)])[-5:]
        self._ck(self._lib.mhsw_align_pairs_async(self._h, C.byref(pt), out.ctypes.data_as(_P) if n else None, 1,
                                                  form), "align_pairs_async")
        return out

    def wait(self) -> None:
        """Completes the batches enqueued by align_pairs_async (mhsw_align_wait)."""
        try:
            self._ck(self._lib.mhsw_align_wait(self._h), "align_wait")
        finally:
            self._pending = None

    def align_pairs_device(self, dev: "DevicePairs", out_dev_ptr: int, form: int = FORM_PLAIN) -> None:
        """Aligns pairs already resident on the device (pointers from DevicePairs);
        results go to the device buffer out_dev_ptr (n x 5 int32)."""
        pt = dev.c_struct()
        self._ck(self._lib.mhsw_align_pairs(self._h, C.byref(pt), _P(out_dev_ptr), 0, form), "align_pairs (device)")

    def align_protein(self, pairs: "Pairs", matrix: np.ndarray, encoding: np.ndarray) -> np.ndarray:
        """Protein pairs (A = SSW ref, B = SSW query): n x 5 int32 (score, a_begin, a_end,
        b_begin, b_end) with a 24 x 24 scoring matrix and a 91-entry byte encoding."""
        n = pairs.n
        out = np.zeros((n, 5), dtype=np.int32)
        mat = np.ascontiguousarray(matrix, dtype=np.int16).reshape(-1)
        enc = np.ascontiguousarray(encoding, dtype=np.int16)
        if mat.shape[0] != 24 * 24 or enc.shape[0] != 91:
            raise RuntimeError("align_protein: a 24 x 24 matrix and a 91-entry encoding")
        pt = pairs.c_struct()
        self._ck(self._lib.mhsw_align_protein(self._h, C.byref(pt), mat.ctypes.data, enc.ctypes.data,
                                              out.ctypes.data if n else None, 1), "align_protein")
        return out

    def last_timing(self) -> dict:
        t = Timing()
        self._ck(self._lib.mhsw_last_timing(self._h, C.byref(t)), "last_timing")
        return t.as_dict()

    def fix_batch_config(self, threads_per_block: int = 0, blocks_per_sm: int = 0, lane_rows: int = 160,
                         wide_try16: bool = False) -> None:
        """Fixes the batched form's configuration (tuner off); threads_per_block=0 turns the
        tuner back on."""
        self._ck(self._lib.mhsw_driver_fix_batch_config(self._h, threads_per_block, blocks_per_sm, lane_rows,
                                                        1 if wide_try16 else 0), "fix_batch_config")

    def call_history(self, max_records: int = 64) -> list[dict]:
        """Device times of the last completed batch calls (mhsw_call_history), oldest first."""
        buf = (CallRecord * max_records)()
        k = C.c_int(0)
        self._ck(self._lib.mhsw_call_history(self._h, buf, max_records, C.byref(k)), "call_history")
        return [buf[i].as_dict() for i in range(k.value)]

    def last_tuning(self) -> dict:
        """The batched form's configuration and its last tuning (mhsw_last_tuning)."""
        t = Tuning()
        self._ck(self._lib.mhsw_last_tuning(self._h, C.byref(t)), "last_tuning")
        return t.as_dict()


@dataclass
class Pairs:
    """A batch as concatenated bytes: A = SSW ref (klign: the read), B = SSW query (contig window)."""

    a_seq: np.ndarray  # uint8
    a_off: np.ndarray  # int64
    a_len: np.ndarray  # int32
    b_seq: np.ndarray
    b_off: np.ndarray
    b_len: np.ndarray

    @property
    def n(self) -> int:
        return int(self.a_len.shape[0])

    def cells(self) -> int:
        return int((self.a_len.astype(np.int64) * self.b_len.astype(np.int64)).sum())

    def extents(self) -> tuple[int, int, float, int, int]:
        """(longest A, longest B, cells, A arena bytes, B arena bytes), cached."""
        ext = getattr(self, "_extents", None)
        if ext is None or ext[0] != self.n:
            if self.n == 0:
                vals = (0, 0, 0.0, 0, 0)
            else:
                vals = (int(self.a_len.max()), int(self.b_len.max()), float(self.cells()),
                        int((self.a_off + self.a_len).max()), int((self.b_off + self.b_len).max()))
            ext = (self.n, vals)
            object.__setattr__(self, "_extents", ext)
        return ext[1]

    def c_struct(self) -> PairsT:
        for arr, dt in ((self.a_seq, np.uint8), (self.b_seq, np.uint8), (self.a_off, np.int64),
                        (self.b_off, np.int64), (self.a_len, np.int32), (self.b_len, np.int32)):
            if arr.dtype != dt or not arr.flags.c_contiguous:
                raise RuntimeError("Pairs arrays must be contiguous with dtypes uint8/int64/int32")
        return PairsT(self.a_seq.ctypes.data, self.a_off.ctypes.data, self.a_len.ctypes.data,
                      self.b_seq.ctypes.data, self.b_off.ctypes.data, self.b_len.ctypes.data, self.n, 0, 0, 0.0, 0, 0)

    def write_file(self, path) -> None:
        """The batch as a pair file (little-endian int64 n, A bytes, B bytes; the two byte
        arenas; int64 A and B offsets; int32 A and B lengths), the input of the C++
        drop-in block benchmark (klign_block_bench)."""
        with open(path, "wb") as f:
            f.write(np.array([self.n, self.a_seq.nbytes, self.b_seq.nbytes], dtype="<i8").tobytes())
            for arr, dt in ((self.a_seq, "u1"), (self.b_seq, "u1"), (self.a_off, "<i8"), (self.b_off, "<i8"),
                            (self.a_len, "<i4"), (self.b_len, "<i4")):
                f.write(np.ascontiguousarray(arr, dtype=dt).tobytes())

    def a(self, i: int) -> bytes:
        o = int(self.a_off[i])
        return self.a_seq[o:o + int(self.a_len[i])].tobytes()

    def b(self, i: int) -> bytes:
        o = int(self.b_off[i])
        return self.b_seq[o:o + int(self.b_len[i])].tobytes()

    def slice(self, lo: int, hi: int) -> "Pairs":
        """Pairs [lo, hi) as a compact batch (offsets re-based)."""
        hi = min(hi, self.n)
        if hi <= lo:
            return Pairs.from_lists([], [])

        def part(seq, off, ln):
            o, l = off[lo:hi], ln[lo:hi]
            s0 = int(o.min())
            s1 = int((o + l).max())
            return np.append(seq[s0:s1], np.uint8(0)), (o - s0).astype(np.int64), l.copy()

        a_seq, a_off, a_len = part(self.a_seq, self.a_off, self.a_len)
        b_seq, b_off, b_len = part(self.b_seq, self.b_off, self.b_len)
        return Pairs(a_seq, a_off, a_len, b_seq, b_off, b_len)

    def subset(self, idx) -> "Pairs":
        return Pairs.from_lists([self.a(int(i)) for i in idx], [self.b(int(i)) for i in idx])

    @staticmethod
    def from_lists(a: Sequence[str | bytes], b: Sequence[str | bytes]) -> "Pairs":
        ab, bb = _as_bytes_list(a), _as_bytes_list(b)
        if len(ab) != len(bb):
            raise ValueError("a and b must have the same length")

        def pack(xs):
            lens = np.array([len(x) for x in xs], dtype=np.int32)
            offs = np.zeros(len(xs), dtype=np.int64)
            if len(xs) > 1:
                offs[1:] = np.cumsum(lens[:-1], dtype=np.int64)
            buf = np.frombuffer(b"".join(xs) + b"\0", dtype=np.uint8).copy()
            return buf, offs, lens

        a_seq, a_off, a_len = pack(ab)
        b_seq, b_off, b_len = pack(bb)
        return Pairs(a_seq, a_off, a_len, b_seq, b_off, b_len)


@dataclass
class DevicePairs:
    """Device pointers of a resident batch (e.g. torch tensors' data_ptr())."""

    a_seq: int
    a_off: int
    a_len: int
    b_seq: int
    b_off: int
    b_len: int
    n: int
    max_a_len: int = 0
    max_b_len: int = 0
    cells: float = 0.0
    a_bytes: int = 0
    b_bytes: int = 0

    def c_struct(self) -> PairsT:
        return PairsT(self.a_seq, self.a_off, self.a_len, self.b_seq, self.b_off, self.b_len, self.n,
                      self.max_a_len, self.max_b_len, self.cells, self.a_bytes, self.b_bytes)
