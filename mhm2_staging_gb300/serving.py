"""The serving form: resident contigs, requests from seed hits, continuous batching.

`Server` wraps the C ABI's mhsw_server_* calls (include/mhsw.h).  `generate_contigs` and
`generate_requests` make the seeded serving workload (csrc/gen_workloads.cpp): contigs
with lognormal(ln 2000, 1.0) lengths in [200, 200000] and reads U[100, 250] bp taken from
them with 2% divergence, each request naming the contig and position of its seed hit.
`windows` turns requests into the (read, contig window) pairs the server aligns, the
window klign cuts around a seed hit (reference src/klign.cpp:670-739) with the flank
given; tests and the benchmark use it to check the server against the oracle and the
driver's own entry point.  `run_open_loop` offers request batches at Poisson arrival
times and reports latency percentiles beside throughput.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import driver as D
from .driver import FORM_BATCHED, Pairs
from .workloads import _gen

_P = C.c_void_p


@dataclass
class Contigs:
    seq: np.ndarray  # uint8
    off: np.ndarray  # int64
    len: np.ndarray  # int32

    @property
    def n(self) -> int:
        return int(self.len.shape[0])


@dataclass
class Requests:
    seq: np.ndarray  # uint8, reads concatenated
    off: np.ndarray  # int64
    len: np.ndarray  # int32
    cid: np.ndarray  # int32 contig id
    pos: np.ndarray  # int32 seed-hit position in the contig

    @property
    def n(self) -> int:
        return int(self.len.shape[0])

    def slice(self, i: int, j: int) -> "Requests":
        return Requests(self.seq, self.off[i:j].copy(), self.len[i:j].copy(), self.cid[i:j].copy(),
                        self.pos[i:j].copy())

    def subset(self, idx) -> "Requests":
        idx = np.asarray(idx)
        return Requests(self.seq, self.off[idx].copy(), self.len[idx].copy(), self.cid[idx].copy(),
                        self.pos[idx].copy())


def _arr(ptr, dt, k):
    if k == 0:
        return np.zeros(0, dtype=dt)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (k,)).copy()


def _bind_serving(g: C.CDLL) -> None:
    if getattr(g, "_serving_bound", False):
        return
    g.mhsw_gen_contigs.restype = _P
    g.mhsw_gen_contigs.argtypes = [C.c_uint64, C.c_int64, C.c_int]
    g.mhsw_gen_requests.restype = _P
    g.mhsw_gen_requests.argtypes = [_P, _P, _P, C.c_int64, C.c_uint64, C.c_int64, C.c_int64, C.c_int]
    for f in ("contig_count", "request_count"):
        getattr(g, "mhsw_gen_" + f).restype = C.c_int64
        getattr(g, "mhsw_gen_" + f).argtypes = [_P]
    for f in ("contig_seq", "contig_off", "contig_len", "request_reads", "request_off", "request_len",
              "request_cid", "request_pos"):
        getattr(g, "mhsw_gen_" + f).restype = _P
        getattr(g, "mhsw_gen_" + f).argtypes = [_P]
    for f in ("contigs_free", "requests_free"):
        getattr(g, "mhsw_gen_" + f).restype = None
        getattr(g, "mhsw_gen_" + f).argtypes = [_P]
    g._serving_bound = True


def generate_contigs(total_bytes: int = 200 << 20, seed: int = 3, threads: int | None = None) -> Contigs:
    """Contig set of the serving workload (lengths lognormal(ln 2000, 1.0) in [200, 200000])."""
    g = _gen()
    _bind_serving(g)
    h = g.mhsw_gen_contigs(seed, total_bytes, threads or min(32, os.cpu_count() or 4))
    try:
        n = g.mhsw_gen_contig_count(h)
        off = _arr(g.mhsw_gen_contig_off(h), np.int64, n + 1)
        ln = _arr(g.mhsw_gen_contig_len(h), np.int32, n)
        seq = np.zeros(int(off[-1]) + 1, dtype=np.uint8)
        C.memmove(seq.ctypes.data, g.mhsw_gen_contig_seq(h), int(off[-1]))
    finally:
        g.mhsw_gen_contigs_free(h)
    return Contigs(seq, off[:-1].copy(), ln)


def generate_requests(contigs: Contigs, n: int, seed: int = 3, first: int = 0,
                      threads: int | None = None) -> Requests:
    """Requests [first, first + n) against `contigs` (reads U[100,250] bp, 2% divergence)."""
    g = _gen()
    _bind_serving(g)
    h = g.mhsw_gen_requests(contigs.seq.ctypes.data, contigs.off.ctypes.data, contigs.len.ctypes.data, contigs.n,
                            seed, first, n, threads or min(32, os.cpu_count() or 4))
    try:
        cnt = g.mhsw_gen_request_count(h)
        off = _arr(g.mhsw_gen_request_off(h), np.int64, cnt + 1)
        ln = _arr(g.mhsw_gen_request_len(h), np.int32, cnt)
        cid = _arr(g.mhsw_gen_request_cid(h), np.int32, cnt)
        pos = _arr(g.mhsw_gen_request_pos(h), np.int32, cnt)
        seq = np.zeros(int(off[-1]) + 1, dtype=np.uint8)
        if off[-1]:
            C.memmove(seq.ctypes.data, g.mhsw_gen_request_reads(h), int(off[-1]))
    finally:
        g.mhsw_gen_requests_free(h)
    return Requests(seq, off[:-1].copy(), ln, cid, pos)


def windows(contigs: Contigs, req: Requests, flank: int = 200) -> tuple[Pairs, np.ndarray]:
    """The (read, contig window) pairs of `req` and each window's start in its contig:
    window = [max(0, pos - flank), min(contig_len, pos + read_len + flank))."""
    cl = contigs.len[req.cid].astype(np.int64)
    ws = np.maximum(0, req.pos.astype(np.int64) - flank)
    we = np.minimum(cl, req.pos.astype(np.int64) + req.len.astype(np.int64) + flank)
    pairs = Pairs(req.seq, req.off.astype(np.int64), req.len.astype(np.int32), contigs.seq,
                  (contigs.off[req.cid] + ws).astype(np.int64), (we - ws).astype(np.int32))
    return pairs, ws


@dataclass
class Ticket:
    id: int
    n: int
    out5: np.ndarray
    win_start: np.ndarray
    keep: tuple  # request arrays referenced until completion


class Server:
    """Serving-form aligner on one device (C ABI: mhsw_server_*)."""

    def __init__(self, device: int = 0, slots: int = 3, max_pairs_per_batch: int = 65536, flank: int = 200,
                 hbm_budget: int = 0, queue_budget: int = 0, scores=(1, -3, -5, -2, -2), form: int = FORM_BATCHED):
        self._lib = D.load_library()
        cfg = D.ServerConfig(device, slots, max_pairs_per_batch, flank, hbm_budget, queue_budget, *scores, form)
        h = _P()
        err = C.create_string_buffer(512)
        rc = self._lib.mhsw_server_create(C.byref(cfg), C.byref(h), err, len(err))
        if rc != 0:
            raise RuntimeError(f"server create failed (status {rc}): {err.value.decode()}")
        self._h = h
        self.flank = flank

    def _ck(self, rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what} failed (status {rc}): {self._lib.mhsw_server_last_error(self._h).decode()}")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mhsw_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def load_contigs(self, contigs: Contigs) -> None:
        self._ck(self._lib.mhsw_server_load_contigs(self._h, contigs.seq.ctypes.data, contigs.off.ctypes.data,
                                                     contigs.len.ctypes.data, contigs.n), "load_contigs")

    def submit(self, req: Requests, wait_for_room: bool = True) -> Ticket | None:
        """Queues a request batch; returns None when the queue is full and wait_for_room
        is False."""
        n = req.n
        off = np.ascontiguousarray(req.off, dtype=np.int64)
        ln = np.ascontiguousarray(req.len, dtype=np.int32)
        cid = np.ascontiguousarray(req.cid, dtype=np.int32)
        pos = np.ascontiguousarray(req.pos, dtype=np.int32)
        out5 = np.zeros((n, 5), dtype=np.int32)
        ws = np.zeros(n, dtype=np.int64)
        rt = D.RequestsT(req.seq.ctypes.data, off.ctypes.data, ln.ctypes.data, cid.ctypes.data, pos.ctypes.data, n)
        t = C.c_uint64(0)
        rc = self._lib.mhsw_server_submit(self._h, C.byref(rt), out5.ctypes.data if n else None,
                                          ws.ctypes.data if n else None, 0 if wait_for_room else 1, C.byref(t))
        if rc == 8 and not wait_for_room:
            return None
        self._ck(rc, "submit")
        return Ticket(int(t.value), n, out5, ws, (req.seq, off, ln, cid, pos))

    def done(self, ticket: Ticket) -> bool:
        d = C.c_int(0)
        self._ck(self._lib.mhsw_server_test(self._h, ticket.id, C.byref(d)), "test")
        return bool(d.value)

    def wait(self, ticket: Ticket) -> tuple[np.ndarray, np.ndarray, tuple[float, float, float]]:
        """(out5, window starts, (submit, first dispatch, completion) seconds)."""
        times = (C.c_double * 3)()
        self._ck(self._lib.mhsw_server_wait(self._h, ticket.id, times), "wait")
        return ticket.out5, ticket.win_start, (times[0], times[1], times[2])

    def stats(self) -> dict:
        st = D.ServerStats()
        self._ck(self._lib.mhsw_server_stats_get(self._h, C.byref(st)), "stats")
        return st.as_dict()


def run_open_loop(server: Server, batches: list[Requests], rate_hz: float, seed: int = 0) -> dict:
    """Offers `batches` at Poisson arrival times of mean rate `rate_hz` (an open loop: a
    batch is submitted at its arrival time whatever is still running) and waits for all.
    Returns per-batch latency percentiles (completion minus submission, ms), the achieved
    throughput and the server's counters."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(batches))
    arrivals = np.cumsum(gaps) - gaps[0]
    tickets: list[Ticket] = []
    lat = np.zeros(len(batches))
    waits: list[threading.Thread] = []
    lock = threading.Lock()

    def waiter(k: int, t: Ticket):
        _, _, tm = server.wait(t)
        with lock:
            lat[k] = (tm[2] - tm[0]) * 1e3

    t0 = time.perf_counter()
    for k, b in enumerate(batches):
        delay = arrivals[k] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        t = server.submit(b)
        tickets.append(t)
        th = threading.Thread(target=waiter, args=(k, t))
        th.start()
        waits.append(th)
    for th in waits:
        th.join()
    wall = time.perf_counter() - t0
    pairs = sum(b.n for b in batches)
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "wall_s": wall, "pairs_per_s": pairs / wall,
            "offered_batches_per_s": rate_hz, "batches": len(batches)}
