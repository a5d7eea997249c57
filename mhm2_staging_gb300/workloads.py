"""Seeded synthetic workloads (the five measured configurations of the alignment path).

Thin ctypes wrapper over libmhsw_gen.so (csrc/gen_workloads.cpp).  Pairs come back in
klign's orientation: A = the read (SSW ref), B = the reference/contig window (SSW query).

  config 0: 10,000 pairs; 150 bp reads; 300 bp refs (2% subs, 0.5% indels, flank)
  config 1: 1,000,000 pairs; reads U[100,250]; refs L+U[50,774] <= 1024; 0.1% N; 30% unrelated
  config 2: 4,000,000 pairs; 60% 150 / 30% 250 / 10% U[50,150] bp; refs lognormal(ln 400, 0.6) in [64,2048]
  config 4: 200,000 pairs; 250 bp reads; refs U[2048,8192]; 20% near-identical (0.1%)
  (config 3, the serving loop, lives in mhm2_staging_gb300.serving)
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build
from .driver import Pairs

CONFIG_PAIRS = {0: 10_000, 1: 1_000_000, 2: 4_000_000, 4: 200_000}
_GEN: dict = {}


def _gen(path=None) -> C.CDLL:
    p = Path(path) if path else _build.gen_lib_path()
    if p not in _GEN:
        if not p.exists():
            raise RuntimeError(f"{p} missing: run mhm2_staging_gb300.build.build()")
        g = C.CDLL(str(p))
        g.mhsw_gen_pairs.restype = C.c_void_p
        g.mhsw_gen_pairs.argtypes = [C.c_int, C.c_uint64, C.c_int64, C.c_int64, C.c_int]
        for f in ("reads", "refs", "read_off", "ref_off", "read_len", "ref_len"):
            fn = getattr(g, "mhsw_gen_" + f)
            fn.restype = C.c_void_p
            fn.argtypes = [C.c_void_p]
        g.mhsw_gen_count.restype = C.c_int64
        g.mhsw_gen_count.argtypes = [C.c_void_p]
        g.mhsw_gen_free.restype = None
        g.mhsw_gen_free.argtypes = [C.c_void_p]
        _GEN[p] = g
    return _GEN[p]


def generate(config: int, n: int | None = None, seed: int | None = None, first: int = 0,
             threads: int | None = None, gen_lib=None) -> Pairs:
    """Pairs [first, first+n) of `config` (seed defaults to the config number).  gen_lib
    names another build of the generator library (the same source)."""
    if config not in CONFIG_PAIRS:
        raise ValueError(f"unknown config {config}")
    g = _gen(gen_lib)
    n = CONFIG_PAIRS[config] if n is None else n
    seed = config if seed is None else seed
    threads = threads or min(32, os.cpu_count() or 4)
    h = g.mhsw_gen_pairs(config, seed, first, n, threads)
    try:
        cnt = g.mhsw_gen_count(h)

        def arr(ptr, dt, k):
            if k == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (k,)).copy()

        roff = arr(g.mhsw_gen_read_off(h), np.int64, cnt + 1)
        foff = arr(g.mhsw_gen_ref_off(h), np.int64, cnt + 1)
        rlen = arr(g.mhsw_gen_read_len(h), np.int32, cnt)
        flen = arr(g.mhsw_gen_ref_len(h), np.int32, cnt)
        rseq = np.zeros(int(roff[-1]) + 1, dtype=np.uint8)
        fseq = np.zeros(int(foff[-1]) + 1, dtype=np.uint8)
        if roff[-1]:
            C.memmove(rseq.ctypes.data, g.mhsw_gen_reads(h), int(roff[-1]))
        if foff[-1]:
            C.memmove(fseq.ctypes.data, g.mhsw_gen_refs(h), int(foff[-1]))
    finally:
        g.mhsw_gen_free(h)
    return Pairs(rseq, roff[:-1].copy(), rlen, fseq, foff[:-1].copy(), flen)
