"""ADEPT on the same GPU: the reference's own CUDA kernels for this path, as a performance
comparator (test and measurement infrastructure only: run by bench.py's reference arm and
the tests, never by the product).

`sequence_dna_kernel` and `sequence_dna_reverse` (reference src/adept-sw/kernel.cpp:160-509)
are compiled for sm_103a from the reference checkout by oracle/Makefile into
_ref/adept_sm103a.cubin (device code only: nothing of the reference's host code is built).
This module loads that cubin through the CUDA driver API and launches the two kernels the
way the reference's driver does (src/adept-sw/driver.cpp:281-416), on device-resident
inputs:
  * A = contig windows, B = reads (driver.cpp:296-301), each packed back to back, with
    inclusive `unsigned` prefix sums of the lengths (:308-327);
  * forward: one block per pair, min(max read length, max contig length) threads, dynamic
    shared memory 3 * (threads + 1) shorts + 4 + (4 - that % 4) bytes (:348-352);
  * the ends come back to the host, and the reverse launch takes
    min(max A end, max B end) threads (get_new_min_length, :170-180; :377-416);
  * scores as klign passes them: match, -mismatch, -gap open, -gap extend (klign.cpp:464-465).
ADEPT is not bit-exact with SSW (raw-byte compares, diagonal-order ties); only its top
scores are compared with the oracle, as a check that the launches are right.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "adept_sm103a.cubin"
_FWD = b"_ZN7gpu_bsw19sequence_dna_kernelEPcS0_PjS1_PsS2_S2_S2_S2_ssss"
_REV = b"_ZN7gpu_bsw20sequence_dna_reverseEPcS0_PjS1_PsS2_S2_S2_S2_ssss"
_CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8


def available() -> bool:
    return CUBIN.exists()


class Adept:
    """The two ADEPT kernels loaded on the current device (torch's primary context)."""

    def __init__(self, device: int = 0):
        import torch

        if not available():
            raise RuntimeError(f"{CUBIN} is missing (built from the reference checkout by oracle/Makefile)")
        torch.cuda.set_device(device)
        torch.zeros(1, device=f"cuda:{device}")  # makes the primary context current
        self._torch = torch
        self.device = device
        self._cu = C.CDLL("libcuda.so.1")
        self._mod = C.c_void_p()
        self._ck(self._cu.cuModuleLoad(C.byref(self._mod), str(CUBIN).encode()), "cuModuleLoad")
        self._fwd, self._rev = C.c_void_p(), C.c_void_p()
        self._ck(self._cu.cuModuleGetFunction(C.byref(self._fwd), self._mod, _FWD), "cuModuleGetFunction forward")
        self._ck(self._cu.cuModuleGetFunction(C.byref(self._rev), self._mod, _REV), "cuModuleGetFunction reverse")

    @staticmethod
    def _ck(rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what} failed (CUresult {rc})")

    def upload(self, pairs) -> dict:
        """Packs a Pairs batch the way the reference driver does: A = contig windows (our B
        side), B = reads (our A side), back to back, with inclusive uint32 prefix sums."""
        torch = self._torch
        dev = f"cuda:{self.device}"

        def pack(seq, off, ln):
            ln = ln.astype(np.int64)
            total = int(ln.sum())
            if total >= 2 ** 32:
                raise ValueError("ADEPT's prefix sums are 32-bit")
            starts = np.zeros(len(ln), dtype=np.int64)
            starts[1:] = np.cumsum(ln)[:-1]
            if np.array_equal(off.astype(np.int64), starts):
                buf = np.ascontiguousarray(seq[:total])
            else:
                idx = np.repeat(off.astype(np.int64) - starts, ln) + np.arange(total, dtype=np.int64)
                buf = seq[idx]
            pre = np.cumsum(ln).astype(np.uint32)
            return (torch.from_numpy(buf.view(np.uint8)).to(dev),
                    torch.from_numpy(pre.view(np.int32)).to(dev))

        a, pa = pack(pairs.b_seq, pairs.b_off, pairs.b_len)  # contig windows
        b, pb = pack(pairs.a_seq, pairs.a_off, pairs.a_len)  # reads
        n = pairs.n
        out = {k: torch.zeros(n, dtype=torch.int16, device=dev) for k in ("a_beg", "a_end", "b_beg", "b_end", "score")}
        return {"a": a, "b": b, "pa": pa, "pb": pb, "n": n, "out": out,
                "max_read": int(pairs.a_len.max()), "max_contig": int(pairs.b_len.max())}

    def _launch(self, fn, grid: int, block: int, smem: int, batch: dict, scoring, stream: int) -> None:
        o = batch["out"]
        m, x, go, ge = scoring[:4]
        ptrs = [C.c_void_p(t.data_ptr()) for t in (batch["a"], batch["b"], batch["pa"], batch["pb"], o["a_beg"],
                                                   o["a_end"], o["b_beg"], o["b_end"], o["score"])]
        shorts = [C.c_short(v) for v in (m, -x, -go, -ge)]
        args = ptrs + shorts
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(v), C.c_void_p) for v in args])
        self._ck(self._cu.cuLaunchKernel(fn, C.c_uint(grid), C.c_uint(1), C.c_uint(1), C.c_uint(block), C.c_uint(1),
                                         C.c_uint(1), C.c_uint(smem), C.c_void_p(stream), params, None),
                 "cuLaunchKernel")

    def run(self, batch: dict, scoring=(1, 3, 5, 2, 2), stream: int = 0, events=None) -> None:
        """Forward, ends to the host and the reverse-launch width, reverse (the reference
        driver's forwards -> block -> backwards protocol).  events: optional four CUDA
        events recorded around the two kernels."""
        torch = self._torch
        threads = min(batch["max_read"], batch["max_contig"])
        if not 0 < threads <= 1024:
            raise ValueError("ADEPT needs the shorter sequence within 1..1024 bases")
        shm = 3 * (threads + 1) * 2
        smem = shm + 4 + (4 - shm % 4)
        for fn in (self._fwd, self._rev):
            self._ck(self._cu.cuFuncSetAttribute(fn, _CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, C.c_int(smem)),
                     "cuFuncSetAttribute")
        n = batch["n"]
        if events:
            events[0].record()
        self._launch(self._fwd, n, threads, smem, batch, scoring, stream)
        if events:
            events[1].record()
        o = batch["out"]
        new_min = min(int(o["b_end"].max().item()), int(o["a_end"].max().item()))  # host reduction (:170-180)
        if new_min <= 0:
            new_min = 1
        if events:
            events[2].record()
        self._launch(self._rev, n, new_min, smem, batch, scoring, stream)
        if events:
            events[3].record()
        torch.cuda.synchronize(self.device)

    def scores(self, batch: dict) -> np.ndarray:
        return batch["out"]["score"].cpu().numpy().astype(np.int32)
