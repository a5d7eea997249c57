"""klign's caller side on the device: seed-hit candidates in, klign's Aln fields out.

`ResidentContigs` keeps a contig set on the device (mhsw_contigs_create); `klign_align`
runs mhsw_klign_align (include/mhsw.h) -- orientation, the seed-diagonal window, the
perfect-match shortcut, the alignments of the rest and klign's result mapping
(src/klign.cpp:218-266, :369-381, :670-739) -- for a candidate batch on a GPUDriver.
`generate_candidates` makes the seeded synthetic candidate workload: reads taken from the
contigs (40% exact, the rest with 2% substitutions, 0.2% N and, for a fifth of them, one
indel), half of them found on the reverse strand, each with a seed k-mer inside the read.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import driver as D
from .serving import Contigs

_P = C.c_void_p
_COMP = np.zeros(256, dtype=np.uint8)
for _a, _b in zip(b"ACGTN", b"TGCAN"):
    _COMP[_a] = _b


@dataclass
class Candidates:
    read_seq: np.ndarray     # uint8, reads as found (before orientation)
    read_off: np.ndarray     # int64
    read_len: np.ndarray     # int32
    cid: np.ndarray          # int32, contig of the seed hit
    pos_in_ctg: np.ndarray   # int32, seed k-mer start in the contig
    pos_in_read: np.ndarray  # int32, seed k-mer start in the read as found
    strand: np.ndarray       # uint8, bit 0: read k-mer reverse-complemented, bit 1: contig k-mer
    kmer_len: int

    @property
    def n(self) -> int:
        return int(self.read_len.shape[0])

    def slice(self, i: int, j: int) -> "Candidates":
        return Candidates(self.read_seq, self.read_off[i:j].copy(), self.read_len[i:j].copy(), self.cid[i:j].copy(),
                          self.pos_in_ctg[i:j].copy(), self.pos_in_read[i:j].copy(), self.strand[i:j].copy(),
                          self.kmer_len)


class ResidentContigs:
    """A contig set uploaded to (and translated on) one device."""

    def __init__(self, contigs: Contigs, device: int = 0):
        self._lib = D.load_library()
        self.contigs = contigs
        h = _P()
        off = np.ascontiguousarray(contigs.off, dtype=np.int64)
        ln = np.ascontiguousarray(contigs.len, dtype=np.int32)
        rc = self._lib.mhsw_contigs_create(device, contigs.seq.ctypes.data, off.ctypes.data, ln.ctypes.data,
                                           contigs.n, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"mhsw_contigs_create failed (status {rc})")
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mhsw_contigs_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def klign_align(drv: "D.GPUDriver", rc: ResidentContigs, cand: Candidates, cigars: bool = False,
                cigar_ops: bool = False) -> dict:
    """Aln fields per candidate (rstart, rstop, cstart, cstop, score1, score2, identity,
    orient as b'+'/b'-' codes, perfect) and n_aligned, as mhsw_klign_align computes them;
    with cigars (the driver in CIGAR mode) also klign's SAM CIGAR string and mismatches;
    with cigar_ops the same as arrays: cigar_slot (index into the batch, -1 for a perfect
    match) and cigar_batch (driver.Cigars of the aligned candidates)."""
    n = cand.n
    arrs = {k: np.zeros(n, dtype=np.int32) for k in ("rstart", "rstop", "cstart", "cstop", "score1", "score2",
                                                     "identity")}
    arrs["orient"] = np.zeros(n, dtype=np.uint8)
    arrs["perfect"] = np.zeros(n, dtype=np.uint8)
    keep = [np.ascontiguousarray(x, dtype=t) for x, t in ((cand.read_off, np.int64), (cand.read_len, np.int32),
                                                           (cand.cid, np.int32), (cand.pos_in_ctg, np.int32),
                                                           (cand.pos_in_read, np.int32), (cand.strand, np.uint8))]
    ct = D.CandidatesT(cand.read_seq.ctypes.data, *(k.ctypes.data for k in keep), n, cand.kmer_len)
    slot = np.full(n, -1, dtype=np.int32)
    at = D.AlnsT(*(arrs[k].ctypes.data for k in ("rstart", "rstop", "cstart", "cstop", "score1", "score2",
                                                  "identity", "orient", "perfect")),
                   slot.ctypes.data if cigars or cigar_ops else None)
    m = C.c_int64(0)
    drv._ck(drv._lib.mhsw_klign_align(drv._h, rc.handle, C.byref(ct), C.byref(at), C.byref(m)), "klign_align")
    arrs["n_aligned"] = int(m.value)
    if cigar_ops and not cigars:
        arrs["cigar_slot"] = slot
        arrs["cigar_batch"] = drv.last_cigar(arrs["n_aligned"])
    if cigars:
        # klign's SAM fields: "<overlap>=" and 0 mismatches for a perfect match (src/klign.cpp:229),
        # SSW's cigar_string and mismatches for the aligned candidates
        cg = drv.last_cigar(arrs["n_aligned"])
        arrs["cigar"] = [cg.string(int(j)) if j >= 0 else f"{arrs['rstop'][i] - arrs['rstart'][i]}="
                         for i, j in enumerate(slot)]
        arrs["mismatches"] = np.where(slot >= 0, cg.mismatches[np.maximum(slot, 0)] if len(cg.mismatches) else 0,
                                      0).astype(np.int32)
    return arrs


def generate_candidates(contigs: Contigs, n: int, seed: int = 5, kmer_len: int = 31, exact_frac: float = 0.4,
                        sub_rate: float = 0.02, n_rate: float = 0.002, indel_frac: float = 0.2,
                        minus_frac: float = 0.5) -> Candidates:
    """Seeded candidates: reads of U[100, 250] bases taken from contigs of at least 300
    bases, mutated as described in the module docstring, with a seed inside the read."""
    rng = np.random.default_rng(seed)
    eligible = np.nonzero(contigs.len >= 300)[0]
    cid = rng.choice(eligible, size=n).astype(np.int32)
    clen = contigs.len[cid].astype(np.int64)
    L = rng.integers(100, 251, size=n)
    pos = (rng.random(n) * (clen - L + 1)).astype(np.int64)
    exact = rng.random(n) < exact_frac
    reads, seeds, pics = [], np.zeros(n, dtype=np.int64), np.zeros(n, dtype=np.int64)
    for i in range(n):
        start = int(contigs.off[cid[i]] + pos[i])
        r = contigs.seq[start:start + int(L[i])].copy()
        if not exact[i]:
            sub = rng.random(r.shape[0]) < sub_rate
            r[sub] = np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, int(sub.sum()))]
            nn = rng.random(r.shape[0]) < n_rate
            r[nn] = ord("N")
            if rng.random() < indel_frac:
                k = int(rng.integers(1, r.shape[0] - 1))
                if rng.random() < 0.5:
                    r = np.delete(r, k)
                else:
                    r = np.insert(r, k, np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4)])
        s = int(rng.integers(0, r.shape[0] - kmer_len + 1))  # seed start in the contig-oriented read
        seeds[i] = s
        pics[i] = min(int(pos[i]) + s, int(clen[i]) - kmer_len)
        reads.append(r)
    minus = rng.random(n) < minus_frac
    read_is_rc = rng.integers(0, 2, n).astype(np.uint8)
    strand = (read_is_rc | ((read_is_rc ^ minus.astype(np.uint8)) << 1)).astype(np.uint8)
    lens = np.array([r.shape[0] for r in reads], dtype=np.int32)
    off = np.zeros(n, dtype=np.int64)
    off[1:] = np.cumsum(lens[:-1])
    seq = np.zeros(int(lens.sum()) + 16, dtype=np.uint8)
    pir = np.zeros(n, dtype=np.int32)
    for i, r in enumerate(reads):
        if minus[i]:  # found on the other strand: the read as found is the reverse complement
            seq[off[i]:off[i] + lens[i]] = _COMP[r[::-1]]
            pir[i] = lens[i] - kmer_len - seeds[i]
        else:
            seq[off[i]:off[i] + lens[i]] = r
            pir[i] = seeds[i]
    return Candidates(seq, off, lens, cid, pics.astype(np.int32), pir, strand, kmer_len)
