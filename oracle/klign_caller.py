"""CPU restatement of klign's caller side around the aligner (test infrastructure only:
used by tests/ and bench.py's CPU-baseline leg to check results and as the timed CPU baseline, never by the product).

For each seed-hit candidate (read, contig, seed positions, strands), as
src/klign.cpp does it:
  * compute_alns_for_read (klign.cpp:670-739): orientation '-' when the read's and the
    contig's seed k-mers differ in strand, the read then reverse-complemented
    (utils.cpp:94-119: ACGTN, IUPAC codes to N, anything else rejected) and the seed
    position mirrored (pos_in_read = rlen - (kmer_len + pos_in_read)); the window
    left = min(pos_in_read, pos_in_ctg), right = min(rlen - kmer_len - pos_in_read,
    clen - pos_in_ctg - kmer_len), cstart = pos_in_ctg - left, rstart = pos_in_read - left,
    overlap = left + kmer_len + right;
  * align_read (:218-241): a window whose bytes equal the oriented read's overlap is a
    perfect match (score1 = overlap * match, rstop = rstart + overlap, cstop = cstart +
    overlap); otherwise the whole oriented read is aligned against the window (SSW ref =
    read, query = window, :257);
  * ssw_align_read / the GPU block's mapping (:260-266, :372-381): rstart = read begin,
    rstop = read end + 1, cstart += window begin, cstop = cstart(window) + window end + 1;
  * switch_orient (utils.cpp:163-167) for '-'; identity = 100 * score1 / match / rlen.
The alignments themselves come from the SW oracle (oracle.align_batch).
"""
from __future__ import annotations

import numpy as np

from . import oracle

_COMP = np.full(256, -1, dtype=np.int16)
for _a, _b in zip(b"ACGTN", b"TGCAN"):
    _COMP[_a] = _b
for _c in b"URYKMSWBDHV":
    _COMP[_c] = ord("N")


def klign_align(contig_seq: np.ndarray, contig_off: np.ndarray, contig_len: np.ndarray, read_seq: np.ndarray,
                read_off: np.ndarray, read_len: np.ndarray, cid: np.ndarray, pos_in_ctg: np.ndarray,
                pos_in_read: np.ndarray, strand: np.ndarray, kmer_len: int, scoring=(1, 3, 5, 2, 2),
                score2: bool = False, threads: int | None = None, cigars: bool = False) -> dict:
    """Per-candidate Aln fields: rstart, rstop, cstart, cstop, score1, score2, identity,
    orient ('+'/'-' as bytes), perfect (0/1); plus n_aligned.  cigars: also klign's SAM
    CIGAR string and mismatches -- "<overlap>=" and 0 for a perfect match (klign.cpp:229),
    SSW's cigar_string and mismatches (report_cigar) for the others (:271, :268)."""
    from mhm2_staging_gb300.driver import Pairs

    n = int(read_len.shape[0])
    match = scoring[0]
    minus = ((strand >> 1) & 1) != (strand & 1)
    rl = read_len.astype(np.int64)
    # oriented reads (the reverse complement is taken of every read, :673)
    ori = read_seq.copy()
    for i in range(n):
        o, L = int(read_off[i]), int(rl[i])
        r = read_seq[o:o + L]
        rc = _COMP[r[::-1]]
        if (rc < 0).any():
            raise ValueError(f"candidate {i}: a read byte revcomp rejects")
        if minus[i]:
            ori[o:o + L] = rc.astype(np.uint8)
    K = int(kmer_len)
    pir = np.where(minus, rl - (K + pos_in_read), pos_in_read).astype(np.int64)
    pic = pos_in_ctg.astype(np.int64)
    cl = contig_len[cid].astype(np.int64)
    left = np.minimum(pir, pic)
    right = np.minimum(rl - K - pir, cl - pic - K)
    cstart = pic - left
    rstart = pir - left
    ov = left + K + right
    coff = contig_off[cid].astype(np.int64) + cstart
    perfect = np.zeros(n, dtype=bool)
    for i in range(n):
        a = contig_seq[coff[i]:coff[i] + ov[i]]
        b = ori[read_off[i] + rstart[i]:read_off[i] + rstart[i] + ov[i]]
        perfect[i] = np.array_equal(a, b)
    idx = np.nonzero(~perfect)[0]
    rs = rstart.copy()
    re = rstart + ov
    cs = cstart.copy()
    ce = cstart + ov
    sc = ov * match
    s2 = np.zeros(n, dtype=np.int64)
    cig = [f"{int(o)}=" for o in ov]
    mism = np.zeros(n, dtype=np.int32)
    if len(idx):
        pairs = Pairs(ori, read_off[idx].astype(np.int64), read_len[idx].astype(np.int32), contig_seq,
                      coff[idx].astype(np.int64), ov[idx].astype(np.int32))
        if cigars:
            cout, cops, cn = oracle.cigar_batch(pairs, scoring, threads, ops_cap=2048)
            for t, i in enumerate(idx):
                cig[i] = oracle.cigar_string(cops[t], max(int(cn[t]), 0))
                mism[i] = cout[t, 5]
        res = oracle.align_batch(pairs, scoring, threads, score2=score2).astype(np.int64)
        sc[idx] = res[:, 0]
        rs[idx] = res[:, 1]
        re[idx] = res[:, 2] + 1
        cs[idx] = cstart[idx] + res[:, 3]
        ce[idx] = cstart[idx] + res[:, 4] + 1
        if score2:
            s2[idx] = res[:, 5]
    rs2 = np.where(minus, rl - re, rs)
    re2 = np.where(minus, rl - rs, re)
    ident = (100 * sc // match) // rl  # C integer division; all operands are non-negative
    return {"rstart": rs2.astype(np.int32), "rstop": re2.astype(np.int32), "cstart": cs.astype(np.int32),
            "cstop": ce.astype(np.int32), "score1": sc.astype(np.int32), "score2": s2.astype(np.int32),
            "identity": ident.astype(np.int32), "orient": np.where(minus, ord("-"), ord("+")).astype(np.uint8),
            "perfect": perfect.astype(np.uint8), "n_aligned": int(len(idx)),
            **({"cigar": cig, "mismatches": mism} if cigars else {})}
