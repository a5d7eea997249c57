"""klign's caller side (CPU): the restatement's invariants and hand-worked cases of
src/klign.cpp:670-739 / :218-266 / utils.cpp switch_orient, and the C ABI's argument
checks that need no GPU."""
import ctypes as C

import numpy as np
import pytest

from mhm2_staging_gb300 import serving as S
from mhm2_staging_gb300.klign import Candidates, generate_candidates
from oracle import klign_caller

SC = (1, 3, 5, 2, 2)


def _run(ct, cand, sc=SC, score2=False):
    return klign_caller.klign_align(ct.seq, ct.off, ct.len, cand.read_seq, cand.read_off, cand.read_len, cand.cid,
                                    cand.pos_in_ctg, cand.pos_in_read, cand.strand, cand.kmer_len, sc, score2)


def _contigs(*seqs):
    seq = np.frombuffer(b"".join(s.encode() for s in seqs) + b"\0" * 16, dtype=np.uint8).copy()
    ln = np.array([len(s) for s in seqs], dtype=np.int32)
    off = np.zeros(len(seqs), dtype=np.int64)
    off[1:] = np.cumsum(ln[:-1])
    return S.Contigs(seq, off, ln)


def _cands(reads, cid, pic, pir, strand, k):
    seq = np.frombuffer(b"".join(r.encode() for r in reads) + b"\0" * 16, dtype=np.uint8).copy()
    ln = np.array([len(r) for r in reads], dtype=np.int32)
    off = np.zeros(len(reads), dtype=np.int64)
    off[1:] = np.cumsum(ln[:-1])
    return Candidates(seq, off, ln, np.array(cid, np.int32), np.array(pic, np.int32), np.array(pir, np.int32),
                      np.array(strand, np.uint8), k)


def test_hand_worked_windows_and_orientation():
    ctg = "TTTTTACGTACGGATTACACCC"       # clen 22
    ct = _contigs(ctg)
    # '+': read = ctg[5:17] exactly, seed "GTACGG" at read 2 / contig 7 -> perfect
    # '-': the same read found reverse-complemented, seed flags differ in strand
    rd = ctg[5:17]
    rc = rd[::-1].translate(str.maketrans("ACGT", "TGCA"))
    cand = _cands([rd, rc, "AC" + rd[2:]], [0, 0, 0], [7, 7, 7], [2, len(rd) - 6 - 2, 2], [0, 1, 2], 6)
    r = _run(ct, cand)
    # candidate 0: left = min(2, 7) = 2, right = min(12-6-2, 22-7-6) = 4 -> cstart 5, overlap 12
    assert (r["perfect"][0], r["rstart"][0], r["rstop"][0], r["cstart"][0], r["cstop"][0]) == (1, 0, 12, 5, 17)
    assert r["score1"][0] == 12 and r["identity"][0] == 100 and r["orient"][0] == ord("+")
    # candidate 1: '-' (bit 0 only), pos_in_read mirrored back to 2; the oriented read is rd
    assert r["orient"][1] == ord("-") and r["perfect"][1] == 1
    # switch_orient(0, 12, 12) -> (0, 12)
    assert (r["rstart"][1], r["rstop"][1], r["cstart"][1], r["cstop"][1]) == (0, 12, 5, 17)
    # candidate 2: '-' (bit 1 only) but the read is given forward: its reverse complement
    # is aligned, not a perfect match
    assert r["orient"][2] == ord("-") and r["perfect"][2] == 0


def test_partial_footprint_is_clipped_to_the_contig():
    ctg = "ACGTTGCAAGGT"
    ct = _contigs(ctg)
    rd = "GGGG" + ctg[:8]                # the read hangs off the contig's left end
    cand = _cands([rd], [0], [0], [4], [0], 4)
    r = _run(ct, cand)
    # left = min(4, 0) = 0, right = min(12-4-4, 12-0-4) = 4: window ctg[0:8] vs read[4:12]
    assert (r["perfect"][0], r["rstart"][0], r["rstop"][0], r["cstart"][0], r["cstop"][0]) == (1, 4, 12, 0, 8)
    assert r["identity"][0] == 100 * 8 // 12


def test_generated_candidates_invariants():
    ct = S.generate_contigs(2 << 20, seed=4)
    cand = generate_candidates(ct, 3000, seed=9)
    r = _run(ct, cand)
    L = cand.read_len
    assert 0.35 < r["perfect"].mean() < 0.6
    assert ((r["rstart"] >= 0) & (r["rstop"] <= L) & (r["rstart"] < r["rstop"])).all()
    p = r["perfect"] == 1
    assert (r["identity"][p] <= 100).all() and (r["score1"][p] == r["rstop"][p] - r["rstart"][p]).all()
    assert (r["cstop"] - r["cstart"] <= L + 1).all()


def test_revcomp_rejects_what_klign_rejects():
    ct = _contigs("ACGTACGTACGT")
    cand = _cands(["ACGTxCGT"], [0], [0], [0], [0], 4)
    with pytest.raises(ValueError):
        _run(ct, cand)


def test_abi_argument_checks(built):
    from mhm2_staging_gb300 import driver as D

    lib = D.load_library()
    ct = D.CandidatesT()
    at = D.AlnsT()
    assert lib.mhsw_klign_align(None, None, C.byref(ct), C.byref(at), None) == 2
    h = C.c_void_p()
    assert lib.mhsw_contigs_create(0, None, None, None, -1, C.byref(h)) == 2
