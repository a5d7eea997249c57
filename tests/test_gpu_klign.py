"""klign's caller side on the GPU (mhsw_klign_align): orientation, windows, the
perfect-match shortcut, the alignments and klign's Aln mapping, bit-exact against the
CPU restatement (oracle/klign_caller.py) on seeded candidates."""
import numpy as np
import pytest

from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, GPUDriver
from mhm2_staging_gb300 import serving as S
from mhm2_staging_gb300.klign import Candidates, ResidentContigs, generate_candidates, klign_align
from oracle import klign_caller

pytestmark = pytest.mark.gpu
FIELDS = ("rstart", "rstop", "cstart", "cstop", "score1", "score2", "identity", "orient", "perfect")


@pytest.fixture(scope="module")
def contigs(built):
    return S.generate_contigs(32 << 20, seed=3)


@pytest.fixture(scope="module")
def resident(contigs):
    rc = ResidentContigs(contigs)
    yield rc
    rc.close()


def _driver(sc=(1, 3, 5, 2, 2), form=FORM_BATCHED, score2=False):
    m, x, go, ge, amb = sc
    d = GPUDriver()
    d.init(0, 1, m, -x, -go, -ge, 0)
    d.set_ambiguity(-amb)
    d.set_form(form)
    d.set_score2(score2)
    return d


def _want(ct, cand, sc, score2):
    return klign_caller.klign_align(ct.seq, ct.off, ct.len, cand.read_seq, cand.read_off, cand.read_len, cand.cid,
                                    cand.pos_in_ctg, cand.pos_in_read, cand.strand, cand.kmer_len, sc, score2)


def _diff(got, want):
    for k in FIELDS:
        bad = np.nonzero(got[k] != want[k])[0]
        if len(bad):
            i = int(bad[0])
            return f"{k}: {len(bad)} differ; first {i}: gpu {got[k][i]} oracle {want[k][i]}"
    return "" if got["n_aligned"] == want["n_aligned"] else f"n_aligned {got['n_aligned']} vs {want['n_aligned']}"


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
@pytest.mark.parametrize("sc,score2", [((1, 3, 5, 2, 2), False), ((2, 4, 4, 2, 1), True)])
def test_klign_caller_matches_restatement(contigs, resident, form, sc, score2):
    cand = generate_candidates(contigs, 30000, seed=21)
    d = _driver(sc, form, score2)
    got = klign_align(d, resident, cand)
    want = _want(contigs, cand, sc, score2)
    assert not _diff(got, want)
    assert 0.3 < got["perfect"].mean() < 0.6 and got["n_aligned"] > 10000
    t = d.last_timing()  # the aligned candidates' device times
    assert t["n_pairs"] == got["n_aligned"] and t["fwd_ms"] > 0 and t["total_ms"] >= t["fwd_ms"]


def test_klign_caller_k21_and_all_reverse(contigs, resident):
    cand = generate_candidates(contigs, 5000, seed=2, kmer_len=21, minus_frac=1.0, exact_frac=0.1)
    got = klign_align(_driver(), resident, cand)
    assert not _diff(got, _want(contigs, cand, (1, 3, 5, 2, 2), False))
    assert (got["orient"] == ord("-")).all()


def test_klign_caller_boundary_seeds_and_iupac(contigs, resident):
    """Seeds on the first and last k-mer of the read and of the contig (windows clipped at
    the contig's ends), reads exactly one k-mer long, and IUPAC codes and U in the reads
    (aligned as found on '+' -- U scores as A there, the others as N -- and turned into N
    by the reverse complement on '-')."""
    base = generate_candidates(contigs, 4000, seed=13)
    K, n = base.kmer_len, base.n
    rng = np.random.default_rng(17)
    q = np.arange(n) % 5
    reads = [base.read_seq[o:o + L].copy() for o, L in zip(base.read_off, base.read_len)]
    pir = base.pos_in_read.copy()
    pic = base.pos_in_ctg.copy()
    clen = contigs.len[base.cid]
    for i in range(n):
        if q[i] == 0:
            pir[i] = 0
        elif q[i] == 1:
            pir[i] = len(reads[i]) - K
        elif q[i] == 2:
            pic[i] = 0
        elif q[i] == 3:
            pic[i] = clen[i] - K
        else:  # one k-mer: the seed itself
            reads[i] = reads[i][pir[i]:pir[i] + K].copy()
            pir[i] = 0
        if rng.random() < 0.15:
            reads[i][rng.integers(0, len(reads[i]))] = np.frombuffer(b"URYKMSWBDHV", dtype=np.uint8)[rng.integers(0, 11)]
    lens = np.array([len(r) for r in reads], dtype=np.int32)
    off = np.zeros(n, dtype=np.int64)
    off[1:] = np.cumsum(lens[:-1])
    seq = np.zeros(int(lens.sum()) + 16, dtype=np.uint8)
    for i, r in enumerate(reads):
        seq[off[i]:off[i] + lens[i]] = r
    cand = Candidates(seq, off, lens, base.cid.copy(), pic.astype(np.int32), pir.astype(np.int32),
                      base.strand.copy(), K)
    for sc, score2 in (((1, 3, 5, 2, 2), False), ((2, 4, 4, 2, 1), True)):
        got = klign_align(_driver(sc, FORM_BATCHED, score2), resident, cand)
        want = _want(contigs, cand, sc, score2)
        assert not _diff(got, want)
        assert got["perfect"][q == 4].mean() > 0.5 and got["n_aligned"] > 1000
    assert (cand.pos_in_ctg[q == 3] + K == clen[q == 3]).all()
    # CIGAR mode at klign's post-assembly scoring: SAM CIGARs and mismatches of the same set
    sc = (2, 4, 4, 2, 1)
    d = _driver(sc)
    d.set_cigar(True)
    got = klign_align(d, resident, cand, cigars=True)
    want = klign_caller.klign_align(contigs.seq, contigs.off, contigs.len, cand.read_seq, cand.read_off,
                                    cand.read_len, cand.cid, cand.pos_in_ctg, cand.pos_in_read, cand.strand,
                                    K, sc, False, cigars=True)
    assert not _diff(got, want)
    bad = [i for i in range(n) if got["cigar"][i] != want["cigar"][i]]
    assert not bad, (len(bad), got["cigar"][bad[0]], want["cigar"][bad[0]])
    assert np.array_equal(got["mismatches"], want["mismatches"])


def test_klign_caller_arena_grows_and_is_reused(contigs, resident):
    """One handle, batches of growing then shrinking size: the call arena kept on the handle
    grows for the larger batch and is reused by the smaller ones."""
    d = _driver()
    for n, seed in ((500, 41), (40000, 42), (500, 43), (3, 44)):
        cand = generate_candidates(contigs, n, seed=seed)
        assert not _diff(klign_align(d, resident, cand), _want(contigs, cand, (1, 3, 5, 2, 2), False)), n


def test_klign_caller_two_threads_share_a_handle(contigs, resident):
    """Calls on one handle from two host threads (ctypes releases the GIL during the call)
    are serialised by the handle: each thread gets its own batch's results."""
    import threading

    d = _driver()
    batches = [generate_candidates(contigs, n, seed=s) for n, s in ((20000, 51), (5000, 52))]
    wants = [_want(contigs, c, (1, 3, 5, 2, 2), False) for c in batches]
    errors = []

    def run(i):
        try:
            for _ in range(3):
                msg = _diff(klign_align(d, resident, batches[i]), wants[i])
                if msg:
                    errors.append((i, msg))
        except Exception as exc:  # reported below
            errors.append((i, repr(exc)))

    th = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors


def test_klign_caller_rejects_bad_candidates(contigs, resident):
    d = _driver()
    cand = generate_candidates(contigs, 10, seed=5)
    bad = cand.slice(0, 10)
    bad.pos_in_read[3] = bad.read_len[3] - bad.kmer_len + 1  # seed past the read's end
    with pytest.raises(RuntimeError, match="status 2"):
        klign_align(d, resident, bad)
    bad = cand.slice(0, 10)
    bad.pos_in_ctg[2] = contigs.len[bad.cid[2]]  # seed past the contig's end
    with pytest.raises(RuntimeError, match="status 2"):
        klign_align(d, resident, bad)
    seq = cand.read_seq.copy()
    seq[cand.read_off[4] + 1] = ord("a")  # revcomp rejects lower case
    bad = Candidates(seq, cand.read_off, cand.read_len, cand.cid, cand.pos_in_ctg, cand.pos_in_read, cand.strand,
                     cand.kmer_len)
    with pytest.raises(RuntimeError, match="status 2"):
        klign_align(d, resident, bad)
    # the driver is still usable afterwards, and an empty batch is fine
    got = klign_align(d, resident, cand)
    assert not _diff(got, _want(contigs, cand, (1, 3, 5, 2, 2), False))
    assert klign_align(d, resident, cand.slice(0, 0))["n_aligned"] == 0


def test_klign_caller_sam_cigars(contigs, resident):
    """CIGAR mode: klign's SAM CIGAR per candidate -- "<overlap>=" for the perfect matches,
    SSW's cigar_string for the aligned ones -- and mismatches, with the post-assembly
    scoring 2/4/4/2/1 klign uses when it asks for CIGARs."""
    sc = (2, 4, 4, 2, 1)
    cand = generate_candidates(contigs, 20000, seed=33)
    d = _driver(sc)
    d.set_cigar(True)
    got = klign_align(d, resident, cand, cigars=True)
    want = klign_caller.klign_align(contigs.seq, contigs.off, contigs.len, cand.read_seq, cand.read_off,
                                    cand.read_len, cand.cid, cand.pos_in_ctg, cand.pos_in_read, cand.strand,
                                    cand.kmer_len, sc, False, cigars=True)
    assert not _diff(got, want)
    bad = [i for i in range(cand.n) if got["cigar"][i] != want["cigar"][i]]
    assert not bad, (len(bad), got["cigar"][bad[0]], want["cigar"][bad[0]])
    assert np.array_equal(got["mismatches"], want["mismatches"])


def test_klign_caller_cigar_ops_arrays(contigs, resident):
    """The array form of CIGAR mode (cigar_ops) returns the batch the strings come from."""
    sc = (2, 4, 4, 2, 1)
    cand = generate_candidates(contigs, 3000, seed=35)
    d = _driver(sc)
    d.set_cigar(True)
    got = klign_align(d, resident, cand, cigar_ops=True)
    s = klign_align(d, resident, cand, cigars=True)
    slot, cb = got["cigar_slot"], got["cigar_batch"]
    strings = [cb.string(int(j)) if j >= 0 else f"{got['rstop'][i] - got['rstart'][i]}=" for i, j in enumerate(slot)]
    assert strings == s["cigar"]
    assert got["n_aligned"] == s["n_aligned"] and len(cb.nops) == got["n_aligned"]
