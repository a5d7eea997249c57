"""CPU oracle pinned against the reference's known answers and the reference SSW itself."""
import json
import random
from pathlib import Path

import numpy as np
import pytest

from mhm2_staging_gb300 import Pairs
from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "ssw_known_answers.json").read_text())
SAMPLES = json.loads((GOLDEN / "ssw_reference_samples.json").read_text())
TEST_SCORINGS = ("ssw_default", "mhm2_aln", "cigar")  # the scorings test/ssw-test.cpp runs


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    return built


def _kat_pairs():
    cases = KAT["cases"]
    return cases, Pairs.from_lists([c["ref"] for c in cases], [c["query"] for c in cases])


@pytest.mark.parametrize("scoring", TEST_SCORINGS)
def test_known_answers_of_reference_test(scoring):
    """test/ssw-test.cpp:151-238: begin/end expectations, and the bounds of the no-match case."""
    cases, pairs = _kat_pairs()
    out = oracle.align_batch(pairs, tuple(KAT["scorings"][scoring]))
    for c, (score, ab, ae, bb, be) in zip(cases, out.tolist()):
        if c["kind"] == "aln":
            assert (bb, be, ab, ae) == (c["qbegin"], c["qend"], c["rbegin"], c["rend"]), c
        else:  # check_not_alns (:142-149)
            assert ae - ab <= 2 and be - bb <= 2 and score <= 4, c


def test_adept_expectations_match_ssw_expectations():
    """The GPU test's expectations (:241-431) equal the CPU test's for every case but the
    no-match one, which only checks bounds (:73-77)."""
    for c in KAT["cases"]:
        if c["kind"] == "aln":
            e = c["adept_expect"]
            assert (e["qbegin"], e["qend"], e["rbegin"], e["rend"]) == (c["qbegin"], c["qend"], c["rbegin"], c["rend"])


@pytest.mark.parametrize("scoring", list(KAT["scorings"]))
def test_known_answers_vs_recorded_reference(scoring):
    cases, pairs = _kat_pairs()
    out = oracle.align_batch(pairs, tuple(KAT["scorings"][scoring]))
    want = np.array([c["reference"][scoring] for c in cases], dtype=np.int32)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("scoring", list(SAMPLES["scorings"]))
def test_samples_vs_recorded_reference(scoring):
    recs = SAMPLES["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    out = oracle.align_batch(pairs, tuple(SAMPLES["scorings"][scoring]))
    want = np.array([r["reference"][scoring] for r in recs], dtype=np.int32)
    bad = np.nonzero((out != want).any(axis=1))[0]
    assert len(bad) == 0, [(recs[i]["set"], out[i].tolist(), want[i].tolist()) for i in bad[:3]]


def test_zero_score_and_empty_conventions():
    """Score 0 -> ref(A) begin/end -1, query(B) begin/end 0 (ssw_core.cpp:241, :1177-1178)."""
    p = Pairs.from_lists(["AAAA", "", "ACGT", "N"], ["CCCC", "ACGT", "", "N"])
    out = oracle.align_batch(p, (1, 3, 5, 2, 2))
    assert out.tolist() == [[0, -1, -1, 0, 0]] * 4


def _tie_heavy_pairs(seed, n=400):
    rng = random.Random(seed)
    alphabets = ["ACGT", "AC", "A", "ACGTN", "acgtU", "ACGTNX"]
    a, b = [], []
    for _ in range(n):
        al = rng.choice(alphabets)
        la, lb = rng.randint(1, 60), rng.randint(1, 90)
        x = "".join(rng.choice(al) for _ in range(la))
        if rng.random() < 0.5:
            y = "".join(rng.choice(al) for _ in range(lb))
        else:
            k = rng.randint(0, lb)
            y = "".join(rng.choice(al) for _ in range(k)) + x + "".join(rng.choice(al) for _ in range(rng.randint(0, 20)))
        a.append(x)
        b.append(y)
    return a, b


@pytest.mark.parametrize("sc", [(1, 3, 5, 2, 2), (2, 4, 4, 2, 1), (1, 2, 3, 1, 4), (2, 2, 3, 1, 2), (1, 1, 1, 1, 1),
                                (1, 3, 5, 2, 0)])
def test_vectorised_restatement_equals_scalar(sc):
    """sw_lanes.cpp (eight pairs per vector, the CPU baseline) against the scalar
    restatement: tie-heavy pairs, empty and all-N sequences, the generated workloads, and
    the scalar fallbacks (scores that could leave int16; ambiguity 0)."""
    from mhm2_staging_gb300 import workloads

    a, b = _tie_heavy_pairs(7, 600)
    a += ["", "ACGT", "NNNN", "A" * 300, "ACGT" * 75]
    b += ["ACGT", "", "NNNN", "A" * 310, "ACGT" * 80]
    batches = [Pairs.from_lists(a, b)] + [workloads.generate(cfg, n=n) for cfg, n in ((0, 600), (1, 900), (2, 900))]
    for p in batches:
        got = oracle.align_batch_lanes(p, sc, 4)
        want = oracle.align_batch(p, sc, 4)
        bad = np.nonzero((got != want).any(axis=1))[0]
        assert len(bad) == 0, (sc, bad[:3].tolist(), got[bad[:3]].tolist(), want[bad[:3]].tolist())


def test_vectorised_restatement_near_the_int16_range():
    """match 90 on 300-base pairs (scores up to 27000) stays in the vector lanes; match 100
    (30000) goes to the scalar restatement; both equal it."""
    rng = random.Random(3)
    a = ["".join(rng.choice("ACGT") for _ in range(300)) for _ in range(20)]
    b = [x[: rng.randint(250, 300)] if k % 2 else x for k, x in enumerate(a)]
    p = Pairs.from_lists(a, b)
    for sc in ((90, 3, 5, 2, 2), (100, 3, 5, 2, 2)):
        assert np.array_equal(oracle.align_batch_lanes(p, sc, 2), oracle.align_batch(p, sc, 2)), sc


@pytest.mark.skipif(not oracle.reference_available(), reason="reference SSW not built (needs the reference checkout)")
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_pairs_vs_live_reference(seed):
    """Tie-heavy random pairs over small alphabets, N, lowercase and U, against the live
    reference SSW built from the reference sources."""
    rng = random.Random(seed)
    alphabets = ["ACGT", "AC", "A", "ACGTN", "acgtU", "ACGTNX"]
    a, b = [], []
    for _ in range(400):
        al = rng.choice(alphabets)
        la, lb = rng.randint(1, 60), rng.randint(1, 90)
        x = "".join(rng.choice(al) for _ in range(la))
        if rng.random() < 0.5:
            y = "".join(rng.choice(al) for _ in range(lb))
        else:
            k = rng.randint(0, lb)
            y = "".join(rng.choice(al) for _ in range(k)) + x + "".join(rng.choice(al) for _ in range(rng.randint(0, 20)))
        a.append(x)
        b.append(y)
    pairs = Pairs.from_lists(a, b)
    for sc in [(1, 3, 5, 2, 2), (2, 2, 3, 1, 2), (1, 1, 1, 1, 1), (2, 4, 4, 2, 1)]:
        got = oracle.align_batch(pairs, sc)
        want = oracle.ref_align_batch(pairs, sc)
        bad = np.nonzero((got != want).any(axis=1))[0]
        assert len(bad) == 0, (sc, [(a[i], b[i], got[i].tolist(), want[i].tolist()) for i in bad[:3]])


@pytest.mark.skipif(not oracle.reference_available(), reason="reference SSW not built (needs the reference checkout)")
def test_generated_workloads_vs_live_reference():
    from mhm2_staging_gb300 import workloads

    for cfg, n in ((0, 2000), (1, 2000), (2, 2000), (4, 100)):
        p = workloads.generate(cfg, n=n)
        got = oracle.align_batch(p)
        want = oracle.ref_align_batch(p)
        assert np.array_equal(got, want), cfg


@pytest.mark.parametrize("scoring", list(SAMPLES["scorings"]))
def test_second_best_vs_recorded_reference(scoring):
    """score2 / a_end2 (SSW's sw_score_next_best / ref_end_next_best, maskLen = max(len/2, 15))
    against the recorded reference outputs; the first five columns are unchanged."""
    recs = SAMPLES["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    out = oracle.align_batch(pairs, tuple(SAMPLES["scorings"][scoring]), score2=True)
    want = np.array([r["reference"][scoring] + r["reference_next_best"][scoring] for r in recs], dtype=np.int32)
    bad = np.nonzero((out != want).any(axis=1))[0]
    assert len(bad) == 0, [(recs[i]["set"], out[i].tolist(), want[i].tolist()) for i in bad[:3]]
    cases, kp = _kat_pairs()
    kout = oracle.align_batch(kp, tuple(KAT["scorings"][scoring]), score2=True)
    kwant = np.array([c["reference"][scoring] + c["reference_next_best"][scoring] for c in cases], dtype=np.int32)
    assert np.array_equal(kout, kwant)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference SSW not built (needs the reference checkout)")
def test_second_best_vs_live_reference():
    """Including the word path (scores >= 255 - bias with match 2) and SSW's zero-score
    query padding, which reaches into maxColumn."""
    from mhm2_staging_gb300 import workloads

    for cfg, n in ((0, 1500), (1, 3000), (2, 1500), (4, 120)):
        p = workloads.generate(cfg, n=n, first=321)
        for sc in [(1, 3, 5, 2, 2), (2, 2, 3, 1, 2), (2, 4, 4, 2, 1)]:
            got = oracle.align_batch(p, sc, score2=True)
            want = oracle.ref_align_batch(p, sc, score2=True)
            bad = np.nonzero((got != want).any(axis=1))[0]
            assert len(bad) == 0, (cfg, sc, got[bad[:2]].tolist(), want[bad[:2]].tolist())


# ---- CIGARs (report_cigar) ------------------------------------------------------------

def _cigar_rows(pairs, sc):
    out, ops, nops = oracle.cigar_batch(pairs, sc, ops_cap=1024)
    assert (nops >= 0).all()
    return out, [oracle.cigar_string(ops[i], int(nops[i])) for i in range(pairs.n)]


@pytest.mark.parametrize("scoring", TEST_SCORINGS)
def test_cigar_known_answers_of_reference_test(scoring):
    """test/ssw-test.cpp:159-236: the CIGAR strings and mismatch counts the reference's own
    unit test expects with ssw_filter_cigar (e.g. 8=1X7=, 8=1I8=, 4=1D11=, 3S16=)."""
    cases, pairs = _kat_pairs()
    out, cig = _cigar_rows(pairs, tuple(KAT["scorings"][scoring]))
    n_checked = 0
    for c, o, s in zip(cases, out.tolist(), cig):
        if c["kind"] == "aln":
            assert (s, o[5]) == (c["cigar"], c["mismatches"]), (c["query"], c["ref"], s, o)
            n_checked += 1
    assert n_checked == 17


@pytest.mark.parametrize("scoring", list(SAMPLES["scorings"]))
def test_cigar_vs_recorded_reference(scoring):
    """CIGAR strings and mismatches against the reference's recorded report_cigar output.
    Score-0 pairs are left out: there SSW's CalculateNumberMismatch reads the base before
    its reference buffer (ref += ref_begin = -1), so its output is not defined; the oracle
    returns no CIGAR for them."""
    recs = SAMPLES["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    out, cig = _cigar_rows(pairs, tuple(SAMPLES["scorings"][scoring]))
    n = 0
    for r, o, s in zip(recs, out.tolist(), cig):
        if r["reference"][scoring][0] == 0:
            assert s == "" and o[5] == 0
            continue
        assert [s, o[5]] == r["reference_cigar"][scoring], (r["set"], r["a"], r["b"], s, o)
        n += 1
    assert n >= 190
    cases, kp = _kat_pairs()
    kout, kcig = _cigar_rows(kp, tuple(KAT["scorings"][scoring]))
    for c, o, s in zip(cases, kout.tolist(), kcig):
        if c["reference"][scoring][0] > 0:
            assert [s, o[5]] == c["reference_cigar"][scoring], c


@pytest.mark.skipif(not oracle.reference_available(), reason="reference SSW not built (needs the reference checkout)")
def test_cigar_vs_live_reference():
    """Generated workloads plus indel-heavy, N-rich and unrelated pairs (bands that must
    double, boxes much longer than wide) against the live reference with report_cigar."""
    from mhm2_staging_gb300 import workloads

    rng = random.Random(11)
    a, b = [], []
    for k in range(3000):
        x = "".join(rng.choice("ACGT") for _ in range(rng.randint(1, 260)))
        if k % 4 == 0:
            y = "".join(rng.choice("ACGTN") for _ in range(rng.randint(1, 300)))
        else:
            y = []
            ind = (0.02, 0.12, 0.3)[k % 3]
            for ch in x:
                r = rng.random()
                if r < ind / 2:
                    continue
                if r < ind:
                    y.append("".join(rng.choice("ACGT") for _ in range(rng.randint(1, 6))))
                y.append(ch if rng.random() > 0.04 else rng.choice("ACGTN"))
            y = "".join(rng.choice("ACGT") for _ in range(rng.randint(0, 40))) + "".join(y) + "A"
        a.append(x)
        b.append(y)
    sets = [Pairs.from_lists(a, b)] + [workloads.generate(cfg, n=n, first=77)
                                       for cfg, n in ((0, 1500), (1, 1500), (2, 1500), (4, 60))]
    for pairs in sets:
        for sc in [(1, 3, 5, 2, 2), (2, 4, 4, 2, 1), (2, 2, 3, 1, 2)]:
            got = oracle.cigar_batch(pairs, sc, ops_cap=1024)
            want = oracle.ref_cigar_batch(pairs, sc, ops_cap=1024)
            live = want[0][:, 0] > 0
            assert np.array_equal(got[0][live], want[0][live]), sc
            assert np.array_equal(got[2][live], want[2][live]), sc
            for i in np.nonzero(live)[0]:
                k = int(got[2][i])
                assert np.array_equal(got[1][i, :k], want[1][i, :k]), (sc, i)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference SSW not built (needs the reference checkout)")
def test_equal_gap_penalties_are_outside_the_contract():
    """With gap open == gap extend SSW's striped lazy-F loop stops early and can report a
    score below the local-alignment optimum; the oracle computes the optimum.  klign's
    scorings all open gaps dearer than they extend them (5/2 and 4/2), where the two
    agree (the tests above); this records the boundary."""
    rng = random.Random(3)
    a, b = [], []
    for _ in range(3000):  # indel-heavy reads: scores on SSW's word path, long gaps
        x = "".join(rng.choice("ACGT") for _ in range(rng.randint(150, 300)))
        y = []
        for ch in x:
            r = rng.random()
            if r < 0.125:
                continue
            if r < 0.25:
                y.append("".join(rng.choice("ACGT") for _ in range(rng.randint(1, 8))))
            y.append(ch if rng.random() > 0.02 else rng.choice("ACGT"))
        a.append(x)
        b.append("".join(y))
    pairs = Pairs.from_lists(a, b)
    got = oracle.align_batch(pairs, (2, 2, 2, 2, 2))
    want = oracle.ref_align_batch(pairs, (2, 2, 2, 2, 2))
    assert (got[:, 0] >= want[:, 0]).all()
    assert (got[:, 0] > want[:, 0]).any()
    assert np.array_equal(oracle.align_batch(pairs, (2, 2, 3, 2, 2)), oracle.ref_align_batch(pairs, (2, 2, 3, 2, 2)))


# ---- protein ---------------------------------------------------------------------------

PROT = json.loads((GOLDEN / "ssw_protein_samples.json").read_text())


@pytest.mark.parametrize("gaps", PROT["gaps"])
def test_protein_oracle_vs_recorded_reference(gaps):
    """The protein restatement against the reference SSW's recorded outputs (a seeded
    24 x 24 matrix, 240 pairs incl. unrelated and mutated ones)."""
    recs = PROT["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    out = oracle.protein_batch(pairs, np.array(PROT["matrix"], np.int16), np.array(PROT["encoding"], np.int16),
                               *gaps)
    want = np.array([r["reference"][f"{gaps[0]}/{gaps[1]}"] for r in recs], dtype=np.int32)
    assert np.array_equal(out, want)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference SSW not built (needs the reference checkout)")
def test_protein_oracle_vs_live_reference():
    rng = random.Random(7)
    letters = oracle.PROTEIN_LETTERS
    a, b = [], []
    for k in range(1500):
        x = "".join(rng.choice(letters) for _ in range(rng.randint(1, 300)))
        y = x[rng.randint(0, len(x) - 1):] if k % 2 else "".join(rng.choice(letters) for _ in range(rng.randint(1, 300)))
        a.append(x)
        b.append(y + rng.choice(letters))
    pairs = Pairs.from_lists(a, b)
    nr = np.random.default_rng(5)
    m = nr.integers(-3, 3, (24, 24))
    m = (np.triu(m) + np.triu(m, 1).T).astype(np.int16)
    np.fill_diagonal(m, nr.integers(3, 9, 24))
    enc = oracle.protein_encoding()
    for go, ge in ((11, 1), (7, 3), (4, 1)):
        assert np.array_equal(oracle.protein_batch(pairs, m, enc, go, ge), oracle.ref_protein_batch(pairs, m, enc, go, ge))


def _config0_record():
    rec = np.load(GOLDEN / "ssw_reference_config0.npz")
    return rec["out"], tuple(int(x) for x in rec["scoring"])


def test_config0_record_vs_oracle():
    """The recorded reference outputs of the 150/300 bp workload (all 10,000 pairs, score2
    fields included) equal the oracle's."""
    from mhm2_staging_gb300 import workloads

    want, sc = _config0_record()
    pairs = workloads.generate(0)
    assert np.array_equal(oracle.align_batch(pairs, sc, score2=True), want)


def test_sse2_shim_build_vs_sse2_build():
    """The reference SSW compiled through oracle/sse2_shim (its portable vector form, on
    this x86_64 host) gives what the genuine SSE2 build gives, on the 150/300 bp workload
    and on samples of the others."""
    from mhm2_staging_gb300 import workloads

    if not (oracle.reference_available() and oracle.REF_SHIM_SO.exists()):
        pytest.skip("needs the reference checkout on x86_64 (SSE2 build and its shim twin)")
    want, sc = _config0_record()
    assert np.array_equal(oracle.ref_align_batch(workloads.generate(0), sc, score2=True,
                                                 lib=oracle.REF_SHIM_SO), want)
    for cfg, n in ((1, 5000), (2, 5000), (4, 500)):
        p = workloads.generate(cfg, n=n, first=7000)
        assert np.array_equal(oracle.ref_align_batch(p, sc, score2=True, lib=oracle.REF_SHIM_SO),
                              oracle.ref_align_batch(p, sc, score2=True)), cfg


@pytest.mark.parametrize("host", ["build_container", pytest.param("gpu_host", marks=pytest.mark.gpu)])
def test_reference_build_vs_x86_record(host):
    """Whatever build of the reference SSW this host has -- SSE2 on x86_64, the NEON shim
    on the GPU host's aarch64 -- reproduces the x86_64 SSE2 record of the 150/300 bp
    workload bit for bit (the GPU-marked case runs where the GPU tests run, the host
    that times the reference as the CPU baseline)."""
    from mhm2_staging_gb300 import workloads

    if not oracle.reference_available():
        pytest.skip("reference SSW not built on this host")
    want, sc = _config0_record()
    got = oracle.ref_align_batch(workloads.generate(0), sc, score2=True)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert len(bad) == 0, f"{oracle.reference_build_kind()}: {len(bad)} pairs differ; first {bad[:5].tolist()}"
