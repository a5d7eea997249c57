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
