"""Score2 mode on the GPU: SSW's second-best score (sw_score_next_best, ref_end_next_best)
bit-exact against the oracle and the recorded reference outputs, through the C ABI."""
import json
from pathlib import Path

import numpy as np
import pytest

from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, GPUDriver, Pairs, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _driver(scoring=(1, 3, 5, 2, 2)):
    m, x, go, ge, amb = scoring
    d = GPUDriver()
    d.init(0, 1, m, -x, -go, -ge, 0)
    d.set_ambiguity(-amb)
    d.set_score2(True)
    return d


def _run(d, pairs, form):
    out5 = d.align_pairs(pairs, form=form)
    return np.concatenate([out5, d.last_score2(pairs.n)], axis=1)


def _diff(got, want):
    bad = np.nonzero((got != want).any(axis=1))[0]
    if len(bad):
        i = int(bad[0])
        return f"{len(bad)} of {len(got)} differ; first {i}: gpu={got[i].tolist()} oracle={want[i].tolist()}"
    return ""


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
@pytest.mark.parametrize("cfg,n", [(0, 10000), (1, 8000), (2, 8000), (4, 400)])
def test_score2_matches_oracle(built, cfg, n, form):
    pairs = workloads.generate(cfg, n=n, first=2024)
    want = oracle.align_batch(pairs, (1, 3, 5, 2, 2), score2=True)
    assert not _diff(_run(_driver(), pairs, form), want)


@pytest.mark.parametrize("seed", range(8))
def test_score2_random_scorings(built, seed):
    """Randomly drawn scorings (match 1-4, mismatch 1-8, gap open 1-10, gap extend 1-10,
    ambiguity 0-6): SSW's byte or word path (its bias is the largest penalty of the
    substitution matrix) per pair, both forms, against the oracle."""
    import random

    rng = random.Random(3000 + seed)
    sc = (rng.randint(1, 4), rng.randint(1, 8), rng.randint(1, 10), rng.randint(1, 10), rng.randint(0, 6))
    pairs = workloads.generate(1 if seed % 2 else 2, n=2500, seed=seed)
    want = oracle.align_batch(pairs, sc, score2=True)
    for form in (FORM_PLAIN, FORM_BATCHED):
        assert not _diff(_run(_driver(sc), pairs, form), want), (sc, form)


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
def test_score2_word_path_and_int32(built, form):
    """Match 2 on 250 bp reads: scores past 255 - bias take SSW's word path (padding to a
    multiple of 8, recomputed by the int32 engine); then every pair forced into int32."""
    sc = (2, 2, 3, 1, 2)
    pairs = workloads.generate(4, n=300, first=77)
    want = oracle.align_batch(pairs, sc, score2=True)
    assert (want[:, 0] + 2 >= 255).any()
    d = _driver(sc)
    assert not _diff(_run(d, pairs, form), want)
    d.set_int16_ceiling(40)
    assert not _diff(_run(d, pairs, form), want)


def test_score2_long_a_strips(built):
    src = workloads.generate(4, n=48, first=9)
    a = [src.b(i)[:300 + 41 * i] for i in range(48)]  # A longer than one wavefront strip
    b = [src.a(i) for i in range(48)]
    pairs = Pairs.from_lists(a, b)
    want = oracle.align_batch(pairs, (1, 3, 5, 2, 2), score2=True)
    d = _driver()
    for form in (FORM_PLAIN, FORM_BATCHED):
        assert not _diff(_run(d, pairs, form), want)


@pytest.mark.parametrize("scoring", ["ssw_default", "mhm2_aln", "cigar", "measured"])
def test_score2_recorded_reference(built, scoring):
    samples = json.loads((GOLDEN / "ssw_reference_samples.json").read_text())
    recs = samples["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    want = np.array([r["reference"][scoring] + r["reference_next_best"][scoring] for r in recs], dtype=np.int32)
    d = _driver(tuple(samples["scorings"][scoring]))
    for form in (FORM_PLAIN, FORM_BATCHED):
        assert not _diff(_run(d, pairs, form), want), form


def test_score2_through_dropin_protocol(built):
    pairs = workloads.generate(1, n=2000, first=31)
    reads = [pairs.a(i) for i in range(pairs.n)]
    ctgs = [pairs.b(i) for i in range(pairs.n)]
    want = oracle.align_batch(pairs, (1, 3, 5, 2, 2), score2=True)
    d = _driver()
    d.run_kernel_forwards(reads, ctgs, max(map(len, reads)), max(map(len, ctgs)))
    d.kernel_block()
    r = d.get_aln_results()
    assert np.array_equal(r.score2, want[:, 5]) and np.array_equal(r.a_end2, want[:, 6])
    d.run_kernel_backwards(reads, ctgs, max(map(len, reads)), max(map(len, ctgs)))
    d.kernel_block()
    r = d.get_aln_results()
    got = np.stack([r.top_scores32, r.query_begin32, r.query_end32, r.ref_begin32, r.ref_end32], axis=1)
    assert not _diff(got, want[:, :5])
    # off again: the default path, no score2 views
    d.set_score2(False)
    d.run_kernel_forwards(reads, ctgs, max(map(len, reads)), max(map(len, ctgs)))
    d.kernel_block()
    assert d.get_aln_results().score2 is None
