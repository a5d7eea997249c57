"""GPU results against the reference's golden vectors (tests/golden/, made from the reference
test file and the reference SSW), through the C ABI."""
import json
from pathlib import Path

import numpy as np
import pytest

from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, GPUDriver, ORIENT_REF_IS_A, Pairs

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "ssw_known_answers.json").read_text())
SAMPLES = json.loads((GOLDEN / "ssw_reference_samples.json").read_text())


def _driver(sc, orientation=None):
    m, x, go, ge, amb = sc
    d = GPUDriver()
    d.set_ambiguity(-amb)
    d.init(0, 1, m, -x, -go, -ge, 300)
    if orientation is not None:
        d.set_orientation(orientation)
    return d


@pytest.mark.parametrize("scoring", ["ssw_default", "mhm2_aln", "cigar"])
def test_reference_unit_test_through_dropin(built, scoring):
    """TEST(MHMTest, AdeptSW) (test/ssw-test.cpp:241-431) with the test's call sequence:
    run_kernel_forwards(query, ref) -> block -> backwards -> block, results translated as
    translate_adept_to_ssw (:22-40) does; expectations of the CPU test (:151-238)."""
    d = _driver(KAT["scorings"][scoring], ORIENT_REF_IS_A)
    cases = KAT["cases"]
    queries = [c["query"] for c in cases]
    refs = [c["ref"] for c in cases]
    mq, mr = max(map(len, queries)), max(map(len, refs))
    d.run_kernel_forwards(queries, refs, mq, mr)
    d.kernel_block()
    d.run_kernel_backwards(queries, refs, mq, mr)
    d.kernel_block()
    r = d.get_aln_results()
    for i, c in enumerate(cases):
        got = (int(r.query_begin[i]), int(r.query_end[i]), int(r.ref_begin[i]), int(r.ref_end[i]))
        if c["kind"] == "aln":
            assert got == (c["qbegin"], c["qend"], c["rbegin"], c["rend"]), (i, c["query"], c["ref"], got)
        else:
            assert got[3] - got[2] <= 3 and got[1] - got[0] <= 3 and int(r.top_scores[i]) <= 4
        sc, ab, ae, bb, be = c["reference"][scoring]
        assert (int(r.top_scores[i]), int(r.ref_begin[i]), int(r.ref_end[i]), int(r.query_begin[i]),
                int(r.query_end[i])) == (sc, ab, ae, bb, be)


@pytest.mark.parametrize("scoring", list(SAMPLES["scorings"]))
@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
def test_recorded_reference_samples(built, scoring, form):
    recs = SAMPLES["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    d = _driver(SAMPLES["scorings"][scoring])
    got = d.align_pairs(pairs, form=form)
    want = np.array([r["reference"][scoring] for r in recs], dtype=np.int32)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert len(bad) == 0, [(recs[i]["set"], got[i].tolist(), want[i].tolist()) for i in bad[:3]]
