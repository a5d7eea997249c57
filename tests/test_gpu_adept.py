"""The same-GPU comparator: ADEPT's own kernels (compiled for sm_103a from the reference
sources into oracle/_ref) launched as the reference driver launches them.  ADEPT is not
bit-exact with SSW, but on inputs without N its top scores are SSW's; agreement on
nearly every pair shows the launches (packing, shapes, score signs) are the reference's."""
import numpy as np
import pytest

from mhm2_staging_gb300 import workloads
from oracle import adept, oracle

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(not adept.available(), reason="ADEPT cubin not built (needs the reference checkout)")
@pytest.mark.parametrize("cfg,n", [(0, 10000), (2, 5000)])
def test_adept_top_scores_match_ssw(built, cfg, n):
    pairs = workloads.generate(cfg, n=n)
    ad = adept.Adept(0)
    batch = ad.upload(pairs)
    ad.run(batch, (1, 3, 5, 2, 2))
    got = ad.scores(batch)
    want = oracle.align_batch(pairs, (1, 3, 5, 2, 2))[:, 0]
    assert (got == want).mean() > 0.99
