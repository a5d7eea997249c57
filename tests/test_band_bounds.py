"""The begin pass's band placement: every alignment the oracle reports (its CIGAR from SSW's
traceback) keeps its vertical and horizontal gap cells within the two side bounds the
band kernels place their band by (band_sides in mhm2_staging_gb300/csrc/mhsw_kernels.cu,
restated here), at the row count the alignment spans.  A CPU check of the bound's
derivation; the GPU parity tests check the kernels themselves."""
import numpy as np
import pytest

from mhm2_staging_gb300 import workloads
from oracle import oracle

# BAM op codes.  The oracle's CIGARs are SSW's, where A is on the reference side: a D op
# takes rows of A with no column of B (a vertical gap), an I op columns of B alone.
BAM_I, BAM_D = 1, 2


def band_sides(t: int, n2: int, s: int, sc) -> tuple[int, int, int]:
    """(I, J, g): the vertical and horizontal drift bounds and the total gap bound of an
    alignment scoring s within t rows of A and n2 columns of B."""
    m, _x, go, ge, _amb = sc
    gmin = min(go, ge)
    g1 = gmin if gmin > 0 else 1
    c = max(go - ge, 0)
    slack = min(t, n2) * m - s - c
    g = 0 if slack < g1 else slack // g1
    mg = m + g1
    st, sn = t * m - s - c, n2 * m - s - c
    i_b = 0 if st < mg else st // mg
    j_b = 0 if sn < mg else sn // mg
    return min(i_b, g), min(j_b, g), g


@pytest.mark.parametrize("cfg,sc", [(2, (1, 3, 5, 2, 2)), (1, (1, 3, 5, 2, 2)), (2, (2, 4, 4, 2, 1)),
                                    (1, (3, 2, 6, 1, 2)), (2, (20, 3, 5, 2, 2))])
def test_alignment_gaps_within_side_bounds(cfg, sc):
    pairs = workloads.generate(cfg, n=4000, seed=77)
    out, ops, nops = oracle.cigar_batch(pairs, sc, ops_cap=512)
    checked = tighter = skipped = 0
    for p in range(pairs.n):
        s, ib, ie, jb, je = (int(v) for v in out[p, :5])
        if s <= 0 or nops[p] <= 0:
            continue
        code = ops[p, :nops[p]]
        lens, kinds = code >> 4, code & 15
        vert = int(lens[kinds == BAM_D].sum())
        horiz = int(lens[kinds == BAM_I].sum())
        rows = ie - ib + 1
        if rows != int(lens[(kinds == 0) | (kinds == 7) | (kinds == 8)].sum()) + vert:
            skipped += 1  # SSW's banded traceback can end short of the begin (its CIGAR then
            continue      # spans fewer rows than the coordinates); the oracle keeps that
        i_b, j_b, g = band_sides(rows, je + 1, s, sc)
        assert vert <= i_b and horiz <= j_b, (p, sc, s, vert, horiz, i_b, j_b)
        checked += 1
        tighter += i_b + j_b < 2 * g
    assert checked > 1000 and skipped < checked // 100
    assert tighter > 0  # the two-sided band is narrower than the symmetric one for some pairs
