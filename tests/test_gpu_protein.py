"""Protein alignment on the GPU (mhsw_align_protein): score and coordinates bit-exact
against the reference SSW's recorded outputs and the oracle, through the C ABI."""
import ctypes as C
import json
import random
from pathlib import Path

import numpy as np
import pytest

from mhm2_staging_gb300 import GPUDriver, Pairs
from oracle import oracle

pytestmark = pytest.mark.gpu
PROT = json.loads((Path(__file__).resolve().parent / "golden" / "ssw_protein_samples.json").read_text())
MAT = np.array(PROT["matrix"], np.int16)
ENC = np.array(PROT["encoding"], np.int16)


def _driver(go=11, ge=1):
    d = GPUDriver()
    d.init(0, 1, 1, -1, -go, -ge, 0)  # match/mismatch unused by the protein path
    return d


def _diff(got, want):
    bad = np.nonzero((got != want).any(axis=1))[0]
    if len(bad):
        i = int(bad[0])
        return f"{len(bad)} of {len(got)} differ; first {i}: gpu={got[i].tolist()} oracle={want[i].tolist()}"
    return ""


@pytest.mark.parametrize("gaps", PROT["gaps"])
def test_protein_recorded_reference(built, gaps):
    recs = PROT["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    want = np.array([r["reference"][f"{gaps[0]}/{gaps[1]}"] for r in recs], dtype=np.int32)
    assert not _diff(_driver(*gaps).align_protein(pairs, MAT, ENC), want)


def _proteins(n, seed, lo, hi):
    rng = random.Random(seed)
    L = oracle.PROTEIN_LETTERS
    a, b = [], []
    for k in range(n):
        x = "".join(rng.choice(L) for _ in range(rng.randint(lo, hi)))
        if k % 3 == 0:
            y = "".join(rng.choice(L) for _ in range(rng.randint(lo, hi)))
        else:
            y = "".join(c if rng.random() > 0.1 else rng.choice(L) for c in x if rng.random() > 0.02)
            y = "".join(rng.choice(L) for _ in range(rng.randint(0, 30))) + y + "W"
        a.append(x)
        b.append(y)
    return Pairs.from_lists(a, b)


@pytest.mark.parametrize("lo,hi,n", [(1, 40, 3000), (100, 600, 2000), (600, 3000, 40)])
def test_protein_matches_oracle(built, lo, hi, n):
    """Short, typical and long proteins (A over several 256-row strips)."""
    pairs = _proteins(n, lo, lo, hi)
    for go, ge in ((11, 1), (5, 2)):
        want = oracle.protein_batch(pairs, MAT, ENC, go, ge)
        assert not _diff(_driver(go, ge).align_protein(pairs, MAT, ENC), want), (go, ge)


def test_protein_call_arena_grows_and_is_reused(built):
    """One handle, batches of growing then shrinking size: the call arena kept on the handle
    grows for the larger batch and is reused by the smaller ones."""
    d = _driver()
    for n, hi in ((50, 120), (3000, 500), (50, 120), (7, 60)):
        pairs = _proteins(n, n + hi, 20, hi)
        assert not _diff(d.align_protein(pairs, MAT, ENC), oracle.protein_batch(pairs, MAT, ENC, 11, 1)), n


def test_protein_device_resident_batch(built):
    torch = pytest.importorskip("torch")
    from mhm2_staging_gb300.driver import DevicePairs

    pairs = _proteins(500, 9, 50, 400)
    dev = torch.device("cuda:0")
    tens = [torch.from_numpy(x).to(dev) for x in (pairs.a_seq, pairs.a_off, pairs.a_len, pairs.b_seq, pairs.b_off,
                                                 pairs.b_len)]
    dp = DevicePairs(*(t.data_ptr() for t in tens), n=pairs.n)
    out = torch.zeros((pairs.n, 5), dtype=torch.int32, device=dev)
    d = _driver()
    mat = np.ascontiguousarray(MAT.reshape(-1))
    pt = dp.c_struct()
    rc = d._lib.mhsw_align_protein(d._h, C.byref(pt), mat.ctypes.data, ENC.ctypes.data, out.data_ptr(), 0)
    assert rc == 0
    assert not _diff(out.cpu().numpy(), oracle.protein_batch(pairs, MAT, ENC, 11, 1))


def test_protein_rejects_bad_input(built):
    d = _driver()
    pairs = Pairs.from_lists(["ACDEFGHIK", "MKV" + chr(120)], ["ACDEFGHIK", "MKVL"])  # 'x' is >= 91
    with pytest.raises(RuntimeError, match="status 2"):
        d.align_protein(pairs, MAT, ENC)
    enc = ENC.copy()
    enc[65] = 30
    with pytest.raises(RuntimeError, match="status 2"):
        d.align_protein(Pairs.from_lists(["AC"], ["AC"]), MAT, enc)
    # still usable; empty batch
    assert d.align_protein(Pairs.from_lists([], []), MAT, ENC).shape == (0, 5)
    ok = Pairs.from_lists(["ACDEFGHIK"], ["ACDEFGHIK"])
    assert not _diff(d.align_protein(ok, MAT, ENC), oracle.protein_batch(ok, MAT, ENC, 11, 1))
