"""The allocation-free forward entry point, mhsw_forward_noalloc, through the C ABI.

Compared with the driver's entry point (mhsw_align_pairs: score, a_end and b_end are
columns 0, 2 and 4 of its result) on the same device-resident batch, on two calls in a
row, so the second call runs on scratch the first one left behind.
"""
import ctypes as C

import numpy as np
import pytest

from mhm2_staging_gb300 import Pairs, workloads
from mhm2_staging_gb300 import driver as D

pytestmark = pytest.mark.gpu
SCORES = (1, -3, -5, -2, -2)


def _batch() -> Pairs:
    parts = [workloads.generate(1, n=1200, first=500), workloads.generate(4, n=40, first=900),
             workloads.generate(2, n=600, first=321)]
    a = [p.a(i) for p in parts for i in range(p.n)]
    b = [p.b(i) for p in parts for i in range(p.n)]
    # edge cases: empty sides, all-N, lowercase, a single base, A longer than many strips
    a += [b"", b"ACGT", b"NNNNNNNN", b"acgtacgtac", b"A", b"ACGTTGCA" * 80]
    b += [b"ACGT", b"", b"ACGTNNAC", b"ACGTACGTAC", b"A", b"TGCAACGT" * 60]
    return Pairs.from_lists(a, b)


def _upload(pairs: Pairs, torch):
    dev = torch.device("cuda:0")
    tens = [torch.from_numpy(x).to(dev) for x in
            (pairs.a_seq, pairs.a_off, pairs.a_len, pairs.b_seq, pairs.b_off, pairs.b_len)]
    dp = D.DevicePairs(*(t.data_ptr() for t in tens), n=pairs.n, max_a_len=int(pairs.a_len.max()),
                       max_b_len=int(pairs.b_len.max()))
    return dp, tens


def test_noalloc_matches_align_pairs_twice(gpu):
    torch = pytest.importorskip("torch")
    pairs = _batch()
    want = gpu.align_pairs(pairs)[:, [0, 2, 4]]
    dp, keep = _upload(pairs, torch)
    out3 = torch.full((pairs.n, 3), -7, dtype=torch.int32, device="cuda:0")
    for call in range(2):
        out3.fill_(-7)
        torch.cuda.synchronize()
        D.forward_noalloc(dp, out3.data_ptr(), SCORES)
        torch.cuda.synchronize()
        got = out3.cpu().numpy()
        bad = np.nonzero((got != want).any(axis=1))[0]
        assert len(bad) == 0, (f"call {call}: {len(bad)} of {pairs.n} differ; first {int(bad[0])}: "
                               f"noalloc={got[bad[0]].tolist()} align_pairs={want[bad[0]].tolist()}")
    del keep


def test_noalloc_limits(gpu):
    torch = pytest.importorskip("torch")
    lib = D.load_library()
    pairs = Pairs.from_lists([b"ACGTACGTAC", b"ACGTACGTACGT"], [b"ACGTACGTAC", b"ACGTACGTACGTACGT"])
    dp, keep = _upload(pairs, torch)
    out3 = torch.full((pairs.n, 3), -7, dtype=torch.int32, device="cuda:0")
    err = C.create_string_buffer(256)
    # stated maxima beyond the limits: rejected before any launch
    dp.max_b_len = 70000
    pt = dp.c_struct()
    rc = lib.mhsw_forward_noalloc(C.byref(pt), *SCORES, D._P(out3.data_ptr()), None, err, len(err))
    assert rc == 5 and b"max_b_len" in err.value  # MHSW_ERR_LIMIT
    # the stated maxima are required
    dp.max_b_len = 0
    pt = dp.c_struct()
    assert lib.mhsw_forward_noalloc(C.byref(pt), *SCORES, D._P(out3.data_ptr()), None, err, len(err)) == 2
    # a pair longer than the stated maxima gets -1, -1, -1; the other is aligned
    dp.max_a_len, dp.max_b_len = 10, 10
    D.forward_noalloc(dp, out3.data_ptr(), SCORES)
    torch.cuda.synchronize()
    got = out3.cpu().numpy()
    assert got[0].tolist() == [10, 9, 9]
    assert got[1].tolist() == [-1, -1, -1]
    del keep
