"""The allocation-free forward entry point, mhsw_forward_noalloc, through the C ABI.

Compared with the driver's entry point (mhsw_align_pairs: score, a_end and b_end are
columns 0, 2 and 4 of its result) and with the oracle on the same device-resident batch,
on two calls in a row, so the second call runs on scratch the first one left behind.
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


def _run_twice(pairs: Pairs, want: np.ndarray, torch, max_a: int | None = None, max_b: int | None = None):
    dp, keep = _upload(pairs, torch)
    if max_a:
        dp.max_a_len, dp.max_b_len = max_a, max_b
    out3 = torch.full((pairs.n, 3), -7, dtype=torch.int32, device="cuda:0")
    for call in range(2):
        out3.fill_(-7)
        torch.cuda.synchronize()
        D.forward_noalloc(dp, out3.data_ptr(), SCORES)
        torch.cuda.synchronize()
        got = out3.cpu().numpy()
        bad = np.nonzero((got != want).any(axis=1))[0]
        assert len(bad) == 0, (f"call {call}: {len(bad)} of {pairs.n} differ; first {int(bad[0])}: "
                               f"noalloc={got[bad[0]].tolist()} want={want[bad[0]].tolist()}")
    del keep


def test_noalloc_matches_oracle_twice(gpu):
    from oracle import oracle

    torch = pytest.importorskip("torch")
    pairs = _batch()
    _run_twice(pairs, oracle.align_batch(pairs, tuple(abs(x) for x in SCORES))[:, [0, 2, 4]], torch)


def test_noalloc_scratch_reused_within_a_call(gpu):
    """Stated maxima far above the pairs' own lengths (500,000 A, 60,000 B bytes) leave
    room in the scratch array for only a few dozen lane groups, so each group aligns many
    pairs of a call one after another on its own share: mixed lengths, A of several
    strips, B of tens of thousands of bases.  (The entry point's limits leave room for at
    least 19 groups, so a block never has fewer than its 8 groups.)"""
    from oracle import oracle

    torch = pytest.importorskip("torch")
    parts = [workloads.generate(2, n=1500, first=77), workloads.generate(1, n=400, first=9)]
    a = [p.a(i) for p in parts for i in range(p.n)]
    b = [p.b(i) for p in parts for i in range(p.n)]
    rng = np.random.default_rng(5)
    def bases(k: int) -> bytes:
        return np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, k)].tobytes()

    for la, lb in ((300, 50000), (2000, 20000), (5000, 6000), (130, 59000)):
        read = bases(la)
        a.append(read)
        b.append(bases(lb // 2) + read + bases(max(lb - lb // 2 - la, 10)))
    pairs = Pairs.from_lists(a, b)
    want = oracle.align_batch(pairs, tuple(abs(x) for x in SCORES))[:, [0, 2, 4]]
    _run_twice(pairs, want, torch, max_a=500_000, max_b=60_000)


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
