"""Serving form on the GPU: resident contigs, budgeted admission, continuous batching.

Every result is checked bit-exact against the oracle on the same (read, window) pairs,
and a request batch gives the same results alone and mixed with concurrent traffic.
"""
import threading

import numpy as np
import pytest

from mhm2_staging_gb300 import serving as S
from oracle import oracle

pytestmark = pytest.mark.gpu
SC = (1, 3, 5, 2, 2)


@pytest.fixture(scope="module")
def contigs(built):
    return S.generate_contigs(16 << 20, seed=3)


@pytest.fixture(scope="module")
def requests(contigs):
    return S.generate_requests(contigs, 24000, seed=7)


def _want(contigs, req, flank=200):
    pairs, ws = S.windows(contigs, req, flank)
    return oracle.align_batch(pairs, SC), ws


def _diff(got, want):
    bad = np.nonzero((got != want).any(axis=1))[0]
    if len(bad):
        i = int(bad[0])
        return f"{len(bad)} of {len(got)} differ; first {i}: server={got[i].tolist()} oracle={want[i].tolist()}"
    return ""


def test_server_matches_oracle_on_uneven_batches(contigs, requests):
    srv = S.Server(slots=3, max_pairs_per_batch=4096)
    srv.load_contigs(contigs)
    cuts = [0, 1, 1000, 1003, 9000, 9001, 17000, requests.n]  # includes 1-pair and empty batches
    tickets = [srv.submit(requests.slice(a, b)) for a, b in zip(cuts[:-1], cuts[1:])]
    got = [srv.wait(t) for t in tickets]
    out5 = np.concatenate([g[0] for g in got])
    ws = np.concatenate([g[1] for g in got])
    want, wsw = _want(contigs, requests)
    assert not _diff(out5, want)
    assert np.array_equal(ws, wsw)
    st = srv.stats()
    assert st["pairs_done"] == requests.n and st["completed"] == len(tickets)
    assert st["micro_batches"] >= requests.n // 4096
    srv.close()


def test_reads_in_any_order_of_the_callers_buffer(contigs, requests):
    """Request batches whose reads are not one run of the caller's buffer (a permuted
    subset: each read packed on its own), and contiguous slices (packed as one run), mixed
    in the same micro-batches: both match the oracle."""
    srv = S.Server(slots=2, max_pairs_per_batch=3000)
    srv.load_contigs(contigs)
    rng = np.random.default_rng(11)
    batches = [requests.subset(rng.permutation(np.arange(2000, 4500))), requests.slice(100, 1900),
               requests.subset(np.arange(12000, 8000, -1)), requests.slice(20000, 21000)]
    tickets = [srv.submit(b) for b in batches]
    for b, t in zip(batches, tickets):
        out5, ws = srv.wait(t)[:2]
        want, wsw = _want(contigs, b)
        assert not _diff(out5, want)
        assert np.array_equal(ws, wsw)
    srv.close()


@pytest.mark.parametrize("form", [0, 1])
def test_same_result_alone_and_in_the_mix(contigs, requests, form):
    probe = requests.slice(5000, 6500)
    others = [requests.slice(a, a + 2500) for a in range(7000, 24000, 2500)]
    # alone: a fresh server with nothing else in flight
    srv = S.Server(slots=3, max_pairs_per_batch=1024, form=form)
    srv.load_contigs(contigs)
    alone, ws_alone, _ = srv.wait(srv.submit(probe))
    # in the mix: concurrent submitters keep every slot busy; the probe is split across
    # micro-batches shared with the other requests and overlaps them on the device
    results = {}

    def feed(k, batches):
        ts = [srv.submit(b) for b in batches]
        results[k] = [srv.wait(t)[0] for t in ts]

    threads = [threading.Thread(target=feed, args=(k, others[k::3])) for k in range(3)]
    for th in threads:
        th.start()
    mixed_t = srv.submit(probe)
    for th in threads:
        th.join()
    mixed, ws_mixed, times = srv.wait(mixed_t)
    assert np.array_equal(alone, mixed) and np.array_equal(ws_alone, ws_mixed)
    want, _ = _want(contigs, probe)
    assert not _diff(mixed, want)
    for k in range(3):
        for b, got in zip(others[k::3], results[k]):
            w, _ = _want(contigs, b)
            assert not _diff(got, w)
    assert times[0] <= times[1] <= times[2]
    srv.close()


def test_admission_by_queue_budget(contigs, requests):
    big = requests.slice(0, 20000)
    small = requests.slice(20000, 20010)
    srv = S.Server(slots=1, max_pairs_per_batch=2048, queue_budget=64 << 10)
    srv.load_contigs(contigs)
    t1 = srv.submit(big)  # admitted although larger than the budget: nothing else in flight
    assert srv.submit(small, wait_for_room=False) is None  # queue full: refused, not queued
    t2 = srv.submit(small)  # waits for room, then runs
    o1 = srv.wait(t1)[0]
    o2 = srv.wait(t2)[0]
    w1, _ = _want(contigs, big)
    w2, _ = _want(contigs, small)
    assert not _diff(o1, w1) and not _diff(o2, w2)
    srv.close()


def test_budget_sizes_the_slots(contigs):
    srv = S.Server(slots=8, max_pairs_per_batch=65536, hbm_budget=(16 << 20) + (96 << 20))
    srv.load_contigs(contigs)
    st = srv.stats()
    assert 1 <= st["slots"] < 8 and st["device_bytes"] <= (16 << 20) + (96 << 20) + (1 << 20)
    srv.close()
    with pytest.raises(RuntimeError, match="status 4"):
        tiny = S.Server(hbm_budget=1 << 20)
        tiny.load_contigs(contigs)


def test_bad_requests_are_rejected(contigs, requests):
    srv = S.Server(slots=1)
    srv.load_contigs(contigs)
    bad = requests.slice(0, 3)
    bad.cid[1] = contigs.n + 5
    with pytest.raises(RuntimeError, match="status 2"):
        srv.submit(bad)
    bad = requests.slice(0, 3)
    bad.pos[2] = contigs.len[bad.cid[2]]
    with pytest.raises(RuntimeError, match="status 2"):
        srv.submit(bad)
    srv.close()


def test_full_size_contig_set_with_concurrent_batches(built):
    """The serving workload's own contig set (200 MB, lognormal lengths up to 200 kb)
    resident on the device; request batches of 1k..64k submitted together from several
    threads (their micro-batches overlap on the device), every result bit-exact against
    the oracle on the same (read, window) pairs."""
    big = S.generate_contigs(200 << 20, seed=3)
    req = S.generate_requests(big, 60000, seed=11)
    srv = S.Server(slots=3, max_pairs_per_batch=65536)
    srv.load_contigs(big)
    cuts = [0, 1024, 9000, 42000, 60000]
    out = [None] * (len(cuts) - 1)

    def one(k):
        out[k] = srv.wait(srv.submit(req.slice(cuts[k], cuts[k + 1])))

    th = [threading.Thread(target=one, args=(k,)) for k in range(len(cuts) - 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    out5 = np.concatenate([o[0] for o in out])
    want, _ = _want(big, req)
    assert not _diff(out5, want)
    srv.close()
