"""Serving workload and server host-side behaviour without a GPU."""
import numpy as np
import pytest

from mhm2_staging_gb300 import driver as D
from mhm2_staging_gb300 import serving as S
from oracle import oracle


@pytest.fixture(scope="module")
def contigs(built):
    return S.generate_contigs(4 << 20, seed=3)


def test_contig_lengths_and_determinism(contigs):
    assert contigs.len.min() >= 200 and contigs.len.max() <= 200000
    assert int(contigs.len.astype(np.int64).sum()) >= 4 << 20
    again = S.generate_contigs(4 << 20, seed=3)
    assert np.array_equal(again.len, contigs.len) and np.array_equal(again.seq, contigs.seq)
    assert set(np.unique(contigs.seq[:-1])) <= set(b"ACGT")


def test_requests_slices_and_windows(contigs):
    r = S.generate_requests(contigs, 3000, seed=5)
    assert r.len.min() >= 1 and r.len.max() <= 260
    part = S.generate_requests(contigs, 100, seed=5, first=1500)
    assert np.array_equal(part.len, r.len[1500:1600]) and np.array_equal(part.pos, r.pos[1500:1600])
    for k in range(0, 100, 7):
        i = 1500 + k
        a = part.seq[part.off[k]:part.off[k] + part.len[k]]
        b = r.seq[r.off[i]:r.off[i] + r.len[i]]
        assert np.array_equal(a, b)
    pairs, ws = S.windows(contigs, r, flank=200)
    cl = contigs.len[r.cid]
    assert (r.pos >= 0).all() and (r.pos < cl).all()
    assert (ws == np.maximum(0, r.pos - 200)).all()
    assert (ws + pairs.b_len == np.minimum(cl, r.pos.astype(np.int64) + r.len + 200)).all()
    # reads come from their seed-hit windows: most align near-perfectly
    out = oracle.align_batch(pairs.subset(np.arange(300)), (1, 3, 5, 2, 2))
    frac = out[:, 0] / np.maximum(1, pairs.a_len[:300])
    assert np.median(frac) > 0.8


def test_server_needs_a_gpu_or_loaded_contigs(built):
    if D.get_num_node_gpus() == 0:
        with pytest.raises(RuntimeError, match="status 6"):
            S.Server()
    else:
        srv = S.Server(slots=1)
        r = S.Requests(np.frombuffer(b"ACGT\0", dtype=np.uint8).copy(), np.zeros(1, np.int64),
                       np.full(1, 4, np.int32), np.zeros(1, np.int32), np.zeros(1, np.int32))
        with pytest.raises(RuntimeError, match="status 3"):
            srv.submit(r)
        srv.close()
