"""The batched form's tuner: a handle re-tunes when its batch's length signature moves
(on a sample of the batch, within a bounded time), keeps its configuration while it does
not, takes back the configuration of a signature it tuned for before, and every
configuration it picks stays bit-exact against the oracle."""
import numpy as np
import pytest

from mhm2_staging_gb300 import FORM_BATCHED, GPUDriver, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu
SCORING = (1, 3, 5, 2, 2)


@pytest.fixture(scope="module")
def drv(built):
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 300)
    d.set_ambiguity(-2)
    return d


def _check(drv, pairs):
    got = drv.align_pairs(pairs, FORM_BATCHED)
    want = oracle.align_batch(pairs, SCORING)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} of {pairs.n} differ; first {bad[:3].tolist()}"
    return drv.last_tuning()


def test_retunes_from_150_300_bp_pairs_to_the_uneven_workload(drv):
    p0 = workloads.generate(0, n=10_000)
    p2 = workloads.generate(2, n=300_000)  # more than the tuner's 256k-pair sample: strided
    t = _check(drv, p0)
    assert t["last_call_tuned"] == 1 and t["tunings"] == 1 and t["sample_pairs"] == 10_000
    assert t["trials"] >= 5 and len(t["trial_ms"]) == t["trials"]
    shape0 = (t["threads_per_block"], t["blocks_per_sm"], t["lane_rows"], t["wide_try16"])
    t = _check(drv, p0)  # same workload: no tuning
    assert t["last_call_tuned"] == 0 and t["tunings"] == 1
    t = _check(drv, p2)  # new length mix and sizes: re-tuned on every second pair
    assert t["last_call_tuned"] == 1 and t["tunings"] == 2 and t["sample_pairs"] == 150_000
    # the 150 bp reads (129..160 rows) let the tuner try them in 16-lane groups
    assert t["trials"] >= 6
    assert t["lane_rows"] in (128, 160) and t["threads_per_block"] in (64, 128, 256)
    t = _check(drv, workloads.generate(2, n=300_000, first=300_000))  # same mix, other pairs
    assert t["last_call_tuned"] == 0 and t["tunings"] == 2
    t = _check(drv, p0)  # back again: the configuration tuned for it is taken back, no trials
    assert t["last_call_tuned"] == 0 and t["tunings"] == 2
    assert (t["threads_per_block"], t["blocks_per_sm"], t["lane_rows"], t["wide_try16"]) == shape0
    t = _check(drv, p2)  # and forth
    assert t["last_call_tuned"] == 0 and t["tunings"] == 2


def _mix(seed: int, n: int, lo: int, hi: int, tail: int):
    """Reads of lo..hi bases, 3% substitutions, inside random flank of up to tail bases."""
    from mhm2_staging_gb300 import Pairs

    rng = np.random.default_rng(seed)
    a, b = [], []
    for _ in range(n):
        read = "".join(rng.choice(list("ACGT"), int(rng.integers(lo, hi + 1))))
        mut = "".join(c if rng.random() > 0.03 else rng.choice(list("ACGT")) for c in read)
        b.append("".join(rng.choice(list("ACGT"), int(rng.integers(0, tail)))) + mut +
                 "".join(rng.choice(list("ACGT"), 50)))
        a.append(read)
    return Pairs.from_lists(a, b)


@pytest.mark.parametrize("threads,blocks,lane_rows,try16", [(128, 0, 160, 0), (128, 0, 128, 0), (64, 0, 128, 1),
                                                            (256, 1, 160, 1), (128, 2, 160, 0)])
def test_every_configuration_is_exact(built, threads, blocks, lane_rows, try16):
    """Each configuration the tuner can pick gives the oracle's results: reads around the
    8/16-lane threshold (120..170 rows) and, at match 20, pairs whose score bound exceeds
    the int16 keys (straight to int32, or int16 first with the re-run of those that
    overflow)."""
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 300)
    d.set_ambiguity(-2)
    d.fix_batch_config(threads, blocks, lane_rows, bool(try16))
    pairs = _mix(threads + lane_rows + try16, 3000, 120, 170, 300)
    _check(d, pairs)
    t = d.last_tuning()
    assert t["tunings"] == 0 and (t["threads_per_block"], t["lane_rows"], t["wide_try16"]) == (threads, lane_rows,
                                                                                                  try16)
    d20 = GPUDriver()
    d20.init(0, 1, 20, -3, -5, -2, 300)
    d20.set_ambiguity(-2)
    d20.fix_batch_config(threads, blocks, lane_rows, bool(try16))
    long_pairs = _mix(7 + try16, 600, 150, 400, 200)  # 20 * 201+ rows > 4032: bound above the keys
    got = d20.align_pairs(long_pairs, FORM_BATCHED)
    want = oracle.align_batch(long_pairs, (20, 3, 5, 2, 2))
    assert np.array_equal(got, want)
    assert d20.last_timing()["n_overflow16"] > 0
