"""GPU parity: the CUDA path through the C ABI against the CPU oracle, bit-exact."""
import numpy as np
import pytest

from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, GPUDriver, ORIENT_REF_IS_A, Pairs, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu
SC = (1, 3, 5, 2, 2)


def _diff(got, want, pairs=None):
    bad = np.nonzero((got != want).any(axis=1))[0]
    if len(bad):
        i = int(bad[0])
        extra = ""
        if pairs is not None:
            extra = f" A={pairs.a(i)[:80]!r} B={pairs.b(i)[:80]!r}"
        return f"{len(bad)} of {len(got)} differ; first {i}: gpu={got[i].tolist()} oracle={want[i].tolist()}{extra}"
    return ""


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
def test_config0_all_pairs(gpu, form):
    pairs = workloads.generate(0)
    got = gpu.align_pairs(pairs, form=form)
    want = oracle.align_batch(pairs, SC)
    assert not _diff(got, want, pairs)


_SAMPLES: dict = {}


def _sample(cfg: int, n: int):
    """Pairs and oracle results of a workload sample, computed once for both forms (the
    long-reference sample through the oracle's vectorised form, bit-exact with the scalar
    one: tests/test_oracle.py)."""
    if (cfg, n) not in _SAMPLES:
        pairs = workloads.generate(cfg, n=n)
        want = oracle.align_batch_lanes(pairs, SC) if cfg == 4 else oracle.align_batch(pairs, SC)
        _SAMPLES[(cfg, n)] = (pairs, want)
    return _SAMPLES[(cfg, n)]


@pytest.mark.parametrize("cfg,n", [(1, 20000), (2, 20000), (4, 20000)])
@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
def test_config_samples(gpu, cfg, n, form):
    pairs, want = _sample(cfg, n)
    got = gpu.align_pairs(pairs, form=form)
    assert not _diff(got, want, pairs)


@pytest.mark.parametrize("cfg,form", [(2, FORM_BATCHED), (1, FORM_PLAIN), (1, FORM_BATCHED), (4, FORM_BATCHED)])
def test_whole_workloads_match_oracle(built, cfg, form):
    """Whole workloads at their full sizes -- the benchmark's uneven batch (4M pairs,
    3.34e11 cells), the 1M-pair read mix in both forms, the 200k long-reference pairs --
    every pair against the oracle's vectorised form (bit-exact with the scalar one:
    tests/test_oracle.py)."""
    pairs = workloads.generate(cfg)
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 0)
    d.set_ambiguity(-2)
    got = d.align_pairs(pairs, form=form)
    want = oracle.align_batch_lanes(pairs, SC)
    assert not _diff(got, want, pairs)


def test_dropin_protocol_klign(gpu):
    pairs = workloads.generate(1, n=3000)
    reads = [pairs.a(i) for i in range(pairs.n)]
    ctgs = [pairs.b(i) for i in range(pairs.n)]
    mr, mc = max(map(len, reads)), max(map(len, ctgs))
    gpu.run_kernel_forwards(reads, ctgs, mr, mc)
    gpu.kernel_block()
    r1 = gpu.get_aln_results()
    gpu.run_kernel_backwards(reads, ctgs, mr, mc)
    gpu.kernel_block()
    assert gpu.kernel_is_done()
    r = gpu.get_aln_results()
    want = oracle.align_batch(pairs, SC)
    got = np.stack([r.top_scores32, r.query_begin32, r.query_end32, r.ref_begin32, r.ref_end32], axis=1)
    assert not _diff(got, want, pairs)
    # short views equal the int32 ones in range; ends were already valid after forwards
    assert np.array_equal(r.top_scores.astype(np.int32), r.top_scores32)
    assert np.array_equal(r1.query_end32, r.query_end32) and np.array_equal(r1.ref_end32, r.ref_end32)


@pytest.mark.parametrize("sc", [(1, 6, 4, 1, 3), (1, 2, 3, 1, 4)])
@pytest.mark.parametrize("cfg", [1, 2])
def test_penalties_above_gap_open(built, sc, cfg):
    """A mismatch or ambiguity penalty above the gap-open penalty: the forward pass takes
    the generic engine (not the keyed one) and the begin pass the band kernels' offset-128
    score table."""
    m, x, go, ge, amb = sc
    d = GPUDriver()
    d.init(0, 1, m, -x, -go, -ge, 0)
    d.set_ambiguity(-amb)
    pairs = workloads.generate(cfg, n=6000)
    want = oracle.align_batch(pairs, sc)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = d.align_pairs(pairs, form=form)
        assert not _diff(got, want, pairs)


@pytest.mark.parametrize("seed", range(12))
def test_random_scorings(built, seed):
    """Randomly drawn scorings (match 1-4, mismatch 1-8, gap open 1-10, gap extend 1-10,
    ambiguity 0-6): the keyed or the generic forward engine, the biased or the offset-128
    band table, as each scoring selects; both forms against the oracle."""
    import random

    rng = random.Random(1000 + seed)
    sc = (rng.randint(1, 4), rng.randint(1, 8), rng.randint(1, 10), rng.randint(1, 10), rng.randint(0, 6))
    m, x, go, ge, amb = sc
    d = GPUDriver()
    d.init(0, 1, m, -x, -go, -ge, 0)
    d.set_ambiguity(-amb)
    pairs = workloads.generate(1 if seed % 2 else 2, n=3000, seed=seed)
    want = oracle.align_batch(pairs, sc)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = d.align_pairs(pairs, form=form)
        assert not _diff(got, want, pairs), (sc, form)


def _embedded_reads(seed: int, n: int, lo: int, hi: int) -> Pairs:
    """Reads of lo..hi bases with 2% substitutions, each inside a window of up to 120
    random flanking bases: the score climbs from the first rows on."""
    rng = np.random.default_rng(seed)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    a, b = [], []
    for _ in range(n):
        read = acgt[rng.integers(0, 4, int(rng.integers(lo, hi + 1)))]
        mut = read.copy()
        sub = rng.random(len(read)) < 0.02
        mut[sub] = acgt[rng.integers(0, 4, int(sub.sum()))]
        left = acgt[rng.integers(0, 4, int(rng.integers(0, 120)))]
        right = acgt[rng.integers(0, 4, int(rng.integers(0, 120)))]
        a.append(read.tobytes().decode())
        b.append(np.concatenate([left, mut, right]).tobytes().decode())
    return Pairs.from_lists(a, b)


@pytest.mark.parametrize("match", [16, 40, 63])
def test_high_match_scorings(built, match):
    """Match scores of 16-63 take H above 255 within the first lane's rows of every lane
    group size and row count per lane (reads of 24-260 bases), on the keyed int16 engine
    where the score bound fits its keys and on the int32 engine (or the int16 try and its
    re-run) where it does not; both forms against the oracle."""
    sc = (match, 4, 6, 1, 2)
    d = GPUDriver()
    d.init(0, 1, match, -4, -6, -1, 0)
    d.set_ambiguity(-2)
    pairs = _embedded_reads(match, 1500, 24, 260)
    want = oracle.align_batch(pairs, sc)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = d.align_pairs(pairs, form=form)
        assert not _diff(got, want, pairs), (sc, form)


def test_forced_int32_rerun(built):
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 300)
    d.set_ambiguity(-2)
    d.set_int16_ceiling(60)
    pairs = workloads.generate(0, n=1500)
    want = oracle.align_batch(pairs, SC)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = d.align_pairs(pairs, form=form)
        t = d.last_timing()
        assert not _diff(got, want, pairs)
        assert t["n_overflow16"] == int((want[:, 0] > 60).sum())


def test_long_a_strips(built):
    """A (rows) longer than one wavefront strip (> 256 rows) in both engines."""
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 300)
    d.set_ambiguity(-2)
    src = workloads.generate(4, n=64)
    a = [src.b(i)[:300 + 37 * i] for i in range(64)]  # long A = contig prefixes
    b = [src.a(i) for i in range(64)]                 # B = reads
    pairs = Pairs.from_lists(a, b)
    want = oracle.align_batch(pairs, SC)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = d.align_pairs(pairs, form=form)
        assert not _diff(got, want, pairs)
    d.set_int16_ceiling(40)
    got = d.align_pairs(pairs, form=FORM_PLAIN)
    assert not _diff(got, want, pairs)


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
def test_scores_at_the_packed_begin_cap(built, form):
    """Identical and near-identical pairs whose scores lie just below, at and above 16,000,
    the largest score the packed int16 begin bands take: at or below it the begin search
    runs in a packed band (values up to the score plus gap-open and match inside int16),
    above it in the int32 wavefront."""
    import random

    rng = random.Random(16000)
    a, b = [], []
    for n, subs in ((15990, 0), (16000, 0), (16001, 0), (16010, 1), (16012, 2)):
        x = "".join(rng.choice("ACGT") for _ in range(n))
        y = list(x)
        for _ in range(subs):
            k = rng.randrange(2000, n - 2000)
            y[k] = rng.choice([c for c in "ACGT" if c != y[k]])
        flank = "".join(rng.choice("ACGT") for _ in range(37))
        a.append(x)
        b.append(flank + "".join(y) + flank)
    pairs = Pairs.from_lists(a, b)
    want = oracle.align_batch(pairs, SC, 5)
    assert sorted(want[:, 0].tolist())[0] < 16000 and want[:, 0].max() > 16000 and 16000 in want[:, 0]
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 0)
    d.set_ambiguity(-2)
    got = d.align_pairs(pairs, form=form)
    assert not _diff(got, want, pairs)


def test_high_scores_long_near_identical_pairs(built):
    """Near-identical 20,000-base pairs with about 20 substitutions and an indel: scores
    above 16,000 whose gap bound exceeds the widest begin band, so the begin search takes
    the int32 wavefront on the reversed box; and a 33,000-base pair whose score passes
    32,767, beyond SSW's 16-bit range (the oracle is int32)."""
    import random

    rng = random.Random(11)

    def mutate(x, subs, indel):
        y = list(x)
        for _ in range(subs):
            k = rng.randrange(len(y))
            y[k] = rng.choice([c for c in "ACGT" if c != y[k]])
        if indel:
            del y[rng.randrange(len(y))]
        return "".join(y)

    a, b = [], []
    for n, subs in ((20000, 20), (20000, 24), (20000, 30), (33000, 3)):
        x = "".join(rng.choice("ACGT") for _ in range(n))
        a.append(x)
        b.append(mutate(x, subs, True))
    pairs = Pairs.from_lists(a, b)
    want = oracle.align_batch(pairs, SC, 4)
    assert want[:3, 0].min() > 16000 and want[3, 0] > 32767
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 0)
    d.set_ambiguity(-2)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = d.align_pairs(pairs, form=form)
        assert not _diff(got, want)


def test_size_limits(built):
    """B of exactly the largest length the kernels take, in both forms, bit-exact; one byte
    more is refused with the limit error and the handle stays usable; A has no limit
    (strips): a 70,000-base A against a short B."""
    import random

    from mhm2_staging_gb300.driver import limits

    rng = random.Random(5)
    lim = limits().max_b_len
    read = "".join(rng.choice("ACGT") for _ in range(150))
    flank = "".join(rng.choice("ACGT") for _ in range(lim - 150))
    window = flank[: lim // 2] + read[:70] + "T" + read[71:] + flank[lim // 2:]
    assert len(window) == lim
    long_a = "".join(rng.choice("ACGT") for _ in range(70000))
    pairs = Pairs.from_lists([read, read, long_a], [window, read[::-1], long_a[30000:30200]])
    want = oracle.align_batch(pairs, SC)
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 0)
    d.set_ambiguity(-2)
    for form in (FORM_PLAIN, FORM_BATCHED):
        assert not _diff(d.align_pairs(pairs, form=form), want, pairs)
    too_long = Pairs.from_lists([read], [window + "A"])
    for form in (FORM_PLAIN, FORM_BATCHED):
        with pytest.raises(RuntimeError):
            d.align_pairs(too_long, form=form)
    assert not _diff(d.align_pairs(pairs, form=FORM_BATCHED), want, pairs)


def test_edge_cases(gpu):
    cases = [
        (b"A", b"A"), (b"A", b"C"), (b"N", b"N"), (b"ACGT", b"acgt"), (b"UUUU", b"AAAA"),
        (b"", b"ACGT"), (b"ACGT", b""), (b"NNNNNNNNNN", b"ACGTACGTAC"), (b"GATTACA" * 3, b"GATTACA"),
        (b"ACGTXYZ-ACGT", b"ACGT.ACGT"), (bytes(range(65, 91)), bytes(range(97, 123))),
        (b"A" * 500, b"A" * 700), (b"AC" * 200, b"CA" * 300), (b"T" * 40, b"T"),
    ]
    pairs = Pairs.from_lists([c[0] for c in cases], [c[1] for c in cases])
    want = oracle.align_batch(pairs, SC)
    for form in (FORM_PLAIN, FORM_BATCHED):
        got = gpu.align_pairs(pairs, form=form)
        assert not _diff(got, want, pairs)


def test_single_pair_and_empty_batch(gpu):
    p = Pairs.from_lists([b"ACGTACGT"], [b"TTACGTACGTTT"])
    assert not _diff(gpu.align_pairs(p), oracle.align_batch(p, SC))
    e = Pairs.from_lists([], [])
    assert gpu.align_pairs(e).shape == (0, 5)


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
def test_repeated_device_batch_replays_a_cuda_graph(built, form):
    """The same device-resident batch aligned repeatedly: the second call is captured into
    a CUDA graph and later calls replay it; every call gives the oracle's results."""
    torch = pytest.importorskip("torch")
    from mhm2_staging_gb300.driver import DevicePairs

    pairs = workloads.generate(2, n=30000, first=4242)
    want = oracle.align_batch(pairs, SC)
    dev = torch.device("cuda:0")
    tens = [torch.from_numpy(x).to(dev) for x in (pairs.a_seq, pairs.a_off, pairs.a_len, pairs.b_seq, pairs.b_off,
                                                 pairs.b_len)]
    dp = DevicePairs(*(t.data_ptr() for t in tens), n=pairs.n, max_a_len=int(pairs.a_len.max()),
                     max_b_len=int(pairs.b_len.max()), cells=float(pairs.cells()),
                     a_bytes=int((pairs.a_off + pairs.a_len).max()), b_bytes=int((pairs.b_off + pairs.b_len).max()))
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 0)
    d.set_ambiguity(-2)
    out = torch.full((pairs.n, 5), -9, dtype=torch.int32, device=dev)
    replays = []
    for call in range(4):
        out.fill_(-9)
        torch.cuda.synchronize()
        d.align_pairs_device(dp, out.data_ptr(), form=form)
        got = out.cpu().numpy()
        assert not _diff(got, want, pairs), f"call {call}"
        replays.append(d.last_timing()["graph_replays"])
    assert replays == [0, 1, 2, 3], replays


def test_host_batch_with_stated_extents(gpu):
    pairs = workloads.generate(1, n=5000, first=777)
    want = oracle.align_batch(pairs, SC)
    got = gpu.align_pairs(pairs, form=FORM_BATCHED, hints=True)
    assert not _diff(got, want, pairs)


def test_async_halves_alternating_handles(built):
    """mhsw_align_pairs_async / mhsw_align_wait on two handles in turn (one batch's copies
    overlapping the other's kernels): every batch gives the oracle's results; a later call
    on a handle completes its pending batch first."""
    batches = [workloads.generate(cfg, n=n, first=100 + k) for k, (cfg, n) in
               enumerate([(2, 20000), (1, 15000), (2, 20000), (0, 10000), (4, 200)])]
    handles = []
    for _ in range(2):
        d = GPUDriver()
        d.init(0, 1, 1, -3, -5, -2, 0)
        d.set_ambiguity(-2)
        handles.append(d)
    outs = [None] * len(batches)
    pending = [None, None]
    for k, b in enumerate(batches):
        h = k % 2
        if pending[h] is not None:
            handles[h].wait()
        outs[k] = handles[h].align_pairs_async(b, form=FORM_BATCHED, hints=True)
        pending[h] = k
    for h in range(2):
        handles[h].wait()
    for k, b in enumerate(batches):
        assert not _diff(outs[k], oracle.align_batch(b, SC), b), f"batch {k}"
    # a pending batch is completed by the next call on its handle
    o = handles[0].align_pairs_async(batches[3], form=FORM_PLAIN)
    assert handles[0].last_timing()["n_pairs"] == batches[3].n
    assert not _diff(o, oracle.align_batch(batches[3], SC), batches[3])
    handles[0].wait()  # nothing pending: a no-op


def test_async_calls_in_flight_on_one_handle(built):
    """Several host batches enqueued back to back on one handle (four in flight, the
    copies of later ones overlapping earlier ones' kernels): every result matches the
    oracle."""
    batches = [workloads.generate(cfg, n=n, first=300 + k) for k, (cfg, n) in
               enumerate([(2, 30000), (1, 10000), (2, 30000), (0, 10000), (2, 5000), (1, 1)])]
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 0)
    d.set_ambiguity(-2)
    outs = [d.align_pairs_async(b, form=FORM_BATCHED, hints=True) for b in batches]
    d.wait()
    for k, b in enumerate(batches):
        assert not _diff(outs[k], oracle.align_batch(b, SC), b), f"batch {k}"
    # plain form and unhinted batches go the same way
    outs = [d.align_pairs_async(b, form=FORM_PLAIN) for b in batches[:3]]
    d.wait()
    for k, b in enumerate(batches[:3]):
        assert not _diff(outs[k], oracle.align_batch(b, SC), b), f"plain batch {k}"
