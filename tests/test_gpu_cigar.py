"""CIGAR mode on the GPU: SSW's report_cigar output (banded traceback, soft clips, =/X
runs, mismatches) bit-exact against the oracle, the reference's recorded outputs and the
CIGARs its own unit test expects, through the C ABI."""
import json
import random
from pathlib import Path

import numpy as np
import pytest

from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, GPUDriver, Pairs, workloads
from mhm2_staging_gb300.driver import DevicePairs
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
MEASURED = (1, 3, 5, 2, 2)
POST_ASSEMBLY = (2, 4, 4, 2, 1)  # klign's scoring when it asks for CIGARs (src/klign.cpp:1061-1064)


def _driver(scoring=MEASURED, score2=False):
    m, x, go, ge, amb = scoring
    d = GPUDriver()
    d.init(0, 1, m, -x, -go, -ge, 0)
    d.set_ambiguity(-amb)
    d.set_cigar(True)
    d.set_score2(score2)
    return d


def _check(d, pairs, scoring, form=FORM_BATCHED):
    """Aligns in CIGAR mode and compares everything with the oracle; returns the timing."""
    out5 = d.align_pairs(pairs, form=form)
    cg = d.last_cigar(pairs.n)
    want, wops, wn = oracle.cigar_batch(pairs, scoring, ops_cap=2048)
    assert np.array_equal(out5, want[:, :5])
    bad = np.nonzero(cg.nops != wn)[0]
    assert len(bad) == 0, [(int(i), int(cg.nops[i]), int(wn[i])) for i in bad[:5]]
    assert np.array_equal(cg.mismatches, want[:, 5])
    assert cg.op_off[-1] == int(np.maximum(wn, 0).sum())
    for i in range(pairs.n):
        k = int(wn[i])
        if k > 0 and not np.array_equal(cg.of(i), wops[i, :k]):
            raise AssertionError(f"pair {i}: gpu {cg.string(i)} oracle {oracle.cigar_string(wops[i], k)}")
    return d.last_timing()


@pytest.mark.parametrize("form", [FORM_PLAIN, FORM_BATCHED])
@pytest.mark.parametrize("cfg,n", [(0, 10000), (1, 8000), (2, 8000), (4, 300)])
def test_cigar_matches_oracle(built, cfg, n, form):
    pairs = workloads.generate(cfg, n=n, first=4242)
    for sc in (MEASURED, POST_ASSEMBLY):
        _check(_driver(sc), pairs, sc, form)


def _adversarial(n, seed):
    """Indel-heavy, N-rich and unrelated pairs: bands that double, wide bands beyond the
    register kernels, boxes longer than wide, ties."""
    rng = random.Random(seed)
    a, b = [], []
    for k in range(n):
        x = "".join(rng.choice("ACGT") for _ in range(rng.randint(1, 300)))
        kind = k % 5
        if kind == 0:
            y = "".join(rng.choice("ACGTN") for _ in range(rng.randint(1, 400)))
        else:
            ind = (0.02, 0.1, 0.25, 0.05)[kind - 1]
            y = []
            for ch in x:
                r = rng.random()
                if r < ind / 2:
                    continue
                if r < ind:
                    y.append("".join(rng.choice("ACGT") for _ in range(rng.randint(1, 8 if kind == 3 else 2))))
                y.append(ch if rng.random() > (0.15 if kind == 4 else 0.03) else rng.choice("ACGTN"))
            y = ("".join(rng.choice("ACGT") for _ in range(rng.randint(0, 60))) + "".join(y) +
                 "".join(rng.choice("ACGT") for _ in range(rng.randint(0, 60))) or "A")
        if rng.random() < 0.5:
            a.append(x)
            b.append(y)
        else:
            a.append(y)
            b.append(x)
    return Pairs.from_lists(a, b)


@pytest.mark.parametrize("scoring", [MEASURED, POST_ASSEMBLY, (2, 2, 3, 1, 2)])
def test_cigar_adversarial(built, scoring):
    pairs = _adversarial(20000, 5)
    t = _check(_driver(scoring), pairs, scoring)
    assert t["n_cigar_generic"] > 0  # some bands outgrew the register kernels
    assert t["cigar_ms"] > 0


@pytest.mark.parametrize("seed", range(8))
def test_cigar_random_scorings(built, seed):
    """Randomly drawn scorings (match 1-4, mismatch 1-8, gap open 1-10, gap extend 1-10,
    ambiguity 0-6) on adversarial and uneven pairs: the register band kernels where the
    lazy-F identity holds (gap open >= gap extend), the generic kernel elsewhere."""
    rng = random.Random(2000 + seed)
    sc = (rng.randint(1, 4), rng.randint(1, 8), rng.randint(1, 10), rng.randint(1, 10), rng.randint(0, 6))
    adv = _adversarial(2500, 100 + seed)
    unev = workloads.generate(2, n=1500, seed=seed)
    a = [adv.a(i) for i in range(adv.n)] + [unev.a(i) for i in range(unev.n)]
    b = [adv.b(i) for i in range(adv.n)] + [unev.b(i) for i in range(unev.n)]
    _check(_driver(sc), Pairs.from_lists(a, b), sc, FORM_PLAIN if seed % 2 else FORM_BATCHED)


def test_cigar_long_boxes_take_the_generic_kernel(built):
    """Boxes longer than the register kernels' row capacity (512): 600-2000 bp reads
    against their own mutated copies."""
    rng = random.Random(9)
    a, b = [], []
    for _ in range(64):
        x = "".join(rng.choice("ACGT") for _ in range(rng.randint(600, 2000)))
        y = "".join(c if rng.random() > 0.02 else rng.choice("ACGT") for c in x if rng.random() > 0.005)
        a.append(x)
        b.append("GATTACA" + y + "TT")
    pairs = Pairs.from_lists(a, b)
    t = _check(_driver(), pairs, MEASURED)
    assert t["n_cigar_generic"] == 64


def test_cigar_arena_grows(built):
    """Alternating mismatches under a scoring that keeps them: ~one =/X op per base, far
    beyond the arena's first size (32 ops per pair), so the pass runs again in a grown arena."""
    rng = random.Random(4)
    a, b = [], []
    for _ in range(2000):
        x = "".join(rng.choice("ACGT") for _ in range(250))
        y = "".join(c if i % 2 else {"A": "C", "C": "G", "G": "T", "T": "A"}[c] for i, c in enumerate(x))
        a.append(x)
        b.append(y)
    pairs = Pairs.from_lists(a, b)
    sc = (3, 1, 6, 1, 1)
    d = _driver(sc)
    _check(d, pairs, sc)
    cg = d.last_cigar(pairs.n)
    assert cg.op_off[-1] > 32 * pairs.n


@pytest.mark.parametrize("scoring", ["ssw_default", "mhm2_aln", "cigar", "measured"])
def test_cigar_recorded_reference(built, scoring):
    samples = json.loads((GOLDEN / "ssw_reference_samples.json").read_text())
    recs = samples["pairs"]
    pairs = Pairs.from_lists([r["a"] for r in recs], [r["b"] for r in recs])
    d = _driver(tuple(samples["scorings"][scoring]))
    for form in (FORM_PLAIN, FORM_BATCHED):
        out5 = d.align_pairs(pairs, form=form)
        cg = d.last_cigar(pairs.n)
        for i, r in enumerate(recs):
            assert out5[i].tolist() == r["reference"][scoring]
            if r["reference"][scoring][0] == 0:  # SSW's CIGAR is not defined there
                assert cg.nops[i] == 0
                continue
            assert [cg.string(i), int(cg.mismatches[i])] == r["reference_cigar"][scoring], (r["set"], r["a"], r["b"])


@pytest.mark.parametrize("scoring", ["ssw_default", "mhm2_aln", "cigar"])
def test_cigar_known_answers_of_reference_test(built, scoring):
    """The CIGARs test/ssw-test.cpp:159-236 expects (8=1X7=, 8=1I8=, 4=1D11=, 3S16=, ...)."""
    ka = json.loads((GOLDEN / "ssw_known_answers.json").read_text())
    cases = ka["cases"]
    pairs = Pairs.from_lists([c["ref"] for c in cases], [c["query"] for c in cases])
    d = _driver(tuple(ka["scorings"][scoring]))
    d.align_pairs(pairs)
    cg = d.last_cigar(pairs.n)
    for i, c in enumerate(cases):
        if c["kind"] == "aln":
            assert (cg.string(i), int(cg.mismatches[i])) == (c["cigar"], c["mismatches"]), c


def test_cigar_through_dropin_protocol_with_score2(built):
    """run_kernel_forwards / backwards / kernel_block, then the CIGARs and klign's SAM
    fields (score, score2, mismatches) of the same round."""
    pairs = workloads.generate(1, n=3000, first=808)
    reads = [pairs.a(i) for i in range(pairs.n)]
    ctgs = [pairs.b(i) for i in range(pairs.n)]
    d = _driver(POST_ASSEMBLY, score2=True)
    d.run_kernel_forwards(reads, ctgs, max(map(len, reads)), max(map(len, ctgs)))
    d.kernel_block()
    d.run_kernel_backwards(reads, ctgs, max(map(len, reads)), max(map(len, ctgs)))
    d.kernel_block()
    cg = d.last_cigar(pairs.n)
    want, wops, wn = oracle.cigar_batch(pairs, POST_ASSEMBLY, ops_cap=2048)
    assert np.array_equal(cg.nops, wn) and np.array_equal(cg.mismatches, want[:, 5])
    for i in range(pairs.n):
        assert np.array_equal(cg.of(i), wops[i, :max(int(wn[i]), 0)])
    s2 = oracle.align_batch(pairs, POST_ASSEMBLY, score2=True)
    r = d.get_aln_results()
    assert np.array_equal(r.score2, s2[:, 5])


def test_cigar_graph_replay(built):
    """A device-resident batch with stated extents in CIGAR mode: captured into a CUDA
    graph on the second call and replayed after; the same CIGARs every time."""
    torch = pytest.importorskip("torch")
    pairs = workloads.generate(2, n=20000, first=17)
    dev = torch.device("cuda:0")
    tens = [torch.from_numpy(x).to(dev) for x in (pairs.a_seq, pairs.a_off, pairs.a_len, pairs.b_seq, pairs.b_off,
                                                 pairs.b_len)]
    dp = DevicePairs(*(t.data_ptr() for t in tens), n=pairs.n, max_a_len=int(pairs.a_len.max()),
                     max_b_len=int(pairs.b_len.max()), cells=float(pairs.cells()),
                     a_bytes=int((pairs.a_off + pairs.a_len).max()), b_bytes=int((pairs.b_off + pairs.b_len).max()))
    d = _driver()
    out = torch.full((pairs.n, 5), -9, dtype=torch.int32, device=dev)
    want, wops, wn = oracle.cigar_batch(pairs, MEASURED, ops_cap=2048)
    replays = []
    first = None
    for call in range(3):
        out.fill_(-9)
        torch.cuda.synchronize()
        d.align_pairs_device(dp, out.data_ptr(), form=FORM_BATCHED)
        cg = d.last_cigar(pairs.n)
        got = (out.cpu().numpy(), cg.nops.copy(), cg.mismatches.copy(), cg.op_off.copy(), cg.ops.copy())
        assert np.array_equal(got[0], want[:, :5]) and np.array_equal(got[1], wn), f"call {call}"
        if first is None:
            first = got
        else:
            assert all(np.array_equal(x, y) for x, y in zip(first, got)), f"call {call}"
        replays.append(d.last_timing()["graph_replays"])
    assert replays == [0, 1, 2], replays
    for i in range(pairs.n):
        k = int(wn[i])
        assert np.array_equal(first[4][first[3][i]:first[3][i] + max(k, 0)], wops[i, :max(k, 0)])


def test_cigar_off_again(built):
    pairs = workloads.generate(0, n=500, first=3)
    d = _driver()
    d.align_pairs(pairs)
    assert d.last_cigar(pairs.n).op_off[-1] > 0
    d.set_cigar(False)
    d.align_pairs(pairs)
    with pytest.raises(RuntimeError, match="status 3"):
        d.last_cigar(pairs.n)


def test_cigar_through_cpp_dropin_header(built, tmp_path):
    """A klign-style C++ caller of include/adept-sw/driver.hpp: forwards, backwards,
    kernel_block, then SSW's cigar_string and mismatches per pair."""
    import shutil
    import subprocess

    from mhm2_staging_gb300 import build as mbuild

    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    root = Path(__file__).resolve().parent.parent
    src = tmp_path / "cigar_driver.cpp"
    src.write_text(r'''
#include <cstdio>
#include <string>
#include <vector>
#include "adept-sw/driver.hpp"
int main() {
  adept_sw::GPUDriver drv;
  drv.init(0, 1, 2, -4, -4, -2, 300);  // klign's scoring when it asks for CIGARs
  drv.set_ambiguity(-1);
  drv.set_cigar(true);
  std::vector<std::string> reads = {"AAAATTTTCCCCGGGG", "AAAATTTTCCCCGGGG", "ACGT"};
  std::vector<std::string> ctgs = {"GCTAAAATTTTCCCCGGGGACT", "AAAATTTTACCCCGGGG", "NNNN"};
  drv.run_kernel_forwards(reads, ctgs, 16, 22);
  drv.kernel_block();
  drv.run_kernel_backwards(reads, ctgs, 16, 22);
  drv.kernel_block();
  std::vector<std::string> cig;
  std::vector<int32_t> mm;
  drv.get_cigars(cig, mm);
  for (size_t i = 0; i < cig.size(); i++) std::printf("%s %d\n", cig[i].c_str(), mm[i]);
  return 0;
}
''')
    exe = tmp_path / "cigar_driver"
    lib = mbuild.lib_path()
    subprocess.run(["g++", "-std=c++14", "-O1", "-I", str(root / "include"), str(src), "-o", str(exe), str(lib),
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    # test/ssw-test.cpp:213-231 expects 3S16=3S-style clips and 8=1I8=; all-N scores 0
    assert r.stdout.split("\n")[:3] == ["3S16=3S 0", "8=1I8= 1", " 0"], r.stdout
