"""klign's GPU call sequence through the C++ drop-in header, at klign's block size:
klign_block_bench (run_kernel_forwards -> kernel_block -> run_kernel_backwards ->
kernel_block -> get_aln_results on 20,000-pair std::vector<std::string> blocks) gives
the oracle's results for every pair."""
import json
import subprocess

import numpy as np
import pytest

from mhm2_staging_gb300 import build as mbuild
from mhm2_staging_gb300 import workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("config,n,form", [(0, 10_000, "plain"), (2, 45_000, "plain"), (2, 45_000, "batched")])
def test_block_sequence_matches_oracle(built, tmp_path, config, n, form):
    pairs = workloads.generate(config, n=n, first=123)
    f = tmp_path / "pairs.bin"
    pairs.write_file(f)
    res = tmp_path / "out.bin"
    r = subprocess.run([str(mbuild.block_bench_path()), str(f), "20000", "1", form, str(res)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rec = json.loads(r.stdout.strip().splitlines()[-1])
    assert rec["pairs"] == n and rec["blocks"] == (n + 19_999) // 20_000 and rec["form"] == form
    got = np.fromfile(res, dtype=np.int32).reshape(n, 5)
    want = oracle.align_batch(pairs, (1, 3, 5, 2, 2))
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} pairs differ; first {bad[:3].tolist()}"
