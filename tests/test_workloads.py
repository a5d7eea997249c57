"""Seeded generators: deterministic, sliceable, and shaped like the measured workloads."""
import numpy as np
import pytest

from mhm2_staging_gb300 import workloads


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    return built


def test_deterministic_and_sliceable():
    a = workloads.generate(2, n=3000)
    b = workloads.generate(2, n=3000, threads=1)
    assert np.array_equal(a.a_seq, b.a_seq) and np.array_equal(a.b_seq, b.b_seq)
    s = workloads.generate(2, n=500, first=1200)
    for i in range(500):
        assert s.a(i) == a.a(1200 + i) and s.b(i) == a.b(1200 + i)


def test_config0_shape():
    p = workloads.generate(0)
    assert p.n == 10_000
    assert (p.a_len == 150).all() and (p.b_len == 300).all()
    assert set(np.unique(p.a_seq[:-1])) <= set(b"ACGT")


def test_config1_shape():
    p = workloads.generate(1, n=20000)
    assert p.a_len.min() >= 100 and p.a_len.max() <= 250
    assert (p.b_len - p.a_len >= 50).all() and p.b_len.max() <= 1024
    n_frac = (p.a_seq[:-1] == ord("N")).mean()
    assert 0.0005 < n_frac < 0.002


def test_uneven_workload_shape():
    p = workloads.generate(2, n=40000)
    frac150 = (p.a_len == 150).mean()
    frac250 = (p.a_len == 250).mean()
    assert 0.57 < frac150 < 0.63 + 0.01 and 0.27 < frac250 < 0.33
    assert p.b_len.min() >= 64 and p.b_len.max() <= 2048
    assert 330 < np.median(p.b_len) < 480


def test_config4_shape():
    p = workloads.generate(4, n=500)
    assert (p.a_len == 250).all()
    assert p.b_len.min() >= 2048 and p.b_len.max() <= 8192
