"""The C ABI library without a GPU: every declared symbol exported, host-side checks,
and the header-only C++ drop-in compiling and linking against it."""
import ctypes as C
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from mhm2_staging_gb300 import build as mbuild
from mhm2_staging_gb300 import driver as D

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mhsw.h"


@pytest.fixture(scope="module")
def lib(built):
    return D.load_library()


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mhsw_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(D.SIGNATURES), set(names) ^ set(D.SIGNATURES)


def _no_gpu(lib) -> bool:
    c = C.c_int(-1)
    lib.mhsw_get_num_node_gpus(C.byref(c))
    return c.value == 0


def test_host_side_status_codes(lib):
    h = C.c_void_p()
    assert lib.mhsw_driver_create(C.byref(h)) == 0
    try:
        assert lib.mhsw_driver_set_orientation(h, 7) == 2  # MHSW_ERR_ARG
        assert lib.mhsw_driver_set_form(h, 9) == 2
        assert lib.mhsw_driver_set_int16_ceiling(h, -1) == 2
        assert lib.mhsw_driver_set_ambiguity(h, 5) == 2  # penalties are passed negated
        assert lib.mhsw_driver_set_ambiguity(h, -2) == 0
        assert lib.mhsw_kernel_block(h) == 0  # nothing in flight
        done = C.c_int(0)
        assert lib.mhsw_kernel_is_done(h, C.byref(done)) == 0 and done.value == 1
        assert lib.mhsw_run_kernel_backwards(h, None, None, None, None, 0, 0, 0) == 3  # MHSW_ERR_STATE
        assert b"not initialised" in lib.mhsw_driver_last_error(h)
        if _no_gpu(lib):
            t = C.c_double(0)
            assert lib.mhsw_driver_init(h, 0, 1, 1, -3, -5, -2, 300, C.byref(t)) == 6  # MHSW_ERR_NO_GPU
        assert lib.mhsw_driver_init(h, 0, 1, 1, 3, -5, -2, 300, None) == 2  # positive penalty rejected
    finally:
        lib.mhsw_driver_destroy(h)


def test_tuning_record_of_a_fresh_handle(lib):
    """A handle that never ran the batched form reports the default configuration."""
    h = C.c_void_p()
    assert lib.mhsw_driver_create(C.byref(h)) == 0
    try:
        t = D.Tuning()
        assert lib.mhsw_last_tuning(h, C.byref(t)) == 0
        assert (t.threads_per_block, t.blocks_per_sm, t.lane_rows, t.wide_try16) == (128, 0, 160, 0)
        assert (t.tunings, t.trials, t.last_call_tuned) == (0, 0, 0)
        assert lib.mhsw_last_tuning(h, None) == 2  # MHSW_ERR_ARG
    finally:
        lib.mhsw_driver_destroy(h)


def test_cigar_format_and_state_checks(lib):
    """mhsw_cigar_format is host code: SAM text of BAM-encoded ops (Alignment::cigar_string)."""
    ops = (C.c_uint32 * 5)((3 << 4) | 4, (8 << 4) | 7, (1 << 4) | 8, (12 << 4) | 1, (150 << 4) | 2)
    buf = C.create_string_buffer(64)
    n = lib.mhsw_cigar_format(ops, 5, buf, 64)
    assert buf.value == b"3S8=1X12I150D" and n == len(buf.value)
    assert lib.mhsw_cigar_format(ops, 5, buf, 8) == -1  # too small: refused, nothing claimed
    assert lib.mhsw_cigar_format(ops, 0, buf, 64) == 0 and buf.value == b""
    h = C.c_void_p()
    assert lib.mhsw_driver_create(C.byref(h)) == 0
    try:
        assert lib.mhsw_driver_set_cigar(h, 1) == 0
        total = C.c_int64(0)
        # not initialised, nothing aligned: a state error (MHSW_ERR_STATE), not a crash
        assert lib.mhsw_last_cigar(h, None, None, None, None, 0, C.byref(total), 1) == 3
    finally:
        lib.mhsw_driver_destroy(h)


def test_limits(lib):
    lim = D.Limits()
    assert lib.mhsw_limits(C.byref(lim)) == 0
    assert lim.max_b_len >= 8192 and lim.int16_ceiling >= 250


def test_python_mirror_raises_like_reference(built):
    if D.get_num_node_gpus() == 0:
        d = D.GPUDriver()
        with pytest.raises(RuntimeError):
            d.init(0, 1, 1, -3, -5, -2, 300)
        with pytest.raises(RuntimeError):
            d.run_kernel_forwards(["ACGT"], ["ACGT"], 4, 4)


def test_missing_library_fails_loudly(tmp_path):
    """No CPU fallback: without the built library the package raises instead of computing."""
    with pytest.raises(RuntimeError, match="libmhsw.so not found"):
        D.load_library(tmp_path / "libmhsw.so")


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_dropin_header_compiles_and_links(built, tmp_path):
    src = tmp_path / "use_driver.cpp"
    src.write_text(r'''
#include <cstdio>
#include <string>
#include <vector>
#include "adept-sw/driver.hpp"
int main() {
  int n = adept_sw::get_num_node_gpus();
  std::printf("gpus=%d\n", n);
  if (n == 0) {
    adept_sw::GPUDriver drv;
    try {
      drv.init(0, 1, 1, -3, -5, -2, 300);
      return 1;
    } catch (const std::runtime_error &e) {
      std::printf("init threw: %s\n", e.what());
    }
    return 0;
  }
  adept_sw::GPUDriver drv;
  drv.init(0, 1, 1, -3, -5, -2, 300);
  std::vector<std::string> reads = {"ACGTACGT"}, ctgs = {"TTACGTACGTTT"};
  drv.run_kernel_forwards(reads, ctgs, 8, 12);
  drv.kernel_block();
  drv.run_kernel_backwards(reads, ctgs, 8, 12);
  drv.kernel_block();
  auto &r = drv.get_aln_results();
  std::printf("score=%d qb=%d qe=%d rb=%d re=%d\n", r.top_scores[0], r.query_begin[0], r.query_end[0],
              r.ref_begin[0], r.ref_end[0]);
  return (r.top_scores[0] == 8 && r.ref_begin[0] == 2 && r.ref_end[0] == 9) ? 0 : 1;
}
''')
    exe = tmp_path / "use_driver"
    lib = mbuild.lib_path()
    subprocess.run(["g++", "-std=c++14", "-O1", "-I", str(ROOT / "include"), str(src), "-o", str(exe), str(lib),
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
