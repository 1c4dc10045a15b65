"""The C-ABI library: it loads, exports every symbol include/szp_gb300.h
declares, its host-side logic agrees with the oracle, and without a GPU its
compute entry points fail with an error instead of computing on the CPU."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, HAS_GPU

HEADER = os.path.join(ROOT, "include", "szp_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    return sorted(set(re.findall(r"\b(szp_\w+)\s*\(", src)))


def test_header_declares_reference_api():
    names = declared_functions()
    for ref in ["szp_compress", "szp_decompress", "szp_float_openmp_threadblock",
                "szp_float_openmp_threadblock_arg", "szp_float_single_thread_arg",
                "szp_float_single_thread_arg_record", "szp_float_openmp_threadblock_randomaccess",
                "szp_float_openmp_threadblock_randomaccess_arg", "szp_float_decompress_openmp_threadblock",
                "szp_float_decompress_openmp_threadblock_arg", "szp_float_decompress_single_thread_arg",
                "szp_float_decompress_single_thread_arg_record",
                "szp_float_decompress_openmp_threadblock_randomaccess",
                "szp_float_decompress_openmp_threadblock_randomaccess_arg"]:
        assert ref in names


def test_library_exports_every_declared_symbol(szp):
    out = subprocess.run(["nm", "-D", "--defined-only", szp.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if " T " in line)
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    # and ctypes can resolve them in this process
    for f in declared_functions():
        getattr(szp.lib, f)


def test_thresholds_match_oracle(szp, port):
    assert np.array_equal(szp.bitcount_thresholds(), port.thresholds())


def test_max_stream_bytes_bounds_oracle(szp, port):
    rng = np.random.default_rng(5)
    for n in (0, 1, 2, 33, 1000, 12345):
        for T in (1, 3, 8):
            for L in (1, 7, 32, 64):
                for mode in (1, 2):
                    bound = szp.max_stream_bytes(n, L, T, mode)
                    x = rng.normal(0, 1e9, n).astype(np.float32)  # incompressible
                    s = port.compress(x, 1e-3, L, T, mode)
                    assert len(s) <= bound, (n, T, L, mode)


def test_segments_setting(szp):
    szp.set_segments(5)
    assert szp.get_segments() == 5
    szp.set_segments(0)
    assert szp.get_segments() >= 1


@pytest.mark.skipif(HAS_GPU, reason="checks behaviour without a GPU")
def test_no_cpu_fallback_without_gpu(szp):
    x = np.arange(100, dtype=np.float32)
    with pytest.raises(szp.SzpError) as e:
        szp.szp_compress(x, szp.ABS, 1e-3)
    assert e.value.status == szp.ECUDA
    with pytest.raises(szp.SzpError):
        szp.szp_decompress(b"\0" * 64, 10)
    with pytest.raises(szp.SzpError) as e:
        szp.szp_compress(x.astype(np.float64), szp.ABS, 1e-3, 0.0, 32, 1, szp.SZ_DOUBLE)
    assert e.value.status == szp.ECUDA
    # the device entry points fail before touching their (here meaningless) pointers
    with pytest.raises(szp.SzpError) as e:
        szp.reduce_sum_dev(1 << 20, 64, 1 << 21, 64, 10, 1 << 22, 4096)
    assert e.value.status == szp.ECUDA
