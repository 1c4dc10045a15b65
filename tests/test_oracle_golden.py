"""The oracle (CPU restatement) against the reference's own outputs.

Fixtures in tests/golden/golden.npz were written by the reference library
compiled from its sources (tests/golden/make_golden.py).  When those sources
are present the restatement is also compared with the live reference on
fresh random inputs.
"""
import os

import numpy as np
import pytest

from conftest import eb_of


def test_golden_streams(port, golden):
    assert len(golden) >= 60
    for c in golden:
        s = port.compress(c["x"], eb_of(c["s"]), c["L"], c["T"], c["mode"])
        assert s == c["s"], c["name"]


def test_golden_decompress(port, golden):
    for c in golden:
        y = port.decompress(c["s"], c["n"], c["L"], c["T"], c["mode"])
        assert np.array_equal(y.view(np.uint32), c["y"].view(np.uint32)), c["name"]


def test_golden_rel_bound(port, golden):
    rel = [c for c in golden if c["eb_mode"] == 1]
    assert rel
    for c in rel:
        assert port.rel_bound(c["x"], c["bound"]) == eb_of(c["s"]), c["name"]


def test_bitcount_thresholds_exhaustive(port):
    """bit count is non-decreasing over all 2^32 inputs, so the table is exact."""
    thr = port.thresholds()
    assert list(thr[:22]) == [0] + [1 << k for k in range(21)]
    assert port.verify_thresholds(thr) == 0


def _reference():
    from oracle.oracle import Reference, REF_SO
    ref_src = "/root/reference/SZp/src"
    if not os.path.exists(REF_SO) and not os.path.isdir(ref_src):
        pytest.skip("reference sources not present")
    return Reference()


@pytest.mark.parametrize("T", [1, 2, 6])
@pytest.mark.parametrize("mode", [1, 2])
def test_live_reference_random(port, T, mode):
    from oracle.oracle import reference_compress_arg, reference_decompress_arg
    from szp_gb300.workloads import walk
    ref = _reference()
    rng = np.random.default_rng(1000 + T * 10 + mode)
    for n in (4096, 50001):
        x = walk(n, rng) * np.float32(rng.uniform(0.1, 100))
        eb = float(np.float32(10 ** rng.uniform(-5, -2) * (x.max() - x.min())))
        s_ref = reference_compress_arg(ref, x, eb, 32, T, mode)
        assert port.compress(x, eb, 32, T, mode) == s_ref
        y_ref = reference_decompress_arg(ref, s_ref, n, 32, T, mode)
        assert np.array_equal(port.decompress(s_ref, n, 32, T, mode).view(np.uint32), y_ref.view(np.uint32))
