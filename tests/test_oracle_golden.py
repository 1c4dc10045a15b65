"""The oracle (CPU restatement) against the reference's own outputs.

Fixtures in tests/golden/golden.npz were written by the reference library
compiled from its sources (tests/golden/make_golden.py).  When those sources
are present the restatement is also compared with the live reference on
fresh random inputs.
"""
import numpy as np
import pytest

from conftest import eb_of, eb_of_double


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


def test_golden_double_streams(port, golden_double):
    """float64 (szp_double_* of the reference): streams byte for byte."""
    assert len(golden_double) >= 50
    for c in golden_double:
        s = port.compress_d(c["x"], eb_of_double(c["s"]), c["L"], c["T"], c["mode"])
        assert s == c["s"], c["name"]


def test_golden_double_decompress(port, golden_double):
    for c in golden_double:
        y = port.decompress_d(c["s"], c["n"], c["L"], c["T"], c["mode"])
        assert np.array_equal(y.view(np.uint64), c["y"].view(np.uint64)), c["name"]


def test_golden_double_rel_bound(port, golden_double):
    rel = [c for c in golden_double if c["eb_mode"] == 1]
    assert rel
    for c in rel:
        assert port.rel_bound_d(c["x"], c["bound"]) == eb_of_double(c["s"]), c["name"]


def test_golden_record_tallies(port, golden_record):
    """The single-thread _record tallies (szp_float.cc:607-750,
    szpd_float.cc:216-318 and the double twins) against the values the
    reference returned, and the T = 1 streams byte for byte."""
    assert len(golden_record) >= 15
    assert any(c["dbl"] for c in golden_record) and any(not c["dbl"] for c in golden_record)
    for c in golden_record:
        comp = port.compress_d if c["dbl"] else port.compress
        assert comp(c["x"], c["bound"], c["L"], 1, 1) == c["s"], c["name"]
        assert port.record_compress(c["s"], c["n"], c["L"], c["dbl"]) == c["rec_c"], c["name"]
        assert port.record_decompress(c["s"], c["n"], c["L"], c["dbl"]) == c["rec_d"], c["name"]


def test_bitcount_thresholds_exhaustive(port):
    """bit count is non-decreasing over all 2^32 inputs, so the table is exact."""
    thr = port.thresholds()
    assert list(thr[:22]) == [0] + [1 << k for k in range(21)]
    assert port.verify_thresholds(thr) == 0


def _reference():
    from oracle.oracle import Reference
    try:
        return Reference()
    except FileNotFoundError:
        pytest.skip("reference library not built (its sources are not present here)")


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


@pytest.mark.parametrize("mode", [1, 2])
def test_live_reference_random_double(port, mode):
    from szp_gb300.workloads import walk64
    ref = _reference()
    rng = np.random.default_rng(2000 + mode)
    for n, T in ((4096, 3), (50001, 6)):
        x = walk64(n, rng) * rng.uniform(0.1, 100)
        eb = 10 ** rng.uniform(-9, -3) * float(x.max() - x.min())
        s = ref.compress(x, L=32, T=T, mode=mode, eb_mode=0, abs_eb=eb)
        assert s == port.compress_d(x, eb, 32, T, mode)
        y = ref.decompress(s, n, L=32, T=T, mode=mode, dtype=np.float64)
        assert np.array_equal(y.view(np.uint64), port.decompress_d(s, n, 32, T, mode).view(np.uint64))
        s = ref.compress(x, L=32, T=T, mode=mode, eb_mode=1, rel=1e-6)
        assert s == port.compress_d(x, port.rel_bound_d(x, 1e-6), 32, T, mode)
