"""The homomorphic sum of two streams (hZCCL's use of fZ-light streams) in
the oracle: the stream of the summed quantization codes.  Not a reference
function, so its properties are checked: commutativity, the zero stream as
identity, the decompressed values (q_a + q_b) * eb, and the 2 * eb bound on
the sum of the two original fields."""
import numpy as np
import pytest

from szp_gb300.workloads import walk64


def _walk32(n, rng):
    return np.cumsum(rng.normal(0.0, 0.05, n)).astype(np.float32)


@pytest.mark.parametrize("L", [8, 32, 64])
@pytest.mark.parametrize("mode", [1, 2])
def test_reduce_sum_float(port, L, mode):
    rng = np.random.default_rng(40 + L + mode)
    n, T, eb = 20011, 3, 1e-3
    x1, x2 = _walk32(n, rng), _walk32(n, rng)
    a = port.compress(x1, eb, L, T, mode)
    b = port.compress(x2, eb, L, T, mode)
    s = port.reduce_sum(a, b, n, L, T, mode, hb=4)
    assert s[:4] == a[:4]
    assert s == port.reduce_sum(b, a, n, L, T, mode, hb=4)
    z = port.compress(np.zeros(n, np.float32), eb, L, T, mode)
    assert port.reduce_sum(a, z, n, L, T, mode, hb=4) == a
    ebf = np.float32(eb)
    qa = np.rint(port.decompress(a, n, L, T, mode) / ebf).astype(np.int32)
    qb = np.rint(port.decompress(b, n, L, T, mode) / ebf).astype(np.int32)
    ys = port.decompress(s, n, L, T, mode)
    assert np.array_equal(ys, (qa + qb).astype(np.float32) * ebf)
    assert np.abs(ys.astype(np.float64) - (x1.astype(np.float64) + x2)).max() <= 2 * eb * (1 + 1e-4)


@pytest.mark.parametrize("mode", [1, 2])
def test_reduce_sum_double(port, mode):
    rng = np.random.default_rng(7 + mode)
    n, T, L, eb = 30011, 4, 32, 1e-6
    x1, x2 = walk64(n, rng), walk64(n, rng)
    a = port.compress_d(x1, eb, L, T, mode)
    b = port.compress_d(x2, eb, L, T, mode)
    s = port.reduce_sum(a, b, n, L, T, mode, hb=8)
    assert s[:8] == a[:8] and s == port.reduce_sum(b, a, n, L, T, mode, hb=8)
    qa = np.rint(port.decompress_d(a, n, L, T, mode) / eb).astype(np.int64)
    qb = np.rint(port.decompress_d(b, n, L, T, mode) / eb).astype(np.int64)
    ys = port.decompress_d(s, n, L, T, mode)
    assert np.array_equal(ys, (qa + qb).astype(np.float64) * eb)
    assert np.abs(ys - (x1 + x2)).max() <= 2 * eb * (1 + 1e-9)


def test_reduce_sum_rejects_different_bounds(port):
    rng = np.random.default_rng(1)
    x = _walk32(5000, rng)
    a = port.compress(x, 1e-3, 32, 2, 1)
    b = port.compress(x, 2e-3, 32, 2, 1)
    with pytest.raises(RuntimeError):
        port.reduce_sum(a, b, 5000, 32, 2, 1, hb=4)
