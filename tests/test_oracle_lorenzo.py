"""The oracle's multidimensional Lorenzo variant (no reference code: its
parity is its own round trip, the error bound, and the stream layout it
defines).  CPU only."""
import numpy as np
import pytest

SHAPES = [(1, 1, 1), (1, 1, 37), (1, 5, 7), (3, 5, 7), (4, 33, 65), (9, 16, 31)]


@pytest.mark.parametrize("dims", SHAPES)
@pytest.mark.parametrize("T", [1, 3])
def test_round_trip_within_bound(port, dims, T):
    rng = np.random.default_rng(hash(dims) % 1000 + T)
    nz, ny, nx = dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = (np.sin(0.3 * x) * np.cos(0.2 * y) + 0.1 * z + 1e-3 * rng.standard_normal(x.shape)).astype(np.float32).ravel()
    eb = float(np.float32(1e-3 * (f.max() - f.min()) + 1e-6))
    s = port.lorenzo_compress(f, dims, eb, T)
    assert np.frombuffer(s[:12], dtype="<u4").tolist() == [nx, ny, nz]
    g = port.lorenzo_decompress(s, dims, T)
    # fastmode1's arithmetic: truncation by a float inverse of eb, then a float
    # product q * eb; each rounds within 2^-24 of its operands' magnitude
    err = np.abs(g.astype(np.float64) - f.astype(np.float64))
    assert np.all(err <= eb * (1 + 2.0 ** -22) + np.abs(f.astype(np.float64)) * 2.0 ** -22)


def test_codes_are_lorenzo_residuals(port):
    """The packed stream is fastmode1's over r = q - q[j-1] - q[k-1] +
    q[j-1][k-1]: decoding its fastmode1 part as codes gives r, and r summed
    along y and z gives the codes of the plain fastmode1 stream."""
    rng = np.random.default_rng(5)
    dims = (6, 10, 12)
    f = np.cumsum(rng.standard_normal(np.prod(dims))).astype(np.float32)
    eb = float(np.float32(0.05))
    s = port.lorenzo_compress(f, dims, eb, 1)
    inner = s[12:]
    # the same fastmode1 stream decoded to floats is r * eb; r summed back is q
    r = np.round(port.decompress(inner, f.size, 32, 1, 1) / np.float32(eb)).astype(np.int64).reshape(dims)
    q = np.cumsum(np.cumsum(r, axis=1), axis=0)
    y1 = port.decompress(port.compress(f, eb, 32, 1, 1), f.size, 32, 1, 1)
    assert np.array_equal(np.round(y1 / np.float32(eb)).astype(np.int64), q.ravel())


def test_wrong_dims_rejected(port):
    f = np.arange(60, dtype=np.float32)
    s = port.lorenzo_compress(f, (3, 4, 5), 0.5, 1)
    with pytest.raises(RuntimeError):
        port.lorenzo_decompress(s, (5, 4, 3), 1)
