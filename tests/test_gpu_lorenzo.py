"""The multidimensional Lorenzo variant on the GPU against the oracle's
restatement: streams byte for byte, decompressed floats bit for bit, through
the C ABI's device entry points."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.asarray(a, dtype=np.float32).view(np.uint32)


def _field(dims, rng):
    nz, ny, nx = dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = np.sin(0.05 * x + 0.3) * np.cos(0.07 * y) + np.sin(0.03 * z) + 1e-3 * rng.standard_normal(x.shape)
    return f.astype(np.float32).ravel()


@pytest.mark.parametrize("dims,T,mode", [((1, 1, 1), 1, "abs"), ((1, 1, 1000), 3, "rel"), ((1, 300, 217), 7, "abs"),
                                         ((33, 65, 129), 16, "rel"), ((64, 64, 64), 5, "abs"),
                                         ((2, 3, 700_001), 4, "rel")])
def test_lorenzo_parity(szp, port, dims, T, mode):
    import torch
    rng = np.random.default_rng(sum(dims) + T)
    f = _field(dims, rng)
    if mode == "rel":
        rel = 1e-3
        eb = port.rel_bound(f, rel)
        eb_mode, abs_eb = szp.REL, 0.0
    else:
        eb = float(np.float32(1e-4 * (f.max() - f.min()) + 1e-6))
        eb_mode, abs_eb, rel = szp.ABS, eb, 0.0
    want = port.lorenzo_compress(f, dims, eb, T)
    df = torch.from_numpy(f).cuda()
    cap = szp.lorenzo_max_stream_bytes(dims, T)
    ds = torch.empty(cap, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    size = szp.lorenzo_compress_dev(df.data_ptr(), dims, ds.data_ptr(), cap, eb_mode, abs_eb, rel, T, st)
    assert ds[:size].cpu().numpy().tobytes() == want
    dy = torch.empty(f.size, dtype=torch.float32, device="cuda")
    szp.lorenzo_decompress_dev(ds.data_ptr(), size, dims, dy.data_ptr(), T, st)
    y = dy.cpu().numpy()
    assert np.array_equal(bits(y), bits(port.lorenzo_decompress(want, dims, T)))
    # fastmode1's arithmetic: truncation by a float inverse of eb, then a float
    # product q * eb; each rounds within 2^-24 of its operands' magnitude
    err = np.abs(y.astype(np.float64) - f.astype(np.float64))
    assert np.all(err <= eb * (1 + 2.0 ** -22) + np.abs(f.astype(np.float64)) * 2.0 ** -22)


def test_lorenzo_errors_and_specials(szp, port):
    import torch
    rng = np.random.default_rng(3)
    dims = (4, 8, 40)
    f = _field(dims, rng)
    f[17] = np.nan  # codes INT_MIN like the reference's quantizer; a notice, not an error
    eb = 0.01
    T = 2
    df = torch.from_numpy(f).cuda()
    cap = szp.lorenzo_max_stream_bytes(dims, T)
    ds = torch.empty(cap, dtype=torch.uint8, device="cuda")
    size = szp.lorenzo_compress_dev(df.data_ptr(), dims, ds.data_ptr(), cap, szp.ABS, eb, 0.0, T)
    assert szp.last_notices() == 1
    want = port.lorenzo_compress(f, dims, eb, T)
    assert ds[:size].cpu().numpy().tobytes() == want
    dy = torch.empty(f.size, dtype=torch.float32, device="cuda")
    szp.lorenzo_decompress_dev(ds.data_ptr(), size, dims, dy.data_ptr(), T)
    assert np.array_equal(bits(dy.cpu().numpy()), bits(port.lorenzo_decompress(want, dims, T)))
    with pytest.raises(szp.SzpError):  # other dims than the stream's
        szp.lorenzo_decompress_dev(ds.data_ptr(), size, (8, 4, 40), dy.data_ptr(), T)
    with pytest.raises(szp.SzpError):  # capacity below the header
        szp.lorenzo_compress_dev(df.data_ptr(), dims, ds.data_ptr(), 8, szp.ABS, eb, 0.0, T)
    with pytest.raises(szp.SzpError):  # misaligned input
        szp.lorenzo_compress_dev(df.data_ptr() + 1, dims, ds.data_ptr(), cap, szp.ABS, eb, 0.0, T)
