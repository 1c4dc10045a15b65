"""Homomorphic sum of two device streams (szp_gb300_reduce_sum_dev) against
the oracle's reduce_sum, byte for byte, for float and double streams."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need CUDA"
    return t


def _walk32(n, rng):
    return np.cumsum(rng.normal(0.0, 0.05, n)).astype(np.float32)


@pytest.mark.parametrize("L", [8, 32, 256])
@pytest.mark.parametrize("mode", [1, 2])
def test_reduce_sum_float_streams(szp, port, torch, L, mode):
    rng = np.random.default_rng(90 + L + mode)
    n, T, eb = 1_000_003, 7, 1e-3
    x1, x2 = _walk32(n, rng), _walk32(n, rng)
    st = torch.cuda.current_stream().cuda_stream
    cap = szp.max_stream_bytes(n, L, T, mode)
    bufs = [torch.empty(cap, dtype=torch.uint8, device="cuda") for _ in range(3)]
    sizes = []
    for x, buf in zip((x1, x2), bufs):
        dx = torch.from_numpy(x).cuda()
        sizes.append(szp.compress_dev(dx.data_ptr(), n, buf.data_ptr(), cap, szp.ABS, eb, 0.0, L, T, mode, st))
    a = bufs[0][: sizes[0]].cpu().numpy().tobytes()
    b = bufs[1][: sizes[1]].cpu().numpy().tobytes()
    size = szp.reduce_sum_dev(bufs[0].data_ptr(), sizes[0], bufs[1].data_ptr(), sizes[1], n, bufs[2].data_ptr(), cap,
                              L, T, mode, szp.SZ_FLOAT, st)
    s = bufs[2][:size].cpu().numpy().tobytes()
    assert s == port.reduce_sum(a, b, n, L, T, mode, hb=4)
    dy = torch.empty(n, dtype=torch.float32, device="cuda")
    szp.decompress_dev(bufs[2].data_ptr(), size, n, dy.data_ptr(), L, T, mode, st)
    torch.cuda.synchronize()
    assert np.array_equal(dy.cpu().numpy().view(np.int32), port.decompress(s, n, L, T, mode).view(np.int32))


@pytest.mark.parametrize("mode", [1, 2])
def test_reduce_sum_double_streams(szp, port, torch, mode):
    from szp_gb300.workloads import walk64
    rng = np.random.default_rng(3 + mode)
    n, T, L = 777_777, 5, 32
    x1, x2 = walk64(n, rng), walk64(n, rng)
    st = torch.cuda.current_stream().cuda_stream
    cap = szp.max_stream_bytes_f64(n, L, T, mode)
    bufs = [torch.empty(cap, dtype=torch.uint8, device="cuda") for _ in range(3)]
    sizes = []
    for x, buf in zip((x1, x2), bufs):
        dx = torch.from_numpy(x).cuda()
        sizes.append(szp.compress_dev_f64(dx.data_ptr(), n, buf.data_ptr(), cap, szp.ABS, 1e-6, 0.0, L, T, mode, st))
    a = bufs[0][: sizes[0]].cpu().numpy().tobytes()
    b = bufs[1][: sizes[1]].cpu().numpy().tobytes()
    size = szp.reduce_sum_dev(bufs[0].data_ptr(), sizes[0], bufs[1].data_ptr(), sizes[1], n, bufs[2].data_ptr(), cap,
                              L, T, mode, szp.SZ_DOUBLE, st)
    assert bufs[2][:size].cpu().numpy().tobytes() == port.reduce_sum(a, b, n, L, T, mode, hb=8)


def test_reduce_sum_refusals(szp, torch):
    n, T, L = 10_000, 2, 32
    st = torch.cuda.current_stream().cuda_stream
    dx = torch.linspace(0, 1, n, device="cuda")
    cap = szp.max_stream_bytes(n, L, T, 1)
    a = torch.empty(cap, dtype=torch.uint8, device="cuda")
    b = torch.empty(cap, dtype=torch.uint8, device="cuda")
    out = torch.empty(cap, dtype=torch.uint8, device="cuda")
    sa = szp.compress_dev(dx.data_ptr(), n, a.data_ptr(), cap, szp.ABS, 1e-3, 0.0, L, T, 1, st)
    sb = szp.compress_dev(dx.data_ptr(), n, b.data_ptr(), cap, szp.ABS, 2e-3, 0.0, L, T, 1, st)
    with pytest.raises(szp.SzpError):  # different bounds
        szp.reduce_sum_dev(a.data_ptr(), sa, b.data_ptr(), sb, n, out.data_ptr(), cap, L, T, 1, szp.SZ_FLOAT, st)
    s7 = szp.compress_dev(dx.data_ptr(), n, b.data_ptr(), cap, szp.ABS, 1e-3, 0.0, 7, T, 1, st)
    with pytest.raises(szp.SzpError):  # blockSize outside the pipelines' 8..256
        szp.reduce_sum_dev(b.data_ptr(), s7, b.data_ptr(), s7, n, out.data_ptr(), cap, 7, T, 1, szp.SZ_FLOAT, st)
    # the device still works
    size = szp.reduce_sum_dev(a.data_ptr(), sa, a.data_ptr(), sa, n, out.data_ptr(), cap, L, T, 1, szp.SZ_FLOAT, st)
    assert size > 0


def test_reduce_sum_wraps_with_notice(szp, port, torch):
    """Codes near 1.5e9 sum past 2^31: the result holds the wrapped codes,
    as the oracle's, and the call reports a notice."""
    rng = np.random.default_rng(11)
    n, T, L = 200_000, 3, 32
    x = (1.5e9 + 128.0 * rng.integers(-1000, 1000, n)).astype(np.float32)  # exact floats, codes ~1.5e9 at eb 1
    st = torch.cuda.current_stream().cuda_stream
    cap = szp.max_stream_bytes(n, L, T, 1)
    a = torch.empty(cap, dtype=torch.uint8, device="cuda")
    out = torch.empty(cap, dtype=torch.uint8, device="cuda")
    dx = torch.from_numpy(x).cuda()
    sa = szp.compress_dev(dx.data_ptr(), n, a.data_ptr(), cap, szp.ABS, 1.0, 0.0, L, T, 1, st)
    size = szp.reduce_sum_dev(a.data_ptr(), sa, a.data_ptr(), sa, n, out.data_ptr(), cap, L, T, 1, szp.SZ_FLOAT, st)
    assert szp._lib.szp_gb300_last_notices() == 1
    sbytes = a[:sa].cpu().numpy().tobytes()
    assert out[:size].cpu().numpy().tobytes() == port.reduce_sum(sbytes, sbytes, n, L, T, 1, hb=4)
