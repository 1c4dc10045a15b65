"""float64 data (the reference's szp_double_* path): the CUDA library against
the reference's golden vectors and the oracle.  Streams byte for byte,
decompressed doubles bit for bit."""
import ctypes

import numpy as np
import pytest

from conftest import eb_of_double

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need CUDA"
    return t


@pytest.fixture(autouse=True)
def _reset_segments(szp):
    yield
    szp.set_segments(0)


def bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


def test_golden_double_host_api(szp, golden_double):
    for c in golden_double:
        szp.set_segments(c["T"])
        if c["eb_mode"] == 1:
            s = szp.szp_compress(c["x"], szp.REL, 0.0, c["bound"], c["L"], c["mode"], szp.SZ_DOUBLE)
        else:
            s = szp.szp_compress(c["x"], szp.ABS, eb_of_double(c["s"]), 0.0, c["L"], c["mode"], szp.SZ_DOUBLE)
        assert s == c["s"], c["name"]
        y = szp.szp_decompress(c["s"], c["n"], c["L"], c["mode"], szp.SZ_DOUBLE)
        assert np.array_equal(bits(y), bits(c["y"])), c["name"]


def test_golden_double_per_type_entries(szp, golden_double):
    lib = szp._lib
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [ctypes.c_void_p]
    for c in golden_double[:24]:
        if c["eb_mode"] != 0:
            continue
        szp.set_segments(c["T"])
        x = np.ascontiguousarray(c["x"], dtype=np.float64)
        eb = eb_of_double(c["s"])
        n, L = c["n"], c["L"]
        size = ctypes.c_size_t(0)
        fn = lib.szp_double_openmp_threadblock if c["mode"] == 1 else lib.szp_double_openmp_threadblock_randomaccess
        p = fn(x.ctypes.data, ctypes.byref(size), eb, n, L)
        assert p, c["name"]
        assert ctypes.string_at(p, size.value) == c["s"], c["name"]
        libc.free(p)
        out = np.zeros(8 + 8 * n + 64, dtype=np.uint8)
        fn = lib.szp_double_openmp_threadblock_arg if c["mode"] == 1 else \
            lib.szp_double_openmp_threadblock_randomaccess_arg
        fn(out.ctypes.data, x.ctypes.data, ctypes.byref(size), eb, n, L)
        assert out[: size.value].tobytes() == c["s"], c["name"]
        buf = np.frombuffer(c["s"], dtype=np.uint8).copy()
        fn = lib.szp_double_decompress_openmp_threadblock if c["mode"] == 1 else \
            lib.szp_double_decompress_openmp_threadblock_randomaccess
        q = fn(n, eb, L, buf.ctypes.data + 8)
        assert q, c["name"]
        y = np.frombuffer(ctypes.string_at(q, 8 * n), dtype=np.float64)
        assert np.array_equal(bits(y), bits(c["y"])), c["name"]
        libc.free(q)
        y2 = np.zeros(n, dtype=np.float64)
        fn = lib.szp_double_decompress_openmp_threadblock_arg if c["mode"] == 1 else \
            lib.szp_double_decompress_openmp_threadblock_randomaccess_arg
        fn(y2.ctypes.data, n, eb, L, buf.ctypes.data + 8)
        assert np.array_equal(bits(y2), bits(c["y"])), c["name"]
    # the single-thread entries are the T = 1 stream
    c = next(c for c in golden_double if c["T"] == 1 and c["mode"] == 1 and c["eb_mode"] == 0)
    x = np.ascontiguousarray(c["x"], dtype=np.float64)
    out = np.zeros(8 + 8 * c["n"] + 64, dtype=np.uint8)
    size = ctypes.c_size_t(0)
    lib.szp_double_single_thread_arg(out.ctypes.data, x.ctypes.data, ctypes.byref(size), eb_of_double(c["s"]),
                                     c["n"], c["L"])
    assert out[: size.value].tobytes() == c["s"]


@pytest.mark.parametrize("L", [32, 7, 64])
@pytest.mark.parametrize("mode", [1, 2])
def test_double_device_api_vs_oracle(szp, port, torch, L, mode):
    from szp_gb300.workloads import walk64
    rng = np.random.default_rng(300 + L + mode)
    n, T = 1_000_003, 13
    x = walk64(n, rng) * 1e3
    dx = torch.from_numpy(x).cuda()
    cap = szp.max_stream_bytes_f64(n, L, T, mode)
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for rel in (1e-4, 1e-8):
        size = szp.compress_dev_f64(dx.data_ptr(), n, dout.data_ptr(), cap, szp.REL, 0.0, rel, L, T, mode, st)
        s = dout[:size].cpu().numpy().tobytes()
        assert s == port.compress_d(x, port.rel_bound_d(x, rel), L, T, mode)
        dy = torch.empty(n, dtype=torch.float64, device="cuda")
        szp.decompress_dev_f64(dout.data_ptr(), size, n, dy.data_ptr(), L, T, mode, st)
        assert np.array_equal(bits(dy.cpu().numpy()), bits(port.decompress_d(s, n, L, T, mode)))


def test_double_large_field(szp, port, torch):
    """2^25 doubles (256 MiB, larger than L2) at 16 segments, both fastmodes."""
    from szp_gb300.workloads import walk64
    rng = np.random.default_rng(77)
    n, T, L = 1 << 25, 16, 32
    x = walk64(n, rng)
    dx = torch.from_numpy(x).cuda()
    st = torch.cuda.current_stream().cuda_stream
    for mode in (1, 2):
        cap = szp.max_stream_bytes_f64(n, L, T, mode)
        dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
        size = szp.compress_dev_f64(dx.data_ptr(), n, dout.data_ptr(), cap, szp.REL, 0.0, 1e-6, L, T, mode, st)
        s = dout[:size].cpu().numpy().tobytes()
        assert s == port.compress_d(x, port.rel_bound_d(x, 1e-6), L, T, mode)
        dy = torch.empty(n, dtype=torch.float64, device="cuda")
        szp.decompress_dev_f64(dout.data_ptr(), size, n, dy.data_ptr(), L, T, mode, st)
        assert np.array_equal(bits(dy.cpu().numpy()), bits(port.decompress_d(s, n, L, T, mode)))


def test_double_host_api_tiny_and_empty(szp, port):
    szp.set_segments(4)
    for n in (0, 1, 5, 8, 33):
        x = np.linspace(-2.0, 3.0, n)
        s = szp.szp_compress(x, szp.ABS, 1e-3, 0.0, 32, 1, szp.SZ_DOUBLE)
        assert s == port.compress_d(x, 1e-3, 32, 4, 1), n
        y = szp.szp_decompress(s, n, 32, 1, szp.SZ_DOUBLE)
        assert np.array_equal(bits(y), bits(port.decompress_d(s, n, 32, 4, 1))), n


@pytest.mark.parametrize("L", [8, 32, 256, 24])
@pytest.mark.parametrize("mode", [1, 2])
def test_double_views_off_16_byte_boundaries(szp, port, torch, L, mode):
    """Input and output one double past a 16-byte boundary (the quantization
    and dequantization passes' ragged heads), for the pipeline blockSizes and
    the one-warp-per-block kernels alike."""
    from szp_gb300.workloads import walk64
    rng = np.random.default_rng(500 + L + mode)
    n, T = 300_007, 5
    x = walk64(n + 1, rng)
    dx = torch.from_numpy(x).cuda()[1:]
    assert dx.data_ptr() % 16 == 8
    xs = x[1:].copy()
    st = torch.cuda.current_stream().cuda_stream
    cap = szp.max_stream_bytes_f64(n, L, T, mode)
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    size = szp.compress_dev_f64(dx.data_ptr(), n, dout.data_ptr(), cap, szp.REL, 0.0, 1e-5, L, T, mode, st)
    s = dout[:size].cpu().numpy().tobytes()
    assert s == port.compress_d(xs, port.rel_bound_d(xs, 1e-5), L, T, mode)
    dy = torch.full((n + 1,), 7.0, dtype=torch.float64, device="cuda")
    szp.decompress_dev_f64(dout.data_ptr(), size, n, dy[1:].data_ptr(), L, T, mode, st)
    y = dy.cpu().numpy()
    assert y[0] == 7.0
    assert np.array_equal(bits(y[1:]), bits(port.decompress_d(s, n, L, T, mode)))


def test_double_misaligned_pointers_rejected(szp, torch):
    """A double pointer off its 8-byte alignment is refused before any launch."""
    dx = torch.zeros(1024, dtype=torch.float64, device="cuda")
    cap = szp.max_stream_bytes_f64(1000, 32, 4, 1)
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    with pytest.raises(szp.SzpError):
        szp.compress_dev_f64(dx.data_ptr() + 4, 1000, dout.data_ptr(), cap, szp.ABS, 1e-3, 0.0, 32, 4, 1, st)
    size = szp.compress_dev_f64(dx.data_ptr(), 1000, dout.data_ptr(), cap, szp.ABS, 1e-3, 0.0, 32, 4, 1, st)
    with pytest.raises(szp.SzpError):
        szp.decompress_dev_f64(dout.data_ptr(), size, 1000, dx.data_ptr() + 4, 32, 4, 1, st)
