"""Parity of the CUDA library (through its C ABI) with the reference's golden
vectors and with the oracle, plus its error paths.  Bit-exact throughout:
streams byte for byte, decompressed floats bit for bit."""
import ctypes

import numpy as np
import pytest

from conftest import eb_of

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
    return np.asarray(a, dtype=np.float32).view(np.uint32)


def test_golden_host_api(szp, golden):
    for c in golden:
        szp.set_segments(c["T"])
        if c["eb_mode"] == 1:
            s = szp.szp_compress(c["x"], szp.REL, 0.0, c["bound"], c["L"], c["mode"])
        else:
            s = szp.szp_compress(c["x"], szp.ABS, eb_of(c["s"]), 0.0, c["L"], c["mode"])
        assert s == c["s"], c["name"]
        y = szp.szp_decompress(c["s"], c["n"], c["L"], c["mode"])
        assert np.array_equal(bits(y), bits(c["y"])), c["name"]


def test_golden_per_type_entries(szp, golden):
    """szp_float_* entry points, including the length-less decompressors."""
    for c in golden:
        if c["eb_mode"] == 1:
            continue
        szp.set_segments(c["T"])
        eb = eb_of(c["s"])
        if c["mode"] == 1:
            assert szp.szp_float_openmp_threadblock(c["x"], eb, c["L"]) == c["s"], c["name"]
            if len(c["s"]) <= 4 + 4 * c["n"]:
                assert szp.szp_float_openmp_threadblock_arg(c["x"], eb, c["L"]) == c["s"], c["name"]
            if c["T"] == 1 and len(c["s"]) <= 4 + 4 * c["n"]:
                assert szp.szp_float_single_thread_arg(c["x"], eb, c["L"]) == c["s"], c["name"]
                y1 = szp.szp_float_decompress_arg(c["s"], c["n"], c["L"], "single_thread_arg")
                assert np.array_equal(bits(y1), bits(c["y"])), c["name"]
            y = szp.szp_float_decompress_openmp_threadblock(c["s"], c["n"], c["L"], 1)
            y2 = szp.szp_float_decompress_arg(c["s"], c["n"], c["L"], "openmp_threadblock_arg")
        else:
            assert szp.szp_float_openmp_threadblock_randomaccess(c["x"], eb, c["L"]) == c["s"], c["name"]
            y = szp.szp_float_decompress_openmp_threadblock(c["s"], c["n"], c["L"], 2)
            y2 = szp.szp_float_decompress_arg(c["s"], c["n"], c["L"], "openmp_threadblock_randomaccess_arg")
        assert np.array_equal(bits(y), bits(c["y"])), c["name"]
        assert np.array_equal(bits(y2), bits(c["y"])), c["name"]


def _fields(rng, n):
    from szp_gb300.workloads import walk, laplace_zero_patches, specials
    kind = rng.integers(0, 4)
    if kind == 0:
        return walk(n, rng) * np.float32(rng.uniform(0.01, 1000))
    if kind == 1:
        side = int(np.sqrt(n)) + 1
        return laplace_zero_patches(side, side, rng).ravel()[:n]
    if kind == 2:
        x = specials(rng, max(n, 50))[:n]
        return x
    # wide dynamic range: exercises the exact-quantization slow path
    return (rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 6, n)).astype(np.float32)


def test_random_parity_vs_oracle(szp, port):
    rng = np.random.default_rng(77)
    for it in range(60):
        n = int(rng.choice([1, 2, 5, 31, 32, 33, 100, 1000, 4097, 65536, 200001, 1 << 20]))
        T = int(rng.choice([1, 2, 3, 7, 8, 16, 72, 150]))
        L = int(rng.choice([32, 32, 32, 8, 16, 64, 128, 1, 3, 33]))
        mode = int(rng.choice([1, 1, 2]))
        x = _fields(rng, n)
        finite = x[np.isfinite(x)]
        with np.errstate(over="ignore"):
            rng_v = float(finite.max() - finite.min()) if finite.size else 1.0  # may be inf: eb = inf
        eb = float(np.float32(max(rng_v, 1e-6) * 10 ** rng.uniform(-7, -1)))
        szp.set_segments(T)
        s = szp.szp_compress(x, szp.ABS, eb, 0.0, L, mode)
        s_or = port.compress(x, eb, L, T, mode)
        assert s == s_or, (it, n, T, L, mode, eb)
        y = szp.szp_decompress(s, n, L, mode)
        assert np.array_equal(bits(y), bits(port.decompress(s_or, n, L, T, mode))), (it, n, T, L, mode)


def test_rel_parity_vs_oracle(szp, port):
    rng = np.random.default_rng(78)
    from szp_gb300.workloads import walk
    for it in range(12):
        n = int(rng.integers(1, 300000))
        x = walk(n, rng)
        if it % 3 == 0:
            x[0] = np.nan  # range becomes NaN, like the reference's loop
        if it % 4 == 1:
            x[:] = np.float32(2.5)  # constant field: range 0
        rel = float(10 ** rng.uniform(-5, -2))
        T = int(rng.integers(1, 20))
        szp.set_segments(T)
        s = szp.szp_compress(x, szp.REL, 0.0, rel, 32, 1)
        eb = port.rel_bound(x, rel)
        s_or = port.compress(x, eb, 32, T, 1)
        assert s == s_or, (it, n, T, rel)


def test_rel_range_pass_offsets(szp, port, torch):
    """The range pass over inputs of 256 Ki values and more streams the
    16-byte-aligned body by bulk copy and reads the elements before and after
    it one by one: inputs starting 0-3 floats past a 16-byte boundary, lengths
    of every residue mod 4, the extremes placed in the head and the tail, and
    NaNs (skipped, or the range itself when x[0] is NaN)."""
    rng = np.random.default_rng(86)
    from szp_gb300.workloads import walk
    N = 1_200_011
    base = walk(N, rng)
    dbase = torch.from_numpy(base).cuda()
    st = torch.cuda.current_stream().cuda_stream
    T = 11
    for off in range(4):
        for k, case in enumerate(["extremes", "nan_inside", "nan_first"]):
            n = N - off - 4 - k
            x = base[off:off + n].copy()
            if case == "extremes":
                x[1] = np.float32(x.max() + 7.0)    # in the scalar head when the start is unaligned
                x[n - 1] = np.float32(x.min() - 5.0)  # in the scalar tail when n - head is not a multiple of 4
            elif case == "nan_inside":
                x[n // 2] = np.nan
            else:
                x[0] = np.nan
            dbase[off:off + n].copy_(torch.from_numpy(x))
            rel = 1e-3
            cap = szp.max_stream_bytes(n, 32, T, 1)
            dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
            ptr = dbase.data_ptr() + 4 * off
            size = szp.compress_dev(ptr, n, dout.data_ptr(), cap, szp.REL, 0.0, rel, 32, T, 1, st)
            s = dout[:size].cpu().numpy().tobytes()
            eb = port.rel_bound(x, rel)
            assert s == port.compress(x, eb, 32, T, 1), (off, case)
            dbase[off:off + n].copy_(torch.from_numpy(base[off:off + n]))


def test_device_api(szp, port, torch):
    rng = np.random.default_rng(79)
    from szp_gb300.workloads import walk
    n, T = 1_000_003, 13
    x = walk(n, rng)
    eb = float(np.float32(1e-4 * (x.max() - x.min())))
    dx = torch.from_numpy(x).cuda()
    cap = szp.max_stream_bytes(n, 32, T, 1)
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    size = szp.compress_dev(dx.data_ptr(), n, dout.data_ptr(), cap, szp.ABS, eb, 0.0, 32, T, 1, st)
    s = dout[:size].cpu().numpy().tobytes()
    assert s == port.compress(x, eb, 32, T, 1)
    dy = torch.empty(n, dtype=torch.float32, device="cuda")
    szp.decompress_dev(dout.data_ptr(), size, n, dy.data_ptr(), 32, T, 1, st)
    assert szp.sync_status(st) == 0
    assert np.array_equal(bits(dy.cpu().numpy()), bits(port.decompress(s, n, 32, T, 1)))
    # async size into device memory
    dsize = torch.zeros(1, dtype=torch.int64, device="cuda")
    szp.compress_dev_async(dx.data_ptr(), n, dout.data_ptr(), cap, dsize.data_ptr(), szp.ABS, eb, 0.0, 32, T, 1, st)
    assert szp.sync_status(st) == 0
    assert int(dsize.item()) == size


def test_host_api_large_results(szp, port):
    """Results above 32 MiB leave the device in pieces while host threads map
    the malloc'd pages ahead: the bytes must be those of the oracle."""
    rng = np.random.default_rng(81)
    from szp_gb300.workloads import walk
    n, T = 24_000_003, 16
    x = walk(n, rng)
    eb = float(np.float32(1e-7 * (x.max() - x.min())))
    szp.set_segments(T)
    s = szp.szp_compress(x, szp.ABS, eb, 0.0, 32, 1)
    assert len(s) > 32 << 20
    assert s == port.compress(x, eb, 32, T, 1)
    y = szp.szp_decompress(s, n, 32, 1)
    assert np.array_equal(bits(y), bits(port.decompress(s, n, 32, T, 1)))


def test_bounded_wait_gives_up(szp, port):
    """A device wait on a barrier that nothing completes gives up after its
    limit and reports a timeout; the device stays usable."""
    rc, waited = szp.wait_probe(50_000_000)
    assert rc == szp.ETIMEOUT
    assert 50_000_000 <= waited < 2_000_000_000
    x = np.linspace(-1.0, 1.0, 100_000, dtype=np.float32)
    szp.set_segments(4)
    s = szp.szp_compress(x, szp.ABS, 1e-3, 0.0, 32, 1)
    assert s == port.compress(x, 1e-3, 32, 4, 1)


def test_empty_and_tiny(szp, port):
    for T in (1, 4):
        szp.set_segments(T)
        for n in (0, 1, 2, 3):
            x = np.linspace(-1, 1, n).astype(np.float32)
            s = szp.szp_compress(x, szp.ABS, 1e-3, 0.0, 32, 1)
            assert s == port.compress(x, 1e-3, 32, T, 1), (T, n)
            y = szp.szp_decompress(s, n, 32, 1)
            assert np.array_equal(bits(y), bits(port.decompress(s, n, 32, T, 1)))


def test_bitcount_probe(szp, port, torch):
    thr = port.thresholds().astype(np.int64)
    vals = [0, 1, 2, 3, 0xFFFFFFFF, 0x80000000, 0x7FFFFFFF]
    for t in thr[1:]:
        for d in range(-3, 4):
            v = int(t) + d
            if 0 <= v <= 0xFFFFFFFF:
                vals.append(v)
    rng = np.random.default_rng(3)
    vals += list(rng.integers(0, 2 ** 32, 100000, dtype=np.uint64))
    v = np.array(vals, dtype=np.uint32)
    dv = torch.from_numpy(v.view(np.int32)).cuda()
    db = torch.zeros(v.size, dtype=torch.uint8, device="cuda")
    assert szp.lib.szp_gb300_bitcount_probe(dv.data_ptr(), db.data_ptr(), v.size, None) == 0
    torch.cuda.synchronize()
    got = db.cpu().numpy()
    want = np.array([port.bitcount(int(m)) for m in v], dtype=np.uint8)
    assert np.array_equal(got, want)


def test_corrupt_streams_fail_cleanly(szp, port):
    from szp_gb300.workloads import walk
    rng = np.random.default_rng(80)
    n, T = 50000, 4
    x = walk(n, rng)
    eb = 1e-3
    s = bytearray(port.compress(x, eb, 32, T, 1))
    szp.set_segments(T)
    # bit count byte out of range right after segment 1's seed
    off1 = int.from_bytes(s[4 + 8:4 + 16], "little")
    bad = bytearray(s)
    bad[4 + 8 * T + off1 + 4] = 200
    with pytest.raises(szp.SzpError) as e:
        szp.szp_decompress(bytes(bad), n, 32, 1)
    assert e.value.status == szp.ECORRUPT
    # offsets past the end
    bad = bytearray(s)
    bad[4 + 8:4 + 16] = (len(s) * 4).to_bytes(8, "little")
    with pytest.raises(szp.SzpError):
        szp.szp_decompress(bytes(bad), n, 32, 1)
    # truncated stream
    with pytest.raises(szp.SzpError):
        szp.szp_decompress(bytes(s[: len(s) // 2]), n, 32, 1)
    # the library still works afterwards
    y = szp.szp_decompress(bytes(s), n, 32, 1)
    assert np.array_equal(bits(y), bits(port.decompress(bytes(s), n, 32, T, 1)))


def test_capacity_error(szp, torch):
    n = 100000
    x = torch.randn(n, device="cuda") * 1e6
    cap = 4 + 8 * 2 + 100
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    size = ctypes.c_size_t(0)
    rc = szp.lib.szp_gb300_compress_dev(1, x.data_ptr(), n, szp.ABS, 1e-3, 0.0, 32, 2, dout.data_ptr(), cap,
                                        ctypes.byref(size), None)
    assert rc == szp.ECAPACITY
    assert size.value > cap  # the needed size is reported


def test_bad_arguments(szp):
    x = np.ones(10, np.float32)
    with pytest.raises(szp.SzpError):
        szp.szp_compress(x, szp.ABS, 1e-3, 0.0, 0, 1)  # blockSize 0 loops forever in the reference
    with pytest.raises(szp.SzpError):
        szp.szp_compress(x, szp.ABS, 1e-3, 0.0, 32, 3)
    with pytest.raises(szp.SzpError):
        szp.szp_compress(x, szp.ABS, 1e-3, 0.0, 0, 1, data_type=szp.SZ_DOUBLE)
    with pytest.raises(szp.SzpError):  # segment offsets past the stream's end
        szp.szp_decompress(b"\xff" * 400, 10, 32, 1, data_type=szp.SZ_DOUBLE)


@pytest.mark.parametrize("overlap", [0, 3, 40])
def test_locate_repair_path(szp, port, overlap):
    """Short overlaps make speculative chunk walks miss the header chain; the
    in-order repair must still recover every block."""
    from szp_gb300.workloads import walk, laplace_zero_patches
    rng = np.random.default_rng(81 + overlap)
    szp.set_locate_overlap(overlap)
    try:
        for T, n, L in ((1, 400_000, 32), (5, 1_000_000, 32), (3, 300_000, 64), (2, 200_000, 8)):
            x = walk(n, rng) if T != 5 else laplace_zero_patches(1000, 1000, rng).ravel()
            eb = float(np.float32(1e-5 * (x.max() - x.min()) + 1e-7))
            s = port.compress(x, eb, L, T, 1)
            szp.set_segments(T)
            y = szp.szp_decompress(s, n, L, 1)
            assert np.array_equal(bits(y), bits(port.decompress(s, n, L, T, 1))), (overlap, T, n, L)
    finally:
        szp.set_locate_overlap(-1)


def test_decode_ticket_schedule(szp, port):
    """A single field's decode runs cooperatively with a static tile order; when
    a cooperative launch is refused it draws tile tickets instead.  Both
    schedules must decode every stream the same, fastmode1 and fastmode2."""
    from szp_gb300.workloads import walk
    rng = np.random.default_rng(87)
    cases = ((16, 3_000_001, 32, 1), (7, 1_000_000, 8, 1), (4, 2_000_003, 32, 2))
    try:
        for T, n, L, mode in cases:
            x = walk(n, rng)
            eb = float(np.float32(1e-4 * (x.max() - x.min())))
            s = port.compress(x, eb, L, T, mode)
            want = bits(port.decompress(s, n, L, T, mode))
            szp.set_segments(T)
            for tickets in (False, True):
                szp.set_decode_tickets(tickets)
                y = szp.szp_decompress(s, n, L, mode)
                assert np.array_equal(bits(y), want), (T, n, L, mode, tickets)
    finally:
        szp.set_decode_tickets(False)
