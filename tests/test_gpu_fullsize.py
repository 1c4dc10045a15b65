"""The benchmark configurations at full size, through the device C ABI,
checked bit for bit against the oracle (the C restatement runs them in a
few seconds on the host cores):

* random walk, 2^24 floats, ABS eb = 1e-4 * range
* 512^3 Fourier field, REL 1e-2 / 1e-3 / 1e-4 (and fastmode2 at 1e-3)
* 8192^2 Laplace field with 40% zero blocks, ABS 1e-5

plus size-independent properties: decompressed values equal the oracle's,
and the set of points with |x - x'| > eb equals the oracle's.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T_HOST = min(os.cpu_count() or 8, 72)


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


def _roundtrip(szp, torch, dx, n, eb_mode, bound, T, mode=1):
    cap = szp.max_stream_bytes(n, 32, T, mode)
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    size = szp.compress_dev(dx.data_ptr(), n, dout.data_ptr(), cap, eb_mode,
                            bound if eb_mode == szp.ABS else 0.0, bound if eb_mode == szp.REL else 0.0,
                            32, T, mode, st)
    dy = torch.empty(n, dtype=torch.float32, device="cuda")
    szp.decompress_dev(dout.data_ptr(), size, n, dy.data_ptr(), 32, T, mode, st)
    assert szp.sync_status(st) == 0, szp.last_error()
    return dout[:size].cpu().numpy().tobytes(), dy.cpu().numpy()


def _check(szp, port, torch, x, eb_mode, bound, T=T_HOST, mode=1):
    dx = torch.from_numpy(x).cuda()
    s, y = _roundtrip(szp, torch, dx, x.size, eb_mode, bound, T, mode)
    eb = port.rel_bound(x, bound) if eb_mode == szp.REL else bound
    s_or = port.compress(x, eb, 32, T, mode)
    assert len(s) == len(s_or)
    assert s == s_or
    y_or = port.decompress(s_or, x.size, 32, T, mode)
    assert np.array_equal(y.view(np.uint32), y_or.view(np.uint32))
    ebf = np.float32(eb)
    viol = np.abs(x.astype(np.float64) - y.astype(np.float64)) > float(ebf)
    viol_or = np.abs(x.astype(np.float64) - y_or.astype(np.float64)) > float(ebf)
    assert np.array_equal(viol, viol_or)
    return len(s), int(viol.sum())


def test_walk_2p24(szp, port, torch):
    from szp_gb300.workloads import walk
    x = walk(1 << 24, np.random.default_rng(1))
    eb = float(np.float32(1e-4 * (float(x.max()) - float(x.min()))))
    size, nviol = _check(szp, port, torch, x, szp.ABS, eb)
    assert 4 * x.size / size > 4.0  # smooth field compresses


@pytest.mark.parametrize("rel", [1e-2, 1e-3, 1e-4])
def test_fourier_512cube(szp, port, torch, rel):
    from szp_gb300.workloads import fourier3d_torch
    x = fourier3d_torch(512, 2, device="cuda").cpu().numpy()
    _check(szp, port, torch, x, szp.REL, rel)


def test_fourier_512cube_fastmode2(szp, port, torch):
    """fastmode2 (a seed per block, no cross-block prefix) at full size."""
    from szp_gb300.workloads import fourier3d_torch
    x = fourier3d_torch(512, 2, device="cuda").cpu().numpy()
    _check(szp, port, torch, x, szp.REL, 1e-3, mode=2)


def test_laplace_8192sq(szp, port, torch):
    from szp_gb300.workloads import laplace_zero_patches
    x = laplace_zero_patches(8192, 8192, np.random.default_rng(3)).ravel()
    _check(szp, port, torch, x, szp.ABS, 1e-5)


def test_segment_counts_fullsize(szp, port, torch):
    """T changes the stream; a few T at 2^24 incl. the reference's default."""
    from szp_gb300.workloads import walk
    x = walk(1 << 24, np.random.default_rng(4))
    eb = float(np.float32(1e-3 * (float(x.max()) - float(x.min()))))
    for T in (1, 2, 16, 144):
        _check(szp, port, torch, x, szp.ABS, eb, T)
