"""The allocation-free compressor, szp_gb300_compress_dev_noalloc.

It exists for callers that cannot allocate device memory while they compress
-- a process whose GPU memory all belongs to its own pool, or a serving loop
that must not take the device-wide synchronisation of cudaMalloc/cudaFree.
They pass device input and output buffers; the kernels' working memory is a
static device array inside the library.  Its stream must be byte-for-byte the
one the allocating entry point (szp_gb300_compress_dev) produces, and the
oracle's, on consecutive calls that reuse the shared array.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _calls(szp, rng):
    from szp_gb300.workloads import walk, laplace_zero_patches
    return [
        (walk(3_000_001, rng), szp.REL, 1e-4),
        (laplace_zero_patches(1500, 1500, rng).ravel(), szp.ABS, 1e-5),
    ]


def test_noalloc_matches_allocating_entry_on_consecutive_calls(szp, port):
    import torch

    assert torch.cuda.is_available()
    rng = np.random.default_rng(2024)
    T = 7
    for x, mode, bound in _calls(szp, rng):  # two calls in a row share the static array
        dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        cap = szp.max_stream_bytes(x.size, 32, T, 1)
        d_ref = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        d_new = torch.full((cap,), 0xAB, dtype=torch.uint8, device="cuda")
        abs_eb = bound if mode == szp.ABS else 0.0
        rel = bound if mode == szp.REL else 0.0
        size_ref = szp.compress_dev(dx.data_ptr(), x.size, d_ref.data_ptr(), cap, mode, abs_eb, rel, 32, T, 1, 0)
        size_new = szp.compress_dev_noalloc(dx.data_ptr(), x.size, d_new.data_ptr(), cap, mode, abs_eb, rel, 32, T, 0)
        assert size_new == size_ref
        assert torch.equal(d_new[:size_new], d_ref[:size_ref])
        # and directly against the oracle, not only the other device path
        eb = port.rel_bound(x, bound) if mode == szp.REL else bound
        assert d_new[:size_new].cpu().numpy().tobytes() == port.compress(x, eb, 32, T, 1)


def test_noalloc_allocates_no_device_memory(szp):
    import torch

    rng = np.random.default_rng(7)
    x, mode, bound = _calls(szp, rng)[0]
    dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    cap = szp.max_stream_bytes(x.size, 32, 5, 1)
    dout = torch.empty(cap, dtype=torch.uint8, device="cuda")
    szp.compress_dev_noalloc(dx.data_ptr(), x.size, dout.data_ptr(), cap, mode, 0.0, bound, 32, 5, 0)  # set-up call
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        szp.compress_dev_noalloc(dx.data_ptr(), x.size, dout.data_ptr(), cap, mode, 0.0, bound, 32, 5, 0)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_reports_quantization_notices(szp):
    import torch

    x = np.linspace(-1.0, 1.0, 100_000, dtype=np.float32)
    x[777] = np.nan
    dx = torch.from_numpy(x).cuda()
    cap = szp.max_stream_bytes(x.size, 32, 2, 1)
    d_ref = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    d_new = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    szp.compress_dev(dx.data_ptr(), x.size, d_ref.data_ptr(), cap, szp.ABS, 1e-3, 0.0, 32, 2, 1, 0)
    assert szp.last_notices() == 1
    clean = torch.linspace(-1.0, 1.0, 1000, device="cuda")
    szp.compress_dev_noalloc(clean.data_ptr(), 1000, d_new.data_ptr(), cap, szp.ABS, 1e-3, 0.0, 32, 2, 0)
    assert szp.last_notices() == 0
    size = szp.compress_dev_noalloc(dx.data_ptr(), x.size, d_new.data_ptr(), cap, szp.ABS, 1e-3, 0.0, 32, 2, 0)
    assert szp.last_notices() == 1
    assert torch.equal(d_new[:size], d_ref[:size])


def test_noalloc_rejects_misaligned_input_before_launch(szp):
    import torch

    buf = torch.zeros(4097, dtype=torch.float32, device="cuda")
    dout = torch.empty(1 << 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(szp.SzpError) as e:  # a host-side check: nothing is launched
        szp.compress_dev_noalloc(buf.data_ptr() + 1, 4096, dout.data_ptr(), dout.numel(), szp.ABS, 1e-3, 0.0, 32, 1, 0)
    assert e.value.status == szp.EINVAL
    assert "aligned" in str(e.value)


def test_noalloc_rejects_inputs_beyond_its_limit(szp):
    import torch

    n = (1 << 27) + 2  # 16385 tiles of 256 blocks at T = 1: one more than the array holds
    dx = torch.zeros(n, dtype=torch.float32, device="cuda")
    dout = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    with pytest.raises(szp.SzpError) as e:
        szp.compress_dev_noalloc(dx.data_ptr(), n, dout.data_ptr(), dout.numel(), szp.ABS, 1e-3, 0.0, 32, 1, 0)
    assert e.value.status == szp.EINVAL
    assert "too large" in str(e.value)
