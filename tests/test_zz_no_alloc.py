"""The allocation-free compressor, szp_gb300_compress_dev_noalloc.

It exists for callers that cannot allocate device memory while they compress
-- a process whose GPU memory all belongs to its own pool, or a serving loop
that must not take the device-wide synchronisation of cudaMalloc/cudaFree.
They pass device input and output buffers; the kernels' working memory is a
static device array inside the library.  Its stream must be byte-for-byte the
one the allocating entry point (szp_gb300_compress_dev) produces, on
consecutive calls that reuse the shared array.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_on_consecutive_calls(szp):
    import torch
    from szp_gb300.workloads import walk, laplace_zero_patches

    assert torch.cuda.is_available()
    rng = np.random.default_rng(2024)
    T = 7
    calls = [
        (walk(3_000_001, rng), szp.REL, 1e-4),
        (laplace_zero_patches(1500, 1500, rng).ravel(), szp.ABS, 1e-5),
    ]
    for x, mode, bound in calls:  # two calls in a row share the static array
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


def test_noalloc_rejects_inputs_beyond_its_limit(szp):
    import torch

    n = (1 << 27) + 2  # 16385 tiles of 256 blocks at T = 1: one more than the array holds
    dx = torch.zeros(n, dtype=torch.float32, device="cuda")
    dout = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    with pytest.raises(szp.SzpError) as e:
        szp.compress_dev_noalloc(dx.data_ptr(), n, dout.data_ptr(), dout.numel(), szp.ABS, 1e-3, 0.0, 32, 1, 0)
    assert e.value.status == szp.EINVAL
    assert "too large" in str(e.value)
