"""The request server (szp_gb300_server_*): continuous batching.

Each request's result must be the same alone (a server that runs one request
at a time) and in the mix (requests batched and overlapped on several lanes),
and equal to the oracle's: streams byte-identical, decoded values
bit-identical (decompress requests read streams the oracle wrote).  Under an HBM budget smaller than all results together, every
request still completes as the client releases earlier results, and the
server never holds more than the budget.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T = 8


def _pool(szp, port, rng):
    """Fields with their oracle stream and decoded values.  Decompress
    requests read the oracle's stream (uploaded to the device); compress
    results and decoded values are compared with the oracle's, and the
    single-field device calls are checked against it too."""
    import torch
    from szp_gb300.workloads import walk, laplace_zero_patches

    sizes = [0, 1, 5, 40, 1000, 33_000, 250_000, 1_200_000]
    sizes += [int(v) for v in np.clip(np.exp(rng.normal(np.log(1.5e5), 1.0, 8)), 1024, 2_000_000)]
    pool = []
    for i, n in enumerate(sizes):
        x = walk(n, rng) if i % 3 else laplace_zero_patches(max(1, int(np.sqrt(max(n, 1)))),
                                                            max(1, n // max(1, int(np.sqrt(max(n, 1))))), rng).ravel()[:n]
        x = np.ascontiguousarray(x, dtype=np.float32)
        n = x.size
        dx = torch.from_numpy(x).cuda() if n else torch.zeros(1, device="cuda")
        mode = szp.REL if i % 2 else szp.ABS
        bound = float(10 ** rng.uniform(-5, -2)) * (1.0 if mode == szp.REL else max(float(np.ptp(x)) if n else 1.0, 1e-3))
        cap = szp.max_stream_bytes(n, 32, T, 1)
        d_s = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        abs_eb, rel = (bound, 0.0) if mode == szp.ABS else (0.0, bound)
        size = szp.compress_dev(dx.data_ptr(), n, d_s.data_ptr(), cap, mode, abs_eb, rel, 32, T, 1, 0)
        y = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
        szp.decompress_dev(d_s.data_ptr(), size, n, y.data_ptr(), 32, T, 1, 0)
        eb = port.rel_bound(x, rel) if mode == szp.REL else float(np.float32(abs_eb))
        o_stream = port.compress(x, eb, 32, T, 1)
        o_y = port.decompress(o_stream, n, 32, T, 1)
        assert d_s[:size].cpu().numpy().tobytes() == o_stream
        assert np.array_equal(y[:n].cpu().numpy().view(np.uint32), o_y.view(np.uint32))
        d_o = torch.from_numpy(np.frombuffer(o_stream, dtype=np.uint8).copy()).cuda()
        pool.append(dict(x=dx, n=n, mode=mode, abs=abs_eb, rel=rel, stream=d_o, size=len(o_stream),
                         ref_stream=o_stream, ref_y=torch.from_numpy(o_y)))
    return pool


def _requests(szp, pool, rng, count):
    reqs = []
    for _ in range(count):
        p = pool[int(rng.integers(0, len(pool)))]
        if rng.random() < 0.6:
            reqs.append((p, dict(op=szp.BATCH_COMPRESS, input=p["x"].data_ptr(), nbEle=p["n"],
                                 errBoundMode=p["mode"], absErrBound=p["abs"], relBoundRatio=p["rel"])))
        else:
            reqs.append((p, dict(op=szp.BATCH_DECOMPRESS, input=p["stream"].data_ptr(), input_bytes=p["size"],
                                 nbEle=p["n"])))
    return reqs


def _check(szp, p, req, res):
    import torch
    assert res["status"] == 0
    if req["op"] == szp.BATCH_COMPRESS:
        assert res["output_bytes"] == p["size"]
        got = torch.empty(p["size"], dtype=torch.uint8, device="cuda")
        _copy(got.data_ptr(), res["output"], p["size"])
        assert got.cpu().numpy().tobytes() == p["ref_stream"]
    else:
        assert res["output_bytes"] == 4 * p["n"]
        got = torch.empty(max(p["n"], 1), dtype=torch.float32, device="cuda")
        _copy(got.data_ptr(), res["output"], 4 * p["n"])
        assert torch.equal(got[:p["n"]].cpu().view(torch.int32), p["ref_y"].view(torch.int32))


def _copy(dst, src, nbytes):
    """Device-to-device copy of nbytes from the server's memory."""
    import ctypes
    import glob
    import os
    import torch
    if nbytes == 0:
        return
    if not _CUDART:
        libs = ["libcudart.so", "libcudart.so.13", "libcudart.so.12"]
        libs += sorted(glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart*.so*")))
        libs += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
        for cand in libs:
            try:
                lib = ctypes.CDLL(cand)
            except OSError:
                continue
            lib.cudaMemcpy.restype = ctypes.c_int
            lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            _CUDART.append(lib)
            break
    torch.cuda.synchronize()
    assert _CUDART[0].cudaMemcpy(dst, src, nbytes, 3) == 0  # cudaMemcpyDeviceToDevice


_CUDART = []


def test_results_same_alone_and_in_the_mix(szp, port):
    rng = np.random.default_rng(5)
    pool = _pool(szp, port, rng)
    reqs = _requests(szp, pool, rng, 160)
    # alone: one request at a time
    alone = szp.Server(512 << 20, max_batch=1, lanes=1, segments=T)
    for p, r in reqs[:40]:
        rid = alone.submit([r])[0]
        res = alone.wait(rid)
        _check(szp, p, r, res)
        alone.release(rid)
    alone.close()
    # in the mix: everything at once, batched and overlapped on three lanes
    mix = szp.Server(1 << 30, max_batch=64, lanes=3, segments=T)
    ids = mix.submit([r for _, r in reqs])
    for (p, r), rid in zip(reqs, ids):
        res = mix.wait(rid)
        _check(szp, p, r, res)
        mix.release(rid)
    st = mix.stats()
    assert st["requests"] == len(reqs) and st["memory_used"] == 0
    mix.close()


def test_admission_under_a_tight_budget(szp, port):
    rng = np.random.default_rng(9)
    pool = _pool(szp, port, rng)
    reqs = _requests(szp, pool, rng, 120)
    budget = 24 << 20  # far below what all results need together
    srv = szp.Server(budget, max_batch=32, lanes=2, segments=T)
    big = [i for i, (p, _) in enumerate(reqs) if 4 * p["n"] + 4096 > budget]
    assert not big
    ids = srv.submit([r for _, r in reqs])
    pending = dict(zip(ids, reqs))
    import time
    t_end = time.time() + 120
    while pending and time.time() < t_end:
        for res in srv.completed():
            p, r = pending.pop(res["id"])
            _check(szp, p, r, res)
            srv.release(res["id"])
        time.sleep(0.001)
    assert not pending
    st = srv.stats()
    assert st["memory_peak"] <= budget
    with pytest.raises(szp.SzpError):
        srv.submit([dict(op=szp.BATCH_DECOMPRESS, input=pool[-1]["stream"].data_ptr(), input_bytes=10,
                         nbEle=budget)])  # 4 * nbEle exceeds the budget
    srv.close()
