"""Batched fastmode1 (szp_gb300_batch_*): many fields in one launch per stage.

Every field of a batch must come out byte-identical (streams) and
bit-identical (decoded values) to the single-field calls on that field alone,
for every tile size, with and without graph replay, across repeated runs (the
range pass and the look-back words are reused), including empty and one-element
fields.  Field sizes and bounds mimic the batched benchmark configuration
(log-normal sizes, REL drawn log-uniform in [1e-5, 1e-2], some ABS fields).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _make_fields(rng, szp, T):
    import torch
    from szp_gb300.workloads import walk, laplace_zero_patches

    sizes = [0, 1, 2, 17, 33, 100, 1000, 4097, 65536, 300_001, 1_000_003]
    sizes += [int(v) for v in np.clip(np.exp(rng.normal(np.log(2e5), 1.2, 9)), 1024, 4_000_000)]
    out = []
    for i, n in enumerate(sizes):
        if i % 3 == 2 and n >= 1024:
            side = int(np.sqrt(n))
            x = laplace_zero_patches(side, max(1, n // side), rng).ravel()
        else:
            x = walk(n, rng)
        x = np.ascontiguousarray(x, dtype=np.float32)
        mode = szp.ABS if i % 4 == 3 else szp.REL
        bound = float(10 ** rng.uniform(-5, -2))
        if mode == szp.ABS:
            bound *= float(np.ptp(x)) if x.size else 1.0
            bound = max(bound, 1e-6)
        out.append(dict(x=torch.from_numpy(x).cuda(), n=x.size, mode=mode, bound=bound,
                        cap=szp.max_stream_bytes(x.size, 32, T, 1)))
    return out


def _single(szp, port, f, T):
    """The single-field device calls on f, each checked against the oracle
    (so a batch that matches them matches the oracle too)."""
    import torch
    d_s = torch.zeros(f["cap"], dtype=torch.uint8, device="cuda")
    abs_eb = f["bound"] if f["mode"] == szp.ABS else 0.0
    rel = f["bound"] if f["mode"] == szp.REL else 0.0
    size = szp.compress_dev(f["x"].data_ptr(), f["n"], d_s.data_ptr(), f["cap"], f["mode"], abs_eb, rel, 32, T, 1, 0)
    y = torch.empty(max(f["n"], 1), dtype=torch.float32, device="cuda")
    szp.decompress_dev(d_s.data_ptr(), size, f["n"], y.data_ptr(), 32, T, 1, 0)
    stream, yv = d_s[:size].cpu().numpy().tobytes(), y[:f["n"]].cpu()
    x = f["x"][:f["n"]].cpu().numpy()
    eb = port.rel_bound(x, rel) if f["mode"] == szp.REL else float(np.float32(abs_eb))
    assert stream == port.compress(x, eb, 32, T, 1), f["n"]
    assert np.array_equal(yv.numpy().view(np.uint32), port.decompress(stream, f["n"], 32, T, 1).view(np.uint32))
    return stream, yv


@pytest.mark.parametrize("T,flags", [(16, "autotune"), (7, "rounds1"), (16, "rounds2"), (3, "nograph")])
def test_batch_matches_single_field_calls(szp, port, T, flags):
    import torch

    fl = {"autotune": szp.BATCH_AUTOTUNE, "rounds1": 1 << 8, "rounds2": 2 << 8,
          "nograph": szp.BATCH_NO_GRAPH | (4 << 8)}[flags]
    rng = np.random.default_rng(77 + T)
    fields = _make_fields(rng, szp, T)
    ref = [_single(szp, port, f, T) for f in fields]
    streams = [torch.full((f["cap"],), 0xCD, dtype=torch.uint8, device="cuda") for f in fields]
    outs = [torch.full((max(f["n"], 1),), float("nan"), dtype=torch.float32, device="cuda") for f in fields]
    cf = [dict(input=f["x"].data_ptr(), output=s.data_ptr(), output_bytes=f["cap"], nbEle=f["n"],
               errBoundMode=f["mode"], absErrBound=f["bound"] if f["mode"] == szp.ABS else 0.0,
               relBoundRatio=f["bound"] if f["mode"] == szp.REL else 0.0) for f, s in zip(fields, streams)]
    cb = szp.Batch(szp.BATCH_COMPRESS, cf, 32, T, fl)
    cb.run()
    sizes, status = cb.sync()
    base = cb.sizes_dev()
    df = [dict(input=s.data_ptr(), input_bytes=f["cap"], input_len_dev=base + 8 * i, output=o.data_ptr(),
               output_bytes=4 * max(f["n"], 1), nbEle=f["n"])
          for i, (f, s, o) in enumerate(zip(fields, streams, outs))]
    db = szp.Batch(szp.BATCH_DECOMPRESS, df, 32, T, fl)
    for rep in range(2):  # replays reuse the range state and the look-back words
        for s in streams:
            s.fill_(0xCD)
        for o in outs:
            o.fill_(float("nan"))
        cb.run()
        db.run()
        sizes, status = cb.sync()
        _, dstatus = db.sync()
        assert status == [0] * len(fields) and dstatus == [0] * len(fields)
        for i, (f, (rs, ry)) in enumerate(zip(fields, ref)):
            assert sizes[i] == len(rs), (i, f["n"])
            assert streams[i][:sizes[i]].cpu().numpy().tobytes() == rs, (i, f["n"])
            assert torch.equal(outs[i][:f["n"]].cpu().view(torch.int32), ry.view(torch.int32)), (i, f["n"])
    if flags == "rounds1":
        assert cb.tile_rounds() == 1 and db.tile_rounds() == 1
    cb.close()
    db.close()


def test_batch_reports_field_errors(szp):
    import torch

    T = 4
    x = torch.linspace(0, 1, 100_000, device="cuda")
    small = torch.zeros(64, dtype=torch.uint8, device="cuda")  # header fits, data does not
    good = torch.zeros(szp.max_stream_bytes(100_000, 32, T, 1), dtype=torch.uint8, device="cuda")
    cf = [dict(input=x.data_ptr(), output=good.data_ptr(), output_bytes=good.numel(), nbEle=100_000,
               errBoundMode=szp.ABS, absErrBound=1e-4),
          dict(input=x.data_ptr(), output=small.data_ptr(), output_bytes=small.numel(), nbEle=100_000,
               errBoundMode=szp.ABS, absErrBound=1e-4)]
    b = szp.Batch(szp.BATCH_COMPRESS, cf, 32, T)
    b.run()
    sizes, status = b.sync(check=False)
    assert status == [szp.OK, szp.ECAPACITY]
    b.close()
    with pytest.raises(szp.SzpError):
        szp.Batch(szp.BATCH_COMPRESS, cf, 64, T)  # the batched path is blockSize 32
