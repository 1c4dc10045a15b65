"""bench.py -- SZp fastmode1 float32 compress + decompress on GB300.

Workload (one step): the 512^3 Fourier field (16 random modes, |k| 1-32,
amplitude ~ |k|^-5/3, plus N(0,1e-3) noise; 512 MiB, larger than L2) is
compressed with REL error bound (cycling 1e-2, 1e-3, 1e-4 step by step; the
device computes the value range), block size 32, T segments (the OpenMP
thread count of the host, as the reference decides it), then decompressed.
Inputs are seeded synthetic data created in HBM before timing.

value   uncompressed bytes per step (4n) / device time of the step's
        compress + decompress, GB/s (CUDA events, max over ranks).
e2e     the same metric through the host C API (szp_compress /
        szp_decompress on pinned host buffers), copies included.
roofline  the kernel with the most device time: algorithmic bytes per
        launch / its average CUDA-event duration, against the measured HBM
        copy bandwidth.
cpu_baseline  the oracle (C restatement of the reference, OpenMP on all host
        cores, same T) on the full field: median of 10 round trips after 2
        warm-ups.
configs the other single-field configurations: the 2^24-value random walk
        (ABS 1e-4 of its range) and the 8192^2 Laplace field with 40% zero
        blocks (ABS 1e-5), GB/s and per-kernel roofline fractions.
lorenzo the multidimensional Lorenzo variant of the same field at REL 1e-3
        and 1e-4: its ratio beside fastmode1's, GB/s and per-pass times.

--impl reference times the reference's CPU algorithm (the oracle port; the
reference's sources are not present where the benchmark runs) on the same
full field at T = all host threads, plus the median at T = 1.
Multi-GPU: replicas only (each rank runs the same step on its own GPU).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "compress & decompress GB/s (uncompressed) vs HBM roofline; batched/served p50/p99"
RELS = (1e-2, 1e-3, 1e-4)
N_SIDE = 512
L = 32
CPU_SAMPLE = 1 << 25


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--side", type=int, default=N_SIDE)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-fm2", action="store_true")
    ap.add_argument("--no-lorenzo", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--no-reduce", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the 2^24 walk and 8192^2 Laplace legs")
    ap.add_argument("--serving-window", type=float, default=0.2, help="seconds of arrivals per rate")
    ap.add_argument("--batched-fields", type=int, default=1024)
    return ap.parse_args()


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """SM clock, clock-event reasons and power while the timed steps run.

    Read-only NVML queries (libnvidia-ml, part of the driver) every ~1 ms from
    a thread, so that even a few-millisecond timed region holds samples;
    nvidia-smi at 200 ms is the fallback.  Only samples taken between mark(True)
    and mark(False) are reported.
    """

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index):
        self.index = index
        self.samples = []  # (t, sm_mhz, reasons bitmask or None, watts)
        self.window = None
        self.max_mhz = None
        self.stop_flag = False
        self.proc = None
        self.nv = self.handle = None

    def _nvml(self):
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return False
        h = ctypes.c_void_p()
        rc = -1
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.index)
            bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
            rc = nv.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(h))
        except Exception:
            rc = -1
        if rc != 0:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            idx = self.index
            try:
                idx = int(vis.split(",")[self.index]) if vis else self.index
            except (ValueError, IndexError):
                pass
            rc = nv.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h))
        if rc != 0:
            return False
        mx = ctypes.c_uint()
        if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:  # NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
        self.reason_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(nv, "nvmlDeviceGetCurrentClocksThrottleReasons")
        self.nv, self.handle = nv, h
        return True

    def _poll_nvml(self):
        nv, h = self.nv, self.handle
        mhz, rs, mw = ctypes.c_uint(), ctypes.c_ulonglong(), ctypes.c_uint()
        while not self.stop_flag:
            t = time.perf_counter()
            if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0:
                r = rs.value if self.reason_fn(h, ctypes.byref(rs)) == 0 else None
                w = mw.value / 1000.0 if nv.nvmlDeviceGetPowerUsage(h, ctypes.byref(mw)) == 0 else None
                self.samples.append((t, float(mhz.value), r, w))
            time.sleep(0.0005)

    def _poll_smi(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                      "--format=csv,noheader,nounits", "-lms", "200"],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        bits = [0x8, 0x40, 0x20, 0x4]
        for line in self.proc.stdout:
            f = [v.strip() for v in line.split(",")]
            try:
                r = sum(b for b, v in zip(bits, f[3:7]) if v.lower() == "active")
                self.max_mhz = float(f[1])
                self.samples.append((time.perf_counter(), float(f[0]), r, float(f[2])))
            except (ValueError, IndexError):
                continue

    def start(self):
        try:
            ok = self._nvml()
        except Exception:
            ok = False
        self.source = "nvml" if ok else "nvidia-smi"
        self.t = threading.Thread(target=self._poll_nvml if ok else self._poll_smi, daemon=True)
        self.t.start()
        t0 = time.perf_counter()
        while not self.samples and time.perf_counter() - t0 < 3.0:  # the sampler is running
            time.sleep(0.001)

    def mark(self, begin):
        if begin:
            self.window = [time.perf_counter(), None]
        else:
            self.window[1] = time.perf_counter()

    def stop(self):
        self.stop_flag = True
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.t.join(timeout=2)
        t0, t1 = self.window if self.window else (0.0, 0.0)
        inw = [s for s in list(self.samples) if t0 <= s[0] <= t1]
        if not inw:
            return None
        reasons = set()
        for _, _, r, _ in inw:
            for b, nm in self.REASONS.items():
                if r is not None and r & b:
                    reasons.add(nm)
        watts = [w for _, _, _, w in inw if w is not None]
        return {"sm_mhz": statistics.median(s[1] for s in inw), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(reasons), "samples": len(inw), "source": self.source,
                "power_w": round(statistics.median(watts), 1) if watts else None}


def batched_workload(szp, torch, dev, T, nfields, reps=3, seed=11):
    """1024 fields, log-normal sizes 4 KB..64 MB (median 1 MB), each a random
    walk or a slice of a 3-D Fourier field, REL drawn log-uniform in
    [1e-5, 1e-2]: one compress + decompress call per field against one batched
    graph per direction, both on one stream, CUDA-event timed."""
    from szp_gb300.workloads import fourier3d_torch, walk_torch
    rng = np.random.default_rng(seed)
    nbytes = np.clip(np.exp(rng.normal(np.log(1 << 20), 1.4, nfields)), 4096, 64 << 20)
    ns = [int(b) // 4 for b in nbytes]
    rels = [float(10 ** rng.uniform(-5, -2)) for _ in range(nfields)]
    kinds = rng.integers(0, 2, nfields)
    base = fourier3d_torch(384, seed, dev)
    xs = []
    for i, n in enumerate(ns):
        if kinds[i] == 1 and n <= base.numel():
            off = int(rng.integers(0, base.numel() - n + 1))
            xs.append(base[off:off + n].clone())
        else:
            xs.append(walk_torch(n, seed * 100003 + i, dev))
    del base
    caps = [szp.max_stream_bytes(n, L, T, 1) for n in ns]
    streams = [torch.empty(c, dtype=torch.uint8, device=dev) for c in caps]
    outs = [torch.empty(max(n, 1), dtype=torch.float32, device=dev) for n in ns]
    d_sizes = torch.zeros(nfields, dtype=torch.int64, device=dev)
    total = 4.0 * sum(ns)
    st = torch.cuda.current_stream(dev).cuda_stream

    def per_field():
        for i in range(nfields):
            szp.compress_dev_async(xs[i].data_ptr(), ns[i], streams[i].data_ptr(), caps[i],
                                   d_sizes.data_ptr() + 8 * i, szp.REL, 0.0, rels[i], L, T, 1, st)
            szp.decompress_dev_async(streams[i].data_ptr(), caps[i], d_sizes.data_ptr() + 8 * i, ns[i],
                                     outs[i].data_ptr(), L, T, 1, st)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1)
            best = t if best is None else min(best, t)
        return best

    ms_single = timed(per_field)
    assert szp.sync_status(st) == 0, szp.last_error()
    ref = [outs[i][:ns[i]].clone() for i in range(0, nfields, 97)]
    cf = [dict(input=xs[i].data_ptr(), output=streams[i].data_ptr(), output_bytes=caps[i], nbEle=ns[i],
               errBoundMode=szp.REL, relBoundRatio=rels[i]) for i in range(nfields)]
    cb = szp.Batch(szp.BATCH_COMPRESS, cf, L, T, szp.BATCH_AUTOTUNE)
    cb.run(st)
    cb.sync()
    df = [dict(input=streams[i].data_ptr(), input_bytes=caps[i], input_len_dev=cb.sizes_dev() + 8 * i,
               output=outs[i].data_ptr(), output_bytes=4 * max(ns[i], 1), nbEle=ns[i]) for i in range(nfields)]
    db = szp.Batch(szp.BATCH_DECOMPRESS, df, L, T, szp.BATCH_AUTOTUNE)

    def batched():
        cb.run(st)
        db.run(st)

    ms_batch = timed(batched)
    cb.sync()
    db.sync()
    for k, i in enumerate(range(0, nfields, 97)):
        assert torch.equal(outs[i][:ns[i]], ref[k]), "batched result differs from the per-field calls"
    res = {"fields": nfields, "bytes": int(total), "median_field_bytes": int(np.median(nbytes)),
           "per_field_ms": round(ms_single, 3), "batched_ms": round(ms_batch, 3),
           "per_field_gbs": round(total / (ms_single / 1e3) / 1e9, 2),
           "batched_gbs": round(total / (ms_batch / 1e3) / 1e9, 2),
           "speedup": round(ms_single / ms_batch, 2),
           "tile_rounds": {"compress": cb.tile_rounds(), "decompress": db.tile_rounds()},
           "metric": "aggregate round-trip GB/s (compress + decompress, uncompressed bytes)",
           "launches": "per field: 5 kernels x %d fields; batched: 2 graphs (5 kernels)" % nfields}
    cb.close()
    db.close()
    return res


def serving_workload(szp, torch, dev, T, window, rates=(2000, 5000, 10000, 20000, 50000, 100000, 200000, 400000),
                     seed=13, budget=40 << 30, npool=192):
    """Poisson arrivals, 60% compress / 40% decompress, sizes log-normal
    (median 1 MB, 4 KB..64 MB), REL log-uniform in [1e-5, 1e-2], results kept
    on the device under a 40 GB admission budget.  The continuous-batching
    server (64 requests per group, 3 lanes) against the same server taking one
    request at a time; latency is completion minus scheduled arrival.  Rates
    above the server's capacity show where its GB/s falls below the offered
    load; above 100k req/s the window shrinks so that each rate offers at
    most 20k requests."""
    from szp_gb300.workloads import fourier3d_torch, walk_torch
    rng = np.random.default_rng(seed)
    ns = [int(b) // 4 for b in np.clip(np.exp(rng.normal(np.log(1 << 20), 1.4, npool)), 4096, 64 << 20)]
    base = fourier3d_torch(256, seed, dev)
    st = torch.cuda.current_stream(dev).cuda_stream  # the stream the fields are made on
    pool = []
    for i, n in enumerate(ns):
        if i % 2 and n <= base.numel():
            off = int(rng.integers(0, base.numel() - n + 1))
            x = base[off:off + n].clone()
        else:
            x = walk_torch(n, seed * 7919 + i, dev)
        cap = szp.max_stream_bytes(n, L, T, 1)
        d_s = torch.empty(cap, dtype=torch.uint8, device=dev)
        rel = float(10 ** rng.uniform(-5, -2))
        size = szp.compress_dev(x.data_ptr(), n, d_s.data_ptr(), cap, szp.REL, 0.0, rel, L, T, 1, st)
        pool.append((x, n, rel, d_s, size))
    del base
    torch.cuda.synchronize()

    def run(rate, max_batch, lanes):
        srv = szp.Server(budget, max_batch=max_batch, lanes=lanes, segments=T)
        # warm-up: a burst of both kinds before the timed arrivals (a server runs continuously)
        warm = []
        for x, n, rel, d_s, size in pool[:16]:
            warm.append(dict(op=szp.BATCH_COMPRESS, input=x.data_ptr(), nbEle=n, errBoundMode=szp.REL,
                             relBoundRatio=rel))
            warm.append(dict(op=szp.BATCH_DECOMPRESS, input=d_s.data_ptr(), input_bytes=size, nbEle=n))
        for rid in srv.submit(warm):
            assert srv.wait(rid)["status"] == 0
            srv.release(rid)
        srv.completed()
        base_bytes = srv.stats()["bytes"]
        r2 = np.random.default_rng(seed + rate)
        count = max(1, int(rate * min(window, 20000.0 / rate)))
        arr = np.cumsum(r2.exponential(1.0 / rate, count))
        reqs = []
        for k in range(count):
            x, n, rel, d_s, size = pool[int(r2.integers(0, npool))]
            if r2.random() < 0.6:
                reqs.append(dict(op=szp.BATCH_COMPRESS, input=x.data_ptr(), nbEle=n, errBoundMode=szp.REL,
                                 relBoundRatio=float(10 ** r2.uniform(-5, -2))))
            else:
                reqs.append(dict(op=szp.BATCH_DECOMPRESS, input=d_s.data_ptr(), input_bytes=size, nbEle=n))
        t0 = srv.clock() + 0.002
        nxt, lat, nbytes, done, last = 0, [], 0, 0, t0
        while done < count:
            now = srv.clock()
            k = nxt
            while k < count and t0 + arr[k] <= now:
                k += 1
            if k > nxt:
                batch = reqs[nxt:k]
                for j, r in enumerate(batch):
                    r["arrival"] = t0 + arr[nxt + j]
                srv.submit(batch)
                nxt = k
            for res in srv.completed():
                assert res["status"] == 0, res
                lat.append(res["done"] - res["arrival"])
                last = max(last, res["done"])
                srv.release(res["id"])
                done += 1
        st = srv.stats()
        nbytes = st["bytes"] - base_bytes
        srv.close()
        lat = np.array(lat) * 1e3
        span = last - t0
        return {"requests": count, "p50_ms": round(float(np.percentile(lat, 50)), 3),
                "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "gbs": round(nbytes / span / 1e9, 2), "offered_gbs": round(nbytes / (arr[-1] + 1e-9) / 1e9, 2),
                "peak_memory_gb": round(st["memory_peak"] / 1e9, 2)}

    out = {"window_s": window, "budget_gb": budget / 1e9, "pool_fields": npool, "rates": {}}
    for rate in rates:
        out["rates"][str(rate)] = {"batched": run(rate, 64, 3), "one_at_a_time": run(rate, 1, 1)}
    return out


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if args.impl == "gb300":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        pg = dist
    return rank, world, local, pg


def max_over_ranks(pg, value, device="cpu"):
    """The largest of every rank's value (the job's time is its slowest
    replica's); the value itself on one process."""
    if not pg:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def field(side, seed, device):
    from szp_gb300.workloads import fourier3d_torch
    return fourier3d_torch(side, seed, device=device)


def config_leg(szp, torch, dev, T, x, eb, peak, reps=6):
    """One of the other single-field configurations through the device API:
    x (host float32) uploaded once, then compress + decompress round trips at
    ABS bound eb, CUDA-event kernel times (first two round trips dropped).
    GB/s are uncompressed bytes (4n) per device time; each kernel's achieved
    bandwidth counts its algorithmic bytes (compress: 4n read + stream
    written; locate: stream read + 4 B per block written; decode: stream and
    block positions read + 4n written)."""
    n = x.size
    dx = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(dev)
    cap = szp.max_stream_bytes(n, L, T, 1)
    ds = torch.empty(cap, dtype=torch.uint8, device=dev)
    dy = torch.empty(n, dtype=torch.float32, device=dev)
    dsz = torch.zeros(1, dtype=torch.int64, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    size = szp.compress_dev(dx.data_ptr(), n, ds.data_ptr(), cap, szp.ABS, eb, 0.0, L, T, 1, st)
    szp.set_timing(True)
    for i in range(reps + 2):
        if i == 2:
            torch.cuda.synchronize()
            for slot in range(5):
                szp.kernel_time(slot)
        szp.compress_dev_async(dx.data_ptr(), n, ds.data_ptr(), cap, dsz.data_ptr(), szp.ABS, eb, 0.0, L, T, 1, st)
        szp.decompress_dev_async(ds.data_ptr(), cap, dsz.data_ptr(), n, dy.data_ptr(), L, T, 1, st)
    torch.cuda.synchronize()
    assert szp.sync_status(st) == 0, szp.last_error()
    kt = {name: szp.kernel_time(slot) for slot, name in
          enumerate(["rel_range", "compress", "dec_setup", "locate", "decode"])}
    szp.set_timing(False)
    avg = {k: v[0] / v[1] for k, v in kt.items() if v[1]}
    nb = 4.0 * n / L
    alg = {"compress": 4.0 * n + size, "locate": size + nb, "decode": size + nb + 4.0 * n}
    comp = avg["compress"]
    dec = avg.get("dec_setup", 0) + avg["locate"] + avg["decode"]
    err = float((dx - dy).abs().max())
    return {"n": n, "abs_eb": eb, "stream_bytes": int(size), "ratio": round(4.0 * n / size, 3),
            "compress_gbs": round(4.0 * n / (comp / 1e3) / 1e9, 2),
            "decompress_gbs": round(4.0 * n / (dec / 1e3) / 1e9, 2),
            "round_trip_gbs": round(4.0 * n / ((comp + dec) / 1e3) / 1e9, 2),
            "kernels_ms": {k: round(v, 4) for k, v in avg.items()},
            "roofline": {k: {"achieved_gbs": round(alg[k] / (avg[k] / 1e3) / 1e9, 1),
                             "frac": round(alg[k] / (avg[k] / 1e3) / 1e9 / peak, 3),
                             "alg_bytes": int(alg[k])} for k in alg},
            "max_abs_err_over_eb": round(err / float(np.float32(eb)), 4)}


def config_legs(szp, torch, dev, T, peak):
    """The 2^24-value random walk at ABS 1e-4 of its range and the 8192^2
    Laplace field with 40% zero blocks at ABS 1e-5, the seeded inputs of the
    full-size parity tests."""
    from szp_gb300.workloads import walk, laplace_zero_patches
    w = walk(1 << 24, np.random.default_rng(1))
    eb = float(np.float32(1e-4 * (float(w.max()) - float(w.min()))))
    out = {"walk2^24": dict(config_leg(szp, torch, dev, T, w, eb, peak), bound="ABS 1e-4 of the range")}
    del w
    z = laplace_zero_patches(8192, 8192, np.random.default_rng(3)).ravel()
    zb = z[1:1 + ((z.size - 1) // L) * L].reshape(-1, L)
    leg = config_leg(szp, torch, dev, T, z, 1e-5, peak)
    leg["bound"] = "ABS 1e-5"
    leg["zero_block_fraction"] = round(float((zb == 0).all(axis=1).mean()), 3)
    out["laplace8192^2"] = leg
    return out


def cpu_port_median(port, x, T, reps=10, warmup=2, rels=RELS):
    """Oracle round trips on x at T segments and threads (REL bounds in
    turn): 2 warm-ups, then the median of reps; seconds per round trip."""
    for i in range(warmup):
        cpu_port_roundtrip(port, x, rels[i % len(rels)], T)
    t = [cpu_port_roundtrip(port, x, rels[i % len(rels)], T) for i in range(reps)]
    return statistics.median(t)


def cpu_port_roundtrip(port, x, rel, T, reps=1):
    """Oracle port round trip; returns seconds per round trip."""
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        eb = port.rel_bound(x, rel)
        s = port.compress(x, eb, L, T, 1)
        port.decompress(s, x.size, L, T, 1)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best


def cpu_row_baselines(port, xs, T, reps=2):
    """The oracle on the host cores for the rows beyond fastmode1, on bounded
    samples: fastmode2 and the homomorphic sum on xs (floats), float64 on the
    first 2^24 values of xs as doubles.  GB/s of uncompressed input."""
    def best(fn):
        fn()
        t = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            t.append(time.perf_counter() - t0)
        return min(t)
    out = {}

    def fm2():
        eb = port.rel_bound(xs, 1e-3)
        s = port.compress(xs, eb, L, T, 2)
        port.decompress(s, xs.size, L, T, 2)
    out["fastmode2"] = {"gbs": round(4.0 * xs.size / best(fm2) / 1e9, 3),
                        "sample": "%d floats, REL 1e-3 round trip" % xs.size}
    xd = xs[: 1 << 24].astype(np.float64)

    def f64():
        eb = port.rel_bound_d(xd, 1e-6)
        s = port.compress_d(xd, eb, L, T, 1)
        port.decompress_d(s, xd.size, L, T, 1)
    out["float64"] = {"gbs": round(8.0 * xd.size / best(f64) / 1e9, 3),
                      "sample": "%d doubles, REL 1e-6 round trip" % xd.size}
    eb = 1e-3 * float(xs.max() - xs.min())
    sa = port.compress(xs, eb, L, T, 1)
    sb = port.compress(np.ascontiguousarray(xs[::-1]), eb, L, T, 1)
    out["reduce"] = {"gbs": round(8.0 * xs.size / best(lambda: port.reduce_sum(sa, sb, xs.size, L, T, 1, 4)) / 1e9, 3),
                     "sample": "two streams of %d floats" % xs.size}
    return out


def run_reference(args, rank, world, pg):
    """The reference's CPU algorithm (the oracle restatement; the reference's
    own sources are not where the benchmark runs) on the host cores, rank 0
    only: each step one round trip of the full field at T = all host threads,
    REL bounds in turn; then the median of 10 round trips at T = 1 (REL 1e-3)
    after 2 warm-ups."""
    if rank != 0:
        return
    import torch
    from oracle.oracle import Port
    port = Port()
    T = port.max_threads()
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    x = np.ascontiguousarray(field(args.side, 2, dev).cpu().numpy())
    for i in range(args.warmup):
        cpu_port_roundtrip(port, x, RELS[i % 3], T)
    times = []
    for i in range(args.steps):
        times.append(cpu_port_roundtrip(port, x, RELS[i % 3], T))
    total = sum(times)
    gbs = 4.0 * x.size * args.steps / total / 1e9
    t1 = cpu_port_median(port, x, 1, reps=10, warmup=2, rels=(1e-3,))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "median_ms_per_step": round(1e3 * statistics.median(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32->int32",
        "data": "synthetic (seeded %d^3 Fourier field)" % args.side,
        "config": {"workload": "fourier%d^3 REL {1e-2,1e-3,1e-4} blockSize 32 fastmode1 round trip" % args.side,
                   "n": int(x.size), "segments": T, "block_size": L, "l2": "inputs > L2"},
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": T, "kind": "port",
                         "sample": "the full %d^3 field, one compress+decompress per step" % args.side,
                         "t1": {"value": round(4.0 * x.size / t1 / 1e9, 3), "unit": "GB/s", "cores": 1,
                                "sample": "the full field at T = 1, REL 1e-3, median of 10 after 2 warm-ups"}},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
        return
    import torch
    import szp_gb300 as szp

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    T = szp.get_segments()
    side = args.side
    n = side ** 3
    x = field(side, 2 + rank, dev)
    cap = szp.max_stream_bytes(n, L, T, 1)
    d_stream = torch.empty(cap, dtype=torch.uint8, device=dev)
    d_y = torch.empty(n, dtype=torch.float32, device=dev)
    d_size = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    st = stream.cuda_stream

    sizes = {}

    def step(i):
        rel = RELS[i % 3]
        szp.compress_dev_async(x.data_ptr(), n, d_stream.data_ptr(), cap, d_size.data_ptr(), szp.REL, 0.0, rel,
                               L, T, 1, st)
        szp.decompress_dev_async(d_stream.data_ptr(), cap, d_size.data_ptr(), n, d_y.data_ptr(), L, T, 1, st)

    # sizes per bound (also validates once)
    for i, rel in enumerate(RELS):
        sz = szp.compress_dev(x.data_ptr(), n, d_stream.data_ptr(), cap, szp.REL, 0.0, rel, L, T, 1, st)
        sizes[rel] = sz
    szp.set_timing(True)
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    assert szp.sync_status(st) == 0, szp.last_error()
    for s in range(5):
        szp.kernel_time(s)  # drop warm-up timings

    clocks = ClockSampler(local)
    clocks.start()
    l0 = szp.kernel_launches()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.mark(True)
    e0.record(stream)
    for i in range(args.steps):
        step(i)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.mark(False)
    if pg:
        pg.barrier()
    launches = szp.kernel_launches() - l0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    status = szp.sync_status(st)
    assert status == 0, szp.last_error()
    ktimes = {name: szp.kernel_time(slot) for slot, name in
              enumerate(["rel_range", "compress", "dec_setup", "locate", "decode"])}
    szp.set_timing(False)
    ms = max_over_ranks(pg, ms, dev)

    mean_out = float(np.mean([sizes[RELS[i % 3]] for i in range(args.steps)]))
    gbs = world * 4.0 * n * args.steps / (ms / 1e3) / 1e9
    # per-kernel achieved bandwidth from algorithmic bytes
    alg = {"rel_range": 4.0 * n, "compress": 4.0 * n + mean_out, "dec_setup": 8.0 * T,
           "locate": mean_out + 4.0 * n / L, "decode": mean_out + 4.0 * n + 4.0 * n / L}
    peak, peak_kind = measured_peak_gbs()
    kern = {}
    for k, (tot, cnt) in ktimes.items():
        if cnt > 0 and tot > 0:
            avg = tot / cnt
            kern[k] = {"avg_ms": round(avg, 4), "launches": cnt, "gbs": round(alg[k] / (avg / 1e3) / 1e9, 1),
                       "share": None}
    tsum = sum(v["avg_ms"] * v["launches"] for v in kern.values())
    for v in kern.values():
        v["share"] = round(v["avg_ms"] * v["launches"] / tsum, 3) if tsum else None
    dom = max(kern, key=lambda k: kern[k]["avg_ms"] * kern[k]["launches"])
    ach = kern[dom]["gbs"]
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if os.path.exists(tfile):
        for ln in open(tfile):
            f = dict(kv.split("=", 1) for kv in ln.split() if "=" in kv)
            if f.get("bench_kernel") == dom and "bytes_per_element" in f:
                traffic = round(float(f["bytes_per_element"]) * n)
    roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 3),
            "traffic": traffic, "kernel": dom, "peak_source": peak_kind,
            "alg_bytes_per_launch": alg[dom]}

    # ---- e2e through the host C API, as a C caller uses it ----
    e2e = None
    if not args.no_e2e:
        lib = szp._lib
        libc = ctypes.CDLL(None)
        libc.free.argtypes = [ctypes.c_void_p]
        hx = torch.empty(n, dtype=torch.float32, pin_memory=True)
        hx.copy_(x)
        size = ctypes.c_size_t(0)

        def host_step(i):
            p = lib.szp_compress(1, 0, hx.data_ptr(), ctypes.byref(size), szp.REL, 0.0, RELS[i % 3], n, L)
            assert p, szp.last_error()
            sz = size.value
            q = lib.szp_decompress(1, 0, p, sz, n, L)
            assert q, szp.last_error()
            return p, q, sz

        for i in range(2):
            p, q, sz = host_step(i)
            if i == 0:  # the host path returns what the device path computed
                ref = torch.empty(n, dtype=torch.float32, device=dev)
                szp.compress_dev(x.data_ptr(), n, d_stream.data_ptr(), cap, szp.REL, 0.0, RELS[0], L, T, 1, st)
                szp.decompress_dev(d_stream.data_ptr(), sizes[RELS[0]], n, ref.data_ptr(), L, T, 1, st)
                got = torch.from_numpy(np.ctypeslib.as_array((ctypes.c_float * n).from_address(q)))
                assert torch.equal(got, ref.cpu()), "host API result differs from the device path"
                del got, ref
            libc.free(p)
            libc.free(q)
        h2d = d2h = 0
        t0 = time.perf_counter()
        for i in range(args.steps):
            p, q, sz = host_step(i)
            libc.free(p)
            libc.free(q)
            h2d += 4 * n + sz
            d2h += sz + 4 * n
        dt = time.perf_counter() - t0
        e2e = {"value": round(world * 4.0 * n * args.steps / dt / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps),
               "api": "szp_compress + szp_decompress (C ABI via ctypes; pinned input, library-malloc'd results)"}
        # the same with the input in ordinary malloc'd (pageable) memory, as
        # the reference's example drivers pass it
        hx_pinned = hx
        hx = torch.from_numpy(np.ascontiguousarray(hx_pinned.numpy()).copy())
        del hx_pinned
        p, q, sz = host_step(0)
        libc.free(p)
        libc.free(q)
        t0 = time.perf_counter()
        for i in range(args.steps):
            p, q, sz = host_step(i)
            libc.free(p)
            libc.free(q)
        dt = time.perf_counter() - t0
        e2e["pageable"] = {"value": round(world * 4.0 * n * args.steps / dt / 1e9, 3), "unit": "GB/s",
                           "api": "the same calls on a malloc'd (pageable) input array"}
        del hx

    # fastmode2 (SZP_RANDOMACCESS: a seed per block) on the same field, REL 1e-3
    fm2 = None
    if not args.no_fm2:
        cap2 = szp.max_stream_bytes(n, L, T, 2)
        d_s2 = torch.empty(cap2, dtype=torch.uint8, device=dev)
        szp.set_timing(True)
        for i in range(4):
            szp.compress_dev_async(x.data_ptr(), n, d_s2.data_ptr(), cap2, d_size.data_ptr(), szp.REL, 0.0, 1e-3,
                                   L, T, 2, st)
            szp.decompress_dev_async(d_s2.data_ptr(), cap2, d_size.data_ptr(), n, d_y.data_ptr(), L, T, 2, st)
            if i == 0:
                torch.cuda.synchronize()
                for slot in range(5):
                    szp.kernel_time(slot)  # drop the first round trip
        torch.cuda.synchronize()
        assert szp.sync_status(st) == 0, szp.last_error()
        kt = {name: szp.kernel_time(slot) for slot, name in
              enumerate(["rel_range", "compress", "dec_setup", "locate", "decode"])}
        szp.set_timing(False)
        avg = {k: v[0] / v[1] for k, v in kt.items() if v[1]}
        size2 = int(d_size.item())
        # both fastmodes quantize and dequantize alike: fastmode1 at the same bound
        # must give the same floats bit for bit
        y1 = torch.empty_like(d_y)
        szp.compress_dev_async(x.data_ptr(), n, d_stream.data_ptr(), cap, d_size.data_ptr(), szp.REL, 0.0, 1e-3,
                               L, T, 1, st)
        szp.decompress_dev_async(d_stream.data_ptr(), cap, d_size.data_ptr(), n, y1.data_ptr(), L, T, 1, st)
        torch.cuda.synchronize()
        assert szp.sync_status(st) == 0, szp.last_error()
        assert torch.equal(y1.view(torch.int32), d_y.view(torch.int32)), "fastmode2 and fastmode1 results differ"
        del y1
        fm2 = {"rel": 1e-3, "ratio": round(4.0 * n / size2, 3),
               "compress_gbs": round(4.0 * n / ((avg["rel_range"] + avg["compress"]) / 1e3) / 1e9, 2),
               "decompress_gbs": round(4.0 * n / ((avg["dec_setup"] + avg["locate"] + avg["decode"]) / 1e3) / 1e9, 2),
               "kernels_ms": {k: round(v, 4) for k, v in avg.items()}}
        del d_s2

    # the multidimensional Lorenzo variant on the same field (its own stream):
    # ratio against fastmode1's at the same bound, and the device time of its
    # passes (the codes pass + fastmode1 over the codes; decode of the codes +
    # the inverse sums)
    lorenzo = None
    if not args.no_lorenzo:
        dims = (args.side, args.side, args.side)
        capl = szp.lorenzo_max_stream_bytes(dims, T)
        d_sl = torch.empty(capl, dtype=torch.uint8, device=dev)
        lorenzo = {"dims": list(dims), "by_rel": {}}
        for rel in (1e-3, 1e-4):
            szp.set_timing(True)
            for i in range(4):
                szl = szp.lorenzo_compress_dev(x.data_ptr(), dims, d_sl.data_ptr(), capl, szp.REL, 0.0, rel, T, st)
                szp.lorenzo_decompress_dev(d_sl.data_ptr(), szl, dims, d_y.data_ptr(), T, st)
                if i == 0:
                    torch.cuda.synchronize()
                    for slot in range(7):
                        szp.kernel_time(slot)  # drop the first round trip
            torch.cuda.synchronize()
            kt = {name: szp.kernel_time(slot) for slot, name in
                  enumerate(["rel_range", "compress", "dec_setup", "locate", "decode", "codes", "inverse"])}
            szp.set_timing(False)
            avg = {k: v[0] / v[1] for k, v in kt.items() if v[1]}
            ebl = rel * float(x.max() - x.min())
            errl = float((x - d_y).abs().max())
            # fastmode1's arithmetic: a float inverse of eb and a float product q * eb
            assert errl <= ebl * (1 + 2.0 ** -22) + float(x.abs().max()) * 2.0 ** -22, \
                "Lorenzo round trip exceeds the bound"
            c_ms = avg["rel_range"] + avg["codes"] + avg["compress"]
            d_ms = avg["dec_setup"] + avg["locate"] + avg["decode"] + avg["inverse"]
            lorenzo["by_rel"][str(rel)] = {
                "ratio": round(4.0 * n / szl, 3), "fastmode1_ratio": round(4.0 * n / sizes[rel], 3),
                "compress_gbs": round(4.0 * n / (c_ms / 1e3) / 1e9, 2),
                "decompress_gbs": round(4.0 * n / (d_ms / 1e3) / 1e9, 2),
                "kernels_ms": {k: round(v, 4) for k, v in avg.items()},
                "max_abs_err_over_eb": round(errl / ebl, 4)}
        del d_sl

    # float64 data (szp_double_*): 2^26 doubles (512 MiB) of the field, REL 1e-6
    f64 = None
    if not args.no_f64:
        nd = min(n, 1 << 26)
        xd = x[:nd].double()
        capd = szp.max_stream_bytes_f64(nd, L, T, 1)
        d_sd = torch.empty(capd, dtype=torch.uint8, device=dev)
        yd = torch.empty_like(xd)
        szp.set_timing(True)
        for i in range(4):
            szd = szp.compress_dev_f64(xd.data_ptr(), nd, d_sd.data_ptr(), capd, szp.REL, 0.0, 1e-6, L, T, 1, st)
            szp.decompress_dev_f64(d_sd.data_ptr(), szd, nd, yd.data_ptr(), L, T, 1, st)
            if i == 0:
                torch.cuda.synchronize()
                for slot in range(5):
                    szp.kernel_time(slot)  # drop the first round trip
        torch.cuda.synchronize()
        kt = {name: szp.kernel_time(slot) for slot, name in
              enumerate(["rel_range", "compress", "dec_setup", "locate", "decode"])}
        szp.set_timing(False)
        avg = {k: v[0] / v[1] for k, v in kt.items() if v[1]}
        ebd = 1e-6 * float(xd.max() - xd.min())
        errd = float((xd - yd).abs().max())
        assert errd <= ebd * (1 + 1e-9), "float64 round trip exceeds the bound"
        f64 = {"n": nd, "rel": 1e-6, "ratio": round(8.0 * nd / szd, 3),
               "compress_gbs": round(8.0 * nd / ((avg["rel_range"] + avg["compress"]) / 1e3) / 1e9, 2),
               "decompress_gbs": round(8.0 * nd / ((avg["dec_setup"] + avg["locate"] + avg["decode"]) / 1e3) / 1e9,
                                       2),
               "kernels_ms": {k: round(v, 4) for k, v in avg.items()}}
        del xd, yd, d_sd

    # homomorphic sum of two streams: the field and its values reversed
    # at one ABS bound: device time of both decodes, the add and the encode
    reduce = None
    if not args.no_reduce:
        ebr = 1e-3 * float(x.max() - x.min())
        x2 = torch.flip(x, [0])
        capr = szp.max_stream_bytes(n, L, T, 1)
        bufs = [torch.empty(capr, dtype=torch.uint8, device=dev) for _ in range(3)]
        szr = [szp.compress_dev(v.data_ptr(), n, b.data_ptr(), capr, szp.ABS, ebr, 0.0, L, T, 1, st)
               for v, b in zip((x, x2), bufs)]
        del x2
        szp.set_timing(True)
        wall = []
        for i in range(4):
            if i == 1:
                torch.cuda.synchronize()
                for slot in range(5):
                    szp.kernel_time(slot)  # drop the first
            t0 = time.perf_counter()
            szo = szp.reduce_sum_dev(bufs[0].data_ptr(), szr[0], bufs[1].data_ptr(), szr[1], n, bufs[2].data_ptr(),
                                     capr, L, T, 1, szp.SZ_FLOAT, st)
            if i:
                wall.append(time.perf_counter() - t0)
        kt = {name: szp.kernel_time(slot) for slot, name in
              enumerate(["rel_range", "compress", "dec_setup", "locate", "decode"])}
        szp.set_timing(False)
        dev_ms = sum(v[0] for v in kt.values()) / 3
        reduce = {"bound": "ABS 1e-3 of the range", "inputs": "the field and its values in reverse order",
                  "stream_bytes": [int(szr[0]), int(szr[1]), int(szo)],
                  "kernels_ms_per_sum": {k: round(v[0] / 3, 4) for k, v in kt.items() if v[1]},
                  "device_ms": round(dev_ms, 4), "wall_ms": round(1e3 * min(wall), 4),
                  "fields_gbs": round(2 * 4.0 * n / (dev_ms / 1e3) / 1e9, 2),
                  "metric": "uncompressed bytes of both fields per device time of the sum"}
        del bufs

    configs = None
    if not args.no_configs:
        configs = config_legs(szp, torch, dev, T, peak)

    batched = None
    if not args.no_batched:
        batched = batched_workload(szp, torch, dev, T, args.batched_fields)

    serving = None
    if not args.no_serving:
        serving = serving_workload(szp, torch, dev, T, args.serving_window)

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle.oracle import Port
        port = Port()
        Tc = port.max_threads()
        xf = np.ascontiguousarray(x.cpu().numpy())
        sec = cpu_port_median(port, xf, Tc)
        cpu = {"value": round(4.0 * xf.size / sec / 1e9, 3), "unit": "GB/s", "cores": Tc, "kind": "port",
               "sample": "the full field, REL 1e-2/1e-3/1e-4 round trips in turn, median of 10 after 2 warm-ups"}
        del xf
        xs = np.ascontiguousarray(x[:CPU_SAMPLE].cpu().numpy())
        # the oracle beside each further row's GPU number
        rows = cpu_row_baselines(port, xs, Tc)
        for key, leg in (("fastmode2", fm2), ("float64", f64), ("reduce", reduce)):
            if leg is not None:
                leg["cpu_port"] = rows[key]

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32->int32",
            "data": "synthetic (seeded %d^3 Fourier field generated in HBM)" % args.side,
            "config": {"workload": "fourier%d^3 REL {1e-2,1e-3,1e-4} blockSize 32 fastmode1 round trip" % args.side,
                       "n": n, "segments": T, "block_size": L, "parallelism": "replicas",
                       "l2": "inputs %s than L2 (%d MiB)" % ("larger" if 4 * n > 129e6 else "smaller",
                                                            4 * n >> 20),
                       "ratio": {str(r): round(4.0 * n / sizes[r], 3) for r in RELS}},
            "compress_gbs": round(world * 4.0 * n / (kern["compress"]["avg_ms"] / 1e3 +
                                                    kern.get("rel_range", {"avg_ms": 0})["avg_ms"] / 1e3) / 1e9, 2),
            "decompress_gbs": round(world * 4.0 * n / sum(kern[k]["avg_ms"] / 1e3 for k in
                                                          ("dec_setup", "locate", "decode") if k in kern) / 1e9, 2),
            "kernels": kern,
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "fastmode2": fm2,
            "lorenzo": lorenzo,
            "float64": f64,
            "reduce": reduce,
            "configs": configs,
            "batched": batched,
            "serving": serving,
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
