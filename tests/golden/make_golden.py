"""Writes tests/golden/golden.npz (float32), golden_double.npz (float64) and
golden_record.npz (the single-thread _record entry points' return values):
inputs, streams and decompressed outputs produced by the REFERENCE library
(built from its own sources by oracle/Makefile into oracle/_ref/).  Run here,
where the reference sources exist; the fixtures then travel with the
repository.

    python tests/golden/make_golden.py            # all three files
    python tests/golden/make_golden.py --double   # golden_double.npz and golden_record.npz
    python tests/golden/make_golden.py --record   # golden_record.npz only

Each case records x (float32 input), the reference stream, the reference
decompressed values, and meta (L, T, fastmode, eb mode and bound).  Cases are
kept small and compressible enough that the reference's own fixed-size
per-thread buffers (4n/T bytes, SZp/src/szp_float.cc:190) are not overrun.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Port, Reference, reference_compress_arg, reference_decompress_arg  # noqa: E402
from szp_gb300.workloads import walk, walk64, fourier3d, laplace_zero_patches, bitcount_sweep, specials, \
    specials64  # noqa: E402
import ctypes  # noqa: E402


def usable(req):
    """glibc malloc usable size of a request (x86-64 and aarch64)."""
    return max(24, ((req + 8 + 15) & ~15) - 8)


def seg_sizes(stream, T):
    off = np.frombuffer(stream[4:4 + 8 * T], dtype="<u8").astype(np.int64)
    ends = np.append(off[1:], len(stream) - 4 - 8 * T)
    return ends - off


def main():
    ref, port = Reference(), Port()
    rng = np.random.default_rng(20241203)
    cases = []

    def add(name, x, L, T, mode, eb_mode, bound):
        print("case", name, flush=True)
        x = np.ascontiguousarray(x, dtype=np.float32)
        # predict the reference's buffer use with the restatement before running it
        eb_pred = port.rel_bound(x, bound) if eb_mode == 1 else bound
        pred = port.compress(x, eb_pred, L, T, mode)
        per_thread = (4 * x.size + T - 1) // T  # malloc request; fortified memcpy checks it
        if x.size and seg_sizes(pred, T).max() > per_thread:
            print("skip %s: reference per-thread buffer would overflow" % name)
            return
        if eb_mode == 1 and len(pred) > 4 * x.size + 4:
            print("skip %s: reference output buffer would overflow" % name)
            return
        if eb_mode == 1:
            s = ref.compress(x, L=L, T=T, mode=mode, eb_mode=1, rel=bound)
        else:
            s = reference_compress_arg(ref, x, bound, L, T, mode)
        y = reference_decompress_arg(ref, s, x.size, L, T, mode)
        cases.append(dict(name=name, x=x, s=np.frombuffer(s, np.uint8).copy(), y=y,
                          meta=dict(L=L, T=T, mode=mode, eb_mode=eb_mode, bound=bound, n=int(x.size))))

    w = walk(5003, rng)
    eb = float(np.float32(1e-4 * (w.max() - w.min())))
    for T in (1, 4, 7):
        for mode in (1, 2):
            add("walk_T%d_m%d" % (T, mode), w, 32, T, mode, 0, eb)
    for L in (1, 2, 7, 8, 16, 33, 64, 128):
        for mode in (1, 2):
            add("walk_L%d_m%d" % (L, mode), w[:3001], L, 3, mode, 0, eb)
    f = fourier3d(16, rng).ravel()
    for rel in (1e-2, 1e-3, 1e-4):
        add("fourier_rel%g" % rel, f, 32, 4, 1, 1, rel)
    add("fourier_rel_m2", f, 32, 2, 2, 1, 1e-3)
    z = laplace_zero_patches(64, 64, rng).ravel()
    add("zeros_T1", z, 32, 1, 1, 0, 1e-5)
    add("zeros_T5", z, 32, 5, 1, 0, 1e-5)
    add("zeros_m2", z, 32, 3, 2, 0, 1e-5)
    b = bitcount_sweep(rng)
    add("bitcounts_T1", b, 32, 1, 1, 0, 1.0)
    add("bitcounts_T3", b, 32, 3, 1, 0, 1.0)
    add("bitcounts_m2", b, 32, 2, 2, 0, 1.0)
    sp = specials(rng)
    add("specials_T1", sp, 32, 1, 1, 0, 1e-3)
    add("specials_T2_m2", sp, 32, 2, 2, 0, 1e-3)
    for n in (1, 2, 3, 31, 32, 33, 34, 64, 65):
        for T in (1, 2, 5):
            add("tiny_n%d_T%d" % (n, T), w[:n], 32, T, 1, 0, eb)
            add("tiny_n%d_T%d_m2" % (n, T), w[:n], 32, T, 2, 0, eb)

    out = {}
    meta = []
    for i, c in enumerate(cases):
        out["x%d" % i] = c["x"]
        out["s%d" % i] = c["s"]
        out["y%d" % i] = c["y"]
        meta.append(dict(c["meta"], name=c["name"]))
        # the restatement must already agree; a mismatch here is a bug to fix first
        m = c["meta"]
        eb_hdr = float(np.frombuffer(c["s"][:4].tobytes()[::-1], np.float32)[0])
        ps = port.compress(c["x"], eb_hdr, m["L"], m["T"], m["mode"])
        if ps != c["s"].tobytes():
            print("WARNING: restatement differs on", c["name"])
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print("wrote %d cases to %s (%d bytes)" % (len(cases), path, os.path.getsize(path)))


def _ref_double(ref):
    lib = ref.lib
    for name in ("szp_double_openmp_threadblock_arg", "szp_double_openmp_threadblock_randomaccess_arg"):
        f = getattr(lib, name)
        f.restype = None
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_double,
                      ctypes.c_size_t, ctypes.c_int]
    for name in ("szp_double_decompress_openmp_threadblock_arg",
                 "szp_double_decompress_openmp_threadblock_randomaccess_arg"):
        f = getattr(lib, name)
        f.restype = None
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    return lib


def main_double():
    """float64 cases: szp_double_* of the reference (SZp/src/szp_double.cc,
    szpd_double.cc); REL cases through szp_compress(SZ_DOUBLE)."""
    ref, port = Reference(), Port()
    lib = _ref_double(ref)
    rng = np.random.default_rng(20261203)
    cases = []

    def seg_sizes_d(stream, T):
        off = np.frombuffer(stream[8:8 + 8 * T], dtype="<u8").astype(np.int64)
        ends = np.append(off[1:], len(stream) - 8 - 8 * T)
        return ends - off

    def add(name, x, L, T, mode, eb_mode, bound):
        print("case", name, flush=True)
        x = np.ascontiguousarray(x, dtype=np.float64)
        eb_pred = port.rel_bound_d(x, bound) if eb_mode == 1 else bound
        pred = port.compress_d(x, eb_pred, L, T, mode)
        per_thread = (8 * x.size + T - 1) // T  # the reference's per-thread buffer
        if x.size and seg_sizes_d(pred, T).max() > per_thread:
            print("skip %s: reference per-thread buffer would overflow" % name)
            return
        if x.size < 2 * T:
            print("skip %s: n < 2T overruns the reference's buffers" % name)
            return
        ref.set_threads(T)
        if eb_mode == 1:
            s = ref.compress(x, L=L, T=T, mode=mode, eb_mode=1, rel=bound)
        else:
            cap = 64 + 8 * T + 16 * x.size + 200 * (x.size // max(L, 1) + T + 2)
            out = np.zeros(cap, dtype=np.uint8)
            size = ctypes.c_size_t(0)
            fn = lib.szp_double_openmp_threadblock_arg if mode == 1 else \
                lib.szp_double_openmp_threadblock_randomaccess_arg
            fn(out.ctypes.data, x.ctypes.data, ctypes.byref(size), bound, x.size, L)
            s = out[: size.value].tobytes()
        eb = float(np.frombuffer(s[:8][::-1], dtype=np.float64)[0])
        y = np.zeros(max(x.size, 1), dtype=np.float64)
        buf = np.frombuffer(s, dtype=np.uint8).copy()
        fn = lib.szp_double_decompress_openmp_threadblock_arg if mode == 1 else \
            lib.szp_double_decompress_openmp_threadblock_randomaccess_arg
        fn(y.ctypes.data, x.size, eb, L, buf.ctypes.data + 8)
        cases.append(dict(name=name, x=x, s=np.frombuffer(s, np.uint8).copy(), y=y[: x.size],
                          meta=dict(L=L, T=T, mode=mode, eb_mode=eb_mode, bound=bound, n=int(x.size))))

    w = walk64(5003, rng)
    eb = 1e-6 * float(w.max() - w.min())
    for T in (1, 4, 7):
        for mode in (1, 2):
            add("walk_T%d_m%d" % (T, mode), w, 32, T, mode, 0, eb)
    for L in (1, 2, 7, 8, 16, 33, 64, 128):
        for mode in (1, 2):
            add("walk_L%d_m%d" % (L, mode), w[:3001], L, 3, mode, 0, eb)
    f = fourier3d(16, rng).astype(np.float64).ravel() + rng.normal(0.0, 1e-9, 16 ** 3)
    for rel in (1e-3, 1e-5, 1e-7):
        add("fourier_rel%g" % rel, f, 32, 4, 1, 1, rel)
    add("fourier_rel_m2", f, 32, 2, 2, 1, 1e-6)
    z = laplace_zero_patches(64, 64, rng).astype(np.float64).ravel()
    add("zeros_T5", z, 32, 5, 1, 0, 1e-5)
    add("zeros_m2", z, 32, 3, 2, 0, 1e-5)
    b = bitcount_sweep(rng, dtype=np.float64)
    add("bitcounts_T1", b, 32, 1, 1, 0, 1.0)
    add("bitcounts_T3", b, 32, 3, 1, 0, 1.0)
    add("bitcounts_m2", b, 32, 2, 2, 0, 1.0)
    sp = specials64(rng)
    add("specials_T1", sp, 32, 1, 1, 0, 1e-3)
    add("specials_T2_m2", sp, 32, 2, 2, 0, 1e-3)
    for n in (2, 3, 31, 32, 33, 34, 64, 65):
        for T in (1, 2):
            add("tiny_n%d_T%d" % (n, T), w[:n], 32, T, 1, 0, eb)
            add("tiny_n%d_T%d_m2" % (n, T), w[:n], 32, T, 2, 0, eb)

    out = {}
    meta = []
    for i, c in enumerate(cases):
        out["x%d" % i] = c["x"]
        out["s%d" % i] = c["s"]
        out["y%d" % i] = c["y"]
        meta.append(dict(c["meta"], name=c["name"]))
        m = c["meta"]
        eb_hdr = float(np.frombuffer(c["s"][:8].tobytes()[::-1], np.float64)[0])
        if port.compress_d(c["x"], eb_hdr, m["L"], m["T"], m["mode"]) != c["s"].tobytes():
            print("WARNING: restatement differs on", c["name"])
        yp = port.decompress_d(c["s"].tobytes(), m["n"], m["L"], m["T"], m["mode"])
        if not np.array_equal(yp.view(np.uint64), c["y"].view(np.uint64)):
            print("WARNING: restatement decodes differently on", c["name"])
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_double.npz")
    np.savez_compressed(path, **out)
    print("wrote %d cases to %s (%d bytes)" % (len(cases), path, os.path.getsize(path)))


def main_record():
    """The single-thread _record entry points: the reference's stream, its
    `total_memaccess` return values (szp_float.cc:607-750, szpd_float.cc:216-318
    and the double twins) and decompressed values, float32 and float64."""
    from oracle.oracle import reference_record
    ref, port = Reference(), Port()
    rng = np.random.default_rng(20261204)
    out, meta = {}, []

    def add(name, x, L, bound):
        dbl = x.dtype == np.float64
        pred = port.compress_d(x, bound, L, 1, 1) if dbl else port.compress(x, bound, L, 1, 1)
        hb = 8 if dbl else 4
        if len(pred) - hb - 8 > x.itemsize * x.size:
            print("skip %s: reference per-thread buffer would overflow" % name)
            return
        s, rc, y, rd = reference_record(ref, x, bound, L)
        assert s == pred, name
        i = len(meta)
        out["x%d" % i], out["s%d" % i], out["y%d" % i] = x, np.frombuffer(s, np.uint8).copy(), y
        meta.append(dict(name=name, L=L, n=int(x.size), bound=bound, dbl=bool(dbl), rec_c=rc, rec_d=rd))
        print("case", name, rc, rd, flush=True)

    w = walk(100000, rng)
    eb = float(np.float32(1e-3 * (w.max() - w.min())))
    add("walk_L32", w, 32, eb)
    for L in (8, 7, 64):
        add("walk_L%d" % L, w[:12000], L, eb)
    for n in (1, 2, 3, 33, 34, 65):
        add("walk_n%d" % n, w[:n], 32, eb)
    f = fourier3d(16, rng).ravel()
    add("fourier", f, 32, float(np.float32(1e-4 * (f.max() - f.min()))))
    z = laplace_zero_patches(64, 64, rng).ravel()
    add("zeros", z, 32, 1e-5)
    add("bitcounts", bitcount_sweep(rng), 32, 1.0)
    w64 = walk64(12000, rng)
    ebd = 1e-6 * float(w64.max() - w64.min())
    for L in (32, 16, 9):
        add("walk64_L%d" % L, w64, L, ebd)
    for n in (1, 2, 33):
        add("walk64_n%d" % n, w64[:n], 32, ebd)
    add("zeros64", z.astype(np.float64), 32, 1e-5)
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_record.npz")
    np.savez_compressed(path, **out)
    print("wrote %d cases to %s (%d bytes)" % (len(meta), path, os.path.getsize(path)))


if __name__ == "__main__":
    if "--record" in sys.argv:
        main_record()
        sys.exit(0)
    if "--double" not in sys.argv:
        main()
    main_double()
    main_record()
