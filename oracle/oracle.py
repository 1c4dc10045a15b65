"""Python handle on the oracle -- TEST INFRASTRUCTURE ONLY.

Two CPU implementations of SZp's fastmode1/fastmode2 codec (float32 and
float64 data) live here:

* ``Port``: the C restatement in ``oracle/szp_oracle.c`` (explicit segment
  count T, caller buffers).  The tests compare the CUDA library against it,
  and bench.py times it as the "port" CPU baseline.
* ``Reference``: the reference library compiled from its own sources into
  ``oracle/_ref/libszp_ref.so`` (only where the sources exist).  Its segment
  count is the OpenMP thread count, set here with ``omp_set_num_threads``.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this
module.  The product package ``szp_gb300`` never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libszp_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libszp_ref.so")

_c_size_p = ctypes.POINTER(ctypes.c_size_t)


def build(ref=True):
    """Compile the restatement (and the reference when its sources exist)."""
    targets = ["_build/libszp_oracle.so"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


class Port:
    """ctypes binding of oracle/szp_oracle.c."""

    def __init__(self, path=PORT_SO):
        if not os.path.exists(path):
            build(ref=False)
        lib = ctypes.CDLL(path)
        lib.szo_compress.restype = ctypes.c_int
        lib.szo_compress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, _c_size_p]
        lib.szo_decompress.restype = ctypes.c_int
        lib.szo_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.szo_rel_bound.restype = ctypes.c_float
        lib.szo_rel_bound.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double]
        lib.szo_bitcount.restype = ctypes.c_int
        lib.szo_bitcount.argtypes = [ctypes.c_uint32]
        lib.szo_bitcount_thresholds.restype = None
        lib.szo_bitcount_thresholds.argtypes = [ctypes.c_void_p]
        lib.szo_bitcount_verify.restype = ctypes.c_uint64
        lib.szo_bitcount_verify.argtypes = [ctypes.c_void_p]
        lib.szo_max_stream_bytes.restype = ctypes.c_size_t
        lib.szo_max_stream_bytes.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.szo_max_threads.restype = ctypes.c_int
        lib.szo_compress_d.restype = ctypes.c_int
        lib.szo_compress_d.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, _c_size_p]
        lib.szo_decompress_d.restype = ctypes.c_int
        lib.szo_decompress_d.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.szo_rel_bound_d.restype = ctypes.c_double
        lib.szo_rel_bound_d.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double]
        lib.szo_max_stream_bytes_d.restype = ctypes.c_size_t
        lib.szo_max_stream_bytes_d.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.szo_reduce_sum.restype = ctypes.c_int
        lib.szo_reduce_sum.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_size_t, _c_size_p]
        lib.szo_lorenzo_max_stream_bytes.restype = ctypes.c_size_t
        lib.szo_lorenzo_max_stream_bytes.argtypes = [ctypes.c_size_t] * 3 + [ctypes.c_int]
        lib.szo_lorenzo_compress.restype = ctypes.c_int
        lib.szo_lorenzo_compress.argtypes = [ctypes.c_void_p] + [ctypes.c_size_t] * 3 + [
            ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, _c_size_p]
        lib.szo_lorenzo_decompress.restype = ctypes.c_int
        lib.szo_lorenzo_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t] + [ctypes.c_size_t] * 3 + [
            ctypes.c_int, ctypes.c_void_p]
        for name in ("szo_record_compress", "szo_record_decompress"):
            f = getattr(lib, name)
            f.restype = ctypes.c_uint64
            f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
        self.lib = lib

    def record_compress(self, stream, n, L=32, dbl=False):
        """The reference's single-thread compressor _record tally for the
        T = 1 stream it writes (szp_float.cc:607-750, szp_double.cc:613-756)."""
        buf = np.frombuffer(stream, dtype=np.uint8)
        return int(self.lib.szo_record_compress(buf.ctypes.data, buf.size, n, L, int(dbl)))

    def record_decompress(self, stream, n, L=32, dbl=False):
        """The reference's single-thread decompressor _record tally
        (szpd_float.cc:216-318, szpd_double.cc:219-321)."""
        buf = np.frombuffer(stream, dtype=np.uint8)
        return int(self.lib.szo_record_decompress(buf.ctypes.data, buf.size, n, L, int(dbl)))

    def lorenzo_compress(self, x, dims, eb, T=1):
        """The multidimensional Lorenzo variant's stream of x (shape dims =
        (nz, ny, nx), x fastest) at absolute bound eb, T segments."""
        x = _f32(x)
        nz, ny, nx = dims
        assert x.size == nx * ny * nz
        cap = self.lib.szo_lorenzo_max_stream_bytes(nx, ny, nz, T)
        out = np.empty(cap, dtype=np.uint8)
        size = ctypes.c_size_t(0)
        rc = self.lib.szo_lorenzo_compress(x.ctypes.data, nx, ny, nz, ctypes.c_float(eb), T, out.ctypes.data, cap,
                                           ctypes.byref(size))
        if rc != 0:
            raise RuntimeError("oracle lorenzo_compress failed: %d" % rc)
        return out[: size.value].tobytes()

    def lorenzo_decompress(self, stream, dims, T=1):
        nz, ny, nx = dims
        buf = np.frombuffer(stream, dtype=np.uint8)
        y = np.empty(nx * ny * nz, dtype=np.float32)
        rc = self.lib.szo_lorenzo_decompress(buf.ctypes.data, buf.size, nx, ny, nz, T, y.ctypes.data)
        if rc != 0:
            raise RuntimeError("oracle lorenzo_decompress failed: %d" % rc)
        return y

    def max_threads(self):
        return self.lib.szo_max_threads()

    def compress(self, x, eb, L=32, T=1, mode=1):
        """Stream bytes for x at absolute bound eb (float32), T segments."""
        x = _f32(x)
        cap = self.lib.szo_max_stream_bytes(x.size, L, T, mode)
        out = np.empty(cap, dtype=np.uint8)
        size = ctypes.c_size_t(0)
        rc = self.lib.szo_compress(x.ctypes.data, x.size, ctypes.c_float(eb), L, T, mode,
                                   out.ctypes.data, cap, ctypes.byref(size))
        if rc != 0:
            raise RuntimeError("oracle compress failed: %d" % rc)
        return out[: size.value].tobytes()

    def decompress(self, stream, n, L=32, T=1, mode=1):
        buf = np.frombuffer(stream, dtype=np.uint8)
        y = np.empty(n, dtype=np.float32)
        rc = self.lib.szo_decompress(buf.ctypes.data, buf.size, n, L, T, mode, y.ctypes.data)
        if rc != 0:
            raise RuntimeError("oracle decompress failed: %d" % rc)
        return y

    def compress_d(self, x, eb, L=32, T=1, mode=1):
        """Stream bytes for float64 x at absolute bound eb (double), T segments."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        cap = self.lib.szo_max_stream_bytes_d(x.size, L, T, mode)
        out = np.empty(cap, dtype=np.uint8)
        size = ctypes.c_size_t(0)
        rc = self.lib.szo_compress_d(x.ctypes.data, x.size, float(eb), L, T, mode, out.ctypes.data, cap,
                                     ctypes.byref(size))
        if rc != 0:
            raise RuntimeError("oracle compress_d failed: %d" % rc)
        return out[: size.value].tobytes()

    def decompress_d(self, stream, n, L=32, T=1, mode=1):
        buf = np.frombuffer(stream, dtype=np.uint8)
        y = np.empty(n, dtype=np.float64)
        rc = self.lib.szo_decompress_d(buf.ctypes.data, buf.size, n, L, T, mode, y.ctypes.data)
        if rc != 0:
            raise RuntimeError("oracle decompress_d failed: %d" % rc)
        return y

    def reduce_sum(self, a, b, n, L=32, T=1, mode=1, hb=4):
        """The stream of the summed quantization codes of streams a and b
        (same eb header, blockSize, T, mode); hb 4 for float streams, 8 for
        double streams."""
        ba = np.frombuffer(a, dtype=np.uint8)
        bb = np.frombuffer(b, dtype=np.uint8)
        cap = (self.lib.szo_max_stream_bytes_d if hb == 8 else self.lib.szo_max_stream_bytes)(n, L, T, mode)
        out = np.empty(cap, dtype=np.uint8)
        size = ctypes.c_size_t(0)
        rc = self.lib.szo_reduce_sum(ba.ctypes.data, ba.size, bb.ctypes.data, bb.size, n, L, T, mode, hb,
                                     out.ctypes.data, cap, ctypes.byref(size))
        if rc != 0:
            raise RuntimeError("oracle reduce_sum failed: %d" % rc)
        return out[: size.value].tobytes()

    def rel_bound_d(self, x, rel):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return float(self.lib.szo_rel_bound_d(x.ctypes.data, x.size, rel))

    def rel_bound(self, x, rel):
        x = _f32(x)
        return float(np.float32(self.lib.szo_rel_bound(x.ctypes.data, x.size, rel)))

    def bitcount(self, m):
        return self.lib.szo_bitcount(m)

    def thresholds(self):
        thr = np.zeros(34, dtype=np.uint32)
        self.lib.szo_bitcount_thresholds(thr.ctypes.data)
        return thr

    def verify_thresholds(self, thr):
        thr = np.ascontiguousarray(thr, dtype=np.uint32)
        return int(self.lib.szo_bitcount_verify(thr.ctypes.data))


class Reference:
    """ctypes binding of the reference library built from its sources."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            build(ref=True)
        if not os.path.exists(path):
            raise FileNotFoundError("reference library not built (sources absent)")
        self.gomp = ctypes.CDLL("libgomp.so.1", mode=ctypes.RTLD_GLOBAL)
        self.libc = ctypes.CDLL(None)
        self.libc.free.argtypes = [ctypes.c_void_p]
        lib = ctypes.CDLL(path)
        lib.szp_compress.restype = ctypes.c_void_p
        lib.szp_compress.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, _c_size_p, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_size_t, ctypes.c_int]
        lib.szp_decompress.restype = ctypes.c_void_p
        lib.szp_decompress.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_size_t, ctypes.c_int]
        lib.szp_float_single_thread_arg.restype = None
        lib.szp_float_single_thread_arg.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _c_size_p, ctypes.c_float,
                                                    ctypes.c_size_t, ctypes.c_int]
        lib.szp_float_decompress_single_thread_arg.restype = None
        lib.szp_float_decompress_single_thread_arg.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float,
                                                               ctypes.c_int, ctypes.c_void_p]
        self.lib = lib

    def set_threads(self, T):
        self.gomp.omp_set_num_threads(int(T))

    def compress(self, x, L=32, T=1, mode=1, eb_mode=0, abs_eb=0.0, rel=0.0):
        """szp_compress(mode, SZ_FLOAT or SZ_DOUBLE (float64 x), ...) with T OpenMP threads."""
        dbl = np.asarray(x).dtype == np.float64
        x = np.ascontiguousarray(x, dtype=np.float64) if dbl else _f32(x)
        self.set_threads(T)
        size = ctypes.c_size_t(0)
        p = self.lib.szp_compress(mode, 1 if dbl else 0, x.ctypes.data, ctypes.byref(size), eb_mode, abs_eb, rel,
                                  x.size, L)
        if not p:
            raise RuntimeError("reference compress returned NULL")
        out = ctypes.string_at(p, size.value)
        self.libc.free(p)
        return out

    def decompress(self, stream, n, L=32, T=1, mode=1, dtype=np.float32):
        self.set_threads(T)
        dt = np.dtype(dtype)
        buf = np.frombuffer(stream, dtype=np.uint8).copy()
        p = self.lib.szp_decompress(mode, 1 if dt == np.float64 else 0, buf.ctypes.data, buf.size, n, L)
        if not p and n:
            raise RuntimeError("reference decompress returned NULL")
        y = np.frombuffer(ctypes.string_at(p, dt.itemsize * n), dtype=dt).copy() if n else np.empty(0, dt)
        if p:
            self.libc.free(p)
        return y


def _ref_arg_setup(lib):
    for name in ("szp_float_openmp_threadblock_arg", "szp_float_openmp_threadblock_randomaccess_arg"):
        f = getattr(lib, name)
        f.restype = None
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _c_size_p, ctypes.c_float, ctypes.c_size_t, ctypes.c_int]
    for name in ("szp_float_decompress_openmp_threadblock_arg",
                 "szp_float_decompress_openmp_threadblock_randomaccess_arg"):
        f = getattr(lib, name)
        f.restype = None
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]


def reference_record(ref, x, eb, L):
    """The reference's single-thread _record pair on x (float32 or float64)
    at absolute bound eb: (stream, compress tally, decompressed values,
    decompress tally).  Callers keep the stream within the reference's own
    4n-byte (8n for doubles) working buffer (szp_float.cc:634)."""
    lib = ref.lib
    dbl = np.asarray(x).dtype == np.float64
    x = np.ascontiguousarray(x, dtype=np.float64 if dbl else np.float32)
    ct = ctypes.c_double if dbl else ctypes.c_float
    pre = "szp_double" if dbl else "szp_float"
    fc = getattr(lib, pre + "_single_thread_arg_record")
    fc.restype = ctypes.c_size_t
    fc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _c_size_p, ct, ctypes.c_size_t, ctypes.c_int]
    fd = getattr(lib, pre + "_decompress_single_thread_arg_record")
    fd.restype = ctypes.c_size_t
    fd.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ct, ctypes.c_int, ctypes.c_void_p]
    hb = 8 if dbl else 4
    cap = 64 + hb + 16 * x.size + 200 * (x.size // max(L, 1) + 2)
    out = np.zeros(cap, dtype=np.uint8)
    size = ctypes.c_size_t(0)
    rc = int(fc(out.ctypes.data, x.ctypes.data, ctypes.byref(size), ct(eb), x.size, L))
    s = out[: size.value].tobytes()
    y = np.zeros(max(x.size, 1), dtype=x.dtype)
    buf = np.frombuffer(s, dtype=np.uint8).copy()
    rd = int(fd(y.ctypes.data, x.size, ct(eb), L, buf.ctypes.data + hb))
    return s, rc, y[: x.size], rd


def reference_compress_arg(ref, x, eb, L, T, mode):
    """Reference _arg compressor into a generous caller buffer (no final-buffer overflow)."""
    _ref_arg_setup(ref.lib)
    x = _f32(x)
    ref.set_threads(T)
    cap = 64 + 8 * T + 8 * x.size + 200 * (x.size // max(L, 1) + T + 2)
    out = np.zeros(cap, dtype=np.uint8)
    size = ctypes.c_size_t(0)
    fn = ref.lib.szp_float_openmp_threadblock_arg if mode == 1 else \
        ref.lib.szp_float_openmp_threadblock_randomaccess_arg
    fn(out.ctypes.data, x.ctypes.data, ctypes.byref(size), ctypes.c_float(eb), x.size, L)
    return out[: size.value].tobytes()


def reference_decompress_arg(ref, stream, n, L, T, mode):
    _ref_arg_setup(ref.lib)
    ref.set_threads(T)
    buf = np.frombuffer(stream, dtype=np.uint8).copy()
    eb = float(np.frombuffer(bytes(stream[:4])[::-1], dtype=np.float32)[0])
    y = np.zeros(max(n, 1), dtype=np.float32)
    fn = ref.lib.szp_float_decompress_openmp_threadblock_arg if mode == 1 else \
        ref.lib.szp_float_decompress_openmp_threadblock_randomaccess_arg
    fn(y.ctypes.data, n, ctypes.c_float(eb), L, buf.ctypes.data + 4)
    return y[:n]
