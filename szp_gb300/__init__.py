"""szp_gb300 -- Python mirror of SZp's C API over libszp_gb300.so.

The functions keep the reference's names and argument meaning
(SZp/include/szp.h:33-36, szp_float.h, szpd_float.h) and take numpy arrays
for host data.  ``compress_dev`` / ``decompress_dev`` take raw device
pointers (e.g. ``tensor.data_ptr()``) and a CUDA stream handle.

Everything runs in the CUDA library; there is no CPU path.  The first call
fails loudly when the library has not been built.
"""
import ctypes
import os
import weakref

import numpy as np

ABS, REL = 0, 1
SZP_NONRANDOMACCESS, SZP_RANDOMACCESS = 1, 2
SZ_FLOAT, SZ_DOUBLE = 0, 1

OK, EINVAL, ECUDA, ECAPACITY, ECORRUPT, ETIMEOUT, ENOMEM = 0, -1, -2, -3, -4, -5, -6

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libszp_gb300.so")

_sz = ctypes.c_size_t
_szp = ctypes.POINTER(ctypes.c_size_t)
_vp = ctypes.c_void_p


_SIGS = []


def _sig(name, res, args):
    _SIGS.append((name, res, args))


_sig("szp_compress", _vp, [ctypes.c_int, ctypes.c_int, _vp, _szp, ctypes.c_int, ctypes.c_double,
                           ctypes.c_double, _sz, ctypes.c_int])
_sig("szp_decompress", _vp, [ctypes.c_int, ctypes.c_int, _vp, _sz, _sz, ctypes.c_int])
_sig("szp_float_openmp_threadblock", _vp, [_vp, _szp, ctypes.c_float, _sz, ctypes.c_int])
_sig("szp_float_openmp_threadblock_arg", None, [_vp, _vp, _szp, ctypes.c_float, _sz, ctypes.c_int])
_sig("szp_float_single_thread_arg", None, [_vp, _vp, _szp, ctypes.c_float, _sz, ctypes.c_int])
_sig("szp_float_single_thread_arg_record", _sz, [_vp, _vp, _szp, ctypes.c_float, _sz, ctypes.c_int])
_sig("szp_float_openmp_threadblock_randomaccess", _vp, [_vp, _szp, ctypes.c_float, _sz, ctypes.c_int])
_sig("szp_float_openmp_threadblock_randomaccess_arg", None, [_vp, _vp, _szp, ctypes.c_float, _sz, ctypes.c_int])
_sig("szp_float_decompress_openmp_threadblock", _vp, [_sz, ctypes.c_float, ctypes.c_int, _vp])
_sig("szp_float_decompress_openmp_threadblock_arg", None, [_vp, _sz, ctypes.c_float, ctypes.c_int, _vp])
_sig("szp_float_decompress_single_thread_arg", None, [_vp, _sz, ctypes.c_float, ctypes.c_int, _vp])
_sig("szp_float_decompress_single_thread_arg_record", _sz, [_vp, _sz, ctypes.c_float, ctypes.c_int, _vp])
_sig("szp_float_decompress_openmp_threadblock_randomaccess", _vp, [_sz, ctypes.c_float, ctypes.c_int, _vp])
_sig("szp_float_decompress_openmp_threadblock_randomaccess_arg", None,
     [_vp, _sz, ctypes.c_float, ctypes.c_int, _vp])
_sig("szp_gb300_set_segments", None, [ctypes.c_int])
_sig("szp_gb300_get_segments", ctypes.c_int, [])
_sig("szp_gb300_last_error", ctypes.c_char_p, [])
_sig("szp_gb300_last_status", ctypes.c_int, [])
_sig("szp_gb300_last_notices", ctypes.c_int, [])
_sig("szp_gb300_max_stream_bytes", _sz, [_sz, ctypes.c_int, ctypes.c_int, ctypes.c_int])
_sig("szp_gb300_compress_dev", ctypes.c_int, [ctypes.c_int, _vp, _sz, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int, ctypes.c_int, _vp, _sz, _szp, _vp])
_sig("szp_gb300_compress_dev_async", ctypes.c_int, [ctypes.c_int, _vp, _sz, ctypes.c_int, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_int, ctypes.c_int, _vp, _sz, _vp,
                                                    _vp])
_sig("szp_gb300_decompress_dev", ctypes.c_int, [ctypes.c_int, _vp, _sz, _sz, ctypes.c_int, ctypes.c_int, _vp, _vp])
_sig("szp_gb300_max_stream_bytes_f64", _sz, [_sz, ctypes.c_int, ctypes.c_int, ctypes.c_int])
_sig("szp_gb300_compress_dev_f64", ctypes.c_int, [ctypes.c_int, _vp, _sz, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_int, ctypes.c_int, _vp, _sz, _szp, _vp])
_sig("szp_gb300_decompress_dev_f64", ctypes.c_int, [ctypes.c_int, _vp, _sz, _sz, ctypes.c_int, ctypes.c_int, _vp,
                                                    _vp])
_sig("szp_gb300_reduce_sum_dev", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, _sz, _vp, _sz, _sz, ctypes.c_int,
                                                ctypes.c_int, _vp, _sz, _szp, _vp])
for _n in ("szp_double_openmp_threadblock", "szp_double_openmp_threadblock_randomaccess"):
    _sig(_n, _vp, [_vp, _szp, ctypes.c_double, _sz, ctypes.c_int])
for _n in ("szp_double_openmp_threadblock_arg", "szp_double_single_thread_arg",
           "szp_double_openmp_threadblock_randomaccess_arg"):
    _sig(_n, None, [_vp, _vp, _szp, ctypes.c_double, _sz, ctypes.c_int])
_sig("szp_double_single_thread_arg_record", _sz, [_vp, _vp, _szp, ctypes.c_double, _sz, ctypes.c_int])
for _n in ("szp_double_decompress_openmp_threadblock", "szp_double_decompress_openmp_threadblock_randomaccess"):
    _sig(_n, _vp, [_sz, ctypes.c_double, ctypes.c_int, _vp])
for _n in ("szp_double_decompress_openmp_threadblock_arg", "szp_double_decompress_single_thread_arg",
           "szp_double_decompress_openmp_threadblock_randomaccess_arg"):
    _sig(_n, None, [_vp, _sz, ctypes.c_double, ctypes.c_int, _vp])
_sig("szp_double_decompress_single_thread_arg_record", _sz, [_vp, _sz, ctypes.c_double, ctypes.c_int, _vp])
_sig("szp_gb300_decompress_dev_async", ctypes.c_int, [ctypes.c_int, _vp, _sz, _vp, _sz, ctypes.c_int,
                                                      ctypes.c_int, _vp, _vp])
_sig("szp_gb300_sync_status", ctypes.c_int, [_vp])
_sig("szp_gb300_compress_dev_noalloc", ctypes.c_int, [_vp, _sz, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                      ctypes.c_int, ctypes.c_int, _vp, _sz, _szp, _vp])
_sig("szp_gb300_bitcount_thresholds", None, [_vp])
_sig("szp_gb300_bitcount_probe", ctypes.c_int, [_vp, _vp, _sz, _vp])
_sig("szp_gb300_set_timing", None, [ctypes.c_int])
_sig("szp_gb300_set_locate_overlap", None, [ctypes.c_int])
_sig("szp_gb300_set_decode_tickets", None, [ctypes.c_int])
_sig("szp_gb300_lorenzo_max_stream_bytes", _sz, [_sz, _sz, _sz, ctypes.c_int])
_sig("szp_gb300_lorenzo_compress_dev", ctypes.c_int, [_vp, _sz, _sz, _sz, ctypes.c_int, ctypes.c_double,
                                                      ctypes.c_double, ctypes.c_int, _vp, _sz,
                                                      ctypes.POINTER(ctypes.c_size_t), _vp])
_sig("szp_gb300_lorenzo_decompress_dev", ctypes.c_int, [_vp, _sz, _sz, _sz, _sz, ctypes.c_int, _vp, _vp])
_sig("szp_gb300_kernel_ms", ctypes.c_double, [ctypes.c_int])
_sig("szp_gb300_kernel_time", ctypes.c_double, [ctypes.c_int, ctypes.POINTER(ctypes.c_int)])
_sig("szp_gb300_kernel_launches", ctypes.c_ulonglong, [])


class Field(ctypes.Structure):
    """szp_gb300_field: one field of a batch (device buffers)."""
    _fields_ = [("input", _vp), ("input_bytes", _sz), ("input_len_dev", _vp), ("output", _vp),
                ("output_bytes", _sz), ("nbEle", _sz), ("errBoundMode", ctypes.c_int),
                ("absErrBound", ctypes.c_double), ("relBoundRatio", ctypes.c_double)]


_sig("szp_gb300_batch_create", ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(Field), ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int])
_sig("szp_gb300_batch_run", ctypes.c_int, [_vp, _vp])
_sig("szp_gb300_batch_sync", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_int)])
_sig("szp_gb300_batch_sizes_dev", _vp, [_vp])
_sig("szp_gb300_batch_tile_rounds", ctypes.c_int, [_vp])
_sig("szp_gb300_batch_destroy", None, [_vp])


class Request(ctypes.Structure):
    """szp_gb300_request."""
    _fields_ = [("op", ctypes.c_int), ("input", _vp), ("input_bytes", _sz), ("nbEle", _sz),
                ("errBoundMode", ctypes.c_int), ("absErrBound", ctypes.c_double), ("relBoundRatio", ctypes.c_double),
                ("arrival", ctypes.c_double)]


class Result(ctypes.Structure):
    """szp_gb300_result."""
    _fields_ = [("id", ctypes.c_ulonglong), ("status", ctypes.c_int), ("output", _vp), ("output_bytes", _sz),
                ("arrival", ctypes.c_double), ("admitted", ctypes.c_double), ("done", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", _sz), ("max_batch", ctypes.c_int), ("lanes", ctypes.c_int),
                ("segments", ctypes.c_int), ("tile_rounds", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_ulonglong) for k in
                ("requests", "bytes", "queued", "in_flight", "memory_used", "memory_peak")]


_sig("szp_gb300_server_create", ctypes.c_int, [ctypes.POINTER(_vp), ctypes.POINTER(ServerConfig)])
_sig("szp_gb300_server_submit", ctypes.c_int, [_vp, ctypes.POINTER(Request), ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_ulonglong)])
_sig("szp_gb300_server_completed", ctypes.c_int, [_vp, ctypes.POINTER(Result), ctypes.c_int])
_sig("szp_gb300_server_wait", ctypes.c_int, [_vp, ctypes.c_ulonglong, ctypes.POINTER(Result)])
_sig("szp_gb300_server_release", ctypes.c_int, [_vp, ctypes.c_ulonglong])
_sig("szp_gb300_server_drain", ctypes.c_int, [_vp])
_sig("szp_gb300_server_get_stats", ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)])
_sig("szp_gb300_server_clock", ctypes.c_double, [_vp])
_sig("szp_gb300_server_destroy", None, [_vp])
_sig("szp_gb300_last_repairs", ctypes.c_int, [])
_sig("szp_gb300_wait_probe", ctypes.c_int, [ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)])

_libc = ctypes.CDLL(None)
_libc.free.argtypes = [_vp]
_libc.free.restype = None


def _owned_f64(p, n):
    """float64 array over n doubles the library malloc'd at p, freed with the array (no copy)."""
    if n == 0:
        _libc.free(p)
        return np.empty(0, np.float64)
    buf = (ctypes.c_double * n).from_address(p)
    weakref.finalize(buf, _libc.free, p)
    return np.frombuffer(buf, dtype=np.float64)


def _owned_f32(p, n):
    """float32 array over n floats the library malloc'd at p, freed with the array (no copy)."""
    if n == 0:
        _libc.free(p)
        return np.empty(0, np.float32)
    buf = (ctypes.c_float * n).from_address(p)
    weakref.finalize(buf, _libc.free, p)
    return np.frombuffer(buf, dtype=np.float32)


class _Lib:
    """Loads libszp_gb300.so on first use; raises if it has not been built."""

    def __init__(self):
        self._h = None

    def _load(self):
        if not os.path.exists(LIB_PATH):
            raise ImportError("libszp_gb300.so is not built: run __graft_entry__.build() "
                              "or python szp_gb300/build.py")
        h = ctypes.CDLL(LIB_PATH)
        for name, res, args in _SIGS:
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        self._h = h
        return h

    def __getattr__(self, name):
        h = self.__dict__.get("_h") or self._load()
        return getattr(h, name)


_lib = _Lib()
lib = _lib


class SzpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


def last_error():
    return (_lib.szp_gb300_last_error() or b"").decode()


def last_status():
    return _lib.szp_gb300_last_status()


def last_notices():
    """1 when the last call met a value the reference quantizes outside its
    int32 range (NaN or |x/eb| >= 2^31), else 0."""
    return _lib.szp_gb300_last_notices()


def _raise(what):
    raise SzpError(last_status(), "%s failed: %s" % (what, last_error()))


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32).ravel()


def set_segments(T):
    """Fix the segment count T (0 = OpenMP default, like the reference)."""
    _lib.szp_gb300_set_segments(int(T))


def get_segments():
    return _lib.szp_gb300_get_segments()


def max_stream_bytes(n, block_size=32, segments=0, fast_mode=1):
    return _lib.szp_gb300_max_stream_bytes(n, block_size, segments, fast_mode)


def szp_compress(data, err_bound_mode=ABS, abs_err_bound=0.0, rel_bound_ratio=0.0, block_size=32,
                 fast_mode=SZP_NONRANDOMACCESS, data_type=SZ_FLOAT):
    """szp_compress (SZp/include/szp.h:33) on a host array -> bytes: float32
    (SZ_FLOAT) or float64 (SZ_DOUBLE)."""
    x = np.ascontiguousarray(data, dtype=np.float64).ravel() if data_type == SZ_DOUBLE else _f32(data)
    size = ctypes.c_size_t(0)
    p = _lib.szp_compress(fast_mode, data_type, x.ctypes.data, ctypes.byref(size), err_bound_mode,
                          abs_err_bound, rel_bound_ratio, x.size, block_size)
    if not p:
        _raise("szp_compress")
    out = ctypes.string_at(p, size.value)
    _libc.free(p)
    return out


def szp_decompress(stream, n, block_size=32, fast_mode=SZP_NONRANDOMACCESS, data_type=SZ_FLOAT,
                   byte_length=None):
    """szp_decompress (SZp/include/szp.h:36) -> float32 (SZ_FLOAT) or float64
    (SZ_DOUBLE) array of n values."""
    buf = np.frombuffer(stream, dtype=np.uint8)
    bl = buf.size if byte_length is None else byte_length
    p = _lib.szp_decompress(fast_mode, data_type, buf.ctypes.data, bl, n, block_size)
    if not p:
        _raise("szp_decompress")
    return _owned_f64(p, n) if data_type == SZ_DOUBLE else _owned_f32(p, n)


def szp_float_openmp_threadblock(data, abs_err_bound, block_size=32):
    x = _f32(data)
    size = ctypes.c_size_t(0)
    p = _lib.szp_float_openmp_threadblock(x.ctypes.data, ctypes.byref(size), abs_err_bound, x.size, block_size)
    if not p:
        _raise("szp_float_openmp_threadblock")
    out = ctypes.string_at(p, size.value)
    _libc.free(p)
    return out


def _arg_compress(fn, data, abs_err_bound, block_size, capacity=None):
    x = _f32(data)
    cap = 4 + 4 * x.size if capacity is None else capacity
    out = np.zeros(max(cap, 1), dtype=np.uint8)
    size = ctypes.c_size_t(0)
    getattr(_lib, fn)(out.ctypes.data, x.ctypes.data, ctypes.byref(size), abs_err_bound, x.size, block_size)
    if size.value == 0:
        _raise(fn)
    return out[: size.value].tobytes()


def szp_float_openmp_threadblock_arg(data, abs_err_bound, block_size=32):
    return _arg_compress("szp_float_openmp_threadblock_arg", data, abs_err_bound, block_size)


def szp_float_single_thread_arg(data, abs_err_bound, block_size=32):
    return _arg_compress("szp_float_single_thread_arg", data, abs_err_bound, block_size)


def szp_float_openmp_threadblock_randomaccess(data, abs_err_bound, block_size=32):
    x = _f32(data)
    size = ctypes.c_size_t(0)
    p = _lib.szp_float_openmp_threadblock_randomaccess(x.ctypes.data, ctypes.byref(size), abs_err_bound, x.size,
                                                       block_size)
    if not p:
        _raise("szp_float_openmp_threadblock_randomaccess")
    out = ctypes.string_at(p, size.value)
    _libc.free(p)
    return out


def szp_float_openmp_threadblock_randomaccess_arg(data, abs_err_bound, block_size=32):
    return _arg_compress("szp_float_openmp_threadblock_randomaccess_arg", data, abs_err_bound, block_size)


def _eb_of(stream):
    return float(np.frombuffer(bytes(stream[:4])[::-1], dtype=np.float32)[0])


def szp_float_decompress_openmp_threadblock(stream, n, block_size=32, fast_mode=1):
    """Per-type decompressor: passes stream+4 and eb like the reference's callers."""
    buf = np.frombuffer(stream, dtype=np.uint8)
    eb = _eb_of(stream)
    fn = (_lib.szp_float_decompress_openmp_threadblock if fast_mode == 1
          else _lib.szp_float_decompress_openmp_threadblock_randomaccess)
    p = fn(n, eb, block_size, buf.ctypes.data + 4)
    if not p:
        _raise("szp_float_decompress_openmp_threadblock")
    y = _owned_f32(p, n)
    return y


def szp_float_decompress_arg(stream, n, block_size=32, which="openmp_threadblock_arg"):
    buf = np.frombuffer(stream, dtype=np.uint8)
    eb = _eb_of(stream)
    y = np.empty(max(n, 1), dtype=np.float32)
    getattr(_lib, "szp_float_decompress_" + which)(y.ctypes.data, n, eb, block_size, buf.ctypes.data + 4)
    if last_status() != 0:
        _raise("szp_float_decompress_" + which)
    return y[:n]


def single_thread_arg_record(data, abs_err_bound, block_size=32):
    """szp_float_single_thread_arg_record / szp_double_single_thread_arg_record
    (SZp/include/szp_float.h:39, szp_double.h:39) on a float32 or float64 host
    array: returns (stream, the reference's memory-access tally)."""
    dbl = np.asarray(data).dtype == np.float64
    x = np.ascontiguousarray(data, dtype=np.float64).ravel() if dbl else _f32(data)
    out = np.zeros(max(x.itemsize * (x.size + 1), 1), dtype=np.uint8)
    size = ctypes.c_size_t(0)
    fn = _lib.szp_double_single_thread_arg_record if dbl else _lib.szp_float_single_thread_arg_record
    tally = fn(out.ctypes.data, x.ctypes.data, ctypes.byref(size), abs_err_bound, x.size, block_size)
    if size.value == 0 or last_status() != 0:
        _raise("single_thread_arg_record")
    return out[: size.value].tobytes(), int(tally)


def decompress_single_thread_arg_record(stream, n, block_size=32, data_type=SZ_FLOAT):
    """szp_float_decompress_single_thread_arg_record (szpd_float.h:27) or its
    double twin (szpd_double.h:27): returns (values, the reference's
    memory-access tally)."""
    buf = np.frombuffer(stream, dtype=np.uint8)
    if data_type == SZ_DOUBLE:
        eb = float(np.frombuffer(bytes(stream[:8])[::-1], dtype=np.float64)[0])
        y = np.empty(max(n, 1), dtype=np.float64)
        tally = _lib.szp_double_decompress_single_thread_arg_record(y.ctypes.data, n, eb, block_size,
                                                                    buf.ctypes.data + 8)
    else:
        y = np.empty(max(n, 1), dtype=np.float32)
        tally = _lib.szp_float_decompress_single_thread_arg_record(y.ctypes.data, n, _eb_of(stream), block_size,
                                                                   buf.ctypes.data + 4)
    if last_status() != 0:
        _raise("decompress_single_thread_arg_record")
    return y[:n], int(tally)


def compress_dev(d_data, n, d_out, capacity, err_bound_mode=ABS, abs_err_bound=0.0, rel_bound_ratio=0.0,
                 block_size=32, segments=0, fast_mode=1, stream=0):
    """Device-pointer compressor; returns the stream size in bytes."""
    size = ctypes.c_size_t(0)
    rc = _lib.szp_gb300_compress_dev(fast_mode, d_data, n, err_bound_mode, abs_err_bound, rel_bound_ratio,
                                     block_size, segments, d_out, capacity, ctypes.byref(size), stream or None)
    if rc != 0:
        raise SzpError(rc, "compress_dev failed: %s" % last_error())
    return size.value


def compress_dev_async(d_data, n, d_out, capacity, d_size, err_bound_mode=ABS, abs_err_bound=0.0,
                       rel_bound_ratio=0.0, block_size=32, segments=0, fast_mode=1, stream=0):
    rc = _lib.szp_gb300_compress_dev_async(fast_mode, d_data, n, err_bound_mode, abs_err_bound, rel_bound_ratio,
                                           block_size, segments, d_out, capacity, d_size, stream or None)
    if rc != 0:
        raise SzpError(rc, "compress_dev_async failed: %s" % last_error())


def max_stream_bytes_f64(n, block_size=32, segments=0, fast_mode=1):
    return _lib.szp_gb300_max_stream_bytes_f64(n, block_size, segments, fast_mode)


def compress_dev_f64(d_data, n, d_out, capacity, err_bound_mode=ABS, abs_err_bound=0.0, rel_bound_ratio=0.0,
                     block_size=32, segments=0, fast_mode=1, stream=0):
    """float64 device-pointer compressor; returns the stream size in bytes."""
    size = ctypes.c_size_t(0)
    rc = _lib.szp_gb300_compress_dev_f64(fast_mode, d_data, n, err_bound_mode, abs_err_bound, rel_bound_ratio,
                                         block_size, segments, d_out, capacity, ctypes.byref(size), stream or None)
    if rc != 0:
        raise SzpError(rc, "compress_dev_f64 failed: %s" % last_error())
    return size.value


def reduce_sum_dev(d_a, len_a, d_b, len_b, n, d_out, capacity, block_size=32, segments=0, fast_mode=1,
                   data_type=SZ_FLOAT, stream=0):
    """Homomorphic sum of two device streams of the same bound; returns the
    result's size (szp_gb300_reduce_sum_dev)."""
    size = ctypes.c_size_t(0)
    rc = _lib.szp_gb300_reduce_sum_dev(fast_mode, data_type, d_a, len_a, d_b, len_b, n, block_size, segments, d_out,
                                       capacity, ctypes.byref(size), stream or None)
    if rc != 0:
        raise SzpError(rc, "reduce_sum_dev failed: %s" % last_error())
    return size.value


def decompress_dev_f64(d_stream, length, n, d_out, block_size=32, segments=0, fast_mode=1, stream=0):
    rc = _lib.szp_gb300_decompress_dev_f64(fast_mode, d_stream, length, n, block_size, segments, d_out,
                                           stream or None)
    if rc != 0:
        raise SzpError(rc, "decompress_dev_f64 failed: %s" % last_error())


def decompress_dev(d_stream, length, n, d_out, block_size=32, segments=0, fast_mode=1, stream=0):
    rc = _lib.szp_gb300_decompress_dev(fast_mode, d_stream, length, n, block_size, segments, d_out, stream or None)
    if rc != 0:
        raise SzpError(rc, "decompress_dev failed: %s" % last_error())


def decompress_dev_async(d_stream, capacity, d_len, n, d_out, block_size=32, segments=0, fast_mode=1, stream=0):
    """Decompress a device stream whose length sits in device memory at d_len."""
    rc = _lib.szp_gb300_decompress_dev_async(fast_mode, d_stream, capacity, d_len, n, block_size, segments, d_out,
                                             stream or None)
    if rc != 0:
        raise SzpError(rc, "decompress_dev_async failed: %s" % last_error())


def compress_dev_noalloc(d_data, n, d_out, capacity, err_bound_mode=ABS, abs_err_bound=0.0, rel_bound_ratio=0.0,
                         block_size=32, segments=0, stream=0):
    """Allocation-free fastmode1 compressor (static device working memory);
    returns the stream size.  For callers that cannot allocate device memory
    while compressing."""
    size = ctypes.c_size_t(0)
    rc = _lib.szp_gb300_compress_dev_noalloc(d_data, n, err_bound_mode, abs_err_bound, rel_bound_ratio, block_size,
                                             segments, d_out, capacity, ctypes.byref(size), stream or None)
    if rc != 0:
        raise SzpError(rc, "compress_dev_noalloc failed: %s" % last_error())
    return size.value


def sync_status(stream=0):
    return _lib.szp_gb300_sync_status(stream or None)


def bitcount_thresholds():
    thr = np.zeros(34, dtype=np.uint32)
    _lib.szp_gb300_bitcount_thresholds(thr.ctypes.data)
    return thr


def set_locate_overlap(nbytes):
    """Bytes walked before a decompression chunk (-1 = default); for tests."""
    _lib.szp_gb300_set_locate_overlap(int(nbytes))


def lorenzo_max_stream_bytes(dims, segments=0):
    """Capacity that always fits the Lorenzo stream of a (nz, ny, nx) field."""
    nz, ny, nx = dims
    return _lib.szp_gb300_lorenzo_max_stream_bytes(nx, ny, nz, segments)


def lorenzo_compress_dev(d_data, dims, d_out, capacity, err_bound_mode=ABS, abs_err_bound=0.0, rel_bound_ratio=0.0,
                         segments=0, stream=0):
    """Multidimensional Lorenzo compressor of a (nz, ny, nx) device field;
    returns the stream size in bytes."""
    nz, ny, nx = dims
    size = ctypes.c_size_t(0)
    rc = _lib.szp_gb300_lorenzo_compress_dev(d_data, nx, ny, nz, err_bound_mode, abs_err_bound, rel_bound_ratio,
                                             segments, d_out, capacity, ctypes.byref(size), stream or None)
    if rc != 0:
        raise SzpError(rc, "lorenzo_compress_dev failed: %s" % last_error())
    return size.value


def lorenzo_decompress_dev(d_stream, length, dims, d_out, segments=0, stream=0):
    nz, ny, nx = dims
    rc = _lib.szp_gb300_lorenzo_decompress_dev(d_stream, length, nx, ny, nz, segments, d_out, stream or None)
    if rc != 0:
        raise SzpError(rc, "lorenzo_decompress_dev failed: %s" % last_error())


def set_decode_tickets(on):
    """Single-field decode with tile tickets instead of the cooperative static
    schedule (the fallback path); for tests."""
    _lib.szp_gb300_set_decode_tickets(1 if on else 0)


def set_timing(on):
    _lib.szp_gb300_set_timing(1 if on else 0)


def kernel_ms(slot):
    return _lib.szp_gb300_kernel_ms(slot)


def kernel_time(slot):
    """(total ms, launches) of kernel `slot` since the last read."""
    cnt = ctypes.c_int(0)
    ms = _lib.szp_gb300_kernel_time(slot, ctypes.byref(cnt))
    return ms, cnt.value


SLOT_REL, SLOT_COMPRESS, SLOT_SETUP, SLOT_LOCATE, SLOT_DECODE = range(5)


def wait_probe(limit_ns):
    """One device wait on a barrier nothing completes, bounded by limit_ns:
    (status, nanoseconds waited); the status is ETIMEOUT when it gave up."""
    waited = ctypes.c_ulonglong(0)
    rc = _lib.szp_gb300_wait_probe(int(limit_ns), ctypes.byref(waited))
    return rc, waited.value


def last_repairs():
    return _lib.szp_gb300_last_repairs()


def kernel_launches():
    return int(_lib.szp_gb300_kernel_launches())


BATCH_COMPRESS, BATCH_DECOMPRESS = 0, 1
BATCH_AUTOTUNE, BATCH_NO_GRAPH = 1, 2


class Batch:
    """A batched compression or decompression (szp_gb300_batch_*).

    ``fields`` is a list of dicts with the keys of szp_gb300_field (device
    pointers as ints).  ``run`` queues one replay on a stream; ``sync`` waits
    and returns (sizes, statuses) per field.
    """

    def __init__(self, direction, fields, block_size=32, segments=0, flags=0):
        self.n = len(fields)
        arr = (Field * max(self.n, 1))()
        for i, f in enumerate(fields):
            for k, v in f.items():
                setattr(arr[i], k, v)
        h = _vp()
        rc = _lib.szp_gb300_batch_create(ctypes.byref(h), direction, arr, self.n, block_size, segments, flags)
        if rc != 0:
            raise SzpError(rc, "batch_create failed: %s" % last_error())
        self._h = h
        self.direction = direction

    def run(self, stream=0):
        rc = _lib.szp_gb300_batch_run(self._h, stream or None)
        if rc != 0:
            raise SzpError(rc, "batch_run failed: %s" % last_error())

    def sync(self, check=True):
        sizes = (ctypes.c_ulonglong * max(self.n, 1))()
        status = (ctypes.c_int * max(self.n, 1))()
        rc = _lib.szp_gb300_batch_sync(self._h, sizes, status)
        if rc != 0 and check:
            raise SzpError(rc, "batch failed: %s" % last_error())
        return [int(v) for v in sizes[:self.n]], [int(v) for v in status[:self.n]]

    def sizes_dev(self):
        """Device address of the per-field stream sizes (unsigned long long[n])."""
        return _lib.szp_gb300_batch_sizes_dev(self._h)

    def tile_rounds(self):
        return _lib.szp_gb300_batch_tile_rounds(self._h)

    def close(self):
        if getattr(self, "_h", None):
            _lib.szp_gb300_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _result_dict(r):
    return dict(id=int(r.id), status=int(r.status), output=r.output or 0, output_bytes=int(r.output_bytes),
                arrival=r.arrival, admitted=r.admitted, done=r.done)


class Server:
    """The request server (szp_gb300_server_*): continuous batching of compress
    and decompress requests on device-resident data under an HBM budget."""

    def __init__(self, hbm_budget, max_batch=256, lanes=3, segments=0, tile_rounds=0):
        cfg = ServerConfig(hbm_budget, max_batch, lanes, segments, tile_rounds)
        h = _vp()
        rc = _lib.szp_gb300_server_create(ctypes.byref(h), ctypes.byref(cfg))
        if rc != 0:
            raise SzpError(rc, "server_create failed: %s" % last_error())
        self._h = h
        self._buf = (Result * 4096)()

    def clock(self):
        return _lib.szp_gb300_server_clock(self._h)

    def submit(self, reqs):
        """reqs: list of dicts with the keys of szp_gb300_request; returns their ids."""
        n = len(reqs)
        arr = (Request * max(n, 1))()
        for i, r in enumerate(reqs):
            arr[i].arrival = -1.0
            for k, v in r.items():
                setattr(arr[i], k, v)
        ids = (ctypes.c_ulonglong * max(n, 1))()
        rc = _lib.szp_gb300_server_submit(self._h, arr, n, ids)
        if rc != 0:
            raise SzpError(rc, "server_submit failed: %s" % last_error())
        return [int(v) for v in ids[:n]]

    def completed(self):
        """Results finished since the last call (dicts)."""
        out = []
        while True:
            k = _lib.szp_gb300_server_completed(self._h, self._buf, len(self._buf))
            out += [_result_dict(self._buf[i]) for i in range(k)]
            if k < len(self._buf):
                return out

    def wait(self, rid):
        r = Result()
        _lib.szp_gb300_server_wait(self._h, rid, ctypes.byref(r))
        return _result_dict(r)

    def release(self, rid):
        rc = _lib.szp_gb300_server_release(self._h, rid)
        if rc != 0:
            raise SzpError(rc, "server_release failed: %s" % last_error())

    def drain(self):
        return _lib.szp_gb300_server_drain(self._h)

    def stats(self):
        st = ServerStats()
        _lib.szp_gb300_server_get_stats(self._h, ctypes.byref(st))
        return {k: int(getattr(st, k)) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            _lib.szp_gb300_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
