"""The single-thread _record entry points through the C ABI: the T = 1
stream byte for byte, the decompressed values bit for bit, and the
reference's `total_memaccess` tallies (szp_float.cc:607-750,
szpd_float.cc:216-318, szp_double.cc:613-756, szpd_double.cc:219-321)
equal to the values the reference itself returned on the same inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_record_entry_points_match_reference(szp, golden_record):
    for c in golden_record:
        if len(c["s"]) > c["x"].itemsize * (c["n"] + 1):
            # the reference's callers size `output` as one value more than the
            # input; a longer stream (tiny n: the header alone is 12-16 bytes)
            # is refused instead of overrunning it
            with pytest.raises(szp.SzpError) as e:
                szp.single_thread_arg_record(c["x"], c["bound"], c["L"])
            assert e.value.status == szp.ECAPACITY, c["name"]
        else:
            s, tally = szp.single_thread_arg_record(c["x"], c["bound"], c["L"])
            assert s == c["s"], c["name"]
            assert tally == c["rec_c"], (c["name"], tally, c["rec_c"])
        dt = szp.SZ_DOUBLE if c["dbl"] else szp.SZ_FLOAT
        y, dtally = szp.decompress_single_thread_arg_record(c["s"], c["n"], c["L"], dt)
        u = np.uint64 if c["dbl"] else np.uint32
        assert np.array_equal(y.view(u), c["y"].view(u)), c["name"]
        assert dtally == c["rec_d"], (c["name"], dtally, c["rec_d"])


def test_record_tally_on_a_field_vs_oracle(szp, port):
    """A larger field than the fixtures (REL-sized bound on a walk): the
    library's tallies equal the oracle's restatement of the reference loops."""
    from szp_gb300.workloads import walk
    x = walk(1 << 20, np.random.default_rng(11))
    eb = float(np.float32(1e-4 * (x.max() - x.min())))
    s, tally = szp.single_thread_arg_record(x, eb, 32)
    assert tally == port.record_compress(s, x.size, 32)
    _, dtally = szp.decompress_single_thread_arg_record(s, x.size, 32)
    assert dtally == port.record_decompress(s, x.size, 32)
