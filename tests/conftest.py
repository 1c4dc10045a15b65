import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import Port
    return Port()


@pytest.fixture(scope="session")
def golden():
    path = os.path.join(ROOT, "tests", "golden", "golden.npz")
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    cases = []
    for i, m in enumerate(meta):
        cases.append(dict(m, x=z["x%d" % i], s=z["s%d" % i].tobytes(), y=z["y%d" % i]))
    return cases


@pytest.fixture(scope="session")
def golden_double():
    path = os.path.join(ROOT, "tests", "golden", "golden_double.npz")
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    cases = []
    for i, m in enumerate(meta):
        cases.append(dict(m, x=z["x%d" % i], s=z["s%d" % i].tobytes(), y=z["y%d" % i]))
    return cases


@pytest.fixture(scope="session")
def szp():
    import szp_gb300
    return szp_gb300


def eb_of(stream):
    return float(np.frombuffer(bytes(stream[:4])[::-1], dtype=np.float32)[0])


def eb_of_double(stream):
    return float(np.frombuffer(bytes(stream[:8])[::-1], dtype=np.float64)[0])


@pytest.fixture(scope="session")
def golden_record():
    """The reference's single-thread _record entry points: stream, tallies
    (rec_c compress, rec_d decompress) and decompressed values."""
    path = os.path.join(ROOT, "tests", "golden", "golden_record.npz")
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    return [dict(m, x=z["x%d" % i], s=z["s%d" % i].tobytes(), y=z["y%d" % i]) for i, m in enumerate(meta)]
