import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "se-grain-growth-gpu_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def gpu_available():
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import glob
            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
            rt = ctypes.CDLL(cands[0]) if cands else None
        except OSError:
            rt = None
    if rt is None:
        return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def engine_mod():
    import build as sevc_build
    sevc_build.build()
    import sevc
    return sevc


@pytest.fixture(scope="session")
def gpu(engine_mod):
    if not gpu_available():
        pytest.fail("a -m gpu test ran without a CUDA device")
    return engine_mod


@pytest.fixture
def tmpdir_clean(tmp_path):
    yield str(tmp_path)
    shutil.rmtree(str(tmp_path), ignore_errors=True)
