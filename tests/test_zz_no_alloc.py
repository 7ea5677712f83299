"""The allocation-free entry point, last in collection order.

sevc_rng_record_noalloc serves callers that cannot let a library call
cudaMalloc (memory handed out only from their own pool, a device budget
already taken by the simulation, or no tolerance for the implicit
synchronisation an allocation can cause).  Its generator-state scratch is a
fixed device array inside the library; the caller supplies the output.
Here the caller's output buffer comes from the CUDA runtime directly, and
the draws of two consecutive calls must equal, bit for bit, those of the
allocating entry point sevc_rng_record.
"""
import ctypes
import glob

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cudart():
    for name in ["libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found")


def test_noalloc_record_matches_allocating_record(gpu):
    rt = cudart()
    nstreams, ndraws = 8192, 12
    ref = gpu.rng_record(nstreams, ndraws)
    nbytes = nstreams * ndraws * 8
    dptr = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(dptr), ctypes.c_size_t(nbytes)) == 0
    try:
        for call in range(2):
            rt.cudaMemset(dptr, 0, ctypes.c_size_t(nbytes))
            gpu.rng_record_noalloc(nstreams, ndraws, dptr.value)
            assert rt.cudaDeviceSynchronize() == 0
            out = np.empty((nstreams, ndraws), np.float64)
            rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            assert rt.cudaMemcpy(out.ctypes.data, dptr, nbytes, 2) == 0   # device to host
            assert np.array_equal(out, ref), "call %d differs from sevc_rng_record" % call
        small = gpu.rng_record(100, 3)
        gpu.rng_record_noalloc(100, 3, dptr.value)
        assert rt.cudaDeviceSynchronize() == 0
        out = np.empty((100, 3), np.float64)
        assert rt.cudaMemcpy(out.ctypes.data, dptr, 100 * 3 * 8, 2) == 0
        assert np.array_equal(out, small)
        # after the first call (which commits the fixed array), further
        # calls take no device memory
        free0, free1, total = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        assert rt.cudaMemGetInfo(ctypes.byref(free0), ctypes.byref(total)) == 0
        for _ in range(3):
            gpu.rng_record_noalloc(nstreams, ndraws, dptr.value)
        assert rt.cudaDeviceSynchronize() == 0
        assert rt.cudaMemGetInfo(ctypes.byref(free1), ctypes.byref(total)) == 0
        assert free1.value == free0.value
    finally:
        rt.cudaFree(dptr)
    with pytest.raises(gpu.SevcError) as e:
        gpu.rng_record_noalloc(8193, 1, 1)
    assert e.value.code == 7 and "8192" in str(e.value)
