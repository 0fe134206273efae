"""The allocation-free <Z_q> reduction (qf_expectation_z_all_noalloc).

It exists for callers that cannot let a library allocate device memory (a
framework that owns all device memory through its own pool, or a loop where
cudaMalloc/cudaFree would synchronise the device). It reads a state from a raw
device pointer and uses only a fixed scratch array in the library's device
image. This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

from quantumforge_gb300 import StateVector
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import _native
from quantumforge_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(lib, device, ptr, n, dtype, stream):
    out = np.full(n, np.nan)
    st = lib.qf_expectation_z_all_noalloc(device, ptr, n, dtype, stream, _native.ptr(out), n)
    _native.check(st)
    return out


@pytest.mark.parametrize("dtype,code,tol", [("c64", A.C64, 1e-5), ("c128", A.C128, 1e-11)])
@pytest.mark.parametrize("n", [1, 5, 8, 9, 14, 21])
def test_noalloc_matches_the_allocating_reduction(backend, dtype, code, tol, n):
    """n = 8 is the smallest state on the chunked kernel (one warp); n = 14
    runs several blocks of 256 threads whose thread-id bits meet the
    block-index bits."""
    import torch

    lib = _native.load()
    ops = W.random_circuit(n, 6, 300 + n, two_qubit="mixed" if n > 3 else "ladder")
    sv = StateVector.zero(n, dtype=dtype, backend=backend)
    sv.apply_ops(ops)
    expected = sv.expectation_z_all()
    amps = sv.amplitudes()
    oracle_z = np.array([O.expectation(amps, 2, q) for q in range(n)])
    dptr, stream = C.c_void_p(), C.c_void_p()
    _native.check(lib.qf_sv_device_ptr(sv._h, C.byref(dptr)))
    _native.check(lib.qf_ctx_stream(backend.handle, C.byref(stream)))
    backend.synchronize()
    device_before = torch.cuda.current_device()
    # two calls in a row share the scratch array: both must be right
    first = _noalloc(lib, backend.ordinal, dptr, n, code, stream)
    second = _noalloc(lib, backend.ordinal, dptr, n, code, stream)
    # the legacy default stream (NULL) as well
    third = _noalloc(lib, backend.ordinal, dptr, n, code, None)
    assert torch.cuda.current_device() == device_before
    for got in (first, second, third):
        assert np.abs(got - expected).max() <= tol
        assert np.abs(got - oracle_z).max() <= tol


def test_noalloc_rejects_states_beyond_its_scratch(backend):
    lib = _native.load()
    out = np.zeros(41)
    st = lib.qf_expectation_z_all_noalloc(backend.ordinal, C.c_void_p(256), 41, A.C64, None, _native.ptr(out), 41)
    assert A.STATUS_NAMES[st] == "StateTooLarge"
    assert "at most 40 qubits" in lib.qf_last_error().decode()
