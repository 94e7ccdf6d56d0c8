"""fxe_thermo_compute_device_fixed: the statmech reduction with library-owned scratch, compared
with fxe_thermo_compute_device on the same device-resident ensembles. Collected last."""
import ctypes as C

import numpy as np
import pytest

from flexaidds_gb300 import capi, evaluator

pytestmark = pytest.mark.gpu

# both reductions are FP64 and merge block partials in a different order; Cv (a variance)
# amplifies that rounding, so the bound is the statmech tolerance of the path, 1e-9 relative
TOL = 1e-9


def _lib():
    lib = evaluator.load_library()
    lib.fxe_thermo_compute_device_fixed.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_double,
                                                    C.c_void_p, C.c_void_p]
    return lib


def _fields(t):
    return {k: getattr(t, k) for k, _ in capi.Thermo._fields_}


def _close(a, b):
    for k in a:
        assert abs(a[k] - b[k]) <= TOL * max(1.0, abs(b[k])), (k, a[k], b[k])


def _fixed(lib, torch, de, dm, n, T, stream):
    dout = torch.zeros(C.sizeof(capi.Thermo), dtype=torch.uint8, device="cuda")
    rc = lib.fxe_thermo_compute_device_fixed(C.c_void_p(de.data_ptr()),
                                             C.c_void_p(dm.data_ptr()) if dm is not None else None,
                                             n, T, C.c_void_p(dout.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.fxe_last_error().decode()
    stream.synchronize()
    return _fields(capi.Thermo.from_buffer_copy(dout.cpu().numpy().tobytes()))


def _existing(lib, de, dm, n, T, stream):
    t = capi.Thermo()
    rc = lib.fxe_thermo_compute_device(C.c_void_p(de.data_ptr()),
                                       C.c_void_p(dm.data_ptr()) if dm is not None else None,
                                       n, T, C.byref(t), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.fxe_last_error().decode()
    return _fields(t)


@pytest.mark.parametrize("n", [1, 4095, 4097, 1_000_000])
def test_fixed_scratch_matches_allocating_entry_point(n):
    torch = pytest.importorskip("torch")
    lib = _lib()
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(n)
    for call in range(2):   # two calls in a row on the shared scratch
        e = rng.normal(-30.0 + 5 * call, 4.0, n)
        m = rng.integers(1, 5, n).astype(np.int32)
        de = torch.from_numpy(e).cuda()
        dm = torch.from_numpy(m).cuda()
        torch.cuda.synchronize()
        for mult in (None, dm):
            _close(_fixed(lib, torch, de, mult, n, 300.0, stream), _existing(lib, de, mult, n, 300.0, stream))


def test_fixed_scratch_allocates_nothing_after_setup():
    torch = pytest.importorskip("torch")
    lib = _lib()
    stream = torch.cuda.Stream()
    de = torch.from_numpy(np.random.default_rng(3).normal(-20.0, 2.0, 200_000)).cuda()
    dout = torch.zeros(C.sizeof(capi.Thermo), dtype=torch.uint8, device="cuda")
    args = (C.c_void_p(de.data_ptr()), None, 200_000, 310.0, C.c_void_p(dout.data_ptr()),
            C.c_void_p(stream.cuda_stream))
    assert lib.fxe_thermo_compute_device_fixed(*args) == 0     # first call: set-up
    stream.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.fxe_thermo_compute_device_fixed(*args) == 0
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_fixed_scratch_rejects_oversized_and_bad_input():
    torch = pytest.importorskip("torch")
    lib = _lib()
    de = torch.zeros(8, dtype=torch.float64, device="cuda")
    dout = torch.zeros(C.sizeof(capi.Thermo), dtype=torch.uint8, device="cuda")
    too_many = (1 << 16) * 256 * 16 + 1
    rc = lib.fxe_thermo_compute_device_fixed(C.c_void_p(de.data_ptr()), None, too_many, 300.0,
                                             C.c_void_p(dout.data_ptr()), None)
    assert rc == 1 and b"exceeds" in lib.fxe_last_error()
    assert lib.fxe_thermo_compute_device_fixed(C.c_void_p(de.data_ptr()), None, 0, 300.0,
                                               C.c_void_p(dout.data_ptr()), None) == 1
    assert lib.fxe_thermo_compute_device_fixed(C.c_void_p(de.data_ptr()), None, 8, 300.0, None, None) == 1
