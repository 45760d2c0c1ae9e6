"""The allocation-free entry point cfem_matvec_energy_noalloc.

It serves callers that cannot allocate device memory (code inside another
framework's memory pool, or a loop that must not pay cudaMalloc's implicit
device synchronisation): the caller passes device input and output, the only
scratch is a fixed array inside the library. Its results must equal those of
the allocating entry point cfem_matvec (and x.y), on two calls in a row, since
the shared scratch keeps the previous call's contents. This file is named to be
collected last.
"""
import ctypes as C

import numpy as np
import pytest

from cudafemproject_gb300 import capi, meshgen

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dim", [3, 2])
def test_noalloc_matches_allocating_matvec(dim):
    torch = pytest.importorskip("torch")
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(6, 5, 14, jitter=0.2, seed=11) if dim == 3 else meshgen.square_2d(24)
    ctx = FemContext(p)
    L = capi.lib()
    rng = np.random.default_rng(7)
    for call in range(2):
        xh = rng.standard_normal(p.n_dof)
        x = torch.tensor(xh, device="cuda")
        y = torch.full_like(x, 123.0)  # stale contents must not leak into the result
        e_dev = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        st = L.cfem_matvec_energy_noalloc(ctx._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                          C.c_void_p(e_dev.data_ptr()))
        capi.check(st, "cfem_matvec_energy_noalloc")
        y_ref = ctx.matvec(xh, "fp64")  # the existing, allocating entry point
        e_ref = float(xh @ y_ref)
        assert _rel(y.cpu().numpy(), y_ref) <= 1e-13, call
        assert abs(e_dev.item() - e_ref) <= 1e-12 * abs(e_ref), call
        e_host = C.c_double(0.0)
        st = L.cfem_matvec_energy_noalloc(ctx._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                          C.byref(e_host))
        capi.check(st, "cfem_matvec_energy_noalloc (host energy)")
        assert abs(e_host.value - e_ref) <= 1e-12 * abs(e_ref), call


def test_noalloc_allocates_no_device_memory():
    """After a first call (which resolves the scratch address on this device),
    further calls leave both the device's free memory and torch's allocator
    untouched, with device and host energy pointers."""
    torch = pytest.importorskip("torch")
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(5, 5, 12, jitter=0.2, seed=3)
    ctx = FemContext(p)
    L = capi.lib()
    x = torch.tensor(np.random.default_rng(1).standard_normal(p.n_dof), device="cuda")
    y = torch.empty_like(x)
    e_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    e_host = C.c_double(0.0)
    args = lambda e: (ctx._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), e)
    capi.check(L.cfem_matvec_energy_noalloc(*args(C.c_void_p(e_dev.data_ptr()))), "warm-up")
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for _ in range(3):
        capi.check(L.cfem_matvec_energy_noalloc(*args(C.c_void_p(e_dev.data_ptr()))), "device energy")
        capi.check(L.cfem_matvec_energy_noalloc(*args(C.byref(e_host))), "host energy")
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0
    assert e_host.value == e_dev.item()


def test_noalloc_rejects_bad_arguments():
    from cudafemproject_gb300.solver import FemContext
    ctx = FemContext(meshgen.square_2d(4))
    L = capi.lib()
    assert L.cfem_matvec_energy_noalloc(ctx._h, None, None, None) == capi.ERR_INVALID_ARGUMENT
    assert b"null argument" in L.cfem_last_error_string()
