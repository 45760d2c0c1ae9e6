"""GPU parity of batched independent meshes (cfem_create_batch): every
instance of one batched solve matches the FP64 oracle of that mesh alone and
its own single-mesh solve."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from conftest import rel
from cudafemproject_gb300 import capi, meshgen

pytestmark = pytest.mark.gpu


def _boxes():
    specs = [(3, 2e7, 0.25, 1e3), (5, 3e6, 0.38, 1e3), (4, 8e7, 0.21, 0.0), (6, 1e6, 0.3, 1e3), (2, 5e7, 0.33, 1e3)]
    return [meshgen.box_3d(n, n, 4 * n, jitter=0.2, seed=10 + i, E=E, nu=nu, traction=(0.0, -t, 0.0))
            for i, (n, E, nu, t) in enumerate(specs)]


@pytest.mark.parametrize("pe", [0, 64])
def test_batch_static_matches_single_meshes(pe):
    from cudafemproject_gb300.solver import BatchContext, FemContext
    probs = _boxes()
    b = BatchContext(probs, patch_elems=pe)
    us, infos = b.static_solve("fp32_refine", tol=1e-4, outer_tol=1e-12)
    for i, p in enumerate(probs):
        if i == 2:  # no load: converges at once to zero
            assert np.all(us[i] == 0.0) and infos[i]["status"] == 0
            continue
        xo, _ = O.Oracle(p, consistent=True).static(tol=1e-14, rule=1)
        assert rel(us[i], xo) <= 1e-8, i
        assert infos[i]["status"] == 0 and infos[i]["rel_residual"] < 1e-11
        u1, _ = FemContext(p, semantics="consistent", patch_elems=pe).static_solve(
            "fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
        assert rel(us[i], u1) <= 1e-9, i
    u32, inf32 = b.static_solve("fp32", tol=1e-6)
    xo, _ = O.Oracle(probs[1], consistent=True).static(tol=1e-14, rule=1)
    assert rel(u32[1], xo) <= 1e-4


def test_batch_context_rejects_single_mesh_calls():
    from cudafemproject_gb300.solver import BatchContext
    b = BatchContext(_boxes()[:2])
    nd = int(b.node_off[-1]) * 3
    x = np.ones(nd)
    y = np.zeros(nd)
    st = capi.lib().cfem_matvec(b._h, capi.FP64, x.ctypes.data, y.ctypes.data)
    assert st == capi.ERR_UNSUPPORTED
    with pytest.raises(capi.CfemError):
        b.static_solve("fp64")
