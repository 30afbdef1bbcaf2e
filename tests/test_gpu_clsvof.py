"""GPU level-set sweeps (include/scf_clsvof.h) against the oracle's literal
restatement of X_Sweep / Y_Sweep's level-set loops (src/Clsvof_Mod.f90:
1074-1123, 1191-1244), bit for bit, through the C-ABI."""
import numpy as np
import pytest

from simcoflow_gb300 import clsvof as CL

from gen.synth import ls_fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dir", [CL.X, CL.Y])
@pytest.mark.parametrize("nx,ny", [(3, 3), (4, 7), (37, 29), (300, 257)])
def test_ls_sweep_bit_exact(cuda, oracle, dir, nx, ny):
    rng = np.random.default_rng(7 * nx + ny + dir)
    f = ls_fields(rng, nx, ny)
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    want = oracle.ls_sweep(dir, nx, ny, f, 3e-3, t)
    got = t.copy(order="F")
    CL.sweep(dir, nx, ny, f, 3e-3, got)
    assert np.array_equal(got, want)


def test_ls_sweep_device_pointers_x_then_y(cuda, oracle):
    """Device-resident fields: an X sweep then a Y sweep on the same temls."""
    import torch
    rng = np.random.default_rng(5)
    nx, ny = 513, 255
    f = ls_fields(rng, nx, ny)
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    want = oracle.ls_sweep(1, nx, ny, f, 1e-3, oracle.ls_sweep(0, nx, ny, f, 1e-3, t))
    dev = {k: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
           for k, a in f.items()}
    tt = torch.from_numpy(np.ascontiguousarray(t.ravel(order="F"))).cuda()
    CL.sweep(CL.X, nx, ny, dev, 1e-3, tt, device_ptrs=True)
    CL.sweep(CL.Y, nx, ny, dev, 1e-3, tt, device_ptrs=True)
    got = tt.cpu().numpy().reshape((nx, ny), order="F")
    assert np.array_equal(got, want)


def test_ls_sweep_rejects_small_grids(cuda):
    from simcoflow_gb300 import projection as P
    rng = np.random.default_rng(1)
    f = ls_fields(rng, 2, 5)
    t = np.asfortranarray(np.zeros((2, 5)))
    with pytest.raises(P.ProjectionError):
        CL.sweep(CL.X, 2, 5, f, 1e-3, t)
