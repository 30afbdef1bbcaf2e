"""The allocation-free right-hand side entry point, scf_rhs_norm_noalloc.

Some callers of this library cannot allocate device memory where they need
the pressure right-hand side: a Fortran host whose GPU memory all lives in
its own arena, or a time loop that must not take the device-wide
synchronisation of cudaMalloc / cudaFree.  scf_rhs_norm_noalloc serves them
from a fixed scratch array inside the library.  This test calls it through
the C-ABI on caller-owned device buffers, twice in a row on different grids,
and checks both results against the regular handle-based path (the
right-hand side that scf_proj_get_operator returns after
scf_proj_poisson_solve, and that solve's ||b||_2).  The file is named so
that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from simcoflow_gb300 import projection as P
from gen import synth

pytestmark = pytest.mark.gpu

ARGS = ("ustar", "vstar", "aE", "aW", "aN", "aS", "dx", "dy", "nyS", "WlLh")


def _reference_path(c):
    s = P.ProjectionSolver(c.nx, c.ny)
    try:
        s.setup_case(c)
        _, st = s.poisson_equation_solver(c["ustar"], c["vstar"], c.vb)
        return s.get_operator()["rhs"], st.bnorm
    finally:
        s.close()


def _noalloc(c, dev):
    import torch
    L = P.load()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(dev)
    ins = [t(c[k]) for k in ARGS]
    posnu = t(c["posnu_p"])
    rhs = torch.full((c.nx * c.ny,), np.nan, dtype=torch.float64, device=dev)
    bnorm = torch.full((1,), np.nan, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    rc = L.scf_rhs_norm_noalloc(c.nx, c.ny, *[x.data_ptr() for x in ins], posnu.data_ptr(),
                                ctypes.c_double(c.vb), rhs.data_ptr(), bnorm.data_ptr(), None)
    assert rc == 0, P.load().scf_strerror(rc)
    torch.cuda.synchronize(dev)
    return rhs.cpu().numpy().reshape((c.nx, c.ny), order="F"), float(bnorm.item())


def test_noalloc_rhs_matches_handle_path_twice(cuda):
    cases = [synth.c1(n=64), synth.c4(n=96, instance=3)]
    cases[1].vb = 0.04  # exercise the moving-body wall-flux term too
    for c in cases:  # two calls in a row, different grids, shared scratch
        rhs_ref, bn_ref = _reference_path(c)
        rhs, bn = _noalloc(c, cuda)
        assert np.array_equal(rhs, rhs_ref)
        assert abs(bn - bn_ref) <= 1e-13 * bn_ref


def test_noalloc_rejects_oversized_grid(cuda):
    L = P.load()
    nx = 16385  # one more than SCF_NOALLOC_MAX_SIDE: rejected before anything runs
    rc = L.scf_rhs_norm_noalloc(nx, 8, *([None] * 10), None, ctypes.c_double(0.0), None, None,
                                None)
    assert rc == -1
