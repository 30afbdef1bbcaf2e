"""Bounded device waits.  The reference stops on a failure with `pause`
(src/ProjectionP_Mod.f90:209-213); the library's device-side waits instead
give up after a bounded number of polls and the call returns
SCF_ERR_TIMEOUT, with the CUDA context still usable.  The test makes one CTA
of the TMA-staged sweep arm its barrier without issuing its copies (nothing
in flight, so the wait can only run out), with a short poll limit, through
the library's fault-injection entry point."""
import numpy as np
import pytest

from gen import synth
from simcoflow_gb300 import projection as P

pytestmark = pytest.mark.gpu

SCF_ERR_TIMEOUT = -6


def _solve(s, c):
    a = c.arrays
    u, v, p = a["u0"].copy(order="F"), a["v0"].copy(order="F"), a["p0"].copy(order="F")
    Pp, mres, st = s.update_puv(a["ustar"], a["vstar"], u, v, p, c.vb, check=False)
    return Pp, u, v, st


def test_tma_wait_runs_out_and_reports_timeout(cuda):
    c = synth.c4(n=256, instance=3)  # fine and next level use the TMA-staged sweep
    clean = P.project_case(c, precision="mixed", rtol=1e-10, maxit=200)
    assert clean["stats"]["status"] == 0
    s = P.ProjectionSolver(c.nx, c.ny, precision="mixed", rtol=1e-10, maxit=200)
    try:
        s.setup_case(c)
        P.inject_tma_timeout(3, 256)
        try:
            _, _, _, st = _solve(s, c)
        finally:
            P.inject_tma_timeout(-1, P.TMA_SPINS_DEFAULT)
        assert st.status == SCF_ERR_TIMEOUT
        assert st.iters < 3  # the first V-cycle's sweep stopped the loop
        # the same handle, re-assembled, solves cleanly and as before
        s.setup_case(c)
        Pp, u, v, st = _solve(s, c)
        assert st.status == 0
        assert np.array_equal(Pp, clean["Pp"])
        assert np.array_equal(u, clean["u"]) and np.array_equal(v, clean["v"])
    finally:
        s.close()
    # and a new handle too
    again = P.project_case(c, precision="mixed", rtol=1e-10, maxit=200)
    assert np.array_equal(again["Pp"], clean["Pp"])
