"""Batched uneven projections (one graph launch): every instance equals its
own single-instance projection bit for bit, and matches the oracle."""
import numpy as np
import pytest

from helpers import rel_l2
from gen import synth

pytestmark = pytest.mark.gpu


def _cases():
    sides = [64, 96, 160, 128, 96, 192]
    return [synth.c5(instance=i, n=n) for i, n in enumerate(sides)]


def test_batch_equals_single_instance_and_oracle(cuda, oracle):
    from simcoflow_gb300 import batch as B
    from simcoflow_gb300 import projection as P
    cases = _cases()
    bp = B.BatchProjector(cases, precision="mixed", rtol=1e-12, maxit=300, tune=True)
    try:
        stats, ms = bp.run()
        assert ms > 0
        for i, (c, st) in enumerate(zip(cases, stats)):
            assert st["status"] == 0 and st["relres_true"] < 1e-11, (i, st)
            got = bp.result(i)
            # the same handle through the single-instance entry point
            inst = bp.insts[i]
            inst.solve_once()
            single = bp.result(i)
            for k in ("Pp", "u", "v", "p", "mres"):
                assert np.array_equal(got[k], single[k]), (i, k)
            if i < 2:
                exp = oracle.project(c)
                assert rel_l2(got["Pp"], exp["Pp"]) <= 1e-8
                assert rel_l2(got["u"], exp["u"]) <= 1e-9
        # a second launch of the same graph gives the same answers
        stats2, _ = bp.run()
        assert [s["iters"] for s in stats2] == [s["iters"] for s in stats]
        # the autotuner chose a schedule, a sweep tile and a coarse-level
        # schedule for every size class
        for cls, entry in bp.table.items():
            assert len(entry) == 5 and entry[3] in B.TILES and entry[4] in B.COARSE, (cls, entry)
    finally:
        bp.close()


def test_batch_rejects_host_pointer_handles(cuda):
    import ctypes as C
    from simcoflow_gb300 import projection as P
    c = synth.c1(n=32)
    s = P.ProjectionSolver(c.nx, c.ny)
    try:
        s.setup_case(c)
        h = (C.c_void_p * 1)(s._h.value)
        b = C.c_void_p()
        assert P.load().scf_batch_create(C.byref(b), h, 1) == -1
    finally:
        s.close()
