"""Shared helpers of the test suite."""
from pathlib import Path

import numpy as np

from gen import synth

GOLDEN = Path(__file__).resolve().parent / "golden"
GOLDEN_CASES = ("c1_n16", "box25x19")


def load_golden(name):
    """(Case, expected outputs) of a committed golden fixture."""
    z = np.load(GOLDEN / f"{name}.npz")
    arrays = {k: np.asfortranarray(z[k]) for k in z.files}
    c = synth.Case(name, int(z["nx"]), int(z["ny"]), arrays, float(z["betaP"]),
                   float(z["betaM"]), vb=float(z["vb"]), bc=tuple(int(b) for b in z["bc"]))
    return c, arrays


def rel_l2(a, b):
    d = np.linalg.norm(np.asarray(a) - np.asarray(b))
    n = np.linalg.norm(np.asarray(b))
    return d / n if n > 0 else d


def rel_l2_finite(a, b):
    """rel_l2 over the finite entries, after checking that both arrays have
    their non-finite entries in the same places.  The reference's top-row
    continuity divides by the north aperture of every top-row cell
    (src/ComputePUV_Mod.f90:177-182), which is 0 / 0 on a solid cell whose V
    cell is not solid enough to be zeroed afterwards (:227-245)."""
    a, b = np.asarray(a), np.asarray(b)
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite entries differ"
    return rel_l2(a[fa], b[fb])
