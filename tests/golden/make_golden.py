"""Generate the golden fixtures of the projection path.

The reference ships no golden vectors and cannot be built here, so these
fixtures pin the oracle (oracle/scf_oracle.c + SuperLU) on small seeded
cases: inputs in the reference's Fortran layouts and the oracle's outputs.
They guard the oracle against drift across machines and edits, and the GPU
tests compare against them.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402
from gen import geometry as G  # noqa: E402
from gen import synth  # noqa: E402

INPUTS = ("dx", "dy", "dxU", "dyV", "vof", "phi", "vofS", "nyS", "WlLh", "aE", "aW", "aN", "aS",
          "posnu_p", "posnu_u", "moex_u", "vofS_u", "posnu_v", "moex_v", "vofS_v", "DpU", "DpV",
          "ustar", "vstar", "u0", "v0", "p0")


def cases():
    yield "c1_n16", synth.c1(n=16)
    # stretched grid, rotated plate, moving body (vb != 0), odd sizes
    rng = np.random.Generator(np.random.PCG64(77))
    xf = G.axis(26, 0.0, 1.0)
    yf = G.axis(20, 0.0, 1.0, True, 0.45, 0.55, 7)
    solids = [G.Solid(G.SOLID_BOX, 0.5, 0.33, hw=0.2, hh=0.06, angle=np.deg2rad(10.0))]
    surf = G.Surface(0.52, [0.03, 0.01], [2 * np.pi, 6 * np.pi], [0.4, 1.3])
    mu, mv = synth._modes(rng, 6), synth._modes(rng, 6)
    c = synth.build_case("box25x19", xf, yf, solids, surf, mu, mv, 2.5e-4, 1000.0 / 1.2, vb=0.05)
    yield "box25x19", c


def main():
    for name, c in cases():
        r = O.project(c)
        out = {k: c.arrays[k] for k in INPUTS}
        out.update({"nx": c.nx, "ny": c.ny, "betaP": c.betaP, "betaM": c.betaM, "vb": c.vb,
                    "bc": np.array(c.bc), "pocoef": r["pocoef"], "matr": r["matr"],
                    "rhm": r["rhm"], "Pp": r["Pp"], "u": r["u"], "v": r["v"], "p": r["p"],
                    "mres": r["mres"]})
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, c.nx, c.ny, "relres", r["relres"], "row_residual", r["row_residual"])


if __name__ == "__main__":
    main()
