"""Seeded cut-cell inputs for the geometry tests: the three cell families'
grids and solid level-set fields (gen.synth's builders) on
optionally stretched grids with circular bodies."""
import numpy as np

from gen.synth import circles_levelset, family_fields, family_grids, frac_v  # noqa: F401


def case(nx, ny, circles, stretch=0.0, seed=0):
    """Grids on [0,1]^2 (optionally randomly stretched) and the circles'
    solid fields."""
    rng = np.random.default_rng(seed)
    xf = np.linspace(0.0, 1.0, nx + 1)
    yf = np.linspace(0.0, 1.0, ny + 1)
    if stretch > 0.0:
        xf[1:-1] += rng.uniform(-stretch, stretch, nx - 1) / nx
        yf[1:-1] += rng.uniform(-stretch, stretch, ny - 1) / ny
    grids = family_grids(xf, yf)
    return grids, family_fields(grids, circles)


CIRCLES = [(0.4, 0.42, 0.17), (0.7, 0.5, 0.09), (0.2, 0.8, 0.061)]
