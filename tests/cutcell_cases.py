"""Seeded cut-cell inputs for the geometry tests: the three cell families'
grids (Mesh_Mod's P, U and V grids, src/Mesh_Mod.f90:120-175) and the solid
level-set fields that Initial_Clsvof leaves in them (circles; the level set
linearised at each cell centre, the solid fraction by frac,
src/Clsvof_Mod.f90:1371-1404)."""
import numpy as np


def frac_v(a, b, p, dx, dy):
    """frac on arrays, in the scalar restatement's operation order."""
    with np.errstate(all="ignore"):
        tnx, tny = np.abs(a), np.abs(b)
        h = 0.5 * (tnx * dx + tny * dy)
        xx = (0.5 * tny * dy - p) / dx / tnx + 0.5
        yy = (0.5 * tnx * dx - p) / dy / tny + 0.5
        top = np.where(yy > 1.0, ((yy - 1.0) / yy) ** 2.0, 0.0)
        right = np.where(xx > 1.0, ((xx - 1.0) / xx) ** 2.0, 0.0)
        gen = 0.5 * xx * yy * (1.0 - top - right)
        v = np.where(tny <= 1e-20, 0.5 - p / dx, gen)
        v = np.where(tnx <= 1e-20, 0.5 - p / dy, v)
        v = np.where(p - h >= 0.0, 0.0, v)
        v = np.where(p + h <= 0.0, 1.0, v)
    v = np.where(v < 1e-14, 0.0, v)
    return np.where(v >= 1.0 - 1e-14, 1.0, v)


def circles_levelset(circles, x, y):
    best = np.full(x.shape, 1e30), np.zeros(x.shape), np.ones(x.shape)
    for cx, cy, r in circles:
        dx, dy = x - cx, y - cy
        d = np.sqrt(dx * dx + dy * dy)
        ph, a, b = d - r, dx / d, dy / d
        m = ph < best[0]
        best = tuple(np.where(m, c, o) for c, o in zip((ph, a, b), best))
    return best


def family_grids(xf, yf):
    """P, U and V grids from the node coordinates (Mesh_Mod's formulas)."""
    F = np.asfortranarray
    nx, ny = len(xf) - 1, len(yf) - 1
    xc, yc = 0.5 * (xf[1:] + xf[:-1]), 0.5 * (yf[1:] + yf[:-1])
    dxc, dyc = xf[1:] - xf[:-1], yf[1:] - yf[:-1]
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    DX, DY = np.meshgrid(dxc, dyc, indexing="ij")
    p = {"x": F(X), "y": F(Y), "dx": F(DX), "dy": F(DY)}
    dxu = DX.copy()
    dxu[:-1, :] = X[1:, :] - X[:-1, :]
    u = {"x": F(X + 0.5 * DX), "y": F(Y.copy()), "dx": F(dxu), "dy": F(DY.copy())}
    dyv = DY.copy()
    dyv[:, :-1] = Y[:, 1:] - Y[:, :-1]
    v = {"x": F(X.copy()), "y": F(Y + 0.5 * DY), "dx": F(DX.copy()), "dy": F(dyv)}
    return {"p": p, "u": u, "v": v}


def family_fields(grids, circles):
    F = np.asfortranarray
    out = {}
    for f, g in grids.items():
        ph, a, b = circles_levelset(circles, g["x"], g["y"])
        out[f] = {"vofS": F(frac_v(a, b, ph, g["dx"], g["dy"])), "phiS": F(ph), "nxS": F(a),
                  "nyS": F(b)}
    return out


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
