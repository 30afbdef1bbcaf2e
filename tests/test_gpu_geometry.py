"""GPU cut-cell geometry (scf_proj_set_solid) against the literal restatement
of Cell_Geo_Cal / DefineMomentumExchangeCell / NumberExternalCell and against
the CPU builder, bit for bit, and a projection on GPU-built geometry."""
import numpy as np
import pytest

from gen import geometry as G
from simcoflow_gb300 import projection as P
from gen import synth

pytestmark = pytest.mark.gpu

KEYS = ("aE", "aW", "aN", "aS", "WlLh", "vofS", "nyS", "vofS_u", "vofS_v", "posnu_p", "posnu_u",
        "posnu_v", "moex_u", "moex_v")


def frac_v(a, b, p, dx, dy):
    """frac (src/Clsvof_Mod.f90:1371-1404) on arrays, in the scalar
    restatement's operation order."""
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


def raw_fields(g, circles):
    """The solid fields Initial_Clsvof leaves in the P, U and V cells."""
    F = lambda a: np.asfortranarray(a)
    x, y, dx, dy = g["x"], g["y"], g["dx"], g["dy"]
    p, a, b = circles_levelset(circles, x, y)
    raw = {"vofS": F(frac_v(a, b, p, dx, dy)), "phiS": F(p), "nxS": F(a), "nyS": F(b)}
    pu, au, bu = circles_levelset(circles, x + 0.5 * dx, y)
    raw["vofS_u"] = F(frac_v(au, bu, pu, g["dxU"], dy))
    pv, av, bv = circles_levelset(circles, x, y + 0.5 * dy)
    raw["vofS_v"] = F(frac_v(av, bv, pv, dx, g["dyV"]))
    return raw


def gpu_geometry(g, raw, vof=None, phi=None, icorprob=True):
    nx, ny = g["dx"].shape
    s = P.ProjectionSolver(nx, ny)
    try:
        s.set_grid(g["dx"], g["dy"], g["dxU"], g["dyV"])
        z = np.zeros((nx, ny), order="F")
        s.set_solid(vof if vof is not None else z, phi if phi is not None else z, raw["vofS"],
                    raw["phiS"], raw["nxS"], raw["nyS"], raw["vofS_u"], raw["vofS_v"], icorprob)
        return s.get_geometry()
    finally:
        s.close()


def check_equal(got, exp, interior_only=()):
    for k in KEYS:
        a, b = got[k], np.asarray(exp[k])
        if k in interior_only:
            a, b = a[1:-1, 1:-1], b[1:-1, 1:-1]
        assert a.shape == b.shape and np.array_equal(a, b), k


@pytest.mark.parametrize("nx,ny", [(28, 22), (41, 37)])
def test_matches_literal_on_circles(cuda, oracle, nx, ny):
    xf, yf = G.axis(nx + 1, 0.0, 1.0), G.axis(ny + 1, 0.0, 1.0)
    circles = [(0.4, 0.42, 0.17), (0.7, 0.5, 0.09)]
    g = G.build(xf, yf, [G.Solid(G.SOLID_CIRCLE, cx, cy, r=r) for cx, cy, r in circles],
                G.Surface(0.55, [0.03], [2 * np.pi], [0.3]))
    raw = raw_fields(g, circles)
    got = gpu_geometry(g, raw)
    lit = oracle.geometry_literal(nx, ny, g["dx"], g["dy"], raw["vofS"], raw["phiS"],
                                  raw["nxS"], raw["nyS"], raw["vofS_u"], raw["vofS_v"])
    check_equal(got, lit)
    assert np.array_equal(got["nxS"], lit["nxS"])


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_matches_literal_on_random_slivers(cuda, oracle, seed):
    """Random level sets close to every cell: many cut and degenerate cells,
    chains of the order-dependent solid/degenerate rule included."""
    rng = np.random.default_rng(seed)
    nx, ny = 36, 30
    xf, yf = G.axis(nx + 1, 0.0, 1.0), G.axis(ny + 1, 0.0, 1.0)
    g = G.build(xf, yf, [], G.Surface(0.5, [0.0], [1.0], [0.0]))
    F = lambda a: np.asfortranarray(a)
    th = rng.uniform(0, 2 * np.pi, (nx, ny))
    a, b = np.cos(th), np.sin(th)
    p = rng.uniform(-0.6, 0.6, (nx, ny)) * g["dx"]
    raw = {"vofS": F(frac_v(a, b, p, g["dx"], g["dy"])), "phiS": F(p), "nxS": F(a), "nyS": F(b),
           "vofS_u": F(rng.choice([0.0, 0.3, 0.9995, 1.0], (nx, ny))),
           "vofS_v": F(rng.choice([0.0, 0.5, 0.9995, 1.0], (nx, ny)))}
    got = gpu_geometry(g, raw)
    lit = oracle.geometry_literal(nx, ny, g["dx"], g["dy"], raw["vofS"], raw["phiS"],
                                  raw["nxS"], raw["nyS"], raw["vofS_u"], raw["vofS_v"])
    check_equal(got, lit)
    solid = (raw["vofS"] > 1 - 1e-3)
    assert (lit["vofS"] == 1.0).sum() > solid.sum()  # the degenerate rule fired


def test_matches_cpu_builder_and_projection(cuda):
    """A 256^2 case: GPU-built geometry equals the CPU builder's, and the
    projection on it equals the projection on the uploaded geometry."""
    c = synth.c2(n=256)
    A = c.arrays
    circles = [(s.cx, s.cy, s.r) for s in c.meta["solids"]]
    g = {k: A[k] for k in ("x", "y", "dx", "dy", "dxU", "dyV")}
    raw = raw_fields(g, circles)
    got = gpu_geometry(g, raw)
    check_equal(got, A, interior_only=("aE", "aW", "aN", "aS", "posnu_p", "posnu_u", "posnu_v"))
    ref = P.project_case(c, rtol=1e-10, maxit=300)
    s = P.ProjectionSolver(c.nx, c.ny, rtol=1e-10, maxit=300)
    try:
        s.set_grid(A["dx"], A["dy"], A["dxU"], A["dyV"])
        s.set_solid(A["vof"], A["phi"], raw["vofS"], raw["phiS"], raw["nxS"], raw["nyS"],
                    raw["vofS_u"], raw["vofS_v"])
        s.assemble(A["DpU"], A["DpV"], c.betaP, c.betaM, c.bc)
        u, v, p = A["u0"].copy(order="F"), A["v0"].copy(order="F"), A["p0"].copy(order="F")
        Pp, mres, st = s.update_puv(A["ustar"], A["vstar"], u, v, p, c.vb)
    finally:
        s.close()
    for k, x in (("Pp", Pp), ("u", u), ("v", v), ("p", p), ("mres", mres)):
        assert np.array_equal(x, ref[k]), k
