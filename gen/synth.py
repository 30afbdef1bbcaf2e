"""Seeded synthetic projection workloads.

The reference publishes no benchmark inputs; every workload here is built
from seeded random numbers with the shapes, sizes and value distributions of
the five configurations the projection is measured on:

  c1  128x128, one circle r=0.1 at (0.5,0.35), surface y=0.5+0.02 sin(2 pi x),
      8 velocity modes, dt=1e-3 (the CPU-runnable case)
  c2  2048x2048, three circles (centres U(0.15,0.85)^2, r U(0.04,0.1)),
      surface y=0.5+0.03 sin(4 pi x + theta), 32 modes, dt=5e-4
  c3  4096x4096 stretched in y (ratio 1.01 outside y in [0.45,0.55]), a
      0.3x0.02 plate rotated 10 degrees at (0.5,0.35), two-mode surface,
      64 modes plus a Gaussian vortex (strength 0.5, sigma 0.05), dt=2.5e-4
  c4  learned-preconditioner cases: 512^2 training, 1024^2 / 4096^2 evaluation;
      0-4 circles r U(0.03,0.12), amplitude U(0,0.05), wavenumber 1-6,
      density ratio log-uniform in [10,1000]
  c5  batch of 64 instances, sides 32*round(exp(U(ln 256, ln 1024))/32),
      density ratio log-uniform in [10,1000], 0-4 circles, 16 modes, dt=1e-3

Densities are water 1000 and air 1000/ratio (1.2 for ratio 1000:1.2); as in
src/ComputePUV_Mod.f90:42-43 with Roref = row (src/Main.f90:148),
betaP = 1 and betaM = rho_w/rho_a.  Dp = dt everywhere (the commented
alternative of src/PredictorUV_mod.f90:699).  Walls W/E/S are no-slip with
Neumann pressure; the top is open with Dirichlet p=0 (BC flags 1,1,1,0 as in
src/ProjectionP_Mod.f90:55).  Seeds are 1000*config + instance.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import geometry as G

RHO_W = 1000.0


@dataclass
class Case:
    name: str
    nx: int
    ny: int
    arrays: dict
    betaP: float
    betaM: float
    vb: float = 0.0
    dt: float = 1e-3
    bc: tuple = (1, 1, 1, 0)
    rtol: float = 1e-8
    meta: dict = field(default_factory=dict)

    def __getitem__(self, k):
        return self.arrays[k]


def _rng(config: int, instance: int, seed=None) -> np.random.Generator:
    s = 1000 * config + instance if seed is None else seed
    return np.random.Generator(np.random.PCG64(s))


def _modes(rng, K, kmax=4):
    a = rng.normal(0.0, 0.1, K)
    kx = rng.integers(1, kmax + 1, K)
    ky = rng.integers(1, kmax + 1, K)
    th = rng.uniform(0.0, 2.0 * np.pi, K)
    return a, kx, ky, th


def _field(xs: np.ndarray, ys: np.ndarray, modes) -> np.ndarray:
    """sum_k a_k sin(2 pi (kx x + ky y) + th_k) on the tensor grid xs x ys,
    Fortran order (len(xs), len(ys)), as one matrix product."""
    a, kx, ky, th = modes
    ax = 2.0 * np.pi * np.outer(xs, kx) + th
    by = 2.0 * np.pi * np.outer(ys, ky)
    A = np.concatenate([a * np.sin(ax), a * np.cos(ax)], axis=1)
    B = np.concatenate([np.cos(by), np.sin(by)], axis=1)
    return np.asfortranarray(A @ B.T)


def _velocities(g, modes_u, modes_v, vortex=None):
    """u* at U faces (xf[i], y_j), i = 0..nx; v* at V faces (x_i, yf[j]), j = 0..ny;
    (0:nx+1,0:ny+1) arrays with no-slip W/E/S walls and zero ghosts."""
    xf, yf = g["xf"], g["yf"]
    nx, ny = len(xf) - 1, len(yf) - 1
    xc = 0.5 * (xf[1:] + xf[:-1])
    yc = 0.5 * (yf[1:] + yf[:-1])
    xu = np.concatenate([xf, [xf[-1]]])          # i = 0..nx+1 (ghost reuses the wall)
    yu = np.concatenate([[yc[0]], yc, [yc[-1]]])  # j = 0..ny+1
    xv = np.concatenate([[xc[0]], xc, [xc[-1]]])
    yv = np.concatenate([yf, [yf[-1]]])
    u = _field(xu, yu, modes_u)
    v = _field(xv, yv, modes_v)
    if vortex is not None:
        gam, sig, x0, y0 = vortex
        X, Y = np.meshgrid(xu, yu, indexing="ij")
        r2 = (X - x0) ** 2 + (Y - y0) ** 2 + 1e-300
        u += np.asfortranarray(-gam / (2 * np.pi) * (Y - y0) / r2 * (1 - np.exp(-r2 / sig**2)))
        X, Y = np.meshgrid(xv, yv, indexing="ij")
        r2 = (X - x0) ** 2 + (Y - y0) ** 2 + 1e-300
        v += np.asfortranarray(gam / (2 * np.pi) * (X - x0) / r2 * (1 - np.exp(-r2 / sig**2)))
    # ghosts and walls
    u[:, 0] = 0.0; u[:, ny + 1] = 0.0; u[nx + 1, :] = 0.0
    u[0, :] = 0.0; u[nx, :] = 0.0
    v[0, :] = 0.0; v[nx + 1, :] = 0.0; v[:, ny + 1] = 0.0
    v[:, 0] = 0.0
    return np.asfortranarray(u), np.asfortranarray(v)


def build_case(name, xf, yf, solids, surface, modes_u, modes_v, dt, ratio, vortex=None,
               vb=0.0, rtol=1e-8, meta=None) -> Case:
    g = G.build(xf, yf, solids, surface)
    nx, ny = len(xf) - 1, len(yf) - 1
    us, vs = _velocities(g, modes_u, modes_v, vortex)
    arrays = {k: g[k] for k in ("dx", "dy", "dxU", "dyV", "vof", "phi", "vofS", "nyS", "WlLh",
                                "aE", "aW", "aN", "aS", "posnu_p", "posnu_u", "moex_u",
                                "vofS_u", "posnu_v", "moex_v", "vofS_v", "x", "y", "phiS",
                                "nxS", "vofS_in", "nxS_in", "nyS_in", "vofS_u_in",
                                "vofS_v_in")}
    arrays["DpU"] = np.full((nx + 2, ny + 2), dt, order="F")
    arrays["DpV"] = np.full((nx + 2, ny + 2), dt, order="F")
    arrays["ustar"], arrays["vstar"] = us, vs
    arrays["u0"], arrays["v0"] = us.copy(order="F"), vs.copy(order="F")
    arrays["p0"] = np.zeros((nx + 2, ny + 2), order="F")
    m = {"n_unknowns": g["n_unknowns"], "solids": solids, "surface": surface,
         "xf": g["xf"], "yf": g["yf"]}
    if meta:
        m.update(meta)
    return Case(name, nx, ny, arrays, betaP=1.0, betaM=float(ratio), vb=vb, dt=dt, rtol=rtol,
                meta=m)


def _circles(rng, n, rlo, rhi):
    out = []
    for _ in range(n):
        cx, cy = rng.uniform(0.15, 0.85, 2)
        out.append(G.Solid(G.SOLID_CIRCLE, float(cx), float(cy), r=float(rng.uniform(rlo, rhi))))
    return out


def c1(n: int = 128, instance: int = 0, seed=None) -> Case:
    rng = _rng(1, instance, seed)
    xf = G.axis(n + 1, 0.0, 1.0)
    yf = G.axis(n + 1, 0.0, 1.0)
    solids = [G.Solid(G.SOLID_CIRCLE, 0.5, 0.35, r=0.1)]
    surf = G.Surface(0.5, [0.02], [2 * np.pi], [0.0])
    mu, mv = _modes(rng, 8), _modes(rng, 8)
    return build_case("c1", xf, yf, solids, surf, mu, mv, 1e-3, RHO_W / 1.2, rtol=1e-10)


def c2(n: int = 2048, instance: int = 0, seed=None) -> Case:
    rng = _rng(2, instance, seed)
    xf = G.axis(n + 1, 0.0, 1.0)
    yf = G.axis(n + 1, 0.0, 1.0)
    solids = _circles(rng, 3, 0.04, 0.1)
    surf = G.Surface(0.5, [0.03], [4 * np.pi], [float(rng.uniform(0, 2 * np.pi))])
    mu, mv = _modes(rng, 32), _modes(rng, 32)
    return build_case("c2", xf, yf, solids, surf, mu, mv, 5e-4, RHO_W / 1.2)


def c3(n: int = 4096, instance: int = 0, seed=None) -> Case:
    rng = _rng(3, instance, seed)
    xf = G.axis(n + 1, 0.0, 1.0)
    # uniform band [0.45, 0.55] holding n - 2*round(n*496/4096) cells, geometric
    # growth (Newton ratio ~1.01 at n=4096) outside, as Initial_Grid with
    # NonUniformMesh=1
    nout = int(round(n * 496 / 4096))
    nrec = n + 1 - 2 * nout
    yf = G.axis(n + 1, 0.0, 1.0, True, 0.45, 0.55, nrec)
    solids = [G.Solid(G.SOLID_BOX, 0.5, 0.35, hw=0.15, hh=0.01, angle=np.deg2rad(10.0))]
    th = rng.uniform(0, 2 * np.pi, 2)
    surf = G.Surface(0.5, [0.02, 0.01], [2 * np.pi, 6 * np.pi], [float(th[0]), float(th[1])])
    mu, mv = _modes(rng, 64), _modes(rng, 64)
    return build_case("c3", xf, yf, solids, surf, mu, mv, 2.5e-4, RHO_W / 1.2,
                      vortex=(0.5, 0.05, 0.5, 0.5))


def random_instance(config: int, n: int, instance: int, nmodes: int = 16, dt: float = 1e-3,
                    seed=None) -> Case:
    """c4 / c5 style instance: 0-4 circles, sinusoidal surface, log-uniform density ratio."""
    rng = _rng(config, instance, seed)
    xf = G.axis(n + 1, 0.0, 1.0)
    yf = G.axis(n + 1, 0.0, 1.0)
    ncirc = int(rng.integers(0, 5))
    solids = _circles(rng, ncirc, 0.03, 0.12)
    amp = float(rng.uniform(0.0, 0.05))
    kw = int(rng.integers(1, 7))
    surf = G.Surface(0.5, [amp], [2 * np.pi * kw], [float(rng.uniform(0, 2 * np.pi))])
    ratio = float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))
    mu, mv = _modes(rng, nmodes), _modes(rng, nmodes)
    return build_case(f"c{config}", xf, yf, solids, surf, mu, mv, dt, ratio,
                      meta={"ratio": ratio, "ncirc": ncirc})


def walls(n: int = 128, instance: int = 0, seed=None, ny: int | None = None) -> Case:
    """Parity workload whose solids cut the first and last rows and the
    first and last columns: circles centred on or just inside the W, S, N
    and E walls, a two-mode surface crossing many faces.  The reference
    averages the two cells' apertures of a face only for i, j = 2..N-1
    (src/Cutcell_Mod.f90:161-204), so on these rows and columns the W / S
    entry of a row and the E / N entry of its neighbour differ (by a few
    per cent here): the assembled matrix is not symmetric."""
    rng = _rng(6, instance, seed)
    ny = n if ny is None else ny
    xf = G.axis(n + 1, 0.0, 1.0)
    yf = G.axis(ny + 1, 0.0, 1.0)
    solids = [G.Solid(G.SOLID_CIRCLE, 0.02, 0.3, r=0.08), G.Solid(G.SOLID_CIRCLE, 0.6, 0.01, r=0.06),
              G.Solid(G.SOLID_CIRCLE, 0.3, 0.99, r=0.05), G.Solid(G.SOLID_CIRCLE, 0.985, 0.7, r=0.05)]
    surf = G.Surface(0.5, [0.03, 0.01], [4 * np.pi, 10 * np.pi],
                     [float(rng.uniform(0, 2 * np.pi)), float(rng.uniform(0, 2 * np.pi))])
    mu, mv = _modes(rng, 16), _modes(rng, 16)
    return build_case("walls", xf, yf, solids, surf, mu, mv, 1e-3, RHO_W / 1.2, vb=0.0)


def c4(n: int = 512, instance: int = 0, seed=None) -> Case:
    return random_instance(4, n, instance, seed=seed)


def c5_sides(count: int = 64, seed=None) -> list[int]:
    rng = _rng(5, 9999, seed)
    s = np.exp(rng.uniform(np.log(256.0), np.log(1024.0), count))
    return [int(32 * round(v / 32.0)) for v in s]


def c5(instance: int = 0, n: int | None = None, seed=None) -> Case:
    side = n if n is not None else c5_sides()[instance]
    return random_instance(5, side, instance, nmodes=16, dt=1e-3, seed=seed)


CONFIGS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4, "c5": c5, "walls": walls}


def make_case(name: str, **kw) -> Case:
    return CONFIGS[name](**kw)


# ---------------------------------------------------------------------------
# Momentum-predictor solves (one velocity component each): the inputs of
# SetMatrix / SetVectors (src/PredictorUV_mod.f90:622-846) on the U or V
# cells of a projection case.  The face fluxes are computed upstream by the
# predictor's flux routines, which are not on this path: here they are
# seeded fields of the same shapes and magnitudes -- diffusive conductances
# nu_mix/nu_ref/Re * (face length / centre distance) * open face fraction
# with the mixture viscosity of the cells' liquid fraction, skew ("ED")
# fluxes of a fraction of that only in cut cells, smooth convective-flux
# divergence and pressure-gradient fields, upwind weights Eta in [0.3, 0.7].
# ---------------------------------------------------------------------------
NU_W, NU_A = 1.0034e-6, 1.506e-5   # src/StateVariables.f90:26-27
BETA_VIS = 0.5                       # src/StateVariables.f90:28


def momentum_inputs(case: Case, comp: str, rey: float = 1.0e5, seed: int = 0) -> dict:
    """Inputs of one component's implicit solve ('u' or 'v') for `case`.
    Array layouts are the reference's (Fortran order): (nx,ny) for grid and
    cell fields, (nx+2,ny+2) for Posnu/EtaE/EtaN/velocities/Dp/Pred,
    (nx+1,ny) for the east-west face fluxes and (nx,ny+1) for north-south."""
    if comp not in ("u", "v"):
        raise ValueError("comp must be 'u' or 'v'")
    A = case.arrays
    nx, ny = case.nx, case.ny
    iu, iv = (1, 0) if comp == "u" else (0, 1)
    rng = _rng(7, seed + (0 if comp == "u" else 1))
    F = lambda a: np.asfortranarray(a)
    vofP, wlP = A["vof"], A["WlLh"]
    if comp == "u":
        dxc, dyc = A["dxU"], A["dy"]
        vof = vofP.copy(order="F")
        vof[:-1, :] = 0.5 * (vofP[:-1, :] + vofP[1:, :])
        wl = wlP.copy(order="F")
        wl[:-1, :] = 0.5 * (wlP[:-1, :] + wlP[1:, :])
        vofS, posnu = A["vofS_u"], A["posnu_u"]
    else:
        dxc, dyc = A["dx"], A["dyV"]
        vof = vofP.copy(order="F")
        vof[:, :-1] = 0.5 * (vofP[:, :-1] + vofP[:, 1:])
        wl = wlP.copy(order="F")
        wl[:, :-1] = 0.5 * (wlP[:, :-1] + wlP[:, 1:])
        vofS, posnu = A["vofS_v"], A["posnu_v"]
    vof = np.asfortranarray(np.minimum(vof, 1.0 - vofS))  # liquid within the open part
    vf = np.clip(vof / np.maximum(1.0 - vofS, 1e-3), 0.0, 1.0)
    visc = ((1.0 - vf) * NU_A / NU_W + vf * NU_W / NU_W) / rey   # nu_mix / nu_ref / Re
    cut = (vofS > 0.0) & (vofS < 1.0)
    # east-west faces i = 1..nx+1 (face i is the west face of cell i)
    vE = np.empty((nx + 1, ny)); vE[1:-1] = 0.5 * (visc[1:] + visc[:-1])
    vE[0], vE[-1] = visc[0], visc[-1]
    gE = np.empty((nx + 1, ny)); gE[1:-1] = dyc[1:] / (0.5 * (dxc[1:] + dxc[:-1]))
    gE[0], gE[-1] = dyc[0] / dxc[0], dyc[-1] / dxc[-1]
    vN = np.empty((nx, ny + 1)); vN[:, 1:-1] = 0.5 * (visc[:, 1:] + visc[:, :-1])
    vN[:, 0], vN[:, -1] = visc[:, 0], visc[:, -1]
    gN = np.empty((nx, ny + 1)); gN[:, 1:-1] = dxc[:, 1:] / (0.5 * (dyc[:, 1:] + dyc[:, :-1]))
    gN[:, 0], gN[:, -1] = dxc[:, 0] / dyc[:, 0], dxc[:, -1] / dyc[:, -1]
    # open fraction of each face (the lesser of its two cells' open fractions)
    op = 1.0 - vofS
    aE = np.empty((nx + 1, ny)); aE[1:-1] = np.minimum(op[1:], op[:-1])
    aE[0], aE[-1] = op[0], op[-1]
    aN = np.empty((nx, ny + 1)); aN[:, 1:-1] = np.minimum(op[:, 1:], op[:, :-1])
    aN[:, 0], aN[:, -1] = op[:, 0], op[:, -1]
    difEW, difNS = F(vE * gE * aE), F(vN * gN * aN)
    cutE = np.zeros((nx + 1, ny), bool); cutE[1:] |= cut; cutE[:-1] |= cut
    cutN = np.zeros((nx, ny + 1), bool); cutN[:, 1:] |= cut; cutN[:, :-1] |= cut
    edEW = F(np.where(cutE, rng.uniform(-0.3, 0.3, (nx + 1, ny)) * difEW, 0.0))
    edNS = F(np.where(cutN, rng.uniform(-0.3, 0.3, (nx, ny + 1)) * difNS, 0.0))
    xs, ys = np.linspace(0, 1, nx + 2), np.linspace(0, 1, ny + 2)
    eta_e = F(0.5 + 0.2 * _field(xs, ys, _modes(rng, 4)) / 0.4)
    eta_n = F(0.5 + 0.2 * _field(xs, ys, _modes(rng, 4)) / 0.4)
    eta_e, eta_n = F(np.clip(eta_e, 0.3, 0.7)), F(np.clip(eta_n, 0.3, 0.7))
    area = dxc * dyc
    xc, yc = np.linspace(0, 1, nx), np.linspace(0, 1, ny)
    flux = F(_field(xc, yc, _modes(rng, 8)) * area)
    gradp = F(_field(xc, yc, _modes(rng, 8)) * area * 10.0)
    vel = A["u0"] if comp == "u" else A["v0"]
    return {"comp": comp, "iu": iu, "iv": iv, "nx": nx, "ny": ny,
            "dx": F(dxc), "dy": F(dyc), "posnu": posnu, "vof": F(vof), "vofS": vofS,
            "etaE": eta_e, "etaN": eta_n, "WlLh": F(wl), "delh": F(0.5 * dxc),
            "difEW": difEW, "difNS": difNS, "edEW": edEW, "edNS": edNS,
            "flux": flux, "gradp": gradp, "u": A["u0"], "v": A["v0"],
            "pred": vel.copy(order="F"),
            "Dp": (A["DpU"] if comp == "u" else A["DpV"]).copy(order="F"),
            "dt": case.dt, "beta_vis": BETA_VIS, "nua": NU_A, "nuw": NU_W, "nuref": NU_W,
            "rey": rey, "fr": 1.0 / np.sqrt(9.81)}


# ---------------------------------------------------------------------------
# Inputs of the three cell families' cut-cell geometry (scf_grid_preprocess)
# ---------------------------------------------------------------------------
def frac_v(a, b, p, dx, dy):
    """frac (src/Clsvof_Mod.f90:1371-1404) on arrays: the solid fraction of
    a cell under the linear level set a x + b y + p."""
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
    """Distance to the nearest circle and its outward normal at (x, y)."""
    best = np.full(x.shape, 1e30), np.zeros(x.shape), np.ones(x.shape)
    for cx, cy, r in circles:
        dx, dy = x - cx, y - cy
        d = np.sqrt(dx * dx + dy * dy)
        ph, a, b = d - r, dx / d, dy / d
        m = ph < best[0]
        best = tuple(np.where(m, c, o) for c, o in zip((ph, a, b), best))
    return best


def family_grids(xf, yf):
    """P, U and V grids (x, y, dx, dy; (nx,ny), Fortran order) from the node
    coordinates, by Mesh_Mod's formulas (src/Mesh_Mod.f90:120-175)."""
    F = np.asfortranarray
    xf, yf = np.asarray(xf, dtype=float), np.asarray(yf, dtype=float)
    xc, yc = 0.5 * (xf[1:] + xf[:-1]), 0.5 * (yf[1:] + yf[:-1])
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    DX, DY = np.meshgrid(xf[1:] - xf[:-1], yf[1:] - yf[:-1], indexing="ij")
    p = {"x": F(X), "y": F(Y), "dx": F(DX), "dy": F(DY)}
    dxu = DX.copy()
    dxu[:-1, :] = X[1:, :] - X[:-1, :]
    u = {"x": F(X + 0.5 * DX), "y": F(Y.copy()), "dx": F(dxu), "dy": F(DY.copy())}
    dyv = DY.copy()
    dyv[:, :-1] = Y[:, 1:] - Y[:, :-1]
    v = {"x": F(X.copy()), "y": F(Y + 0.5 * DY), "dx": F(DX.copy()), "dy": F(dyv)}
    return {"p": p, "u": u, "v": v}


def family_fields(grids, circles):
    """The solid level-set fields (vofS, phiS, nxS, nyS) of each family for
    circular bodies: the level set linearised at the cell centre, the solid
    fraction by frac."""
    F = np.asfortranarray
    out = {}
    for f, g in grids.items():
        ph, a, b = circles_levelset(circles, g["x"], g["y"])
        out[f] = {"vofS": F(frac_v(a, b, ph, g["dx"], g["dy"])), "phiS": F(ph), "nxS": F(a),
                  "nyS": F(b)}
    return out


def cutcell_inputs(case: Case):
    """(grids, fields) of the three cell families for a case with circular
    bodies (c1, c2, c4, c5 and random instances)."""
    circles = []
    for s in case.meta["solids"]:
        if s.kind != G.SOLID_CIRCLE:
            raise ValueError("cutcell_inputs: circular bodies only")
        circles.append((s.cx, s.cy, s.r))
    grids = family_grids(case.meta["xf"], case.meta["yf"])
    return grids, family_fields(grids, circles)


# ---------------------------------------------------------------------------
# Inputs of the CLSVOF sweeps' level-set transport (scf_ls_sweep)
# ---------------------------------------------------------------------------
def ls_fields(rng, nx, ny):
    """Random inputs of one CLSVOF level-set sweep (scf_ls_sweep) on an nx x ny
    grid: level set, solid fractions, spacings and centres, face apertures
    (some closed), face velocities ue (nx+1,ny) and ve (nx,ny+1)."""
    F = np.asfortranarray
    x = np.cumsum(rng.uniform(0.5, 1.5, nx))
    y = np.cumsum(rng.uniform(0.5, 1.5, ny))
    gx = np.gradient(x) if nx > 1 else np.diff(x, prepend=0.0)
    gy = np.gradient(y) if ny > 1 else np.diff(y, prepend=0.0)
    dx = F(np.broadcast_to(gx[:, None], (nx, ny)).copy())
    dy = F(np.broadcast_to(gy[None, :], (nx, ny)).copy())
    f = {"phi": F(rng.standard_normal((nx, ny))),
         "vofS": F(rng.choice([0.0, 0.0, 0.3, 1.0], (nx, ny))),
         "dx": dx, "dy": dy,
         "x": F(np.broadcast_to(x[:, None], (nx, ny)).copy()),
         "y": F(np.broadcast_to(y[None, :], (nx, ny)).copy())}
    for k in ("aE", "aW", "aN", "aS"):
        f[k] = F(rng.choice([0.0, 0.5, 1.0], (nx + 2, ny + 2)) * rng.uniform(0.5, 1, (nx + 2, ny + 2)))
    f["ue"] = F(rng.standard_normal((nx + 1, ny)))
    f["ve"] = F(rng.standard_normal((nx, ny + 1)))
    return f


# ---------------------------------------------------------------------------
# Inputs of the CLSVOF sweeps' VOF transport (scf_clsvof_sweep)
# ---------------------------------------------------------------------------
def vof_fields(rng, nx, ny, f):
    """Random VOF inputs of one CLSVOF sweep on the grid of ls_fields' f:
    liquid fractions (empty, full, slightly outside [0,1] and interface
    cells), the interface normal and distance that Interface_Reconstruct
    leaves, the solid normal and distance, and solid fractions spread over
    every branch of the face-flux routines (none, below 1e-3, cut, nearly
    and fully solid).  Some apertures are set to exactly 1 and some face
    velocities to 0.  Updates f's vofS, apertures and velocities in place
    and returns the VOF fields."""
    F = np.asfortranarray
    shape = (nx, ny)
    kind = rng.integers(0, 8, shape)
    vof = rng.uniform(0.02, 0.98, shape)
    vof[kind == 0] = 0.0
    vof[kind == 1] = 1.0
    vof[kind == 2] = rng.choice([5e-15, -1e-16, 1.0 - 5e-15, 1.0 + 1e-15], int((kind == 2).sum()))
    f["vofS"][:] = F(rng.choice([0.0, 0.0, 0.0, 5e-4, 0.25, 0.6, 0.9995, 1.0], shape))
    th = rng.uniform(0.0, 2.0 * np.pi, shape)
    nxv, nyv = np.cos(th), np.sin(th)
    axis = rng.integers(0, 6, shape)
    nxv[axis == 0], nyv[axis == 0] = 0.0, 1.0
    nxv[axis == 1], nyv[axis == 1] = -1.0, 0.0
    h = np.hypot(f["dx"], f["dy"])
    ths = rng.uniform(0.0, 2.0 * np.pi, shape)
    for k in ("aE", "aW", "aN", "aS"):
        a = f[k]
        a[rng.random(a.shape) < 0.3] = 1.0
    f["ue"][rng.random(f["ue"].shape) < 0.1] = 0.0
    f["ve"][rng.random(f["ve"].shape) < 0.1] = 0.0
    return {"vof": F(vof), "nxv": F(nxv), "nyv": F(nyv),
            "dis": F(rng.uniform(-0.6, 0.6, shape) * h),
            "nxs": F(np.cos(ths)), "nys": F(np.sin(ths)),
            "phiS": F(rng.uniform(-0.5, 0.5, shape) * h)}


def wave_inlet(f):
    """X_Sweep's wave-inlet constants {Amp0, kw, omew, Depthw, NondiT, k}
    with the still-water level inside the grid's first column."""
    y = f["y"][0]
    span = max(y[-1] - y[0], float(f["dy"][0, 0]))
    return np.array([0.05 * span, 2.0 * np.pi / span, 0.7, 0.5 * (y[0] + y[-1]), 1.25, 3.0])


def reconstruct_fields(rng, nx, ny, band=3.0):
    """Random inputs of Interface_Reconstruct on an nx x ny stretched grid:
    a liquid circle's level set (a signed distance, with noise on a third
    of the cells so that both branches of the normal's one-sided tests
    occur), liquid fractions (empty, full, interface values, the edge
    values around 1e-14; interface values within band cells of the circle),
    and a solid half-plane through its centre with its normal, distance and
    solid fractions (the half-plane's, and 5e-4 on a few cells)."""
    F = np.asfortranarray
    xs = np.cumsum(rng.uniform(0.5, 1.5, nx))
    ys = np.cumsum(rng.uniform(0.5, 1.5, ny))
    x = F(np.broadcast_to(xs[:, None], (nx, ny)).copy())
    y = F(np.broadcast_to(ys[None, :], (nx, ny)).copy())
    gx = np.gradient(xs) if nx > 1 else np.ones(1)
    gy = np.gradient(ys) if ny > 1 else np.ones(1)
    dx = F(np.broadcast_to(gx[:, None], (nx, ny)).copy())
    dy = F(np.broadcast_to(gy[None, :], (nx, ny)).copy())
    cx, cy = rng.uniform(0.3, 0.7) * xs[-1], rng.uniform(0.3, 0.7) * ys[-1]
    r = 0.3 * min(xs[-1], ys[-1])
    phi = np.hypot(x - cx, y - cy) - r
    noisy = rng.random((nx, ny)) < 0.33
    phi = np.where(noisy, phi * rng.uniform(0.5, 1.5, (nx, ny)), phi)
    h = np.maximum(dx, dy)
    th = rng.uniform(0.0, 2.0 * np.pi)
    nxs, nys = np.cos(th), np.sin(th)
    c = -(nxs * cx + nys * cy)
    phis = nxs * x + nys * y + c
    vofs = frac_v(nxs, nys, phis, dx, dy)  # the solid part, nxs x + nys y + phis < 0
    vofs[rng.random((nx, ny)) < 0.02] = 5e-4
    fluid = 1.0 - vofs
    vof = np.where(phi < -band * h, fluid,
                   np.where(phi > band * h, 0.0, rng.uniform(0.02, 0.98, (nx, ny)) * fluid))
    edge = rng.random((nx, ny)) < 0.05
    vof[edge] = rng.choice([0.0, 1e-14, 2e-14, 1.0 - 2e-14, 1.0], int(edge.sum()))
    vof = np.minimum(vof, fluid)
    return {"x": x, "y": y, "dx": dx, "dy": dy, "phi": F(phi), "vof": F(vof), "vofS": F(vofs),
            "nxs": F(np.full((nx, ny), nxs)), "nys": F(np.full((nx, ny), nys)),
            "phiS": F(phis)}


def clsvof_step_fields(rng, nx, ny, cfl=0.2):
    """Inputs of one Coupled_LS_VOF step on an nx x ny stretched grid: a
    liquid drop (level set = distance to a circle, liquid fractions from its
    local tangent line) beside a solid half-plane (its fractions, normal and
    distance; face apertures the open part of each face), in a solid-body
    rotation about the drop's centre with the faces inside the solid closed;
    dt gives the sub-steps (dt/6) a Courant number cfl.  Returns
    (fields, vof, phi, dt, wave)."""
    F = np.asfortranarray
    xs = np.cumsum(rng.uniform(0.8, 1.2, nx))
    ys = np.cumsum(rng.uniform(0.8, 1.2, ny))
    gx, gy = np.gradient(xs), np.gradient(ys)
    x = F(np.broadcast_to(xs[:, None], (nx, ny)).copy())
    y = F(np.broadcast_to(ys[None, :], (nx, ny)).copy())
    dx = F(np.broadcast_to(gx[:, None], (nx, ny)).copy())
    dy = F(np.broadcast_to(gy[None, :], (nx, ny)).copy())
    cx, cy = 0.45 * xs[-1], 0.5 * ys[-1]
    r = 0.25 * min(xs[-1], ys[-1])
    phi = np.hypot(x - cx, y - cy) - r
    with np.errstate(all="ignore"):
        nrm = np.hypot(x - cx, y - cy)
        gnx, gny = (x - cx) / nrm, (y - cy) / nrm
    th = rng.uniform(-0.3, 0.3) + np.pi  # solid on the right
    nxs, nys = np.cos(th), np.sin(th)
    c = -(nxs * (cx + 1.1 * r) + nys * cy)
    phis = nxs * x + nys * y + c
    vofs = frac_v(nxs, nys, phis, dx, dy)
    vof = np.minimum(frac_v(gnx, gny, phi, dx, dy), 1.0 - vofs)
    # face apertures: the part of each face with nxs x + nys y + c >= 0
    def open_part(x0, y0, x1, y1):
        f0, f1 = nxs * x0 + nys * y0 + c, nxs * x1 + nys * y1 + c
        with np.errstate(all="ignore"):
            t = np.where(f0 == f1, 0.5, f0 / (f0 - f1))
        return np.where((f0 >= 0) & (f1 >= 0), 1.0, np.where((f0 < 0) & (f1 < 0), 0.0,
                        np.where(f0 >= 0, t, 1.0 - t)))
    aE = np.ones((nx + 2, ny + 2)); aW = np.ones((nx + 2, ny + 2))
    aN = np.ones((nx + 2, ny + 2)); aS = np.ones((nx + 2, ny + 2))
    aE[1:-1, 1:-1] = open_part(x + dx / 2, y - dy / 2, x + dx / 2, y + dy / 2)
    aW[1:-1, 1:-1] = open_part(x - dx / 2, y - dy / 2, x - dx / 2, y + dy / 2)
    aN[1:-1, 1:-1] = open_part(x - dx / 2, y + dy / 2, x + dx / 2, y + dy / 2)
    aS[1:-1, 1:-1] = open_part(x - dx / 2, y - dy / 2, x + dx / 2, y - dy / 2)
    # rotation about the drop's centre, closed faces inside the solid
    xe = np.concatenate([[xs[0] - gx[0] / 2], xs + gx / 2])
    yn = np.concatenate([[ys[0] - gy[0] / 2], ys + gy / 2])
    om = 1.0
    ue = -(ys[None, :] - cy) * om * np.ones((nx + 1, 1))
    ve = (xs[:, None] - cx) * om * np.ones((1, ny + 1))
    ue[1:, :] *= (aE[1:-1, 1:-1] > 0)
    ve[:, 1:] *= (aN[1:-1, 1:-1] > 0)
    umax = max(np.abs(ue).max(), np.abs(ve).max())
    dt = 6.0 * cfl * min(gx.min(), gy.min()) / umax
    fields = {"vofS": F(vofs), "nxs": F(np.full((nx, ny), nxs)), "nys": F(np.full((nx, ny), nys)),
              "phiS": F(phis), "x": x, "y": y, "dx": dx, "dy": dy, "aE": F(aE), "aW": F(aW),
              "aN": F(aN), "aS": F(aS), "ue": F(ue), "ve": F(ve)}
    wave = np.array([0.05 * ys[-1], 2.0 * np.pi / xs[-1], 0.5, 0.3 * ys[-1], 0.0])
    del xe, yn
    return fields, F(vof), F(phi), dt, wave
