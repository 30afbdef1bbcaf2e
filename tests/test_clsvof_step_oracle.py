"""The oracle's Coupled_LS_VOF step (oracle/clsvof_oracle.c:
src/Clsvof_Mod.f90:730-973 with a fixed solid) against the same loop
written in Python over the pure-Python transcriptions of its parts
(X_Sweep / Y_Sweep, Interface_Reconstruct, Redistance), bit for bit; and
the step's liquid volume, which the split sweeps keep to rounding when the
drop stays clear of the boundary."""
import numpy as np
import pytest

from gen.synth import clsvof_step_fields
from test_clsvof_oracle import py_sweep, py_vof_sweep
from test_reconstruct_oracle import py_reconstruct
from test_redistance_oracle import py_redistance

VOFEPS, EPSI, TOLDENO = 1e-14, 1e-3, 1e-24


def _bc(v):
    v[:, 0] = v[:, 1]
    v[:, -1] = v[:, -2]
    v[0, :] = v[1, :]
    v[-1, :] = v[-2, :]


def py_step(nx, ny, f, dt, vof, phi, wave):
    vfl, ph = vof.copy(order="F"), phi.copy(order="F")
    dtv = dt / 6.0
    s = f["vofS"]
    UE = lambda i, j: f["ue"][i, j - 1]
    VE = lambda i, j: f["ve"][i - 1, j]
    A = lambda a, i, j: f[a][i, j]
    dx, dy = f["dx"], f["dy"]

    def rec():
        g = dict(f)
        g.update({"vof": vfl, "phi": ph})
        out, _ = py_reconstruct(nx, ny, g)
        return out

    def sweep(d, k, tv, tl):
        r = rec()
        v = {"vof": vfl, "nxv": r["nxv"], "nyv": r["nyv"], "dis": r["dis"], "nxs": f["nxs"],
             "nys": f["nys"], "phiS": f["phiS"]}
        w = None if (wave is None or d == 1) else list(wave[:5]) + [float(k)]
        g = dict(f)
        g["phi"] = ph
        return py_vof_sweep(d, nx, ny, g, v, dtv, tv, w), py_sweep(d, nx, ny, g, dtv, tl)

    def div(d, i, j):
        if d == 0:
            return UE(i, j) * A("aE", i, j) - UE(i - 1, j) * A("aW", i, j)
        return VE(i, j) * A("aN", i, j) - VE(i, j - 1) * A("aS", i, j)

    for k in range(1, 7):
        d1 = 0 if k % 2 == 1 else 1
        d2 = 1 - d1
        tv1, tl1 = sweep(d1, k, vfl.copy(order="F"), ph.copy(order="F"))
        h1 = dx if d1 == 0 else dy
        for i in range(1, nx + 1):
            for j in range(1, ny + 1):
                c = (i - 1, j - 1)
                den = (1.0 - s[c] + TOLDENO) - dtv / h1[c] * div(d1, i, j)
                tv1[c] = tv1[c] / den
                tl1[c] = tl1[c] / den
                vfl[c] = tv1[c] * (1.0 - s[c])
                ph[c] = tl1[c]
                if vfl[c] >= 1.0 - VOFEPS - s[c]: vfl[c] = 1.0 - s[c]
                if vfl[c] < VOFEPS: vfl[c] = 0.0
        _bc(vfl)
        _bc(ph)
        tv2, tl2 = sweep(d2, k, vfl.copy(order="F"), ph.copy(order="F"))
        h2 = dx if d2 == 0 else dy
        for i in range(1, nx + 1):
            for j in range(1, ny + 1):
                c = (i - 1, j - 1)
                dd = div(d2, i, j)
                tv2[c] = tv2[c] + dtv / h2[c] * tv1[c] * dd
                tl2[c] = tl2[c] + dtv / h2[c] * tl1[c] * dd
                vfl[c] = tv2[c]
                if s[c] < 1.0 - EPSI: ph[c] = tl2[c] / (1.0 - s[c])
        _bc(vfl)
        _bc(ph)
        r = rec()
        g = dict(f)
        g.update({"vof": vfl, **r})
        ph, _ = py_redistance(nx, ny, g, ph)
    return {"vof": vfl, "phi": ph, **r}


@pytest.mark.parametrize("nx,ny,wave", [(9, 8, True), (14, 11, False)])
def test_step_oracle_matches_transcription(oracle, nx, ny, wave):
    f, vof, phi, dt, w = clsvof_step_fields(np.random.default_rng(nx + ny), nx, ny)
    got, _ = oracle.clsvof_step(nx, ny, f, dt, vof, phi, w if wave else None)
    want = py_step(nx, ny, f, dt, vof, phi, w if wave else None)
    for k in ("vof", "phi", "nxv", "nyv", "dis"):
        assert np.array_equal(got[k], want[k], equal_nan=True), k


def test_step_keeps_the_liquid_volume(oracle):
    nx = ny = 96
    f, vof, phi, dt, _ = clsvof_step_fields(np.random.default_rng(3), nx, ny)
    out, ev = oracle.clsvof_step(nx, ny, f, dt, vof, phi, None)
    cell = f["dx"] * f["dy"]
    assert ev == 0
    assert abs((out["vof"] * cell).sum() - (vof * cell).sum()) < 1e-9 * (vof * cell).sum()
    assert np.abs(out["vof"] - vof).max() > 1e-3  # the drop moved
