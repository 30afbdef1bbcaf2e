"""GPU CLSVOF sweeps (include/scf_clsvof.h) against the oracle's literal
restatement of X_Sweep / Y_Sweep after Interface_Reconstruct
(src/Clsvof_Mod.f90:989-1124, 1126-1245): the level-set loops and the VOF
loops with their PLIC face fluxes, bit for bit, through the C-ABI."""
import numpy as np
import pytest

from simcoflow_gb300 import clsvof as CL

from gen.synth import ls_fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dir", [CL.X, CL.Y])
@pytest.mark.parametrize("nx,ny", [(3, 3), (4, 7), (37, 29), (300, 257)])
def test_ls_sweep_bit_exact(cuda, oracle, dir, nx, ny):
    rng = np.random.default_rng(7 * nx + ny + dir)
    f = ls_fields(rng, nx, ny)
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    want = oracle.ls_sweep(dir, nx, ny, f, 3e-3, t)
    got = t.copy(order="F")
    CL.sweep(dir, nx, ny, f, 3e-3, got)
    assert np.array_equal(got, want)


def test_ls_sweep_device_pointers_x_then_y(cuda, oracle):
    """Device-resident fields: an X sweep then a Y sweep on the same temls."""
    import torch
    rng = np.random.default_rng(5)
    nx, ny = 513, 255
    f = ls_fields(rng, nx, ny)
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    want = oracle.ls_sweep(1, nx, ny, f, 1e-3, oracle.ls_sweep(0, nx, ny, f, 1e-3, t))
    dev = {k: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
           for k, a in f.items()}
    tt = torch.from_numpy(np.ascontiguousarray(t.ravel(order="F"))).cuda()
    CL.sweep(CL.X, nx, ny, dev, 1e-3, tt, device_ptrs=True)
    CL.sweep(CL.Y, nx, ny, dev, 1e-3, tt, device_ptrs=True)
    got = tt.cpu().numpy().reshape((nx, ny), order="F")
    assert np.array_equal(got, want)


def test_ls_sweep_rejects_small_grids(cuda):
    from simcoflow_gb300 import projection as P
    rng = np.random.default_rng(1)
    f = ls_fields(rng, 2, 5)
    t = np.asfortranarray(np.zeros((2, 5)))
    with pytest.raises(P.ProjectionError):
        CL.sweep(CL.X, 2, 5, f, 1e-3, t)


# ---------------------------------------------------------------------------
# Whole sweeps: the VOF part (src/Clsvof_Mod.f90:1004-1069, 1141-1189) with
# the PLIC face fluxes, and the fused VOF + level-set kernel
# ---------------------------------------------------------------------------
def _vof_case(seed, nx, ny):
    from gen.synth import vof_fields, wave_inlet
    rng = np.random.default_rng(seed)
    f = ls_fields(rng, nx, ny)
    v = vof_fields(rng, nx, ny, f)
    t = np.asfortranarray(v["vof"] + 0.1 * rng.standard_normal((nx, ny)))
    return f, v, t, wave_inlet(f)


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("dir", [CL.X, CL.Y])
@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 5), (3, 3), (37, 29), (300, 257)])
def test_vof_sweep_bit_exact(cuda, oracle, dir, nx, ny):
    f, v, t, wave = _vof_case(11 * nx + ny + dir, nx, ny)
    for w in (wave, None):
        want = oracle.vof_sweep(dir, nx, ny, f, v, 0.3, t, w)
        got = t.copy(order="F")
        CL.clsvof_sweep(dir, nx, ny, f, v, 0.3, got, wave=w)
        assert _same(got, want)


@pytest.mark.parametrize("dir", [CL.X, CL.Y])
def test_clsvof_sweep_fused_levelset_bit_exact(cuda, oracle, dir):
    """temvf and temls in one kernel: each equals its own literal loops."""
    nx, ny = 129, 67
    f, v, t, wave = _vof_case(40 + dir, nx, ny)
    tl = np.asfortranarray(np.random.default_rng(41).standard_normal((nx, ny)))
    want_v = oracle.vof_sweep(dir, nx, ny, f, v, 0.2, t, wave)
    want_l = oracle.ls_sweep(dir, nx, ny, f, 0.2, tl)
    got_v, got_l = t.copy(order="F"), tl.copy(order="F")
    CL.clsvof_sweep(dir, nx, ny, f, v, 0.2, got_v, temls=got_l, wave=wave)
    assert _same(got_v, want_v)
    assert np.array_equal(got_l, want_l)


def test_clsvof_sweeps_device_pointers_1024(cuda, oracle):
    """Device-resident fields at 1024x1024: an X sweep then a Y sweep on the
    same temvf / temls, as Coupled_LS_VOF's odd sub-steps order them."""
    import torch
    nx = ny = 1024
    f, v, t, wave = _vof_case(77, nx, ny)
    tl = np.asfortranarray(np.random.default_rng(78).standard_normal((nx, ny)))
    want_v = oracle.vof_sweep(1, nx, ny, f, v, 0.1, oracle.vof_sweep(0, nx, ny, f, v, 0.1, t, wave))
    want_l = oracle.ls_sweep(1, nx, ny, f, 0.1, oracle.ls_sweep(0, nx, ny, f, 0.1, tl))
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    df, dv = {k: T(a) for k, a in f.items()}, {k: T(a) for k, a in v.items()}
    tv, tt = T(t), T(tl)
    CL.clsvof_sweep(CL.X, nx, ny, df, dv, 0.1, tv, temls=tt, wave=wave, device_ptrs=True)
    CL.clsvof_sweep(CL.Y, nx, ny, df, dv, 0.1, tv, temls=tt, device_ptrs=True)
    back = lambda x: x.cpu().numpy().reshape((nx, ny), order="F")
    assert _same(back(tv), want_v)
    assert np.array_equal(back(tt), want_l)


def test_vof_sweep_conserves_each_line_2048(cuda):
    """Full size, no solid, open apertures, closed line ends: every row (X)
    and column (Y) keeps its liquid volume to rounding."""
    import torch
    nx = ny = 2048
    f, v, _, _ = _vof_case(9, nx, ny)
    f["vofS"][:] = 0.0
    for k in ("aE", "aW", "aN", "aS"):
        f[k][:] = 1.0
    f["ue"][0, :] = f["ue"][nx, :] = 0.0
    f["ve"][:, 0] = f["ve"][:, ny] = 0.0
    t = np.asfortranarray(v["vof"].copy())
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    df, dv = {k: T(a) for k, a in f.items() if k != "phi"}, {k: T(a) for k, a in v.items()}
    for d in (CL.X, CL.Y):
        tv = T(t)
        CL.clsvof_sweep(d, nx, ny, df, dv, 0.05, tv, device_ptrs=True)
        out = tv.cpu().numpy().reshape((nx, ny), order="F")
        h = f["dx"] if d == CL.X else f["dy"]
        assert np.allclose((out * h).sum(axis=d), (t * h).sum(axis=d), rtol=0, atol=1e-9)
        assert (np.abs(out - t) > 1e-6).mean() > 0.25


def test_clsvof_sweep_rejects_bad_arguments(cuda):
    from simcoflow_gb300 import projection as P
    f, v, t, _ = _vof_case(2, 2, 5)
    with pytest.raises(P.ProjectionError):  # the level-set part needs 3 cells a line
        CL.clsvof_sweep(CL.X, 2, 5, f, v, 1e-3, t.copy(order="F"), temls=t.copy(order="F"))
    with pytest.raises(P.ProjectionError):
        CL.clsvof_sweep(2, 2, 5, f, v, 1e-3, t.copy(order="F"))


# ---------------------------------------------------------------------------
# Interface_Reconstruct (src/Clsvof_Mod.f90:1250-1321)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("nx,ny,band", [(3, 3, 3.0), (4, 9, 3.0), (17, 12, 1e9), (64, 61, 3.0),
                                        (300, 257, 1e9)])
def test_interface_reconstruct_bit_exact(cuda, oracle, nx, ny, band):
    from gen.synth import reconstruct_fields
    f = reconstruct_fields(np.random.default_rng(nx * 7 + ny), nx, ny, band)
    want, ev = oracle.interface_reconstruct(nx, ny, f)
    got, ev2, _ = CL.interface_reconstruct(nx, ny, f)
    for k in ("nxv", "nyv", "dis"):
        assert _same(got[k], want[k]), k
    assert ev2 == ev


def test_interface_reconstruct_carried_values(cuda, oracle):
    """Every interface cell flagged (no solid, vof 0.4 everywhere): the
    boundary rows and columns read the normal component the previous cell
    left, and a column-1 chain runs the whole column."""
    from gen.synth import reconstruct_fields
    nx, ny = 40, 33
    f = reconstruct_fields(np.random.default_rng(8), nx, ny, band=1e9)
    f["vofS"][:] = 0.0
    f["vof"][:] = 0.4
    want, ev = oracle.interface_reconstruct(nx, ny, f)
    got, ev2, _ = CL.interface_reconstruct(nx, ny, f)
    for k in ("nxv", "nyv", "dis"):
        assert _same(got[k], want[k]), k


def test_interface_reconstruct_failed_brackets_carry_the_distance(cuda, oracle):
    """Three-phase cells whose liquid fraction exceeds the non-solid part have
    no Ridders bracket: the reference keeps diss from the cell before (loop
    order), possibly through a run of such cells."""
    from gen.synth import reconstruct_fields
    nx, ny = 48, 40
    f = reconstruct_fields(np.random.default_rng(21), nx, ny, band=1e9)
    cut = (f["vofS"] >= 0.05) & (f["vofS"] < 1 - 1e-3)
    f["vofS"][cut] = 2e-3  # the flag sees a small solid part, the polygon a larger one
    f["vof"][cut] = 0.99
    want, ev = oracle.interface_reconstruct(nx, ny, f)
    assert cut.sum() > 20
    got, ev2, _ = CL.interface_reconstruct(nx, ny, f)
    for k in ("nxv", "nyv", "dis"):
        assert _same(got[k], want[k]), k
    assert ev2 == ev


def test_interface_reconstruct_device_pointers_1024(cuda, oracle):
    import torch
    from gen.synth import reconstruct_fields
    nx = ny = 1024
    f = reconstruct_fields(np.random.default_rng(5), nx, ny, band=6.0)
    want, ev = oracle.interface_reconstruct(nx, ny, f)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    df = {k: T(a) for k, a in f.items()}
    out = {k: torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
           for k in ("nxv", "nyv", "dis")}
    CL.interface_reconstruct(nx, ny, df, out=out, device_ptrs=True)
    for k in ("nxv", "nyv", "dis"):
        assert _same(out[k].cpu().numpy().reshape((nx, ny), order="F"), want[k]), k


# ---------------------------------------------------------------------------
# Redistance (src/Clsvof_Mod.f90:1525-1708)
# ---------------------------------------------------------------------------
def _rd_case(seed, nx, ny, band):
    from gen.synth import reconstruct_fields
    import oracle as O
    f = reconstruct_fields(np.random.default_rng(seed), nx, ny, band)
    rec, _ = O.interface_reconstruct(nx, ny, f)
    g = dict(f)
    g.update(rec)
    return g


@pytest.mark.parametrize("nx,ny,band", [(1, 1, 3.0), (3, 3, 3.0), (9, 7, 1e9), (40, 37, 3.0),
                                        (300, 257, 3.0), (129, 65, 1e9)])
def test_redistance_bit_exact(cuda, oracle, nx, ny, band):
    g = _rd_case(nx * 5 + ny, nx, ny, band) if nx > 2 else None
    if g is None:  # a single cell: no neighbours
        g = _rd_case(3, 3, 3, band)
        g = {k: np.asfortranarray(a[:1, :1]) for k, a in g.items()}
    want, ev = oracle.redistance(nx, ny, g, g["phi"])
    got = g["phi"].copy(order="F")
    ev2, _ = CL.redistance(nx, ny, g, got)
    assert np.array_equal(got, want, equal_nan=True)
    assert ev2 == ev


def test_redistance_device_pointers_1024(cuda, oracle):
    import torch
    nx = ny = 1024
    g = _rd_case(6, nx, ny, 3.0)
    want, ev = oracle.redistance(nx, ny, g, g["phi"])
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    dg = {k: T(a) for k, a in g.items()}
    tp = T(g["phi"])
    CL.redistance(nx, ny, dg, tp, device_ptrs=True)
    assert np.array_equal(tp.cpu().numpy().reshape((nx, ny), order="F"), want, equal_nan=True)


# ---------------------------------------------------------------------------
# Coupled_LS_VOF with a fixed solid (src/Clsvof_Mod.f90:730-973)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("nx,ny,wave", [(3, 3, True), (9, 8, True), (64, 61, False),
                                        (300, 257, True)])
def test_clsvof_step_bit_exact(cuda, oracle, nx, ny, wave):
    from gen.synth import clsvof_step_fields
    f, vof, phi, dt, w = clsvof_step_fields(np.random.default_rng(nx + 2 * ny), nx, ny)
    w = w if wave else None
    want, ev = oracle.clsvof_step(nx, ny, f, dt, vof, phi, w)
    gv, gp = vof.copy(order="F"), phi.copy(order="F")
    out, ev2, _ = CL.clsvof_step(nx, ny, f, dt, gv, gp, wave=w)
    assert _same(gv, want["vof"])
    assert _same(gp, want["phi"])
    for k in ("nxv", "nyv", "dis"):
        assert _same(out[k], want[k]), k
    assert ev2 == ev


def test_clsvof_step_device_pointers_1024(cuda, oracle):
    import torch
    from gen.synth import clsvof_step_fields
    nx = ny = 1024
    f, vof, phi, dt, w = clsvof_step_fields(np.random.default_rng(17), nx, ny)
    want, ev = oracle.clsvof_step(nx, ny, f, dt, vof, phi, w)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    df = {k: T(a) for k, a in f.items()}
    tv, tp = T(vof), T(phi)
    out = {k: torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
           for k in ("nxv", "nyv", "dis")}
    CL.clsvof_step(nx, ny, df, dt, tv, tp, wave=w, out=out, device_ptrs=True)
    back = lambda a: a.cpu().numpy().reshape((nx, ny), order="F")
    assert _same(back(tv), want["vof"])
    assert _same(back(tp), want["phi"])
    for k in ("nxv", "nyv", "dis"):
        assert _same(back(out[k]), want[k]), k
