"""The oracle's restatement of the CLSVOF sweeps' level-set part
(oracle/clsvof_oracle.c) against a second, pure-Python transcription of the
same Fortran loops: X_Sweep (src/Clsvof_Mod.f90:1074-1123) and Y_Sweep
(:1191-1244), statement by statement, on small grids."""
import numpy as np
import pytest

from gen.synth import ls_fields


def py_sweep(dir, nx, ny, f, dtv, t):
    """The Fortran loops with 1-based indices (temls modified in place)."""
    t = t.copy(order="F")
    P = lambda i, j: f["phi"][i - 1, j - 1]
    D = lambda a, i, j: f[a][i - 1, j - 1]
    A = lambda a, i, j: f[a][i, j]
    if dir == 0:
        U = lambda i, j: f["ue"][i, j - 1]
        for j in range(1, ny + 1):
            for i in range(2, nx):
                if U(i, j) >= 0.0: l = (P(i + 1, j) + P(i - 1, j)) / 2.0
                elif i <= nx - 2: l = (P(i + 2, j) + P(i, j)) / 2.0
                else: l = (P(i + 1, j) + P(i - 1, j)) / 2.0
                fl = U(i, j) * l * dtv
                t[i - 1, j - 1] = t[i - 1, j - 1] - fl * A("aE", i, j) / D("dx", i, j)
                t[i, j - 1] = (t[i, j - 1] * (1.0 - D("vofS", i + 1, j)) +
                               fl * A("aW", i + 1, j) / D("dx", i + 1, j))
        for j in range(1, ny + 1):
            if U(1, j) >= 0.0:
                l = P(1, j) + D("dx", 1, j) / 2.0 * (1.0 - U(1, j) * dtv / D("dx", 1, j)) * \
                    (P(2, j) - P(1, j)) / (D("x", 2, j) - D("x", 1, j))
            else:
                l = P(2, j) - D("dx", 2, j) / 2.0 * (1.0 + U(1, j) * dtv / D("dx", 2, j)) * \
                    (P(3, j) - P(1, j)) / (2.0 * D("dx", 2, j))
            fl = l * U(1, j) * dtv
            t[0, j - 1] = t[0, j - 1] - fl * A("aE", 1, j) / D("dx", 1, j)
            t[1, j - 1] = t[1, j - 1] + fl * A("aE", 1, j) / D("dx", 2, j)
            t[0, j - 1] = t[0, j - 1] + P(1, j) * U(0, j) * dtv * A("aW", 1, j) / D("dx", 1, j)
            n = nx
            if U(n, j) > 0.0:
                l = P(n, j) + D("dx", n, j) / 2.0 * (1.0 - U(n, j) * dtv / D("dx", n, j)) * \
                    (P(n, j) - P(n - 1, j)) / (D("x", n, j) - D("x", n - 1, j))
            else:
                l = P(n, j) - D("dx", n - 1, j) / 2.0 * (1.0 + U(n, j) * dtv / D("dx", n - 1, j)) * \
                    (P(n, j) - P(n - 1, j)) / (D("x", n, j) - D("x", n - 1, j))
            fl = l * U(n, j) * dtv
            t[n - 1, j - 1] = t[n - 1, j - 1] - fl * A("aE", n, j) / D("dx", n, j)
    else:
        V = lambda i, j: f["ve"][i - 1, j]
        for j in range(2, ny):
            for i in range(1, nx + 1):
                if V(i, j) >= 0.0: l = (P(i, j + 1) + P(i, j - 1)) / 2.0
                elif j <= ny - 2: l = (P(i, j + 2) + P(i, j)) / 2.0
                else: l = (P(i, j + 1) + P(i, j - 1)) / 2.0
                fl = l * V(i, j) * dtv
                t[i - 1, j - 1] = t[i - 1, j - 1] - fl * A("aN", i, j) / D("dy", i, j)
                t[i - 1, j] = (t[i - 1, j] * (1.0 - D("vofS", i, j + 1)) +
                               fl * A("aS", i, j + 1) / D("dy", i, j + 1))
        for i in range(1, nx + 1):
            if V(i, 1) >= 0.0:
                l = P(i, 1) + D("dy", i, 1) / 2.0 * (1.0 - V(i, 1) * dtv / D("dy", i, 1)) * \
                    (P(i, 2) - P(i, 1)) / (D("y", i, 2) - D("y", i, 1))
            else:
                l = P(i, 2) - D("dy", i, 2) / 2.0 * (1.0 + V(i, 1) * dtv / D("dy", i, 2)) * \
                    (P(i, 3) - P(i, 1)) / (D("y", i, 3) - D("y", i, 1))
            fl = l * V(i, 1) * dtv
            t[i - 1, 0] = t[i - 1, 0] - fl * A("aN", i, 1) / D("dy", i, 1)
            t[i - 1, 1] = t[i - 1, 1] + fl * A("aN", i, 1) / D("dy", i, 2)
            t[i - 1, 0] = t[i - 1, 0] + P(i, 1) * V(i, 0) * dtv * A("aS", i, 1) / D("dy", i, 1)
            n = ny
            if V(i, n) > 0.0:
                l = P(i, n) + D("dy", i, n) / 2.0 * (1.0 - V(i, n) * dtv / D("dy", i, n)) * \
                    (P(i, n) - P(i, n - 1)) / (D("y", i, n) - D("y", i, n - 1))
            else:
                l = P(i, n) - D("dy", i, n - 1) / 2.0 * (1.0 + V(i, n) * dtv / D("dy", i, n - 1)) * \
                    (P(i, n) - P(i, n - 1)) / (D("y", i, n) - D("y", i, n - 1))
            fl = l * V(i, n) * dtv
            t[i - 1, n - 1] = t[i - 1, n - 1] - fl / D("dy", i, n)
    return t


@pytest.mark.parametrize("dir", [0, 1])
@pytest.mark.parametrize("nx,ny", [(3, 3), (4, 7), (9, 5)])
def test_ls_sweep_oracle_matches_transcription(oracle, dir, nx, ny):
    rng = np.random.default_rng(100 * nx + 10 * ny + dir)
    f = ls_fields(rng, nx, ny)
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    got = oracle.ls_sweep(dir, nx, ny, f, 1e-2, t)
    assert np.array_equal(got, py_sweep(dir, nx, ny, f, 1e-2, t))


def test_ls_sweep_at_rest_changes_nothing(oracle):
    """No velocity and no solid: the update leaves temls as it was."""
    rng = np.random.default_rng(3)
    nx, ny = 12, 10
    f = ls_fields(rng, nx, ny)
    f["ue"][:] = 0.0
    f["ve"][:] = 0.0
    f["vofS"][:] = 0.0
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    for d in (0, 1):
        assert np.array_equal(oracle.ls_sweep(d, nx, ny, f, 1e-2, t), t)
