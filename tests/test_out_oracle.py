"""The oracle's Tecplot restatement (oracle/out_oracle.c) on the CPU.

Pins the "(f24.14)" number format against Python's own correctly rounded
fixed-point formatting (round half to even on the exact binary value), and
the file layout against the records Print_Result_Tecplot_PCent / _UCent /
_VCent write (src/PrintResult.f90:39-168)."""
import numpy as np
import pytest

pytestmark = pytest.mark.filterwarnings("ignore::RuntimeWarning")


def py_f24_14(x: float) -> bytes:
    if np.isnan(x):
        return b"NaN".rjust(24)
    if np.isinf(x):
        return (b"-Infinity" if x < 0 else b"Infinity").rjust(24)
    s = ("%24.14f" % x).encode()
    return s if len(s) == 24 else b"*" * 24


def edge_values(rng, n):
    """Values around every case of the format: tiny, ties at the 15th
    decimal (odd multiples of 2^-15), carries into the integer part, the
    width limit, special values."""
    v = [0.0, -0.0, 1.0, -1.0, 0.5, 2.0**-15, 3 * 2.0**-15, -5 * 2.0**-15, 1e-15, -1e-15,
         0.99999999999999995, 9.999999999999999e8, 999999999.99999999, 99999999.999999994,
         -99999999.999999994, 1e9, -1e8, 123456789.12345678, -12345678.123456789,
         5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf, -np.inf,
         np.nan, 0.1, 0.2, 0.3, 1 / 3, 2 / 3, 4503599627370496.0, 2.0**52 - 0.5]
    v += list(rng.standard_normal(n))
    v += list(rng.standard_normal(n) * 10.0 ** rng.integers(-16, 10, n))
    v += list((rng.integers(-2**20, 2**20, n) * 2 + 1) * 2.0**-15)  # exact decimal ties
    v += list(rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64))
    return np.array(v, dtype=np.float64)


def test_f24_14_matches_python_formatting(oracle):
    rng = np.random.default_rng(3)
    v = edge_values(rng, 20000)
    got = oracle.f24_14(v)
    for k, x in enumerate(v):
        assert got[24 * k:24 * k + 24] == py_f24_14(float(x)), repr(x)


def test_f24_14_known_answers(oracle):
    cases = {0.5: b"        0.50000000000000", -0.0: b"       -0.00000000000000",
             -1e-20: b"       -0.00000000000000", 2.0**-15: b"        0.00003051757812",
             3 * 2.0**-15: b"        0.00009155273438", 1e9: b"*" * 24,
             -123.456: b"     -123.45600000000000", np.nan: b"                     NaN"}
    for x, want in cases.items():
        assert oracle.f24_14([x]) == want, x


def fields(rng, nx, ny):
    F = lambda a: np.asfortranarray(a)
    f = {k: F(rng.standard_normal((nx, ny))) for k in ("x", "y", "phi", "phiS", "mres", "nxS",
                                                      "nyS")}
    f["vof"] = F(rng.uniform(0, 1, (nx, ny)))
    f["vofS"] = F(rng.choice([0.0, 0.25, 1.0], (nx, ny)))
    for k in ("p", "u", "v"):
        f[k] = F(rng.standard_normal((nx + 2, ny + 2)))
    f["flux"] = F(rng.standard_normal((nx + 2, ny + 2, 2)))
    return f


def test_pcell_file_layout(oracle):
    rng = np.random.default_rng(5)
    nx, ny = 7, 5
    f = fields(rng, nx, ny)
    txt = oracle.tecplot_pcell(nx, ny, f)
    lines = txt.split(b"\n")
    assert lines[0] == b' title = "flow"'
    assert lines[1] == (b' variables ="x","y","p","u","v","phi","vof","phiS","vofS","vofA",'
                        b'"Mres","FluxU","FluxV","nxS","nyS"')
    assert lines[2] == b" zone i=    7,k=    5,f=block"
    recs = lines[3:-1]
    assert len(recs) == 15 * nx * ny and lines[-1] == b""
    blk = lambda b: [float(r) for r in recs[b * nx * ny:(b + 1) * nx * ny]]
    order = lambda a: [a[i, j] for j in range(ny) for i in range(nx)]  # i fastest
    np.testing.assert_allclose(blk(0), order(f["x"]), atol=1e-14)
    np.testing.assert_allclose(blk(2), order(f["p"][1:-1, 1:-1]), atol=1e-14)
    u = f["u"]
    np.testing.assert_allclose(blk(3), order(0.5 * (u[:-2, 1:-1] + u[1:-1, 1:-1])), atol=1e-14)
    v = f["v"]
    np.testing.assert_allclose(blk(4), order(0.5 * (v[1:-1, :-2] + v[1:-1, 1:-1])), atol=1e-14)
    np.testing.assert_allclose(blk(9), order(1.0 - f["vof"] - f["vofS"]), atol=1e-14)
    np.testing.assert_allclose(blk(11), order(f["flux"][1:-1, 1:-1, 0]), atol=1e-14)
    np.testing.assert_allclose(blk(12), order(f["flux"][1:-1, 1:-1, 1]), atol=1e-14)


def test_vcell_file_layout(oracle):
    rng = np.random.default_rng(6)
    nx, ny = 6, 4
    f = fields(rng, nx, ny)
    f["vel"] = f["u"]
    for comp, name in ((0, b'"u"'), (1, b'"v"')):
        txt = oracle.tecplot_vcell(comp, nx, ny, f)
        lines = txt.split(b"\n")
        assert lines[1] == b' variables ="x","y",' + name + b',"phi","vof","phiS","vofS","vofA"'
        assert len(lines) == 3 + 8 * nx * ny + 1
