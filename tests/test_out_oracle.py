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


# ---------------------------------------------------------------------------
# ParaView VTR file (Print_Result_VTK_2D, src/PrintResult.f90:165-190)
# ---------------------------------------------------------------------------
def py_e15_8(x: float) -> bytes:
    f = float(np.float32(x))
    if np.isnan(f):
        return b"NaN".rjust(15)
    if np.isinf(f):
        return (b"-Infinity" if f < 0 else b"Infinity").rjust(15)
    return ("%.8E" % f).encode().rjust(15)


def real4_edges(rng, n):
    """REAL(4) values on every case of the 15-character text: zero and its
    sign, subnormals, the extremes, powers of ten and two, exact decimal ties
    at the 10th significant digit (odd m / 8 with m in [8e6, 2^24)), doubles
    that round to the next float or overflow, special values, random bit
    patterns."""
    v = [0.0, -0.0, 1.0, -1.0, 0.1, -0.1, 1.5, 1e-45, -1e-45, 1.4e-45, 1.1754942e-38,
         1.17549435e-38, 3.4028235e38, -3.4028235e38, 3.5e38, -1e39, np.inf, -np.inf, np.nan,
         9.9999999e8, 999999999.0, 1e9, 1e10, 99999999.5, 1249999.875, 1249999.625]
    v += [10.0 ** k for k in range(-45, 39)] + [-(10.0 ** k) for k in range(-45, 39)]
    v += [2.0 ** k for k in range(-149, 128)]
    m = rng.integers(8_000_000, 2**24, n) | 1
    v += list(m / 8.0)
    with np.errstate(invalid="ignore"):  # signalling NaN patterns among the bits
        v += list(rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
                  .view(np.float32).astype(np.float64))
    v += list(rng.standard_normal(n) * 10.0 ** rng.integers(-40, 38, n))
    return np.array(v, dtype=np.float64)


def test_e15_8_matches_python_formatting(oracle):
    rng = np.random.default_rng(13)
    v = real4_edges(rng, 20000)
    got = oracle.e15_8(v)
    for k, x in enumerate(v):
        assert got[15 * k:15 * k + 15] == py_e15_8(float(x)), repr(x)


def test_e15_8_known_answers_and_round_trip(oracle):
    cases = {1.0: b" 1.00000000E+00", -0.0: b"-0.00000000E+00", 0.1: b" 1.00000001E-01",
             1249999.875: b" 1.24999988E+06", 1249999.625: b" 1.24999962E+06",
             1e-45: b" 1.40129846E-45", 3.4028235e38: b" 3.40282347E+38",
             1e39: b"       Infinity", np.nan: b"            NaN"}
    for x, want in cases.items():
        assert oracle.e15_8([x]) == want, x
    # nine significant digits give back the same REAL(4)
    rng = np.random.default_rng(14)
    v = rng.integers(0, 2**32, 50000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    v = v[np.isfinite(v)]
    txt = oracle.e15_8(v.astype(np.float64))
    back = np.array([float(txt[15 * k:15 * k + 15]) for k in range(v.size)], dtype=np.float32)
    assert np.array_equal(back.view(np.uint32), v.view(np.uint32))


def vtr_fields(rng, nx, ny):
    F = lambda a: np.asfortranarray(a)
    f = {k: F(rng.standard_normal((nx, ny))) for k in ("x", "y", "phi", "phiS")}
    f["vof"] = F(rng.uniform(0, 1, (nx, ny)))
    f["vofS"] = F(rng.choice([0.0, 0.25, 1.0], (nx, ny)))
    for k in ("p", "u", "v"):
        f[k] = F(rng.standard_normal((nx + 2, ny + 2)))
    return f


def test_vtr_file_layout(oracle):
    """The XML records of src/VTR_mod.f90 and every value list read back as
    the REAL(4) of the arrays Print_Result_VTK_2D passes."""
    import xml.etree.ElementTree as ET
    rng = np.random.default_rng(15)
    nx, ny = 7, 6
    f = vtr_fields(rng, nx, ny)
    txt = oracle.vtr(nx, ny, f)
    lines = txt.split(b"\n")
    assert lines[0] == b'<VTKFile type="RectilinearGrid" version="0.1" format="ascii">'
    assert lines[1] == b' <RectilinearGrid WholeExtent="1 7 1 6 1 1 ">'
    assert lines[2] == b'  <Piece Extent="1 7 1 6 1 1 ">'
    assert lines[-5:] == [b"     </PointData>", b"   </Piece>", b"  </RectilinearGrid>",
                          b"</VTKFile>", b""]
    vals = [ln for ln in lines if ln.startswith(b" ") and not ln.lstrip().startswith(b"<")]
    assert all(len(ln) <= 80 for ln in vals)
    root = ET.fromstring(txt)
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=np.float32)
              for a in root.iter("DataArray")}
    r4 = lambda a: np.asarray(a, dtype=np.float64).astype(np.float32)
    order = lambda a: r4(a).ravel(order="F")  # i fastest
    assert np.array_equal(arrays["X_COORDINATES"], r4(f["x"][:, 0]))
    assert np.array_equal(arrays["Y_COORDINATES"], r4(f["y"][0, :]))
    assert np.array_equal(arrays["Z_COORDINATES"], r4([0.0]))
    u, v = f["u"][1:-1, 1:-1], f["v"][1:-1, 1:-1]
    vel = np.stack([order(u), order(v), np.zeros(nx * ny, np.float32)], axis=1).ravel()
    assert np.array_equal(arrays["Velocity"], vel)
    assert np.array_equal(arrays["X_Velocity"], order(u))
    assert np.array_equal(arrays["Y_Velocity"], order(v))
    assert np.array_equal(arrays["Pressure"], order(f["p"][1:-1, 1:-1]))
    for name, key in (("Levelset", "phi"), ("SolidLvs", "phiS"), ("Vof", "vof"),
                      ("SolidVof", "vofS")):
        assert np.array_equal(arrays[name], order(f[key])), name
    assert list(arrays) == ["X_COORDINATES", "Y_COORDINATES", "Z_COORDINATES", "Velocity",
                            "X_Velocity", "Y_Velocity", "Pressure", "Levelset", "SolidLvs",
                            "Vof", "SolidVof"]
