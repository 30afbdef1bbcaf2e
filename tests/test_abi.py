"""The C-ABI libraries load and export every symbol their headers declare
(no GPU needed: no compute call is made)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared(header, folder="include"):
    text = (ROOT / folder / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(scf_[a-z_0-9]+)\s*\(", text)))


def test_proj_library_exports_header_symbols(built):
    from simcoflow_gb300 import build
    lib = ctypes.CDLL(str(build.build_proj()))
    names = _declared("scf_proj.h")
    assert "scf_proj_update_puv" in names and "scf_proj_create" in names
    for n in names:
        assert hasattr(lib, n), n
    from simcoflow_gb300 import projection
    assert sorted(projection.EXPORTS) == sorted(n for n in names)


def test_proj_library_exports_unet_header_symbols(built):
    from simcoflow_gb300 import build, projection
    lib = ctypes.CDLL(str(build.build_proj()))
    names = _declared("scf_unet.h")
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(projection.UNET_EXPORTS) == names


def test_generator_library_exports_header_symbols(built):
    """The synthetic-input generator (gen/, not part of the product) and the
    oracle's copy of it, which the benchmark's CPU arm loads."""
    from gen import build as gen_build
    import build as oracle_build  # oracle/build.py
    for path in (gen_build.build(), oracle_build.geom_lib()):
        lib = ctypes.CDLL(str(path))
        for n in _declared("scf_geom.h", "gen"):
            assert hasattr(lib, n), n


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of scf_opts and scf_stats have the header's layout."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        import pytest
        pytest.skip("no C compiler")
    from simcoflow_gb300 import projection as P
    src = tmp_path / "lay.c"
    fields = [n for n, _ in P.Stats._fields_]
    ofields = [n for n, _ in P.Opts._fields_]
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "scf_proj.h"\n'
        "int main(void) {\n"
        '  printf("%zu %zu\\n", sizeof(scf_opts), sizeof(scf_stats));\n'
        + "".join(f'  printf("%zu\\n", offsetof(scf_stats, {n}));\n' for n in fields)
        + "".join(f'  printf("%zu\\n", offsetof(scf_opts, {n}));\n' for n in ofields)
        + "  return 0;\n}\n")
    exe = tmp_path / "lay"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(P.Opts)
    assert int(out[1]) == ctypes.sizeof(P.Stats)
    for n, off in zip(fields, out[2:2 + len(fields)]):
        assert int(off) == getattr(P.Stats, n).offset, n
    for n, off in zip(ofields, out[2 + len(fields):]):
        assert int(off) == getattr(P.Opts, n).offset, n


def test_host_only_entry_points(built):
    from simcoflow_gb300 import projection
    L = projection.load()
    assert L.scf_strerror(0) == b"ok"
    assert b"NaN" in L.scf_strerror(-3)
    o = projection.Opts()
    L.scf_opts_default(ctypes.byref(o))
    assert o.maxit == 200 and o.rtol == 1e-8 and o.coarse_max == 64
    # argument checks happen before any CUDA call
    h = ctypes.c_void_p()
    assert L.scf_proj_create(ctypes.byref(h), 1, 5, ctypes.byref(o)) == -1
    bad = projection.Opts()
    L.scf_opts_default(ctypes.byref(bad))
    bad.coarse_max = 1000
    assert L.scf_proj_create(ctypes.byref(h), 8, 8, ctypes.byref(bad)) == -1
    for field, value in (("coarse_sweeps", 9), ("coarse_sweeps", -1), ("coarse_from", -1)):
        bad = projection.Opts()
        L.scf_opts_default(ctypes.byref(bad))
        assert bad.coarse_sweeps == 0 and bad.coarse_from == 0
        setattr(bad, field, value)
        assert L.scf_proj_create(ctypes.byref(h), 8, 8, ctypes.byref(bad)) == -1, field
    assert L.scf_proj_set_coarse_sweeps(None, 1, 4) == -1
    assert L.scf_proj_destroy(None) == 0


def test_proj_library_exports_momentum_header_symbols(built):
    from simcoflow_gb300 import build, momentum
    lib = ctypes.CDLL(str(build.build_proj()))
    names = _declared("scf_mom.h")
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(momentum.EXPORTS) == names


def test_momentum_input_struct_layout(tmp_path):
    """The ctypes mirror of scf_mom_in has the header's layout."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        import pytest
        pytest.skip("no C compiler")
    from simcoflow_gb300 import momentum as M
    src = tmp_path / "lay.c"
    fields = [n for n, _ in M.MomIn._fields_]
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "scf_mom.h"\n'
        "int main(void) {\n"
        '  printf("%zu\\n", sizeof(scf_mom_in));\n'
        + "".join(f'  printf("%zu\\n", offsetof(scf_mom_in, {n}));\n' for n in fields)
        + "  return 0;\n}\n")
    exe = tmp_path / "lay"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(M.MomIn)
    for n, off in zip(fields, out[1:]):
        assert int(off) == getattr(M.MomIn, n).offset, n


def test_proj_library_exports_output_header_symbols(built):
    from simcoflow_gb300 import build, output
    lib = ctypes.CDLL(str(build.build_proj()))
    names = _declared("scf_out.h")
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(output.EXPORTS) == names


def test_output_field_struct_layouts(tmp_path):
    """The ctypes mirrors of scf_tecplot_pcell / _vcell and scf_vtr_fields
    have the header's layout."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        import pytest
        pytest.skip("no C compiler")
    from simcoflow_gb300 import output as O
    for cname, S in (("scf_tecplot_pcell", O.PCellFields), ("scf_tecplot_vcell", O.VCellFields),
                     ("scf_vtr_fields", O.VtrFields)):
        src = tmp_path / f"{cname}.c"
        fields = [n for n, _ in S._fields_]
        src.write_text(
            '#include <stdio.h>\n#include <stddef.h>\n#include "scf_out.h"\n'
            "int main(void) {\n"
            f'  printf("%zu\\n", sizeof({cname}));\n'
            + "".join(f'  printf("%zu\\n", offsetof({cname}, {n}));\n' for n in fields)
            + "  return 0;\n}\n")
        exe = tmp_path / cname
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
        assert int(out[0]) == ctypes.sizeof(S)
        for n, off in zip(fields, out[1:]):
            assert int(off) == getattr(S, n).offset, n


def test_tecplot_size_host_only(built):
    """scf_tecplot_size is host arithmetic: header plus 25 bytes per record."""
    from simcoflow_gb300 import output as O
    L = O.load()
    hdr_p = len(' title = "flow"\n') + len(
        ' variables ="x","y","p","u","v","phi","vof","phiS","vofS","vofA","Mres","FluxU",'
        '"FluxV","nxS","nyS"\n') + len(" zone i=   37,k=   29,f=block\n")
    assert L.scf_tecplot_size(O.PCELL, 37, 29) == hdr_p + 15 * 37 * 29 * 25
    assert L.scf_tecplot_size(O.UCELL, 37, 29) > 8 * 37 * 29 * 25
    assert L.scf_tecplot_size(7, 37, 29) == -1


def test_proj_library_exports_cutcell_header_symbols(built):
    from simcoflow_gb300 import build, cutcell
    lib = ctypes.CDLL(str(build.build_proj()))
    names = _declared("scf_cutcell.h")
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(cutcell.EXPORTS) == names


def test_cutcell_struct_layouts(tmp_path):
    """The ctypes mirrors of scf_cell_grid / _solid / _geom have the header's layout."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        import pytest
        pytest.skip("no C compiler")
    from simcoflow_gb300 import cutcell as CU
    for cname, S in (("scf_cell_grid", CU.CellGrid), ("scf_cell_solid", CU.CellSolid),
                     ("scf_cell_geom", CU.CellGeom)):
        src = tmp_path / f"{cname}.c"
        fields = [n for n, _ in S._fields_]
        src.write_text(
            '#include <stdio.h>\n#include <stddef.h>\n#include "scf_cutcell.h"\n'
            "int main(void) {\n"
            f'  printf("%zu\\n", sizeof({cname}));\n'
            + "".join(f'  printf("%zu\\n", offsetof({cname}, {n}));\n' for n in fields)
            + "  return 0;\n}\n")
        exe = tmp_path / cname
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
        assert int(out[0]) == ctypes.sizeof(S)
        for n, off in zip(fields, out[1:]):
            assert int(off) == getattr(S, n).offset, n


def test_vtr_size_host_only(built, oracle):
    """scf_vtr_size is host arithmetic, equal to the oracle file's length."""
    import numpy as np
    from simcoflow_gb300 import output as O
    from test_out_oracle import vtr_fields
    L = O.load()
    for nx, ny in ((1, 1), (5, 3), (64, 33)):
        f = vtr_fields(np.random.default_rng(nx), nx, ny)
        assert L.scf_vtr_size(nx, ny) == len(oracle.vtr(nx, ny, f))
    assert L.scf_vtr_size(0, 4) == -1


def test_proj_library_exports_clsvof_header_symbols(built):
    from simcoflow_gb300 import build, clsvof
    lib = ctypes.CDLL(str(build.build_proj()))
    names = _declared("scf_clsvof.h")
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(clsvof.EXPORTS) == names


@pytest.mark.parametrize("cname,pyname,rename", [
    ("scf_ls_fields", "LsFields", {}),
    ("scf_vof_fields", "VofFields", {"nxv": "nx", "nyv": "ny"}),
    ("scf_vof_wave", "VofWave", {}),
    ("scf_ir_fields", "IrFields", {}),
    ("scf_rd_fields", "RdFields", {"nxv": "nx", "nyv": "ny"}),
    ("scf_clsvof_fields", "StepFields", {})])
def test_clsvof_struct_layouts(tmp_path, cname, pyname, rename):
    """The ctypes mirrors of scf_ls_fields, scf_vof_fields and scf_vof_wave
    have the header's layouts."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    from simcoflow_gb300 import clsvof
    cls = getattr(clsvof, pyname)
    fields = [n for n, _ in cls._fields_]
    src = tmp_path / "ls.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "scf_clsvof.h"\n'
                   f'int main(void) {{\n  printf("%zu\\n", sizeof({cname}));\n'
                   + "".join(f'  printf("%zu\\n", offsetof({cname}, {rename.get(n, n)}));\n'
                             for n in fields) + "  return 0;\n}\n")
    exe = tmp_path / "ls"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(cls)
    for n, off in zip(fields, out[1:]):
        assert int(off) == getattr(cls, n).offset, n
