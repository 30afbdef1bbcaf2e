"""GPU result-file writers (include/scf_out.h) against the oracle's
restatement of Print_Result_Tecplot_PCent / _UCent / _VCent
(src/PrintResult.f90:39-168) and of Print_Result_VTK_2D's ParaView file
(:165-190, src/VTR_mod.f90), byte for byte, through the C-ABI."""
import numpy as np
import pytest

from simcoflow_gb300 import output as O

from test_out_oracle import edge_values, fields, real4_edges, vtr_fields

pytestmark = pytest.mark.gpu


def test_f24_14_matches_oracle(cuda, oracle):
    rng = np.random.default_rng(21)
    v = edge_values(rng, 200000)
    assert O.f24_14(v) == oracle.f24_14(v)


@pytest.mark.parametrize("nx,ny", [(7, 5), (37, 29), (300, 257)])
def test_pcell_text_matches_oracle(cuda, oracle, nx, ny):
    rng = np.random.default_rng(nx * 1000 + ny)
    f = fields(rng, nx, ny)
    # values on the format's edges inside the fields
    edges = edge_values(rng, 0)
    flat = f["phi"].ravel(order="F")  # a view of the Fortran-ordered array
    n = min(flat.size, edges.size)
    flat[:n] = edges[:n]
    assert O.text("p", nx, ny, f) == oracle.tecplot_pcell(nx, ny, f)


@pytest.mark.parametrize("comp", ["u", "v"])
def test_vcell_text_matches_oracle(cuda, oracle, comp):
    rng = np.random.default_rng(7)
    nx, ny = 65, 33
    f = fields(rng, nx, ny)
    f["vel"] = f[comp]
    assert O.text(comp, nx, ny, f) == oracle.tecplot_vcell(0 if comp == "u" else 1, nx, ny, f)


def test_device_pointers_and_file(cuda, oracle, tmp_path):
    """Device-resident fields, written to dir/Tecplot/Pressure_<iter>.dat in
    several 64 MiB chunks (2.2 M records)."""
    import torch
    rng = np.random.default_rng(9)
    nx, ny = 400, 380
    f = fields(rng, nx, ny)
    dev = {k: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
           for k, a in f.items()}
    (tmp_path / "Tecplot").mkdir()
    ms = O.write("p", nx, ny, dev, 1234, str(tmp_path) + "/", device_ptrs=True)
    data = (tmp_path / "Tecplot" / "Pressure_00001234.dat").read_bytes()
    assert data == oracle.tecplot_pcell(nx, ny, f)
    assert ms > 0.0


def test_missing_directory_is_an_io_error(cuda, tmp_path):
    from simcoflow_gb300 import projection as P
    rng = np.random.default_rng(2)
    f = fields(rng, 4, 4)
    f["vel"] = f["u"]
    with pytest.raises(P.ProjectionError) as e:
        O.write("u", 4, 4, f, 1, str(tmp_path / "nowhere") + "/")
    assert e.value.code == -9


def test_device_format_matches_records(cuda, oracle):
    """scf_tecplot_format: the records alone into a device buffer."""
    import torch
    rng = np.random.default_rng(11)
    nx, ny = 50, 41
    f = fields(rng, nx, ny)
    f["vel"] = f["v"]
    dev = {k: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
           for k, a in f.items()}
    out = torch.zeros(8 * nx * ny * 25, dtype=torch.uint8, device="cuda")
    O.format_device("v", nx, ny, dev, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    txt = oracle.tecplot_vcell(1, nx, ny, f)
    body = txt[txt.index(b"f=block\n") + len(b"f=block\n"):]
    assert bytes(out.cpu().numpy()) == body


def test_e15_8_matches_oracle(cuda, oracle):
    rng = np.random.default_rng(31)
    v = real4_edges(rng, 200000)
    # doubles just either side of float rounding boundaries
    f = rng.integers(0, 2**31, 100000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    f = f[np.isfinite(f)].astype(np.float64)
    half = np.abs(f) * 2.0**-25
    v = np.concatenate([v, f + half, f - half, f + half * (1 + 2.0**-20)])
    assert O.e15_8(v) == oracle.e15_8(v)


@pytest.mark.parametrize("nx,ny", [(1, 1), (7, 5), (37, 29), (301, 257)])
def test_vtr_text_matches_oracle(cuda, oracle, nx, ny):
    rng = np.random.default_rng(nx * 997 + ny)
    f = vtr_fields(rng, nx, ny)
    flat = f["phi"].ravel(order="F")  # a view of the Fortran-ordered array
    edges = real4_edges(rng, 0)
    n = min(flat.size, edges.size)
    flat[:n] = edges[:n]
    assert O.vtr_text(nx, ny, f) == oracle.vtr(nx, ny, f)


def test_vtr_device_pointers_and_file(cuda, oracle, tmp_path):
    """Device-resident fields, written to dir/Paraview/FlowField_<iter>.vtr in
    several 16 MiB chunks (3.3 M values)."""
    import torch
    rng = np.random.default_rng(19)
    nx, ny = 600, 550
    f = vtr_fields(rng, nx, ny)
    dev = {k: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
           for k, a in f.items()}
    (tmp_path / "Paraview").mkdir()
    ms = O.vtr_write(nx, ny, dev, 77, str(tmp_path) + "/", device_ptrs=True)
    data = (tmp_path / "Paraview" / "FlowField_00000077.vtr").read_bytes()
    assert data == oracle.vtr(nx, ny, f)
    assert len(data) == O.load().scf_vtr_size(nx, ny)
    assert ms > 0.0
