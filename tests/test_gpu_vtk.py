"""Round trip of the legacy ASCII VTK writers (PostProcessingEngine.writeVTK
and writeVTKpsi, the reference's PostProcessing.py:70-156): a Shan-Chen
lattice is advanced on the GPU, written, and the file is read back.  The
grid must be NX x NY (NX+2 x NY+2 for psi, whose field carries a one-node
halo) with x fastest; the density (total_rho in the units C_rho), the
optional temperature, the velocity (in the units Cu) and psi must equal the
device fields to the 8 decimals the writer prints."""
import numpy as np
import pytest

from tests.cases import build_from_case, load_fixture, run_staged

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def read_vtk(path):
    """(dimensions, points, {name: array}) of a legacy ASCII structured grid."""
    lines = open(path).read().split("\n")
    assert lines[0] == "# vtk DataFile Version 3.0" and lines[2] == "ASCII"
    i = 3
    data, dims, pts = {}, None, None
    while i < len(lines):
        w = lines[i].split()
        if not w:
            i += 1
            continue
        if w[0] == "DIMENSIONS":
            dims = tuple(int(v) for v in w[1:])
        elif w[0] == "POINTS":
            n = int(w[1])
            pts = np.loadtxt(lines[i + 1:i + 1 + n])
            i += n
        elif w[0] == "POINT_DATA":
            npts = int(w[1])
        elif w[0] == "SCALARS":
            data[w[1]] = np.loadtxt(lines[i + 2:i + 2 + npts])
            i += 1 + npts
        elif w[0] == "VECTORS":
            data[w[1]] = np.loadtxt(lines[i + 1:i + 1 + npts])
            i += npts
        i += 1
    return dims, pts, data


def test_vtk_round_trip(tl, tmp_path):
    meta, arrays = load_fixture("sc_cs_bgk_f32")
    lb, me, coll, be, sc, bsc = build_from_case(tl, meta, arrays)
    run_staged(lb, me, coll, be, sc, bsc, meta["step_kind"], 10)
    nx, ny = lb.NX, lb.NY
    post = tl.PostProcessingEngine()
    dims, pts, data = read_vtk(post.writeVTK(str(tmp_path / "fields"), lb, Tflag=True))
    assert dims == (nx, ny, 1)
    xs, ys = np.meshgrid(np.arange(nx), np.arange(ny))
    assert np.array_equal(pts, np.column_stack((xs.ravel(), ys.ravel(), np.zeros(nx * ny))))
    rho = lb.total_rho.to_numpy() * lb.C_rho
    vel = lb.vel.to_numpy() * lb.Cu
    assert np.abs(data["density"] - rho.T.ravel()).max() <= 1e-8
    assert np.abs(data["T"] - lb.T.to_numpy().T.ravel()).max() <= 1e-8
    assert np.abs(data["velocity"][:, 0] - vel[:, :, 0].T.ravel()).max() <= 1e-8
    assert np.abs(data["velocity"][:, 1] - vel[:, :, 1].T.ravel()).max() <= 1e-8
    assert not data["velocity"][:, 2].any()
    dims, pts, data = read_vtk(post.writeVTKpsi(str(tmp_path / "psi"), lb))
    assert dims == (nx + 2, ny + 2, 1) and pts.shape == ((nx + 2) * (ny + 2), 3)
    psi = sc.psi_field.to_numpy()[:, :, 0]
    assert psi.shape == (nx + 2, ny + 2)
    assert np.abs(data["PSI"] - psi.T.ravel()).max() <= 1e-8
    assert np.ptp(data["PSI"]) > 0  # a real field, not a constant
