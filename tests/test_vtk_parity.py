"""VTK output byte for byte against the reference engine's own writer.

tests/golden/vtk_ref.npz holds outputN.vtk files written by the compiled
engine (src/output.cpp:59-229) for three runs: the birth-death lattice, a
static lattice with deterministic chemistry (C[] and D[] fields), and the
moving dam break with species (velocities, densities and boundary volume
fractions that change).  Beside each file it holds the full-precision state
the engine wrote it from.  spatialpy_gb300.vtk formats that state; the text
must equal the engine's file exactly: %.10e points, %lf (6-decimal)
velocities and densities, 9 values per line, and output 0's FIELD count,
which leaves out the species arrays because the engine's RDME state is not
initialised when it is written (output.cpp:151-158).
"""
import numpy as np
import pytest

from spatialpy_gb300 import vtk

from .conftest import golden

CASES = ("bd", "chem", "dam")


@pytest.mark.parametrize("case", CASES)
def test_vtk_files_equal_reference_writer(case):
    g = golden("vtk_ref.npz")
    names = [str(x) for x in g[f"{case}/names"]]
    chem_on = bool(int(g[f"{case}/chem_on"]))
    k = 0
    while f"{case}/file{k}" in g:
        want = g[f"{case}/file{k}"].tobytes().decode()
        got = vtk.format_step(g[f"{case}/x"][k], g[f"{case}/type"], g[f"{case}/v"][k],
                              g[f"{case}/rho"][k], g[f"{case}/mass"], g[f"{case}/bvf_phi"][k],
                              g[f"{case}/nu"][k], names, g[f"{case}/counts"][k], k,
                              g[f"{case}/chem"][k] if chem_on else None)
        assert got == want, f"{case} output{k}: first difference at character " \
                            f"{next(i for i, (a, b) in enumerate(zip(got, want)) if a != b)}"
        k += 1
    assert k >= 2


def test_vtk_bounding_box_and_reader_round_trip(tmp_path):
    """The bounding-box file equals the engine's, and read_step recovers the
    written arrays of the moving case (to the printed precision)."""
    g = golden("vtk_ref.npz")
    x = g["dam/x"][0]
    bbox = (x[:, 0].min(), x[:, 0].max(), x[:, 1].min(), x[:, 1].max(), x[:, 2].min(),
            x[:, 2].max())
    n = x.shape[0]
    paths = vtk.write_outputs(tmp_path, g["dam/x"], g["dam/type"], g["dam/mass"], g["dam/rho"],
                              g["dam/nu"][0], ["S"], g["dam/counts"], v=g["dam/v"],
                              bbox=bbox)
    assert open(tmp_path / "output0_boundingBox.vtk", "rb").read() == g["dam/bbox"].tobytes()
    pts, arrays = vtk.read_step(paths[1])
    np.testing.assert_allclose(pts, g["dam/x"][1], rtol=1e-9)
    np.testing.assert_array_equal(arrays["D[S]"], g["dam/counts"][1][:, 0])
    assert arrays["rho"].shape == (n,)
