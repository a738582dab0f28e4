"""SU2 mesh input (ocsl_mesh_read_su2): the finite-volume arrays the
reference builds from the same file (Read_SU2_mesh, Cgeometry,
CFVM::create_FVM_from_geometry), recorded in tests/golden/mesh_<cells>.npz
and flow_box3d.npz.

* The numbering is the reference's exactly: interior faces (left / right
  cells), boundary faces (their cells, marker by marker), and the matrix
  pattern built from them equals the reference's CSR.
* The metrics (area vectors, alpha, distances, unit vectors, geometric
  weights, boundary perpendicular distances, cell volumes) agree to 1e-13
  relative: the reference is compiled with -ffast-math, the reader is not.
* O(cells + faces): a 48^3 box (110,592 hexahedra) reads in seconds.
* Files the reader cannot take are refused with a reason.
"""
import os
import time

import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import workloads as W

import flow_cases as FC

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
METRICS = ("face_geo_aver", "face_ksi_A", "face_area_vector", "face_alpha", "face_distance",
           "face_unit", "bc_area", "bc_area_vector", "bc_alpha", "bc_distance", "bc_unit",
           "bc_perp_dist", "bc_ksi_A", "cell_volume")


def _compare(m, ref):
    for k in ("face_left", "face_right", "bc_left"):
        assert np.array_equal(m[k], ref[k]), k
    for k in METRICS:
        err = np.abs(m[k] - ref[k]).max() / np.abs(ref[k]).max()
        assert err <= 1e-13, (k, err)
    rp, col = ocsl.build_pattern(m["n_cells"], m["face_left"], m["face_right"], m["bc_left"])
    assert np.array_equal(rp, ref["row_ptr"]) and np.array_equal(col, ref["column_index"])


@pytest.mark.parametrize("cells", ["hex", "tet", "wedge"])
def test_reader_matches_reference(lib_built, tmp_path, cells):
    path = str(tmp_path / "m.su2")
    W.write_su2_box(path, 5, 4, 3, cells=cells)
    m = ocsl.read_su2(path)
    assert m["markers"] == ["inlet", "walls", "outlet"]
    _compare(m, np.load(os.path.join(GOLDEN, f"mesh_{cells}.npz")))
    # boundary faces come marker by marker
    assert np.all(np.diff(m["bc_marker"]) >= 0)


def test_reader_matches_recorded_3d_run(lib_built, tmp_path):
    path = str(tmp_path / "box3d.su2")
    W.write_su2_box(path, 10, 6, 4)
    _compare(ocsl.read_su2(path), FC.Golden("box3d").setup)


def test_reader_scales_linearly(lib_built, tmp_path):
    path = str(tmp_path / "big.su2")
    W.write_su2_box(path, 48, 48, 48)
    t0 = time.perf_counter()
    m = ocsl.read_su2(path)
    dt = time.perf_counter() - t0
    assert m["n_cells"] == 48 ** 3 and m["n_faces"] == 3 * 47 * 48 * 48
    assert m["n_bc"] == 6 * 48 * 48
    assert np.all(m["cell_volume"] > 0)
    print(f"48^3 hexahedra read in {dt:.2f} s")
    assert dt < 20.0


@pytest.mark.parametrize("text,why", [
    ("NDIME= 3\n", "NELEM"),
    ("NELEM= 1\n14 0 1 2 3 4 0\nNPOIN= 5\n", "element type"),
    ("NELEM= 1\n10 0 1 2 3 0\nNPOIN= 4\n0 0 0 0\n1 0 0 1\n0 1 0 2\n0 0 1 3\nNMARK= 1\n"
     "MARKER_TAG= a\nMARKER_ELEMS= 1\n5 0 1 9\n", "boundary element"),
])
def test_reader_refuses_bad_files(lib_built, tmp_path, text, why):
    path = tmp_path / "bad.su2"
    path.write_text(text)
    with pytest.raises(ocsl.OcslError) as e:
        ocsl.read_su2(str(path))
    assert why in str(e.value)
