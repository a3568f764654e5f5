"""Host side of the library (no GPU): task.xml + mesh readers + edge topology.

The library's readers must build the reference's Grid bit for bit from the same
files (golden fixtures made by the reference itself), and report the
reference's error codes on bad input.
"""
import os

import numpy as np
import pytest

from conftest import golden_names, load_golden, write_case
from test_oracle_golden import bits_equal

KEYS = ("cell_edges", "cell_S", "cell_c", "edge_n12", "edge_c12", "edge_npts", "edge_n", "edge_l", "edge_pts",
        "edge_bnd")


@pytest.mark.parametrize("name", golden_names())
def test_unv_reader_matches_reference_grid(capi, tmp_path, name):
    g = load_golden(name)
    m = capi.Mesh(task_xml=write_case(tmp_path, g)).export()
    for k in KEYS:
        assert bits_equal(m[k], g["grid_" + k]), k


@pytest.mark.parametrize("variant", ["crlf", "no_final_newline", "split_across_threads"])
def test_unv_reader_line_handling(capi, tmp_path, variant):
    """The reader cuts the file into lines in parallel chunks: CRLF line ends, a last
    line without a newline and a file large enough to be split across threads (the
    same records repeated in a block the reader skips) all give the reference's Grid."""
    g = load_golden("vortex_limits")
    text = str(g["mesh_unv"])
    if variant == "crlf":
        text = text.replace("\n", "\r\n")
    elif variant == "no_final_newline":
        text = text.rstrip("\n")
    else:  # a block id no reader handles, ~4 MB, ahead of the mesh
        text = "    -1\n  9999\n" + ("  1.0 -1.5 2.0\n" * 250000) + "    -1\n" + text
    path = write_case(tmp_path, g)
    (tmp_path / "mesh.unv").write_bytes(text.encode())
    m = capi.Mesh(task_xml=path).export()
    for k in KEYS:
        assert bits_equal(m[k], g["grid_" + k]), k


def test_triangle_reader_matches_reference_grid(capi, tmp_path):
    g = load_golden("berkeley_triangle")
    m = capi.Mesh(task_xml=write_case(tmp_path, g)).export()
    for k in KEYS:
        if k == "edge_pts":  # one point per edge: only the midpoint is defined
            assert bits_equal(m[k][:, 0], g["grid_" + k][:, 0])
        else:
            assert bits_equal(m[k], g["grid_" + k]), k


def test_arrays_path_matches_file_path(capi, tmp_path):
    g = load_golden("shuffled_mesh")
    a = capi.Mesh(nodes=g["nodes"], tris=g["tris"], bsegs=g["bsegs"], bseg_bnd=g["bseg_bnd"]).export()
    b = capi.Mesh(task_xml=write_case(tmp_path, g)).export()
    for k in KEYS:
        assert bits_equal(a[k], b[k]), k


def test_rcm_order_is_a_permutation_and_tightens_bandwidth(capi):
    g = load_golden("shuffled_mesh")
    m = capi.Mesh(nodes=g["nodes"], tris=g["tris"], bsegs=g["bsegs"], bseg_bnd=g["bseg_bnd"])
    p = m.order(rcm=True)
    assert np.array_equal(np.sort(p), np.arange(m.nc))
    ex = m.export()
    inv = np.empty_like(p); inv[p] = np.arange(len(p))
    c12 = ex["edge_c12"]; inner = c12[:, 1] >= 0
    bw_orig = np.abs(c12[inner, 0] - c12[inner, 1]).max()
    bw_rcm = np.abs(inv[c12[inner, 0]] - inv[c12[inner, 1]]).max()
    assert bw_rcm < bw_orig


def _edit(tmp_path, g, old, new, unv=None):
    xml = str(g["task_xml"])
    assert old in xml
    (tmp_path / "task.xml").write_text(xml.replace(old, new))
    (tmp_path / "mesh.unv").write_text(unv if unv is not None else str(g["mesh_unv"]))
    return str(tmp_path / "task.xml")


def _code(capi, path):
    with pytest.raises(capi.CfdError) as e:
        capi.Mesh(task_xml=path)
    return e.value.code


def test_error_codes_follow_the_reference(capi, tmp_path):
    g = load_golden("shock_tube_4bc")
    assert _code(capi, _edit(tmp_path, g, "salome_unv", "gmsh")) == 201            # MeshReader::getType
    assert _code(capi, _edit(tmp_path, g, "<name>left</name>", "<name>west</name>")) == 3  # unknown region
    assert _code(capi, _edit(tmp_path, g, "<name>bnd1</name>", "<name>xxx</name>")) == 4   # unknown edge type
    assert _code(capi, _edit(tmp_path, g, "BOUND_OUTLET", "BOUND_PERIODIC")) == 102
    assert _code(capi, _edit(tmp_path, g, '<Vx value="0.1" />', "")) == 101       # inlet parameter missing
    assert _code(capi, _edit(tmp_path, g, "<control>", "<control")) == 1          # XML syntax
    assert _code(capi, _edit(tmp_path, g, '<CFL value="0.5" />', "")) == 2        # missing element
    unv = str(g["mesh_unv"])
    assert _code(capi, _edit(tmp_path, g, "mesh.unv", "missing.unv")) == 301
    # a triangle element of an unknown type (UNV 2412 type 42)
    bad = unv.replace("        41         2         1         7         3", "        42         2         1         7         3", 1)
    assert _code(capi, _edit(tmp_path, g, "salome_unv", "salome_unv", unv=bad)) == 221


def test_boundary_edge_without_unv_element_is_222(capi, tmp_path):
    from cfd2d import meshgen as mg
    g = load_golden("shock_tube_4bc")
    m = mg.Mesh(g["nodes"], g["tris"], g["cell_region"], g["bsegs"][1:], g["bseg_bnd"][1:])
    unv = mg.write_unv(m, [str(x) for x in g["region_names"]], [str(x) for x in g["bnd_names"]])
    assert _code(capi, _edit(tmp_path, g, "salome_unv", "salome_unv", unv=unv)) == 222
