"""Host side of the implicit method (no GPU): FVM_TVD_IMPLICIT task files, the mesh as
Grid::initFromFiles builds it, bindings by cell and edge type, and the error codes."""
import numpy as np
import pytest

from conftest import implicit_golden_names, load_golden, write_case


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


@pytest.mark.parametrize("name", implicit_golden_names())
def test_implicit_mesh_matches_oracle_loader(capi, oracle, tmp_path, name):
    """The library's mesh of an implicit task equals the oracle's restatement of
    Grid::initFromFiles (src/mesh/grid.cpp:51-252), which reproduces the reference's runs."""
    from cfd2d import meshgen as mg
    g = load_golden(name)
    lib = capi.Mesh(task_xml=write_case(tmp_path, g)).export()
    nb = mg.triangle_neighbours(g["tris"])
    om = oracle.OracleMesh(g["nodes"], g["tris"], g["bsegs"], g["bseg_bnd"], berkeley_neigh=np.where(nb >= 0, nb, -2),
                           legacy=True).export()
    for k in ("cell_edges", "cell_S", "cell_c", "edge_n12", "edge_c12", "edge_npts", "edge_n", "edge_l",
              "edge_pts", "edge_bnd"):
        assert bits_equal(lib[k], om[k]), k


def _edit(tmp_path, g, old, new):
    xml = str(g["task_xml"])
    assert old in xml, old
    write_case(tmp_path, g)
    (tmp_path / "task.xml").write_text(xml.replace(old, new, 1))
    return str(tmp_path / "task.xml")


def _code(capi, path):
    with pytest.raises(capi.CfdError) as e:
        capi.Mesh(task_xml=path)
    return e.value.code


def test_implicit_error_codes(capi, tmp_path):
    g = load_golden("implicit_bc_steady")
    assert _code(capi, _edit(tmp_path, g, "BOUND_WALL", "BOUND_PERIODIC")) == 102       # unsupported type
    assert _code(capi, _edit(tmp_path, g, '<cell type="0" />', '<cell type="5" />')) == 3   # unknown cell type
    assert _code(capi, _edit(tmp_path, g, 'edgeType="3"', 'edgeType="9"')) == 4         # unknown edge type
    assert _code(capi, _edit(tmp_path, g, "<start ", "<begin ")) == 2                  # steady CFL block incomplete
    assert _code(capi, _edit(tmp_path, g, "<smoothing>", "<smoothin>")) in (1, 2)      # malformed / missing
    assert _code(capi, _edit(tmp_path, g, '<name value="mesh" />', '<name value="nomesh" />')) == 301
    gm = '<FLUX value="LAX" />'
    assert _code(capi, _edit(tmp_path, g, gm, gm + '<GMRES krylov="0" />')) == 2


def test_implicit_unsteady_task_needs_no_cfl_block(capi, tmp_path):
    """FVM_TVD_IMPLICIT::init reads <CFL> only when STEADY=1 (:49-58)."""
    g = load_golden("implicit_vortex_lax")
    xml = str(g["task_xml"])
    a, b = xml.index("<CFL>"), xml.index("</CFL>") + len("</CFL>")
    write_case(tmp_path, g)
    (tmp_path / "task.xml").write_text(xml[:a] + xml[b:])
    m = capi.Mesh(task_xml=str(tmp_path / "task.xml"))
    assert m.export()["cell_S"].shape == (128,)
