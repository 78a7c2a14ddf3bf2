"""The library's SU2 reader (nlgpu_su2_*: host code, no GPU) against the
reference's own parser: for the exact file the reference read, nodes, 2D
elements (in the reference's hashed-container order) and every boundary group
must come out bit-identical to what the reference's mesh_container_2d held."""
import numpy as np
import pytest

import golden_cases as gc


@pytest.fixture(scope="module")
def thermal():
    from nonlocal_gb300 import build
    build.build()
    from nonlocal_gb300 import thermal as T
    return T


@pytest.mark.parametrize("name", gc.SU2_CASES)
def test_reader_matches_reference_parser(thermal, name, tmp_path):
    fx = gc.load(name)
    m = thermal.read_su2(gc.write_su2_text(fx, str(tmp_path / "mesh.su2")))
    nodes, elements = gc.mesh_before_renumbering(fx)
    assert np.array_equal(m.nodes, nodes)
    assert np.array_equal(m.elements, elements)
    assert m.element == ("bilinear" if elements.shape[1] == 4 else "serendipity")
    if "nodes_before_renumbering" in fx:
        m = m.renumbered(fx["cm_" + fx["config"]["renumber"]])
    groups = [str(g) for g in fx["groups_1d"]]
    assert sorted(k for k, v in m.groups.items() if v[0] == 1) == sorted(groups)
    for g in groups:
        assert np.array_equal(m.boundary(g), fx["bnd_" + g]), g
    # 2D groups tile the 2D elements in container order, 1D groups follow them
    spans2 = sorted((first, len(el)) for dim, el, first in m.groups.values() if dim == 2)
    assert spans2[0][0] == 0 and sum(c for _, c in spans2) == len(m.elements)
    assert all(a[0] + a[1] == b[0] for a, b in zip(spans2, spans2[1:]))


def test_two_dimensional_marker_and_default_group(thermal, tmp_path):
    fx = gc.load("b6_groups_local")
    m = thermal.read_su2(gc.write_su2_text(fx, str(tmp_path / "mesh.su2")))
    dim, members, first = m.groups["inclusion"]
    assert dim == 2 and len(members) == 14
    assert np.array_equal(m.elements[first:first + 14], members)
    assert m.groups["DEFAULT"][0] == 2 and len(m.groups["DEFAULT"][1]) == 36 - 14


def test_reader_errors(thermal, tmp_path):
    from nonlocal_gb300 import _lib
    with pytest.raises(_lib.NlgpuError):
        thermal.read_su2(str(tmp_path / "missing.su2"))
    bad = tmp_path / "bad.su2"
    bad.write_text("NDIME= 2\nNELEM= 1\n99 0 1 2 3 0\nNPOIN= 4\n0 0 0\n1 0 1\n1 1 2\n0 1 3\nNMARK= 0\n")
    with pytest.raises(_lib.NlgpuError, match="Unknown element type"):
        thermal.read_su2(str(bad))
    reserved = tmp_path / "reserved.su2"
    reserved.write_text("NDIME= 2\nNELEM= 1\n9 0 1 2 3 0\nNPOIN= 4\n0 0 0\n1 0 1\n1 1 2\n0 1 3\n"
                        "NMARK= 1\nMARKER_TAG= DEFAULT\nMARKER_ELEMS= 1\n3 0 1\n")
    with pytest.raises(_lib.NlgpuError, match="reserved group name"):
        thermal.read_su2(str(reserved))
