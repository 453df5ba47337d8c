"""The synthetic mesher reproduces the reference's topology and dual mesh
(edge numbering, orientation, cell-edge maps and signs, patches, areas) bit
for bit; checked against fixtures made by the reference's own
mesh_build_topology / dual_mesh_build (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh


def _compare(m, g):
    assert np.array_equal(m.edges(), g["edges"])
    assert np.array_equal(m.cell_edges(), g["cell_edges"])
    assert np.array_equal(m.cell_edge_signs(), g["cell_edge_signs"])
    assert np.array_equal(m.edge_lengths(), g["edge_lengths"])
    assert np.array_equal(m.edge_directions(), g["edge_directions"])
    assert np.array_equal(m.region_areas("edge"), g["edge_region_areas"])
    assert np.array_equal(m.region_areas("node"), g["node_region_areas"])
    ep = m.patches("edge")
    assert np.array_equal([len(p) for p in ep], g["edge_patch_counts"])
    assert np.array_equal(np.concatenate(ep).reshape(-1, 12), g["edge_patches"])
    npch = m.patches("node")
    assert np.array_equal([len(p) for p in npch], g["node_patch_counts"])
    assert np.array_equal(np.concatenate(npch).reshape(-1, 12), g["node_patches"])


@pytest.mark.parametrize("name", ["plate4", "plate8", "box421", "plate_msh"])
def test_topology_and_dual_from_arrays(name):
    g = golden(name)
    with SynthMesh.from_arrays(g["xyz"], g["quads"]) as m:
        _compare(m, g)


def test_generated_plate_matches_reference_numbering():
    g = golden("plate8")
    with SynthMesh.plate(1.0, 1.0, 8, 8) as m:
        assert np.array_equal(m.array("xyz", (m.n_nodes, 3)), g["xyz"])
        assert np.array_equal(m.array("quads", (m.n_quads, 4), np.int32), g["quads"])
        _compare(m, g)


def test_generated_box_5cm():
    """2.0 x 1.0 x 0.5 m box at 5 cm: 2800 cells, 5600 edges, 2802 nodes."""
    g = golden("box_5cm_topology")
    with SynthMesh.box(2.0, 1.0, 0.5, 40, 20, 10) as m:
        assert (m.n_quads, m.n_edges, m.n_nodes) == (2800, 5600, 2802)
        assert np.array_equal(m.array("xyz", (m.n_nodes, 3)), g["xyz"])
        assert np.array_equal(m.array("quads", (m.n_quads, 4), np.int32), g["quads"])
        _compare(m, g)
        # closed, consistently wound surface: every edge in exactly two cells,
        # once along and once against its orientation
        ce, cs = m.cell_edges().ravel(), m.cell_edge_signs().ravel()
        assert np.array_equal(np.bincount(ce, minlength=m.n_edges), np.full(m.n_edges, 2))
        assert np.array_equal(np.bincount(ce, weights=cs, minlength=m.n_edges), np.zeros(m.n_edges))


def test_box_counts_match_config_sizes():
    with SynthMesh.box(2.0, 1.0, 0.5, 80, 40, 20) as m:
        assert (m.n_quads, m.n_edges, m.n_nodes) == (11200, 22400, 11202)


def test_bad_inputs_rejected():
    with pytest.raises(RuntimeError):
        SynthMesh.plate(1.0, 1.0, 0, 4)
    with pytest.raises(RuntimeError):
        SynthMesh.from_arrays(np.zeros((3, 3)), np.array([[0, 1, 2, 7]]))
