"""High-order tet meshing: the host builder's mesh against the reference's own high-order meshes
(golden fixtures made by Mesh.GetHighOrderMesh, Florence/MeshGeneration/Mesh.py:1339-1410),
equal up to a permutation of node numbers; and the node-layout classification of the device
mesher (fl_TetNodeLayout, a host-only entry point)."""
import itertools

import numpy as np
import pytest

from conftest import load_golden
from florence_gb300 import meshes

REFERENCE_TET_MESHES = ["tet_p2_mr", "tet_p2_nimr", "tet_p2_amr", "tet_p3_mr_jitter"]


def linear_part(points, elements):
    """The linear tets under a high-order mesh: vertex nodes (local nodes 0-3) renumbered
    compactly in increasing id order."""
    verts = np.unique(elements[:, :4])
    remap = np.full(int(elements.max()) + 1, -1, np.int64)
    remap[verts] = np.arange(len(verts))
    return points[verts], remap[elements[:, :4]]


def permutation_between(Ea, Eb):
    """m with Eb == m[Ea] element by element, or None when no node permutation relates them."""
    Ea = np.asarray(Ea, np.int64)
    Eb = np.asarray(Eb, np.int64)
    if Ea.shape != Eb.shape or Ea.min() < 0 or Eb.min() < 0:
        return None
    n = int(Ea.max()) + 1
    if int(Eb.max()) + 1 != n:
        return None
    m = np.full(n, -1, np.int64)
    m[Ea.ravel()] = Eb.ravel()
    if (m < 0).any() or not np.array_equal(m[Ea], Eb) or len(np.unique(m)) != n:
        return None
    return m


def equispaced_pattern(p):
    """Barycentric coordinates (i, j, k, l) / p, i + j + k + l = p, vertices first."""
    rows = [c for c in itertools.product(range(p + 1), repeat=4) if sum(c) == p]
    rows.sort(key=lambda c: (-max(c), [-x for x in c]))
    return np.array(rows, np.float64) / p


@pytest.mark.parametrize("name", REFERENCE_TET_MESHES)
def test_host_builder_reproduces_reference_high_order_mesh(name):
    d = load_golden(name)
    P_ref, E_ref = d["points"], d["elements"].astype(np.int64)
    lam = meshes.local_pattern(P_ref, E_ref, 0, "tet")
    P_lin, E_lin = linear_part(P_ref, E_ref)
    P, E = meshes.raise_tet_order(P_lin, E_lin, lam)
    assert P.shape == P_ref.shape
    m = permutation_between(E, E_ref)
    assert m is not None, "node numbering is not a permutation of the reference's"
    scale = np.abs(P_ref).max()
    assert np.abs(P - P_ref[m]).max() <= 1e-12 * scale


@pytest.mark.parametrize("name,expected", [("tet_p2_mr", (1, 0, 0)), ("tet_p3_mr_jitter", (2, 1, 0))])
def test_node_layout_of_reference_elements(name, expected):
    d = load_golden(name)
    lam = meshes.local_pattern(d["points"], d["elements"], 0, "tet")
    assert meshes.tet_node_layout(lam) == expected


@pytest.mark.parametrize("p,expected", [(1, (0, 0, 0)), (2, (1, 0, 0)), (3, (2, 1, 0)), (4, (3, 3, 1))])
def test_node_layout_equispaced(p, expected):
    assert meshes.tet_node_layout(equispaced_pattern(p)) == expected


def test_node_layout_rejects_asymmetric_and_oversized_layouts():
    lam = equispaced_pattern(3).copy()
    edge = np.nonzero((np.abs(lam) > 1e-10).sum(1) == 2)[0][0]
    k = np.nonzero(lam[edge])[0]
    lam[edge, k[0]] += 0.05  # one edge node moved along its edge: no longer mirror-symmetric
    lam[edge, k[1]] -= 0.05
    with pytest.raises(ValueError):
        meshes.tet_node_layout(lam)
    with pytest.raises(ValueError):
        meshes.tet_node_layout(equispaced_pattern(5))  # 56 nodes: above the 35 supported
    bad = equispaced_pattern(2)
    bad[0] = 0.0  # a node with no vertex weight
    with pytest.raises(ValueError):
        meshes.tet_node_layout(bad)


def test_host_builder_equispaced_p4_counts():
    P_lin = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float64)
    E_lin = np.array([[0, 1, 2, 3], [1, 2, 3, 4]], np.int64)
    P, E = meshes.raise_tet_order(P_lin, E_lin, equispaced_pattern(4))
    # 5 vertices, 9 edges x 3, 7 faces x 3, 2 interiors x 1
    assert P.shape[0] == 5 + 27 + 21 + 2
    assert np.array_equal(E[:, :4], E_lin)


# ------------------------------------------------------------------------------------------------
# hexes (HighOrderMeshHex, Florence/MeshGeneration/HigherOrderMeshing/HigherOrderMeshingHex.py)
# ------------------------------------------------------------------------------------------------
REFERENCE_HEX_MESHES = ["hex_p2_nh_q5", "hex_p2_mr", "hex_p3_nh", "hex_p4_nh"]


def linear_hex_part(points, elements):
    """The linear hexes under a high-order hex mesh: vertex nodes (local nodes 0-7) renumbered
    compactly in increasing id order."""
    verts = np.unique(elements[:, :8])
    remap = np.full(int(elements.max()) + 1, -1, np.int64)
    remap[verts] = np.arange(len(verts))
    return points[verts], remap[elements[:, :8]]


@pytest.mark.parametrize("name", REFERENCE_HEX_MESHES)
def test_host_hex_builder_reproduces_reference_mesh(name):
    """The reference's own p = 2, 3, 4 hex meshes (GetHighOrderMesh on a Florence box, Gauss-Lobatto
    nodes) rebuilt from their linear hexes and one element's node layout: the same mesh up to a
    node permutation, positions within 1e-12."""
    d = load_golden(name)
    P_ref, E_ref = d["points"], d["elements"].astype(np.int64)
    xi = meshes.local_pattern(P_ref, E_ref, 0, "hex")
    P_lin, E_lin = linear_hex_part(P_ref, E_ref)
    Ph, Eh = meshes.raise_hex_order(P_lin, E_lin, xi)
    m = permutation_between(Eh, E_ref)
    assert m is not None
    assert np.abs(Ph - P_ref[m]).max() <= 1e-12 * np.abs(P_ref).max()


@pytest.mark.parametrize("p", [2, 3, 4])
def test_host_hex_builder_matches_structured_builder(p):
    """A 5 x 4 x 3 box raised from its linear hexes against the structured builder of the same
    order: the same mesh up to a node permutation (shared edges and faces in every orientation a
    structured box has), and the classification the device mesher makes of the layout."""
    d = load_golden({2: "hex_p2_nh_q5", 3: "hex_p3_nh", 4: "hex_p4_nh"}[p])
    xi = meshes.local_pattern(d["points"], d["elements"], 0, "hex")
    P_s, E_s = meshes.structured_hex((5, 4, 3), (2.0, 1.5, 1.0), xi)
    P_lin, E_lin = linear_hex_part(P_s, E_s)
    Ph, Eh = meshes.raise_hex_order(P_lin, E_lin, xi)
    m = permutation_between(Eh, E_s)
    assert m is not None
    assert np.abs(Ph - P_s[m]).max() <= 1e-12 * np.abs(P_s).max()
    assert meshes.hex_node_layout(xi) == (p - 1, (p - 1) ** 2, (p - 1) ** 3)


def test_hex_layout_without_symmetry_is_rejected():
    d = load_golden("hex_p2_nh_q5")
    xi = meshes.local_pattern(d["points"], d["elements"], 0, "hex").copy()
    edge_nodes = [a for a in range(8, xi.shape[0]) if (np.abs(np.abs(xi[a]) - 1.0) < 1e-9).sum() == 2]
    xi[edge_nodes[0]] += 0.1 * (np.abs(np.abs(xi[edge_nodes[0]]) - 1.0) > 1e-9)  # off the edge's midpoint
    with pytest.raises(ValueError):
        meshes.hex_node_layout(xi)
