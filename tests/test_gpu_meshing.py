"""GPU tests of the device high-order tet mesher (fl_RaiseTetOrder): node numbers identical to the
host builder's, positions within a few rounding errors of its, and the reference's own
high-order meshes (golden fixtures) reproduced up to a permutation of node numbers."""
import numpy as np
import pytest

from conftest import load_golden
from florence_gb300 import meshes
from test_meshing import REFERENCE_TET_MESHES, equispaced_pattern, linear_part, permutation_between

pytestmark = pytest.mark.gpu

POS_TOL = 1e-15  # relative to the largest coordinate: the sums differ only in rounding order


def device_raise(P, el, lam):
    Pd, Ed = meshes.raise_tet_order_device(P, el, lam)
    return Pd.cpu().numpy(), Ed.cpu().numpy()


def assert_same_as_host(P, el, lam):
    Ph, Eh = meshes.raise_tet_order(P, el, lam)
    Pd, Ed = device_raise(P, el, lam)
    assert Pd.shape == Ph.shape
    assert np.array_equal(Ed, Eh)
    assert np.abs(Pd - Ph).max() <= POS_TOL * max(1.0, np.abs(Ph).max()) * 4
    return Pd, Ed


@pytest.mark.parametrize("name", REFERENCE_TET_MESHES)
def test_device_reproduces_reference_high_order_mesh(name):
    d = load_golden(name)
    P_ref, E_ref = d["points"], d["elements"].astype(np.int64)
    lam = meshes.local_pattern(P_ref, E_ref, 0, "tet")
    P_lin, E_lin = linear_part(P_ref, E_ref)
    Pd, Ed = assert_same_as_host(P_lin, E_lin, lam)
    m = permutation_between(Ed, E_ref)
    assert m is not None
    assert np.abs(Pd - P_ref[m]).max() <= 1e-12 * np.abs(P_ref).max()


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_device_matches_host_on_jittered_delaunay(p):
    lam = equispaced_pattern(p)
    P, el = meshes.jittered_tet_beam((6, 3, 3), (2.0, 1.0, 1.0), 7, np.eye(4))  # linear tets
    assert_same_as_host(P, el, lam)


def test_device_matches_host_with_reference_p3_layout_and_unused_vertices():
    d = load_golden("tet_p3_mr_jitter")
    lam = meshes.local_pattern(d["points"], d["elements"], 0, "tet")
    P, el = meshes.kuhn_tet_box((5, 4, 3), (2.0, 1.0, 1.0))
    # a shuffled element order, and vertices no element uses (dropped from the numbering)
    el = el[np.random.default_rng(3).permutation(len(el))]
    P = np.vstack([[[9.0, 9.0, 9.0]], P, [[8.0, 8.0, 8.0]]])
    el = el + 1
    Pd, Ed = assert_same_as_host(P, el, lam)
    assert np.abs(Pd[:120] - P[1:121]).max() <= 1e-14  # the 6 x 5 x 4 used vertices, in id order
    assert not np.any(np.abs(Pd - 8.0).max(1) < 1.5)  # the unused ones are gone


def test_device_kuhn_box_node_count():
    lam = equispaced_pattern(3)
    n = (12, 10, 9)
    P, el = meshes.kuhn_tet_box(n)
    Pd, Ed = assert_same_as_host(P, el, lam)
    nv = np.prod([k + 1 for k in n])
    edges = np.unique(np.sort(el[:, [[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]]].reshape(-1, 2), 1), axis=0)
    faces = np.unique(np.sort(el[:, [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]]].reshape(-1, 3), 1), axis=0)
    assert Pd.shape[0] == nv + 2 * len(edges) + len(faces)
    # every element's vertex nodes are the first four local nodes, in the compact vertex numbering
    assert np.array_equal(Ed[:, :4], el)
    # preallocated outputs (one call, no counting call): the same mesh
    import torch
    op = torch.full((Pd.shape[0] + 17, 3), np.nan, dtype=torch.float64, device="cuda")
    oe = torch.full(Ed.shape, -1, dtype=torch.int64, device="cuda")
    P2, E2 = meshes.raise_tet_order_device(P, el, lam, out_points=op, out_elements=oe)
    assert P2.data_ptr() == op.data_ptr() and E2.data_ptr() == oe.data_ptr()
    assert np.array_equal(E2.cpu().numpy(), Ed) and np.array_equal(P2.cpu().numpy(), Pd)


def test_device_rejects_bad_meshes():
    lam = equispaced_pattern(2)
    P, el = meshes.kuhn_tet_box((2, 2, 2))
    bad = el.copy()
    bad[3, 2] = bad[3, 1]  # repeated vertex
    with pytest.raises(ValueError):
        meshes.raise_tet_order_device(P, bad, lam)
    bad = el.copy()
    bad[5, 0] = len(P)  # vertex id out of range
    with pytest.raises(RuntimeError):
        meshes.raise_tet_order_device(P, bad, lam)


# ------------------------------------------------------------------------------------------------
# hexes (fl_RaiseHexOrder)
# ------------------------------------------------------------------------------------------------
from test_meshing import REFERENCE_HEX_MESHES, linear_hex_part  # noqa: E402


def assert_hex_same_as_host(P, el, xi):
    Ph, Eh = meshes.raise_hex_order(P, el, xi)
    Pd, Ed = meshes.raise_hex_order_device(P, el, xi)
    Pd, Ed = Pd.cpu().numpy(), Ed.cpu().numpy()
    assert Pd.shape == Ph.shape
    assert np.array_equal(Ed, Eh)
    assert np.array_equal(Pd, Ph)  # the same products and sums in the same order
    return Pd, Ed


@pytest.mark.parametrize("name", REFERENCE_HEX_MESHES)
def test_device_reproduces_reference_high_order_hex_mesh(name):
    d = load_golden(name)
    P_ref, E_ref = d["points"], d["elements"].astype(np.int64)
    xi = meshes.local_pattern(P_ref, E_ref, 0, "hex")
    P_lin, E_lin = linear_hex_part(P_ref, E_ref)
    Pd, Ed = assert_hex_same_as_host(P_lin, E_lin, xi)
    m = permutation_between(Ed, E_ref)
    assert m is not None
    assert np.abs(Pd - P_ref[m]).max() <= 1e-12 * np.abs(P_ref).max()


@pytest.mark.parametrize("p", [2, 3, 4])
def test_device_hex_matches_host_on_distorted_shuffled_box(p):
    """A 7 x 5 x 4 box with jittered vertices, shuffled elements, every element's vertices
    relabelled by one of the cube's symmetries (so shared edges and faces are seen in every
    orientation) and two unused vertices."""
    d = load_golden({2: "hex_p2_nh_q5", 3: "hex_p3_nh", 4: "hex_p4_nh"}[p])
    xi = meshes.local_pattern(d["points"], d["elements"], 0, "hex")
    P_s, E_s = meshes.structured_hex((7, 5, 4), (2.0, 1.5, 1.0), xi)
    P, el = linear_hex_part(P_s, E_s)
    rng = np.random.default_rng(p)
    P = P + rng.uniform(-0.02, 0.02, P.shape)
    el = el[rng.permutation(len(el))]
    # the cube's rotations as permutations of the reference vertices (sign patterns of xi[:8])
    sg = np.where(xi[:8] > 0, 1, -1)
    perms = []
    for axes in ([0, 1, 2], [1, 2, 0], [2, 0, 1]):
        for flip in ([1, 1, 1], [-1, -1, 1], [-1, 1, -1], [1, -1, -1]):
            t = sg[:, axes] * np.array(flip)
            perms.append([int(np.nonzero((sg == t[k]).all(1))[0][0]) for k in range(8)])
    pick = rng.integers(0, len(perms), len(el))
    el = np.stack([el[i, perms[pick[i]]] for i in range(len(el))])
    P = np.vstack([[[9.0, 9.0, 9.0]], P, [[8.0, 8.0, 8.0]]])
    el = el + 1
    Pd, Ed = assert_hex_same_as_host(P, el, xi)
    assert not np.any(np.abs(Pd - 8.0).max(1) < 1.5)  # the unused vertices are gone
    nv = P.shape[0] - 2
    ne, nf, ni = meshes.hex_node_layout(xi)
    edges = 3 * 7 * 5 * 4 + 2 * (7 * 5 + 5 * 4 + 7 * 4) + 7 + 5 + 4  # edges of a 7 x 5 x 4 box
    faces = 3 * 7 * 5 * 4 + 7 * 5 + 5 * 4 + 7 * 4
    assert Pd.shape[0] == nv + edges * ne + faces * nf + len(el) * ni
