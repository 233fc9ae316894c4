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
