"""Host logic of the p-multigrid transfers (no GPU): the prolongation from the vertices reproduces
every linear field at the nodes of the high-order tetrahedra exactly, and the restriction is its
transpose."""
import numpy as np

from conftest import load_golden


def _dense(ptr, cols, w, nrows, ncols):
    A = np.zeros((nrows, ncols))
    for r in range(nrows):
        for k in range(ptr[r], ptr[r + 1]):
            A[r, cols[k]] += w[k]
    return A


def test_prolongation_interpolates_linear_fields_and_restriction_is_its_transpose():
    from florence_gb300 import meshes
    from florence_gb300.multigrid import vertex_transfer
    d = load_golden("tet_p3_mr_jitter")
    pat = meshes.local_pattern(d["points"], d["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((3, 2, 2), (2.0, 1.0, 1.0), 4, pat)
    verts, el_c, (pp, pc, pw), (rp, rc, rw) = vertex_transfer(el, pat, P.shape[0])
    assert el_c.max() + 1 == verts.shape[0] and np.array_equal(verts[el_c], el[:, :4])
    Pm = _dense(pp, pc, pw, P.shape[0], verts.shape[0])
    Rm = _dense(rp, rc, rw, verts.shape[0], P.shape[0])
    assert np.array_equal(Rm, Pm.T)
    rng = np.random.default_rng(0)
    A, c = rng.standard_normal((3, 3)), rng.standard_normal(3)
    lin = P @ A.T + c                                 # a linear field at every node
    assert np.abs(Pm @ lin[verts] - lin).max() < 1e-12
    assert np.allclose(Pm.sum(1), 1.0)                 # partition of unity
