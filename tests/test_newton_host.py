"""CPU checks of the Newton driver's host preprocessing (Neumann face loads, problem set-up)."""
import numpy as np

from conftest import load_golden


def test_face_weights_integrate_polynomials():
    from florence_gb300.newton import _face_weights
    from florence_gb300 import meshes
    d = load_golden("tet_p3_mr_jitter")
    lam = meshes.local_pattern(d["points"], d["elements"], 0, "tet")
    nodes = np.nonzero(np.abs(lam[:, 3]) < 1e-10)[0]
    st = lam[nodes][:, 1:3]
    w = _face_weights(st)
    assert len(w) == 10 and abs(w.sum() - 1.0) < 1e-13
    # exact for cubics: the integral of s^2 t over the triangle is 2! 1! / 5! = 1/60, its mean 1/30
    assert abs(np.sum(w * st[:, 0] ** 2 * st[:, 1]) - 1.0 / 30.0) < 1e-13


def test_beam_problem_loads_and_supports():
    from florence_gb300.newton import build_beam_problem
    P, el, Jm, w, fixed, f = build_beam_problem(nx=8, ny=2, nz=2, traction=0.01)
    assert el.shape[1] == 20 and Jm.shape == (3, 20, 14)
    fz = f.reshape(-1, 3)
    assert abs(fz[:, 2].sum() + 0.01 * 1.0) < 1e-14       # traction x face area (1 x 1)
    assert np.abs(fz[:, :2]).max() == 0.0
    assert np.all(np.abs(P[fz[:, 2] != 0, 0] - 4.0) < 1e-12)  # loads only on x = 4
    assert fixed.reshape(-1, 3)[:, 0].sum() == np.sum(np.abs(P[:, 0]) < 1e-9)
