"""GPU tests of the p-multigrid linear step (florence_gb300/multigrid.py): on the tet p=3 beam
(24x6x6 lattice) the flexible CG with the two-level cycle solves the Newton system to the same
solution as a tight block-Jacobi PCG in far fewer iterations, and Newton with it converges to
the same displacement as Newton with the block-Jacobi PCG."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def beam():
    import florence_gb300 as fl
    from florence_gb300 import meshes
    from florence_gb300.newton import build_beam_problem
    P, el, Jm, w, fixed, f = build_beam_problem(24, 6, 6, traction=0.01)
    asm = fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode="csr")
    t = np.load(os.path.join(os.path.dirname(__file__), "golden", "tet_p3_mr_jitter.npz"))
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    return asm, P, fixed, f, pat


def test_flexible_cg_with_pmg_matches_block_jacobi(beam):
    from florence_gb300.multigrid import PMultigrid, fcg
    from florence_gb300.newton import pcg
    asm, P, fixed, f, pat = beam
    u = torch.zeros(P.size, dtype=torch.float64, device="cuda")
    V, T = asm.assemble(torch.from_numpy(P).cuda())
    fx = torch.from_numpy(fixed.astype(np.int8)).cuda()
    b = torch.from_numpy(np.where(fixed, 0.0, f)).cuda()
    x_ref, it_ref, rel_ref = pcg(asm, V, b, fx, rtol=1e-12, maxiter=200000, spmv="fp64")
    mg = PMultigrid(asm, pat, fixed)
    mg.update(V, u)
    x, it, rel = fcg(mg, b, rtol=1e-10, maxiter=400)
    assert rel <= 1e-10
    err = float(torch.linalg.vector_norm(x - x_ref) / torch.linalg.vector_norm(x_ref))
    assert err < 1e-7, (err, it, it_ref)
    assert it * 10 < it_ref, (it, it_ref)


def test_newton_with_pmg_matches_newton_with_block_jacobi(beam):
    from florence_gb300.newton import NewtonSolver
    asm, P, fixed, f, pat = beam
    a = NewtonSolver(asm, fixed, f, n_increments=2, tol=1e-10).solve()
    b = NewtonSolver(asm, fixed, f, n_increments=2, tol=1e-10, linear="pmg", pattern=pat).solve()
    assert not a["failed"] and not b["failed"]
    d = float(torch.linalg.vector_norm(b["u"] - a["u"]) / torch.linalg.vector_norm(a["u"]))
    assert d < 1e-7, d
