"""GPU tests of the p-multigrid linear step (florence_gb300/multigrid.py): on the tet p=3 beam
(24x6x6 lattice) the flexible CG with the two-level cycle solves the Newton system to the same
solution as a tight block-Jacobi PCG in far fewer iterations, and Newton with it converges to
the same displacement as Newton with the block-Jacobi PCG; its pieces -- the node-block masked
products (float-pair and FP32 values) against scipy, and the coarse PCG in one cooperative launch
against scipy's direct solve of the coarse system."""
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


def test_node_block_products_and_coarse_solve(beam):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from florence_gb300.multigrid import PMultigrid
    asm, P, fixed, f, pat = beam
    V, _ = asm.assemble(torch.from_numpy(P).cuda())
    mg = PMultigrid(asm, pat, fixed)
    mg.update(V, torch.zeros(P.size, dtype=torch.float64, device="cuda"))
    n = P.size
    free = ~fixed.astype(bool)
    x = torch.from_numpy(np.where(free, np.random.default_rng(3).standard_normal(n), 0.0)).cuda()
    K = sp.csr_matrix((V.cpu().numpy(), asm.indices.cpu().numpy(), asm.indptr.cpu().numpy()), shape=(n, n))
    ref = np.where(free, K @ x.cpu().numpy(), 0.0)
    y = torch.empty_like(x)
    mg.matvec(x, y)   # float pairs, ~2^-44 per product
    assert np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-12
    mg.smooth_matvec(x, y)
    assert np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-5
    # the coarse PCG (one cooperative launch) to 1e-10 against a direct solve of the coarse system
    c = mg.coarse
    nc = mg.nc
    fc = mg.fixed_c.cpu().numpy().astype(bool)
    Kc = sp.csr_matrix((mg.Vc.cpu().numpy(), c.indices.cpu().numpy(), c.indptr.cpu().numpy()), shape=(nc, nc))
    bc = np.where(fc, 0.0, np.random.default_rng(4).standard_normal(nc))
    mg.coarse_rtol, mg.coarse_maxiter = 1e-10, 20000
    it0 = mg.coarse_iters
    xc = mg.coarse_solve(torch.from_numpy(bc).cuda()).cpu().numpy()
    mg.check_flags()
    its = mg.coarse_iters - it0
    xr = spla.spsolve(Kc[~fc][:, ~fc].tocsc(), bc[~fc])
    assert 0 < its < 20000 and np.all(xc[fc] == 0.0)
    assert np.linalg.norm(xc[~fc] - xr) / np.linalg.norm(xr) < 1e-7


def test_coarse_fallback_path_matches(beam):
    """A coarse system too large for the one-launch solve (each SM's rows in its shared memory)
    is solved by the block-Jacobi PCG launched per iteration instead: the outer flexible CG
    converges to the same solution either way."""
    from florence_gb300.multigrid import PMultigrid, fcg
    asm, P, fixed, f, pat = beam
    V, _ = asm.assemble(torch.from_numpy(P).cuda())
    b = torch.from_numpy(np.where(fixed, 0.0, f)).cuda()
    sols = []
    for fast in (True, False):
        mg = PMultigrid(asm, pat, fixed)
        assert mg._coarse_fast  # this coarse system fits
        mg._coarse_fast = fast
        mg.update(V, torch.zeros(P.size, dtype=torch.float64, device="cuda"))
        x, it, rel = fcg(mg, b, rtol=1e-10, maxiter=400)
        assert rel <= 1e-10
        sols.append(x)
    assert float(torch.linalg.vector_norm(sols[0] - sols[1]) / torch.linalg.vector_norm(sols[1])) < 1e-8


@pytest.mark.parametrize("m", [32, 64, 128])
def test_multi_column_product(beam, m):
    """fl_MaskedMatMatBlocksF32 (the warm start's K Phi): FP32 values and columns against scipy's
    FP64 product, fixed rows zero."""
    import scipy.sparse as sp
    from florence_gb300 import _native as N
    from florence_gb300.assembly import _ptr, _stream
    asm, P, fixed, f, pat = beam
    V, _ = asm.assemble(torch.from_numpy(P).cuda())
    n = P.size
    free = ~fixed.astype(bool)
    X = np.random.default_rng(m).standard_normal((n, m)) * free[:, None]
    X32 = torch.from_numpy(X).float().cuda().contiguous()
    Y = torch.empty_like(X32)
    fx = torch.from_numpy(fixed.astype(np.int8)).cuda()
    V32 = V.float().contiguous()
    N.check(N.lib().fl_MaskedMatMatBlocksF32(_ptr(asm.indptr), _ptr(asm.indices), _ptr(V32), n, _ptr(fx), _ptr(X32),
                                             _ptr(Y), m, _stream()), "fl_MaskedMatMatBlocksF32")
    K = sp.csr_matrix((V.cpu().numpy(), asm.indices.cpu().numpy(), asm.indptr.cpu().numpy()), shape=(n, n))
    ref = (K @ X32.double().cpu().numpy()) * free[:, None]
    got = Y.double().cpu().numpy()
    assert np.all(got[~free] == 0.0)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
