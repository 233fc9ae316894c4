"""GPU tests of Newton's linear step (block-Jacobi PCG) and of the Newton load stepping, against
CPU references built from the oracle assembly and scipy's direct solver on the reduced system
(the reference's own approach: BoundaryCondition.GetReducedMatrices + LinearSolver, see
Florence/Solver/FEMSolver.py:951-954).

Tolerances: PCG solution 1e-8 relative (run to 1e-12); converged Newton displacement 1e-8
relative (the benchmark spec's bar for the converged displacement).
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_beam():
    from florence_gb300.newton import build_beam_problem
    return build_beam_problem(nx=8, ny=2, nz=2, traction=0.01)


def _asm(P, el, Jm, w):
    import florence_gb300 as fl
    return fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode="csr")


@pytest.mark.parametrize("spmv", ["fp64", "split"])
def test_pcg_matches_direct_solve(small_beam, spmv):
    """Both FP64-valued products: FP64 arithmetic and the float-pair split on the FP32 pipe."""
    from florence_gb300.newton import pcg
    P, el, Jm, w, fixed, f = small_beam
    asm = _asm(P, el, Jm, w)
    V, T = asm.assemble(torch.from_numpy(P).cuda())
    n = P.shape[0] * 3
    rng = np.random.default_rng(5)
    b = rng.standard_normal(n)
    b[fixed] = 0.0
    x, its, rel = pcg(asm, V, torch.from_numpy(b).cuda(), torch.from_numpy(fixed.astype(np.int8)).cuda(),
                      rtol=1e-12, maxiter=20000, spmv=spmv)
    assert rel <= 1e-12 and its > 0
    K = sp.csr_matrix((V.cpu().numpy(), asm.indices.cpu().numpy(), asm.indptr.cpu().numpy()), shape=(n, n))
    free = ~fixed
    xr = spla.spsolve(K[free][:, free].tocsc(), b[free])
    xg = x.cpu().numpy()
    assert np.all(xg[fixed] == 0.0)
    assert rel_fro(xg[free], xr) < 1e-8


@pytest.mark.parametrize("spmv", ["fp64", "split"])
def test_pcg_device_loop_matches_host_loop(small_beam, spmv):
    """The iterations as one CUDA graph (conditional WHILE node, the default) and launched from the
    host with a poll every 16 iterations: the same kernels in the same order, so the same
    iteration count (up to the order of the FP64 atomic adds of the dot products' block sums) and
    the same solution; and the maximum-iteration stop holds in the device loop (a count that is
    not a multiple of the host's poll interval)."""
    from florence_gb300.newton import get_pcg_device_loop, pcg, set_pcg_device_loop
    P, el, Jm, w, fixed, f = small_beam
    asm = _asm(P, el, Jm, w)
    V, _ = asm.assemble(torch.from_numpy(P).cuda())
    n = P.shape[0] * 3
    b = torch.from_numpy(np.where(fixed, 0.0, np.random.default_rng(7).standard_normal(n))).cuda()
    fx = torch.from_numpy(fixed.astype(np.int8)).cuda()
    assert get_pcg_device_loop()
    xd, itd, reld = pcg(asm, V, b, fx, rtol=1e-10, maxiter=20000, spmv=spmv)
    try:
        set_pcg_device_loop(False)
        xh, ith, relh = pcg(asm, V, b, fx, rtol=1e-10, maxiter=20000, spmv=spmv)
    finally:
        set_pcg_device_loop(True)
    assert abs(itd - ith) <= 2 and itd > 16 and reld <= 1e-10 and relh <= 1e-10
    assert rel_fro(xd.cpu().numpy(), xh.cpu().numpy()) < 1e-8
    x7, it7, rel7 = pcg(asm, V, b, fx, rtol=1e-30, maxiter=37, spmv=spmv)
    assert it7 == 37 and rel7 > 1e-10


def test_pcg_zero_rhs_returns_immediately(small_beam):
    from florence_gb300.newton import pcg
    P, el, Jm, w, fixed, f = small_beam
    asm = _asm(P, el, Jm, w)
    V, _ = asm.assemble(torch.from_numpy(P).cuda())
    x, its, rel = pcg(asm, V, torch.zeros(P.shape[0] * 3, dtype=torch.float64, device="cuda"),
                      torch.from_numpy(fixed.astype(np.int8)).cuda())
    assert its == 0 and float(x.abs().sum()) == 0.0


def cpu_newton(P, el, Jm, w, fixed, f, n_inc, tol, oracle):
    """Reference-style Newton on the CPU: oracle CSR assembly, direct solve of the reduced system."""
    spa = oracle.sparsity(el, P.shape[0])
    ind, ptr = spa[0], spa[1]
    n = P.shape[0] * 3
    free = ~fixed
    u = np.zeros(n)

    def assemble(u):
        V, T = oracle.assemble_df("MooneyRivlin", (0.5, 0.5, 20.0), P, el, P + u.reshape(-1, 3), Jm, w, mode="csr",
                                  sparsity_arrays=spa, nthreads=oracle.max_threads())
        return sp.csr_matrix((V, ind, ptr), shape=(n, n)), T

    K, T = assemble(u)
    iters = []
    for inc in range(1, n_inc + 1):
        F = f * inc / n_inc
        R = np.where(free, T - F, 0.0)
        it = 0
        while True:
            du = np.zeros(n)
            du[free] = spla.spsolve(K[free][:, free].tocsc(), -R[free])
            u += du
            K, T = assemble(u)
            R = np.where(free, T - F, 0.0)
            a = np.linalg.norm(R)
            if it == 0:
                nf = a
            if a < tol:
                break
            it += 1
            if a / nf <= tol or it > 25:
                break
        iters.append(it)
    return u, iters


def test_newton_matches_cpu_reference(small_beam, oracle):
    from florence_gb300.newton import NewtonSolver
    P, el, Jm, w, fixed, f = small_beam
    asm = _asm(P, el, Jm, w)
    solver = NewtonSolver(asm, fixed, f, n_increments=3, tol=1e-10)
    out = solver.solve()
    assert not out["failed"]
    for inc in out["increments"]:
        assert inc["history"][-1]["rel"] <= 1e-10 or inc["history"][-1]["abs"] < 1e-10
    u_ref, iters_ref = cpu_newton(P, el, Jm, w, fixed, f, 3, 1e-10, oracle)
    u = out["u"].cpu().numpy()
    assert rel_fro(u, u_ref) < 1e-8
    # tip deflection is a genuine bending response (nonlinear regime, not a tiny perturbation)
    tip = np.abs(P[:, 0] - 4.0) < 1e-9
    assert u.reshape(-1, 3)[tip, 2].mean() < -0.05
