"""Device-resident Newton-Raphson load stepping on top of the GPU assembly and PCG.

Mirrors the reference's static solver (Florence/Solver/FEMSolver.py:841-929 StaticSolver and
:932-1045 NewtonRaphson): the load is applied in equal increments; in each increment Newton
iterates  solve K du = -R,  u += du,  re-assemble K and T,  R = T - F  on the free dofs, with the
reference's convergence test -- the residual norm relative to its value after the first update of
the increment (NormForces, :983-997), or the absolute norm below the tolerance (:1001-1002) --
and its failure flags (maximum iterations, NaN or relative residual above 1e6, :1009-1021).

Differences by design: the Dirichlet dofs are masked instead of sliced out of the CSR matrix, and
the linear step is the device FP64 block-Jacobi PCG (fl_BlockJacobiPCG) with an inexact-Newton
forcing term, instead of a direct solver. Everything stays on the GPU; only scalars (norms,
iteration counts) reach the host. With tangent="mixed" the Jacobian is the tensor-core tangent
in FP32 (fl_GlobalAssemblyDF_Mixed) while the residual, the convergence test and the PCG
arithmetic stay FP64, so the converged state is that of the FP64 residual.
"""
import ctypes
import time

import numpy as np
import torch

from . import _native as N
from .assembly import DeviceAssembler, _ptr, _stream


def pcg_value_mode(V, spmv="split"):
    """fl_BlockJacobiPCG value mode of CSR values V: FP32 values -> FL_PCG_F32; FP64 values ->
    FL_PCG_F64_SPLIT (float-pair product on the FP32 pipe, spmv="split") or FL_PCG_F64."""
    if V.dtype == torch.float32:
        return N.FL_PCG_F32
    if spmv not in ("split", "fp64"):
        raise ValueError("spmv must be 'split' or 'fp64'")
    return N.FL_PCG_F64_SPLIT if spmv == "split" else N.FL_PCG_F64


def set_pcg_device_loop(enable=True):
    """PCG iterations as one CUDA graph with a device-side loop (the default), or launched from the
    host with a convergence poll every 16 iterations."""
    N.check(N.lib().fl_SetPCGDeviceLoop(1 if enable else 0), "fl_SetPCGDeviceLoop")


def get_pcg_device_loop():
    return bool(N.lib().fl_GetPCGDeviceLoop())


def pcg_workspace(asm, V, spmv="split"):
    L = N.lib()
    size = L.fl_BlockJacobiPCG_workspace_size(asm.nnode * 3, asm.nnz, pcg_value_mode(V, spmv))
    return torch.empty(size, dtype=torch.uint8, device=asm.device)


def pcg(asm, V, b, fixed, x=None, rtol=1e-8, maxiter=20000, workspace=None, spmv="split"):
    """Solves K_ff x = b_f with the CSR values V of `asm`'s pattern. Returns (x, iterations, relres)."""
    L = N.lib()
    n = asm.nnode * 3
    if x is None:
        x = torch.zeros(n, dtype=torch.float64, device=asm.device)
    if workspace is None:
        workspace = pcg_workspace(asm, V, spmv)
    it = ctypes.c_int64(0)
    rel = ctypes.c_double(0.0)
    bits = pcg_value_mode(V, spmv)
    st = L.fl_BlockJacobiPCG(_ptr(asm.indptr), _ptr(asm.indices), _ptr(V), bits, n, _ptr(fixed), _ptr(b), _ptr(x),
                             float(rtol), int(maxiter), _ptr(workspace), workspace.numel(), ctypes.byref(it),
                             ctypes.byref(rel), _stream())
    N.check(st, "fl_BlockJacobiPCG")
    return x, it.value, rel.value


class NewtonSolver:
    """Static load stepping for a mesh held by a DeviceAssembler (csr mode).

    fixed: bool/uint8 [3N] (Dirichlet dofs, prescribed value 0); f_ext: [3N] total external load.
    """

    def __init__(self, asm, fixed, f_ext, n_increments=10, tol=1e-10, max_iter=25, pcg_maxiter=50000,
                 eta_max=1e-2, eta_min=1e-12, tangent="fp64", criterion="reference", spmv="split",
                 forcing="ew", eta0=1e-3, hybrid_switch=1e-2, linear="pcg", pattern=None):
        if asm.mode != "csr":
            raise ValueError("Newton needs the CSR tangent (mode='csr')")
        self.asm = asm
        dev = asm.device
        self.fixed = torch.as_tensor(np.asarray(fixed, dtype=np.int8), device=dev).contiguous()
        self.free = (self.fixed == 0).to(torch.float64)
        self.f_ext = torch.as_tensor(np.asarray(f_ext, dtype=np.float64), device=dev).contiguous()
        self.n_increments = n_increments
        self.tol = tol
        self.max_iter = max_iter
        self.pcg_maxiter = pcg_maxiter
        self.eta_max = eta_max
        self.eta_min = eta_min
        self.X = asm.points.reshape(-1)
        n = asm.nnode * 3
        if tangent not in ("fp64", "mixed", "hybrid"):
            raise ValueError("tangent must be 'fp64', 'mixed' or 'hybrid'")
        # "hybrid": the split-BF16 tensor-core Jacobian (FP32 values) while the residual is above
        # hybrid_switch x the increment's load, the FP64 Jacobian below. Far from the solution
        # the FP32 Jacobian's error (~1e-7 relative, amplified by the condition number) is small
        # against the Newton step's own linearisation error, and its PCG products move half the
        # bytes; close to the solution it would turn Newton's quadratic convergence linear.
        self.tangent = tangent
        self.hybrid_switch = hybrid_switch
        if criterion not in ("reference", "load"):
            raise ValueError("criterion must be 'reference' or 'load'")
        # "reference": |R| relative to its value after the first update of the increment (the
        # reference's NormForces); "load": |R| relative to the increment's external load, a test
        # that does not depend on how good the initial state was (used to compare warm starts)
        self.criterion = criterion
        self.V64 = torch.zeros(asm.nnz, dtype=torch.float64, device=dev) if tangent != "mixed" else None
        self.V32 = torch.zeros(asm.nnz, dtype=torch.float32, device=dev) if tangent != "fp64" else None
        self.V = self.V64 if tangent != "mixed" else self.V32
        self.T = torch.zeros(n, dtype=torch.float64, device=dev)
        self.spmv = spmv
        if forcing not in ("ew", "rel"):
            raise ValueError("forcing must be 'ew' or 'rel'")
        # PCG tolerance of each Newton step. "rel": 0.1 x the relative residual. "ew":
        # Eisenstat-Walker (choice 2, gamma 0.9, alpha 2): the square of the last residual
        # reduction, so that a Jacobian that only converges linearly (the FP32 tangent) is not
        # solved far below what its own error allows, with the standard safeguards, and never
        # below half of what the convergence test still needs.
        self.forcing = forcing
        self.eta0 = eta0
        self.ws = pcg_workspace(asm, self.V, spmv)   # the FP64 workspace is the larger one
        self.history = []
        # linear step: "pcg" (block-Jacobi PCG, fl_BlockJacobiPCG) or "pmg" (flexible CG with the
        # two-level p-multigrid cycle of multigrid.PMultigrid; FP64 tangent, high-order tets,
        # `pattern` = the element's barycentric node layout)
        if linear not in ("pcg", "pmg"):
            raise ValueError("linear must be 'pcg' or 'pmg'")
        self.mg = None
        if linear == "pmg":
            if tangent != "fp64" or pattern is None:
                raise ValueError("the p-multigrid linear step takes the FP64 tangent and the element's node pattern")
            from .multigrid import PMultigrid
            self.mg = PMultigrid(asm, pattern, np.asarray(fixed, dtype=np.int8))

    def _assemble(self, u, mixed=None):
        """Tangent and residual at u; mixed selects the FP32 tensor-core Jacobian (default: as
        the tangent option says; "hybrid" keeps the Jacobian it currently uses)."""
        if mixed is None:
            mixed = self.tangent == "mixed" or (self.tangent == "hybrid" and self.V is self.V32)
        self.V = self.V32 if mixed else self.V64
        self.V.zero_()
        self.T.zero_()
        if not mixed:
            self.asm.assemble((self.X + u).reshape(-1, 3), V=self.V, T=self.T)
        else:  # FP32 Jacobian from the tensor cores, FP64 residual
            self.asm.assemble_mixed((self.X + u).reshape(-1, 3), V32=self.V, T=self.T)

    def _set_jacobian(self, u, absn, ref):
        """hybrid: the FP32 Jacobian while |R| > hybrid_switch * ref, FP64 below (re-assembles
        at u when the choice changes)."""
        if self.tangent != "hybrid":
            return
        want_mixed = absn > self.hybrid_switch * ref
        if want_mixed != (self.V is self.V32):
            self._assemble(u, mixed=want_mixed)

    def residual_norm(self, F):
        return float(torch.linalg.vector_norm((self.T - F) * self.free))

    def _iterate(self, u, F):
        """Newton iterations of one increment from u (tangent and residual at u assembled).
        Returns (u, iteration log, failed, PCG iterations)."""
        R = (self.T - F) * self.free
        norm_load = float(torch.linalg.vector_norm(F * self.free))
        norm_forces = None
        it = 0
        eta = self.eta0
        r_before = float(torch.linalg.vector_norm(R))
        iters = []
        pcg_total = 0
        failed = False
        while True:
            self._set_jacobian(u, r_before, norm_load)
            if self.mg is not None:
                from .multigrid import fcg
                self.mg.update(self.V, u)
                du, pits, prel = fcg(self.mg, -R, rtol=eta, maxiter=self.pcg_maxiter)
            else:
                du, pits, prel = pcg(self.asm, self.V, -R, self.fixed, rtol=eta, maxiter=self.pcg_maxiter,
                                     workspace=self.ws, spmv=self.spmv)
            pcg_total += pits
            u += du
            self._assemble(u)
            R = (self.T - F) * self.free
            absn = float(torch.linalg.vector_norm(R))
            if self.criterion == "load":
                norm_forces = norm_load if norm_load != 0.0 else 1.0
            elif it == 0:
                norm_forces = absn if absn != 0.0 else 1e-14
            rel = abs(absn / norm_forces)
            iters.append(dict(iter=it, abs=absn, rel=rel, pcg_iters=pits, pcg_relres=prel, eta=eta,
                              jacobian="fp32" if self.V is self.V32 else "fp64"))
            if absn < self.tol:
                break
            it += 1
            if rel <= self.tol and (it > 0 or self.criterion == "load"):
                break
            if it >= self.max_iter or not np.isfinite(rel) or rel > 1e6:
                failed = True
                break
            if self.forcing == "rel":
                # solve to a tolerance proportional to the current relative residual
                eta = float(min(self.eta_max, max(self.eta_min, 0.1 * rel)))
            else:
                e_new = 0.9 * (absn / r_before) ** 2 if r_before > 0 else self.eta_max
                if 0.9 * eta ** 2 > 0.1:
                    e_new = max(e_new, 0.9 * eta ** 2)
                e_new = min(self.eta_max, e_new)
                e_new = max(e_new, 0.5 * self.tol * norm_forces / absn)
                eta = float(min(self.eta_max, max(self.eta_min, e_new)))
            r_before = absn
        return u, iters, failed, pcg_total

    def solve(self, u0=None, guesses=None, keep_states=False):
        """Runs all increments. guesses: optional callable(increment, u_prev) -> candidate initial
        u for the increment (a warm start), a list of candidates, or None. The candidate with the
        smallest FP64 residual is kept if that residual is below the previous increment's
        solution's (the default start) and no element of it is inverted; otherwise the solver
        falls back to the previous solution, and it restarts the increment from there if Newton
        fails from a candidate. keep_states: also return each increment's converged displacement
        (device FP64) under increments[k]["u"]. Returns a dict."""
        dev = self.asm.device
        n = self.asm.nnode * 3
        u = torch.zeros(n, dtype=torch.float64, device=dev) if u0 is None else u0.clone()
        self._assemble(u)
        t0 = time.perf_counter()
        total_newton = 0
        total_pcg = 0
        failed = False
        incs = []
        for inc in range(1, self.n_increments + 1):
            F = self.f_ext * (inc / self.n_increments)
            guess = "previous"
            u_prev = u
            if guesses is not None:
                cands = guesses(inc, u)
                if cands is not None:
                    if isinstance(cands, torch.Tensor):
                        cands = [cands]
                    # the FP64 residual judges every candidate (one with an inverted element,
                    # det F <= 0, is rejected); the previous solution is the fallback
                    best, best_r, best_k = u, self.residual_norm(F), -1
                    for k, g in enumerate(cands):
                        self.asm.flags.zero_()
                        self._assemble(g)
                        r = self.residual_norm(F)
                        if int(self.asm.flags.item()) & N.FL_FLAG_NONPOSITIVE_J:
                            r = np.inf
                        if r < best_r:
                            best, best_r, best_k = g, r, k
                    self.asm.flags.zero_()
                    u = best.clone()
                    if best_k != len(cands) - 1:  # the tangent and residual of the chosen state
                        self._assemble(u)
                    guess = "fallback" if best_k < 0 else "candidate%d" % best_k
            if guess.startswith("candidate"):
                u_keep = u_prev.clone()
            u, iters, inc_failed, pits = self._iterate(u, F)
            total_pcg += pits
            if inc_failed and guess.startswith("candidate"):
                # Newton did not converge from the prediction: restart from the previous solution
                u = u_keep
                self._assemble(u)
                u, iters2, inc_failed, pits = self._iterate(u, F)
                total_pcg += pits
                iters = iters + iters2
                guess = "restarted"
            total_newton += len(iters)
            incs.append(dict(increment=inc, newton_iters=len(iters), history=iters, guess=guess))
            if keep_states:
                incs[-1]["u"] = u.clone()
            if inc_failed:
                failed = True
                break
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        self.history = incs
        out = dict(u=u, wall_s=wall, newton_iters=total_newton, pcg_iters=total_pcg, failed=failed,
                   increments=incs)
        if self.mg is not None:
            out.update(mg_cycles=self.mg.cycles, mg_coarse_iters=self.mg.coarse_iters)
        return out


# ------------------------------------------------------------------------------------------------
# Neumann loads on tetrahedral boundary faces (host preprocessing, once per mesh)
# ------------------------------------------------------------------------------------------------

def _triangle_rule(n=5):
    """Collapsed Gauss rule on the reference triangle {s,t >= 0, s+t <= 1} (exact to degree 2n-2)."""
    x, w = np.polynomial.legendre.leggauss(n)
    x = (x + 1) / 2
    w = w / 2
    S, T, W = [], [], []
    for i in range(n):
        for j in range(n):
            S.append(x[i])
            T.append(x[j] * (1 - x[i]))
            W.append(w[i] * w[j] * (1 - x[i]))
    return np.array(S), np.array(T), np.array(W)


def _face_weights(st):
    """Integrals of the Lagrange basis on the face nodes st [m,2] over the reference triangle,
    divided by its area (they sum to 1)."""
    m = st.shape[0]
    deg = int(round((np.sqrt(8 * m + 1) - 3) / 2))
    mons = [(i, j) for i in range(deg + 1) for j in range(deg + 1 - i)]
    Vm = np.array([[s ** i * t ** j for (i, j) in mons] for s, t in st])
    Cinv = np.linalg.inv(Vm)  # basis_a(s,t) = sum_k Cinv[k,a] mon_k(s,t)
    S, T, W = _triangle_rule(deg + 3)
    mon_int = np.array([np.sum(W * S ** i * T ** j) for (i, j) in mons])
    return (mon_int @ Cinv) / 0.5


def tet_face_loads(points, elements, pattern, on_face, traction):
    """Consistent nodal forces of a uniform dead-load traction on the boundary faces whose three
    vertices satisfy on_face(X) (X: [3] coordinates). pattern: barycentric node layout [npe,4].
    Returns f [3N]."""
    P = np.asarray(points)
    el = np.asarray(elements, dtype=np.int64)
    lam = np.asarray(pattern)
    f = np.zeros(P.shape[0] * 3)
    tr = np.asarray(traction, dtype=np.float64)
    vmask = np.array([[bool(on_face(P[el[e, v]])) for v in range(4)] for e in range(el.shape[0])])
    cache = {}
    for e in np.nonzero(vmask.sum(1) >= 3)[0]:
        for opp in range(4):
            verts = [v for v in range(4) if v != opp]
            if not all(vmask[e, v] for v in verts):
                continue
            nodes = np.nonzero(np.abs(lam[:, opp]) < 1e-10)[0]
            if opp not in cache:
                st = lam[nodes][:, verts[1:]]  # (lambda of 2nd and 3rd face vertex) as (s, t)
                cache[opp] = (nodes, _face_weights(st))
            nodes, wts = cache[opp]
            A = P[el[e, verts]]
            area = 0.5 * np.linalg.norm(np.cross(A[1] - A[0], A[2] - A[0]))
            for a, wa in zip(nodes, wts):
                f[3 * el[e, a]:3 * el[e, a] + 3] += tr * area * wa
    return f


def build_beam_problem(nx=48, ny=12, nz=12, traction=0.01, seed=1):
    """The Newton configuration: p=3 tet beam 4x1x1 (jittered lattice, Delaunay), Mooney-Rivlin
    mu1 = mu2 = 0.5, lambda = 20, x=0 clamped, uniform downward traction on x=4. Returns
    (points, elements, Jm, AllGauss, fixed [3N] bool, f_ext [3N])."""
    import os
    from . import meshes
    here = os.path.dirname(os.path.abspath(__file__))
    t = np.load(os.path.join(here, "..", "tests", "golden", "tet_p3_mr_jitter.npz"))
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((nx, ny, nz), (4.0, 1.0, 1.0), seed, pat)
    fixed = np.repeat(np.abs(P[:, 0]) < 1e-9, 3)
    f = tet_face_loads(P, el, pat, lambda X: abs(X[0] - 4.0) < 1e-9, (0.0, 0.0, -traction))
    return P, el, t["Jm"], t["AllGauss"], fixed, f
