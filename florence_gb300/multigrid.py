"""Two-level p-multigrid preconditioner and flexible CG for Newton's linear step on high-order
tetrahedra (no reference counterpart: the reference reduces the system and calls a direct solver
or scipy's iterative solvers, Florence/Solver/LinearSolver.py:153-330; its AMG option,
:153-173, is the kind of preconditioner this replaces).

Levels: the assembled high-order tangent (fine) and the linear (p=1) tangent of the same mesh on
its vertices (coarse), assembled by the same GPU assembler at the current deformation (the
rediscretised coarse operator of p-multigrid). Transfers: a fine node's value is its element's
vertex values interpolated at the node's barycentric coordinates (prolongation); the restriction
is the transpose. One cycle, for a residual r:

    z  = Chebyshev(block-Jacobi) smoothing of K z = r from z = 0   (degree `nu`)
    z += P  CG_coarse( R (r - K z) )                              (coarse correction)
    z  = Chebyshev smoothing of K z = r from z                     (degree `nu`)

with the Dirichlet dofs masked on both levels. The coarse solve is a block-Jacobi PCG to a
loose tolerance, which makes the cycle a (mildly) nonlinear operator; the outer iteration is
therefore flexible CG (Notay, SIAM J. Sci. Comput. 22, 2000: the Polak-Ribiere form of beta).
Chebyshev smoothing over [lmax / ratio, lmax] of the block-Jacobi preconditioned tangent follows
Adams, Brezina, Hu and Tuminaro (J. Comput. Phys. 188, 2003); lmax comes from the Lanczos
matrix of a few block-Jacobi PCG iterations per tangent.

Everything runs on the GPU through the library's kernels (fl_MaskedMatVec, fl_BlockJacobiApply,
fl_NodalTransfer, the assembly, and the coarse block-Jacobi PCG in one cooperative launch,
fl_CoarsePCG); vector updates and dot products are torch operations on the same stream, and the
outer iteration reads one scalar (|r|) per iteration on the host.
"""
import numpy as np
import torch

from . import _native as N
from .assembly import DeviceAssembler, _ptr, _stream


def p1_tables():
    """(Jm, AllGauss) of the reference's linear tetrahedron (taken from the golden fixtures)."""
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    d = np.load(os.path.join(here, "..", "tests", "golden", "tet_p1_nh.npz"))
    return d["Jm"], np.ravel(d["AllGauss"])


def vertex_transfer(elements, pattern, nnode):
    """Coarse (vertex) numbering and the transfer operators of a high-order tet mesh.

    elements [E, npe] with the four vertices first; pattern [npe, 4] barycentric coordinates of
    the local nodes. Returns (verts [nc] fine ids of the vertices, coarse elements [E, 4],
    P = (ptr, cols, w) over fine nodes, R = (ptr, cols, w) over coarse nodes)."""
    el = np.asarray(elements, np.int64)
    pat = np.asarray(pattern, np.float64)
    npe = el.shape[1]
    verts = np.unique(el[:, :4])
    cmap = np.full(nnode, -1, np.int64)
    cmap[verts] = np.arange(verts.shape[0])
    _, first = np.unique(el.ravel(), return_index=True)      # first (element, local node) of each node
    if first.shape[0] != nnode:
        raise ValueError("every node must belong to an element")
    e, a = first // npe, first % npe
    W = pat[a]                                                # [nnode, 4]
    C = cmap[el[e, :4]]                                       # [nnode, 4]
    keep = np.abs(W) > 1e-13
    counts = keep.sum(1)
    p_ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    p_cols = C[keep].astype(np.int32)
    p_w = W[keep]
    rows = np.repeat(np.arange(nnode), counts)
    order = np.argsort(p_cols, kind="stable")
    r_counts = np.bincount(p_cols, minlength=verts.shape[0])
    r_ptr = np.concatenate([[0], np.cumsum(r_counts)]).astype(np.int32)
    r_cols = rows[order].astype(np.int32)
    r_w = p_w[order]
    return verts, cmap[el[:, :4]], (p_ptr, p_cols, p_w), (r_ptr, r_cols, r_w)


class PMultigrid:
    """The two-level preconditioner for a fine DeviceAssembler (csr mode, high-order tets).

    pattern: barycentric layout of the element's nodes [npe, 4]; fixed: Dirichlet mask [3N];
    nu: Chebyshev degree of each smoothing; coarse_rtol / coarse_maxiter: the coarse PCG."""

    def __init__(self, asm, pattern, fixed, nu=3, ratio=30.0, coarse_rtol=0.1, coarse_maxiter=100,
                 power_iters=20):
        self.asm = asm
        dev = asm.device
        self.dev = dev
        self.n = asm.nnode * 3
        self.fixed = torch.as_tensor(np.asarray(fixed, np.int8).ravel(), device=dev).contiguous()
        el = asm.elements.cpu().numpy()
        verts, el_c, P, R = vertex_transfer(el, pattern, asm.nnode)
        self.verts = torch.from_numpy(verts).to(dev)
        dts = (torch.int32, torch.int32, torch.float64)
        self.P = tuple(torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt) for a, dt in zip(P, dts))
        self.R = tuple(torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt) for a, dt in zip(R, dts))
        Jm1, w1 = p1_tables()
        Pc = asm.points.cpu().numpy()[verts]
        self.coarse = DeviceAssembler(Pc, el_c, Jm1, w1, asm.material, asm.params, mode="csr", device=dev)
        self.nc = self.coarse.nnode * 3
        fx = np.asarray(fixed, np.int8).reshape(-1, 3)[verts].ravel()
        self.fixed_c = torch.from_numpy(fx).to(dev).contiguous()
        self.Vc = torch.zeros(self.coarse.nnz, dtype=torch.float64, device=dev)
        self.Tc = torch.zeros(self.nc, dtype=torch.float64, device=dev)
        self.Binv = torch.empty((asm.nnode, 9), dtype=torch.float64, device=dev)
        self.V32 = torch.empty(asm.nnz, dtype=torch.float32, device=dev)
        self.Vp = torch.empty(2 * asm.nnz, dtype=torch.float32, device=dev)   # the tangent as float pairs
        self._xp = torch.empty(2 * self.n, dtype=torch.float32, device=dev)
        self.Binv_c = torch.empty((self.coarse.nnode, 9), dtype=torch.float64, device=dev)
        self.nu, self.ratio, self.power_iters = nu, ratio, power_iters
        self.coarse_rtol, self.coarse_maxiter = coarse_rtol, coarse_maxiter
        self.flags = torch.zeros(1, dtype=torch.int32, device=dev)
        self.V = None
        self.lmax = None
        self.cycles = 0
        # the coarse solve (fl_CoarsePCG): its workspace, solution and iteration counter on the device
        self._cws = torch.empty(int(N.lib().fl_CoarsePCG_workspace_size(self.nc)), dtype=torch.uint8, device=dev)
        self._xc = torch.zeros(self.nc, dtype=torch.float64, device=dev)
        self._citers = torch.zeros(1, dtype=torch.int64, device=dev)
        # the one-launch coarse solve keeps each SM's share of the coarse rows in shared memory:
        # checked once here; a coarse system too large for it is solved by the block-Jacobi PCG
        # launched iteration by iteration (fl_BlockJacobiPCG) instead
        self._coarse_fast = True
        self._pcg_ws = None
        saved = self.coarse_maxiter
        self.coarse_maxiter = 0
        self.coarse_solve(torch.zeros(self.nc, dtype=torch.float64, device=dev))
        self.coarse_maxiter = saved
        if int(self.flags.item()) & N.FL_FLAG_CAPACITY:
            self._coarse_fast = False
        self.flags.zero_()

    @property
    def coarse_iters(self):
        """Coarse PCG iterations of every cycle so far (reads a device counter)."""
        return int(self._citers.item())

    # -- kernels ------------------------------------------------------------------------------
    def matvec(self, x, y, b=None):
        """y = K_ff x (or b - K_ff x) with the fine tangent; x is zero on the fixed dofs (every
        vector of the cycle and of the outer iteration is). The tangent and x as float pairs
        (~2^-44 relative, FP32 pipe)."""
        L = N.lib()
        N.check(L.fl_SplitPairs(self.n, _ptr(x), _ptr(self._xp), _stream()), "fl_SplitPairs")
        N.check(L.fl_MaskedMatVecBlocksPair(_ptr(self.asm.indptr), _ptr(self.asm.indices), _ptr(self.Vp), self.n,
                                            _ptr(self.fixed), _ptr(self._xp), _ptr(b), _ptr(y), _stream()),
                "fl_MaskedMatVecBlocksPair")
        return y

    def smooth_matvec(self, x, y, b=None):
        """The same product with the tangent's FP32 copy, for the smoother, the residual restricted to
        the coarse level and the Chebyshev interval (the cycle is a preconditioner: the outer
        iteration's products stay FP64)."""
        N.check(N.lib().fl_MaskedMatVecBlocksF32(_ptr(self.asm.indptr), _ptr(self.asm.indices), _ptr(self.V32),
                                                 self.n, _ptr(self.fixed), _ptr(x), _ptr(b), _ptr(y), _stream()),
                "fl_MaskedMatVecBlocksF32")
        return y

    def jacobi(self, r, z, omega=1.0, accumulate=False):
        N.check(N.lib().fl_BlockJacobiApply(self.asm.nnode, _ptr(self.Binv), _ptr(self.fixed), float(omega), _ptr(r),
                                            _ptr(z), 1 if accumulate else 0, _stream()), "fl_BlockJacobiApply")
        return z

    def prolong_add(self, xc, y):
        ptr, cols, w = self.P
        N.check(N.lib().fl_NodalTransfer(self.asm.nnode, _ptr(ptr), _ptr(cols), _ptr(w), _ptr(xc), _ptr(y), 1,
                                         _stream()), "fl_NodalTransfer")

    def restrict(self, r, rc):
        ptr, cols, w = self.R
        N.check(N.lib().fl_NodalTransfer(self.coarse.nnode, _ptr(ptr), _ptr(cols), _ptr(w), _ptr(r), _ptr(rc), 0,
                                         _stream()), "fl_NodalTransfer")

    # -- set-up per tangent ---------------------------------------------------------------------
    def update(self, V, u):
        """New fine tangent values V (FP64, the fine pattern) at displacement u [3N]: block
        inverses, the largest eigenvalue estimate, the coarse tangent at the vertices."""
        self.V = V
        self.V32.copy_(V)
        N.check(N.lib().fl_SplitPairs(self.asm.nnz, _ptr(V), _ptr(self.Vp), _stream()), "fl_SplitPairs")
        N.check(N.lib().fl_BlockJacobiInverse(_ptr(self.asm.indptr), _ptr(self.asm.indices), _ptr(V), self.asm.nnode,
                                              _ptr(self.fixed), _ptr(self.Binv), _ptr(self.flags), _stream()),
                "fl_BlockJacobiInverse")
        self.lmax = 1.05 * self._lanczos_lmax(self.power_iters)
        # coarse tangent at the vertices' current coordinates
        uc = u.reshape(-1, 3)[self.verts]
        self.Vc.zero_()
        self.Tc.zero_()
        self.coarse.assemble((self.coarse.points + uc).contiguous(), V=self.Vc, T=self.Tc)
        c = self.coarse
        N.check(N.lib().fl_BlockJacobiInverse(_ptr(c.indptr), _ptr(c.indices), _ptr(self.Vc), c.nnode,
                                              _ptr(self.fixed_c), _ptr(self.Binv_c), _ptr(self.flags), _stream()),
                "fl_BlockJacobiInverse")

    def _lanczos_lmax(self, steps):
        """Largest eigenvalue of B^-1 K_ff, the top of the Chebyshev interval: `steps` iterations
        of block-Jacobi PCG from a random right-hand side, and the largest eigenvalue of the
        Lanczos tridiagonal matrix their coefficients define (Golub and Van Loan, Matrix
        Computations, section 11.3.5). It approaches the extreme eigenvalues much faster than
        power iterations, which under-estimated it on the 95 M-nonzero beam and let the
        smoother amplify the modes above the estimate. One host read at the end."""
        g = torch.Generator(device=self.dev).manual_seed(0)
        r = torch.rand(self.n, dtype=torch.float64, device=self.dev, generator=g) * (self.fixed == 0)
        z = self.jacobi(r, torch.empty_like(r))
        p = z.clone()
        q = torch.empty_like(r)
        rz = torch.dot(r, z)
        alphas, betas = [], []
        for _ in range(steps):
            self.smooth_matvec(p, q)
            alpha = rz / torch.dot(p, q)
            r.sub_(alpha * q)
            self.jacobi(r, z)
            rz_new = torch.dot(r, z)
            beta = rz_new / rz
            p.mul_(beta).add_(z)
            rz = rz_new
            alphas.append(alpha)
            betas.append(beta)
        a = torch.stack(alphas).cpu().numpy()
        bt = torch.stack(betas).cpu().numpy()
        m = len(a)
        T = np.zeros((m, m))
        for j in range(m):
            T[j, j] = 1.0 / a[j] + (bt[j - 1] / a[j - 1] if j > 0 else 0.0)
            if j + 1 < m:
                T[j, j + 1] = T[j + 1, j] = np.sqrt(max(bt[j], 0.0)) / a[j]
        ev = np.linalg.eigvalsh(T)
        return float(ev[-1]) if np.isfinite(ev[-1]) and ev[-1] > 0 else 1.0

    # -- the cycle --------------------------------------------------------------------------------
    def _chebyshev(self, r, z, first):
        """nu Chebyshev steps on B^-1 K z = B^-1 r over [lmax / ratio, lmax], from z (z = 0 when
        first: the initial residual is r itself)."""
        lmax = self.lmax
        lmin = lmax / self.ratio
        theta, delta = 0.5 * (lmax + lmin), 0.5 * (lmax - lmin)
        sigma = theta / delta
        rho = 1.0 / sigma
        res = torch.empty_like(r)
        d = torch.empty_like(r)
        if first:
            self.jacobi(r, d, 1.0 / theta)
            z.zero_()
        else:
            self.smooth_matvec(z, res, b=r)
            self.jacobi(res, d, 1.0 / theta)
        z += d
        for _ in range(1, self.nu):
            rho_new = 1.0 / (2.0 * sigma - rho)
            self.smooth_matvec(z, res, b=r)
            d *= rho_new * rho
            self.jacobi(res, d, 2.0 * rho_new / delta, accumulate=True)
            z += d
            rho = rho_new
        return z

    def coarse_solve(self, rc):
        """The coarse correction: block-Jacobi PCG on the vertex tangent to coarse_rtol (at most
        coarse_maxiter iterations) in one cooperative launch; returns the device solution."""
        c = self.coarse
        if not self._coarse_fast:
            from .newton import pcg, pcg_workspace
            if self._pcg_ws is None:
                self._pcg_ws = pcg_workspace(c, self.Vc, "fp64")
            xc, it, _ = pcg(c, self.Vc, rc, self.fixed_c, rtol=self.coarse_rtol, maxiter=self.coarse_maxiter,
                            workspace=self._pcg_ws, spmv="fp64")
            self._citers += it
            return xc
        N.check(N.lib().fl_CoarsePCG(_ptr(c.indptr), _ptr(c.indices), _ptr(self.Vc), self.nc, _ptr(self.fixed_c),
                                     _ptr(self.Binv_c), _ptr(rc), _ptr(self._xc), float(self.coarse_rtol),
                                     int(self.coarse_maxiter), _ptr(self._cws), self._cws.numel(), _ptr(self._citers),
                                     None, _ptr(self.flags), _stream()), "fl_CoarsePCG")
        return self._xc

    def check_flags(self):
        f = int(self.flags.item())
        if f & N.FL_FLAG_TIMEOUT:
            raise N.FlorenceGB300Error(N.FL_ERR_CUDA, "p-multigrid coarse solve (a grid barrier wait gave up)")
        if f & N.FL_FLAG_BAD_INDEX:
            raise N.FlorenceGB300Error(N.FL_ERR_ARG, "p-multigrid (missing or singular diagonal block, or a "
                                                     "coarse tangent that is not positive definite)")

    def apply(self, r, z):
        """z = M^-1 r (one cycle)."""
        self._chebyshev(r, z, first=True)
        res = torch.empty_like(r)
        self.smooth_matvec(z, res, b=r)
        rc = torch.empty(self.nc, dtype=torch.float64, device=self.dev)
        self.restrict(res, rc)
        rc *= (self.fixed_c == 0)
        ec = self.coarse_solve(rc)
        self.cycles += 1
        self.prolong_add(ec, z)
        z *= (self.fixed == 0)
        self._chebyshev(r, z, first=False)
        return z


def fcg(mg, b, x=None, rtol=1e-8, maxiter=500):
    """Flexible preconditioned CG on K_ff x = b_f with the cycle of `mg` (its tangent set by
    mg.update). Returns (x, iterations, relative residual)."""
    free = (mg.fixed == 0).to(torch.float64)
    b = b * free
    if x is None:
        x = torch.zeros_like(b)
        r = b.clone()
    else:
        x = x * free
        r = mg.matvec(x, torch.empty_like(b), b=b)
    nb = float(torch.linalg.vector_norm(b))
    if nb == 0.0:
        return x, 0, 0.0
    z = torch.empty_like(b)
    q = torch.empty_like(b)
    p = None
    r_prev = torch.empty_like(b)
    it = 0
    rel = float(torch.linalg.vector_norm(r)) / nb
    # the scalars stay on the device (0-d tensors); the host reads |r| once per iteration
    while it < maxiter and rel > rtol:
        mg.apply(r, z)
        rz_new = torch.dot(r, z)
        if p is None:
            p = z.clone()
        else:
            beta = torch.dot(z, r - r_prev) / rz   # flexible (Polak-Ribiere) beta
            p.mul_(beta).add_(z)
        rz = rz_new
        mg.matvec(p, q)
        alpha = rz / torch.dot(p, q)
        x.add_(alpha * p)
        r_prev.copy_(r)
        r.sub_(alpha * q)
        it += 1
        rel = float(torch.linalg.vector_norm(r)) / nb
        if not np.isfinite(rel) or rel > 1e6:  # diverged (e.g. an indefinite smoother): let the caller fail
            break
    mg.check_flags()
    return x, it, rel
