"""Learned Newton warm start: POD basis + MLP on the GPU.

The method generates its own training data: converged increments of Newton solves over a range
of (material, load) parameters. A 64-mode POD basis of the converged displacements is built by
the method of snapshots, and an MLP 3 -> 256 -> 256 -> 64 (GELU, BF16 arithmetic, FP32 master
weights, Adam; kernels in csrc/fl_mlp.cu) maps three features of the parameters (t/mu, Poisson's
ratio, mu) to the POD coefficients of the displacement per unit load-to-stiffness ratio t/mu. At
solve time the prediction gives two candidate initial states for each increment (the predicted
state, and the previous solution moved by the predicted step); the FP64 residual judges them
against the previous-increment guess, which is the fallback.
"""
import time

import numpy as np
import torch

from . import _native as N
from .assembly import _ptr, _stream


class MLP:
    """The warm-start network; parameters and Adam state on the GPU."""

    def __init__(self, seed=0, device="cuda"):
        L = N.lib()
        self.device = torch.device(device)
        self.n = int(L.fl_MLP_num_params())
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n, np.float32)
        sizes = [(3, 256), (256,), (256, 256), (256,), (256, 64), (64,)]
        off = 0
        for s in sizes:
            k = int(np.prod(s))
            if len(s) == 2:  # He-style uniform init for GELU layers
                bound = np.sqrt(6.0 / s[0])
                p[off:off + k] = rng.uniform(-bound, bound, k).astype(np.float32)
            off += k
        self.params = torch.from_numpy(p).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grads = torch.zeros_like(self.params)
        self.step = 0
        self._ws = {}

    def _workspace(self, batch):
        if batch not in self._ws:
            self._ws[batch] = torch.empty(N.lib().fl_MLP_workspace_size(batch), dtype=torch.uint8, device=self.device)
        return self._ws[batch]

    def forward(self, x):
        x = x.to(self.device, torch.float32).contiguous()
        B = x.shape[0]
        y = torch.empty(B, 64, dtype=torch.float32, device=self.device)
        ws = self._workspace(B)
        N.check(N.lib().fl_MLPForward(_ptr(self.params), _ptr(x), B, _ptr(y), _ptr(ws), ws.numel(), _stream()),
                "fl_MLPForward")
        return y

    def gradients(self, x, t):
        x = x.to(self.device, torch.float32).contiguous()
        t = t.to(self.device, torch.float32).contiguous()
        B = x.shape[0]
        ws = self._workspace(B)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        N.check(N.lib().fl_MLPGradients(_ptr(self.params), _ptr(x), _ptr(t), B, _ptr(self.grads), _ptr(loss),
                                        _ptr(ws), ws.numel(), _stream()), "fl_MLPGradients")
        return self.grads, loss

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        N.check(N.lib().fl_MLPAdamStep(_ptr(self.params), _ptr(self.grads), _ptr(self.m), _ptr(self.v), self.step,
                                       lr, beta1, beta2, eps, _stream()), "fl_MLPAdamStep")

    def train(self, X, Y, steps=20000, batch=64, lr=2e-3, seed=0, lr_final=1e-5, log_every=100):
        """Adam on mini-batches drawn with replacement from (X [S,3], Y [S,64]) (device tensors),
        cosine learning-rate decay from lr to lr_final. Returns the mean loss of every
        `log_every` steps."""
        g = torch.Generator(device=self.device).manual_seed(seed)
        S = X.shape[0]
        batch = min(batch, S)
        hist = []
        tot = torch.zeros(1, device=self.device)
        for it in range(steps):
            idx = torch.randint(0, S, (batch,), generator=g, device=self.device)
            lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * it / max(1, steps - 1)))
            _, loss = self.gradients(X[idx], Y[idx])
            self.adam_step(lr=lr_t)
            tot += loss
            if (it + 1) % log_every == 0:
                hist.append(tot / log_every)
                tot = torch.zeros(1, device=self.device)
        return [float(h) for h in torch.cat(hist).cpu()] if hist else []


def pod_basis(U, modes=64):
    """Method of snapshots: U [n, S] (FP64, device) -> (Phi [n, modes], singular values [modes]).
    Modes whose singular value is below 1e-12 of the largest are numerically absent: their
    columns are zero (their coefficients are then zero too); the others are re-orthonormalised."""
    G = U.T @ U
    w, V = torch.linalg.eigh(G)
    order = torch.argsort(w, descending=True)[:modes]
    w, V = w[order], V[:, order]
    sv = torch.sqrt(torch.clamp(w, min=0.0))
    keep = int((sv > 1e-12 * sv[0]).sum())
    Phi = torch.zeros(U.shape[0], modes, dtype=U.dtype, device=U.device)
    Q, _ = torch.linalg.qr((U @ V[:, :keep]) / sv[:keep])
    Phi[:, :keep] = Q
    out = torch.zeros(modes, dtype=U.dtype, device=U.device)
    out[:sv.shape[0]] = sv
    return Phi, out


def features(x):
    """Network inputs from (mu, lambda/mu, traction): the load-to-stiffness ratio t/mu, Poisson's
    ratio nu = r / (2 (r + 1)) (the small-strain response is (t/mu) g(nu)), and mu."""
    mu, r, t = x[:, 0], x[:, 1], x[:, 2]
    return torch.stack([t / mu, r / (2.0 * (r + 1.0)), mu], 1)


class WarmStart:
    """POD + MLP predictor u(params) = (t/mu) Phi c(features).

    The network maps the three features to the POD coefficients of u / (t/mu): the displacement
    per unit load-to-stiffness ratio, an O(1) shape that varies smoothly with nu and the
    nonlinearity, instead of u itself, whose size spans the whole load range (and which is 0 at
    zero load exactly, by construction). Inputs are standardised per feature; the targets are
    centred and divided by one common scale, so that the training loss is the squared
    displacement error per unit t/mu (the basis is orthonormal)."""

    def __init__(self, Phi, X, C, seed=0):
        self.Phi = Phi                                  # [n, 64] FP64
        F, Y = self._targets(X, C)
        self.fm, self.fs = F.mean(0), F.std(0) + 1e-12
        self.ym = Y.mean(0)
        self.ys = torch.sqrt(((Y - self.ym) ** 2).sum(1).mean()) + 1e-300
        self.net = MLP(seed=seed, device=Phi.device)

    @staticmethod
    def _targets(X, C):
        s = X[:, 2] / X[:, 0]
        keep = s > 0                                    # zero-load states carry no shape
        return features(X[keep]), C[keep] / s[keep, None]

    def fit(self, X, C, **kw):
        F, Y = self._targets(X, C)
        return self.net.train(((F - self.fm) / self.fs).float(), ((Y - self.ym) / self.ys).float(), **kw)

    def predict(self, x):
        """x: [3] or [B,3] parameters (mu, lambda/mu, traction) -> displacement [n] or [B,n] (FP64)."""
        x = torch.as_tensor(x, dtype=torch.float64, device=self.Phi.device).reshape(-1, 3)
        y = self.net.forward(((features(x) - self.fm) / self.fs).float()).double() * self.ys + self.ym
        u = (y * (x[:, 2] / x[:, 0])[:, None]) @ self.Phi.T
        return u[0] if u.shape[0] == 1 else u

    def galerkin(self, newton, u, F, iters=2):
        """Reduced Newton in the POD space from u: c <- c - (Phi^T K Phi)^-1 Phi^T R(Phi c) on the
        free dofs, with the FP64 tangent and residual of the device assembly (two iterations
        converge within the 64-dimensional space). The network's prediction is accurate to its
        BF16 arithmetic, and errors of that size in stiff directions carry large residuals; the
        reduced solve removes them, leaving only what the POD basis cannot represent."""
        asm = newton.asm
        n = asm.nnode * 3
        free = newton.free
        P = self.Phi * free[:, None]
        m = P.shape[1]
        mp = next(k for k in (32, 64, 128, m) if k >= m)
        if mp > 128:
            raise ValueError("the Galerkin correction takes at most 128 modes")
        # K P with the library's node-block product on FP32 values (the projection is a start for
        # the FP64 Newton iteration, which removes the FP32 rounding); the small reduced system is
        # solved on the host
        P32 = torch.zeros((n, mp), dtype=torch.float32, device=P.device)
        P32[:, :m] = P
        KP = torch.empty_like(P32)
        V32 = torch.empty(asm.nnz, dtype=torch.float32, device=P.device)
        c = P.T @ u
        u = P @ c
        for _ in range(iters):
            newton._assemble(u, mixed=False)
            V32.copy_(newton.V)
            N.check(N.lib().fl_MaskedMatMatBlocksF32(_ptr(asm.indptr), _ptr(asm.indices), _ptr(V32), n,
                                                     _ptr(newton.fixed), _ptr(P32), _ptr(KP), mp, _stream()),
                    "fl_MaskedMatMatBlocksF32")
            Kr = P.T @ KP[:, :m].double()
            Rr = P.T @ ((newton.T - F) * free)
            dc = np.linalg.solve(Kr.cpu().numpy(), Rr.cpu().numpy())
            c = c - torch.from_numpy(dc).to(P.device)
            u = P @ c
        return u


# ------------------------------------------------------------------------------------------------
# The plate problem: parametrised static solves that generate the training data
# ------------------------------------------------------------------------------------------------

def build_plate_problem(nx=38, ny=19, nz=4, seed=3):
    """p=2 tet plate [0,2]x[0,1]x[0,0.2] (seeded jittered lattice, Delaunay, about 20k tets),
    face x=0 clamped, a unit in-plane traction (+x) on face x=2. Returns
    (points, elements, Jm, AllGauss, fixed [3N] bool, f_unit [3N])."""
    import os
    from . import meshes
    from .newton import tet_face_loads
    here = os.path.dirname(os.path.abspath(__file__))
    t = np.load(os.path.join(here, "..", "tests", "golden", "tet_p2_mr.npz"))
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((nx, ny, nz), (2.0, 1.0, 0.2), seed, pat)
    fixed = np.repeat(np.abs(P[:, 0]) < 1e-9, 3)
    f = tet_face_loads(P, el, pat, lambda X: abs(X[0] - 2.0) < 1e-9, (1.0, 0.0, 0.0))
    return P, el, t["Jm"], t["AllGauss"], fixed, f


def sample_parameters(n, seed):
    """n parameter sets (mu, lambda/mu, traction): mu ~ U(0.5, 2), lambda/mu ~ U(2, 100),
    traction magnitude ~ U(0, 0.5)."""
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0.5, 2.0, n), rng.uniform(2.0, 100.0, n), rng.uniform(0.0, 0.5, n)], 1)


class PlateSolver:
    """Newton load stepping of the plate for one parameter set at a time (neo-Hookean,
    lambda = mu * ratio, traction t along +x on x=2), converged to |R| <= tol |F| per increment."""

    def __init__(self, problem, n_increments=5, tol=1e-10, tangent="fp64", device="cuda"):
        from .assembly import DeviceAssembler
        from .newton import NewtonSolver
        P, el, Jm, AllGauss, fixed, f_unit = problem
        self.asm = DeviceAssembler(P, el, Jm, AllGauss, "NeoHookean", (1.0, 10.0), mode="csr", device=device)
        self.f_unit = torch.as_tensor(f_unit, dtype=torch.float64, device=self.asm.device)
        self.newton = NewtonSolver(self.asm, fixed, f_unit, n_increments=n_increments, tol=tol,
                                   tangent=tangent, criterion="load")
        self.n_increments = n_increments
        self.ndof = self.asm.nnode * 3

    def solve(self, mu, ratio, traction, guesses=None, keep_states=False):
        self.asm.params = (float(mu), float(mu) * float(ratio), 0.0)
        self.newton.f_ext = self.f_unit * float(traction)
        return self.newton.solve(guesses=guesses, keep_states=keep_states)

    def increment_inputs(self, prm, with_zero=False):
        """Network inputs (mu, ratio, traction at increment k) of every increment of one solve
        (k = 1..n, and k = 0 first when with_zero)."""
        mu, ratio, t = prm
        return np.array([[mu, ratio, t * k / self.n_increments]
                         for k in range(0 if with_zero else 1, self.n_increments + 1)])


def generate_snapshots(solver, params):
    """Training data: for every parameter set one Newton solve; every converged increment is a
    snapshot, and so is the unloaded state (u = 0 at zero traction, which anchors the network's
    prediction at the start of the load path). Returns (X [S,3] FP64 host, U [ndof, S] FP64
    device, solve statistics)."""
    X, cols, stats = [], [], []
    zero = torch.zeros(solver.ndof, dtype=torch.float64, device=solver.asm.device)
    for prm in params:
        r = solver.solve(*prm, keep_states=True)
        if r["failed"]:
            stats.append(dict(params=list(map(float, prm)), failed=True))
            continue
        X.append(solver.increment_inputs(prm, with_zero=True))
        cols += [zero] + [inc["u"] for inc in r["increments"]]
        stats.append(dict(newton=r["newton_iters"], pcg=r["pcg_iters"], wall_s=r["wall_s"], failed=False))
    return np.concatenate(X), torch.stack(cols, 1), stats


def train_warm_start(X, U, modes=64, steps=20000, batch=64, lr=2e-3, seed=0):
    """POD basis of the snapshots U, projection, and the network fit of inputs -> coefficients.
    Returns (WarmStart, loss history, POD singular values, projection error of the snapshots)."""
    Phi, sv = pod_basis(U, modes)
    C = (Phi.T @ U).T                                   # [S, modes]
    proj_err = float(torch.linalg.norm(U - Phi @ C.T) / torch.linalg.norm(U))
    Xd = torch.as_tensor(X, dtype=torch.float64, device=U.device)
    ws = WarmStart(Phi, Xd, C, seed=seed)
    hist = ws.fit(Xd, C, steps=steps, batch=batch, lr=lr, seed=seed)
    return ws, hist, sv, proj_err


def save(ws, path):
    """Checkpoint of a trained warm start: POD basis, normalisation and FP32 master weights."""
    np.savez(path, Phi=ws.Phi.cpu().numpy(), fm=ws.fm.cpu().numpy(), fs=ws.fs.cpu().numpy(),
             ym=ws.ym.cpu().numpy(), ys=ws.ys.cpu().numpy(), params=ws.net.params.cpu().numpy())


def load(path, device="cuda"):
    d = np.load(path)
    dev = torch.device(device)
    t = {k: torch.as_tensor(d[k], device=dev) for k in ("Phi", "fm", "fs", "ym", "ys")}
    ws = WarmStart.__new__(WarmStart)
    ws.Phi, ws.fm, ws.fs, ws.ym, ws.ys = t["Phi"], t["fm"], t["fs"], t["ym"], t["ys"]
    ws.net = MLP(device=dev)
    ws.net.params.copy_(torch.as_tensor(d["params"], device=dev))
    return ws


def evaluate_warm_start(solver, ws, params, warm_solvers=None):
    """Each held-out parameter set solved from the previous increment's solution (the plain
    method, `solver`) and, with every solver in warm_solvers (name -> PlateSolver; default
    {"warm": solver}), from the network's prediction, each candidate kept only if its FP64
    residual beats the previous increment's. Returns per-set records and totals per variant;
    "du" is each variant's converged displacement against the plain one (relative L2)."""
    warm_solvers = warm_solvers or {"warm": solver}
    rows = []
    for prm in params:
        inputs = solver.increment_inputs(prm, with_zero=True)
        base = solver.solve(*prm)
        row = dict(params=list(map(float, prm)),
                   plain=dict(newton=base["newton_iters"], pcg=base["pcg_iters"], wall_s=base["wall_s"],
                              failed=base["failed"]))
        for name, ws_solver in warm_solvers.items():
            t0 = time.perf_counter()
            pred = ws.predict(inputs).reshape(len(inputs), -1)   # [1 + n_increments, ndof], one forward
            torch.cuda.synchronize()
            t_pred = time.perf_counter() - t0
            # candidates: the predicted state after the reduced (POD-Galerkin) correction, and the
            # previous solution moved by the predicted step (the network's error largely cancels
            # in the step)
            nt = ws_solver.newton

            def cands(inc, u_prev, pred=pred, nt=nt):
                F = nt.f_ext * (inc / nt.n_increments)
                return [ws.galerkin(nt, pred[inc], F), u_prev + (pred[inc] - pred[inc - 1])]

            warm = ws_solver.solve(*prm, guesses=cands)
            row[name] = dict(newton=warm["newton_iters"], pcg=warm["pcg_iters"], wall_s=warm["wall_s"] + t_pred,
                             failed=warm["failed"],
                             accepted=sum(i["guess"].startswith("candidate") for i in warm["increments"]),
                             chosen=[i["guess"] for i in warm["increments"]],
                             du=float(torch.linalg.norm(warm["u"] - base["u"]) /
                                      max(1e-300, float(torch.linalg.norm(base["u"])))))
        rows.append(row)
    names = ["plain"] + list(warm_solvers)
    tot = {k: dict(newton=sum(r[k]["newton"] for r in rows), pcg=sum(r[k]["pcg"] for r in rows),
                   wall_s=sum(r[k]["wall_s"] for r in rows), failed=sum(r[k]["failed"] for r in rows))
           for k in names}
    kinds = {"candidate0": "corrected_state", "candidate1": "predicted_step", "fallback": "previous",
             "restarted": "restarted"}
    for k in warm_solvers:
        tot[k]["accepted"] = sum(r[k]["accepted"] for r in rows)
        tot[k]["chosen"] = {v: sum(c == kk for r in rows for c in r[k]["chosen"]) for kk, v in kinds.items()}
        tot[k]["max_du"] = max(r[k]["du"] for r in rows)
        tot[k]["median_du"] = float(np.median([r[k]["du"] for r in rows]))
    tot["increments"] = len(rows) * solver.n_increments
    return rows, tot
