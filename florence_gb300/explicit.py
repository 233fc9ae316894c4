"""Explicit central-difference dynamics with a lumped mass, on the GPU.

Mirrors the lumped-mass branch of the reference's explicit integrator
(Florence/TimeIntegrators/ExplicitStructuralDynamicIntegrator.py:28-245): U_{n+1} = 2U_n - U_{n-1}
+ dt^2 M^-1 (F - T(U_n)), written here in its equivalent leapfrog form (v_{n+1/2} = v_{n-1/2} +
dt M^-1 (F - T_n), u_{n+1} = u_n + dt v_{n+1/2}), with the reference's start
U_{-1} = U_0 - dt V_0 + dt^2/2 A_0 (:77), i.e. v_{1/2} = V_0 + dt/2 A_0.

Harness additions the reference does not have: an initial velocity field (its integrator starts
from rest, :56-59), a critical time step from power iterations of M^-1 K done matrix-free with
the internal-force kernel (the reference has no CFL estimate), and energy bookkeeping with the
textbook central-difference velocity v_n = (u_{n+1} - u_{n-1}) / (2 dt) (the reference computes
(U + U0)/(2 dt) at :152, which only feeds its own energy output).

Internal force per step: FP64 (fl_GlobalAssemblyExplicit_DF_DPF_, the reference's algorithm),
float pairs (fl_InternalForcePair: the total-Lagrangian form in float-pair arithmetic on the FP32
pipe, FP64-level results) or FP32 (fl_InternalForceF32, the same form with FP32 reference
gradients and accumulation); the state u, v stays FP64 in all three. Steps are captured in CUDA
graphs.
"""
import ctypes
import time

import numpy as np
import torch

from . import _native as N
from .assembly import DeviceAssembler, _ptr, _stream


class ExplicitSolver:
    def __init__(self, points, elements, Jm, AllGauss, Bases, mu, lamb, rho, fixed, device="cuda"):
        self.asm = DeviceAssembler(points, elements, Jm, AllGauss, "NeoHookean", (mu, lamb), mode="triplet",
                                   device=device, Bases=Bases)
        a = self.asm
        self.mu, self.lamb, self.rho = float(mu), float(lamb), float(rho)
        self.n = a.nnode * 3
        self.X = a.points.reshape(-1)
        self.fixed = torch.as_tensor(np.asarray(fixed, dtype=np.int8), device=a.device).contiguous()
        self.M = a.lumped_mass(rho)
        free = (self.fixed == 0)
        self.Minv = torch.where(free, 1.0 / self.M, torch.zeros_like(self.M))
        L = N.lib()
        self.grad0 = torch.empty(a.nelem * a.nq * a.npe * 3, dtype=torch.float32, device=a.device)
        self.dV = torch.empty(a.nelem * a.nq, dtype=torch.float32, device=a.device)
        N.check(L.fl_ReferenceGradients(_ptr(a.points), _ptr(a.elements), _ptr(a.Jm), _ptr(a.w), a.nq, a.nelem,
                                        a.npe, a.nnode, _ptr(self.grad0), _ptr(self.dV), _ptr(a.flags), _stream()),
                "fl_ReferenceGradients")
        self.gh = torch.empty(a.nelem * a.nq * a.npe * 3, dtype=torch.float32, device=a.device)
        self.gl = torch.empty_like(self.gh)
        self.dV64 = torch.empty(a.nelem * a.nq, dtype=torch.float64, device=a.device)
        N.check(L.fl_ReferenceGradientsPair(_ptr(a.points), _ptr(a.elements), _ptr(a.Jm), _ptr(a.w), a.nq, a.nelem,
                                            a.npe, a.nnode, _ptr(self.gh), _ptr(self.gl), _ptr(self.dV64),
                                            _ptr(a.flags), _stream()), "fl_ReferenceGradientsPair")
        self.T64 = torch.zeros(self.n, dtype=torch.float64, device=a.device)
        self.T32 = torch.zeros(self.n, dtype=torch.float32, device=a.device)
        self.energy = torch.zeros(1, dtype=torch.float64, device=a.device)

    # -- internal force ---------------------------------------------------------------------------
    def internal_force(self, u, mode="fp64"):
        a = self.asm
        if mode == "fp64":
            self.T64.zero_()
            a.internal_force((self.X + u).reshape(-1, 3), T=self.T64)
            return self.T64
        if mode == "pair":
            self.T64.zero_()
            N.check(N.lib().fl_InternalForcePair(_ptr(a.elements), _ptr(u), _ptr(self.gh), _ptr(self.gl),
                                                 _ptr(self.dV64), a.nq, a.nelem, a.npe, a.nnode,
                                                 N.FL_MATERIAL_NEOHOOKEAN, self.mu, self.lamb, _ptr(self.T64),
                                                 _ptr(a.flags), _stream()), "fl_InternalForcePair")
            return self.T64
        self.T32.zero_()
        N.check(N.lib().fl_InternalForceF32(_ptr(a.elements), _ptr(u), _ptr(self.grad0), _ptr(self.dV), a.nq,
                                            a.nelem, a.npe, a.nnode, N.FL_MATERIAL_NEOHOOKEAN, self.mu, self.lamb,
                                            _ptr(self.T32), _ptr(a.flags), _stream()), "fl_InternalForceF32")
        return self.T32

    def strain_energy(self, u):
        a = self.asm
        self.energy.zero_()
        N.check(N.lib().fl_StrainEnergy(_ptr(a.points), _ptr(a.elements), _ptr((self.X + u).contiguous()),
                                        _ptr(a.Jm), _ptr(a.w), a.nq, a.nelem, a.npe, a.nnode,
                                        N.FL_MATERIAL_NEOHOOKEAN, self.mu, self.lamb, _ptr(self.energy), _stream()),
                "fl_StrainEnergy")
        return float(self.energy.item())

    # -- critical step ----------------------------------------------------------------------------
    def critical_dt(self, iters=30, seed=0):
        """2 / omega_max, omega_max^2 the largest eigenvalue of M^-1 K at the reference state by
        power iteration on M^-1/2 K M^-1/2, K v from central differences of the internal force."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        x = torch.randn(self.n, generator=g, dtype=torch.float64).to(self.asm.device)
        s = self.Minv.sqrt()
        x = x * (self.fixed == 0)
        x /= torch.linalg.vector_norm(x)
        lam = 0.0
        zero = torch.zeros(self.n, dtype=torch.float64, device=self.asm.device)
        for _ in range(iters):
            w = s * x
            eps = 1e-6 / float(w.abs().max())
            Tp = self.internal_force(zero + eps * w).clone()
            Tm = self.internal_force(zero - eps * w).clone()
            y = s * ((Tp - Tm) / (2 * eps))
            lam = float(torch.dot(x, y))
            x = y / torch.linalg.vector_norm(y)
        return 2.0 / np.sqrt(lam), lam

    # -- time stepping ----------------------------------------------------------------------------
    def _update(self, u, v, dt, T, f32):
        N.check(N.lib().fl_CentralDifferenceUpdate(self.n, float(dt), _ptr(T), 1 if f32 else 0, None,
                                                   _ptr(self.Minv), _ptr(self.fixed), _ptr(u), _ptr(v), _stream()),
                "fl_CentralDifferenceUpdate")

    def run(self, v0, dt, nsteps, mode="fp64", energy_every=100, graph_steps=50):
        """Integrates nsteps from u = 0, v = v0. Returns dict(u, v, energy history, wall_s).
        Energy E_n = KE(v_n) + IE(u_n) with v_n = v_{n-1/2} + dt/2 a_n, sampled every energy_every."""
        dev = self.asm.device
        u = torch.zeros(self.n, dtype=torch.float64, device=dev)
        v = torch.as_tensor(np.asarray(v0, dtype=np.float64), device=dev).contiguous() * (self.fixed == 0)
        f32 = mode == "fp32"
        # state (u_n, v_{n-1/2}); start from v_{-1/2} = v_0 - dt/2 a_0, so that the first step gives
        # v_{1/2} = v_0 + dt/2 a_0 and u_1 = u_0 + dt v_0 + dt^2/2 a_0 (the reference's U_{-1} start)
        T = self.internal_force(u, mode)
        a0 = -T.double() * self.Minv
        hist = [(0, self.kinetic(v), 0.0)]
        v -= 0.5 * dt * a0

        def one_step():
            T = self.internal_force(u, mode)
            self._update(u, v, dt, T, f32)

        stream = torch.cuda.Stream(device=dev)
        graph = None
        if graph_steps > 1 and nsteps >= graph_steps:
            # warm up on the side stream, then capture graph_steps steps
            stream.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(stream):
                u_s, v_s = u.clone(), v.clone()
                one_step()
                u.copy_(u_s)
                v.copy_(v_s)
            torch.cuda.current_stream(dev).wait_stream(stream)
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=stream):
                for _ in range(graph_steps):
                    one_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        k = 0
        blowup = False
        norm0 = None
        while k < nsteps:
            if energy_every and k > 0 and k % energy_every == 0:
                hist.append(self._energy_point(k, u, v, dt, mode))
                nu = float(torch.linalg.vector_norm(u))
                if not np.isfinite(nu) or (norm0 is not None and nu > 10 * max(norm0, 1e-30) and k > energy_every * 5):
                    blowup = True
                    break
                norm0 = nu if norm0 is None else max(norm0, nu)
            todo = nsteps - k
            if energy_every:
                todo = min(todo, energy_every - (k % energy_every))
            if graph is not None and todo >= graph_steps:
                graph.replay()
                k += graph_steps
            else:
                one_step()
                k += 1
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if energy_every:
            hist.append(self._energy_point(k, u, v, dt, mode))
        return dict(u=u, v=v, energy=hist, wall_s=wall, steps=k, blowup=blowup)

    def kinetic(self, v):
        return float(0.5 * torch.sum(self.M * v * v))

    def _energy_point(self, k, u, v_half, dt, mode):
        T = self.internal_force(u, "fp64")
        vn = v_half - 0.5 * dt * (T * self.Minv)   # v_{n-1/2} + dt/2 a_n with a_n = -T/M
        return (k, self.kinetic(vn), self.strain_energy(u))


def build_explicit_beam(nx=64, ny=8, nz=8, L=8.0):
    """The explicit configuration: p=2 hex beam [0,L]x[0,1]x[0,1] (nx x ny x nz elements), 27 Gauss
    points, both end faces clamped. Returns (points, elements, Jm, AllGauss, Bases, fixed [3N])."""
    import os
    from . import meshes
    here = os.path.dirname(os.path.abspath(__file__))
    d = np.load(os.path.join(here, "..", "tests", "golden", "box_hex_p2_nh_big.npz"))
    pat = meshes.local_pattern(d["points"], d["elements"], 0, "hex")
    P, el = meshes.structured_hex((nx, ny, nz), (L, 1.0, 1.0), pat)
    ends = (np.abs(P[:, 0]) < 1e-9) | (np.abs(P[:, 0] - L) < 1e-9)
    return P, el, d["Jm"], d["AllGauss"], d["Bases"], np.repeat(ends, 3)
