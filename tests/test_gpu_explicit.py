"""GPU tests of the explicit-dynamics building blocks and the time loop.

* FP32 internal force (total-Lagrangian, FP32 accumulation) against the reference's residual:
  within 2e-6 relative (FP32 arithmetic); the float-pair variant of the same form within 1e-12
  (the FP64 bar);
* reference gradients and the strain energy against numpy restatements;
* the FP64 time loop (CUDA graphs) against a CPU leapfrog built on the oracle's internal force
  and lumped mass: within 1e-10 relative after 200 steps;
* energy conservation of the FP64 loop and the gap between FP32 and FP64 trajectories.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def box():
    return load_golden("box_hex_p2_nh_big")


def _solver(P, el, Jm, w, B, mu, lamb, rho, fixed):
    from florence_gb300.explicit import ExplicitSolver
    return ExplicitSolver(P, el, Jm, w, B, mu, lamb, rho, fixed)


def test_f32_internal_force_matches_reference(box):
    d = box
    fixed = np.zeros(d["points"].size, bool)
    s = _solver(d["points"], d["elements"], d["Jm"], d["AllGauss"], d["Bases"], d["params"][0], d["params"][1], 1.0,
                fixed)
    u = torch.from_numpy((d["Eulerx"] - d["points"]).ravel()).cuda()
    T32 = s.internal_force(u, "fp32").double().cpu().numpy()
    assert rel_fro(T32, d["T"]) < 2e-6
    T64 = s.internal_force(u, "fp64").cpu().numpy()
    assert rel_fro(T64, d["T"]) < 1e-12
    Tp = s.internal_force(u, "pair").cpu().numpy()
    assert rel_fro(Tp, d["T"]) < 1e-12
    s.asm.check_flags()


def test_reference_gradients_and_volume(box):
    d = box
    s = _solver(d["points"], d["elements"], d["Jm"], d["AllGauss"], d["Bases"], 1.0, 1.0, 1.0,
                np.zeros(d["points"].size, bool))
    assert abs(float(s.dV.double().sum()) - 4.0) < 1e-5     # box [0,4]x[0,1]x[0,1]
    # gradients of the coordinate field are the identity: sum_a X_a (x) dN_a/dX = I
    E, nq, npe = s.asm.nelem, s.asm.nq, s.asm.npe
    g = s.grad0.double().cpu().numpy().reshape(E, nq, npe, 3)
    X = d["points"][d["elements"]]                          # [E, npe, 3]
    Id = np.einsum("eak,egad->egkd", X, g)
    assert np.abs(Id - np.eye(3)).max() < 1e-5


def test_strain_energy_matches_numpy(box):
    d = box
    mu, lamb = d["params"]
    s = _solver(d["points"], d["elements"], d["Jm"], d["AllGauss"], d["Bases"], mu, lamb, 1.0,
                np.zeros(d["points"].size, bool))
    u = torch.from_numpy((d["Eulerx"] - d["points"]).ravel()).cuda()
    W = s.strain_energy(u)
    ref = 0.0
    for e in range(d["elements"].shape[0]):
        X = d["points"][d["elements"][e]]
        x = d["Eulerx"][d["elements"][e]]
        for g in range(d["Jm"].shape[2]):
            PX = d["Jm"][:, :, g] @ X
            Px = d["Jm"][:, :, g] @ x
            F = np.linalg.solve(PX, Px).T
            J = np.linalg.det(F)
            ref += (0.5 * mu * (np.sum(F * F) - 3) - mu * np.log(J) + 0.5 * lamb * (J - 1) ** 2) * \
                d["AllGauss"][g] * abs(np.linalg.det(PX))
    assert abs(W - ref) / abs(ref) < 1e-11


@pytest.fixture(scope="module")
def small_beam():
    from florence_gb300.explicit import build_explicit_beam
    return build_explicit_beam(nx=16, ny=2, nz=2, L=2.0)


def test_time_loop_matches_cpu_leapfrog(small_beam, oracle):
    P, el, Jm, w, B, fixed = small_beam
    mu, lamb, rho = 1.0, 1000.0, 1.0
    s = _solver(P, el, Jm, w, B, mu, lamb, rho, fixed)
    dtc, lam = s.critical_dt()
    dt = 0.9 * dtc
    v0 = np.zeros_like(P)
    v0[:, 2] = 0.1 * np.sin(np.pi * P[:, 0] / 2.0)
    v0 = v0.ravel()
    nsteps = 200
    out = s.run(v0, dt, nsteps, mode="fp64", energy_every=0, graph_steps=50)
    assert not out["blowup"]
    # CPU leapfrog with the oracle's internal force and lumped mass
    M = oracle.lumped_mass(rho, P, el, Jm, w, B)
    free = ~fixed
    Minv = np.where(free, 1.0 / M, 0.0)
    u = np.zeros(P.size)
    T = oracle.internal_force("NeoHookean", (mu, lamb), P, el, P, Jm, w, nthreads=oracle.max_threads())
    v = v0 * free - 0.5 * dt * (-T * Minv)
    for _ in range(nsteps):
        T = oracle.internal_force("NeoHookean", (mu, lamb), P, el, P + u.reshape(-1, 3), Jm, w,
                                  nthreads=oracle.max_threads())
        v = np.where(free, v + dt * (-T * Minv), v)
        u = np.where(free, u + dt * v, u)
    assert rel_fro(out["u"].cpu().numpy(), u) < 1e-10
    assert rel_fro(out["v"].cpu().numpy(), v) < 1e-10


def test_energy_and_fp32_trajectory(small_beam):
    P, el, Jm, w, B, fixed = small_beam
    s = _solver(P, el, Jm, w, B, 1.0, 1000.0, 1.0, fixed)
    dtc, _ = s.critical_dt()
    dt = 0.9 * dtc
    v0 = np.zeros_like(P)
    v0[:, 2] = 0.1 * np.sin(np.pi * P[:, 0] / 2.0)
    r64 = s.run(v0.ravel(), dt, 2000, mode="fp64", energy_every=100)
    r32 = s.run(v0.ravel(), dt, 2000, mode="fp32", energy_every=100)
    rp = s.run(v0.ravel(), dt, 2000, mode="pair", energy_every=100)
    # the float-pair trajectory stays on the FP64 one
    assert rel_fro(rp["u"].cpu().numpy(), r64["u"].cpu().numpy()) < 1e-9
    for r in (r64, r32, rp):
        assert not r["blowup"]
        E = np.array([k + i for _, k, i in r["energy"]])
        assert np.abs(E / E[0] - 1.0).max() < 5e-3          # central difference: bounded oscillation
    assert rel_fro(r32["u"].cpu().numpy(), r64["u"].cpu().numpy()) < 1e-3
