"""GPU tests of the mixed-precision (tensor-core, split-BF16) tangent used as an inexact-Newton
Jacobian, and of Newton with it.

Bars: the FP32 Jacobian within 5e-6 relative Frobenius of the FP64 tangent (three-term BF16
split, six products, FP32 accumulation and FP32 storage); the residual, formed in FP64, within
1e-12; Newton with the mixed Jacobian converges to the FP64 Newton's displacement within 1e-8
relative.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", golden_cases())
def test_mixed_tangent_close_to_fp64(case):
    import florence_gb300 as fl
    d = load_golden(case)
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], str(d["material"]),
                             tuple(d["params"]), mode="csr", requires_geometry_update=int(d["update"]),
                             orientations=d.get("orientations"))
    x = torch.from_numpy(d["Eulerx"]).cuda()
    V32, T = asm.assemble_mixed(x)
    asm.check_flags()
    assert V32.dtype == torch.float32
    assert rel_fro(V32.double().cpu().numpy(), d["K_data"]) < 5e-6
    assert rel_fro(T.cpu().numpy(), d["T"]) < 1e-12


def test_mixed_tangent_on_config1_cube():
    import florence_gb300 as fl
    d = load_golden("config1_hex8_p2_q5")
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "NeoHookean", (1.0, 10.0),
                             mode="csr")
    x = torch.from_numpy(d["Eulerx"]).cuda()
    V64, T64 = asm.assemble(x)
    V32, T = asm.assemble_mixed(x)
    assert rel_fro(V32.double().cpu().numpy(), V64.cpu().numpy()) < 5e-6
    assert rel_fro(T.cpu().numpy(), T64.cpu().numpy()) < 1e-13


@pytest.mark.parametrize("mode", ["csr", "squeeze"])
@pytest.mark.parametrize("tiling", [(1, 16), (1, 48), (2, 32), (0, 0)])
@pytest.mark.parametrize("case", ["config1_hex8_p2_q5", "tet_p3_mr_jitter", "hex_p4_nh"])
def test_mixed_tangent_tilings(case, tiling, mode):
    """Every tile group / reduction chunk of the tensor-core kernel (one or several 128-row tiles
    per work item, one or several K chunks per element, scatter through the element-to-nonzero
    maps or by row search) gives the tangent within the split-BF16 bar of the FP64 one."""
    import florence_gb300 as fl
    d = load_golden(case)
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], str(d["material"]),
                             tuple(d["params"]), mode=mode, requires_geometry_update=int(d["update"]))
    x = torch.from_numpy(d["Eulerx"]).cuda()
    V64, T64 = asm.assemble(x)
    try:
        fl.set_tensor_core_tiling(*tiling)
        V32, T = asm.assemble_mixed(x)
        asm.check_flags()
    finally:
        fl.set_tensor_core_tiling(0, 0)
    assert rel_fro(V32.double().cpu().numpy(), V64.cpu().numpy()) < 5e-6
    assert rel_fro(T.cpu().numpy(), T64.cpu().numpy()) < 1e-13


def test_pcg_with_fp32_values_matches_fp64_values():
    import florence_gb300 as fl
    from florence_gb300.newton import build_beam_problem, pcg
    P, el, Jm, w, fixed, f = build_beam_problem(nx=8, ny=2, nz=2, traction=0.01)
    asm = fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode="csr")
    V64, _ = asm.assemble(torch.from_numpy(P).cuda())
    V32 = V64.float()
    b = torch.from_numpy(np.where(fixed, 0.0, np.random.default_rng(3).standard_normal(P.size))).cuda()
    fx = torch.from_numpy(fixed.astype(np.int8)).cuda()
    x64, _, r64 = pcg(asm, V64, b, fx, rtol=1e-10)
    x32, _, r32 = pcg(asm, V32, b, fx, rtol=1e-10)
    assert r64 <= 1e-10 and r32 <= 1e-10
    # each solve is exact for its own matrix; the two matrices differ by FP32 rounding (~6e-8
    # relative per entry), which the condition number (~1e4 here) amplifies in the solution
    assert rel_fro(x32.cpu().numpy(), x64.cpu().numpy()) < 5e-3


@pytest.mark.parametrize("tangent", ["mixed", "hybrid"])
def test_newton_mixed_reaches_fp64_solution(tangent):
    """The split-BF16 Jacobian throughout, or only while the residual is above 1e-2 of the
    load (hybrid), converges to the FP64 Newton's displacement; the hybrid run's log shows both
    Jacobians in use."""
    import florence_gb300 as fl
    from florence_gb300.newton import NewtonSolver, build_beam_problem
    P, el, Jm, w, fixed, f = build_beam_problem(nx=8, ny=2, nz=2, traction=0.01)
    asm = fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode="csr")
    r64 = NewtonSolver(asm, fixed, f, n_increments=3, tol=1e-10, tangent="fp64").solve()
    rmx = NewtonSolver(asm, fixed, f, n_increments=3, tol=1e-10, tangent=tangent).solve()
    assert not r64["failed"] and not rmx["failed"]
    assert rel_fro(rmx["u"].cpu().numpy(), r64["u"].cpu().numpy()) < 1e-8
    used = {h["jacobian"] for i in rmx["increments"] for h in i["history"]}
    assert used == ({"fp32"} if tangent == "mixed" else {"fp32", "fp64"})
