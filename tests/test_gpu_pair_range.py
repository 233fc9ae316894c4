"""Units far from O(1). The default contraction arithmetics (reference-tensor GEMMs, float pairs)
hold each Gauss point's pulled-back tangent as float pairs, i.e. in FP32's exponent range. The
Mooney-Rivlin and neo-Hookean stresses and tangents are linear in the material moduli, so scaling
every modulus by 2^k scales the reference's tangent and residual by exactly 2^k:

* 2^-60 and 2^+60 (in range): every arithmetic meets the 1e-12 bar against the reference's values
  scaled alike, and no flag is raised;
* 2^-100 and 2^+135 (out of range: below the band, and past FP32's overflow): FL_FLAG_PAIR_RANGE
  is set, DeviceAssembler.check_flags raises, the FP64 arithmetic still meets the bar, and the
  drop-in callable assembles again in FP64 by itself and meets it.
"""
import types

import numpy as np
import pytest

from conftest import load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
CASES = ["tet_p3_mr_jitter", "hex_p2_nh_q5"]   # 20-node tets (reference tensor), 27-node hexes (float pairs)


def _scaled(case, k):
    d = load_golden(case)
    s = 2.0 ** k
    return d, tuple(float(p) * s for p in d["params"]), d["K_data"] * s, d["T"] * s


def _asm(fl, d, params, mode="csr"):
    return fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], str(d["material"]), params,
                              mode=mode, requires_geometry_update=int(d["update"]))


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("k", [-60, 60])
@pytest.mark.parametrize("arith", ["reference_tensor", "float_pair", "fp64"])
def test_scaled_units_in_range(case, k, arith):
    import florence_gb300 as fl
    d, params, K, T = _scaled(case, k)
    asm = _asm(fl, d, params)
    with fl.arithmetic(arith):
        V, Tv = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
        torch.cuda.synchronize()
    asm.check_flags()
    assert rel_fro(V.cpu().numpy(), K) < TOL
    assert rel_fro(Tv.cpu().numpy(), T) < TOL


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("k", [-100, 135])
def test_out_of_range_is_flagged_and_fp64_holds(case, k):
    import florence_gb300 as fl
    from florence_gb300._native import FL_FLAG_PAIR_RANGE, FlorenceGB300Error
    d, params, K, T = _scaled(case, k)
    asm = _asm(fl, d, params)
    x = torch.from_numpy(d["Eulerx"]).cuda()
    asm.assemble(x)
    torch.cuda.synchronize()
    assert int(asm.flags.item()) & FL_FLAG_PAIR_RANGE
    with pytest.raises(FlorenceGB300Error):
        asm.check_flags()
    asm.flags.zero_()
    with fl.arithmetic("fp64"):
        V, Tv = asm.assemble(x)
        torch.cuda.synchronize()
    asm.check_flags()
    assert rel_fro(V.cpu().numpy(), K) < TOL
    assert rel_fro(Tv.cpu().numpy(), T) < TOL


@pytest.mark.parametrize("k", [-100, 135])
def test_drop_in_falls_back_to_fp64(k):
    import florence_gb300 as fl
    d, params, K, T = _scaled("tet_p3_mr_jitter", k)
    material = types.SimpleNamespace(H_VoigtSize=6, is_transversely_isotropic=False, rho=1.0, mu1=params[0],
                                     mu2=params[1], lamb=params[2])
    fs = types.SimpleNamespace(Jm=d["Jm"], AllGauss=np.ravel(d["AllGauss"])[:, None])
    form = types.SimpleNamespace(ndim=3, nvar=3, fields="mechanics")
    mesh = types.SimpleNamespace(points=d["points"], elements=d["elements"].astype(np.uint64),
                                 nelem=d["elements"].shape[0])
    solver = types.SimpleNamespace(requires_geometry_update=int(d["update"]), recompute_sparsity_pattern=False,
                                   squeeze_sparsity_pattern=True, indices=d["sp_indices"], indptr=d["sp_indptr"])
    V, Tv = fl._LowLevelAssemblyDF__MooneyRivlin_(solver, fs, form, mesh, material, d["Eulerx"],
                                                  np.zeros(d["points"].shape[0]))
    assert fl.get_arithmetic() == "reference_tensor"
    assert rel_fro(V, K) < TOL
    assert rel_fro(Tv, T) < TOL
    fl.release_device_meshes()
