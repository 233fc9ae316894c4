"""GPU parity of the displacement-potential (electromechanics) assembly against the reference's
own DPF tangents and residuals (golden fixtures made by its numpy DPF path), in the three
scatter modes, and of the registered drop-in."""
import types

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import dpf_cases, load_golden, rel_fro

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _golden_K(d):
    n = 4 * d["points"].shape[0]
    return sp.csr_matrix((d["K_data"], d["K_indices"], d["K_indptr"]), shape=(n, n))


DEVICE_CASES = dpf_cases()


@pytest.mark.parametrize("mode", ["csr", "squeeze", "triplet"])
@pytest.mark.parametrize("case", DEVICE_CASES)
def test_dpf_assembly(case, mode):
    import torch
    import florence_gb300 as fl
    d = load_golden(case)
    n = 4 * d["points"].shape[0]
    asm = fl.DPFAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], tuple(d["params"]),
                          material=str(d["material"]), mode=mode, requires_geometry_update=int(d["update"]),
                          orientations=d.get("orientations"))
    out = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda(), torch.from_numpy(d["Eulerp"]).cuda())
    asm.check_flags()
    if mode == "triplet":
        I, J, V, T = (t.cpu().numpy() for t in out)
        K = sp.csr_matrix((V, (I, J)), shape=(n, n))
    else:
        V, T = (t.cpu().numpy() for t in out)
        K = sp.csr_matrix((V, asm.indices.cpu().numpy(), asm.indptr.cpu().numpy()), shape=(n, n))
        if mode == "csr":  # the device nvar=4 pattern is the reference's
            assert np.array_equal(asm.indices.cpu().numpy(), d["sp_indices"])
            assert np.array_equal(asm.indptr.cpu().numpy(), d["sp_indptr"])
    ref = _golden_K(d)
    assert spla.norm(K - ref) <= TOL * spla.norm(ref)
    assert rel_fro(T, d["T"]) < TOL


@pytest.mark.parametrize("recompute", [True, False])
@pytest.mark.parametrize("case", ["dpf_tet_p2_em108", "dpf_tet_p2_em101", "dpf_hex_p2_em0", "dpf_tet_p2_em106",
                                  "dpf_hex_p2_em105", "dpf_tet_p2_steinmann", "dpf_tet_p2_piezo100"])
def test_dpf_drop_in(case, recompute):
    import florence_gb300 as fl
    d = load_golden(case)
    n = 4 * d["points"].shape[0]
    solver = types.SimpleNamespace(recompute_sparsity_pattern=recompute, squeeze_sparsity_pattern=False,
                                   requires_geometry_update=int(d["update"]), indices=d["sp_indices"],
                                   indptr=d["sp_indptr"], data_local_indices=d["sp_data_local"],
                                   data_global_indices=d["sp_data_global"])
    fs = types.SimpleNamespace(Jm=d["Jm"], AllGauss=np.ravel(d["AllGauss"])[:, None], Bases=d["Bases"])
    form = types.SimpleNamespace(ndim=3, nvar=4, fields="electro_mechanics")
    mesh = types.SimpleNamespace(points=d["points"], elements=d["elements"].astype(np.uint64),
                                 nelem=d["elements"].shape[0])
    name = str(d["material"])
    names = {"IsotropicElectroMechanics_108": ("mu1", "mu2", "lamb", "eps_2"),
             "IsotropicElectroMechanics_106": ("mu1", "mu2", "lamb", "eps_1", "eps_2"),
             "IsotropicElectroMechanics_105": ("mu1", "mu2", "lamb", "eps_1", "eps_2"),
             "SteinmannModel": ("mu", "lamb", "c1", "c2", "eps_1"),
             "Piezoelectric_100": ("mu1", "mu2", "mu3", "lamb", "eps_1", "eps_2", "eps_3")}.get(name, ("mu", "lamb", "eps_1"))
    material = types.SimpleNamespace(H_VoigtSize=9, anisotropic_orientations=d.get("orientations"),
                                     **dict(zip(names, map(float, d["params"]))))
    fn = getattr(fl, "_LowLevelAssemblyDPF__" + name + "_")
    out = fn(solver, fs, form, mesh, material, d["Eulerx"], d["Eulerp"])
    if recompute:
        I, J, V, T = out
        K = sp.csr_matrix((V, (I, J)), shape=(n, n))
    else:
        V, T = out
        K = sp.csr_matrix((V, d["sp_indices"], d["sp_indptr"]), shape=(n, n))
    ref = _golden_K(d)
    assert spla.norm(K - ref) <= TOL * spla.norm(ref)
    assert rel_fro(T, d["T"]) < TOL
