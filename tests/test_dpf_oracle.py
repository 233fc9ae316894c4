"""The displacement-potential (electromechanics) oracle against golden vectors made by the
reference's own numpy DPF path (DisplacementPotentialFormulation.py:108-200 with
IsotropicElectroMechanics_108): element matrices, the global tangent and the residual; and the
reference's nvar=4 sparsity pattern reproduced by the CPU sparsity oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import dpf_cases, load_golden, rel_fro
from oracle import dpf_oracle

TOL = 1e-12


@pytest.mark.parametrize("case", dpf_cases())
def test_dpf_element_matrices(case):
    d = load_golden(case)
    for k, e in enumerate(d["emat_ids"]):
        nodes = d["elements"][e]
        K, t = dpf_oracle.element(str(d["material"]), tuple(d["params"]), d["points"][nodes], d["Eulerx"][nodes],
                                  d["Eulerp"][nodes], d["Jm"], np.ravel(d["AllGauss"]), int(d["update"]),
                                  d["orientations"][e] if "orientations" in d else None)
        assert rel_fro(K, d["emat_K"][k]) < TOL
        assert rel_fro(t, d["emat_t"][k]) < TOL


@pytest.mark.parametrize("case", dpf_cases())
def test_dpf_global_tangent_and_residual(case):
    d = load_golden(case)
    K, T = dpf_oracle.assemble(str(d["material"]), tuple(d["params"]), d["points"], d["elements"], d["Eulerx"],
                               d["Eulerp"], d["Jm"], d["AllGauss"], int(d["update"]), d.get("orientations"))
    n = K.shape[0]
    ref = sp.csr_matrix((d["K_data"], d["K_indices"], d["K_indptr"]), shape=(n, n)).toarray()
    assert rel_fro(K, ref) < TOL
    assert rel_fro(T, d["T"]) < TOL
    # the tangent is symmetric (an enthalpy Hessian); the electric block is negative definite
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()


@pytest.mark.parametrize("case", dpf_cases())
def test_dpf_sparsity_pattern_nvar4(oracle, case):
    d = load_golden(case)
    ind, ptr, dl, dg = oracle.sparsity(d["elements"], d["points"].shape[0], nvar=4)
    assert np.array_equal(ind, d["sp_indices"]) and np.array_equal(ptr, d["sp_indptr"])
    assert np.array_equal(dl, d["sp_data_local"]) and np.array_equal(dg, d["sp_data_global"])


SHIM_MATERIALS = {"IsotropicElectroMechanics_108": 108, "IsotropicElectroMechanics_106": 106,
                  "IsotropicElectroMechanics_105": 105, "IsotropicElectroMechanics_101": 101,
                  "IsotropicElectroMechanics_0": 0, "SteinmannModel": 1, "Piezoelectric_100": 100}


@pytest.fixture(scope="module")
def dpf_host(tmp_path_factory):
    """Host build of the device kernel's DPF arithmetic (florence_gb300/csrc/fl_dpf.cuh)."""
    import ctypes
    import os
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    so = str(tmp_path_factory.mktemp("dpf") / "dpf_shim.so")
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-o", so, os.path.join(here, "dpf_host_shim.cpp")])
    L = ctypes.CDLL(so)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.dpf_element.argtypes = [I, I, I, P, P, P, P, P, I, P, P, P, P, I]
    L.dpf_element.restype = D
    return L


@pytest.mark.parametrize("blocks", [0, 1])
@pytest.mark.parametrize("case", dpf_cases())
def test_device_dpf_arithmetic_on_host(dpf_host, case, blocks):
    """The Gauss-point and tangent functions the device kernel runs, built for the host, give the
    reference's element tangents and residuals: entry by entry, and as the kernel forms them,
    node-pair blocks for a <= b mirrored to b > a (the reference's element tangents are symmetric
    to rounding)."""
    d = load_golden(case)
    Jm = np.ascontiguousarray(d["Jm"], np.float64)
    w = np.ascontiguousarray(np.ravel(d["AllGauss"]), np.float64)
    npe, nq = Jm.shape[1], Jm.shape[2]
    for k, e in enumerate(d["emat_ids"]):
        nodes = d["elements"][e]
        X = np.ascontiguousarray(d["points"][nodes], np.float64)
        x = np.ascontiguousarray(d["Eulerx"][nodes], np.float64)
        phi = np.ascontiguousarray(d["Eulerp"][nodes], np.float64)
        K = np.zeros((4 * npe, 4 * npe))
        t = np.zeros(4 * npe)
        p = np.ascontiguousarray(d["params"], np.float64)
        N = np.ascontiguousarray(d["orientations"][e], np.float64) if "orientations" in d else None
        mat = SHIM_MATERIALS[str(d["material"])]
        minJ = dpf_host.dpf_element(mat, npe, nq, Jm.ctypes.data, w.ctypes.data, X.ctypes.data, x.ctypes.data,
                                    phi.ctypes.data, int(d["update"]), p.ctypes.data,
                                    N.ctypes.data if N is not None else None, K.ctypes.data, t.ctypes.data, blocks)
        assert minJ > 0
        assert rel_fro(K, d["emat_K"][k]) < TOL
        assert rel_fro(t, d["emat_t"][k]) < TOL
