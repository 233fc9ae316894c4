"""Pins the CPU oracle against golden vectors made by the reference's own code.

The golden fixtures come from the reference's numpy assembly path, its compiled
ComputeSparsityPattern and its Python lumped-mass path (tests/golden/make_golden.py).
Tolerance: 1e-13 relative Frobenius for floating point, bit-exact for the sparsity.
"""
import hashlib

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden_cases, load_golden, rel_fro

TOL = 1e-13


@pytest.mark.parametrize("case", golden_cases())
def test_sparsity_bit_exact(oracle, case):
    d = load_golden(case)
    ind, ptr, dl, dg = oracle.sparsity(d["elements"], d["points"].shape[0])
    assert np.array_equal(ptr, d["sp_indptr"])
    assert np.array_equal(ind, d["sp_indices"])
    assert np.array_equal(dl, d["sp_data_local"])
    assert np.array_equal(dg, d["sp_data_global"])
    # the reference's CSR pattern (AssembleForm output) is the same canonical pattern
    assert np.array_equal(ptr, d["K_indptr"]) and np.array_equal(ind, d["K_indices"])


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("mode", ["csr", "squeeze", "triplet"])
def test_assembly_matches_reference(oracle, case, mode):
    d = load_golden(case)
    mat, prm = str(d["material"]), d["params"]
    args = (mat, prm, d["points"], d["elements"], d["Eulerx"], d["Jm"], d["AllGauss"])
    nn = d["points"].shape[0] * 3
    orient = d.get("orientations")
    if mode == "triplet":
        I, J, V, T = oracle.assemble_df(*args, mode="triplet", orientations=orient)
        K = sp.csr_matrix((V, (I, J)), shape=(nn, nn))
        assert np.array_equal(K.indptr, d["K_indptr"]) and np.array_equal(K.indices, d["K_indices"])
        V = K.data
    else:
        spa = oracle.sparsity(d["elements"], d["points"].shape[0])
        V, T = oracle.assemble_df(*args, mode=mode, sparsity_arrays=spa, orientations=orient)
    assert rel_fro(V, d["K_data"]) < TOL
    assert rel_fro(T, d["T"]) < 1e-12
    if "K_triplet_data" in d:
        assert rel_fro(V, d["K_triplet_data"]) < TOL


@pytest.mark.parametrize("case", golden_cases())
def test_element_matrices(oracle, case):
    d = load_golden(case)
    Ke, te = oracle.element_matrices(str(d["material"]), d["params"], d["points"], d["elements"], d["Eulerx"],
                                     d["Jm"], d["AllGauss"], d["emat_ids"], orientations=d.get("orientations"))
    assert rel_fro(Ke, d["emat_K"]) < TOL
    assert rel_fro(te, d["emat_t"]) < 1e-12


@pytest.mark.parametrize("case", golden_cases())
def test_internal_force_matches_residual(oracle, case):
    # the explicit internal force is the implicit residual without the tangent
    d = load_golden(case)
    T = oracle.internal_force(str(d["material"]), d["params"], d["points"], d["elements"], d["Eulerx"], d["Jm"],
                              d["AllGauss"], orientations=d.get("orientations"))
    assert rel_fro(T, d["T"]) < 1e-12


@pytest.mark.parametrize("case", [c for c in golden_cases() if "M_lumped" in load_golden(c)])
def test_lumped_mass(oracle, case):
    d = load_golden(case)
    M = oracle.lumped_mass(float(d["rho"]), d["points"], d["elements"], d["Jm"], d["AllGauss"], d["Bases"])
    assert rel_fro(M, d["M_lumped"]) < TOL


def golden_consistent_mass(d):
    n = d["points"].shape[0] * 3
    return sp.csr_matrix((d["Mc_data"], d["Mc_indices"], d["Mc_indptr"]), shape=(n, n))


@pytest.mark.parametrize("case", [c for c in golden_cases() if "Mc_data" in load_golden(c)])
def test_consistent_mass(oracle, case):
    d = load_golden(case)
    M = oracle.consistent_mass(float(d["rho"]), d["points"], d["elements"], d["Jm"], d["AllGauss"], d["Bases"])
    ref = golden_consistent_mass(d).toarray()
    assert rel_fro(M, ref) < TOL
    # its row sums are the lumped mass, the reference's own lumping
    assert rel_fro(M.sum(1), d["M_lumped"]) < TOL


def test_config1_structure_and_values(oracle):
    """Full-size structured 8x8x8 p=2 hex cube, 125 Gauss points: exact structure hashes and value probes."""
    d = load_golden("config1_hex8_p2_q5")
    ind, ptr, dl, dg = oracle.sparsity(d["elements"], d["points"].shape[0])
    h = lambda a: hashlib.sha256(np.ascontiguousarray(a, "<i4").tobytes()).hexdigest()
    assert h(ptr) == str(d["sha_indptr"]) and h(ind) == str(d["sha_indices"])
    assert h(dl) == str(d["sha_data_local"]) and h(dg) == str(d["sha_data_global"])
    assert ind.shape[0] == int(d["nnz"])
    V, T = oracle.assemble_df("NeoHookean", d["params"], d["points"], d["elements"], d["Eulerx"], d["Jm"],
                              d["AllGauss"], mode="csr", sparsity_arrays=(ind, ptr, dl, dg), nthreads=4)
    n = d["points"].shape[0] * 3
    K = sp.csr_matrix((V, ind, ptr), shape=(n, n))
    v = np.random.default_rng(int(d["matvec_seed"])).standard_normal(n)
    assert rel_fro(K @ v, d["K_matvec"]) < TOL
    assert rel_fro(K.diagonal(), d["K_diag"]) < TOL
    assert abs(np.linalg.norm(V) - float(d["K_fro"])) / float(d["K_fro"]) < TOL
    assert rel_fro(T, d["T"]) < 1e-12
    Ke, te = oracle.element_matrices("NeoHookean", d["params"], d["points"], d["elements"], d["Eulerx"], d["Jm"],
                                     d["AllGauss"], d["emat_ids"])
    assert rel_fro(Ke, d["emat_K"]) < TOL


def test_unreferenced_node_is_rejected(oracle):
    el = np.array([[0, 1, 2, 3]], np.int64)
    with pytest.raises(ValueError):
        oracle.sparsity(el, 5)


def test_mlp_oracle_gradients_match_finite_differences():
    """The network oracle's backward pass (without BF16 rounding) against central differences."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(0)
    n = sum(int(np.prod(s)) for s in M.SIZES)
    p = rng.normal(0, 0.1, n)
    x = rng.normal(0, 1, (5, 3))
    t = rng.normal(0, 1, (5, 64))
    g, _, _ = M.gradients(p, x, t, rounding=False)
    idx = rng.choice(n, 40, replace=False)
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.gradients(pp, x, t, rounding=False)[1] - M.gradients(pm, x, t, rounding=False)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9


def test_mlp_oracle_bf16_rounding_matches_torch():
    import torch
    from oracle import mlp_oracle as M
    x = np.random.default_rng(1).normal(0, 3, 10000).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).double().numpy()
    assert np.array_equal(M._bf16(x), ref)


@pytest.mark.parametrize("case", [c for c in golden_cases() if "F_traction" in load_golden(c)])
def test_external_forces(oracle, case):
    """Surface traction and body force as the reference assembles them (Assembly.py:451-560)."""
    d = load_golden(case)
    n = d["points"].shape[0]
    Ft = oracle.external_traction(d["faces"], d["neumann_flags"], d["applied_neumann"], d["face_Bases"],
                                  d["face_AllGauss"], n)
    Fb = oracle.body_forces(d["elements"], d["Bases"], d["AllGauss"], float(d["rho_body"]), n)
    assert rel_fro(Ft, d["F_traction"]) < 1e-14
    assert rel_fro(Fb, d["F_body"]) < 1e-14
