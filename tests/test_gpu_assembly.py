"""GPU parity tests: the CUDA path through the C ABI against the golden vectors of the reference
and against the CPU oracle.

Tolerances: CSR/sparsity integer arrays bit-exact; FP64 tangent and residual within 1e-12
relative Frobenius (the criterion for the FP64 path); element matrices 1e-12.
"""
import hashlib
import types
import warnings

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import golden_cases, load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def fl():
    import florence_gb300
    from florence_gb300 import _native
    _native.lib()
    return florence_gb300


def _asm(fl, d, mode, **kw):
    kw.setdefault("requires_geometry_update", int(d["update"]))
    if "orientations" in d:  # fibre directions of the transversely isotropic material
        kw.setdefault("orientations", d["orientations"])
    return fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], str(d["material"]),
                              tuple(d["params"]), mode=mode, **kw)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, "<i4").tobytes()).hexdigest()


@pytest.mark.parametrize("case", golden_cases())
def test_device_sparsity_bit_exact(fl, case):
    d = load_golden(case)
    el = torch.from_numpy(d["elements"]).cuda()
    ind, ptr, dl, dg = fl.device_sparsity(el, d["points"].shape[0], 3)
    assert np.array_equal(ptr.cpu().numpy(), d["sp_indptr"])
    assert np.array_equal(ind.cpu().numpy(), d["sp_indices"])
    assert np.array_equal(dl.cpu().numpy(), d["sp_data_local"])
    assert np.array_equal(dg.cpu().numpy(), d["sp_data_global"])


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("mode", ["csr", "squeeze"])
def test_csr_assembly_matches_reference(fl, case, mode):
    d = load_golden(case)
    asm = _asm(fl, d, mode)
    V, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    asm.check_flags()
    assert np.array_equal(asm.indptr.cpu().numpy(), d["K_indptr"])
    assert np.array_equal(asm.indices.cpu().numpy(), d["K_indices"])
    assert rel_fro(V.cpu().numpy(), d["K_data"]) < TOL
    assert rel_fro(T.cpu().numpy(), d["T"]) < TOL


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("mode", ["csr", "squeeze", "triplet"])
def test_both_contraction_arithmetics_match_reference(fl, case, mode):
    """The contraction in FP64 multiply-adds and in float-pair arithmetic on the FP32 pipe (what
    the default reference-tensor arithmetic falls back to in triplet mode and for element types
    its GEMM does not take) both meet the FP64 path's bar (1e-12 relative Frobenius against the
    reference) in every scatter mode; the residual is formed in FP64 either way from kinematics
    summed in FP64 or in float pairs (the two agree to ~1e-14)."""
    d = load_golden(case)
    asm = _asm(fl, d, mode)
    x = torch.from_numpy(d["Eulerx"]).cuda()
    assert fl.get_arithmetic() == "reference_tensor"
    with fl.arithmetic("fp64"):
        assert fl.get_arithmetic() == "fp64"
        out64 = asm.assemble(x)
    assert fl.get_arithmetic() == "reference_tensor"
    with fl.arithmetic("float_pair"):
        out = asm.assemble(x)
    if mode == "triplet":
        n = d["points"].shape[0] * 3
        K64 = sp.csr_matrix((out64[2].cpu().numpy(), (out64[0].cpu().numpy(), out64[1].cpu().numpy())), shape=(n, n))
        ref = sp.csr_matrix((d["K_data"], d["K_indices"], d["K_indptr"]), shape=(n, n))
        assert spla.norm(K64 - ref) / spla.norm(ref) < TOL
    else:
        assert rel_fro(out64[0].cpu().numpy(), d["K_data"]) < TOL
    asm.check_flags()
    V, T = out[-2], out[-1]
    assert rel_fro(T.cpu().numpy(), out64[-1].cpu().numpy()) < 1e-13
    assert rel_fro(T.cpu().numpy(), d["T"]) < TOL
    if mode == "triplet":
        I, J = out[0].cpu().numpy(), out[1].cpu().numpy()
        n = d["points"].shape[0] * 3
        K = sp.csr_matrix((V.cpu().numpy(), (I, J)), shape=(n, n))
        K.sum_duplicates()
        K.sort_indices()
        ref = sp.csr_matrix((d["K_data"], d["K_indices"], d["K_indptr"]), shape=(n, n))
        assert spla.norm(K - ref) / spla.norm(ref) < TOL
    else:
        assert rel_fro(V.cpu().numpy(), d["K_data"]) < TOL


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("mode", ["csr", "squeeze"])
def test_tensor_core_fp64_tangent_matches_reference(fl, case, mode):
    """The contraction on the tensor cores (operands split into six exact BF16 digits, the three
    leading digit levels summed exactly in FP32) meets the FP64 bar against the reference in both
    CSR scatter modes; element types whose reduction does not fit fall back to float pairs and
    meet it too."""
    d = load_golden(case)
    asm = _asm(fl, d, mode)
    x = torch.from_numpy(d["Eulerx"]).cuda()
    with fl.arithmetic("tensor"):
        assert fl.get_arithmetic() == "tensor"
        V, T = asm.assemble(x)
        asm.check_flags()
    assert fl.get_arithmetic() == "reference_tensor"
    assert rel_fro(V.cpu().numpy(), d["K_data"]) < TOL
    assert rel_fro(T.cpu().numpy(), d["T"]) < TOL


def _padded_csr(indptr, indices, every=3, phase=1):
    """The CSR pattern with one extra column in every `every`-th row (the smallest column absent
    from the row): the rows of a node no longer share a column pattern. Returns the padded
    (indptr, indices) and, per original entry, its position in the padded arrays."""
    rows, pos, ptr = [], [], [0]
    for r in range(len(indptr) - 1):
        cols = list(indices[indptr[r]:indptr[r + 1]])
        if r % every == phase:
            c = next(c for c in range(len(cols) + 1) if c not in set(cols))
            cols = sorted(cols + [c])
        base = ptr[-1]
        keep = set(indices[indptr[r]:indptr[r + 1]])
        pos += [base + j for j, c in enumerate(cols) if c in keep]
        rows += cols
        ptr.append(len(rows))
    return np.array(ptr, np.int32), np.array(rows, np.int32), np.array(pos)


@pytest.mark.parametrize("case", ["hex_p2_nh_q5", "tet_p3_mr_jitter"])
def test_row_search_scatter_without_node_blocks(fl, case):
    """Squeeze-mode scatter into a CSR whose rows of one node differ: every entry still lands in
    its column (the node-block shortcut is verified per entry and falls back to a row search),
    the extra entries stay zero. FP64 and split-BF16 tangents."""
    d = load_golden(case)
    ptr, ind, pos = _padded_csr(d["K_indptr"], d["K_indices"])
    asm = _asm(fl, d, "squeeze", sparsity=(ind, ptr, None, None))
    x = torch.from_numpy(d["Eulerx"]).cuda()
    V, T = asm.assemble(x)
    asm.check_flags()
    v = V.cpu().numpy()
    assert rel_fro(v[pos], d["K_data"]) < TOL
    extra = np.setdiff1d(np.arange(v.shape[0]), pos)
    assert extra.size > 0 and np.all(v[extra] == 0.0)
    V32, _ = asm.assemble_mixed(x)
    asm.check_flags()
    v32 = V32.double().cpu().numpy()
    assert rel_fro(v32[pos], d["K_data"]) < 5e-6
    assert np.all(v32[extra] == 0.0)


@pytest.mark.parametrize("case", golden_cases())
def test_triplets_and_element_matrices(fl, case):
    d = load_golden(case)
    asm = _asm(fl, d, "triplet")
    I, J, V, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    asm.check_flags()
    I, J, V = I.cpu().numpy(), J.cpu().numpy(), V.cpu().numpy()
    n = d["points"].shape[0] * 3
    K = sp.csr_matrix((V, (I, J)), shape=(n, n))
    assert np.array_equal(K.indptr, d["K_indptr"]) and np.array_equal(K.indices, d["K_indices"])
    assert rel_fro(K.data, d["K_data"]) < TOL
    ndof = 3 * d["elements"].shape[1]
    Ke = V.reshape(-1, ndof, ndof)[d["emat_ids"]]
    assert rel_fro(Ke, d["emat_K"]) < TOL
    # triplet rows/cols follow the element's own dof order (fill_triplet, _MassIntegrand_.h:68-111)
    e = int(d["emat_ids"][0])
    dofs = (3 * d["elements"][e][:, None] + np.arange(3)).ravel()
    assert np.array_equal(I.reshape(-1, ndof, ndof)[e], np.repeat(dofs[:, None], ndof, 1))
    assert np.array_equal(J.reshape(-1, ndof, ndof)[e], np.repeat(dofs[None, :], ndof, 0))


@pytest.mark.parametrize("case", golden_cases())
def test_element_residual(fl, case):
    d = load_golden(case)
    for k, e in enumerate(d["emat_ids"]):
        el = d["elements"][int(e):int(e) + 1]
        orient = d["orientations"][int(e):int(e) + 1] if "orientations" in d else None
        asm = fl.DeviceAssembler(d["points"], el, d["Jm"], d["AllGauss"], str(d["material"]), tuple(d["params"]),
                                 mode="triplet", orientations=orient)
        _, _, _, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
        dofs = (3 * el[0][:, None] + np.arange(3)).ravel()
        assert rel_fro(T.cpu().numpy()[dofs], d["emat_t"][k]) < TOL


@pytest.mark.parametrize("case", [c for c in golden_cases() if "orientations" not in load_golden(c)])
def test_internal_force(fl, case):
    # (the reference's explicit path has no transversely isotropic material)
    d = load_golden(case)
    asm = _asm(fl, d, "triplet")
    T = asm.internal_force(torch.from_numpy(d["Eulerx"]).cuda())
    asm.check_flags()
    assert rel_fro(T.cpu().numpy(), d["T"]) < TOL


@pytest.mark.parametrize("case", [c for c in golden_cases() if "M_lumped" in load_golden(c)])
def test_lumped_mass(fl, case):
    d = load_golden(case)
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "NeoHookean", (1.0, 1.0),
                             mode="triplet", Bases=d["Bases"])
    M = asm.lumped_mass(float(d["rho"]))
    assert rel_fro(M.cpu().numpy(), d["M_lumped"]) < TOL


def _golden_consistent_mass(d):
    n = d["points"].shape[0] * 3
    return sp.csr_matrix((d["Mc_data"], d["Mc_indices"], d["Mc_indptr"]), shape=(n, n))


@pytest.mark.parametrize("mode", ["csr", "squeeze", "triplet"])
@pytest.mark.parametrize("case", [c for c in golden_cases() if "Mc_data" in load_golden(c)])
def test_consistent_mass(fl, case, mode):
    """Consistent mass against the reference's (golden CSR), in each scatter mode; values off the
    nvar diagonal of the tangent's pattern stay zero."""
    d = load_golden(case)
    n = d["points"].shape[0] * 3
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "NeoHookean", (1.0, 1.0),
                             mode=mode, Bases=d["Bases"])
    out = asm.consistent_mass(float(d["rho"]))
    asm.check_flags()
    if mode == "triplet":
        I, J, V = (t.cpu().numpy() for t in out)
        M = sp.csr_matrix((V, (I, J)), shape=(n, n))
    else:
        M = sp.csr_matrix((out.cpu().numpy(), asm.indices.cpu().numpy(), asm.indptr.cpu().numpy()), shape=(n, n))
    ref = _golden_consistent_mass(d)
    assert spla.norm(M - ref) <= TOL * spla.norm(ref)


@pytest.mark.parametrize("recompute,squeeze", [(True, False), (False, False), (False, True)])
def test_drop_in_consistent_mass(fl, recompute, squeeze):
    d = load_golden("tet_p3_mr_jitter")
    n = d["points"].shape[0] * 3
    rho = float(d["rho"])
    mesh = types.SimpleNamespace(points=d["points"], elements=d["elements"].astype(np.uint64))
    fs = types.SimpleNamespace(Jm=d["Jm"], AllGauss=np.ravel(d["AllGauss"])[:, None], Bases=d["Bases"])
    B = d["Bases"]
    cmi = np.zeros((B.shape[1], 3 * B.shape[0], 3 * B.shape[0]))
    for g in range(B.shape[1]):  # rho N N^T (x) I3, VariationalPrinciple.py:255-290
        cmi[g] = rho * np.kron(np.outer(B[:, g], B[:, g]), np.eye(3))
    form = types.SimpleNamespace(nvar=3, ndim=3, constant_mass_integrand=cmi)
    ref = _golden_consistent_mass(d)
    if recompute:
        _, I, J, V = fl.__TotalConstantMassIntegrand__(mesh, fs, form, "consistent", True)
        M = sp.csr_matrix((V, (I, J)), shape=(n, n))
    else:
        args = (d["sp_indices"], d["sp_indptr"], d["sp_data_global"], d["sp_data_local"])
        _, V = fl.__TotalConstantMassIntegrand__(mesh, fs, form, "consistent", False, squeeze, *args)
        M = sp.csr_matrix((V, d["sp_indices"], d["sp_indptr"]), shape=(n, n))
    assert spla.norm(M - ref) <= TOL * spla.norm(ref)


def test_config1_full_size(fl, oracle):
    """Structured 8x8x8 p=2 hex cube, 125 Gauss points, neo-Hookean: exact structure hashes from the
    reference, value probes from the reference, full CSR values against the oracle."""
    d = load_golden("config1_hex8_p2_q5")
    asm = _asm(fl, d, "csr")
    assert _sha(asm.indptr.cpu().numpy()) == str(d["sha_indptr"])
    assert _sha(asm.indices.cpu().numpy()) == str(d["sha_indices"])
    assert _sha(asm.data_local.cpu().numpy()) == str(d["sha_data_local"])
    assert _sha(asm.data_global.cpu().numpy()) == str(d["sha_data_global"])
    V, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    asm.check_flags()
    V, T = V.cpu().numpy(), T.cpu().numpy()
    n = d["points"].shape[0] * 3
    K = sp.csr_matrix((V, asm.indices.cpu().numpy(), asm.indptr.cpu().numpy()), shape=(n, n))
    v = np.random.default_rng(int(d["matvec_seed"])).standard_normal(n)
    assert rel_fro(K @ v, d["K_matvec"]) < TOL
    assert rel_fro(K.diagonal(), d["K_diag"]) < TOL
    assert abs(np.linalg.norm(V) - float(d["K_fro"])) / float(d["K_fro"]) < TOL
    assert rel_fro(T, d["T"]) < TOL
    spa = (asm.indices.cpu().numpy(), asm.indptr.cpu().numpy(), asm.data_local.cpu().numpy(),
           asm.data_global.cpu().numpy())
    Vo, To = oracle.assemble_df("NeoHookean", d["params"], d["points"], d["elements"], d["Eulerx"], d["Jm"],
                                d["AllGauss"], mode="csr", sparsity_arrays=spa, nthreads=oracle.max_threads())
    assert rel_fro(V, Vo) < TOL
    assert rel_fro(T, To) < TOL
    tri = _asm(fl, d, "triplet")
    _, _, Vt, _ = tri.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    ndof = 81
    assert rel_fro(Vt.cpu().numpy().reshape(-1, ndof, ndof)[d["emat_ids"]], d["emat_K"]) < TOL


def large_deformation(X, seed=7):
    """Smooth finite deformation (about 15% stretch, shear and a rotation) plus small seeded noise;
    det F stays well away from zero, so rounding is not amplified by a near-singular map."""
    c, s = np.cos(0.4), np.sin(0.4)
    R = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    Y = X @ np.diag([1.15, 0.95, 0.9]).T
    Y[:, 0] += 0.1 * np.sin(np.pi * X[:, 1]) + 0.05 * X[:, 2]
    Y[:, 2] += 0.08 * np.sin(np.pi * X[:, 0])
    return Y @ R.T + np.random.default_rng(seed).uniform(-0.005, 0.005, X.shape)


def test_large_displacement_against_oracle(fl, oracle):
    """Mooney-Rivlin on the config-1 mesh under a finite deformation: CUDA vs oracle."""
    d = load_golden("config1_hex8_p2_q5")
    x = large_deformation(d["points"])
    prm = (0.5, 0.5, 20.0)
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "MooneyRivlin", prm, mode="csr")
    V, T = asm.assemble(torch.from_numpy(x).cuda())
    asm.check_flags()
    spa = (asm.indices.cpu().numpy(), asm.indptr.cpu().numpy(), asm.data_local.cpu().numpy(),
           asm.data_global.cpu().numpy())
    Vo, To = oracle.assemble_df("MooneyRivlin", prm, d["points"], d["elements"], x, d["Jm"], d["AllGauss"],
                                mode="csr", sparsity_arrays=spa, nthreads=oracle.max_threads())
    assert rel_fro(V.cpu().numpy(), Vo) < TOL
    assert rel_fro(T.cpu().numpy(), To) < TOL


def test_accumulates_and_is_linear_in_repeats(fl):
    """Outputs are accumulated (+=) like the reference's: two calls into the same buffers give 2x."""
    d = load_golden("hex_p2_nh_q5")
    asm = _asm(fl, d, "csr")
    x = torch.from_numpy(d["Eulerx"]).cuda()
    V1, T1 = asm.assemble(x)
    V2, T2 = asm.assemble(x, V=V1.clone(), T=T1.clone())
    assert rel_fro(V2.cpu().numpy(), 2 * V1.cpu().numpy()) < 1e-15
    assert rel_fro(T2.cpu().numpy(), 2 * T1.cpu().numpy()) < 1e-15


def test_empty_mesh(fl):
    d = load_golden("hex_p1_nh")
    asm = fl.DeviceAssembler(d["points"], d["elements"][:0], d["Jm"], d["AllGauss"], "NeoHookean", (1.0, 10.0),
                             mode="triplet")
    I, J, V, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    assert V.numel() == 0 and float(T.abs().sum()) == 0.0
    assert float(asm.internal_force(torch.from_numpy(d["Eulerx"]).cuda()).abs().sum()) == 0.0


def test_bad_node_id_is_reported(fl):
    """An element node id >= nnode is clamped inside the kernel (in-bounds) and reported."""
    d = load_golden("hex_p1_nh")
    el = d["elements"].copy()
    el[3, 2] = d["points"].shape[0] + 5
    asm = fl.DeviceAssembler(d["points"], el, d["Jm"], d["AllGauss"], "NeoHookean", (1.0, 10.0), mode="triplet")
    asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    with pytest.raises(fl._native.FlorenceGB300Error):
        asm.check_flags()
    with pytest.raises(fl._native.FlorenceGB300Error):
        fl.device_sparsity(torch.from_numpy(el).cuda(), d["points"].shape[0], 3)


def test_unreferenced_node_rejected(fl):
    d = load_golden("hex_p1_nh")
    with pytest.raises(ValueError):
        fl.device_sparsity(torch.from_numpy(d["elements"]).cuda(), d["points"].shape[0] + 1, 3)


def test_inverted_element_warns(fl):
    d = load_golden("hex_p1_nh")
    x = d["Eulerx"].copy()
    x[:, 0] *= -1.0  # mirror: det F < 0 everywhere
    asm = _asm(fl, d, "csr")
    asm.assemble(torch.from_numpy(x).cuda())
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        asm.check_flags()
    assert any("det F" in str(x.message) for x in w)


def _fake_florence_objects(d, recompute, squeeze=False):
    """Objects with the attributes the reference's Cython wrapper reads (_LowLevelAssemblyDF_.pyx:55-113)."""
    mat_name = str(d["material"])
    p = d["params"]
    material = types.SimpleNamespace(H_VoigtSize=6, is_transversely_isotropic=False, rho=1.0, mtype=mat_name)
    if mat_name == "NeoHookean":
        material.mu, material.lamb = p[0], p[1]
    else:
        material.mu1, material.mu2, material.lamb = p[0], p[1], p[2]
    if mat_name == "AnisotropicMooneyRivlin_1":
        material.mu3 = p[3]
        material.is_transversely_isotropic = True
        material.anisotropic_orientations = d["orientations"]
    fs = types.SimpleNamespace(Jm=d["Jm"], AllGauss=d["AllGauss"][:, None], Bases=d["Bases"])
    form = types.SimpleNamespace(ndim=3, nvar=3, fields="mechanics")
    mesh = types.SimpleNamespace(points=d["points"], elements=d["elements"].astype(np.uint64),
                                 nelem=d["elements"].shape[0])
    solver = types.SimpleNamespace(requires_geometry_update=1, recompute_sparsity_pattern=recompute,
                                   squeeze_sparsity_pattern=squeeze, indices=d["sp_indices"], indptr=d["sp_indptr"],
                                   data_local_indices=d["sp_data_local"], data_global_indices=d["sp_data_global"])
    return solver, fs, form, mesh, material


@pytest.mark.parametrize("case", ["hex_p2_nh_q5", "tet_p3_mr_jitter", "tet_p2_amr"])
@pytest.mark.parametrize("recompute,squeeze", [(True, False), (False, False), (False, True)])
def test_drop_in_callables(fl, case, recompute, squeeze):
    d = load_golden(case)
    solver, fs, form, mesh, material = _fake_florence_objects(d, recompute, squeeze)
    fn = getattr(fl, "_LowLevelAssemblyDF__" + str(d["material"]) + "_")
    out = fn(solver, fs, form, mesh, material, d["Eulerx"], np.zeros(d["points"].shape[0]))
    n = d["points"].shape[0] * 3
    if recompute:
        I, J, V, T = out
        assert I.dtype == np.int32 and J.dtype == np.int32 and V.dtype == np.float64
        K = sp.csr_matrix((V, (I, J)), shape=(n, n))
    else:
        V, T = out
        K = sp.csr_matrix((V, d["sp_indices"], d["sp_indptr"]), shape=(n, n))
    assert T.shape == (n,) and T.dtype == np.float64
    assert rel_fro(K.data, d["K_data"]) < TOL and rel_fro(T, d["T"]) < TOL
    if "orientations" in d:  # no explicit path for the transversely isotropic material, as in the reference
        with pytest.raises(NotImplementedError):
            fl._LowLevelAssemblyExplicit_DF_DPF_(fs, form, mesh, material, d["Eulerx"], np.zeros(d["points"].shape[0]))
        return
    Ti = fl._LowLevelAssemblyExplicit_DF_DPF_(fs, form, mesh, material, d["Eulerx"], np.zeros(d["points"].shape[0]))
    assert rel_fro(Ti, d["T"]) < TOL


@pytest.mark.parametrize("case", ["tet_p3_mr_jitter", "hex_p2_nh_q5"])
def test_drop_in_pipelined_assembly(fl, monkeypatch, case):
    """The drop-in's pipelined path (element groups assembled in turn, finished rows copied to the
    host meanwhile; taken for large meshes) forced on a golden case: the reference's values."""
    from florence_gb300 import assembly
    monkeypatch.setattr(assembly, "PIPELINE_MIN_ELEMENTS", 0)
    d = load_golden(case)
    solver, fs, form, mesh, material = _fake_florence_objects(d, False, True)
    fn = getattr(fl, "_LowLevelAssemblyDF__" + str(d["material"]) + "_")
    for _ in range(2):
        V, T = fn(solver, fs, form, mesh, material, d["Eulerx"], np.zeros(d["points"].shape[0]))
        assert rel_fro(V, d["K_data"]) < TOL and rel_fro(T, d["T"]) < TOL
    fl.release_device_meshes()


def test_drop_in_sparsity(fl):
    d = load_golden("tet_p3_mr_jitter")
    mesh = types.SimpleNamespace(points=d["points"], elements=d["elements"].astype(np.uint64))
    ind, ptr, dl, dg = fl.ComputeSparsityPattern(mesh, 3)
    assert np.array_equal(ind, d["sp_indices"]) and np.array_equal(ptr, d["sp_indptr"])
    assert np.array_equal(dl, d["sp_data_local"]) and np.array_equal(dg, d["sp_data_global"])
    ind2, ptr2 = fl.ComputeSparsityPattern(mesh, 3, squeeze_sparsity_pattern=True)
    assert np.array_equal(ind2, ind) and np.array_equal(ptr2, ptr)


def test_unsupported_material_raises(fl):
    d = load_golden("hex_p1_nh")
    solver, fs, form, mesh, material = _fake_florence_objects(d, True)
    with pytest.raises(NotImplementedError):
        fl.material_params(material, "AnisotropicMooneyRivlin_0")


def test_fp64_peak_is_measured(fl):
    g = fl.fp64_peak_gflops()
    assert 100.0 < g < 200000.0


def test_transversely_isotropic_material_needs_fibre_directions(fl):
    """AnisotropicMooneyRivlin_1 takes one fibre direction per element (the reference's
    anisotropic_orientations); without them, or through the explicit path, it is refused."""
    d = load_golden("tet_p2_amr")
    with pytest.raises(ValueError):
        fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "AnisotropicMooneyRivlin_1",
                           tuple(d["params"]), mode="csr")
    asm = _asm(fl, d, "csr")
    with pytest.raises(NotImplementedError):
        asm.internal_force(torch.from_numpy(d["Eulerx"]).cuda())
    # the fibre direction matters: rotating it changes the tangent
    asm2 = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "AnisotropicMooneyRivlin_1",
                              tuple(d["params"]), mode="csr", orientations=d["orientations"][:, [1, 2, 0]])
    x = torch.from_numpy(d["Eulerx"]).cuda()
    assert rel_fro(asm2.assemble(x)[0].cpu().numpy(), d["K_data"]) > 1e-3


@pytest.mark.parametrize("case", [c for c in golden_cases() if "F_traction" in load_golden(c)])
def test_external_forces_match_reference(fl, case):
    """AssembleExternalTractionForces / AssembleBodyForces on the device against the reference's
    (parent-face weights, Assembly.py:451-560), and the physical-face option against a numpy
    integral of the same faces."""
    d = load_golden(case)
    bc = types.SimpleNamespace(neumann_flags=d["neumann_flags"], applied_neumann=d["applied_neumann"])
    mat = types.SimpleNamespace(ndim=3, nvar=3, rho=float(d["rho_body"]))
    mesh = types.SimpleNamespace(points=d["points"], faces=d["faces"].astype(np.uint64),
                                 elements=d["elements"].astype(np.uint64))
    fsf = types.SimpleNamespace(Bases=d["face_Bases"], AllGauss=d["face_AllGauss"][:, None], Jm=d["face_Jm"])
    fse = types.SimpleNamespace(Bases=d["Bases"], AllGauss=d["AllGauss"][:, None])
    Ft = fl.AssembleExternalTractionForces(bc, mesh, mat, fsf)
    Fb = fl.AssembleBodyForces(bc, mesh, mat, fse)
    assert Ft.shape == (d["points"].shape[0] * 3, 1) and Fb.shape == Ft.shape
    assert rel_fro(Ft.ravel(), d["F_traction"]) < 1e-14
    assert rel_fro(Fb.ravel(), d["F_body"]) < 1e-14
    # physical faces: w_g |dX/dxi x dX/deta|
    Fp = fl.AssembleExternalTractionForces(bc, mesh, mat, fsf, physical_faces=True).ravel()
    ref = np.zeros_like(Fp)
    for f in np.nonzero(d["neumann_flags"])[0]:
        X = d["points"][d["faces"][f]]
        d0 = np.einsum("ag,ak->gk", d["face_Jm"][0], X)
        d1 = np.einsum("ag,ak->gk", d["face_Jm"][1], X)
        area = np.linalg.norm(np.cross(d0, d1), axis=1)
        s = d["face_Bases"] @ (d["face_AllGauss"] * area)
        for a, nd in enumerate(d["faces"][f]):
            ref[3 * nd:3 * nd + 3] += d["applied_neumann"][f] * s[a]
    assert rel_fro(Fp, ref) < 1e-13
