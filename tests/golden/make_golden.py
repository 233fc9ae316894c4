"""Generates the golden fixtures in this folder from the reference Florence package.

Test infrastructure only. Run where a checkout of the reference is available, its root
named by ``FLORENCE_REFERENCE`` (it is not present on the GPU machine, which only reads the
committed ``.npz`` files):

    FLORENCE_REFERENCE=<reference checkout> python tests/golden/make_golden.py

Every output is produced by the reference's own pure-numpy assembly path
(``AssembleForm`` -> ``AssemblySmall`` -> ``DisplacementFormulation.GetLocalStiffness``,
Florence/FiniteElements/Assembly/Assembly.py:1454-1495, :99-252 and
Florence/VariationalPrinciple/DisplacementFormulation.py:110-188), by its compiled
``ComputeSparsityPattern`` (Florence/FiniteElements/Assembly/_Assembly_/ComputeSparsityPattern.pyx:44-112)
and by its Python lumped and consistent mass path (Florence/FiniteElements/Assembly/Assembly.py:608-657).
Meshes come from the reference's own generators (``Mesh.Cube``, ``Mesh.Parallelepiped``,
``GetHighOrderMesh``) or from a seeded jittered lattice split by ``scipy.spatial.Delaunay``.
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import florence_harness  # noqa: E402


def sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def make_material(F, name, params):
    if name == "NeoHookean":
        m = F.NeoHookean(3, mu=params[0], lamb=params[1], rho=params[2] if len(params) > 2 else 1.0)
    elif name == "MooneyRivlin":
        m = F.MooneyRivlin(3, mu1=params[0], mu2=params[1], lamb=params[2], rho=params[3] if len(params) > 3 else 1.0)
    elif name == "LinearElastic":
        m = F.LinearElastic(3, mu=params[0], lamb=params[1], rho=1.0)
    elif name == "NearlyIncompressibleMooneyRivlin":
        # params (alpha, beta, kappa): the numpy path reads alpha/beta/kappa, the low-level path
        # (AOT_Assembler.py:66-71, 110-112) mu1/mu2/lamb -- set both to the same values
        m = F.NearlyIncompressibleMooneyRivlin(3, mu=2.0 * params[0], lamb=params[2], rho=1.0)
        m.alpha, m.beta, m.kappa = params
        m.mu1, m.mu2, m.lamb = params
    elif name == "AnisotropicMooneyRivlin_1":
        # params (mu1, mu2, lamb, mu3); fibre directions set per element by make_case
        m = F.AnisotropicMooneyRivlin_1(3, mu1=params[0], mu2=params[1], lamb=params[2], mu3=params[3], rho=1.0)
    elif name == "Piezoelectric_100":
        # params (mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3); fibre directions set per element by make_dpf_case
        m = F.Piezoelectric_100(3, mu1=params[0], mu2=params[1], mu3=params[2], lamb=params[3], eps_1=params[4],
                                eps_2=params[5], eps_3=params[6], rho=1.0)
    elif name == "SteinmannModel":
        # params (mu, lamb, c1, c2, eps_1): W_n(C) + c1 I:(E0 x E0) + c2 C:(E0 x E0) - eps_1/2 J C^-1:(E0 x E0)
        m = F.SteinmannModel(3, mu=params[0], lamb=params[1], c1=params[2], c2=params[3], eps_1=params[4], rho=1.0)
    elif name == "IsotropicElectroMechanics_0":
        # params (mu, lamb, eps_1): electric enthalpy W_n(C) - eps_1/2 J C^-1:(E0 x E0)
        m = F.IsotropicElectroMechanics_0(3, mu=params[0], lamb=params[1], eps_1=params[2], rho=1.0)
    elif name == "IsotropicElectroMechanics_101":
        # params (mu, lamb, eps_1): neo-Hookean electromechanics in terms of internal energy
        m = F.IsotropicElectroMechanics_101(3, mu=params[0], lamb=params[1], eps_1=params[2], rho=1.0)
    elif name == "IsotropicElectroMechanics_105":
        # params (mu1, mu2, lamb, eps_1, eps_2): W_mn + |D0|^2 / (2 eps_1) + |F D0|^2 / (2 eps_2)
        m = F.IsotropicElectroMechanics_105(3, mu1=params[0], mu2=params[1], lamb=params[2], eps_1=params[3],
                                            eps_2=params[4], rho=1.0)
    elif name == "IsotropicElectroMechanics_106":
        # params (mu1, mu2, lamb, eps_1, eps_2): 108's energy plus |D0|^2 / (2 eps_1)
        m = F.IsotropicElectroMechanics_106(3, mu1=params[0], mu2=params[1], lamb=params[2], eps_1=params[3],
                                            eps_2=params[4], rho=1.0)
    elif name == "IsotropicElectroMechanics_108":
        # params (mu1, mu2, lamb, eps_2): internal-energy electromechanics, displacement-potential form
        m = F.IsotropicElectroMechanics_108(3, mu1=params[0], mu2=params[1], lamb=params[2], eps_2=params[3], rho=1.0)
    else:
        raise ValueError(name)
    m.has_low_level_dispatcher = False
    return m


def fibre_directions(nelem, seed):
    """Seeded unit fibre directions per element (the reference's anisotropic_orientations)."""
    v = np.random.default_rng(seed).standard_normal((nelem, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def jittered_tet_mesh(F, nx, ny, nz, L, seed, jitter=0.15):
    """Seeded jittered lattice on [0,L[0]]x[0,L[1]]x[0,L[2]] split by Delaunay, reoriented positive."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    xs = [np.linspace(0, L[i], n + 1) for i, n in enumerate((nx, ny, nz))]
    P = np.stack(np.meshgrid(*xs, indexing="ij"), -1).reshape(-1, 3)
    h = np.array([L[0] / nx, L[1] / ny, L[2] / nz])
    interior = np.all((P > 1e-12) & (P < np.array(L) - 1e-12), axis=1)
    P[interior] += rng.uniform(-jitter, jitter, size=(interior.sum(), 3)) * h
    tri = Delaunay(P)
    el = tri.simplices.astype(np.int64)
    v = P[el]
    vol = np.einsum("ij,ij->i", np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), v[:, 3] - v[:, 0])
    keep = np.abs(vol) > 1e-12 * np.prod(h)
    el = el[keep]
    vol = vol[keep]
    neg = vol < 0
    el[neg, 1], el[neg, 2] = el[neg, 2].copy(), el[neg, 1].copy()
    mesh = F.Mesh()
    mesh.element_type = "tet"
    mesh.elements = el
    mesh.points = P
    mesh.nelem = el.shape[0]
    mesh.nnode = P.shape[0]
    mesh.GetBoundaryFacesTet()
    mesh.GetBoundaryEdgesTet()
    return mesh


def build_mesh(F, spec):
    kind = spec["mesh"]
    if kind == "cube_hex":
        mesh = F.Mesh()
        mesh.Cube(element_type="hex", nx=spec["n"][0], ny=spec["n"][1], nz=spec["n"][2])
    elif kind == "cube_tet":
        mesh = F.Mesh()
        mesh.Cube(element_type="tet", nx=spec["n"][0], ny=spec["n"][1], nz=spec["n"][2])
    elif kind == "box_hex":
        mesh = F.Mesh()
        mesh.Parallelepiped(lower_left_rear_point=(0, 0, 0), upper_right_front_point=spec["L"],
                            nx=spec["n"][0], ny=spec["n"][1], nz=spec["n"][2], element_type="hex")
    elif kind == "jitter_tet":
        mesh = jittered_tet_mesh(F, *spec["n"], L=spec["L"], seed=spec["mesh_seed"])
    else:
        raise ValueError(kind)
    if mesh.element_type == "tet":
        # the reference's numpy element path integrates with the signed Jacobian determinant
        # (DisplacementFormulation.py:146) while its native path uses |det| (_KinematicMeasures_.h:94-99);
        # the two agree only on positively oriented elements, so reorient before raising the order
        el = np.asarray(mesh.elements).astype(np.int64)
        v = np.asarray(mesh.points)[el]
        vol = np.einsum("ij,ij->i", np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), v[:, 3] - v[:, 0])
        neg = vol < 0
        el[neg, 1], el[neg, 2] = el[neg, 2].copy(), el[neg, 1].copy()
        mesh.elements = el
    if spec["p"] > 1:
        mesh.GetHighOrderMesh(p=spec["p"])
    mesh.ChangeType()
    return mesh


def reference_assembly(F, spec, mesh, x, recompute):
    """K (CSR) and T from the reference's AssembleForm, pure-numpy element path."""
    mat = make_material(F, spec["material"], spec["params"])
    if spec.get("fibre_seed") is not None:
        mat.anisotropic_orientations = fibre_directions(mesh.nelem, spec["fibre_seed"])
    kw = {} if spec.get("qdeg") is None else {"quadrature_degree": spec["qdeg"]}
    form = F.DisplacementFormulation(mesh, **kw)
    solver = F.FEMSolver(optimise=False, recompute_sparsity_pattern=recompute,
                         analysis_nature=spec.get("nature", "nonlinear"))
    K, T = F.AssembleForm(form, mesh, mat, solver, Eulerx=x)
    return K.tocsr(), np.asarray(T).ravel(), form, mat, solver


def element_matrices(F, form, mat, solver, mesh, x, elems):
    fs = form.function_spaces[0]
    Ks, ts = [], []
    for e in elems:
        X = mesh.points[mesh.elements[e].astype(np.int64)]
        xe = x[mesh.elements[e].astype(np.int64)]
        K_e, t_e = form.GetLocalStiffness(fs, mat, X, xe, solver, e)
        Ks.append(K_e)
        ts.append(np.asarray(t_e).ravel())
    return np.array(Ks), np.array(ts)


def reference_forces(F, spec, mesh, form, mat):
    """Traction on the faces of the x = max plane (seeded traction per face) and the body force,
    from the reference's AssembleExternalTractionForces / AssembleBodyForces (Assembly.py:451-560)."""
    import types
    from Florence.FiniteElements.Assembly.Assembly import AssembleBodyForces, AssembleExternalTractionForces
    faces = np.asarray(mesh.faces).astype(np.int64)
    xmax = mesh.points[:, 0].max()
    flags = np.all(np.abs(mesh.points[faces][:, :, 0] - xmax) < 1e-9, axis=1)
    traction = np.random.default_rng(spec["seed"] + 100).uniform(-1, 1, (faces.shape[0], 3))
    bc = types.SimpleNamespace(is_applied_neumann_shape_functions_computed=False, neumann_flags=flags,
                               applied_neumann=traction, is_body_force_shape_functions_computed=False)
    mat.nvar, mat.ndim = 3, 3
    fsf = form.function_spaces[-1]
    Ft = AssembleExternalTractionForces(bc, mesh, mat, fsf)
    Fb = AssembleBodyForces(bc, mesh, mat, form.function_spaces[0])
    return dict(faces=faces, neumann_flags=flags, applied_neumann=traction, face_Bases=fsf.Bases,
                face_AllGauss=np.ravel(fsf.AllGauss), face_Jm=fsf.Jm, F_traction=np.ravel(Ft), F_body=np.ravel(Fb),
                rho_body=np.array(float(mat.rho)))


def lumped_mass(F, form, mat, mesh, x):
    from Florence.FiniteElements.Assembly.Assembly import AssembleExplicit_NoLLD_Mass
    fs = form.function_spaces[0]
    form.GetConstantMassIntegrand(fs, mat)
    solver = F.FEMSolver(optimise=False, analysis_type="dynamic", analysis_subtype="explicit", mass_type="lumped")
    solver.is_mass_computed = False
    M = AssembleExplicit_NoLLD_Mass(solver, fs, form, mesh, mat, x, np.zeros(mesh.points.shape[0]))
    return np.asarray(M).ravel()


def consistent_mass(F, form, mat, mesh, x):
    """The reference's consistent mass (Assembly.py:608-657 with mass_type="consistent") as a
    canonical CSR: (indptr, indices, data), duplicates summed, columns sorted."""
    from Florence.FiniteElements.Assembly.Assembly import AssembleExplicit_NoLLD_Mass
    fs = form.function_spaces[0]
    form.GetConstantMassIntegrand(fs, mat)
    solver = F.FEMSolver(optimise=False, analysis_type="dynamic", analysis_subtype="explicit", mass_type="consistent")
    solver.is_mass_computed = False
    M = AssembleExplicit_NoLLD_Mass(solver, fs, form, mesh, mat, x, np.zeros(mesh.points.shape[0])).tocsr()
    M.sum_duplicates()
    M.sort_indices()
    return M.indptr.astype(np.int32), M.indices.astype(np.int32), M.data


CASES = [
    dict(name="hex_p1_nh", mesh="cube_hex", n=(2, 2, 2), p=1, material="NeoHookean", params=(1.0, 10.0), seed=10,
         amp=0.01, qdeg=None, emat=(0, 7), mass=True),
    dict(name="hex_p2_nh_q5", mesh="cube_hex", n=(2, 2, 2), p=2, material="NeoHookean", params=(1.0, 10.0), seed=11,
         amp=0.01, qdeg=5, emat=(0, 3, 7), mass=True, triplet=True),
    dict(name="hex_p2_mr", mesh="cube_hex", n=(2, 2, 1), p=2, material="MooneyRivlin", params=(0.5, 0.5, 20.0),
         seed=12, amp=0.05, qdeg=None, emat=(0, 3), mass=False, forces=True),
    dict(name="box_hex_p2_nh_big", mesh="box_hex", L=(4.0, 1.0, 1.0), n=(4, 2, 2), p=2, material="NeoHookean",
         params=(1.0, 1000.0), seed=13, amp=0.02, qdeg=None, emat=(1,), mass=True),
    dict(name="hex_p3_nh", mesh="cube_hex", n=(1, 1, 2), p=3, material="NeoHookean", params=(1.3, 7.0), seed=14,
         amp=0.01, qdeg=None, emat=(1,), mass=False),
    dict(name="hex_p4_nh", mesh="cube_hex", n=(1, 1, 1), p=4, material="NeoHookean", params=(0.8, 30.0), seed=15,
         amp=0.01, qdeg=None, emat=(0,), mass=False),
    dict(name="tet_p1_nh", mesh="cube_tet", n=(2, 2, 2), p=1, material="NeoHookean", params=(1.0, 10.0), seed=16,
         amp=0.01, qdeg=None, emat=(0, 5), mass=True),
    dict(name="tet_p2_mr", mesh="cube_tet", n=(1, 1, 1), p=2, material="MooneyRivlin", params=(0.5, 0.5, 20.0),
         seed=17, amp=0.02, qdeg=None, emat=(0, 2), mass=True, forces=True),
    # linear analysis (no geometry update, no residual): at x = X the low-level and numpy paths agree
    # (the low-level kinematics take spatial gradients from x even without the update,
    # _KinematicMeasures_.h:95-103; the numpy path then takes material gradients)
    dict(name="hex_p2_le", mesh="cube_hex", n=(2, 2, 1), p=2, material="LinearElastic", params=(1.0, 2.5), seed=19,
         amp=0.0, qdeg=None, emat=(0, 2), mass=False, nature="linear"),
    dict(name="tet_p2_nimr", mesh="cube_tet", n=(1, 1, 1), p=2, material="NearlyIncompressibleMooneyRivlin",
         params=(0.4, 0.1, 15.0), seed=20, amp=0.03, qdeg=None, emat=(0, 3), mass=False, triplet=True),
    dict(name="hex_p2_amr", mesh="cube_hex", n=(2, 1, 1), p=2, material="AnisotropicMooneyRivlin_1",
         params=(0.5, 0.3, 20.0, 0.7), fibre_seed=21, seed=22, amp=0.04, qdeg=None, emat=(0, 1), mass=False),
    dict(name="tet_p2_amr", mesh="cube_tet", n=(1, 1, 1), p=2, material="AnisotropicMooneyRivlin_1",
         params=(0.4, 0.2, 10.0, 1.1), fibre_seed=23, seed=24, amp=0.03, qdeg=None, emat=(0, 3), mass=False,
         triplet=True),
    dict(name="tet_p3_mr_jitter", mesh="jitter_tet", L=(4.0, 1.0, 1.0), n=(4, 1, 1), mesh_seed=1, p=3,
         material="MooneyRivlin", params=(0.5, 0.5, 20.0), seed=18, amp=0.01, qdeg=None, emat=(0, 4), mass=True,
         triplet=True),
]


def make_case(F, spec):
    t0 = time.time()
    mesh = build_mesh(F, spec)
    rng = np.random.default_rng(spec["seed"])
    x = mesh.points + rng.uniform(-spec["amp"], spec["amp"], size=mesh.points.shape)
    K, T, form, mat, solver = reference_assembly(F, spec, mesh, x, recompute=False)
    fs = form.function_spaces[0]
    out = dict(
        points=mesh.points, elements=mesh.elements.astype(np.int64), Eulerx=x,
        Jm=fs.Jm, AllGauss=fs.AllGauss.ravel(), Bases=fs.Bases,
        material=np.array(spec["material"]), params=np.array(spec["params"], np.float64),
        update=np.array(int(solver.requires_geometry_update)),
        **({"orientations": np.asarray(mat.anisotropic_orientations, np.float64)}
           if spec.get("fibre_seed") is not None else {}),
        K_indptr=K.indptr.astype(np.int32), K_indices=K.indices.astype(np.int32), K_data=K.data, T=T,
        sp_indices=solver.indices.astype(np.int32), sp_indptr=solver.indptr.astype(np.int32),
        sp_data_local=solver.data_local_indices.astype(np.int32),
        sp_data_global=solver.data_global_indices.astype(np.int32),
    )
    if spec.get("triplet"):
        K2, T2, *_ = reference_assembly(F, spec, build_mesh(F, spec), x, recompute=True)
        out["K_triplet_data"] = K2.data
        assert np.array_equal(K2.indptr, K.indptr) and np.array_equal(K2.indices, K.indices)
    emat = list(spec["emat"])
    Ke, te = element_matrices(F, form, mat, solver, mesh, x, emat)
    out["emat_ids"] = np.array(emat, np.int64)
    out["emat_K"] = Ke
    out["emat_t"] = te
    if spec.get("forces"):
        out.update(reference_forces(F, spec, mesh, form, mat))
    if spec.get("mass"):
        rho = 1.0
        out["M_lumped"] = lumped_mass(F, form, mat, mesh, x)
        out["rho"] = np.array(rho)
        out["Mc_indptr"], out["Mc_indices"], out["Mc_data"] = consistent_mass(F, form, mat, mesh, x)
    np.savez_compressed(os.path.join(HERE, spec["name"] + ".npz"), **out)
    print("%-22s E=%-4d npe=%-3d nq=%-3d nnz=%-8d %.1fs" % (spec["name"], mesh.nelem, mesh.elements.shape[1],
          fs.AllGauss.shape[0], K.nnz, time.time() - t0), flush=True)


DPF_CASES = [
    dict(name="dpf_tet_p2_em108", mesh="cube_tet", n=(1, 1, 1), p=2, material="IsotropicElectroMechanics_108",
         params=(0.5, 0.3, 10.0, 2.0), seed=30, amp=0.02, phi_amp=0.1, emat=(0, 4)),
    dict(name="dpf_hex_p2_em108", mesh="box_hex", n=(2, 1, 1), L=(2.0, 1.0, 1.0), p=2,
         material="IsotropicElectroMechanics_108", params=(0.4, 0.2, 15.0, 1.5), seed=31, amp=0.03, phi_amp=0.2,
         emat=(0, 1)),
    dict(name="dpf_hex_p2_em0", mesh="box_hex", n=(2, 1, 1), L=(2.0, 1.0, 1.0), p=2,
         material="IsotropicElectroMechanics_0", params=(1.1, 9.0, 0.6), seed=33, amp=0.03, phi_amp=0.3,
         emat=(0, 1)),
    dict(name="dpf_tet_p2_em106", mesh="cube_tet", n=(1, 1, 1), p=2, material="IsotropicElectroMechanics_106",
         params=(0.5, 0.3, 10.0, 1.5, 2.5), seed=34, amp=0.03, phi_amp=0.2, emat=(1, 5)),
    dict(name="dpf_hex_p2_em105", mesh="box_hex", n=(2, 1, 1), L=(2.0, 1.0, 1.0), p=2,
         material="IsotropicElectroMechanics_105", params=(0.6, 0.25, 12.0, 2.0, 1.2), seed=35, amp=0.03,
         phi_amp=0.25, emat=(0, 1)),
    dict(name="dpf_tet_p2_steinmann", mesh="cube_tet", n=(1, 1, 1), p=2, material="SteinmannModel",
         params=(1.0, 8.0, 0.15, 0.1, 1.3), seed=36, amp=0.03, phi_amp=0.25, emat=(2, 3)),
    dict(name="dpf_tet_p2_piezo100", mesh="cube_tet", n=(1, 1, 1), p=2, material="Piezoelectric_100",
         params=(0.5, 0.3, 0.4, 10.0, 1.5, 2.0, 3.0), fibre_seed=37, seed=38, amp=0.03, phi_amp=0.2, emat=(0, 2)),
    dict(name="dpf_tet_p2_em101", mesh="cube_tet", n=(1, 1, 1), p=2, material="IsotropicElectroMechanics_101",
         params=(0.8, 12.0, 1.7), seed=32, amp=0.02, phi_amp=0.15, emat=(0, 3)),
]


def make_dpf_case(F, spec):
    """Displacement-potential formulation (nvar 4: three displacements and the electric potential)
    through the reference's numpy element path (DisplacementPotentialFormulation.GetLocalStiffness,
    Florence/VariationalPrinciple/DisplacementPotentialFormulation.py:108-200): tangent CSR and
    residual at seeded displacements and potentials, with the reference's nvar=4 sparsity."""
    t0 = time.time()
    mesh = build_mesh(F, spec)
    rng = np.random.default_rng(spec["seed"])
    x = mesh.points + rng.uniform(-spec["amp"], spec["amp"], size=mesh.points.shape)
    phi = rng.uniform(-spec["phi_amp"], spec["phi_amp"], size=mesh.points.shape[0])
    mat = make_material(F, spec["material"], spec["params"])
    if spec.get("fibre_seed") is not None:
        mat.anisotropic_orientations = fibre_directions(mesh.nelem, spec["fibre_seed"])
    form = F.DisplacementPotentialFormulation(mesh)
    solver = F.FEMSolver(optimise=False, recompute_sparsity_pattern=False)
    K, T = F.AssembleForm(form, mesh, mat, solver, Eulerx=x, Eulerp=phi)
    K = K.tocsr()
    fs = form.function_spaces[0]
    Ks, ts = [], []
    for e in spec["emat"]:
        nodes = mesh.elements[e].astype(np.int64)
        K_e, t_e = form.GetLocalStiffness(fs, mat, mesh.points[nodes], x[nodes], phi[nodes], solver, e)
        Ks.append(K_e)
        ts.append(np.asarray(t_e).ravel())
    out = dict(
        points=mesh.points, elements=mesh.elements.astype(np.int64), Eulerx=x, Eulerp=phi,
        Jm=fs.Jm, AllGauss=fs.AllGauss.ravel(), Bases=fs.Bases, nvar=np.array(4),
        material=np.array(spec["material"]), params=np.array(spec["params"], np.float64),
        update=np.array(int(solver.requires_geometry_update)),
        **({"orientations": np.asarray(mat.anisotropic_orientations, np.float64)}
           if spec.get("fibre_seed") is not None else {}),
        K_indptr=K.indptr.astype(np.int32), K_indices=K.indices.astype(np.int32), K_data=K.data,
        T=np.asarray(T).ravel(),
        sp_indices=solver.indices.astype(np.int32), sp_indptr=solver.indptr.astype(np.int32),
        sp_data_local=solver.data_local_indices.astype(np.int32),
        sp_data_global=solver.data_global_indices.astype(np.int32),
        emat_ids=np.array(spec["emat"], np.int64), emat_K=np.array(Ks), emat_t=np.array(ts),
    )
    np.savez_compressed(os.path.join(HERE, spec["name"] + ".npz"), **out)
    print("%-22s E=%-4d npe=%-3d nq=%-3d nnz=%-8d %.1fs" % (spec["name"], mesh.nelem, mesh.elements.shape[1],
          fs.AllGauss.shape[0], K.nnz, time.time() - t0), flush=True)


def make_config1(F):
    """Structured 8x8x8 p=2 hex cube, Gauss order 5 (125 points), neo-Hookean mu=1, lambda=10,
    u ~ U(-0.01, 0.01) per dof from default_rng(0). The full CSR is too large to commit, so the
    fixture keeps the inputs, hashes of the exact integer structure, and value probes."""
    t0 = time.time()
    spec = dict(mesh="cube_hex", n=(8, 8, 8), p=2, material="NeoHookean", params=(1.0, 10.0), qdeg=5)
    mesh = build_mesh(F, spec)
    rng = np.random.default_rng(0)
    x = mesh.points + rng.uniform(-0.01, 0.01, size=mesh.points.shape)
    K, T, form, mat, solver = reference_assembly(F, spec, mesh, x, recompute=False)
    fs = form.function_spaces[0]
    v = np.random.default_rng(42).standard_normal(K.shape[0])
    emat = [0, 137, 511]
    Ke, te = element_matrices(F, form, mat, solver, mesh, x, emat)
    out = dict(
        points=mesh.points, elements=mesh.elements.astype(np.int64), Eulerx=x,
        Jm=fs.Jm, AllGauss=fs.AllGauss.ravel(), Bases=fs.Bases,
        material=np.array("NeoHookean"), params=np.array([1.0, 10.0]),
        nnz=np.array(K.nnz), K_fro=np.array(np.linalg.norm(K.data)), K_sum=np.array(K.data.sum()),
        K_matvec=K @ v, matvec_seed=np.array(42), T=T,
        K_diag=K.diagonal(),
        sha_indptr=np.array(sha(K.indptr, "<i4")), sha_indices=np.array(sha(K.indices, "<i4")),
        sha_data_local=np.array(sha(solver.data_local_indices, "<i4")),
        sha_data_global=np.array(sha(solver.data_global_indices, "<i4")),
        emat_ids=np.array(emat, np.int64), emat_K=Ke, emat_t=te,
    )
    np.savez_compressed(os.path.join(HERE, "config1_hex8_p2_q5.npz"), **out)
    print("config1 E=%d nnz=%d %.1fs" % (mesh.nelem, K.nnz, time.time() - t0), flush=True)


if __name__ == "__main__":
    F = florence_harness.import_florence()
    only = sys.argv[1:]
    for spec in CASES:
        if not only or spec["name"] in only:
            make_case(F, spec)
    for spec in DPF_CASES:
        if not only or spec["name"] in only:
            make_dpf_case(F, spec)
    if not only or "config1" in only:
        make_config1(F)
