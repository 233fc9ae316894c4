"""numpy restatement of the displacement-potential (electromechanics) assembly.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker, never by the product path. Pinned
against golden vectors made by the reference's own code (tests/golden/make_golden.py,
``DPF_CASES``; tests/test_dpf_oracle.py).

What it restates (paths inside the Florence repository):
* the element integral of DisplacementPotentialFormulation.GetLocalStiffness
  (VariationalPrinciple/DisplacementPotentialFormulation.py:108-200): per Gauss point the
  kinematics, the spatial electric field E = -grad(phi), the material's electric displacement,
  Cauchy stress and 9x9 Hessian, the constitutive term B H B^T and the residual B [sigma; D], the
  geometric term on the displacement dofs; weights w |det dX/dxi| |J|;
* the DPF strain-displacement matrix and total traction (Voigt order xx, yy, zz, xy, xz, yz;
  electric rows carry grad N; VariationalPrinciple/_ConstitutiveStiffness_/
  DisplacementPotentialApproachIndices.pyx:1-50, :203-230);
* Piezoelectric_100 (MaterialLibrary/Piezoelectric_100.py:43-170), transversely isotropic with one
  fibre direction per element;
* IsotropicElectroMechanics_0 and SteinmannModel, electric-enthalpy models whose Hessians are
  given directly (MaterialLibrary/IsotropicElectroMechanics_0.py:43-100, SteinmannModel.py:40-120);
* IsotropicElectroMechanics_101 (MaterialLibrary/IsotropicElectroMechanics_101.py:38-94),
  IsotropicElectroMechanics_105 (IsotropicElectroMechanics_105.py:41-104),
  IsotropicElectroMechanics_106 (IsotropicElectroMechanics_106.py:41-125) and
  IsotropicElectroMechanics_108, internal-energy models (MaterialLibrary/
  IsotropicElectroMechanics_108.py:36-113, LLDispatch/CythonSource/_IsotropicElectroMechanics_108_.h):
  D = eps_2 E, the internal-energy elasticity, coupling and dielectric tensors turned into the
  electric-enthalpy Hessian by the Legendre transform (LegendreTransform/LegendreTransform.py:22-40);
* symmetric Voigt reduction of 4th- and 3rd-order tensors (Tensor/Numeric.pyx:166-270): the
  average over the last pair's (4th order) or first pair's (3rd order) index swap.
Global dof of (node n, field v) is 4 n + v (v = 3: the electric potential).
"""
import numpy as np

NVAR = 4
VOIGT_PAIRS = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


def voigt4(C):
    """6x6 symmetric Voigt form: V[I, J] = (C[i,j,k,l] + C[i,j,l,k]) / 2 for I <= J, mirrored."""
    V = np.zeros((6, 6))
    for I, (i, j) in enumerate(VOIGT_PAIRS):
        for J in range(I, 6):
            k, l = VOIGT_PAIRS[J]
            V[I, J] = 0.5 * (C[i, j, k, l] + C[i, j, l, k])
            V[J, I] = V[I, J]
    return V


def voigt3(e):
    """6x3 Voigt form of a 3rd-order tensor: V[I, k] = (e[i,j,k] + e[j,i,k]) / 2."""
    V = np.zeros((6, 3))
    for I, (i, j) in enumerate(VOIGT_PAIRS):
        V[I] = 0.5 * (e[i, j] + e[j, i])
    return V


def em108_tensors(b, J, D, mu1, mu2, lamb, eps_2):
    """Internal-energy elasticity W_el[i,j,k,l] and coupling W_cp[i,j,k] of IsotropicElectroMechanics_108."""
    d = np.eye(3)
    DD = D @ D
    # 4th-order identities and b products, index order (i, j, k, l)
    dd_ij_kl = d[:, :, None, None] * d[None, None, :, :]
    dd_ik_jl = d[:, None, :, None] * d[None, :, None, :]
    dd_il_jk = d[:, None, None, :] * d[None, :, :, None]
    bb_ij_kl = b[:, :, None, None] * b[None, None, :, :]
    bb_ik_jl = b[:, None, :, None] * b[None, :, None, :]
    bb_il_jk = b[:, None, None, :] * b[None, :, :, None]
    sym = dd_ik_jl + dd_il_jk
    W_el = (2.0 * mu2 / J) * (2.0 * bb_ij_kl - bb_ik_jl - bb_il_jk) + (2.0 * (mu1 + 2.0 * mu2) / J) * sym \
        + lamb * (2.0 * J - 1.0) * dd_ij_kl - lamb * (J - 1.0) * sym \
        + (0.5 * DD * (sym + dd_ij_kl) - d[:, :, None, None] * np.outer(D, D)[None, None]
           - np.outer(D, D)[:, :, None, None] * d[None, None]) / eps_2
    # coupling W_cp[i,j,k] = (delta_ik D_j + D_i delta_jk - delta_ij D_k) / eps_2
    W_cp = (d[:, None, :] * D[None, :, None] + D[:, None, None] * d[None, :, :]
            - d[:, :, None] * D[None, None, :]) / eps_2
    return W_el, W_cp


def em108_from_D(F, D, mu1, mu2, lamb, eps_2):
    """(J, sigma, b) of IsotropicElectroMechanics_108's stress at a given electric displacement."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    sigma = (2.0 * mu1 / J) * b + (2.0 * mu2 / J) * (np.trace(b) * b - b @ b) \
        - (2.0 * (mu1 + 2.0 * mu2) / J) * d + lamb * (J - 1.0) * d \
        + (np.outer(D, D) - 0.5 * (D @ D) * d) / eps_2
    return J, sigma, b


def em108(F, E, mu1, mu2, lamb, eps_2):
    """(D, sigma, H[9x9]) of IsotropicElectroMechanics_108 at deformation gradient F and spatial
    electric field E: D = eps_2 E, dielectric tensor I / eps_2."""
    D = eps_2 * E
    J, sigma, b = em108_from_D(F, D, mu1, mu2, lamb, eps_2)
    W_el, W_cp = em108_tensors(b, J, D, mu1, mu2, lamb, eps_2)
    return D, sigma, enthalpy_hessian(W_el, W_cp, np.eye(3) / eps_2)


def enthalpy_hessian(W_el, W_cp, W_di):
    """9x9 electric-enthalpy Hessian [[C, -P], [-P^T, H_di]] from the internal energy's
    elasticity, coupling and dielectric tensors (the Legendre transform)."""
    H_di = -np.linalg.inv(W_di)
    H_cp = -np.tensordot(W_cp, H_di, axes=([2], [0]))         # H_cp[k,l,j] = -sum_i W_cp[k,l,i] H_di[i,j]
    H_el = W_el - np.einsum("ijk,mlk->ijlm", W_cp, H_cp)     # sum_k W_cp[i,j,k] H_cp[m,l,k]
    C_V, P_V = voigt4(H_el), voigt3(H_cp)
    H = np.zeros((9, 9))
    H[:6, :6] = C_V
    H[:6, 6:] = -P_V
    H[6:, :6] = -P_V.T
    H[6:, 6:] = H_di
    return H


def em106(F, E, mu1, mu2, lamb, eps_1, eps_2):
    """(D, sigma, H[9x9]) of IsotropicElectroMechanics_106 (MaterialLibrary/IsotropicElectroMechanics_106.py:41-125,
    LLDispatch/CythonSource/_IsotropicElectroMechanics_106_.h): 108's stress, elasticity and
    coupling with the dielectric tensor J/eps_1 b^-1 + I/eps_2, D = (that tensor)^-1 E."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    W_di = (J / eps_1) * np.linalg.inv(b) + d / eps_2
    D = np.linalg.solve(W_di, E)
    _, sigma, _ = em108_from_D(F, D, mu1, mu2, lamb, eps_2)
    W_el, W_cp = em108_tensors(b, J, D, mu1, mu2, lamb, eps_2)
    return D, sigma, enthalpy_hessian(W_el, W_cp, W_di)


def em105(F, E, mu1, mu2, lamb, eps_1, eps_2):
    """(D, sigma, H[9x9]) of IsotropicElectroMechanics_105 (MaterialLibrary/IsotropicElectroMechanics_105.py:41-104,
    LLDispatch/CythonSource/_IsotropicElectroMechanics_105_.h): internal energy
    W_mn(C) + |D0|^2 / (2 eps_1) + |F D0|^2 / (2 eps_2); dielectric tensor J/eps_1 b^-1 + J/eps_2 I,
    D = (that tensor)^-1 E."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    W_di = (J / eps_1) * np.linalg.inv(b) + (J / eps_2) * d
    D = np.linalg.solve(W_di, E)
    sigma = (2.0 * mu1 / J) * b + (2.0 * mu2 / J) * (np.trace(b) * b - b @ b) \
        - (2.0 * (mu1 + 2.0 * mu2) / J) * d + lamb * (J - 1.0) * d + (J / eps_2) * np.outer(D, D)
    W_el, _ = em108_tensors(b, J, np.zeros(3), mu1, mu2, lamb, eps_2)   # the mechanical part alone
    W_cp = (J / eps_2) * (d[:, None, :] * D[None, :, None] + D[:, None, None] * d[None, :, :])
    return D, sigma, enthalpy_hessian(W_el, W_cp, W_di)


def em101(F, E, mu, lamb, eps_1):
    """(D, sigma, H[9x9]) of IsotropicElectroMechanics_101 (MaterialLibrary/IsotropicElectroMechanics_101.py:38-94,
    LLDispatch/CythonSource/_IsotropicElectroMechanics_101_.h): internal energy
    W(C, D0) = W_neo(C) + |F D0|^2 / (2 eps_1), D = eps_1 / J E."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    D = (eps_1 / J) * E
    sigma = (mu / J) * (b - d) + lamb * (J - 1.0) * d + (J / eps_1) * np.outer(D, D)
    dd_ij_kl = d[:, :, None, None] * d[None, None, :, :]
    sym = d[:, None, :, None] * d[None, :, None, :] + d[:, None, None, :] * d[None, :, :, None]
    W_el = lamb * (2.0 * J - 1.0) * dd_ij_kl + (mu / J - lamb * (J - 1.0)) * sym
    W_cp = (J / eps_1) * (d[:, None, :] * D[None, :, None] + D[:, None, None] * d[None, :, :])
    W_di = (J / eps_1) * d
    return D, sigma, enthalpy_hessian(W_el, W_cp, W_di)


def em0(F, E, mu, lamb, eps_1):
    """(D, sigma, H[9x9]) of IsotropicElectroMechanics_0 (MaterialLibrary/IsotropicElectroMechanics_0.py:43-100):
    electric enthalpy W(C, E0) = W_n(C) - eps_1/2 J C^-1:(E0 x E0); the Hessian is given in
    enthalpy form directly, D = eps_1 E."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    EE = np.outer(E, E)
    D = eps_1 * E
    sigma = (mu / J) * (b - d) + (lamb / J) * np.log(J) * d + eps_1 * (EE - 0.5 * (E @ E) * d)
    dd_ij_kl = d[:, :, None, None] * d[None, None, :, :]
    sym = d[:, None, :, None] * d[None, :, None, :] + d[:, None, None, :] * d[None, :, :, None]
    d_ij_EE_kl = d[:, :, None, None] * EE[None, None]
    EE_ij_d_kl = EE[:, :, None, None] * d[None, None]
    EE_ik_d_jl = EE[:, None, :, None] * d[None, :, None, :]
    EE_il_d_jk = EE[:, None, None, :] * d[None, :, :, None]
    d_ik_EE_jl = d[:, None, :, None] * EE[None, :, None, :]
    d_il_EE_jk = d[:, None, None, :] * EE[None, :, :, None]
    C = (lamb / J) * dd_ij_kl - (lamb * np.log(J) - mu) / J * sym \
        + eps_1 * (d_ij_EE_kl + EE_ij_d_kl - EE_ik_d_jl - EE_il_d_jk - d_ik_EE_jl - d_il_EE_jk) \
        + eps_1 * (E @ E) * 0.5 * (sym - dd_ij_kl)
    # coupling P[i,j,k] = eps_1 (delta_ik E_j + delta_jk E_i - delta_ij E_k)
    P = eps_1 * (d[:, None, :] * E[None, :, None] + E[:, None, None] * d[None, :, :] - d[:, :, None] * E[None, None, :])
    H = np.zeros((9, 9))
    H[:6, :6] = voigt4(C)
    H[:6, 6:] = -voigt3(P)
    H[6:, :6] = -voigt3(P).T
    H[6:, 6:] = -eps_1 * d
    return D, sigma, H


def steinmann(F, E, mu, lamb, c1, c2, eps_1):
    """(D, sigma, H[9x9]) of SteinmannModel (MaterialLibrary/SteinmannModel.py:40-120,
    LLDispatch/CythonSource/_SteinmannModel_.h): electric enthalpy
    W_n(C) + c1 I:(E0 x E0) + c2 C:(E0 x E0) - eps_1/2 J C^-1:(E0 x E0), Hessian given directly:
    material 0's plus c2 terms in the stress and coupling and c1, c2 terms in the dielectric block."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    be = b @ E
    D0, sigma0, H = em0(F, E, mu, lamb, eps_1)
    D = eps_1 * E - (2.0 * c1 / J) * be - (2.0 * c2 / J) * (b @ b) @ E
    sigma = sigma0 + (2.0 * c2 / J) * np.outer(be, be)
    P = eps_1 * (d[:, None, :] * E[None, :, None] + E[:, None, None] * d[None, :, :] - d[:, :, None] * E[None, None, :]) \
        + (2.0 * c2 / J) * (b[:, None, :] * be[None, :, None] + be[:, None, None] * b[None, :, :])
    H[:6, 6:] = -voigt3(P)
    H[6:, :6] = -voigt3(P).T
    H[6:, 6:] = -eps_1 * d + (2.0 * c1 / J) * b + (2.0 * c2 / J) * (b @ b)
    return D, sigma, H


def piezo100(F, E, N, mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3):
    """(D, sigma, H[9x9]) of Piezoelectric_100 (MaterialLibrary/Piezoelectric_100.py:43-170), a
    transversely isotropic internal-energy model with fibre direction N (one per element):
    D = W_di^-1 (E - 2 s F N + 2 s / J H N), s = sqrt(mu3 / eps_3), H = J F^-T."""
    d = np.eye(3)
    J = np.linalg.det(F)
    b = F @ F.T
    Hc = J * np.linalg.inv(F).T
    FN, HN = F @ N, Hc @ N
    s = np.sqrt(mu3 / eps_3)
    W_di = (J / eps_1) * np.linalg.inv(b) + d / eps_2 + 2.0 * J * s * d
    D = np.linalg.solve(W_di, E - 2.0 * s * FN + (2.0 / J) * s * HN)
    hh = HN @ HN
    sigma = (2.0 * mu1 / J) * b + (2.0 * mu2 / J) * (np.trace(b) * b - b @ b) \
        - (2.0 * (mu1 + 2.0 * mu2 + mu3) / J) * d + lamb * (J - 1.0) * d \
        + (2.0 * mu3 / J) * (np.outer(FN, FN) + hh * d - np.outer(HN, HN)) \
        + (np.outer(D, D) - 0.5 * (D @ D) * d) / eps_2 + 2.0 * J * s * np.outer(D, D) \
        + 2.0 * s * (np.outer(D, FN) + np.outer(FN, D))
    dd_ij_kl = d[:, :, None, None] * d[None, None, :, :]
    sym = d[:, None, :, None] * d[None, :, None, :] + d[:, None, None, :] * d[None, :, :, None]
    hnhn = np.outer(HN, HN)
    # 108's tensors: its mechanical elasticity (at D = 0), its electric elasticity and coupling at D
    W_mech, _ = em108_tensors(b, J, np.zeros(3), mu1, mu2, lamb, eps_2)
    W_elec, W_cp108 = em108_tensors(b, J, D, 0.0, 0.0, 0.0, eps_2)
    # the fibre terms: delta_il HN_j HN_k + delta_jl HN_i HN_k + delta_ik HN_j HN_l + delta_jk HN_i HN_l
    fibre = (d[:, None, None, :] * hnhn[None, :, :, None] + d[None, :, None, :] * hnhn[:, None, :, None]
             + d[:, None, :, None] * hnhn[None, :, None, :] + d[None, :, :, None] * hnhn[:, None, None, :])
    W_el = W_mech + W_elec + (2.0 * mu3 / J) * sym \
        - (4.0 * mu3 / J) * (d[:, :, None, None] * hnhn[None, None] + hnhn[:, :, None, None] * d[None, None]) \
        + (2.0 * mu3 / J) * hh * (2.0 * dd_ij_kl - sym) + (2.0 * mu3 / J) * fibre
    W_cp = W_cp108 + 2.0 * J * s * (d[:, None, :] * D[None, :, None] + D[:, None, None] * d[None, :, :]) \
        + 2.0 * s * (d[:, None, :] * FN[None, :, None] + FN[:, None, None] * d[None, :, :])
    return D, sigma, enthalpy_hessian(W_el, W_cp, W_di)


# materials whose kinetics take the element's fibre direction (after F and E)
ORIENTED = {"Piezoelectric_100"}

MATERIALS = {"IsotropicElectroMechanics_108": em108, "SteinmannModel": steinmann, "Piezoelectric_100": piezo100, "IsotropicElectroMechanics_101": em101,
             "IsotropicElectroMechanics_0": em0, "IsotropicElectroMechanics_106": em106,
             "IsotropicElectroMechanics_105": em105}


def b_matrix(SG):
    """DPF strain-displacement matrix [4 npe, 9] from spatial gradients SG [3, npe]."""
    npe = SG.shape[1]
    B = np.zeros((NVAR * npe, 9))
    for a in range(npe):
        gx, gy, gz = SG[:, a]
        r = NVAR * a
        B[r + 0, 0], B[r + 1, 1], B[r + 2, 2] = gx, gy, gz
        B[r + 0, 3], B[r + 1, 3] = gy, gx
        B[r + 0, 4], B[r + 2, 4] = gz, gx
        B[r + 1, 5], B[r + 2, 5] = gz, gy
        B[r + 3, 6:9] = SG[:, a]
    return B


def element(material, params, X, x, phi, Jm, w, update=1, orientation=None):
    """(K_e [4 npe, 4 npe], t_e [4 npe]) of one element (orientation: its fibre direction, for the
    transversely isotropic materials)."""
    kin = MATERIALS[material]
    npe = X.shape[0]
    K = np.zeros((NVAR * npe, NVAR * npe))
    t = np.zeros(NVAR * npe)
    for g in range(w.shape[0]):
        dN = Jm[:, :, g]                      # [3, npe] parent gradients
        GX = dN @ X                           # dX/dxi
        MG = np.linalg.solve(GX, dN)          # material gradients [3, npe]
        F = x.T @ MG.T
        if update:
            SG = np.linalg.solve(dN @ x, dN)  # spatial gradients
            dv = w[g] * abs(np.linalg.det(GX)) * abs(np.linalg.det(F))
        else:
            SG = MG
            dv = w[g] * abs(np.linalg.det(GX))
        E = -SG @ phi
        D, sigma, H = kin(F, E, np.asarray(orientation, np.float64), *params) if material in ORIENTED \
            else kin(F, E, *params)
        B = b_matrix(SG)
        Kg = B @ H @ B.T
        geo = SG.T @ sigma @ SG               # grad N_a . sigma . grad N_b
        for v in range(3):
            Kg[v::NVAR, v::NVAR] += geo
        K += Kg * dv
        if update:
            tt = np.array([sigma[0, 0], sigma[1, 1], sigma[2, 2], sigma[0, 1], sigma[0, 2], sigma[1, 2], *D])
            t += (B @ tt) * dv
    return K, t


def assemble(material, params, points, elements, Eulerx, Eulerp, Jm, AllGauss, update=1, orientations=None):
    """Dense global tangent [4N, 4N] and residual [4N]. For small meshes."""
    P = np.asarray(points, np.float64)
    x = np.asarray(Eulerx, np.float64)
    phi = np.asarray(Eulerp, np.float64)
    el = np.asarray(elements, np.int64)
    Jm = np.asarray(Jm, np.float64)
    w = np.ravel(AllGauss).astype(np.float64)
    n = NVAR * P.shape[0]
    K = np.zeros((n, n))
    T = np.zeros(n)
    for e in range(el.shape[0]):
        nodes = el[e]
        Ke, te = element(material, params, P[nodes], x[nodes], phi[nodes], Jm, w, update,
                         None if orientations is None else orientations[e])
        dofs = (NVAR * nodes[:, None] + np.arange(NVAR)[None, :]).ravel()
        K[np.ix_(dofs, dofs)] += Ke
        T[dofs] += te
    return K, T
