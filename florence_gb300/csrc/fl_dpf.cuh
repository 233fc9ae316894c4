// fl_dpf.cuh -- Gauss-point and matrix-entry arithmetic of the displacement-potential
// (electromechanics) assembly: three displacements and the electric potential per node (nvar 4),
// a 9x9 Hessian (6 Voigt stresses + 3 electric displacements). Plain C++ so that the device kernel
// (fl_dpf.cu) and a host build of the same source use identical arithmetic.
//
// Reference (paths inside the Florence repository):
//   the element integral     FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDPF_.h:8-198,
//                            VariationalPrinciple/DisplacementPotentialFormulation.py:108-200
//   B rows and traction      VariationalPrinciple/_ConstitutiveStiffness_/DisplacementPotentialApproachIndices.pyx:1-50, :203-230
//                            (Voigt order xx, yy, zz, xy, xz, yz; the potential's row carries grad N)
//   materials 0, 101, 105, 106, 108, Steinmann, Piezoelectric_100
//                            MaterialLibrary/LLDispatch/CythonSource/_IsotropicElectroMechanics_0_.h, _101_.h, _105_.h, _106_.h,
//                            _IsotropicElectroMechanics_108_.h:32-112
//   Legendre transform       MaterialLibrary/LLDispatch/CythonSource/_LegendreTransform_.h (InternalEnergyToEnthalpy)
//   symmetric Voigt forms    Tensor/Numeric.pyx:166-270
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define FL_HD __host__ __device__ __forceinline__
#else
#define FL_HD inline
#endif

namespace fl {
namespace dpf {

constexpr int NV = 4;  // fields per node
constexpr int HV = 9;  // Hessian size

// Voigt index I -> tensor index pair: 0 xx, 1 yy, 2 zz, 3 xy, 4 xz, 5 yz
FL_HD int vp0(int I) { return I < 3 ? I : (I == 5 ? 1 : 0); }
FL_HD int vp1(int I) { return I < 3 ? I : (I == 3 ? 1 : 2); }
FL_HD double kd(int i, int j) { return i == j ? 1.0 : 0.0; }

FL_HD double det3(const double *m) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// inverse of a 3x3 matrix (row-major) by cofactors; returns the determinant
FL_HD double inv3(const double *m, double *r) {
    const double d = det3(m);
    const double id = 1.0 / d;
    r[0] = (m[4] * m[8] - m[5] * m[7]) * id;
    r[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    r[3] = (m[5] * m[6] - m[3] * m[8]) * id;
    r[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    r[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    r[6] = (m[3] * m[7] - m[4] * m[6]) * id;
    r[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    r[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return d;
}

// Electric-enthalpy Hessian H[9x9] = [[C, -P], [-P^T, -eps I]] of an internal-energy model whose
// dielectric tensor is isotropic, W_di = I / eps: the Legendre transform inverts it to -eps I,
// the enthalpy coupling is eps times the internal one, and the enthalpy elasticity subtracts
// eps sum_n W_cp(i,j,n) W_cp(k,l,n); C and P are their symmetric Voigt forms. Pt supplies the
// internal energy's elasticity wel(i,j,k,l) and coupling wcp(i,j,k) (symmetric in i, j).
template <class Pt>
FL_HD void enthalpy_hessian(const Pt &pt, double eps, double *H) {
    for (int I = 0; I < 6; ++I) {
        const int i = vp0(I), j = vp1(I);
        for (int K = I; K < 6; ++K) {
            const int k = vp0(K), l = vp1(K);
            double h1 = pt.wel(i, j, k, l), h2 = pt.wel(i, j, l, k);
            for (int n = 0; n < 3; ++n) {
                h1 -= eps * pt.wcp(i, j, n) * pt.wcp(k, l, n);
                h2 -= eps * pt.wcp(i, j, n) * pt.wcp(l, k, n);
            }
            H[I * HV + K] = H[K * HV + I] = 0.5 * (h1 + h2);
        }
        for (int k = 0; k < 3; ++k) {
            const double P = 0.5 * eps * (pt.wcp(i, j, k) + pt.wcp(j, i, k));
            H[I * HV + 6 + k] = H[(6 + k) * HV + I] = -P;
        }
    }
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) H[(6 + k) * HV + 6 + l] = -eps * kd(k, l);
}

FL_HD void left_cauchy_green(const double *F, double *b) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) b[i * 3 + j] = F[i * 3] * F[j * 3] + F[i * 3 + 1] * F[j * 3 + 1] + F[i * 3 + 2] * F[j * 3 + 2];
}

// IsotropicElectroMechanics_108: internal energy
//   W(C, D) = mu1 C:I + mu2 G:I - 2 (mu1 + 2 mu2) ln J + lamb/2 (J - 1)^2 + |F D0|^2 / (2 eps_2 J)
struct Em108 {
    double mu1, mu2, lamb, eps2;
};

struct Em108Point {
    const double *b, *D;
    double J, DD, ie;
    Em108 m;
    // elasticity tensor of the internal energy
    FL_HD double wel(int i, int j, int k, int l) const {
        const double sym = kd(i, k) * kd(j, l) + kd(i, l) * kd(j, k);
        const double dd = kd(i, j) * kd(k, l);
        return 2.0 * m.mu2 / J * (2.0 * b[i * 3 + j] * b[k * 3 + l] - b[i * 3 + k] * b[j * 3 + l] - b[i * 3 + l] * b[j * 3 + k]) +
               (2.0 * (m.mu1 + 2.0 * m.mu2) / J - m.lamb * (J - 1.0)) * sym + m.lamb * (2.0 * J - 1.0) * dd +
               ie * (0.5 * DD * (sym + dd) - kd(i, j) * D[k] * D[l] - D[i] * D[j] * kd(k, l));
    }
    // coupling tensor, (delta_ik D_j + D_i delta_jk - delta_ij D_k) / eps_2
    FL_HD double wcp(int i, int j, int k) const { return ie * (kd(i, k) * D[j] + D[i] * kd(j, k) - kd(i, j) * D[k]); }
};

// Cauchy stress of IsotropicElectroMechanics_108 (and 106) at electric displacement D
FL_HD void em108_stress(const Em108 &m, const double *b, double J, const double *D, double DD, double *sigma) {
    const double trb = b[0] + b[4] + b[8];
    const double ie = 1.0 / m.eps2;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double bb = b[i * 3] * b[j] + b[i * 3 + 1] * b[3 + j] + b[i * 3 + 2] * b[6 + j];
            sigma[i * 3 + j] = 2.0 * m.mu1 / J * b[i * 3 + j] + 2.0 * m.mu2 / J * (trb * b[i * 3 + j] - bb) -
                               2.0 * (m.mu1 + 2.0 * m.mu2) / J * kd(i, j) + m.lamb * (J - 1.0) * kd(i, j) +
                               ie * (D[i] * D[j] - 0.5 * DD * kd(i, j));
        }
}

// D = eps_2 E, Cauchy stress sigma[9] and the enthalpy Hessian; dielectric tensor I / eps_2
FL_HD void material_point(const Em108 &m, const double *F, const double *E, double *D, double *sigma, double *H) {
    const double J = det3(F);
    double b[9];
    left_cauchy_green(F, b);
    for (int k = 0; k < 3; ++k) D[k] = m.eps2 * E[k];
    const double DD = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    em108_stress(m, b, J, D, DD, sigma);
    const Em108Point pt{b, D, J, DD, 1.0 / m.eps2, m};
    enthalpy_hessian(pt, m.eps2, H);
}

// Electric-enthalpy Hessian for a general (symmetric) dielectric tensor W_di, given its inverse
// Winv: enthalpy coupling Q(i,j,k) = sum_n W_cp(i,j,n) Winv(n,k), enthalpy elasticity
// W_el(i,j,k,l) - sum_n Q(i,j,n) W_cp(k,l,n), dielectric block -Winv; symmetric Voigt forms
template <class Pt>
FL_HD void enthalpy_hessian_general(const Pt &pt, const double *Winv, double *H) {
    double Q[27];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                double q = 0.0;
                for (int n = 0; n < 3; ++n) q += pt.wcp(i, j, n) * Winv[n * 3 + k];
                Q[(i * 3 + j) * 3 + k] = q;
            }
    for (int I = 0; I < 6; ++I) {
        const int i = vp0(I), j = vp1(I);
        for (int K = I; K < 6; ++K) {
            const int k = vp0(K), l = vp1(K);
            double h1 = pt.wel(i, j, k, l), h2 = pt.wel(i, j, l, k);
            for (int n = 0; n < 3; ++n) {
                h1 -= Q[(i * 3 + j) * 3 + n] * pt.wcp(k, l, n);
                h2 -= Q[(i * 3 + j) * 3 + n] * pt.wcp(l, k, n);
            }
            H[I * HV + K] = H[K * HV + I] = 0.5 * (h1 + h2);
        }
        for (int k = 0; k < 3; ++k) {
            const double P = 0.5 * (Q[(i * 3 + j) * 3 + k] + Q[(j * 3 + i) * 3 + k]);
            H[I * HV + 6 + k] = H[(6 + k) * HV + I] = -P;
        }
    }
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) H[(6 + k) * HV + 6 + l] = -Winv[k * 3 + l];
}

// IsotropicElectroMechanics_106 (MaterialLibrary/IsotropicElectroMechanics_106.py:41-125,
// LLDispatch/CythonSource/_IsotropicElectroMechanics_106_.h): 108's stress, elasticity and
// coupling with the dielectric tensor J/eps_1 b^-1 + I/eps_2; D = (that tensor)^-1 E
struct Em106 {
    double mu1, mu2, lamb, eps1, eps2;
};

FL_HD void material_point(const Em106 &m, const double *F, const double *E, double *D, double *sigma, double *H) {
    const double J = det3(F);
    double b[9], ib[9], W[9], Winv[9];
    left_cauchy_green(F, b);
    inv3(b, ib);
    for (int k = 0; k < 9; ++k) W[k] = J / m.eps1 * ib[k] + (k % 4 == 0 ? 1.0 / m.eps2 : 0.0);
    inv3(W, Winv);
    for (int k = 0; k < 3; ++k) D[k] = Winv[k * 3] * E[0] + Winv[k * 3 + 1] * E[1] + Winv[k * 3 + 2] * E[2];
    const double DD = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    const Em108 m8{m.mu1, m.mu2, m.lamb, m.eps2};
    em108_stress(m8, b, J, D, DD, sigma);
    const Em108Point pt{b, D, J, DD, 1.0 / m.eps2, m8};
    enthalpy_hessian_general(pt, Winv, H);
}

// IsotropicElectroMechanics_101 (MaterialLibrary/IsotropicElectroMechanics_101.py:38-94,
// LLDispatch/CythonSource/_IsotropicElectroMechanics_101_.h): internal energy
//   W(C, D0) = W_neo-Hookean(C) + |F D0|^2 / (2 eps_1)
struct Em101 {
    double mu, lamb, eps1;
};

struct Em101Point {
    const double *D;
    double J, c;  // c = J / eps_1
    Em101 m;
    FL_HD double wel(int i, int j, int k, int l) const {
        return m.lamb * (2.0 * J - 1.0) * kd(i, j) * kd(k, l) +
               (m.mu / J - m.lamb * (J - 1.0)) * (kd(i, k) * kd(j, l) + kd(i, l) * kd(j, k));
    }
    // J / eps_1 (delta_ik D_j + D_i delta_jk)
    FL_HD double wcp(int i, int j, int k) const { return c * (kd(i, k) * D[j] + D[i] * kd(j, k)); }
};

// D = eps_1 / J E, Cauchy stress and the enthalpy Hessian; dielectric tensor J / eps_1 I
FL_HD void material_point(const Em101 &m, const double *F, const double *E, double *D, double *sigma, double *H) {
    const double J = det3(F);
    double b[9];
    left_cauchy_green(F, b);
    for (int k = 0; k < 3; ++k) D[k] = m.eps1 / J * E[k];
    const double c = J / m.eps1;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            sigma[i * 3 + j] = m.mu / J * (b[i * 3 + j] - kd(i, j)) + m.lamb * (J - 1.0) * kd(i, j) + c * D[i] * D[j];
    const Em101Point pt{D, J, c, m};
    enthalpy_hessian(pt, m.eps1 / J, H);
}

// IsotropicElectroMechanics_105 (MaterialLibrary/IsotropicElectroMechanics_105.py:41-104,
// LLDispatch/CythonSource/_IsotropicElectroMechanics_105_.h): internal energy
//   W_mn(C) + |D0|^2 / (2 eps_1) + |F D0|^2 / (2 eps_2): 108's mechanical elasticity, coupling
//   J/eps_2 (delta_ik D_j + D_i delta_jk), dielectric tensor J/eps_1 b^-1 + J/eps_2 I
struct Em105 {
    double mu1, mu2, lamb, eps1, eps2;
};

struct Em105Point {
    const double *b, *D;
    double J, c;  // c = J / eps_2
    Em105 m;
    FL_HD double wel(int i, int j, int k, int l) const {
        const double sym = kd(i, k) * kd(j, l) + kd(i, l) * kd(j, k);
        return 2.0 * m.mu2 / J * (2.0 * b[i * 3 + j] * b[k * 3 + l] - b[i * 3 + k] * b[j * 3 + l] - b[i * 3 + l] * b[j * 3 + k]) +
               (2.0 * (m.mu1 + 2.0 * m.mu2) / J - m.lamb * (J - 1.0)) * sym + m.lamb * (2.0 * J - 1.0) * kd(i, j) * kd(k, l);
    }
    FL_HD double wcp(int i, int j, int k) const { return c * (kd(i, k) * D[j] + D[i] * kd(j, k)); }
};

FL_HD void material_point(const Em105 &m, const double *F, const double *E, double *D, double *sigma, double *H) {
    const double J = det3(F);
    double b[9], ib[9], W[9], Winv[9];
    left_cauchy_green(F, b);
    inv3(b, ib);
    for (int k = 0; k < 9; ++k) W[k] = J / m.eps1 * ib[k] + (k % 4 == 0 ? J / m.eps2 : 0.0);
    inv3(W, Winv);
    for (int k = 0; k < 3; ++k) D[k] = Winv[k * 3] * E[0] + Winv[k * 3 + 1] * E[1] + Winv[k * 3 + 2] * E[2];
    const double trb = b[0] + b[4] + b[8];
    const double c = J / m.eps2;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double bb = b[i * 3] * b[j] + b[i * 3 + 1] * b[3 + j] + b[i * 3 + 2] * b[6 + j];
            sigma[i * 3 + j] = 2.0 * m.mu1 / J * b[i * 3 + j] + 2.0 * m.mu2 / J * (trb * b[i * 3 + j] - bb) -
                               2.0 * (m.mu1 + 2.0 * m.mu2) / J * kd(i, j) + m.lamb * (J - 1.0) * kd(i, j) +
                               c * D[i] * D[j];
        }
    const Em105Point pt{b, D, J, c, m};
    enthalpy_hessian_general(pt, Winv, H);
}

// IsotropicElectroMechanics_0 (MaterialLibrary/IsotropicElectroMechanics_0.py:43-100,
// LLDispatch/CythonSource/_IsotropicElectroMechanics_0_.h): electric enthalpy
//   W(C, E0) = mu/2 (C:I - 3) - mu ln J + lamb/2 (ln J)^2 - eps_1/2 J C^-1:(E0 x E0),
// its Hessian given in enthalpy form directly (no Legendre transform), D = eps_1 E
struct Em0 {
    double mu, lamb, eps1;
};

struct Em0Point {
    const double *E;
    double J, lnJ, EE;  // EE = E.E
    Em0 m;
    FL_HD double ee(int i, int j) const { return E[i] * E[j]; }
    FL_HD double c(int i, int j, int k, int l) const {
        const double sym = kd(i, k) * kd(j, l) + kd(i, l) * kd(j, k);
        const double dd = kd(i, j) * kd(k, l);
        return m.lamb / J * dd - (m.lamb * lnJ - m.mu) / J * sym +
               m.eps1 * (kd(i, j) * ee(k, l) + ee(i, j) * kd(k, l) - ee(i, k) * kd(j, l) - ee(i, l) * kd(j, k) -
                         kd(i, k) * ee(j, l) - kd(i, l) * ee(j, k)) +
               m.eps1 * EE * 0.5 * (sym - dd);
    }
    // eps_1 (delta_ik E_j + delta_jk E_i - delta_ij E_k)
    FL_HD double p(int i, int j, int k) const { return m.eps1 * (kd(i, k) * E[j] + kd(j, k) * E[i] - kd(i, j) * E[k]); }
};

FL_HD void material_point(const Em0 &m, const double *F, const double *E, double *D, double *sigma, double *H) {
    const double J = det3(F);
    const double lnJ = std::log(J);
    double b[9];
    left_cauchy_green(F, b);
    for (int k = 0; k < 3; ++k) D[k] = m.eps1 * E[k];
    const double EE = E[0] * E[0] + E[1] * E[1] + E[2] * E[2];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            sigma[i * 3 + j] = m.mu / J * (b[i * 3 + j] - kd(i, j)) + m.lamb / J * lnJ * kd(i, j) +
                               m.eps1 * (E[i] * E[j] - 0.5 * EE * kd(i, j));
    const Em0Point pt{E, J, lnJ, EE, m};
    for (int I = 0; I < 6; ++I) {
        const int i = vp0(I), j = vp1(I);
        for (int K = I; K < 6; ++K) {
            const int k = vp0(K), l = vp1(K);
            H[I * HV + K] = H[K * HV + I] = 0.5 * (pt.c(i, j, k, l) + pt.c(i, j, l, k));
        }
        for (int k = 0; k < 3; ++k) {
            const double P = 0.5 * (pt.p(i, j, k) + pt.p(j, i, k));
            H[I * HV + 6 + k] = H[(6 + k) * HV + I] = -P;
        }
    }
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) H[(6 + k) * HV + 6 + l] = -m.eps1 * kd(k, l);
}

// SteinmannModel (MaterialLibrary/SteinmannModel.py:40-120, LLDispatch/CythonSource/_SteinmannModel_.h):
// electric enthalpy W_n(C) + c1 I:(E0 x E0) + c2 C:(E0 x E0) - eps_1/2 J C^-1:(E0 x E0); material
// 0's Hessian with 2 c2/J (b_ik (bE)_j + (bE)_i b_jk) added to the coupling, dielectric block
// -eps_1 I + 2 c1/J b + 2 c2/J b^2, D = eps_1 E - 2 c1/J bE - 2 c2/J b^2 E
struct EmSteinmann {
    double mu, lamb, c1, c2, eps1;
};

FL_HD void material_point(const EmSteinmann &m, const double *F, const double *E, double *D, double *sigma,
                          double *H) {
    const double J = det3(F);
    double b[9], bb[9], be[3], bbe[3];
    left_cauchy_green(F, b);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) bb[i * 3 + j] = b[i * 3] * b[j] + b[i * 3 + 1] * b[3 + j] + b[i * 3 + 2] * b[6 + j];
    for (int i = 0; i < 3; ++i) {
        be[i] = b[i * 3] * E[0] + b[i * 3 + 1] * E[1] + b[i * 3 + 2] * E[2];
        bbe[i] = bb[i * 3] * E[0] + bb[i * 3 + 1] * E[1] + bb[i * 3 + 2] * E[2];
    }
    const Em0 m0{m.mu, m.lamb, m.eps1};
    material_point(m0, F, E, D, sigma, H);
    const double g = 2.0 * m.c2 / J;
    for (int k = 0; k < 3; ++k) D[k] = m.eps1 * E[k] - 2.0 * m.c1 / J * be[k] - g * bbe[k];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sigma[i * 3 + j] += g * be[i] * be[j];
    for (int I = 0; I < 6; ++I) {
        const int i = vp0(I), j = vp1(I);
        for (int k = 0; k < 3; ++k) {
            // coupling of material 0 plus g (b_ik be_j + be_i b_jk), symmetrised over i, j
            const double pij = m.eps1 * (kd(i, k) * E[j] + kd(j, k) * E[i] - kd(i, j) * E[k]) +
                               g * (b[i * 3 + k] * be[j] + be[i] * b[j * 3 + k]);
            const double pji = m.eps1 * (kd(j, k) * E[i] + kd(i, k) * E[j] - kd(j, i) * E[k]) +
                               g * (b[j * 3 + k] * be[i] + be[j] * b[i * 3 + k]);
            H[I * HV + 6 + k] = H[(6 + k) * HV + I] = -0.5 * (pij + pji);
        }
    }
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
            H[(6 + k) * HV + 6 + l] = -m.eps1 * kd(k, l) + 2.0 * m.c1 / J * b[k * 3 + l] + g * bb[k * 3 + l];
}

// Piezoelectric_100 (MaterialLibrary/Piezoelectric_100.py:43-170, LLDispatch/CythonSource/
// _Piezoelectric_100_.h): transversely isotropic internal energy with fibre direction N (one per
// element); with s = sqrt(mu3 / eps_3), H = J F^-T: dielectric tensor
// J/eps_1 b^-1 + (1/eps_2 + 2 J s) I, D = (that tensor)^-1 (E - 2 s F N + 2 s / J H N)
struct EmPiezo100 {
    double mu1, mu2, mu3, lamb, eps1, eps2, eps3;
};

struct EmPiezo100Point {
    const double *b, *D, *FN, *HN;
    double J, DD, hh, s;
    EmPiezo100 m;
    FL_HD double wel(int i, int j, int k, int l) const {
        const double sym = kd(i, k) * kd(j, l) + kd(i, l) * kd(j, k);
        const double dd = kd(i, j) * kd(k, l);
        const double c = 2.0 * m.mu3 / J;
        return 2.0 * m.mu2 / J * (2.0 * b[i * 3 + j] * b[k * 3 + l] - b[i * 3 + k] * b[j * 3 + l] - b[i * 3 + l] * b[j * 3 + k]) +
               (2.0 * (m.mu1 + 2.0 * m.mu2) / J - m.lamb * (J - 1.0)) * sym + m.lamb * (2.0 * J - 1.0) * dd +
               (0.5 * DD * (sym + dd) - kd(i, j) * D[k] * D[l] - D[i] * D[j] * kd(k, l)) / m.eps2 + c * sym -
               2.0 * c * (kd(i, j) * HN[k] * HN[l] + HN[i] * HN[j] * kd(k, l)) + c * hh * (2.0 * dd - sym) +
               c * (kd(i, l) * HN[j] * HN[k] + kd(j, l) * HN[i] * HN[k] + kd(i, k) * HN[j] * HN[l] + kd(j, k) * HN[i] * HN[l]);
    }
    FL_HD double wcp(int i, int j, int k) const {
        return (kd(i, k) * D[j] + D[i] * kd(j, k) - kd(i, j) * D[k]) / m.eps2 +
               2.0 * J * s * (kd(i, k) * D[j] + D[i] * kd(j, k)) + 2.0 * s * (kd(i, k) * FN[j] + FN[i] * kd(j, k));
    }
};

FL_HD void material_point_n(const EmPiezo100 &m, const double *F, const double *E, const double *N, double *D,
                            double *sigma, double *H) {
    const double J = det3(F);
    double b[9], ib[9], iF[9], W[9], Winv[9], FN[3], HN[3], r[3];
    left_cauchy_green(F, b);
    inv3(b, ib);
    inv3(F, iF);
    const double s = std::sqrt(m.mu3 / m.eps3);
    for (int i = 0; i < 3; ++i) {
        FN[i] = F[i * 3] * N[0] + F[i * 3 + 1] * N[1] + F[i * 3 + 2] * N[2];
        HN[i] = J * (iF[i] * N[0] + iF[3 + i] * N[1] + iF[6 + i] * N[2]);  // (J F^-T N)_i
    }
    for (int k = 0; k < 9; ++k) W[k] = J / m.eps1 * ib[k] + (k % 4 == 0 ? 1.0 / m.eps2 + 2.0 * J * s : 0.0);
    inv3(W, Winv);
    for (int i = 0; i < 3; ++i) r[i] = E[i] - 2.0 * s * FN[i] + 2.0 / J * s * HN[i];
    for (int k = 0; k < 3; ++k) D[k] = Winv[k * 3] * r[0] + Winv[k * 3 + 1] * r[1] + Winv[k * 3 + 2] * r[2];
    const double DD = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    const double hh = HN[0] * HN[0] + HN[1] * HN[1] + HN[2] * HN[2];
    const double trb = b[0] + b[4] + b[8];
    const double c = 2.0 * m.mu3 / J;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double bb = b[i * 3] * b[j] + b[i * 3 + 1] * b[3 + j] + b[i * 3 + 2] * b[6 + j];
            sigma[i * 3 + j] = 2.0 * m.mu1 / J * b[i * 3 + j] + 2.0 * m.mu2 / J * (trb * b[i * 3 + j] - bb) -
                               2.0 * (m.mu1 + 2.0 * m.mu2 + m.mu3) / J * kd(i, j) + m.lamb * (J - 1.0) * kd(i, j) +
                               c * (FN[i] * FN[j] + hh * kd(i, j) - HN[i] * HN[j]) +
                               (D[i] * D[j] - 0.5 * DD * kd(i, j)) / m.eps2 + 2.0 * J * s * D[i] * D[j] +
                               2.0 * s * (D[i] * FN[j] + FN[i] * D[j]);
        }
    const EmPiezo100Point pt{b, D, FN, HN, J, DD, hh, s, m};
    enthalpy_hessian_general(pt, Winv, H);
}

// materials without a fibre direction ignore N
template <class MAT>
FL_HD void material_point_n(const MAT &m, const double *F, const double *E, const double *, double *D, double *sigma,
                            double *H) {
    material_point(m, F, E, D, sigma, H);
}

// Gauss point g of one element: spatial gradients SG[d * npe + a] (material gradients when the
// geometry is not updated), the weight dv = w |det dX/dxi| (|J| too with the update), the spatial
// electric field E = -grad phi, and the material's D, sigma and H. X, x [npe * 3], phi [npe];
// Jm [3 * npe * nq] (d-major, then node, then point); N the element's fibre direction (transversely
// isotropic materials; ignored by the others). Returns det F.
template <class MAT>
FL_HD double gauss_point(int npe, int nq, int g, const double *Jm, double w, const double *X, const double *x,
                         const double *phi, int update, const MAT &m, const double *N, double *SG, double *dv,
                         double *D, double *sigma, double *H) {
    double GX[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, iGX[9];
    for (int a = 0; a < npe; ++a)
        for (int d = 0; d < 3; ++d) {
            const double j = Jm[(d * npe + a) * nq + g];
            for (int k = 0; k < 3; ++k) GX[d * 3 + k] += j * X[a * 3 + k];
        }
    const double detX = inv3(GX, iGX);
    double F[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < npe; ++a) {
        double mg[3];
        for (int J = 0; J < 3; ++J)
            mg[J] = iGX[J * 3] * Jm[a * nq + g] + iGX[J * 3 + 1] * Jm[(npe + a) * nq + g] +
                    iGX[J * 3 + 2] * Jm[(2 * npe + a) * nq + g];
        for (int i = 0; i < 3; ++i)
            for (int J = 0; J < 3; ++J) F[i * 3 + J] += x[a * 3 + i] * mg[J];
        if (!update)
            for (int d = 0; d < 3; ++d) SG[d * npe + a] = mg[d];
    }
    const double detF = det3(F);
    if (update) {
        double Gx[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, iGx[9];
        for (int a = 0; a < npe; ++a)
            for (int d = 0; d < 3; ++d) {
                const double j = Jm[(d * npe + a) * nq + g];
                for (int k = 0; k < 3; ++k) Gx[d * 3 + k] += j * x[a * 3 + k];
            }
        inv3(Gx, iGx);
        for (int a = 0; a < npe; ++a)
            for (int l = 0; l < 3; ++l)
                SG[l * npe + a] = iGx[l * 3] * Jm[a * nq + g] + iGx[l * 3 + 1] * Jm[(npe + a) * nq + g] +
                                  iGx[l * 3 + 2] * Jm[(2 * npe + a) * nq + g];
        *dv = w * std::fabs(detX) * std::fabs(detF);
    } else {
        *dv = w * std::fabs(detX);
    }
    double E[3] = {0, 0, 0};
    for (int a = 0; a < npe; ++a)
        for (int k = 0; k < 3; ++k) E[k] -= SG[k * npe + a] * phi[a];
    material_point_n(m, F, E, N, D, sigma, H);
    return detF;
}

// nonzero columns and values of the B row of field v (0-2 displacement, 3 potential) of a node
// with spatial gradient (gx, gy, gz)
FL_HD void brow(int v, double gx, double gy, double gz, int *c, double *s) {
    if (v == 0) {
        c[0] = 0; c[1] = 3; c[2] = 4;
        s[0] = gx; s[1] = gy; s[2] = gz;
    } else if (v == 1) {
        c[0] = 1; c[1] = 3; c[2] = 5;
        s[0] = gy; s[1] = gx; s[2] = gz;
    } else if (v == 2) {
        c[0] = 2; c[1] = 4; c[2] = 5;
        s[0] = gz; s[1] = gx; s[2] = gy;
    } else {
        c[0] = 6; c[1] = 7; c[2] = 8;
        s[0] = gx; s[1] = gy; s[2] = gz;
    }
}

// one Gauss point's contribution (without dv) to the tangent entry of (node a, field v) x
// (node b, field u): B H B^T plus the geometric term grad N_a . sigma . grad N_b on equal
// displacement fields
FL_HD double entry(int a, int v, int b, int u, int npe, const double *SG, const double *H, const double *sigma) {
    const double ga[3] = {SG[a], SG[npe + a], SG[2 * npe + a]};
    const double gb[3] = {SG[b], SG[npe + b], SG[2 * npe + b]};
    int ca[3], cb[3];
    double sa[3], sb[3];
    brow(v, ga[0], ga[1], ga[2], ca, sa);
    brow(u, gb[0], gb[1], gb[2], cb, sb);
    double r = 0.0;
    for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) r += sa[p] * H[ca[p] * HV + cb[q]] * sb[q];
    if (v == u && v < 3)
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) r += ga[k] * sigma[k * 3 + l] * gb[l];
    return r;
}

// one Gauss point's contribution (without dv) to the 4 x 4 block of node pair (a, b), added to
// K[v][u]: the same B H B^T plus geometric term as entry(), grouped as sum_p sa[p] W_u[ca[p]] with
// W_u[c] = sum_q H[c][cb[q]] sb[q] formed once for the block's four columns (~10 FP64 operations
// per entry instead of ~25)
FL_HD void pair_block(int a, int b, int npe, const double *SG, const double *H, const double *sigma, double w,
                      double K[NV][NV]) {
    const double ga[3] = {SG[a], SG[npe + a], SG[2 * npe + a]};
    const double gb[3] = {SG[b], SG[npe + b], SG[2 * npe + b]};
    double W[NV][HV];
    for (int u = 0; u < NV; ++u) {
        int cb[3];
        double sb[3];
        brow(u, gb[0], gb[1], gb[2], cb, sb);
        for (int c = 0; c < HV; ++c) W[u][c] = H[c * HV + cb[0]] * sb[0] + H[c * HV + cb[1]] * sb[1] + H[c * HV + cb[2]] * sb[2];
    }
    for (int v = 0; v < NV; ++v) {
        int ca[3];
        double sa[3];
        brow(v, ga[0], ga[1], ga[2], ca, sa);
        for (int u = 0; u < NV; ++u) K[v][u] += w * (sa[0] * W[u][ca[0]] + sa[1] * W[u][ca[1]] + sa[2] * W[u][ca[2]]);
    }
    double geo = 0.0;
    for (int k = 0; k < 3; ++k) geo += ga[k] * (sigma[k * 3] * gb[0] + sigma[k * 3 + 1] * gb[1] + sigma[k * 3 + 2] * gb[2]);
    for (int v = 0; v < 3; ++v) K[v][v] += w * geo;
}

// one Gauss point's contribution (without dv) to the residual of (node a, field v): the B row
// against (sigma_xx, sigma_yy, sigma_zz, sigma_xy, sigma_xz, sigma_yz, D)
FL_HD double residual(int a, int v, int npe, const double *SG, const double *D, const double *sigma) {
    const double tt[9] = {sigma[0], sigma[4], sigma[8], sigma[1], sigma[2], sigma[5], D[0], D[1], D[2]};
    int c[3];
    double s[3];
    brow(v, SG[a], SG[npe + a], SG[2 * npe + a], c, s);
    return s[0] * tt[c[0]] + s[1] * tt[c[1]] + s[2] * tt[c[2]];
}

}  // namespace dpf
}  // namespace fl
