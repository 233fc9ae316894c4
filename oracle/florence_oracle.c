/*
 * florence_oracle.c -- CPU restatement of Florence's low-level displacement-formulation
 * assembly. TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU-baseline
 * leg of the benchmark call it as the checker. The product (florence_gb300) never links or
 * calls it.
 *
 * Parity pinning: every function here is checked against golden vectors produced by the
 * reference's own numpy assembly path and its compiled ComputeSparsityPattern
 * (tests/golden/make_golden.py); see tests/test_oracle.py.
 *
 * The reference's C++ (Fastor + CBLAS + <immintrin.h>) cannot be compiled here, so this file
 * restates its algorithm in plain C, following the loop structure of:
 *   - _GlobalAssemblyDF_                Florence/FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDF_.h:8-176
 *   - KinematicMeasures_<3>             Florence/FiniteElements/LocalAssembly/_KinematicMeasures_/_KinematicMeasures_.h:64-119
 *   - _NeoHookean_::_KineticMeasures_   Florence/MaterialLibrary/LLDispatch/CythonSource/_NeoHookean_.h:26-51
 *   - _MooneyRivlin_::_KineticMeasures_ Florence/MaterialLibrary/LLDispatch/CythonSource/_MooneyRivlin_.h:26-69
 *   - _ConstitutiveStiffnessIntegrandDF_Filler_ / FillConstitutiveB_ / GetTotalTraction_
 *                                       Florence/VariationalPrinciple/_ConstitutiveStiffness_/_ConstitutiveStiffnessDF_.h:15-156
 *   - _GeometricStiffnessFiller_        Florence/VariationalPrinciple/_GeometricStiffness_/_GeometricStiffness_.h:61-99
 *   - fill_triplet / fill_global_data   Florence/VariationalPrinciple/_Mass_/_MassIntegrand_.h:68-168
 *   - SparseAssemblyNativeCSR_[RecomputeDataIndex_]
 *                                       Florence/FiniteElements/Assembly/_Assembly_/SparseAssemblyNative.h:32-111
 *   - ComputeSparsityPattern            Florence/FiniteElements/Assembly/_Assembly_/ComputeSparsityPattern.pyx:44-112,
 *                                       ComputeSparsityPattern.h:22-125
 *   - _GlobalAssemblyExplicit_DF_DPF_<3> Florence/FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyExplicit_DF_DPF_.h:459-720
 *   - _GenericConstantMassIntegrand_ (lumped)
 *                                       Florence/VariationalPrinciple/_Mass_/_MassIntegrand_.h:249-400
 *
 * Element loops may run on several OpenMP threads (the CPU baseline); shared outputs are then
 * accumulated with atomic adds, so with more than one thread only the summation order differs.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_NEOHOOKEAN 1
#define ORC_MOONEYRIVLIN 2
#define ORC_NEARLYINCOMPRESSIBLEMOONEYRIVLIN 3
#define ORC_LINEARELASTIC 10
#define ORC_ANISOTROPICMOONEYRIVLIN_1 11

/* Fibre direction N per element [nelem][3] for the transversely isotropic material (the
 * reference's anisotropic_orientations, read as &anisotropic_orientations[elem*ndim],
 * AOT_Assembler.py:72-75); set before an assembly call, NULL otherwise. */
static const double *g_orient = NULL;
void orc_set_orientations(const double *orient) { g_orient = orient; }

/* Voigt pairs in the reference's order xx,yy,zz,xy,xz,yz (_ConstitutiveStiffnessDF_.h:17-22). */
static const int VI[6] = {0, 1, 2, 0, 0, 1};
static const int VJ[6] = {0, 1, 2, 1, 2, 2};

static double inv3(const double *m, double *r) {
    /* adjugate / determinant of a row-major 3x3 */
    r[0] = m[4] * m[8] - m[5] * m[7];
    r[1] = m[2] * m[7] - m[1] * m[8];
    r[2] = m[1] * m[5] - m[2] * m[4];
    r[3] = m[5] * m[6] - m[3] * m[8];
    r[4] = m[0] * m[8] - m[2] * m[6];
    r[5] = m[2] * m[3] - m[0] * m[5];
    r[6] = m[3] * m[7] - m[4] * m[6];
    r[7] = m[1] * m[6] - m[0] * m[7];
    r[8] = m[0] * m[4] - m[1] * m[3];
    double det = m[0] * r[0] + m[1] * r[3] + m[2] * r[6];
    double s = 1.0 / det;
    for (int i = 0; i < 9; ++i) r[i] *= s;
    return det;
}

static double det3(const double *m) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

/* Kinematics at one Gauss point (KinematicMeasures_<3>): sp[a*3+d] = spatial gradient of N_a,
 * F row-major, returns detJ = w*|det(dx/dxi)| (update) or w*|det(dX/dxi)|. */
static double kinematics_qp(const double *Jm, const double *w, const double *X, const double *x, int npe, int nq,
                            int g, int update, double *sp, double *F) {
    double PX[9] = {0}, Px[9] = {0}, iPX[9], iPx[9];
    for (int d = 0; d < 3; ++d)
        for (int a = 0; a < npe; ++a) {
            double j = Jm[(size_t)d * npe * nq + (size_t)a * nq + g];
            for (int k = 0; k < 3; ++k) {
                PX[d * 3 + k] += j * X[a * 3 + k];
                Px[d * 3 + k] += j * x[a * 3 + k];
            }
        }
    double detX = inv3(PX, iPX);
    double detx = inv3(Px, iPx);
    double detJ = update ? w[g] * fabs(detx) : w[g] * fabs(detX);
    double cF[9] = {0};
    for (int a = 0; a < npe; ++a) {
        double mg[3], s[3];
        for (int d = 0; d < 3; ++d) {
            mg[d] = 0.0;
            s[d] = 0.0;
            for (int e = 0; e < 3; ++e) {
                double j = Jm[(size_t)e * npe * nq + (size_t)a * nq + g];
                mg[d] += iPX[d * 3 + e] * j;
                s[d] += iPx[d * 3 + e] * j;
            }
            sp[a * 3 + d] = s[d];
        }
        /* current_F[d][k] = sum_a MaterialGradient[d][a] x[a][k]; F = transpose(current_F) */
        for (int d = 0; d < 3; ++d)
            for (int k = 0; k < 3; ++k) cF[d * 3 + k] += mg[d] * x[a * 3 + k];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) F[i * 3 + j] = cF[j * 3 + i];
    return detJ;
}

/* Cauchy stress (row-major 3x3) and the Voigt elasticity H (6x6) of the material at F (N: the
 * element's fibre direction, transversely isotropic material only). */
static void material_qp(int mat, const double *prm, const double *F, const double *N, double *sig, double *H) {
    double J = det3(F);
    double b[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += F[i * 3 + k] * F[j * 3 + k];
            b[i * 3 + j] = s;
        }
    double c1, c2, cbb = 0.0; /* c = c1 (d_ik d_jl + d_il d_jk) + c2 d_ij d_kl + cbb (2 b_ij b_kl - b_ik b_jl - b_il b_jk) */
    /* nearly incompressible Mooney-Rivlin (_NearlyIncompressibleMooneyRivlin_.h:26-90, parameters
     * alpha, beta, kappa): c += kbI (b_ij d_kl + d_ij b_kl) + kgI (g_ij d_kl + d_ij g_kl)
     * + kg4 (g_ik d_jl + g_il d_jk + d_ik g_jl + d_il g_jk) + kgg g_ij g_kl, g = cof(F) cof(F)^T */
    double kbI = 0.0, kgI = 0.0, kg4 = 0.0, kgg = 0.0, g[9] = {0};
    if (mat == ORC_LINEARELASTIC) { /* _LinearElastic_.h:26-60: stress from the small strain */
        double mu = prm[0], lamb = prm[1];
        double tre = F[0] + F[4] + F[8] - 3.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                sig[i * 3 + j] = mu * (F[i * 3 + j] + F[j * 3 + i] - 2.0 * (i == j)) + (i == j ? lamb * tre : 0.0);
        c1 = mu;
        c2 = lamb;
    } else if (mat == ORC_NEARLYINCOMPRESSIBLEMOONEYRIVLIN) {
        double alpha = prm[0], beta = prm[1], kappa = prm[2];
        double iF[9];
        inv3(F, iF);
        double H[9]; /* cofactor J F^-T */
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) H[i * 3 + j] = J * iF[j * 3 + i];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += H[i * 3 + k] * H[j * 3 + k];
                g[i * 3 + j] = s;
            }
        double trb = b[0] + b[4] + b[8], trg = g[0] + g[4] + g[8];
        double A = 2.0 * alpha * pow(J, -5.0 / 3.0);
        double B3 = beta / (J * J * J) * trg * sqrt(trg), B1 = 3.0 * beta / (J * J * J) * sqrt(trg);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double d = (i == j) ? 1.0 : 0.0;
                sig[i * 3 + j] = A * b[i * 3 + j] - A / 3.0 * trb * d + B3 * d - B1 * g[i * 3 + j] + kappa * (J - 1.0) * d;
            }
        kbI = -2.0 / 3.0 * A;
        c2 = 2.0 / 9.0 * A * trb + B3 + kappa * (2.0 * J - 1.0);
        c1 = A / 3.0 * trb - B3 - kappa * (J - 1.0);
        kgI = -B1;
        kg4 = B1;
        kgg = B1 / trg;
    } else if (mat == ORC_ANISOTROPICMOONEYRIVLIN_1) {
        /* _AnisotropicMooneyRivlin_1_.h:31-88 (parameters mu1, mu2, lamb, mu3), with HN = cof(F) N:
         * sigma = 2mu1/J b + 2mu2/J (tr b b - b b) - 2(mu1+2mu2+mu3)/J I + lamb (J-1) I
         *       + 2mu3/J (FN FN^T + |HN|^2 I - HN HN^T);
         * elasticity: the Mooney-Rivlin terms with mu1+2mu2+mu3, and with m = HN HN^T
         * -4mu3/J (I m + m I) + 2mu3/J |HN|^2 (2 II - I_ik I_jl - I_il I_jk)
         * + 2mu3/J (I_ik m_jl + I_il m_jk + m_ik I_jl + m_il I_jk) */
        static const double N0[3] = {0.0, 0.0, 0.0};
        double mu1 = prm[0], mu2 = prm[1], lamb = prm[2], mu3 = prm[3];
        double iF[9], Hc[9], FN[3], HN[3];
        if (!N) N = N0; /* no fibre directions given */
        inv3(F, iF);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Hc[i * 3 + j] = J * iF[j * 3 + i];
        for (int i = 0; i < 3; ++i) {
            FN[i] = F[i * 3] * N[0] + F[i * 3 + 1] * N[1] + F[i * 3 + 2] * N[2];
            HN[i] = Hc[i * 3] * N[0] + Hc[i * 3 + 1] * N[1] + Hc[i * 3 + 2] * N[2];
        }
        double inHN = HN[0] * HN[0] + HN[1] * HN[1] + HN[2] * HN[2];
        double trb = b[0] + b[4] + b[8];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double bb = 0.0;
                for (int k = 0; k < 3; ++k) bb += b[i * 3 + k] * b[k * 3 + j];
                double d = (i == j) ? 1.0 : 0.0;
                g[i * 3 + j] = HN[i] * HN[j];
                sig[i * 3 + j] = 2.0 * mu1 / J * b[i * 3 + j] + 2.0 * mu2 / J * (trb * b[i * 3 + j] - bb) -
                                 2.0 * (mu1 + 2.0 * mu2 + mu3) / J * d + lamb * (J - 1.0) * d +
                                 2.0 * mu3 / J * (FN[i] * FN[j] + inHN * d - HN[i] * HN[j]);
            }
        c1 = 2.0 * (mu1 + 2.0 * mu2 + mu3) / J - lamb * (J - 1.0) - 2.0 * mu3 / J * inHN;
        c2 = lamb * (2.0 * J - 1.0) + 4.0 * mu3 / J * inHN;
        cbb = 2.0 * mu2 / J;
        kgI = -4.0 * mu3 / J;
        kg4 = 2.0 * mu3 / J;
    } else if (mat == ORC_NEOHOOKEAN) {
        double mu = prm[0], lamb = prm[1];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                sig[i * 3 + j] = mu / J * (b[i * 3 + j] - (i == j)) + (i == j ? lamb * (J - 1.0) : 0.0);
        c1 = mu / J - lamb * (J - 1.0);
        c2 = lamb * (2.0 * J - 1.0);
    } else {
        double mu1 = prm[0], mu2 = prm[1], lamb = prm[2];
        double trb = b[0] + b[4] + b[8];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double bb = 0.0;
                for (int k = 0; k < 3; ++k) bb += b[i * 3 + k] * b[k * 3 + j];
                double d = (i == j) ? 1.0 : 0.0;
                sig[i * 3 + j] = 2.0 * mu1 / J * b[i * 3 + j] + 2.0 * mu2 / J * (trb * b[i * 3 + j] - bb) -
                                 2.0 * (mu1 + 2.0 * mu2) / J * d + lamb * (J - 1.0) * d;
            }
        c1 = 2.0 * (mu1 + 2.0 * mu2) / J - lamb * (J - 1.0);
        c2 = lamb * (2.0 * J - 1.0);
        cbb = 2.0 * mu2 / J;
    }
    for (int I = 0; I < 6; ++I)
        for (int K = 0; K < 6; ++K) {
            int i = VI[I], j = VJ[I], k = VI[K], l = VJ[K];
            double v = c1 * ((i == k) * (j == l) + (i == l) * (j == k)) + c2 * (i == j) * (k == l);
            if (cbb != 0.0) v += cbb * (2.0 * b[i * 3 + j] * b[k * 3 + l] - b[i * 3 + k] * b[j * 3 + l] - b[i * 3 + l] * b[j * 3 + k]);
            if (mat == ORC_NEARLYINCOMPRESSIBLEMOONEYRIVLIN || mat == ORC_ANISOTROPICMOONEYRIVLIN_1) {
                double dij = (i == j), dkl = (k == l), dik = (i == k), djl = (j == l), dil = (i == l), djk = (j == k);
                v += kbI * (b[i * 3 + j] * dkl + dij * b[k * 3 + l]) + kgI * (g[i * 3 + j] * dkl + dij * g[k * 3 + l]) +
                     kg4 * (g[i * 3 + k] * djl + g[i * 3 + l] * djk + dik * g[j * 3 + l] + dil * g[j * 3 + k]) +
                     kgg * g[i * 3 + j] * g[k * 3 + l];
            }
            H[I * 6 + K] = v;
        }
}

/* Element tangent K_e (row-major ndof x ndof, dofs interleaved a*3+i) and residual t_e.
 * Dense B*H*B^T per Gauss point plus geometric stiffness, as in the reference. Work arrays:
 * B[ndof*6], HBT[6*ndof]. */
static void element_df(int mat, const double *prm, const double *N, const double *Jm, const double *w, const double *X,
                       const double *x, int npe, int nq, int update, double *Ke, double *te, double *sp, double *B,
                       double *HBT) {
    int ndof = 3 * npe;
    memset(Ke, 0, sizeof(double) * ndof * ndof);
    memset(te, 0, sizeof(double) * ndof);
    memset(B, 0, sizeof(double) * ndof * 6);
    for (int g = 0; g < nq; ++g) {
        double F[9], sig[9], H[36];
        double detJ = kinematics_qp(Jm, w, X, x, npe, nq, g, update, sp, F);
        material_qp(mat, prm, F, N, sig, H);
        /* FillConstitutiveB_: rows (a,x),(a,y),(a,z) */
        for (int a = 0; a < npe; ++a) {
            double a0 = sp[a * 3], a1 = sp[a * 3 + 1], a2 = sp[a * 3 + 2];
            double *r = B + (size_t)a * 18;
            r[0] = a0; r[3] = a1; r[4] = a2;
            r[7] = a1; r[9] = a0; r[11] = a2;
            r[14] = a2; r[16] = a0; r[17] = a1;
        }
        /* HBT = H * B^T  (6 x ndof) */
        for (int I = 0; I < 6; ++I)
            for (int c = 0; c < ndof; ++c) {
                double s = 0.0;
                for (int K = 0; K < 6; ++K) s += H[I * 6 + K] * B[c * 6 + K];
                HBT[I * ndof + c] = s;
            }
        /* K += detJ * B * HBT */
        for (int r = 0; r < ndof; ++r) {
            const double *br = B + r * 6;
            double *kr = Ke + (size_t)r * ndof;
            for (int c = 0; c < ndof; ++c) {
                double s = 0.0;
                for (int K = 0; K < 6; ++K) s += br[K] * HBT[K * ndof + c];
                kr[c] += s * detJ;
            }
        }
        if (update) {
            double tv[6] = {sig[0], sig[4], sig[8], sig[1], sig[2], sig[5]};
            for (int r = 0; r < ndof; ++r) {
                double s = 0.0;
                for (int K = 0; K < 6; ++K) s += B[r * 6 + K] * tv[K];
                te[r] += s * detJ;
            }
        }
        /* geometric stiffness (ABI==1 branch); the reference builds the linear elastic assembler
         * without it (AOT_Assembler.py:74-81) */
        if (mat != ORC_LINEARELASTIC)
        for (int a = 0; a < npe; ++a) {
            double a0 = sp[a * 3], a1 = sp[a * 3 + 1], a2 = sp[a * 3 + 2];
            for (int b = 0; b < npe; ++b) {
                double b0 = sp[b * 3], b1 = sp[b * 3 + 1], b2 = sp[b * 3 + 2];
                double dum = a0 * (sig[0] * b0 + sig[1] * b1 + sig[2] * b2) + a1 * (sig[1] * b0 + sig[4] * b1 + sig[5] * b2) +
                             a2 * (sig[2] * b0 + sig[5] * b1 + sig[8] * b2);
                dum *= detJ;
                for (int c = 0; c < 3; ++c) Ke[(size_t)(a * 3 + c) * ndof + b * 3 + c] += dum;
            }
        }
    }
}

static void gather(const double *src, const int64_t *el, int npe, double *dst) {
    for (int a = 0; a < npe; ++a)
        for (int k = 0; k < 3; ++k) dst[a * 3 + k] = src[el[a] * 3 + k];
}

static inline void atomic_add(double *p, double v, int nthreads) {
    if (nthreads > 1) {
#pragma omp atomic
        *p += v;
    } else {
        *p += v;
    }
}

/* binary search for val in a sorted row; returns its offset (binary_locate in the reference) */
static int64_t locate(const int32_t *row, int64_t n, int32_t val) {
    int64_t lo = 0, hi = n;
    while (hi - lo > 1) {
        int64_t mid = lo + (hi - lo) / 2;
        if (val < row[mid]) hi = mid; else lo = mid;
    }
    return lo;
}

/* Element tangents for a list of elements (parity of element matrices). Ke_out[n][ndof][ndof]. */
void orc_element_matrices(int mat, const double *prm, const double *points, const int64_t *elements,
                          const double *Eulerx, const double *Jm, const double *w, int64_t npe, int64_t nq,
                          int update, const int64_t *elem_ids, int64_t nids, double *Ke_out, double *te_out) {
    int ndof = 3 * (int)npe;
    double *X = malloc(sizeof(double) * npe * 3), *x = malloc(sizeof(double) * npe * 3);
    double *sp = malloc(sizeof(double) * npe * 3), *B = malloc(sizeof(double) * ndof * 6);
    double *HBT = malloc(sizeof(double) * ndof * 6);
    for (int64_t n = 0; n < nids; ++n) {
        const int64_t *el = elements + elem_ids[n] * npe;
        gather(points, el, (int)npe, X);
        gather(Eulerx, el, (int)npe, x);
        element_df(mat, prm, g_orient ? g_orient + elem_ids[n] * 3 : NULL, Jm, w, X, x, (int)npe, (int)nq, update,
                   Ke_out + n * ndof * ndof, te_out + n * ndof, sp, B, HBT);
    }
    free(X); free(x); free(sp); free(B); free(HBT);
}

/* _GlobalAssemblyDF_: mode 0 = triplets (I,J,V sized nelem*ndof^2), 1 = CSR through the data
 * index maps, 2 = CSR by binary search in each row (squeeze). T is accumulated (+=). */
int orc_assemble_df(int mat, const double *prm, const double *points, const int64_t *elements, const double *Eulerx,
                    const double *Jm, const double *w, int64_t nelem, int64_t npe, int64_t nq, int update, int mode,
                    int32_t *I, int32_t *J, double *V, double *T, const int32_t *indptr, const int32_t *indices,
                    const int32_t *data_local, const int32_t *data_global, int nthreads) {
    int ndof = 3 * (int)npe;
    int64_t cap = (int64_t)ndof * ndof;
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        double *X = malloc(sizeof(double) * npe * 3), *x = malloc(sizeof(double) * npe * 3);
        double *sp = malloc(sizeof(double) * npe * 3), *B = malloc(sizeof(double) * ndof * 6);
        double *HBT = malloc(sizeof(double) * ndof * 6);
        double *Ke = malloc(sizeof(double) * cap), *te = malloc(sizeof(double) * ndof);
        int64_t *dofs = malloc(sizeof(int64_t) * ndof);
#pragma omp for schedule(static)
        for (int64_t e = 0; e < nelem; ++e) {
            const int64_t *el = elements + e * npe;
            gather(points, el, (int)npe, X);
            gather(Eulerx, el, (int)npe, x);
            element_df(mat, prm, g_orient ? g_orient + e * 3 : NULL, Jm, w, X, x, (int)npe, (int)nq, update, Ke, te, sp,
                       B, HBT);
            for (int a = 0; a < npe; ++a)
                for (int c = 0; c < 3; ++c) dofs[a * 3 + c] = el[a] * 3 + c;
            if (mode == 0) {
                for (int r = 0; r < ndof; ++r)
                    for (int c = 0; c < ndof; ++c) {
                        int64_t k = e * cap + (int64_t)r * ndof + c;
                        I[k] = (int32_t)dofs[r];
                        J[k] = (int32_t)dofs[c];
                        V[k] = Ke[(int64_t)r * ndof + c];
                    }
            } else if (mode == 1) {
                for (int64_t k = 0; k < cap; ++k)
                    atomic_add(&V[data_global[e * cap + k]], Ke[data_local[e * cap + k]], nthreads);
            } else {
                for (int r = 0; r < ndof; ++r) {
                    int64_t row = dofs[r], start = indptr[row], n = indptr[row + 1] - start;
                    for (int c = 0; c < ndof; ++c) {
                        int64_t pos = start + locate(indices + start, n, (int32_t)dofs[c]);
                        atomic_add(&V[pos], Ke[(int64_t)r * ndof + c], nthreads);
                    }
                }
            }
            for (int r = 0; r < ndof; ++r) atomic_add(&T[dofs[r]], te[r], nthreads);
        }
        free(X); free(x); free(sp); free(B); free(HBT); free(Ke); free(te); free(dofs);
    }
    return 0;
}

/* _GlobalAssemblyExplicit_DF_DPF_<3> (mechanics): T += sum_g detJ * (sigma . grad N_a), matrix free. */
int orc_internal_force(int mat, const double *prm, const double *points, const int64_t *elements, const double *Eulerx,
                       const double *Jm, const double *w, int64_t nelem, int64_t npe, int64_t nq, double *T,
                       int nthreads) {
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        double *X = malloc(sizeof(double) * npe * 3), *x = malloc(sizeof(double) * npe * 3);
        double *sp = malloc(sizeof(double) * npe * 3), *tr = malloc(sizeof(double) * npe * 3);
#pragma omp for schedule(static)
        for (int64_t e = 0; e < nelem; ++e) {
            const int64_t *el = elements + e * npe;
            gather(points, el, (int)npe, X);
            gather(Eulerx, el, (int)npe, x);
            memset(tr, 0, sizeof(double) * npe * 3);
            for (int g = 0; g < nq; ++g) {
                double F[9], sig[9], H[36];
                double detJ = kinematics_qp(Jm, w, X, x, (int)npe, (int)nq, g, 1, sp, F);
                material_qp(mat, prm, F, g_orient ? g_orient + e * 3 : NULL, sig, H);
                for (int a = 0; a < npe; ++a) {
                    double a0 = sp[a * 3], a1 = sp[a * 3 + 1], a2 = sp[a * 3 + 2];
                    tr[a * 3 + 0] += (a0 * sig[0] + a1 * sig[1] + a2 * sig[2]) * detJ;
                    tr[a * 3 + 1] += (a0 * sig[1] + a1 * sig[4] + a2 * sig[5]) * detJ;
                    tr[a * 3 + 2] += (a0 * sig[2] + a1 * sig[5] + a2 * sig[8]) * detJ;
                }
            }
            for (int a = 0; a < npe; ++a)
                for (int c = 0; c < 3; ++c) atomic_add(&T[el[a] * 3 + c], tr[a * 3 + c], nthreads);
        }
        free(X); free(x); free(sp); free(tr);
    }
    return 0;
}

/* Lumped mass (_GenericConstantMassIntegrand_, mass_type 0): row sums of
 * sum_g rho N N^T w_g |det dX/dxi|, scattered to M[3*node+c]. Bases[a*nq+g]. */
int orc_lumped_mass(double rho, const double *points, const int64_t *elements, const double *Jm, const double *w,
                    const double *Bases, int64_t nelem, int64_t npe, int64_t nq, double *M) {
    double *X = malloc(sizeof(double) * npe * 3), *lump = malloc(sizeof(double) * npe);
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t *el = elements + e * npe;
        gather(points, el, (int)npe, X);
        memset(lump, 0, sizeof(double) * npe);
        for (int g = 0; g < nq; ++g) {
            double PX[9] = {0};
            for (int d = 0; d < 3; ++d)
                for (int a = 0; a < npe; ++a) {
                    double j = Jm[(size_t)d * npe * nq + (size_t)a * nq + g];
                    for (int k = 0; k < 3; ++k) PX[d * 3 + k] += j * X[a * 3 + k];
                }
            double detJ = w[g] * fabs(det3(PX));
            for (int a = 0; a < npe; ++a) {
                double row = 0.0;
                for (int b = 0; b < npe; ++b) row += rho * Bases[a * nq + g] * Bases[b * nq + g];
                lump[a] += row * detJ;
            }
        }
        for (int a = 0; a < npe; ++a)
            for (int c = 0; c < 3; ++c) M[el[a] * 3 + c] += lump[a];
    }
    free(X); free(lump);
    return 0;
}

/* ---------------------------------------------------------------------------------------------
 * Sparsity pattern (ComputeSparsityPattern.pyx:44-112, ComputeSparsityPattern.h:22-125).
 * Phase 1 returns nnz; phase 2 fills indptr[nnode*nvar+1], indices[nnz] and, if the pointers are
 * non-null, data_local/data_global[nelem*ndof^2]. Returns -1 when a node belongs to no element
 * (the reference fails on such meshes).
 * --------------------------------------------------------------------------------------------- */
static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

typedef struct { int64_t *start, *list; } node_elems_t;

static int node_to_elements(const int64_t *elements, int64_t nelem, int64_t npe, int64_t nnode, node_elems_t *ne) {
    ne->start = calloc(nnode + 1, sizeof(int64_t));
    ne->list = malloc(sizeof(int64_t) * nelem * npe);
    for (int64_t k = 0; k < nelem * npe; ++k) ne->start[elements[k] + 1]++;
    for (int64_t n = 0; n < nnode; ++n) {
        if (ne->start[n + 1] == 0) return -1;
        ne->start[n + 1] += ne->start[n];
    }
    int64_t *fill = malloc(sizeof(int64_t) * nnode);
    memcpy(fill, ne->start, sizeof(int64_t) * nnode);
    for (int64_t k = 0; k < nelem * npe; ++k) ne->list[fill[elements[k]]++] = k / npe;
    free(fill);
    return 0;
}

/* sorted unique neighbour nodes of node n into buf; returns the count */
static int64_t neighbours(const int64_t *elements, int64_t npe, const node_elems_t *ne, int64_t n, int64_t *buf) {
    int64_t m = 0;
    for (int64_t j = ne->start[n]; j < ne->start[n + 1]; ++j)
        for (int64_t k = 0; k < npe; ++k) buf[m++] = elements[ne->list[j] * npe + k];
    qsort(buf, m, sizeof(int64_t), cmp_i64);
    int64_t u = 0;
    for (int64_t k = 0; k < m; ++k)
        if (u == 0 || buf[k] != buf[u - 1]) buf[u++] = buf[k];
    return u;
}

int64_t orc_sparsity_nnz(const int64_t *elements, int64_t nelem, int64_t npe, int64_t nnode, int64_t nvar) {
    node_elems_t ne;
    if (node_to_elements(elements, nelem, npe, nnode, &ne) != 0) { free(ne.start); free(ne.list); return -1; }
    int64_t maxdeg = 0;
    for (int64_t n = 0; n < nnode; ++n) if (ne.start[n + 1] - ne.start[n] > maxdeg) maxdeg = ne.start[n + 1] - ne.start[n];
    int64_t *buf = malloc(sizeof(int64_t) * (maxdeg * npe + 1));
    int64_t all = nnode * nvar, nnz = 0;
    for (int64_t n = 0; n < nnode; ++n) {
        int64_t c = neighbours(elements, npe, &ne, n, buf) * nvar;
        nnz += nvar * (c <= all ? c : all);
    }
    free(buf); free(ne.start); free(ne.list);
    return nnz;
}

int orc_sparsity(const int64_t *elements, int64_t nelem, int64_t npe, int64_t nnode, int64_t nvar, int32_t *indptr,
                 int32_t *indices, int32_t *data_local, int32_t *data_global) {
    node_elems_t ne;
    if (node_to_elements(elements, nelem, npe, nnode, &ne) != 0) { free(ne.start); free(ne.list); return -1; }
    int64_t maxdeg = 0;
    for (int64_t n = 0; n < nnode; ++n) if (ne.start[n + 1] - ne.start[n] > maxdeg) maxdeg = ne.start[n + 1] - ne.start[n];
    int64_t *buf = malloc(sizeof(int64_t) * (maxdeg * npe + 1));
    int64_t all = nnode * nvar, nnz = 0;
    indptr[0] = 0;
    for (int64_t n = 0; n < nnode; ++n) {
        int64_t cnt = neighbours(elements, npe, &ne, n, buf);
        for (int64_t j = 0; j < nvar; ++j) {
            for (int64_t k = 0; k < cnt; ++k)
                for (int64_t l = 0; l < nvar; ++l) indices[nnz++] = (int32_t)(nvar * buf[k] + l);
            int64_t c = cnt * nvar;
            indptr[n * nvar + j + 1] = (int32_t)(indptr[n * nvar + j] + (c <= all ? c : all));
        }
    }
    free(buf); free(ne.start); free(ne.list);
    if (!data_local || !data_global) return 0;
    int64_t ndof = npe * nvar, cap = ndof * ndof;
    int64_t *sorter = malloc(sizeof(int64_t) * npe), *rc = malloc(sizeof(int64_t) * ndof), *rcl = malloc(sizeof(int64_t) * ndof);
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t *el = elements + e * npe;
        /* sorter = argsort of the element's node list (values are distinct) */
        for (int64_t k = 0; k < npe; ++k) sorter[k] = k;
        for (int64_t k = 1; k < npe; ++k) { /* insertion sort of indices by node id */
            int64_t s = sorter[k], m = k;
            while (m > 0 && el[sorter[m - 1]] > el[s]) { sorter[m] = sorter[m - 1]; --m; }
            sorter[m] = s;
        }
        for (int64_t k = 0; k < npe; ++k)
            for (int64_t c = 0; c < nvar; ++c) {
                rc[nvar * k + c] = nvar * el[sorter[k]] + c;
                rcl[nvar * k + c] = sorter[k] * nvar + c;
            }
        for (int64_t i = 0; i < ndof; ++i) {
            int64_t row = rc[i], start = indptr[row], n = indptr[row + 1] - start;
            for (int64_t j = 0; j < ndof; ++j) {
                data_global[e * cap + i * ndof + j] = (int32_t)(start + locate(indices + start, n, (int32_t)rc[j]));
                data_local[e * cap + i * ndof + j] = (int32_t)(rcl[i] * ndof + rcl[j]);
            }
        }
    }
    free(sorter); free(rc); free(rcl);
    return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
