// fl_common.cuh -- device helpers shared by the sm_103a kernels: 3x3 algebra, the hyperelastic
// materials at one Gauss point, and the launch/error plumbing of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/florence_gb300.h"


namespace fl {

#define FL_CUDA_TRY(expr)                         \
    do {                                          \
        cudaError_t _e = (expr);                  \
        if (_e != cudaSuccess) return FL_ERR_CUDA; \
    } while (0)

inline int launch_status() { return cudaGetLastError() == cudaSuccess ? FL_OK : FL_ERR_CUDA; }

// Raises a kernel's dynamic shared-memory limit only when a launch needs more than any earlier
// one did on this device (one attribute call per kernel, device and size in steady state, so
// repeated launches -- e.g. inside a captured time loop -- make no runtime calls besides the
// launch itself). Kernel is the kernel's address as a template argument: one record per kernel.
template <auto Kernel>
inline int ensure_smem(size_t bytes) {
    constexpr int MAXDEV = 64;
    static size_t set_bytes[MAXDEV] = {};
    if (bytes <= 48 * 1024) return FL_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FL_ERR_CUDA;
    if (dev >= 0 && dev < MAXDEV && bytes <= set_bytes[dev]) return FL_OK;
    if (cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
        return FL_ERR_CUDA;
    if (dev >= 0 && dev < MAXDEV) set_bytes[dev] = bytes;
    return FL_OK;
}

// Material numbers (FL_MATERIAL_*), as the reference's explicit dispatcher numbers them
// (_LowLevelAssemblyExplicit_DF_DPF_.pyx:72-106)
enum { NEOHOOKEAN = 1, MOONEYRIVLIN = 2, NEARLYINCOMPRESSIBLEMR = 3, LINEARELASTIC = 10, ANISOTROPICMR1 = 11 };

// Extra elasticity terms of the nearly incompressible Mooney-Rivlin material:
//   c += kbI (b_ij d_kl + d_ij b_kl) + kgI (g_ij d_kl + d_ij g_kl)
//      + kg4 (g_ik d_jl + g_il d_jk + d_ik g_jl + d_il g_jk) + kgg g_ij g_kl,  g = cof(F) cof(F)^T
struct ExtraTangent {
    double kbI, kgI, kg4, kgg;
    double g[6];
};

struct MatParams {
    double p0, p1, p2;  // neo-Hookean: mu, lamb; Mooney-Rivlin: mu1, mu2, lamb
    double p3 = 0.0;    // transversely isotropic Mooney-Rivlin: mu3 (p0..p2 as Mooney-Rivlin)
};

// Inverse of a row-major 3x3 by adjugate over determinant; returns the determinant.
__device__ __forceinline__ double inv3(const double *m, double *r) {
    r[0] = m[4] * m[8] - m[5] * m[7];
    r[1] = m[2] * m[7] - m[1] * m[8];
    r[2] = m[1] * m[5] - m[2] * m[4];
    r[3] = m[5] * m[6] - m[3] * m[8];
    r[4] = m[0] * m[8] - m[2] * m[6];
    r[5] = m[2] * m[3] - m[0] * m[5];
    r[6] = m[3] * m[7] - m[4] * m[6];
    r[7] = m[1] * m[6] - m[0] * m[7];
    r[8] = m[0] * m[4] - m[1] * m[3];
    const double det = m[0] * r[0] + m[1] * r[3] + m[2] * r[6];
    const double s = 1.0 / det;
#pragma unroll
    for (int i = 0; i < 9; ++i) r[i] *= s;
    return det;
}

__device__ __forceinline__ double det3(const double *m) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// Symmetric 3x3 stored as xx,yy,zz,xy,xz,yz (the reference's Voigt order).
__device__ __forceinline__ int s6(int i, int j) {
    return i == j ? i : (i + j == 1 ? 3 : (i + j == 2 ? 4 : 5));
}

// Cauchy stress sigma (sym6), J = det F, b = F F^T (sym6) and the coefficients of the spatial
// elasticity tensor written as
//   c_ijkl = c1 (d_ik d_jl + d_il d_jk) + c2 d_ij d_kl + cbb (2 b_ij b_kl - b_ik b_jl - b_il b_jk).
// Neo-Hookean (_NeoHookean_.h:34-46):  sigma = mu/J (b - I) + lamb (J-1) I,
//   c1 = mu/J - lamb (J-1), c2 = lamb (2J-1), cbb = 0.
// Mooney-Rivlin (_MooneyRivlin_.h:38-64): sigma = 2mu1/J b + 2mu2/J (tr(b) b - b^2) - 2(mu1+2mu2)/J I
//   + lamb (J-1) I, c1 = 2(mu1+2mu2)/J - lamb (J-1), c2 = lamb (2J-1), cbb = 2 mu2/J.
template <int MAT>
__device__ __forceinline__ void material(const double *F, const MatParams &mp, double *sig, double *b, double &J,
                                         double &c1, double &c2, double &cbb, ExtraTangent *ex = nullptr,
                                         const double *N = nullptr) {
    J = det3(F);
    if constexpr (MAT == LINEARELASTIC) {  // _LinearElastic_.h:26-60: sigma = 2 mu eps + lamb tr(eps) I, eps = sym(F - I)
        const double mu = mp.p0, lamb = mp.p1;
        const double tre = F[0] + F[4] + F[8] - 3.0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                b[s6(i, j)] = 0.0;
                sig[s6(i, j)] = mu * (F[i * 3 + j] + F[j * 3 + i]) + (i == j ? lamb * tre - 2.0 * mu : 0.0);
            }
        c1 = mu;
        c2 = lamb;
        cbb = 0.0;
        (void)ex;
        return;
    } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j)
            b[s6(i, j)] = F[i * 3 + 0] * F[j * 3 + 0] + F[i * 3 + 1] * F[j * 3 + 1] + F[i * 3 + 2] * F[j * 3 + 2];
    const double iJ = 1.0 / J;
    if (MAT == NEOHOOKEAN) {
        const double mu = mp.p0, lamb = mp.p1;
        const double a = mu * iJ, dv = lamb * (J - 1.0);
        sig[0] = a * (b[0] - 1.0) + dv;
        sig[1] = a * (b[1] - 1.0) + dv;
        sig[2] = a * (b[2] - 1.0) + dv;
        sig[3] = a * b[3];
        sig[4] = a * b[4];
        sig[5] = a * b[5];
        c1 = a - dv;
        c2 = lamb * (2.0 * J - 1.0);
        cbb = 0.0;
    } else if (MAT == NEARLYINCOMPRESSIBLEMR) {
        // _NearlyIncompressibleMooneyRivlin_.h:26-90, parameters (alpha, beta, kappa)
        const double alpha = mp.p0, beta = mp.p1, kappa = mp.p2;
        double iF[9], g[6];
        inv3(F, iF);
        // cof(F) = J F^-T, g = cof cof^T = J^2 F^-T F^-1: g_ij = J^2 sum_k iF[k][i] iF[k][j]
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j)
                g[s6(i, j)] = J * J * (iF[0 * 3 + i] * iF[0 * 3 + j] + iF[1 * 3 + i] * iF[1 * 3 + j] + iF[2 * 3 + i] * iF[2 * 3 + j]);
        const double trb = b[0] + b[1] + b[2], trg = g[0] + g[1] + g[2];
        const double A = 2.0 * alpha * pow(J, -5.0 / 3.0), iJ3 = iJ * iJ * iJ, strg = sqrt(trg);
        const double B3 = beta * iJ3 * trg * strg, B1 = 3.0 * beta * iJ3 * strg, dv = kappa * (J - 1.0);
        const double diag = -A / 3.0 * trb + B3 + dv;
#pragma unroll
        for (int k = 0; k < 6; ++k) sig[k] = A * b[k] - B1 * g[k] + (k < 3 ? diag : 0.0);
        c1 = A / 3.0 * trb - B3 - dv;
        c2 = 2.0 / 9.0 * A * trb + B3 + kappa * (2.0 * J - 1.0);
        cbb = 0.0;
        if (ex) {
            ex->kbI = -2.0 / 3.0 * A;
            ex->kgI = -B1;
            ex->kg4 = B1;
            ex->kgg = B1 / trg;
#pragma unroll
            for (int k = 0; k < 6; ++k) ex->g[k] = g[k];
        }
    } else if (MAT == ANISOTROPICMR1) {
        // _AnisotropicMooneyRivlin_1_.h:31-88, parameters (mu1, mu2, lamb, mu3) and the element's
        // fibre direction N; with HN = cof(F) N = J F^-T N and m = HN HN^T:
        // sigma = 2mu1/J b + 2mu2/J (tr b b - b b) - 2(mu1+2mu2+mu3)/J I + lamb (J-1) I
        //       + 2mu3/J (FN FN^T + |HN|^2 I - m);
        // elasticity = the Mooney-Rivlin terms with mu1+2mu2+mu3, -4mu3/J (I m + m I),
        // 2mu3/J |HN|^2 (2 II - I_ik I_jl - I_il I_jk), 2mu3/J (I_ik m_jl + I_il m_jk + m_ik I_jl + m_il I_jk):
        // the last two fold into c1, c2 and the g-terms (kgI, kg4) of the shared tangent form
        const double mu1 = mp.p0, mu2 = mp.p1, lamb = mp.p2, mu3 = mp.p3;
        const double n0 = N ? N[0] : 0.0, n1 = N ? N[1] : 0.0, n2 = N ? N[2] : 0.0;
        double iF[9], FN[3], HN[3], m[6], bb[6];
        inv3(F, iF);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            FN[i] = fma(F[i * 3], n0, fma(F[i * 3 + 1], n1, F[i * 3 + 2] * n2));
            HN[i] = J * fma(iF[0 * 3 + i], n0, fma(iF[1 * 3 + i], n1, iF[2 * 3 + i] * n2));
        }
        const double inHN = HN[0] * HN[0] + HN[1] * HN[1] + HN[2] * HN[2];
        const double trb = b[0] + b[1] + b[2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                m[s6(i, j)] = HN[i] * HN[j];
                bb[s6(i, j)] = b[s6(i, 0)] * b[s6(0, j)] + b[s6(i, 1)] * b[s6(1, j)] + b[s6(i, 2)] * b[s6(2, j)];
                sig[s6(i, j)] = 2.0 * mu1 * iJ * b[s6(i, j)] + 2.0 * mu2 * iJ * (trb * b[s6(i, j)] - bb[s6(i, j)]) +
                                2.0 * mu3 * iJ * (FN[i] * FN[j] - HN[i] * HN[j]);
            }
        const double C = 2.0 * (mu1 + 2.0 * mu2 + mu3) * iJ, dv = lamb * (J - 1.0), a3 = 2.0 * mu3 * iJ;
        sig[0] += dv - C + a3 * inHN;
        sig[1] += dv - C + a3 * inHN;
        sig[2] += dv - C + a3 * inHN;
        c1 = C - dv - a3 * inHN;
        c2 = lamb * (2.0 * J - 1.0) + 2.0 * a3 * inHN;
        cbb = 2.0 * mu2 * iJ;
        if (ex) {
            ex->kbI = 0.0;
            ex->kgI = -2.0 * a3;
            ex->kg4 = a3;
            ex->kgg = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) ex->g[k] = m[k];
        }
    } else {
        const double mu1 = mp.p0, mu2 = mp.p1, lamb = mp.p2;
        const double trb = b[0] + b[1] + b[2];
        double bb[6];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j)
                bb[s6(i, j)] = b[s6(i, 0)] * b[s6(0, j)] + b[s6(i, 1)] * b[s6(1, j)] + b[s6(i, 2)] * b[s6(2, j)];
        const double A = 2.0 * mu1 * iJ, B = 2.0 * mu2 * iJ, C = 2.0 * (mu1 + 2.0 * mu2) * iJ, dv = lamb * (J - 1.0);
#pragma unroll
        for (int k = 0; k < 6; ++k) sig[k] = A * b[k] + B * (trb * b[k] - bb[k]);
        sig[0] += dv - C;
        sig[1] += dv - C;
        sig[2] += dv - C;
        c1 = C - dv;
        c2 = lamb * (2.0 * J - 1.0);
        cbb = B;
    }
    }  // not the linear elastic material
}

// Kinematics at one Gauss point from the reference-element gradients jm(d, a) (a callable) and
// the element's reference/current coordinates X, x [npe*3]:
//   Px = dx/dxi, PX = dX/dxi (rows d = xi direction), G = Px^{-1} (spatial gradients are
//   grad N_a[j] = sum_d G[j][d] jm(d,a)), F[i][j] = sum_d Px[d][i] PX^{-1}[j][d], and
//   detJ = w |det Px| (update) or w |det PX|, as _KinematicMeasures_.h:64-119 defines them.
template <int NPE, class JmFn, class CoordFn>
__device__ __forceinline__ double kinematics_fn(JmFn jm, CoordFn coords, double w, int update, double *G, double *F) {
    double PX[9], Px[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) PX[k] = Px[k] = 0.0;
#pragma unroll 4
    for (int a = 0; a < NPE; ++a) {
        const double j0 = jm(0, a), j1 = jm(1, a), j2 = jm(2, a);
        double X0, X1, X2, x0, x1, x2;
        coords(a, X0, X1, X2, x0, x1, x2);
        PX[0] += j0 * X0; PX[1] += j0 * X1; PX[2] += j0 * X2;
        PX[3] += j1 * X0; PX[4] += j1 * X1; PX[5] += j1 * X2;
        PX[6] += j2 * X0; PX[7] += j2 * X1; PX[8] += j2 * X2;
        Px[0] += j0 * x0; Px[1] += j0 * x1; Px[2] += j0 * x2;
        Px[3] += j1 * x0; Px[4] += j1 * x1; Px[5] += j1 * x2;
        Px[6] += j2 * x0; Px[7] += j2 * x1; Px[8] += j2 * x2;
    }
    double iPX[9];
    const double detX = inv3(PX, iPX);
    const double detx = inv3(Px, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            F[i * 3 + j] = Px[0 * 3 + i] * iPX[j * 3 + 0] + Px[1 * 3 + i] * iPX[j * 3 + 1] + Px[2 * 3 + i] * iPX[j * 3 + 2];
    return update ? w * fabs(detx) : w * fabs(detX);
}

// kinematics_fn with the reference-configuration part read from a per-mesh table: iPX = (dX/dxi)^-1
// and detX = det(dX/dxi) at the Gauss point (reference_geometry_kernel) -- the same values the sums
// over the reference coordinates give, so the results are identical; only the current
// configuration's sums are formed. coords(a, x0, x1, x2): current coordinates of node a.
template <int NPE, class JmFn, class CoordFn>
__device__ __forceinline__ double kinematics_ref(JmFn jm, CoordFn coords, const double *iPX, double detX, double w,
                                                 int update, double *G, double *F) {
    double Px[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Px[k] = 0.0;
#pragma unroll 4
    for (int a = 0; a < NPE; ++a) {
        const double j0 = jm(0, a), j1 = jm(1, a), j2 = jm(2, a);
        double x0, x1, x2;
        coords(a, x0, x1, x2);
        Px[0] += j0 * x0; Px[1] += j0 * x1; Px[2] += j0 * x2;
        Px[3] += j1 * x0; Px[4] += j1 * x1; Px[5] += j1 * x2;
        Px[6] += j2 * x0; Px[7] += j2 * x1; Px[8] += j2 * x2;
    }
    const double detx = inv3(Px, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            F[i * 3 + j] = Px[0 * 3 + i] * iPX[j * 3 + 0] + Px[1 * 3 + i] * iPX[j * 3 + 1] + Px[2 * 3 + i] * iPX[j * 3 + 2];
    return update ? w * fabs(detx) : w * fabs(detX);
}

// kinematics_fn with the element coordinates in arrays X, x [npe*3]
template <int NPE, class JmFn>
__device__ __forceinline__ double kinematics(JmFn jm, const double *X, const double *x, double w, int update, double *G,
                                             double *F) {
    auto coords = [&](int a, double &X0, double &X1, double &X2, double &x0, double &x1, double &x2) {
        X0 = X[a * 3]; X1 = X[a * 3 + 1]; X2 = X[a * 3 + 2];
        x0 = x[a * 3]; x1 = x[a * 3 + 1]; x2 = x[a * 3 + 2];
    };
    return kinematics_fn<NPE>(jm, coords, w, update, G, F);
}

// Float-pair number hi + lo (|lo| <= ulp(hi) / 2) with FP32-pipe arithmetic: products error-free
// in their leading part (fma), sums by Knuth's two-sum, ~2^-46 relative per operation. Used for
// the Gauss-point tangent of the FP64 path and the float-pair explicit internal force, whose
// FP64 forms would hold GB300's FP64 pipe.
namespace fpair {  // its own namespace: the overloads are found by argument lookup only, so they
                  // do not hide the FP64 fma of namespace fl's callers
struct FloatPair {
    float h, l;
    FloatPair() = default;
    __device__ constexpr FloatPair(float h_, float l_) : h(h_), l(l_) {}
    __device__ explicit FloatPair(double x) : h((float)x), l((float)(x - (double)(float)x)) {}
    __device__ explicit FloatPair(int x) : h((float)x), l(0.f) {}
};
__device__ __forceinline__ FloatPair df_renorm(float s, float e) {
    const float h = s + e;
    return FloatPair(h, e - (h - s));
}
__device__ __forceinline__ FloatPair operator+(FloatPair a, FloatPair b) {
    const float s = a.h + b.h, bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb) + (a.l + b.l);
    return df_renorm(s, e);
}
__device__ __forceinline__ FloatPair operator-(FloatPair a) { return FloatPair(-a.h, -a.l); }
__device__ __forceinline__ FloatPair operator-(FloatPair a, FloatPair b) { return a + (-b); }
__device__ __forceinline__ FloatPair &operator+=(FloatPair &a, FloatPair b) { return a = a + b; }
__device__ __forceinline__ FloatPair operator*(FloatPair a, FloatPair b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p) + fmaf(a.h, b.l, a.l * b.h);
    return df_renorm(p, e);
}
__device__ __forceinline__ FloatPair fma(FloatPair a, FloatPair b, FloatPair c) {  // a b + c
    const float p = a.h * b.h;
    const float pe = fmaf(a.h, b.h, -p) + fmaf(a.h, b.l, a.l * b.h);
    const float s = p + c.h, bb = s - p;
    const float e = (p - (s - bb)) + (c.h - bb) + (pe + c.l);
    return df_renorm(s, e);
}
}  // namespace fpair
using fpair::FloatPair;
// kinematics_fn with the coordinate sums in float-pair arithmetic on the FP32 pipe: PX = sum_a
// dN_a/dxi X_a and Pu = sum_a dN_a/dxi u_a (u = x - X, so small strains keep their relative
// precision) from float-pair gradients jp(d, a) and node data nodep(a, X, u); both sums are then
// taken to FP64 (Px = PX + Pu) and the rest is kinematics_fn's FP64 code.
template <int NPE, class JpFn, class NodeFn>
__device__ __forceinline__ double kinematics_pair(JpFn jp, NodeFn nodep, double w, int update, double *G, double *F) {
    FloatPair PXp[9], Pup[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) PXp[k] = Pup[k] = FloatPair(0.f, 0.f);
#pragma unroll 2
    for (int a = 0; a < NPE; ++a) {
        FloatPair X[3], U[3];
        nodep(a, X, U);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const FloatPair j = jp(d, a);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                PXp[d * 3 + k] = fma(j, X[k], PXp[d * 3 + k]);
                Pup[d * 3 + k] = fma(j, U[k], Pup[d * 3 + k]);
            }
        }
    }
    double PX[9], Px[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        PX[k] = (double)PXp[k].h + (double)PXp[k].l;
        Px[k] = PX[k] + ((double)Pup[k].h + (double)Pup[k].l);
    }
    double iPX[9];
    const double detX = inv3(PX, iPX);
    const double detx = inv3(Px, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            F[i * 3 + j] = Px[0 * 3 + i] * iPX[j * 3 + 0] + Px[1 * 3 + i] * iPX[j * 3 + 1] + Px[2 * 3 + i] * iPX[j * 3 + 2];
    return update ? w * fabs(detx) : w * fabs(detX);
}

namespace fpair {
__device__ __forceinline__ FloatPair operator/(FloatPair a, FloatPair b) {  // a / b, one correction step
    const float q1 = a.h / b.h;
    const FloatPair r = a - FloatPair(q1, 0.f) * b;
    return df_renorm(q1, r.h / b.h);
}
__device__ __forceinline__ double to_double(FloatPair a) { return (double)a.h + (double)a.l; }
}  // namespace fpair

}  // namespace fl
