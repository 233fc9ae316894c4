// fl_explicit.cu -- matrix-free internal force for explicit dynamics
// (replaces _GlobalAssemblyExplicit_DF_DPF_<3>, Florence/FiniteElements/Assembly/_Assembly_/
//  _LowLevelAssemblyExplicit_DF_DPF_.h:459-720) and the lumped mass
// (replaces _GenericConstantMassIntegrand_ with mass_type 0, Florence/VariationalPrinciple/_Mass_/
//  _MassIntegrand_.h:249-400).
//
// Internal force, EPC elements per CTA:
//   one thread per (element, Gauss point): kinematics and stress, S[i][d] = detJ sum_j sigma_ij G[j][d];
//   one thread per (element, node, component): t = sum_g sum_d Jm[d][a][g] S_g[i][d], added into T.
// Same quantity as the implicit residual: T_(a,i) = sum_g detJ (sigma . grad N_a)_i.
#include <algorithm>

#include "fl_common.cuh"

namespace fl {

constexpr int IF_EPC = 8, IF_NT = 256;

struct IfArgs {
    const double *points;
    const uint64_t *elements;
    const double *Eulerx;
    const double *Jm;
    const double *w;
    int64_t nelem, nnode;
    int nq;
    double *T;
    MatParams mp;
    int *flags;
};

template <int NPE, int MAT>
__global__ void __launch_bounds__(IF_NT) internal_force_kernel(const IfArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nq = A.nq;
    double *Xs = reinterpret_cast<double *>(smem_raw);  // [EPC][NPE*3]
    double *xs = Xs + IF_EPC * NPE * 3;
    double *Ss = xs + IF_EPC * NPE * 3;                  // [EPC][nq][9]
    int *nodes = reinterpret_cast<int *>(Ss + (size_t)IF_EPC * nq * 9);
    __shared__ int s_flag;
    const int64_t e0 = (int64_t)blockIdx.x * IF_EPC;
    int flag = 0;
    if (threadIdx.x == 0) s_flag = 0;
    for (int idx = threadIdx.x; idx < IF_EPC * NPE; idx += IF_NT) {
        const int slot = idx / NPE, a = idx % NPE;
        const int64_t e = e0 + slot;
        if (e >= A.nelem) continue;
        uint64_t nd = A.elements[e * NPE + a];
        if (nd >= (uint64_t)A.nnode) {
            flag |= FL_FLAG_BAD_INDEX;
            nd = 0;
        }
        nodes[idx] = (int)nd;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            Xs[idx * 3 + k] = A.points[nd * 3 + k];
            xs[idx * 3 + k] = A.Eulerx[nd * 3 + k];
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < IF_EPC * nq; idx += IF_NT) {
        const int slot = idx / nq, g = idx % nq;
        if (e0 + slot >= A.nelem) continue;
        auto jm = [&](int d, int a) { return __ldg(A.Jm + ((size_t)d * NPE + a) * nq + g); };
        double G[9], F[9];
        const double detJ = kinematics<NPE>(jm, Xs + slot * NPE * 3, xs + slot * NPE * 3, __ldg(A.w + g), 1, G, F);
        double sig[6], b[6], J, c1, c2, cbb;
        material<MAT>(F, A.mp, sig, b, J, c1, c2, cbb);
        if (!(J > 0.0)) flag |= FL_FLAG_NONPOSITIVE_J;
        double *S = Ss + (size_t)idx * 9;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                S[i * 3 + d] = detJ * (sig[s6(i, 0)] * G[0 * 3 + d] + sig[s6(i, 1)] * G[1 * 3 + d] + sig[s6(i, 2)] * G[2 * 3 + d]);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < IF_EPC * NPE * 3; idx += IF_NT) {
        const int slot = idx / (NPE * 3), r = idx % (NPE * 3), a = r / 3, i = r % 3;
        if (e0 + slot >= A.nelem) continue;
        const double *S = Ss + (size_t)slot * nq * 9 + i * 3;
        double t = 0.0;
        for (int g = 0; g < nq; ++g, S += 9) {
            t = fma(__ldg(A.Jm + (size_t)a * nq + g), S[0], t);
            t = fma(__ldg(A.Jm + ((size_t)NPE + a) * nq + g), S[1], t);
            t = fma(__ldg(A.Jm + ((size_t)2 * NPE + a) * nq + g), S[2], t);
        }
        atomicAdd(A.T + 3 * (int64_t)nodes[slot * NPE + a] + i, t);
    }
    if (flag) atomicOr(&s_flag, flag);
    __syncthreads();
    if (threadIdx.x == 0 && s_flag && A.flags) atomicOr(A.flags, s_flag);
}

template <int NPE, int MAT>
static int launch_if(const IfArgs &A, cudaStream_t s) {
    const size_t smem = sizeof(double) * ((size_t)2 * IF_EPC * NPE * 3 + (size_t)IF_EPC * A.nq * 9) + sizeof(int) * IF_EPC * NPE;
    if (smem > 227 * 1024) return FL_ERR_UNSUPPORTED;
    { const int st = ensure_smem<internal_force_kernel<NPE, MAT>>(smem); if (st != FL_OK) return st; }
    const int64_t grid = (A.nelem + IF_EPC - 1) / IF_EPC;
    if (grid == 0) return FL_OK;
    internal_force_kernel<NPE, MAT><<<(unsigned)grid, IF_NT, smem, s>>>(A);
    return launch_status();
}

template <int MAT>
static int dispatch_if(int npe, const IfArgs &A, cudaStream_t s) {
    switch (npe) {
        case 4: return launch_if<4, MAT>(A, s);
        case 8: return launch_if<8, MAT>(A, s);
        case 10: return launch_if<10, MAT>(A, s);
        case 20: return launch_if<20, MAT>(A, s);
        case 27: return launch_if<27, MAT>(A, s);
        case 35: return launch_if<35, MAT>(A, s);
        case 64: return launch_if<64, MAT>(A, s);
        case 125: return launch_if<125, MAT>(A, s);
        default: return FL_ERR_UNSUPPORTED;
    }
}

// Lumped mass: thread per (element, Gauss point) computes w|det dX/dxi| and sum_b N_b; thread
// per (element, node) sums rho N_a (sum_b N_b) w|det| over the points.
constexpr int LM_EPC = 8, LM_NT = 256;

__global__ void __launch_bounds__(LM_NT)
    lumped_mass_kernel(const double *points, const uint64_t *elements, const double *bases, const double *Jm,
                       const double *w, int64_t nelem, int npe, int nq, int64_t nnode, double rho, double *M,
                       int *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *dJ = reinterpret_cast<double *>(smem_raw);  // [EPC][nq]
    double *Nsum = dJ + LM_EPC * nq;                      // [nq]
    const int64_t e0 = (int64_t)blockIdx.x * LM_EPC;
    for (int g = threadIdx.x; g < nq; g += LM_NT) {
        double s = 0.0;
        for (int b = 0; b < npe; ++b) s += bases[(size_t)b * nq + g];
        Nsum[g] = s;
    }
    for (int idx = threadIdx.x; idx < LM_EPC * nq; idx += LM_NT) {
        const int slot = idx / nq, g = idx % nq;
        const int64_t e = e0 + slot;
        if (e >= nelem) continue;
        double PX[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < npe; ++a) {
            uint64_t nd = elements[e * npe + a];
            if (nd >= (uint64_t)nnode) {
                if (err) atomicOr(err, FL_FLAG_BAD_INDEX);
                nd = 0;
            }
            const double X0 = points[nd * 3], X1 = points[nd * 3 + 1], X2 = points[nd * 3 + 2];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double j = Jm[((size_t)d * npe + a) * nq + g];
                PX[d * 3] += j * X0;
                PX[d * 3 + 1] += j * X1;
                PX[d * 3 + 2] += j * X2;
            }
        }
        dJ[idx] = w[g] * fabs(det3(PX));
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < LM_EPC * npe; idx += LM_NT) {
        const int slot = idx / npe, a = idx % npe;
        const int64_t e = e0 + slot;
        if (e >= nelem) continue;
        double m = 0.0;
        for (int g = 0; g < nq; ++g) m += rho * bases[(size_t)a * nq + g] * Nsum[g] * dJ[slot * nq + g];
        uint64_t nd = elements[e * npe + a];
        if (nd >= (uint64_t)nnode) continue;
        for (int c = 0; c < 3; ++c) atomicAdd(M + 3 * nd + c, m);
    }
}

}  // namespace fl

extern "C" {

int fl_GlobalAssemblyExplicit_DF_DPF_(const double *points, const uint64_t *elements, const double *Eulerx,
                                      const double *Eulerp, const double *bases, const double *Jm,
                                      const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss,
                                      int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t H_VoigtSize,
                                      int64_t requires_geometry_update, double *T, double rho, double mu,
                                      double mu1, double mu2, double mu3, double mue, double lamb, double eps_1,
                                      double eps_2, double eps_3, double eps_e,
                                      const double *anisotropic_orientations, int material_number,
                                      int formulation_number, int *flags, fl_stream_t stream) {
    (void)Eulerp; (void)bases; (void)H_VoigtSize; (void)requires_geometry_update; (void)rho; (void)mue;
    (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e; (void)anisotropic_orientations;
    if (ndim != 3 || nvar != 3 || formulation_number != 0) return FL_ERR_ARG;
    if (nelem == 0 && nnode > 0 && ngauss > 0) return FL_OK;  // nothing is read or written
    if (!points || !elements || !Eulerx || !Jm || !AllGauss || !T || nelem < 0 || nnode <= 0 || ngauss <= 0)
        return FL_ERR_ARG;
    fl::IfArgs A{points, elements, Eulerx, Jm, AllGauss, nelem, nnode, (int)ngauss, T, {0, 0, 0}, flags};
    if (material_number == FL_MATERIAL_NEOHOOKEAN) {
        A.mp = {mu, lamb, 0.0};
        return fl::dispatch_if<fl::NEOHOOKEAN>((int)nodeperelem, A, (cudaStream_t)stream);
    }
    if (material_number == FL_MATERIAL_MOONEYRIVLIN) {
        A.mp = {mu1, mu2, lamb};
        return fl::dispatch_if<fl::MOONEYRIVLIN>((int)nodeperelem, A, (cudaStream_t)stream);
    }
    if (material_number == FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN) {  // (alpha, beta, kappa) as (mu1, mu2, mu3)
        A.mp = {mu1, mu2, mu3};
        return fl::dispatch_if<fl::NEARLYINCOMPRESSIBLEMR>((int)nodeperelem, A, (cudaStream_t)stream);
    }
    if (material_number == FL_MATERIAL_LINEARELASTIC) {
        A.mp = {mu, lamb, 0.0};
        return fl::dispatch_if<fl::LINEARELASTIC>((int)nodeperelem, A, (cudaStream_t)stream);
    }
    return FL_ERR_UNSUPPORTED;
}

int fl_LumpedMass(const double *points, const uint64_t *elements, const double *bases, const double *Jm,
                  const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss, int64_t nelem,
                  int64_t nodeperelem, int64_t nnode, double rho, double *M, int *flags, fl_stream_t stream) {
    if (ndim != 3 || nvar != 3) return FL_ERR_ARG;
    if (nelem == 0 && nnode > 0 && ngauss > 0) return FL_OK;  // nothing is read or written
    if (!points || !elements || !bases || !Jm || !AllGauss || !M || nelem < 0 || nnode <= 0 || ngauss <= 0 ||
        nodeperelem <= 0)
        return FL_ERR_ARG;
    const size_t smem = sizeof(double) * ((size_t)fl::LM_EPC * ngauss + ngauss);
    if (smem > 227 * 1024) return FL_ERR_UNSUPPORTED;
    { const int st = fl::ensure_smem<fl::lumped_mass_kernel>(smem); if (st != FL_OK) return st; }
    const int64_t grid = (nelem + fl::LM_EPC - 1) / fl::LM_EPC;
    if (grid == 0) return FL_OK;
    fl::lumped_mass_kernel<<<(unsigned)grid, fl::LM_NT, smem, (cudaStream_t)stream>>>(
        points, elements, bases, Jm, AllGauss, nelem, (int)nodeperelem, (int)ngauss, nnode, rho, M, flags);
    return fl::launch_status();
}

}  // extern "C"

// ================================================================================================
// Explicit central-difference time stepping (replaces the lumped-mass loop of
// ExplicitStructuralDynamicIntegrator.Solver, Florence/TimeIntegrators/
// ExplicitStructuralDynamicIntegrator.py:28-245): reference gradients for the FP32 internal force,
// the FP32 internal force, the leapfrog update, and the strain energy for energy bookkeeping.
// ================================================================================================
namespace fl {

// grad0[((e*nq + g)*npe + a)*3 + d] = dN_a/dX_d at Gauss point g (FP32), dV[e*nq + g] = w |det dX/dxi|
template <int NPE>
__global__ void __launch_bounds__(128) ref_grad_kernel(const double *points, const uint64_t *elements, const double *Jm,
                                                       const double *w, int64_t nelem, int nq, int64_t nnode,
                                                       float *grad0, float *dV, int *flags) {
    const int64_t t = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (t >= nelem * nq) return;
    const int64_t e = t / nq;
    const int g = (int)(t % nq);
    double PX[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < NPE; ++a) {
        uint64_t nd = elements[e * NPE + a];
        if (nd >= (uint64_t)nnode) {
            if (flags) atomicOr(flags, FL_FLAG_BAD_INDEX);
            nd = 0;
        }
        for (int d = 0; d < 3; ++d) {
            const double j = Jm[((size_t)d * NPE + a) * nq + g];
            PX[d * 3] = fma(j, points[nd * 3], PX[d * 3]);
            PX[d * 3 + 1] = fma(j, points[nd * 3 + 1], PX[d * 3 + 1]);
            PX[d * 3 + 2] = fma(j, points[nd * 3 + 2], PX[d * 3 + 2]);
        }
    }
    double iPX[9];
    const double det = inv3(PX, iPX);
    dV[t] = (float)(w[g] * fabs(det));
    for (int a = 0; a < NPE; ++a) {
        const double j0 = Jm[((size_t)0 * NPE + a) * nq + g], j1 = Jm[((size_t)1 * NPE + a) * nq + g],
                     j2 = Jm[((size_t)2 * NPE + a) * nq + g];
        for (int d = 0; d < 3; ++d)  // dN_a/dX_d = sum_k (dX/dxi)^{-1}[d][k] dN_a/dxi_k
            grad0[((size_t)t * NPE + a) * 3 + d] = (float)fma(iPX[d * 3], j0, fma(iPX[d * 3 + 1], j1, iPX[d * 3 + 2] * j2));
    }
}

// FP32 internal force (total Lagrangian form, neo-Hookean): H = grad_0 u, F = I + H,
// P = mu/J (q I + H + H^T + j H - cof H) + lamb j cof F with j = J - 1 = tr H + q and
// q = (tr^2 H - tr H^2)/2 + det H, cof F = (1 + tr H) I - H^T + cof H -- every term formed from
// H directly, so small strains keep FP32's relative precision. T_a += P grad_0 N_a dV in FP32.
// This is the same internal force as the reference's sum_g detJ sigma grad N_a, rewritten in the
// reference configuration.
constexpr int F32_EPC = 4, F32_NT = 128;

template <int NPE>
__global__ void __launch_bounds__(F32_NT) internal_force_f32_kernel(const uint64_t *elements, const double *u,
                                                                    const float *grad0, const float *dV, int64_t nelem,
                                                                    int nq, int64_t nnode, float mu, float lamb,
                                                                    float *T, int *flags) {
    __shared__ float us[F32_EPC][NPE * 3];
    __shared__ float Ps[F32_EPC][32][9];  // first Piola stress x dV per Gauss point (nq <= 32)
    __shared__ int nodes[F32_EPC][NPE];
    const int64_t e0 = (int64_t)blockIdx.x * F32_EPC;
    int flag = 0;
    for (int idx = threadIdx.x; idx < F32_EPC * NPE; idx += F32_NT) {
        const int s = idx / NPE, a = idx % NPE;
        if (e0 + s >= nelem) continue;
        uint64_t nd = elements[(e0 + s) * NPE + a];
        if (nd >= (uint64_t)nnode) {
            flag |= FL_FLAG_BAD_INDEX;
            nd = 0;
        }
        nodes[s][a] = (int)nd;
        us[s][a * 3] = (float)u[nd * 3];
        us[s][a * 3 + 1] = (float)u[nd * 3 + 1];
        us[s][a * 3 + 2] = (float)u[nd * 3 + 2];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < F32_EPC * nq; idx += F32_NT) {
        const int s = idx / nq, g = idx % nq;
        const int64_t e = e0 + s;
        if (e >= nelem) continue;
        const float *gr = grad0 + ((size_t)(e * nq + g) * NPE) * 3;
        float H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < NPE; ++a) {
            const float g0 = gr[a * 3], g1 = gr[a * 3 + 1], g2 = gr[a * 3 + 2];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float ui = us[s][a * 3 + i];
                H[i * 3] = fmaf(ui, g0, H[i * 3]);
                H[i * 3 + 1] = fmaf(ui, g1, H[i * 3 + 1]);
                H[i * 3 + 2] = fmaf(ui, g2, H[i * 3 + 2]);
            }
        }
        const float trH = H[0] + H[4] + H[8];
        const float trH2 = H[0] * H[0] + H[4] * H[4] + H[8] * H[8] + 2.f * (H[1] * H[3] + H[2] * H[6] + H[5] * H[7]);
        float cH[9];  // cofactor of H
        cH[0] = H[4] * H[8] - H[5] * H[7];
        cH[1] = H[5] * H[6] - H[3] * H[8];
        cH[2] = H[3] * H[7] - H[4] * H[6];
        cH[3] = H[2] * H[7] - H[1] * H[8];
        cH[4] = H[0] * H[8] - H[2] * H[6];
        cH[5] = H[1] * H[6] - H[0] * H[7];
        cH[6] = H[1] * H[5] - H[2] * H[4];
        cH[7] = H[2] * H[3] - H[0] * H[5];
        cH[8] = H[0] * H[4] - H[1] * H[3];
        const float detH = H[0] * cH[0] + H[1] * cH[1] + H[2] * cH[2];
        const float q = 0.5f * (trH * trH - trH2) + detH;
        const float j = trH + q;
        const float J = 1.f + j;
        if (!(J > 0.f)) flag |= FL_FLAG_NONPOSITIVE_J;
        const float a1 = mu / J, a2 = lamb * j;
        const float dv = dV[e * nq + g];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float id = (r == c) ? 1.f : 0.f;
                const float A = q * id + H[r * 3 + c] + H[c * 3 + r] + j * H[r * 3 + c] - cH[r * 3 + c];
                const float cofF = (1.f + trH) * id - H[c * 3 + r] + cH[r * 3 + c];
                Ps[s][g][r * 3 + c] = (a1 * A + a2 * cofF) * dv;
            }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < F32_EPC * NPE * 3; idx += F32_NT) {
        const int s = idx / (NPE * 3), r = idx % (NPE * 3), a = r / 3, i = r % 3;
        const int64_t e = e0 + s;
        if (e >= nelem) continue;
        float t = 0.f;
        for (int g = 0; g < nq; ++g) {
            const float *gr = grad0 + ((size_t)(e * nq + g) * NPE + a) * 3;
            t = fmaf(Ps[s][g][i * 3], gr[0], fmaf(Ps[s][g][i * 3 + 1], gr[1], fmaf(Ps[s][g][i * 3 + 2], gr[2], t)));
        }
        atomicAdd(T + 3 * (int64_t)nodes[s][a] + i, t);
    }
    if (flag && flags) atomicOr(flags, flag);
}

// Float-pair internal force: the FP32 kernel's total-Lagrangian neo-Hookean force with every
// quantity an unevaluated float pair (FloatPair, ~2^-46 relative per operation) on the FP32 pipe:
// FP64-level results without FP64 instructions in the loops. Reference gradients come as hi / lo
// float arrays and dV in FP64 (ref_grad_pair_kernel); T is accumulated in FP64.
constexpr int PF_EPC = 4, PF_NT = 128;

template <int NPE>
__global__ void __launch_bounds__(128) ref_grad_pair_kernel(const double *points, const uint64_t *elements,
                                                            const double *Jm, const double *w, int64_t nelem, int nq,
                                                            int64_t nnode, float *gh, float *gl, double *dV,
                                                            int *flags) {
    const int64_t t = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (t >= nelem * nq) return;
    const int64_t e = t / nq;
    const int g = (int)(t % nq);
    double PX[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < NPE; ++a) {
        uint64_t nd = elements[e * NPE + a];
        if (nd >= (uint64_t)nnode) {
            if (flags) atomicOr(flags, FL_FLAG_BAD_INDEX);
            nd = 0;
        }
        for (int d = 0; d < 3; ++d) {
            const double j = Jm[((size_t)d * NPE + a) * nq + g];
            PX[d * 3] = fma(j, points[nd * 3], PX[d * 3]);
            PX[d * 3 + 1] = fma(j, points[nd * 3 + 1], PX[d * 3 + 1]);
            PX[d * 3 + 2] = fma(j, points[nd * 3 + 2], PX[d * 3 + 2]);
        }
    }
    double iPX[9];
    const double det = inv3(PX, iPX);
    dV[t] = w[g] * fabs(det);
    for (int a = 0; a < NPE; ++a) {
        const double j0 = Jm[((size_t)0 * NPE + a) * nq + g], j1 = Jm[((size_t)1 * NPE + a) * nq + g],
                     j2 = Jm[((size_t)2 * NPE + a) * nq + g];
        for (int d = 0; d < 3; ++d) {
            const double v = fma(iPX[d * 3], j0, fma(iPX[d * 3 + 1], j1, iPX[d * 3 + 2] * j2));
            const float h = (float)v;
            gh[((size_t)t * NPE + a) * 3 + d] = h;
            gl[((size_t)t * NPE + a) * 3 + d] = (float)(v - (double)h);
        }
    }
}

template <int NPE>
__global__ void __launch_bounds__(PF_NT) internal_force_pair_kernel(const uint64_t *elements, const double *u,
                                                                     const float *gh, const float *gl,
                                                                     const double *dV, int64_t nelem, int nq,
                                                                     int64_t nnode, double mu_d, double lamb_d,
                                                                     double *T, int *flags) {
    using fpair::to_double;
    __shared__ FloatPair us[PF_EPC][NPE * 3];
    __shared__ FloatPair Ps[PF_EPC][32][9];  // first Piola stress x dV per Gauss point (nq <= 32)
    __shared__ int nodes[PF_EPC][NPE];
    const int64_t e0 = (int64_t)blockIdx.x * PF_EPC;
    int flag = 0;
    for (int idx = threadIdx.x; idx < PF_EPC * NPE; idx += PF_NT) {
        const int s = idx / NPE, a = idx % NPE;
        if (e0 + s >= nelem) continue;
        uint64_t nd = elements[(e0 + s) * NPE + a];
        if (nd >= (uint64_t)nnode) {
            flag |= FL_FLAG_BAD_INDEX;
            nd = 0;
        }
        nodes[s][a] = (int)nd;
#pragma unroll
        for (int i = 0; i < 3; ++i) us[s][a * 3 + i] = FloatPair(u[nd * 3 + i]);
    }
    __syncthreads();
    const FloatPair mu(mu_d), lamb(lamb_d), one(1), half(0.5), two(2);
    for (int idx = threadIdx.x; idx < PF_EPC * nq; idx += PF_NT) {
        const int s = idx / nq, g = idx % nq;
        const int64_t e = e0 + s;
        if (e >= nelem) continue;
        const size_t base = ((size_t)(e * nq + g) * NPE) * 3;
        FloatPair H[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) H[k] = FloatPair(0.f, 0.f);
        for (int a = 0; a < NPE; ++a) {
            const FloatPair g0(gh[base + a * 3], gl[base + a * 3]), g1(gh[base + a * 3 + 1], gl[base + a * 3 + 1]),
                g2(gh[base + a * 3 + 2], gl[base + a * 3 + 2]);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const FloatPair ui = us[s][a * 3 + i];
                H[i * 3] = fma(ui, g0, H[i * 3]);
                H[i * 3 + 1] = fma(ui, g1, H[i * 3 + 1]);
                H[i * 3 + 2] = fma(ui, g2, H[i * 3 + 2]);
            }
        }
        const FloatPair trH = H[0] + H[4] + H[8];
        const FloatPair trH2 = H[0] * H[0] + H[4] * H[4] + H[8] * H[8] + two * (H[1] * H[3] + H[2] * H[6] + H[5] * H[7]);
        FloatPair cH[9];  // cofactor of H
        cH[0] = H[4] * H[8] - H[5] * H[7];
        cH[1] = H[5] * H[6] - H[3] * H[8];
        cH[2] = H[3] * H[7] - H[4] * H[6];
        cH[3] = H[2] * H[7] - H[1] * H[8];
        cH[4] = H[0] * H[8] - H[2] * H[6];
        cH[5] = H[1] * H[6] - H[0] * H[7];
        cH[6] = H[1] * H[5] - H[2] * H[4];
        cH[7] = H[2] * H[3] - H[0] * H[5];
        cH[8] = H[0] * H[4] - H[1] * H[3];
        const FloatPair detH = H[0] * cH[0] + H[1] * cH[1] + H[2] * cH[2];
        const FloatPair q = half * (trH * trH - trH2) + detH;
        const FloatPair j = trH + q;
        const FloatPair J = one + j;
        if (!(J.h > 0.f)) flag |= FL_FLAG_NONPOSITIVE_J;
        const FloatPair a1 = mu / J, a2 = lamb * j;
        const FloatPair dv(dV[e * nq + g]);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                FloatPair A = H[r * 3 + c] + H[c * 3 + r] + j * H[r * 3 + c] - cH[r * 3 + c];
                FloatPair cofF = cH[r * 3 + c] - H[c * 3 + r];
                if (r == c) {
                    A = A + q;
                    cofF = cofF + one + trH;
                }
                Ps[s][g][r * 3 + c] = (a1 * A + a2 * cofF) * dv;
            }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < PF_EPC * NPE * 3; idx += PF_NT) {
        const int s = idx / (NPE * 3), r = idx % (NPE * 3), a = r / 3, i = r % 3;
        const int64_t e = e0 + s;
        if (e >= nelem) continue;
        FloatPair t(0.f, 0.f);
        for (int g = 0; g < nq; ++g) {
            const size_t o = ((size_t)(e * nq + g) * NPE + a) * 3;
            t = fma(Ps[s][g][i * 3], FloatPair(gh[o], gl[o]), t);
            t = fma(Ps[s][g][i * 3 + 1], FloatPair(gh[o + 1], gl[o + 1]), t);
            t = fma(Ps[s][g][i * 3 + 2], FloatPair(gh[o + 2], gl[o + 2]), t);
        }
        atomicAdd(T + 3 * (int64_t)nodes[s][a] + i, to_double(t));
    }
    if (flag && flags) atomicOr(flags, flag);
}

// leapfrog central difference: a = (F - T)/M on free dofs, v += dt a, u += dt v
template <class TT>
__global__ void cd_update_kernel(int64_t n, double dt, const TT *T, const double *Fext, const double *Minv,
                                 const int8_t *fixed, double *u, double *v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (fixed[i]) continue;
        const double f = (Fext ? Fext[i] : 0.0) - (double)T[i];
        const double vi = fma(dt, f * Minv[i], v[i]);
        v[i] = vi;
        u[i] = fma(dt, vi, u[i]);
    }
}

// strain energy sum_e sum_g W(F) w |det dX/dxi|: neo-Hookean W = mu/2 (tr C - 3) - mu ln J + lamb/2 (J-1)^2
// (NeoHookean.InternalEnergy, Florence/MaterialLibrary/NeoHookean.py:70-80)
template <int NPE>
__global__ void __launch_bounds__(128) strain_energy_kernel(const double *points, const uint64_t *elements,
                                                            const double *Eulerx, const double *Jm, const double *w,
                                                            int64_t nelem, int nq, int64_t nnode, double mu,
                                                            double lamb, double *energy) {
    const int64_t t = (int64_t)blockIdx.x * 128 + threadIdx.x;
    double W = 0.0;
    if (t < nelem * nq) {
        const int64_t e = t / nq;
        const int g = (int)(t % nq);
        const uint64_t *el = elements + e * NPE;
        auto jm = [&](int d, int a) { return Jm[((size_t)d * NPE + a) * nq + g]; };
        auto coords = [&](int a, double &X0, double &X1, double &X2, double &x0, double &x1, double &x2) {
            uint64_t nd = el[a];
            if (nd >= (uint64_t)nnode) nd = 0;
            X0 = points[nd * 3]; X1 = points[nd * 3 + 1]; X2 = points[nd * 3 + 2];
            x0 = Eulerx[nd * 3]; x1 = Eulerx[nd * 3 + 1]; x2 = Eulerx[nd * 3 + 2];
        };
        double G[9], F[9];
        const double dV = kinematics_fn<NPE>(jm, coords, w[g], 0, G, F);  // w |det dX/dxi|
        const double J = det3(F);
        double trC = 0.0;
        for (int k = 0; k < 9; ++k) trC = fma(F[k], F[k], trC);
        W = (0.5 * mu * (trC - 3.0) - mu * log(J) + 0.5 * lamb * (J - 1.0) * (J - 1.0)) * dV;
    }
    __shared__ double red[4];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) W += __shfl_down_sync(0xffffffffu, W, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = W;
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(energy, red[0] + red[1] + red[2] + red[3]);
}

}  // namespace fl

#define FL_NPE_CASES(MACRO) MACRO(4) MACRO(8) MACRO(10) MACRO(20) MACRO(27) MACRO(35) MACRO(64) MACRO(125)

extern "C" {

int fl_ReferenceGradients(const double *points, const uint64_t *elements, const double *Jm, const double *AllGauss,
                          int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode, float *grad0, float *dV,
                          int *flags, fl_stream_t stream) {
    if (nelem < 0 || ngauss <= 0 || nnode <= 0) return FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!points || !elements || !Jm || !AllGauss || !grad0 || !dV) return FL_ERR_ARG;
    const unsigned grid = (unsigned)((nelem * ngauss + 127) / 128);
    cudaStream_t s = (cudaStream_t)stream;
    switch (nodeperelem) {
#define FL_CASE(N)                                                                                              \
    case N:                                                                                                     \
        fl::ref_grad_kernel<N><<<grid, 128, 0, s>>>(points, elements, Jm, AllGauss, nelem, (int)ngauss, nnode, \
                                                    grad0, dV, flags);                                          \
        break;
        FL_NPE_CASES(FL_CASE)
#undef FL_CASE
        default: return FL_ERR_UNSUPPORTED;
    }
    return fl::launch_status();
}

int fl_InternalForceF32(const uint64_t *elements, const double *u, const float *grad0, const float *dV, int64_t ngauss,
                        int64_t nelem, int64_t nodeperelem, int64_t nnode, int material_number, double mu, double lamb,
                        float *T, int *flags, fl_stream_t stream) {
    if (material_number != FL_MATERIAL_NEOHOOKEAN) return FL_ERR_UNSUPPORTED;
    if (nelem < 0 || ngauss <= 0 || ngauss > 32 || nnode <= 0) return ngauss > 32 ? FL_ERR_UNSUPPORTED : FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!elements || !u || !grad0 || !dV || !T) return FL_ERR_ARG;
    const unsigned grid = (unsigned)((nelem + fl::F32_EPC - 1) / fl::F32_EPC);
    cudaStream_t s = (cudaStream_t)stream;
    switch (nodeperelem) {
#define FL_CASE(N)                                                                                          \
    case N:                                                                                                 \
        fl::internal_force_f32_kernel<N><<<grid, fl::F32_NT, 0, s>>>(elements, u, grad0, dV, nelem,         \
                                                                     (int)ngauss, nnode, (float)mu,         \
                                                                     (float)lamb, T, flags);                \
        break;
        FL_NPE_CASES(FL_CASE)
#undef FL_CASE
        default: return FL_ERR_UNSUPPORTED;
    }
    return fl::launch_status();
}

int fl_ReferenceGradientsPair(const double *points, const uint64_t *elements, const double *Jm,
                              const double *AllGauss, int64_t ngauss, int64_t nelem, int64_t nodeperelem,
                              int64_t nnode, float *grad0_hi, float *grad0_lo, double *dV, int *flags,
                              fl_stream_t stream) {
    if (nelem < 0 || ngauss <= 0 || nnode <= 0) return FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!points || !elements || !Jm || !AllGauss || !grad0_hi || !grad0_lo || !dV) return FL_ERR_ARG;
    const unsigned grid = (unsigned)((nelem * ngauss + 127) / 128);
    cudaStream_t s = (cudaStream_t)stream;
    switch (nodeperelem) {
#define FL_CASE(N)                                                                                             \
    case N:                                                                                                    \
        fl::ref_grad_pair_kernel<N><<<grid, 128, 0, s>>>(points, elements, Jm, AllGauss, nelem, (int)ngauss,  \
                                                         nnode, grad0_hi, grad0_lo, dV, flags);                \
        break;
        FL_NPE_CASES(FL_CASE)
#undef FL_CASE
        default: return FL_ERR_UNSUPPORTED;
    }
    return fl::launch_status();
}

int fl_InternalForcePair(const uint64_t *elements, const double *u, const float *grad0_hi, const float *grad0_lo,
                         const double *dV, int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                         int material_number, double mu, double lamb, double *T, int *flags, fl_stream_t stream) {
    if (material_number != FL_MATERIAL_NEOHOOKEAN) return FL_ERR_UNSUPPORTED;
    if (nelem < 0 || ngauss <= 0 || ngauss > 32 || nnode <= 0) return ngauss > 32 ? FL_ERR_UNSUPPORTED : FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!elements || !u || !grad0_hi || !grad0_lo || !dV || !T) return FL_ERR_ARG;
    const unsigned grid = (unsigned)((nelem + fl::PF_EPC - 1) / fl::PF_EPC);
    cudaStream_t s = (cudaStream_t)stream;
    switch (nodeperelem) {
#define FL_CASE(N)                                                                                          \
    case N:                                                                                                 \
        fl::internal_force_pair_kernel<N><<<grid, fl::PF_NT, 0, s>>>(elements, u, grad0_hi, grad0_lo, dV,   \
                                                                     nelem, (int)ngauss, nnode, mu, lamb,   \
                                                                     T, flags);                             \
        break;
        FL_NPE_CASES(FL_CASE)
#undef FL_CASE
        default: return FL_ERR_UNSUPPORTED;
    }
    return fl::launch_status();
}

int fl_CentralDifferenceUpdate(int64_t n, double dt, const void *T, int T_is_f32, const double *Fext,
                               const double *Minv, const int8_t *fixed, double *u, double *v, fl_stream_t stream) {
    if (n < 0 || !T || !Minv || !fixed || !u || !v) return FL_ERR_ARG;
    if (n == 0) return FL_OK;
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8);
    cudaStream_t s = (cudaStream_t)stream;
    if (T_is_f32) fl::cd_update_kernel<float><<<grid, 256, 0, s>>>(n, dt, (const float *)T, Fext, Minv, fixed, u, v);
    else fl::cd_update_kernel<double><<<grid, 256, 0, s>>>(n, dt, (const double *)T, Fext, Minv, fixed, u, v);
    return fl::launch_status();
}

int fl_StrainEnergy(const double *points, const uint64_t *elements, const double *Eulerx, const double *Jm,
                    const double *AllGauss, int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                    int material_number, double mu, double lamb, double *energy, fl_stream_t stream) {
    if (material_number != FL_MATERIAL_NEOHOOKEAN) return FL_ERR_UNSUPPORTED;
    if (nelem < 0 || ngauss <= 0 || nnode <= 0 || !energy) return FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!points || !elements || !Eulerx || !Jm || !AllGauss) return FL_ERR_ARG;
    const unsigned grid = (unsigned)((nelem * ngauss + 127) / 128);
    cudaStream_t s = (cudaStream_t)stream;
    switch (nodeperelem) {
#define FL_CASE(N)                                                                                               \
    case N:                                                                                                      \
        fl::strain_energy_kernel<N><<<grid, 128, 0, s>>>(points, elements, Eulerx, Jm, AllGauss, nelem,          \
                                                         (int)ngauss, nnode, mu, lamb, energy);                  \
        break;
        FL_NPE_CASES(FL_CASE)
#undef FL_CASE
        default: return FL_ERR_UNSUPPORTED;
    }
    return fl::launch_status();
}

}  // extern "C"
