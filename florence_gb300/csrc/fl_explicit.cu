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
    FL_CUDA_TRY(cudaFuncSetAttribute(internal_force_kernel<NPE, MAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
    (void)Eulerp; (void)bases; (void)H_VoigtSize; (void)requires_geometry_update; (void)rho; (void)mu3; (void)mue;
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
    FL_CUDA_TRY(cudaFuncSetAttribute(fl::lumped_mass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t grid = (nelem + fl::LM_EPC - 1) / fl::LM_EPC;
    if (grid == 0) return FL_OK;
    fl::lumped_mass_kernel<<<(unsigned)grid, fl::LM_NT, smem, (cudaStream_t)stream>>>(
        points, elements, bases, Jm, AllGauss, nelem, (int)nodeperelem, (int)ngauss, nnode, rho, M, flags);
    return fl::launch_status();
}

}  // extern "C"
