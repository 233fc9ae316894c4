// fl_dpf.cu -- global displacement-potential (electromechanics) assembly: the reference's
// _GlobalAssemblyDPF_ (FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDPF_.h:8-198),
// monomorphised for IsotropicElectroMechanics_0, _101, _105, _106, _108, SteinmannModel and Piezoelectric_100 as
// AOT_Assembler.py:125-220 does it, with its
// tangent scattered like fill_global_data (triplets in element-local order, CSR through the
// element-to-nonzero maps, or CSR by row search) and its residual accumulated into T[4 N].
//
// One CTA per element (grid-stride): the element's coordinates and potentials are staged in
// shared memory; a thread per Gauss point computes the spatial gradients, weight, electric
// displacement, stress and 9x9 Hessian (fl_dpf.cuh) into shared memory; then a thread per node
// pair a <= b sums its 4 x 4 tangent block over the Gauss points and scatters it and its mirror
// (CSR positions found once per row of the block, the block's four columns consecutive in a
// node-blocked pattern), and a thread per dof its residual.
// Node ids and map entries are range-checked (FL_FLAG_BAD_INDEX, the entry is skipped);
// det F <= 0 sets FL_FLAG_NONPOSITIVE_J.
#include <algorithm>

#include "fl_common.cuh"
#include "fl_dpf.cuh"

namespace fl {

constexpr int DP_NT = 128;

struct DpfArgs {
    const double *points, *Eulerx, *Eulerp, *Jm, *w;
    const double *orient;  // [nelem * 3] fibre directions (transversely isotropic materials), or null
    const uint64_t *elements;
    int64_t nelem, nnode;
    int npe, nq, update, mode;  // mode 0 CSR through maps, 1 triplets, 2 CSR by row search
    const int32_t *indptr, *indices, *dl, *dg;
    int64_t nnz;
    int32_t *I, *J;
    double *V, *T;
    int *err;
};

// shared-memory doubles per element: X, x [3 npe], phi [npe], node ids [npe], SG [3 npe nq],
// H [81 nq], sigma [9 nq], D [3 nq], dv [nq]
__host__ __device__ inline size_t dpf_smem_doubles(int npe, int nq) {
    return (size_t)8 * npe + (size_t)3 * npe * nq + (size_t)94 * nq;
}

template <class MAT>
__global__ void __launch_bounds__(DP_NT) dpf_kernel(const DpfArgs A, const MAT mat) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int npe = A.npe, nq = A.nq;
    double *X = reinterpret_cast<double *>(smem_raw);
    double *x = X + 3 * npe;
    double *phi = x + 3 * npe;
    int64_t *node = reinterpret_cast<int64_t *>(phi + npe);
    double *SG = reinterpret_cast<double *>(node + npe);
    double *H = SG + (size_t)3 * npe * nq;
    double *sig = H + (size_t)81 * nq;
    double *D = sig + (size_t)9 * nq;
    double *dv = D + (size_t)3 * nq;
    const int ndof = dpf::NV * npe;
    const int64_t cap = (int64_t)ndof * ndof;
    for (int64_t e = blockIdx.x; e < A.nelem; e += gridDim.x) {
        for (int a = threadIdx.x; a < npe; a += DP_NT) {
            const uint64_t nd = A.elements[e * npe + a];
            const bool ok = nd < (uint64_t)A.nnode;
            if (!ok && A.err) atomicOr(A.err, FL_FLAG_BAD_INDEX);
            node[a] = ok ? (int64_t)nd : -1;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                X[a * 3 + d] = ok ? A.points[nd * 3 + d] : 0.0;
                x[a * 3 + d] = ok ? A.Eulerx[nd * 3 + d] : 0.0;
            }
            phi[a] = ok ? A.Eulerp[nd] : 0.0;
        }
        __syncthreads();
        for (int g = threadIdx.x; g < nq; g += DP_NT) {
            const double J = dpf::gauss_point(npe, nq, g, A.Jm, A.w[g], X, x, phi, A.update, mat,
                                              A.orient ? A.orient + 3 * e : nullptr, SG + (size_t)3 * npe * g, dv + g,
                                              D + 3 * g, sig + 9 * g, H + 81 * g);
            if (!(J > 0.0) && A.err) atomicOr(A.err, FL_FLAG_NONPOSITIVE_J);
        }
        __syncthreads();
        // a thread per node pair a <= b: its 4 x 4 block summed over the Gauss points
        // (dpf::pair_block), scattered at (a, v), (b, u) and, for a != b, mirrored to (b, u), (a, v)
        // (the tangent is symmetric)
        const int npairs = npe * (npe + 1) / 2;
        for (int pi = threadIdx.x; pi < npairs; pi += DP_NT) {
            int a = 0, rem = pi;  // node a has npe - a pairs (a, b >= a)
            while (rem >= npe - a) {
                rem -= npe - a;
                ++a;
            }
            const int b = a + rem;
            double B[dpf::NV][dpf::NV];
#pragma unroll
            for (int v = 0; v < dpf::NV; ++v)
#pragma unroll
                for (int u = 0; u < dpf::NV; ++u) B[v][u] = 0.0;
            for (int g = 0; g < nq; ++g)
                dpf::pair_block(a, b, npe, SG + (size_t)3 * npe * g, H + 81 * g, sig + 9 * g, dv[g], B);
            if (A.mode == 1) {  // triplets, entry e*ndof^2 + r*ndof + c
                const int64_t na = node[a] < 0 ? 0 : node[a], nb = node[b] < 0 ? 0 : node[b];
                for (int v = 0; v < dpf::NV; ++v)
                    for (int u = 0; u < dpf::NV; ++u) {
                        const int64_t k1 = (int64_t)(dpf::NV * a + v) * ndof + dpf::NV * b + u;
                        A.I[e * cap + k1] = (int32_t)(dpf::NV * na + v);
                        A.J[e * cap + k1] = (int32_t)(dpf::NV * nb + u);
                        A.V[e * cap + k1] = B[v][u];
                        if (a != b) {
                            const int64_t k2 = (int64_t)(dpf::NV * b + u) * ndof + dpf::NV * a + v;
                            A.I[e * cap + k2] = (int32_t)(dpf::NV * nb + u);
                            A.J[e * cap + k2] = (int32_t)(dpf::NV * na + v);
                            A.V[e * cap + k2] = B[v][u];
                        }
                    }
            } else {  // CSR (maps or row search alike: the block's four columns are found per row)
                if (node[a] < 0 || node[b] < 0) continue;
                for (int side = 0; side < (a != b ? 2 : 1); ++side) {
                    const int64_t nr = side ? node[b] : node[a], nc = side ? node[a] : node[b];
                    for (int v = 0; v < dpf::NV; ++v) {
                        const int64_t row = dpf::NV * nr + v;
                        const int32_t col0 = (int32_t)(dpf::NV * nc);
                        const int r0 = A.indptr[row], r1 = A.indptr[row + 1];
                        int lo = r0, hi = r1;
                        while (lo < hi) {
                            const int mid = lo + (hi - lo) / 2;
                            if (A.indices[mid] < col0) lo = mid + 1;
                            else hi = mid;
                        }
                        for (int u = 0; u < dpf::NV; ++u) {
                            const double val = side ? B[u][v] : B[v][u];
                            const int p = lo + u;
                            if (p < r1 && A.indices[p] == col0 + u) atomicAdd(A.V + p, val);
                            else if (A.err) atomicOr(A.err, FL_FLAG_BAD_INDEX);
                        }
                    }
                }
            }
        }
        if (A.update)
            for (int r = threadIdx.x; r < ndof; r += DP_NT) {
                const int a = r / dpf::NV, v = r % dpf::NV;
                if (node[a] < 0) continue;
                double s = 0.0;
                for (int g = 0; g < nq; ++g)
                    s += dv[g] * dpf::residual(a, v, npe, SG + (size_t)3 * npe * g, D + 3 * g, sig + 9 * g);
                atomicAdd(A.T + dpf::NV * node[a] + v, s);
            }
        __syncthreads();  // shared memory is reused by the next element
    }
}

// the reference's argument list with the material's parameters already taken out of it
template <class MAT>
static int dpf_assemble(const double *points, const uint64_t *elements, const double *Eulerx, const double *Eulerp,
                        const double *Jm, const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss,
                        int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t H_VoigtSize,
                        int64_t requires_geometry_update, int32_t *I_stiff, int32_t *J_stiff, double *V_stiff,
                        double *T, int recompute_sparsity_pattern, int squeeze_sparsity_pattern,
                        const int32_t *data_local_indices, const int32_t *data_global_indices, const MAT &mat,
                        const double *orientations, int *flags, cudaStream_t stream) {
    if (ndim != 3 || nvar != 4 || H_VoigtSize != 9) return FL_ERR_ARG;
    if (nelem == 0 && nnode > 0 && ngauss > 0) return FL_OK;  // nothing is read or written
    if (!points || !elements || !Eulerx || !Eulerp || !Jm || !AllGauss || !V_stiff || !T || nelem < 0 ||
        nnode <= 0 || ngauss <= 0 || nodeperelem <= 0)
        return FL_ERR_ARG;
    DpfArgs A{};
    A.points = points; A.Eulerx = Eulerx; A.Eulerp = Eulerp; A.Jm = Jm; A.w = AllGauss; A.elements = elements;
    A.nelem = nelem; A.nnode = nnode; A.npe = (int)nodeperelem; A.nq = (int)ngauss;
    A.update = requires_geometry_update ? 1 : 0;
    A.V = V_stiff; A.T = T; A.err = flags; A.orient = orientations;
    const int64_t ndof = 4 * nodeperelem;
    if (recompute_sparsity_pattern) {
        if (!I_stiff || !J_stiff) return FL_ERR_ARG;
        if (nnode * 4 > INT32_MAX || ndof * ndof * nelem > ((int64_t)1 << 62)) return FL_ERR_UNSUPPORTED;
        A.mode = 1; A.I = I_stiff; A.J = J_stiff;
    } else if (squeeze_sparsity_pattern) {
        if (!I_stiff || !J_stiff) return FL_ERR_ARG;  // indptr, indices (the reference's I/J slots)
        A.mode = 2; A.indptr = I_stiff; A.indices = J_stiff;
    } else {
        if (!I_stiff || !J_stiff || !data_local_indices || !data_global_indices) return FL_ERR_ARG;
        // the positions the maps name are found in the pattern itself (the same positions)
        A.mode = 0; A.dl = data_local_indices; A.dg = data_global_indices; A.indptr = I_stiff; A.indices = J_stiff;
        int32_t nnz32 = 0;  // indptr[4 N]: the pattern's size, read once
        FL_CUDA_TRY(cudaMemcpyAsync(&nnz32, I_stiff + 4 * nnode, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
        FL_CUDA_TRY(cudaStreamSynchronize(stream));
        A.nnz = nnz32;
    }
    const size_t smem = sizeof(double) * dpf_smem_doubles((int)nodeperelem, (int)ngauss);
    if (smem > 227 * 1024) return FL_ERR_UNSUPPORTED;
    { const int st = ensure_smem<dpf_kernel<MAT>>(smem); if (st != FL_OK) return st; }
    const unsigned grid = (unsigned)std::min<int64_t>(nelem, 152 * 16);
    dpf_kernel<MAT><<<grid, DP_NT, smem, stream>>>(A, mat);
    return launch_status();
}

}  // namespace fl

#define FL_DPF_FORWARD_O(MAT_VALUE, ORIENT)                                                                    \
    fl::dpf_assemble(points, elements, Eulerx, Eulerp, Jm, AllGauss, ndim, nvar, ngauss, nelem, nodeperelem, nnode, \
                     H_VoigtSize, requires_geometry_update, I_stiff, J_stiff, V_stiff, T, recompute_sparsity_pattern, \
                     squeeze_sparsity_pattern, data_local_indices, data_global_indices, MAT_VALUE, ORIENT, flags,   \
                     (cudaStream_t)stream)

#define FL_DPF_FORWARD(MAT_VALUE) FL_DPF_FORWARD_O(MAT_VALUE, nullptr)

// mu1, mu2, lamb, eps_2 (AOT_Assembler.py:167-168, 213-214)
extern "C" int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu; (void)mu3; (void)mue; (void)eps_1; (void)eps_3; (void)eps_e; (void)anisotropic_orientations;
    if (!(eps_2 != 0.0)) return FL_ERR_ARG;
    return FL_DPF_FORWARD((fl::dpf::Em108{mu1, mu2, lamb, eps_2}));
}

// mu, lamb, eps_1 (AOT_Assembler.py:159-160, 204-205)
extern "C" int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_101_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu1; (void)mu2; (void)mu3; (void)mue; (void)eps_2; (void)eps_3; (void)eps_e;
    (void)anisotropic_orientations;
    if (!(eps_1 != 0.0)) return FL_ERR_ARG;
    return FL_DPF_FORWARD((fl::dpf::Em101{mu, lamb, eps_1}));
}

// mu, lamb, eps_1 (AOT_Assembler.py:153-154, 198-199)
extern "C" int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_0_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu1; (void)mu2; (void)mu3; (void)mue; (void)eps_2; (void)eps_3; (void)eps_e;
    (void)anisotropic_orientations;
    return FL_DPF_FORWARD((fl::dpf::Em0{mu, lamb, eps_1}));
}

// mu1, mu2, lamb, eps_1, eps_2 (AOT_Assembler.py:163-164, 208-209)
extern "C" int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_106_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu; (void)mu3; (void)mue; (void)eps_3; (void)eps_e; (void)anisotropic_orientations;
    if (!(eps_1 != 0.0) || !(eps_2 != 0.0)) return FL_ERR_ARG;
    return FL_DPF_FORWARD((fl::dpf::Em106{mu1, mu2, lamb, eps_1, eps_2}));
}

// mu1, mu2, lamb, eps_1, eps_2 (AOT_Assembler.py:161-162, 206-207)
extern "C" int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_105_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu; (void)mu3; (void)mue; (void)eps_3; (void)eps_e; (void)anisotropic_orientations;
    if (!(eps_1 != 0.0) || !(eps_2 != 0.0)) return FL_ERR_ARG;
    return FL_DPF_FORWARD((fl::dpf::Em105{mu1, mu2, lamb, eps_1, eps_2}));
}

// mu, lamb, c1 (in the eps_3 slot), c2 (eps_2), eps_1 (AOT_Assembler.py:157-158, 202-203)
extern "C" int fl_GlobalAssemblyDPF__SteinmannModel_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu1; (void)mu2; (void)mu3; (void)mue; (void)eps_e; (void)anisotropic_orientations;
    return FL_DPF_FORWARD((fl::dpf::EmSteinmann{mu, lamb, eps_3, eps_2, eps_1}));
}

// mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3 and one fibre direction per element in
// anisotropic_orientations [nelem * 3] (AOT_Assembler.py:169-176, 215-220)
extern "C" int fl_GlobalAssemblyDPF__Piezoelectric_100_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements; (void)sorter;
    (void)rho; (void)mu; (void)mue; (void)eps_e;
    if (!anisotropic_orientations || !(eps_1 != 0.0) || !(eps_2 != 0.0) || !(eps_3 > 0.0) || !(mu3 >= 0.0))
        return FL_ERR_ARG;
    return FL_DPF_FORWARD_O((fl::dpf::EmPiezo100{mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3}), anisotropic_orientations);
}
