// fl_mass.cu -- consistent mass matrix on the device: mass_type 1 of the reference's
// _GenericConstantMassIntegrand_ (Florence/VariationalPrinciple/_Mass_/_MassIntegrand_.h:249-400),
// called from __TotalConstantMassIntegrand__ (_MassIntegrand_.pyx:192-348).
//
// The element mass is sum_g rho N_a N_b w_g |det dX/dxi|_g on the nvar diagonal of every node
// pair (a, b) -- the reference's constant integrand rho N N^T expanded by nvar
// (VariationalPrinciple.py:255-290) times its reference-configuration Jacobian -- and it is
// scattered like the reference's fill_global_data (_MassIntegrand_.h:68-178): as triplets in
// element-local order, into CSR through the element-to-nonzero maps, or into CSR by searching each
// row (the squeeze mode).
//
// One CTA per element: the element's coordinates, the Gauss-point weights w|det| and the npe x npe
// node-pair masses are staged in shared memory, then scattered. Node ids and map entries are
// range-checked (FL_FLAG_BAD_INDEX, the entry is skipped).
#include "fl_common.cuh"

namespace fl {

constexpr int CM_NT = 128;

__global__ void __launch_bounds__(CM_NT)
    consistent_mass_kernel(const double *points, const uint64_t *elements, const double *bases, const double *Jm,
                           const double *w, int64_t nelem, int npe, int nq, int nvar, int64_t nnode, double rho,
                           int mode, const int32_t *indptr, const int32_t *indices, int64_t nnz, const int32_t *dl,
                           const int32_t *dg, int32_t *I, int32_t *J, double *V, int *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *X = reinterpret_cast<double *>(smem_raw);  // [npe][3]
    double *wdet = X + 3 * npe;                          // [nq]
    double *Mab = wdet + nq;                             // [npe][npe]
    int64_t *node = reinterpret_cast<int64_t *>(Mab + (size_t)npe * npe);  // [npe], -1 when out of range
    const int ndof = npe * nvar;
    const int64_t cap = (int64_t)ndof * ndof;
    for (int64_t e = blockIdx.x; e < nelem; e += gridDim.x) {
        for (int a = threadIdx.x; a < npe; a += CM_NT) {
            const uint64_t nd = elements[e * npe + a];
            const bool ok = nd < (uint64_t)nnode;
            if (!ok && err) atomicOr(err, FL_FLAG_BAD_INDEX);
            node[a] = ok ? (int64_t)nd : -1;
#pragma unroll
            for (int d = 0; d < 3; ++d) X[a * 3 + d] = ok ? points[nd * 3 + d] : 0.0;
        }
        __syncthreads();
        for (int g = threadIdx.x; g < nq; g += CM_NT) {
            double PX[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int a = 0; a < npe; ++a)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const double j = Jm[((size_t)d * npe + a) * nq + g];
                    PX[d * 3] += j * X[a * 3];
                    PX[d * 3 + 1] += j * X[a * 3 + 1];
                    PX[d * 3 + 2] += j * X[a * 3 + 2];
                }
            wdet[g] = w[g] * fabs(det3(PX));
        }
        __syncthreads();
        for (int p = threadIdx.x; p < npe * npe; p += CM_NT) {
            const int a = p / npe, b = p % npe;
            double m = 0.0;
            for (int g = 0; g < nq; ++g) m += (rho * (bases[(size_t)a * nq + g] * bases[(size_t)b * nq + g])) * wdet[g];
            Mab[p] = m;
        }
        __syncthreads();
        if (mode == 1) {  // triplets, entry e*ndof^2 + r*ndof + c (fill_triplet)
            for (int64_t k = threadIdx.x; k < cap; k += CM_NT) {
                const int r = (int)(k / ndof), c = (int)(k % ndof);
                const int a = r / nvar, i = r % nvar, b = c / nvar, j = c % nvar;
                const int64_t na = node[a] < 0 ? 0 : node[a], nb = node[b] < 0 ? 0 : node[b];
                I[e * cap + k] = (int32_t)(nvar * na + i);
                J[e * cap + k] = (int32_t)(nvar * nb + j);
                V[e * cap + k] = i == j ? Mab[a * npe + b] : 0.0;
            }
        } else if (mode == 0) {  // CSR through the element-to-nonzero maps
            for (int64_t k = threadIdx.x; k < cap; k += CM_NT) {
                const int32_t lk = dl[e * cap + k], pos = dg[e * cap + k];
                if (lk < 0 || lk >= cap || pos < 0 || pos >= nnz) {
                    if (err) atomicOr(err, FL_FLAG_BAD_INDEX);
                    continue;
                }
                const int r = lk / ndof, c = lk % ndof;
                if (r % nvar != c % nvar) continue;  // off the nvar diagonal: zero
                atomicAdd(V + pos, Mab[(r / nvar) * npe + c / nvar]);
            }
        } else {  // CSR, the column searched in each row
            for (int64_t k = threadIdx.x; k < (int64_t)npe * npe * nvar; k += CM_NT) {
                const int p = (int)(k / nvar), i = (int)(k % nvar);
                const int a = p / npe, b = p % npe;
                if (node[a] < 0 || node[b] < 0) continue;
                const int64_t row = nvar * node[a] + i;
                const int32_t col = (int32_t)(nvar * node[b] + i);
                int lo = indptr[row], hi = indptr[row + 1];
                while (lo < hi) {
                    const int mid = lo + (hi - lo) / 2;
                    if (indices[mid] < col) lo = mid + 1;
                    else hi = mid;
                }
                if (lo < indptr[row + 1] && indices[lo] == col) atomicAdd(V + lo, Mab[p]);
                else if (err) atomicOr(err, FL_FLAG_BAD_INDEX);
            }
        }
        __syncthreads();  // shared memory is reused by the next element
    }
}

}  // namespace fl

extern "C" int fl_ConsistentMass(const double *points, const uint64_t *elements, const double *bases,
                                 const double *Jm, const double *AllGauss, int64_t ndim, int64_t nvar,
                                 int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode, double rho,
                                 int recompute_sparsity_pattern, int squeeze_sparsity_pattern, const int32_t *indptr,
                                 const int32_t *indices, int64_t nnz, const int32_t *data_local_indices,
                                 const int32_t *data_global_indices, int32_t *I_mass, int32_t *J_mass,
                                 double *V_mass, int *flags, fl_stream_t stream) {
    if (ndim != 3 || nvar < 1 || nvar > 4) return FL_ERR_ARG;
    if (nelem == 0 && nnode > 0 && ngauss > 0) return FL_OK;  // nothing is read or written
    if (!points || !elements || !bases || !Jm || !AllGauss || !V_mass || nelem < 0 || nnode <= 0 || ngauss <= 0 ||
        nodeperelem <= 0)
        return FL_ERR_ARG;
    int mode;
    if (recompute_sparsity_pattern) {
        if (!I_mass || !J_mass) return FL_ERR_ARG;
        if (nnode * nvar > INT32_MAX) return FL_ERR_UNSUPPORTED;
        mode = 1;
    } else if (squeeze_sparsity_pattern) {
        if (!indptr || !indices) return FL_ERR_ARG;
        mode = 2;
    } else {
        if (!data_local_indices || !data_global_indices || nnz <= 0) return FL_ERR_ARG;
        mode = 0;
    }
    const size_t smem = sizeof(double) * ((size_t)3 * nodeperelem + ngauss + (size_t)nodeperelem * nodeperelem) +
                        sizeof(int64_t) * (size_t)nodeperelem;
    if (smem > 227 * 1024) return FL_ERR_UNSUPPORTED;
    { const int st = fl::ensure_smem<fl::consistent_mass_kernel>(smem); if (st != FL_OK) return st; }
    const unsigned grid = (unsigned)std::min<int64_t>(nelem, 152 * 16);
    fl::consistent_mass_kernel<<<grid, fl::CM_NT, smem, (cudaStream_t)stream>>>(
        points, elements, bases, Jm, AllGauss, nelem, (int)nodeperelem, (int)ngauss, (int)nvar, nnode, rho, mode,
        indptr, indices, nnz, data_local_indices, data_global_indices, I_mass, J_mass, V_mass, flags);
    return fl::launch_status();
}
