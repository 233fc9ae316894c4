// fl_multigrid.cu -- the pieces of a two-level p-multigrid preconditioner for Newton's linear step
// on high-order tetrahedra (no reference counterpart: the reference solves the reduced system
// directly or with scipy's iterative solvers, Florence/Solver/LinearSolver.py:153-330).
//
// The coarse space is the linear (p=1) field on the mesh's vertices; a fine node's value is the
// interpolation of its element's vertex values at its barycentric coordinates. Both transfers are
// one node-level sparse product with per-entry weights, applied to the three components:
//     prolongation  u_f[3n + i] = sum_k w[k] u_c[3 col[k] + i],  k over fine node n's row
//     restriction   r_c[3v + i] = sum_k w[k] r_f[3 col[k] + i],  k over coarse node v's row
// (the restriction's rows are the transpose of the prolongation's, built once per mesh, so both
// run as gathers without atomics). The fine-level smoother needs the tangent's product with the
// Dirichlet dofs masked (the system K_ff that Newton solves) and the 3x3 nodal block-Jacobi
// inverse, the same blocks the device PCG uses.
#include <algorithm>

#include "fl_common.cuh"

namespace fl {

constexpr int MG_NT = 256;

__global__ void __launch_bounds__(MG_NT) nodal_transfer_kernel(int64_t nrows, const int32_t *ptr, const int32_t *cols,
                                                               const double *w, const double *x, double *y,
                                                               int accumulate) {
    const int64_t r = blockIdx.x * (int64_t)MG_NT + threadIdx.x;
    if (r >= nrows) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
        const int64_t c = 3 * (int64_t)cols[k];
        const double wk = w[k];
        s0 = fma(wk, x[c], s0);
        s1 = fma(wk, x[c + 1], s1);
        s2 = fma(wk, x[c + 2], s2);
    }
    if (accumulate) {
        y[3 * r] += s0;
        y[3 * r + 1] += s1;
        y[3 * r + 2] += s2;
    } else {
        y[3 * r] = s0;
        y[3 * r + 1] = s1;
        y[3 * r + 2] = s2;
    }
}

// y = K_ff x: one warp per row, fixed rows 0 and fixed columns skipped; y = b - K_ff x when b is
// given (the residual form the smoother and the restriction use)
__global__ void __launch_bounds__(MG_NT) masked_spmv_kernel(const int32_t *indptr, const int32_t *indices,
                                                            const double *vals, int64_t n, const int8_t *fixed,
                                                            const double *x, const double *b, double *y) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)MG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * MG_NT) >> 5;
    for (int64_t row = warp; row < n; row += nwarps) {
        double acc = 0.0;
        if (!fixed[row])
            for (int k = indptr[row] + lane; k < indptr[row + 1]; k += 32) {
                const int c = indices[k];
                if (!fixed[c]) acc = fma(vals[k], x[c], acc);
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) y[row] = fixed[row] ? 0.0 : (b ? b[row] - acc : acc);
    }
}

// z (+)= omega B^-1 r per node; fixed dofs of z set to 0
__global__ void __launch_bounds__(MG_NT) block_apply_kernel(int64_t nnode, const double *Binv, const int8_t *fixed,
                                                            double omega, const double *r, double *z, int accumulate) {
    const int64_t m = blockIdx.x * (int64_t)MG_NT + threadIdx.x;
    if (m >= nnode) return;
    const double r0 = r[3 * m], r1 = r[3 * m + 1], r2 = r[3 * m + 2];
    const double *B = Binv + m * 9;
    const double v[3] = {fma(B[0], r0, fma(B[1], r1, B[2] * r2)), fma(B[3], r0, fma(B[4], r1, B[5] * r2)),
                         fma(B[6], r0, fma(B[7], r1, B[8] * r2))};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int64_t d = 3 * m + i;
        const double add = fixed[d] ? 0.0 : omega * v[i];
        z[d] = accumulate && !fixed[d] ? z[d] + add : add;
    }
}

// inverse of the 3x3 diagonal block of each node, fixed rows/columns replaced by the identity
__global__ void __launch_bounds__(MG_NT) block_inverse_kernel(const int32_t *indptr, const int32_t *indices,
                                                              const double *vals, const int8_t *fixed, int64_t nnode,
                                                              double *Binv, int *flags) {
    const int64_t m = blockIdx.x * (int64_t)MG_NT + threadIdx.x;
    if (m >= nnode) return;
    double B[9];
    for (int i = 0; i < 3; ++i) {
        const int64_t row = 3 * m + i;
        int lo = indptr[row], hi = indptr[row + 1];
        const int c0 = (int)(3 * m);
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (indices[mid] < c0) lo = mid + 1; else hi = mid;
        }
        for (int j = 0; j < 3; ++j) {
            const int pos = lo + j;
            const bool ok = pos < indptr[row + 1] && indices[pos] == c0 + j;
            if (!ok && flags) atomicOr(flags, FL_FLAG_BAD_INDEX);
            B[i * 3 + j] = ok ? vals[pos] : 0.0;
        }
    }
    for (int i = 0; i < 3; ++i)
        if (fixed[3 * m + i])
            for (int j = 0; j < 3; ++j) B[i * 3 + j] = B[j * 3 + i] = (i == j) ? 1.0 : 0.0;
    double R[9];
    const double det = inv3(B, R);
    if (!(fabs(det) > 0.0) || !isfinite(det)) {
        if (flags) atomicOr(flags, FL_FLAG_BAD_INDEX);
        for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }
    for (int k = 0; k < 9; ++k) Binv[m * 9 + k] = R[k];
}

static unsigned grid_of(int64_t n, int per_block) {
    return (unsigned)std::max<int64_t>(1, (n + per_block - 1) / per_block);
}

}  // namespace fl

extern "C" {

int fl_NodalTransfer(int64_t nrows, const int32_t *ptr, const int32_t *cols, const double *weights, const double *x,
                     double *y, int accumulate, fl_stream_t stream) {
    if (nrows < 0) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!ptr || !cols || !weights || !x || !y) return FL_ERR_ARG;
    fl::nodal_transfer_kernel<<<fl::grid_of(nrows, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        nrows, ptr, cols, weights, x, y, accumulate);
    return fl::launch_status();
}

int fl_MaskedMatVec(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nrows,
                    const int8_t *fixed, const double *x, const double *b, double *y, fl_stream_t stream) {
    if (nrows < 0) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!indptr || !indices || !values || !fixed || !x || !y) return FL_ERR_ARG;
    const int64_t warps = std::min<int64_t>(nrows, (int64_t)152 * 64);
    fl::masked_spmv_kernel<<<fl::grid_of(warps * 32, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        indptr, indices, values, nrows, fixed, x, b, y);
    return fl::launch_status();
}

int fl_BlockJacobiInverse(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nnode,
                          const int8_t *fixed, double *Binv, int *flags, fl_stream_t stream) {
    if (nnode < 0) return FL_ERR_ARG;
    if (nnode == 0) return FL_OK;
    if (!indptr || !indices || !values || !fixed || !Binv) return FL_ERR_ARG;
    fl::block_inverse_kernel<<<fl::grid_of(nnode, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        indptr, indices, values, fixed, nnode, Binv, flags);
    return fl::launch_status();
}

int fl_BlockJacobiApply(int64_t nnode, const double *Binv, const int8_t *fixed, double omega, const double *r,
                        double *z, int accumulate, fl_stream_t stream) {
    if (nnode < 0) return FL_ERR_ARG;
    if (nnode == 0) return FL_OK;
    if (!Binv || !fixed || !r || !z) return FL_ERR_ARG;
    fl::block_apply_kernel<<<fl::grid_of(nnode, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        nnode, Binv, fixed, omega, r, z, accumulate);
    return fl::launch_status();
}

}  // extern "C"
