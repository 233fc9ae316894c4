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
#include <type_traits>

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

// The same product on a node-blocked pattern (the three rows of a node list the same nodes, three
// columns each, as every assembled tangent's pattern does): one warp per node, lanes over its
// column blocks, nine values and one column index per block. x must be zero on fixed dofs (the
// columns are then masked by x itself); fixed rows give 0 (or nothing subtracted from b). With
// FP32 values (a smoother's copy of the tangent) the products and sums run on the FP32 pipe.
template <class VT>
__global__ void __launch_bounds__(MG_NT) masked_spmv_blocks_kernel(const int32_t *indptr, const int32_t *indices,
                                                                   const VT *vals, int64_t nnode,
                                                                   const int8_t *fixed, const double *x,
                                                                   const double *b, double *y, int64_t ncols) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)MG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * MG_NT) >> 5;
    for (int64_t m = warp; m < nnode; m += nwarps) {
        const int64_t r0 = 3 * m;
        const int p0 = indptr[r0], p1 = indptr[r0 + 1], p2 = indptr[r0 + 2];
        const int nb = (p1 - p0) / 3;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        float f0 = 0.f, f1 = 0.f, f2 = 0.f;
        for (int blk = lane; blk < nb; blk += 32) {
            const int c = indices[p0 + 3 * blk];
            if (c < 0 || c + 2 >= ncols) continue;
            const double x0 = x[c], x1 = x[c + 1], x2 = x[c + 2];
            const VT *v0 = vals + p0 + 3 * blk, *v1 = vals + p1 + 3 * blk, *v2 = vals + p2 + 3 * blk;
            if constexpr (std::is_same<VT, float>::value) {  // FP32 values: the sums in FP32 too
                const float y0 = (float)x0, y1 = (float)x1, y2 = (float)x2;
                f0 = fmaf(v0[0], y0, fmaf(v0[1], y1, fmaf(v0[2], y2, f0)));
                f1 = fmaf(v1[0], y0, fmaf(v1[1], y1, fmaf(v1[2], y2, f1)));
                f2 = fmaf(v2[0], y0, fmaf(v2[1], y1, fmaf(v2[2], y2, f2)));
            } else {
                a0 = fma(v0[0], x0, fma(v0[1], x1, fma(v0[2], x2, a0)));
                a1 = fma(v1[0], x0, fma(v1[1], x1, fma(v1[2], x2, a1)));
                a2 = fma(v2[0], x0, fma(v2[1], x1, fma(v2[2], x2, a2)));
            }
        }
        if constexpr (std::is_same<VT, float>::value) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                f0 += __shfl_down_sync(0xffffffffu, f0, o);
                f1 += __shfl_down_sync(0xffffffffu, f1, o);
                f2 += __shfl_down_sync(0xffffffffu, f2, o);
            }
            a0 = f0;
            a1 = f1;
            a2 = f2;
        } else {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a0 += __shfl_down_sync(0xffffffffu, a0, o);
                a1 += __shfl_down_sync(0xffffffffu, a1, o);
                a2 += __shfl_down_sync(0xffffffffu, a2, o);
            }
        }
        if (lane == 0) {
            const double a[3] = {a0, a1, a2};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int64_t row = r0 + i;
                y[row] = fixed[row] ? 0.0 : (b ? b[row] - a[i] : a[i]);
            }
        }
    }
}

// Y = K_ff X for M columns at once (X, Y row-major [nrows][M], FP32; values FP32), node-blocked
// pattern: a warp per node, lanes over columns (M / 32 each), the node's column blocks in turn
// (their nine values broadcast to the warp); X zero on fixed dofs, fixed rows give 0. For
// projections onto a reduced basis, where FP32 products suffice.
template <int M>
__global__ void __launch_bounds__(MG_NT) masked_spmm_blocks_kernel(const int32_t *indptr, const int32_t *indices,
                                                                   const float *vals, int64_t nnode,
                                                                   const int8_t *fixed, const float *X, float *Y,
                                                                   int64_t ncols) {
    constexpr int CPL = M / 32;  // columns per lane
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)MG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * MG_NT) >> 5;
    for (int64_t m = warp; m < nnode; m += nwarps) {
        const int p0 = indptr[3 * m], p1 = indptr[3 * m + 1], p2 = indptr[3 * m + 2];
        const int nb = (p1 - p0) / 3;
        float acc[3][CPL];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < CPL; ++j) acc[i][j] = 0.f;
        for (int blk = 0; blk < nb; ++blk) {
            const int c = indices[p0 + 3 * blk];
            if (c < 0 || c + 2 >= ncols) continue;
            float v[3][3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                v[0][k] = vals[p0 + 3 * blk + k];
                v[1][k] = vals[p1 + 3 * blk + k];
                v[2][k] = vals[p2 + 3 * blk + k];
            }
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                const int col = lane + 32 * j;
                const float x0 = X[(c + 0) * (int64_t)M + col], x1 = X[(c + 1) * (int64_t)M + col],
                            x2 = X[(c + 2) * (int64_t)M + col];
#pragma unroll
                for (int i = 0; i < 3; ++i) acc[i][j] = fmaf(v[i][0], x0, fmaf(v[i][1], x1, fmaf(v[i][2], x2, acc[i][j])));
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int64_t row = 3 * m + i;
            const bool fr = fixed[row] != 0;
#pragma unroll
            for (int j = 0; j < CPL; ++j) Y[row * M + lane + 32 * j] = fr ? 0.f : acc[i][j];
        }
    }
}

// FP64 values or vectors -> float pairs hi + lo (hi = RN(v), lo = RN(v - hi))
__global__ void __launch_bounds__(MG_NT) split_pairs_kernel(int64_t n, const double *v, float2 *out) {
    for (int64_t i = blockIdx.x * (int64_t)MG_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * MG_NT) {
        const double x = v[i];
        const float h = (float)x;
        out[i] = make_float2(h, (float)(x - (double)h));
    }
}

__device__ __forceinline__ void mg_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (s, c) += (vh + vl)(xh + xl): the leading product error-free by FMA, the sum compensated
__device__ __forceinline__ void mg_pair_mac(float2 v, float2 x, float &s, float &c) {
    const float prod = v.x * x.x;
    const float perr = fmaf(v.x, x.x, -prod);
    float t, e;
    mg_two_sum(s, prod, t, e);
    s = t;
    c += e + perr + fmaf(v.x, x.y, v.y * x.x);
}

// The node-block product with the values and x as float pairs (~2^-44 relative), every operation
// on the FP32 pipe: the outer iteration's product, which GB300's FP64 rate (1/64 of FP32) would
// otherwise bound. LPN lanes per node; x zero on fixed dofs, fixed rows give 0.
template <int LPN>
__global__ void __launch_bounds__(MG_NT) masked_spmv_pair_kernel(const int32_t *indptr, const int32_t *indices,
                                                                 const float2 *vals, int64_t nnode,
                                                                 const int8_t *fixed, const float2 *x,
                                                                 const double *b, double *y, int64_t ncols) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)MG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * MG_NT) >> 5;
    for (int64_t base = warp * (32 / LPN); base < nnode; base += nwarps * (32 / LPN)) {  // warp-uniform
        const int64_t m = base + lane / LPN;
        const int sub = lane & (LPN - 1);
        const bool valid = m < nnode;
        float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
        if (valid) {
            const int p0 = indptr[3 * m], p1 = indptr[3 * m + 1], p2 = indptr[3 * m + 2];
            const int nb = (p1 - p0) / 3;
            for (int blk = sub; blk < nb; blk += LPN) {
                const int c = indices[p0 + 3 * blk];
                if (c < 0 || c + 2 >= ncols) continue;
                const float2 x0 = x[c], x1 = x[c + 1], x2 = x[c + 2];
                const float2 *v0 = vals + p0 + 3 * blk, *v1 = vals + p1 + 3 * blk, *v2 = vals + p2 + 3 * blk;
                mg_pair_mac(v0[0], x0, s0, c0); mg_pair_mac(v0[1], x1, s0, c0); mg_pair_mac(v0[2], x2, s0, c0);
                mg_pair_mac(v1[0], x0, s1, c1); mg_pair_mac(v1[1], x1, s1, c1); mg_pair_mac(v1[2], x2, s1, c1);
                mg_pair_mac(v2[0], x0, s2, c2); mg_pair_mac(v2[1], x1, s2, c2); mg_pair_mac(v2[2], x2, s2, c2);
            }
        }
#pragma unroll
        for (int o = LPN / 2; o > 0; o >>= 1) {
            float t, e;
            mg_two_sum(s0, __shfl_xor_sync(0xffffffffu, s0, o), t, e);
            c0 += e + __shfl_xor_sync(0xffffffffu, c0, o);
            s0 = t;
            mg_two_sum(s1, __shfl_xor_sync(0xffffffffu, s1, o), t, e);
            c1 += e + __shfl_xor_sync(0xffffffffu, c1, o);
            s1 = t;
            mg_two_sum(s2, __shfl_xor_sync(0xffffffffu, s2, o), t, e);
            c2 += e + __shfl_xor_sync(0xffffffffu, c2, o);
            s2 = t;
        }
        if (valid && sub < 3) {
            const int64_t row = 3 * m + sub;
            const double a = sub == 0 ? (double)s0 + (double)c0 : sub == 1 ? (double)s1 + (double)c1
                                                                            : (double)s2 + (double)c2;
            y[row] = fixed[row] ? 0.0 : (b ? b[row] - a : a);
        }
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

// ------------------------------------------------------------------------------------------------
// The coarse problem's block-Jacobi PCG in one cooperative launch. The coarse system is small
// (three dofs per mesh vertex) and needs up to a hundred iterations per cycle; as separate
// launches each iteration would cost three kernel boundaries and a host poll, far more than its
// work. Here one CTA per SM stays resident (cooperative launch) and owns a contiguous range of
// nodes: their CSR rows, block inverses and iteration vectors live in its shared memory for the
// whole solve, so that an iteration reads global memory only to gather the neighbours' search
// directions. An iteration is two phases separated by grid barriers, and the dot products go
// through rotating device slots:
//   phase 1  beta = r.z(k) / r.z(k-1); p_k = z_k + beta p_(k-1), formed on the fly where the
//            product gathers it (and stored by each node's owner); q = K_ff p_k; p_k.q
//            (8 lanes per node of a node-blocked pattern)
//   phase 2  alpha = r.z / p.q; x += alpha p; r -= alpha q; z = B^-1 r; r.z, r.r  (a thread per node)
//   then     stop when r.r <= rtol^2 b.b
// p and z are published in global memory for the gathers, p alternating between two buffers
// (iteration k writes p_k while others still gather p_(k-1)); they are read past L1
// (ld.global.cg). The barrier is an arrival counter (release) and a generation word (acquire).
// Every barrier wait is bounded: on a timeout the kernel records FL_FLAG_TIMEOUT and every CTA
// leaves. A CTA whose rows exceed its shared memory makes every CTA leave at once with
// FL_FLAG_CAPACITY (the caller then solves the coarse system another way).
constexpr int CG_NT = 512;
constexpr int CG_LPN = 8;                    // lanes per node in the product
constexpr int CG_SMEM = 200 * 1024;          // dynamic shared memory per CTA
constexpr long long CG_SPIN_LIMIT = 1ll << 24;

struct CgArgs {
    const int32_t *indptr, *indices;
    const double *vals, *Binv, *b;
    const int8_t *fixed;
    double *x, *z;       // z published for the gathers
    double *pb[2];       // p_k published in pb[k & 1]
    double *sc;          // slot s (iteration mod 3) at sc[4 s]: [0] p.q, [2] r.z, [3] r.r; [12] b.b
    unsigned *bar;       // [0] arrivals, [1] generation
    int *abort_flag;     // set by a CTA whose barrier wait timed out
    int *nofit;          // set by a CTA whose rows do not fit its shared memory
    int64_t n, maxiter;
    double rtol2;
    int64_t *iters;      // optional: the iteration count is added here
    double *relres;      // optional: |r| / |b| at the end
    int *flags;          // optional: FL_FLAG_TIMEOUT, FL_FLAG_BAD_INDEX (non-positive p.q), FL_FLAG_CAPACITY
};

__device__ __forceinline__ double cg_block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < CG_NT / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;  // in thread 0
}

// two block sums in one pass (valid in thread 0)
__device__ __forceinline__ void cg_block_sum2(double &u, double &v, double2 *red2) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        u += __shfl_down_sync(0xffffffffu, u, o);
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    if ((threadIdx.x & 31) == 0) red2[threadIdx.x >> 5] = make_double2(u, v);
    __syncthreads();
    if (threadIdx.x < 32) {
        double2 t = threadIdx.x < CG_NT / 32 ? red2[threadIdx.x] : make_double2(0.0, 0.0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            t.x += __shfl_down_sync(0xffffffffu, t.x, o);
            t.y += __shfl_down_sync(0xffffffffu, t.y, o);
        }
        u = t.x;
        v = t.y;
    }
    __syncthreads();
}

__device__ __forceinline__ unsigned cg_arrive(unsigned *count) {
    unsigned old;
    asm volatile("atom.add.release.gpu.u32 %0, [%1], 1;\n" : "=r"(old) : "l"(count) : "memory");
    return old;
}
__device__ __forceinline__ unsigned cg_load_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void cg_store_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// grid barrier; false when a wait timed out here or elsewhere. The CTA's writes before it (ordered
// by bar.sync, then released by thread 0's arrival) are visible to every CTA after it.
__device__ bool cg_barrier(const CgArgs &a, unsigned &gen, volatile int *s_abort) {
    __syncthreads();
    if (threadIdx.x == 0) {
        if (cg_arrive(&a.bar[0]) == gridDim.x - 1) {
            a.bar[0] = 0;                       // ordered before the release below
            cg_store_release(&a.bar[1], gen + 1);
        } else {
            long long t = 0;
            while (cg_load_acquire(&a.bar[1]) == gen) {
                if (++t > CG_SPIN_LIMIT || ((t & 255) == 0 && *(volatile int *)a.abort_flag)) {
                    atomicExch(a.abort_flag, 1);
                    break;
                }
                __nanosleep(20);
            }
        }
        ++gen;
        *s_abort = *(volatile int *)a.abort_flag;
    }
    __syncthreads();
    return *s_abort == 0;
}

__global__ void __launch_bounds__(CG_NT) coarse_pcg_kernel(const CgArgs a) {
    extern __shared__ __align__(16) unsigned char cg_smem[];
    __shared__ double red[CG_NT / 32];
    __shared__ double2 red2[CG_NT / 32];
    __shared__ volatile int s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t nnode = a.n / 3;
    // this CTA's nodes [n0, n1) and their rows [jlo, jhi) of the CSR arrays
    const int64_t M = (nnode + gridDim.x - 1) / gridDim.x;
    const int64_t n0 = min(nnode, (int64_t)blockIdx.x * M), n1 = min(nnode, n0 + M);
    const int cnt = (int)(n1 - n0);
    const int64_t jlo = a.indptr[3 * n0], jhi = a.indptr[3 * n1];
    const int64_t snnz = jhi - jlo;
    // shared memory: own x, r, z, p, q [3M] each, block inverses [9M], row starts [3M] + block
    // counts [M] (ints), the rows' values and column indices [snnz] each
    double *sx = reinterpret_cast<double *>(cg_smem);
    double *sr = sx + 3 * M, *sz = sr + 3 * M, *sp = sz + 3 * M, *sq = sp + 3 * M, *sB = sq + 3 * M;
    double *sv = sB + 9 * M;
    int *si = reinterpret_cast<int *>(sv + snnz);
    int *srow = si + snnz;  // [3M] local row starts, then [M] block counts
    const size_t need = sizeof(double) * (24 * (size_t)M + (size_t)snnz) + sizeof(int) * ((size_t)snnz + 4 * M);
    unsigned gen = 0;
    if (tid == 0) {
        s_abort = 0;
        if (need > (size_t)CG_SMEM || snnz < 0) atomicOr(a.nofit, 1);
    }
    bool ok = cg_barrier(a, gen, &s_abort);
    if (!ok || *(volatile int *)a.nofit) {
        if (blockIdx.x == 0 && tid == 0 && a.flags) atomicOr(a.flags, ok ? FL_FLAG_CAPACITY : FL_FLAG_TIMEOUT);
        return;
    }
    // the CTA's rows, block inverses and row starts into shared memory
    for (int64_t t = tid; t < snnz; t += CG_NT) {
        sv[t] = a.vals[jlo + t];
        si[t] = a.indices[jlo + t];
    }
    for (int t = tid; t < 9 * cnt; t += CG_NT) sB[t] = a.Binv[9 * n0 + t];
    for (int t = tid; t < cnt; t += CG_NT) {
        const int64_t r0 = 3 * (n0 + t);
        const int j0 = (int)(a.indptr[r0] - jlo), j1 = (int)(a.indptr[r0 + 1] - jlo), j2 = (int)(a.indptr[r0 + 2] - jlo);
        srow[3 * t] = j0;
        srow[3 * t + 1] = j1;
        srow[3 * t + 2] = j2;
        srow[3 * M + t] = (j1 - j0) / 3;
    }
    // r = b, z = B^-1 r, x = 0, p_(-1) = 0 (fixed dofs 0 throughout)
    double *sc = a.sc;
    double rz = 0.0, bb = 0.0;
    for (int t = tid; t < cnt; t += CG_NT) {
        const int64_t g0 = 3 * (n0 + t);
        double rv[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            rv[i] = a.fixed[g0 + i] ? 0.0 : a.b[g0 + i];
            sr[3 * t + i] = rv[i];
            sx[3 * t + i] = 0.0;
            sp[3 * t + i] = 0.0;
            __stcg(a.pb[1] + g0 + i, 0.0);
            bb = fma(rv[i], rv[i], bb);
        }
        const double *B = a.Binv + (n0 + t) * 9;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double zv =
                a.fixed[g0 + i] ? 0.0 : fma(B[3 * i], rv[0], fma(B[3 * i + 1], rv[1], B[3 * i + 2] * rv[2]));
            sz[3 * t + i] = zv;
            __stcg(a.z + g0 + i, zv);
            rz = fma(rv[i], zv, rz);
        }
    }
    cg_block_sum2(rz, bb, red2);
    if (tid == 0) {
        atomicAdd(sc + 2, rz);
        atomicAdd(sc + 12, bb);
    }
    ok = cg_barrier(a, gen, &s_abort);
    const double b2 = __ldcg(sc + 12);
    int64_t k = 0;
    double rr = b2;
    double rzk = __ldcg(sc + 2), rz_prev = 1.0;  // r.z of this and the previous iterate, carried along
    bool bad = false;
    if (b2 > 0.0)
        for (; ok && k < a.maxiter; ++k) {
            const int s0 = (int)(k % 3), s1 = (int)((k + 1) % 3);
            const double beta = k == 0 ? 0.0 : rzk / rz_prev;
            const double *pold = a.pb[(k + 1) & 1];
            double *pnew = a.pb[k & 1];
            // phase 1; the slots of the next iteration are cleared
            if (blockIdx.x == 0 && tid == 0) {
                __stcg(sc + 4 * s1, 0.0);
                __stcg(sc + 4 * s1 + 2, 0.0);
                __stcg(sc + 4 * s1 + 3, 0.0);
            }
            double pq = 0.0;
            for (int base = warp * (32 / CG_LPN); base < cnt; base += (CG_NT / 32) * (32 / CG_LPN)) {
                const int ml = base + lane / CG_LPN;  // warp-uniform trip count: every lane shuffles
                const int sub = lane & (CG_LPN - 1);
                const bool valid = ml < cnt;
                const int j0 = valid ? srow[3 * ml] : 0, j1 = valid ? srow[3 * ml + 1] : 0;
                const int j2 = valid ? srow[3 * ml + 2] : 0, nb = valid ? srow[3 * M + ml] : 0;
                double a0 = 0.0, a1 = 0.0, a2 = 0.0;
                for (int blk = sub; blk < nb; blk += CG_LPN) {
                    const int c = si[j0 + 3 * blk];
                    if (c < 0 || c + 2 >= a.n) continue;
                    const double x0 = fma(beta, __ldcg(pold + c), __ldcg(a.z + c));
                    const double x1 = fma(beta, __ldcg(pold + c + 1), __ldcg(a.z + c + 1));
                    const double x2 = fma(beta, __ldcg(pold + c + 2), __ldcg(a.z + c + 2));
                    const double *v0 = sv + j0 + 3 * blk, *v1 = sv + j1 + 3 * blk, *v2 = sv + j2 + 3 * blk;
                    a0 = fma(v0[0], x0, fma(v0[1], x1, fma(v0[2], x2, a0)));
                    a1 = fma(v1[0], x0, fma(v1[1], x1, fma(v1[2], x2, a1)));
                    a2 = fma(v2[0], x0, fma(v2[1], x1, fma(v2[2], x2, a2)));
                }
#pragma unroll
                for (int o = CG_LPN / 2; o > 0; o >>= 1) {
                    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
                    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
                    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
                }
                if (valid && sub < 3) {  // lane sub of the group finishes row 3 ml + sub
                    const int dl = 3 * ml + sub;
                    const int64_t d = 3 * n0 + dl;
                    const double av = sub == 0 ? a0 : sub == 1 ? a1 : a2;
                    const double pv = fma(beta, sp[dl], sz[dl]);  // 0 on fixed dofs
                    const double qv = a.fixed[d] ? 0.0 : av;
                    sp[dl] = pv;
                    sq[dl] = qv;
                    __stcg(pnew + d, pv);
                    pq = fma(pv, qv, pq);
                }
            }
            pq = cg_block_sum(pq, red);
            if (tid == 0) atomicAdd(sc + 4 * s0, pq);
            if (!(ok = cg_barrier(a, gen, &s_abort))) break;
            // phase 2 (own nodes, shared memory; z published)
            const double pqk = __ldcg(sc + 4 * s0);
            if (!(pqk > 0.0) || !isfinite(pqk)) {  // K_ff not positive definite on p (or no progress)
                bad = true;
                break;
            }
            const double alpha = rzk / pqk;
            double rz1 = 0.0, rr1 = 0.0;
            for (int t = tid; t < cnt; t += CG_NT) {
                double rv[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int dl = 3 * t + i;
                    sx[dl] = fma(alpha, sp[dl], sx[dl]);
                    rv[i] = fma(-alpha, sq[dl], sr[dl]);
                    sr[dl] = rv[i];
                    rr1 = fma(rv[i], rv[i], rr1);
                }
                const double *B = sB + 9 * t;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int dl = 3 * t + i;
                    const double zv = a.fixed[3 * n0 + dl]
                                          ? 0.0
                                          : fma(B[3 * i], rv[0], fma(B[3 * i + 1], rv[1], B[3 * i + 2] * rv[2]));
                    sz[dl] = zv;
                    __stcg(a.z + 3 * n0 + dl, zv);
                    rz1 = fma(rv[i], zv, rz1);
                }
            }
            cg_block_sum2(rz1, rr1, red2);
            if (tid == 0) {
                atomicAdd(sc + 4 * s1 + 2, rz1);
                atomicAdd(sc + 4 * s1 + 3, rr1);
            }
            if (!(ok = cg_barrier(a, gen, &s_abort))) {
                ++k;
                break;
            }
            const double2 zr = __ldcg(reinterpret_cast<const double2 *>(sc + 4 * s1 + 2));  // r.z, r.r: one load
            rz_prev = rzk;
            rzk = zr.x;
            rr = zr.y;
            if (rr <= a.rtol2 * b2) {
                ++k;
                break;
            }
        }
    for (int t = tid; t < 3 * cnt; t += CG_NT) a.x[3 * n0 + t] = sx[t];
    if (blockIdx.x == 0 && tid == 0) {
        if (a.iters) atomicAdd((unsigned long long *)a.iters, (unsigned long long)k);
        if (a.relres) *a.relres = b2 > 0.0 ? sqrt(rr / b2) : 0.0;
        if (a.flags && (!ok || bad)) atomicOr(a.flags, !ok ? FL_FLAG_TIMEOUT : FL_FLAG_BAD_INDEX);
    }
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

int fl_MaskedMatVecBlocks(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nrows,
                          const int8_t *fixed, const double *x, const double *b, double *y, fl_stream_t stream) {
    if (nrows < 0 || nrows % 3) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!indptr || !indices || !values || !fixed || !x || !y) return FL_ERR_ARG;
    const int64_t nnode = nrows / 3;
    const int64_t warps = std::min<int64_t>(nnode, (int64_t)152 * 64);
    fl::masked_spmv_blocks_kernel<double><<<fl::grid_of(warps * 32, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        indptr, indices, values, nnode, fixed, x, b, y, nrows);
    return fl::launch_status();
}

int fl_MaskedMatVecBlocksF32(const int32_t *indptr, const int32_t *indices, const float *values, int64_t nrows,
                             const int8_t *fixed, const double *x, const double *b, double *y, fl_stream_t stream) {
    if (nrows < 0 || nrows % 3) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!indptr || !indices || !values || !fixed || !x || !y) return FL_ERR_ARG;
    const int64_t nnode = nrows / 3;
    const int64_t warps = std::min<int64_t>(nnode, (int64_t)152 * 64);
    fl::masked_spmv_blocks_kernel<float><<<fl::grid_of(warps * 32, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        indptr, indices, values, nnode, fixed, x, b, y, nrows);
    return fl::launch_status();
}

int fl_SplitPairs(int64_t n, const double *v, float *pairs, fl_stream_t stream) {
    if (n < 0) return FL_ERR_ARG;
    if (n == 0) return FL_OK;
    if (!v || !pairs) return FL_ERR_ARG;
    const unsigned grid = (unsigned)std::min<int64_t>((n + fl::MG_NT - 1) / fl::MG_NT, 152 * 16);
    fl::split_pairs_kernel<<<grid, fl::MG_NT, 0, (cudaStream_t)stream>>>(n, v, reinterpret_cast<float2 *>(pairs));
    return fl::launch_status();
}

int fl_MaskedMatVecBlocksPair(const int32_t *indptr, const int32_t *indices, const float *value_pairs, int64_t nrows,
                              const int8_t *fixed, const float *x_pairs, const double *b, double *y,
                              fl_stream_t stream) {
    if (nrows < 0 || nrows % 3) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!indptr || !indices || !value_pairs || !fixed || !x_pairs || !y) return FL_ERR_ARG;
    const int64_t nnode = nrows / 3;
    constexpr int LPN = 16;
    const int64_t warps = std::min<int64_t>((nnode + 32 / LPN - 1) / (32 / LPN), (int64_t)152 * 64);
    fl::masked_spmv_pair_kernel<LPN><<<fl::grid_of(warps * 32, fl::MG_NT), fl::MG_NT, 0, (cudaStream_t)stream>>>(
        indptr, indices, reinterpret_cast<const float2 *>(value_pairs), nnode, fixed,
        reinterpret_cast<const float2 *>(x_pairs), b, y, nrows);
    return fl::launch_status();
}

int fl_MaskedMatMatBlocksF32(const int32_t *indptr, const int32_t *indices, const float *values, int64_t nrows,
                             const int8_t *fixed, const float *X, float *Y, int64_t ncolumns, fl_stream_t stream) {
    if (nrows < 0 || nrows % 3) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!indptr || !indices || !values || !fixed || !X || !Y) return FL_ERR_ARG;
    const int64_t nnode = nrows / 3;
    const int64_t warps = std::min<int64_t>(nnode, (int64_t)152 * 64);
    const unsigned grid = fl::grid_of(warps * 32, fl::MG_NT);
    cudaStream_t st = (cudaStream_t)stream;
    switch (ncolumns) {
        case 32: fl::masked_spmm_blocks_kernel<32><<<grid, fl::MG_NT, 0, st>>>(indptr, indices, values, nnode, fixed, X, Y, nrows); break;
        case 64: fl::masked_spmm_blocks_kernel<64><<<grid, fl::MG_NT, 0, st>>>(indptr, indices, values, nnode, fixed, X, Y, nrows); break;
        case 128: fl::masked_spmm_blocks_kernel<128><<<grid, fl::MG_NT, 0, st>>>(indptr, indices, values, nnode, fixed, X, Y, nrows); break;
        default: return FL_ERR_UNSUPPORTED;
    }
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

size_t fl_CoarsePCG_workspace_size(int64_t nrows) {
    if (nrows < 0) return 0;
    return sizeof(double) * (size_t)(3 * nrows + 16) + 64;
}

int fl_CoarsePCG(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nrows,
                 const int8_t *fixed, const double *Binv, const double *b, double *x, double rtol, int64_t maxiter,
                 void *workspace, size_t workspace_bytes, int64_t *iterations, double *relres, int *flags,
                 fl_stream_t stream) {
    if (nrows < 0 || nrows % 3 || maxiter < 0 || !(rtol >= 0.0)) return FL_ERR_ARG;
    if (nrows == 0) return FL_OK;
    if (!indptr || !indices || !values || !fixed || !Binv || !b || !x || !workspace) return FL_ERR_ARG;
    if (workspace_bytes < fl_CoarsePCG_workspace_size(nrows)) return FL_ERR_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    static int sms[64] = {};
    int dev = 0;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    if (sms[dev & 63] == 0) {
        int coop = 0;
        FL_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) return FL_ERR_UNSUPPORTED;
        FL_CUDA_TRY(cudaFuncSetAttribute(fl::coarse_pcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, fl::CG_SMEM));
        int resident = 0;
        FL_CUDA_TRY(
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, fl::coarse_pcg_kernel, fl::CG_NT, fl::CG_SMEM));
        if (resident < 1) return FL_ERR_UNSUPPORTED;
        FL_CUDA_TRY(cudaDeviceGetAttribute(&sms[dev & 63], cudaDevAttrMultiProcessorCount, dev));
    }
    // one CTA per SM (all resident, as a cooperative launch needs; every grid barrier serialises
    // one arrival per CTA), at most one per 16 nodes
    const int64_t want = (nrows / 3 + 15) / 16;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms[dev & 63]));
    fl::CgArgs a{};
    char *w = (char *)workspace;
    a.sc = (double *)w;
    a.bar = (unsigned *)(w + 16 * sizeof(double));
    a.abort_flag = (int *)(w + 16 * sizeof(double) + 2 * sizeof(unsigned));
    a.nofit = (int *)(w + 16 * sizeof(double) + 3 * sizeof(unsigned));
    double *v = (double *)(w + 16 * sizeof(double) + 64);
    a.z = v;
    a.pb[0] = v + nrows;
    a.pb[1] = v + 2 * nrows;
    a.indptr = indptr;
    a.indices = indices;
    a.vals = values;
    a.Binv = Binv;
    a.b = b;
    a.fixed = fixed;
    a.x = x;
    a.n = nrows;
    a.maxiter = maxiter;
    a.rtol2 = rtol * rtol;
    a.iters = iterations;
    a.relres = relres;
    a.flags = flags;
    FL_CUDA_TRY(cudaMemsetAsync(w, 0, 16 * sizeof(double) + 64, st));
    void *args[] = {(void *)&a};
    FL_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)fl::coarse_pcg_kernel, dim3(grid), dim3(fl::CG_NT), args,
                                            fl::CG_SMEM, st));
    return FL_OK;
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
