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
// work. Here every CTA stays resident (cooperative launch, one CTA per SM), an iteration is two
// phases separated by grid barriers, and the dot products go through rotating device slots:
//   phase 1  beta = r.z(k) / r.z(k-1); p_k = z_k + beta p_(k-1) formed on the fly where the
//            product gathers it (and stored by the owner of each node); q = K_ff p_k; p_k.q
//            (8 lanes per node of a node-blocked pattern)
//   phase 2  alpha = r.z / p.q; x += alpha p; r -= alpha q; z = B^-1 r; r.z, r.r  (a thread per node)
//   then     stop when r.r <= rtol^2 b.b
// p alternates between two buffers (iteration k writes p_k while others still gather p_(k-1)).
// Data written by other CTAs inside the launch are read past L1 (ld.global.cg); the barrier is
// an arrival counter (release) and a generation word (acquire). Every barrier wait is bounded: on
// a timeout the kernel records FL_FLAG_TIMEOUT and every CTA leaves.
constexpr int CG_NT = 512;
constexpr int CG_LPN = 8;  // lanes per node in the product
constexpr long long CG_SPIN_LIMIT = 1ll << 24;

struct CgArgs {
    const int32_t *indptr, *indices;
    const double *vals, *Binv, *b;
    const int8_t *fixed;
    double *x, *r, *z, *q;
    double *pb[2];       // p_k in pb[k & 1]
    double *sc;          // [0..2] p.q, [3..5] r.z, [6..8] r.r (rotating by iteration), [9] b.b
    unsigned *bar;       // [0] arrivals, [1] generation
    int *abort_flag;     // set by a CTA whose barrier wait timed out
    int64_t n, maxiter;
    double rtol2;
    int64_t *iters;      // optional: the iteration count is added here
    double *relres;      // optional: |r| / |b| at the end
    int *flags;          // optional: FL_FLAG_TIMEOUT, FL_FLAG_BAD_INDEX (non-positive p.q)
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
    __shared__ double red[CG_NT / 32];
    __shared__ volatile int s_abort;
    const int lane = threadIdx.x & 31;
    const int64_t gt = blockIdx.x * (int64_t)CG_NT + threadIdx.x, nthr = (int64_t)gridDim.x * CG_NT;
    const int64_t gwarp = gt >> 5, nwarps = nthr >> 5;
    const int64_t nnode = a.n / 3;
    unsigned gen = 0;
    if (threadIdx.x == 0) s_abort = 0;
    __syncthreads();
    double *sc = a.sc;
    // r = b, z = B^-1 r, x = 0, p_(-1) = 0 (fixed dofs 0 throughout)
    double rz = 0.0, bb = 0.0;
    for (int64_t m = gt; m < nnode; m += nthr) {
        double rv[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int64_t d = 3 * m + i;
            rv[i] = a.fixed[d] ? 0.0 : a.b[d];
            __stcg(a.r + d, rv[i]);
            __stcg(a.x + d, 0.0);
            __stcg(a.pb[1] + d, 0.0);
            bb = fma(rv[i], rv[i], bb);
        }
        const double *B = a.Binv + m * 9;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int64_t d = 3 * m + i;
            const double zv = a.fixed[d] ? 0.0 : fma(B[3 * i], rv[0], fma(B[3 * i + 1], rv[1], B[3 * i + 2] * rv[2]));
            __stcg(a.z + d, zv);
            rz = fma(rv[i], zv, rz);
        }
    }
    rz = cg_block_sum(rz, red);
    bb = cg_block_sum(bb, red);
    if (threadIdx.x == 0) {
        atomicAdd(sc + 3, rz);
        atomicAdd(sc + 9, bb);
    }
    bool ok = cg_barrier(a, gen, &s_abort);
    const double b2 = __ldcg(sc + 9);
    int64_t k = 0;
    double rr = b2;
    bool bad = false;
    if (b2 > 0.0)
        for (; ok && k < a.maxiter; ++k) {
            const int s0 = (int)(k % 3), s1 = (int)((k + 1) % 3), sm = (int)((k + 2) % 3);  // sm: k - 1
            const double rzk = __ldcg(sc + 3 + s0);
            const double beta = k == 0 ? 0.0 : rzk / __ldcg(sc + 3 + sm);
            const double *pold = a.pb[(k + 1) & 1];
            double *pnew = a.pb[k & 1];
            // phase 1; the slots of the next iteration are cleared
            if (gt == 0) {
                __stcg(sc + s1, 0.0);
                __stcg(sc + 3 + s1, 0.0);
                __stcg(sc + 6 + s1, 0.0);
            }
            // CG_LPN lanes per node, 32 / CG_LPN nodes per warp at once (a coarse node has ~15
            // column blocks: one pass of dependent loads covers the whole product); warp-uniform
            // trip count, so that every lane takes part in the shuffles
            double pq = 0.0;
            for (int64_t base = gwarp * (32 / CG_LPN); base < nnode; base += nwarps * (32 / CG_LPN)) {
                const int64_t m = base + lane / CG_LPN;
                const int sub = lane & (CG_LPN - 1);
                const bool valid = m < nnode;
                const int64_t r0 = 3 * m;
                int j0 = 0, j1 = 0, j2 = 0, nb = 0;
                if (valid) {
                    j0 = a.indptr[r0];
                    j1 = a.indptr[r0 + 1];
                    j2 = a.indptr[r0 + 2];
                    nb = (j1 - j0) / 3;
                }
                double a0 = 0.0, a1 = 0.0, a2 = 0.0;
                for (int blk = sub; blk < nb; blk += CG_LPN) {
                    const int c = a.indices[j0 + 3 * blk];
                    if (c < 0 || c + 2 >= a.n) continue;
                    const double x0 = fma(beta, __ldcg(pold + c), __ldcg(a.z + c));
                    const double x1 = fma(beta, __ldcg(pold + c + 1), __ldcg(a.z + c + 1));
                    const double x2 = fma(beta, __ldcg(pold + c + 2), __ldcg(a.z + c + 2));
                    const double *v0 = a.vals + j0 + 3 * blk, *v1 = a.vals + j1 + 3 * blk, *v2 = a.vals + j2 + 3 * blk;
                    a0 = fma(__ldg(v0), x0, fma(__ldg(v0 + 1), x1, fma(__ldg(v0 + 2), x2, a0)));
                    a1 = fma(__ldg(v1), x0, fma(__ldg(v1 + 1), x1, fma(__ldg(v1 + 2), x2, a1)));
                    a2 = fma(__ldg(v2), x0, fma(__ldg(v2 + 1), x1, fma(__ldg(v2 + 2), x2, a2)));
                }
#pragma unroll
                for (int o = CG_LPN / 2; o > 0; o >>= 1) {
                    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
                    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
                    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
                }
                if (valid && sub < 3) {  // lane sub of the group finishes row 3m + sub
                    const int64_t d = r0 + sub;
                    const double av = sub == 0 ? a0 : sub == 1 ? a1 : a2;
                    const double pv = fma(beta, __ldcg(pold + d), __ldcg(a.z + d));  // 0 on fixed dofs
                    const double qv = a.fixed[d] ? 0.0 : av;
                    __stcg(pnew + d, pv);
                    __stcg(a.q + d, qv);
                    pq = fma(pv, qv, pq);
                }
            }
            pq = cg_block_sum(pq, red);
            if (threadIdx.x == 0) atomicAdd(sc + s0, pq);
            if (!(ok = cg_barrier(a, gen, &s_abort))) break;
            // phase 2
            const double pqk = __ldcg(sc + s0);
            if (!(pqk > 0.0) || !isfinite(pqk)) {  // K_ff not positive definite on p (or no progress)
                bad = true;
                break;
            }
            const double alpha = rzk / pqk;
            double rz1 = 0.0, rr1 = 0.0;
            for (int64_t m = gt; m < nnode; m += nthr) {
                double rv[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int64_t d = 3 * m + i;
                    __stcg(a.x + d, fma(alpha, __ldcg(pnew + d), __ldcg(a.x + d)));
                    rv[i] = fma(-alpha, __ldcg(a.q + d), __ldcg(a.r + d));
                    __stcg(a.r + d, rv[i]);
                    rr1 = fma(rv[i], rv[i], rr1);
                }
                const double *B = a.Binv + m * 9;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int64_t d = 3 * m + i;
                    const double zv =
                        a.fixed[d] ? 0.0 : fma(B[3 * i], rv[0], fma(B[3 * i + 1], rv[1], B[3 * i + 2] * rv[2]));
                    __stcg(a.z + d, zv);
                    rz1 = fma(rv[i], zv, rz1);
                }
            }
            rz1 = cg_block_sum(rz1, red);
            rr1 = cg_block_sum(rr1, red);
            if (threadIdx.x == 0) {
                atomicAdd(sc + 3 + s1, rz1);
                atomicAdd(sc + 6 + s1, rr1);
            }
            if (!(ok = cg_barrier(a, gen, &s_abort))) {
                ++k;
                break;
            }
            rr = __ldcg(sc + 6 + s1);
            if (rr <= a.rtol2 * b2) {
                ++k;
                break;
            }
        }
    if (gt == 0) {
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
    return sizeof(double) * (size_t)(5 * nrows + 16) + 64;
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
    static int per_sm[64] = {}, sms[64] = {};
    int dev = 0;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    if (per_sm[dev & 63] == 0) {
        int coop = 0;
        FL_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) return FL_ERR_UNSUPPORTED;
        FL_CUDA_TRY(cudaDeviceGetAttribute(&sms[dev & 63], cudaDevAttrMultiProcessorCount, dev));
        int b = 0;
        FL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fl::coarse_pcg_kernel, fl::CG_NT, 0));
        per_sm[dev & 63] = std::max(1, b);
    }
    // enough CTAs for a warp per node, at most one per SM: every grid barrier serialises one atomic
    // arrival per CTA, so fewer, larger CTAs make the barriers cheaper (a cooperative launch also
    // needs them all resident, which per_sm >= 1 guarantees)
    const int64_t want = (nrows / 3 + fl::CG_NT / 32 - 1) / (fl::CG_NT / 32);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms[dev & 63]));
    fl::CgArgs a{};
    char *w = (char *)workspace;
    a.sc = (double *)w;
    a.bar = (unsigned *)(w + 16 * sizeof(double));
    a.abort_flag = (int *)(w + 16 * sizeof(double) + 2 * sizeof(unsigned));
    double *v = (double *)(w + 16 * sizeof(double) + 64);
    a.r = v;
    a.z = v + nrows;
    a.pb[0] = v + 2 * nrows;
    a.pb[1] = v + 3 * nrows;
    a.q = v + 4 * nrows;
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
    FL_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)fl::coarse_pcg_kernel, dim3(grid), dim3(fl::CG_NT), args, 0, st));
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
