// fl_pcg.cu -- Newton's linear step on the device: FP64 conjugate gradients on the assembled CSR
// tangent with a 3x3 nodal block-Jacobi preconditioner and Dirichlet dofs masked out (the
// reference reduces the system by slicing the CSR matrix, BoundaryCondition.GetReducedMatrices,
// Florence/BoundaryCondition/BoundaryCondition.py:842-857, then calls a direct solver,
// Florence/Solver/LinearSolver.py:208-330).
//
// Masking instead of slicing: the iteration vectors are zero on fixed dofs, the matrix-vector
// product zeroes fixed rows, and the preconditioner block of a node with fixed dofs has those
// rows and columns replaced by the identity. This is CG on the reduced system K_ff, with the
// matrix left as assembled.
//
// With the float-pair products (split FP64 values, or FP32 values) the iteration vectors x, r, z, p
// and the block inverses are float pairs as well (pcg_k2_pair, pcg_k3_pair), converted from and
// to FP64 once per solve.
//
// One iteration = three kernels:
//   K1  q = K p, p.q
//   K2  alpha = rz_k / p.q;  x += alpha p;  r -= alpha q;  z = B^-1 r;  r.z and r.r
//   K3  beta = rz_{k+1} / rz_k;  p = z + beta p;  convergence test, done flag
// Matrix values: FP64 (FP64 products), FP32 (an inexact-Newton Jacobian) or FP64 split once per
// solve into float pairs hi + lo in the workspace (FL_PCG_F64_SPLIT): the product then runs on
// the FP32 pipe in float-pair arithmetic (~2^-44 relative), which GB300's FP64 rate (1/64 of its
// FP32 rate) would otherwise bound.
// The product K p reads the matrix as 3x3 node blocks when the pattern has the structure every
// assembled tangent has (the three rows of a node list the same nodes, 3 columns each): one warp
// per node row, lanes over neighbour nodes, 9 values and one column index per block, so the
// column indices of two of the three rows are never read. Other patterns use one warp per row.
// Dot products are block-reduced and added into device scalar slots with one FP64 atomic per
// block; the scalars never travel to the host inside the iteration (kernels read them from the
// slots), and the host checks the done flag every PCG_CHECK iterations.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "fl_common.cuh"

namespace fl {

constexpr int PCG_NT = 256;
constexpr int PCG_CHECK = 16;

struct PcgState {
    double *r, *z, *p, *q, *Binv;  // vectors [n], block inverses [n/3][9]
    float *ph, *pl;                // p as a float pair (p ~ ph + pl), for the float-pair products
    float *qh, *ql;                // q = K p as a float pair, written by the float-pair products
    double *acc;                   // [0] p.q, [1],[2] r.z of even/odd iterates, [3] r.r, [4] |b|^2
    int *done;                     // [0] done flag, [1] iterations at convergence, [2] error bits,
                                   // [3] the iteration index k (advanced by pcg_tail)
    // float-pair iteration vectors (with the float-pair products): x, r, z as hi/lo floats [n],
    // the block inverses as hi/lo floats [n/3][9]
    float *xh, *xl, *rh, *rl, *zh, *zl, *Bh, *Bl;
};

static size_t pcg_layout(int64_t n, int64_t nnz, PcgState *s, char *base, float2 **vsplit = nullptr) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    PcgState t;
    t.r = (double *)take(sizeof(double) * n);
    t.z = (double *)take(sizeof(double) * n);
    t.p = (double *)take(sizeof(double) * n);
    t.q = (double *)take(sizeof(double) * n);
    t.Binv = (double *)take(sizeof(double) * (n / 3) * 9);
    t.ph = (float *)take(sizeof(float) * n);
    t.pl = (float *)take(sizeof(float) * n);
    t.qh = (float *)take(sizeof(float) * n);
    t.ql = (float *)take(sizeof(float) * n);
    t.xh = (float *)take(sizeof(float) * n);
    t.xl = (float *)take(sizeof(float) * n);
    t.rh = (float *)take(sizeof(float) * n);
    t.rl = (float *)take(sizeof(float) * n);
    t.zh = (float *)take(sizeof(float) * n);
    t.zl = (float *)take(sizeof(float) * n);
    t.Bh = (float *)take(sizeof(float) * (n / 3) * 9);
    t.Bl = (float *)take(sizeof(float) * (n / 3) * 9);
    t.acc = (double *)take(sizeof(double) * 8);
    t.done = (int *)take(sizeof(int) * 4);
    float2 *vs = (float2 *)take(sizeof(float2) * (size_t)nnz);
    if (vsplit) *vsplit = vs;
    if (s) *s = t;
    return off;
}

// p as a float pair
__device__ __forceinline__ void split_store(const PcgState &s, int64_t d, double v) {
    const float h = (float)v;
    s.ph[d] = h;
    s.pl[d] = (float)(v - (double)h);
}

// Block sum of one value per thread, added to *out with one atomic.
__device__ __forceinline__ void block_atomic_add(double v, double *out) {
    __shared__ double red[PCG_NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double w = threadIdx.x < PCG_NT / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
        if (threadIdx.x == 0) atomicAdd(out, w);
    }
    __syncthreads();
}

// 3x3 diagonal block of node m, fixed rows/columns replaced by the identity, inverted.
template <class VT>
__global__ void __launch_bounds__(PCG_NT) bj_setup(const int32_t *indptr, const int32_t *indices, const VT *vals,
                                                   const int8_t *fixed, int64_t nnode, double *Binv, int *err) {
    for (int64_t m = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; m < nnode; m += (int64_t)gridDim.x * PCG_NT) {
        double B[9];
        for (int i = 0; i < 3; ++i) {
            const int64_t row = 3 * m + i;
            int lo = indptr[row], hi = indptr[row + 1];
            const int c0 = (int)(3 * m);
            // first entry >= c0
            while (lo < hi) {
                const int mid = lo + (hi - lo) / 2;
                if (indices[mid] < c0) lo = mid + 1; else hi = mid;
            }
            for (int j = 0; j < 3; ++j) {
                const int pos = lo + j;
                double v = 0.0;
                if (pos < indptr[row + 1] && indices[pos] == c0 + j) v = (double)vals[pos];
                else atomicOr(err, 1);  // diagonal block entry missing from the pattern
                B[i * 3 + j] = v;
            }
        }
        for (int i = 0; i < 3; ++i)
            if (fixed[3 * m + i])
                for (int j = 0; j < 3; ++j) B[i * 3 + j] = B[j * 3 + i] = (i == j) ? 1.0 : 0.0;
        double R[9];
        const double det = inv3(B, R);
        if (!(fabs(det) > 0.0) || !isfinite(det)) {
            atomicOr(err, 2);
            for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.0 : 0.0;
        }
        for (int k = 0; k < 9; ++k) Binv[m * 9 + k] = R[k];
    }
}

// r = mask(b - K x), z = B^-1 r, p = z, partials of r.z (rz[0]) and |b|^2
template <class VT>
__global__ void __launch_bounds__(PCG_NT) pcg_init(const int32_t *indptr, const int32_t *indices, const VT *vals,
                                                   const int8_t *fixed, const double *b, const double *x, int64_t n,
                                                   PcgState s) {
    // (1) r = b - K x with one warp per row
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)PCG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * PCG_NT) >> 5;
    double bb = 0.0;
    for (int64_t row = warp; row < n; row += nwarps) {
        double acc = 0.0;
        for (int k = indptr[row] + lane; k < indptr[row + 1]; k += 32) acc = fma((double)vals[k], x[indices[k]], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            const double bi = fixed[row] ? 0.0 : b[row];
            s.r[row] = fixed[row] ? 0.0 : bi - acc;
            bb = fma(bi, bi, bb);
        }
    }
    block_atomic_add(bb, s.acc + 4);
}

// z = B^-1 r, p = z, partial r.z  (after pcg_init's r is complete)
__global__ void __launch_bounds__(PCG_NT) pcg_init2(int64_t nnode, PcgState s) {
    double rz = 0.0;
    for (int64_t m = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; m < nnode; m += (int64_t)gridDim.x * PCG_NT) {
        const double r0 = s.r[3 * m], r1 = s.r[3 * m + 1], r2 = s.r[3 * m + 2];
        const double *B = s.Binv + m * 9;
        const double z0 = fma(B[0], r0, fma(B[1], r1, B[2] * r2));
        const double z1 = fma(B[3], r0, fma(B[4], r1, B[5] * r2));
        const double z2 = fma(B[6], r0, fma(B[7], r1, B[8] * r2));
        s.z[3 * m] = s.p[3 * m] = z0;
        s.z[3 * m + 1] = s.p[3 * m + 1] = z1;
        s.z[3 * m + 2] = s.p[3 * m + 2] = z2;
        split_store(s, 3 * m, z0);
        split_store(s, 3 * m + 1, z1);
        split_store(s, 3 * m + 2, z2);
        rz = fma(r0, z0, fma(r1, z1, fma(r2, z2, rz)));
    }
    block_atomic_add(rz, s.acc + 1);
}

// Node-block product with NB lanes per node (32 / NB nodes per warp; NB = 4, 8, 16 or 32,
// chosen per matrix by timing, pick_lanes): lanes over neighbour slots s,
// m = indices[indptr[3n] + 3s] / 3, values V[indptr[3n+i] + 3s + j]; the NB partial sums are
// combined with log2(NB) shuffle steps. FP64 values: FP64 products (node_block_row). FP32 values
// and split FP64 values: each product and sum is carried as an unevaluated float pair
// (error-free product by FMA, compensated two-sum), with p given as a float pair too, so the
// matrix is applied to ~2^-44 relative accuracy while every operation runs on the FP32 pipe
// (node_block_pair; GB300's FP64 rate would otherwise bound this loop).

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (s, c) += v * (ph + pl)
__device__ __forceinline__ void df_mac(float v, float ph, float pl, float &s, float &c) {
    const float prod = v * ph;
    const float perr = fmaf(v, ph, -prod);
    float t, e;
    two_sum(s, prod, t, e);
    s = t;
    c += e + fmaf(v, pl, perr);
}

template <int NB>
__device__ __forceinline__ void node_block_row(const int32_t *indptr, const int32_t *indices, const double *vals,
                                               const PcgState &st, int64_t node, bool valid, int sub, double &y0,
                                               double &y1, double &y2) {
    y0 = y1 = y2 = 0.0;
    if (valid) {
        const int r0 = indptr[3 * node], r1 = indptr[3 * node + 1], r2 = indptr[3 * node + 2];
        const int nb = (r1 - r0) / 3;
        for (int sl = sub; sl < nb; sl += NB) {
            const int m3 = indices[r0 + 3 * sl];
            const double x0 = st.p[m3], x1 = st.p[m3 + 1], x2 = st.p[m3 + 2];
            const double *v0 = vals + r0 + 3 * sl, *v1 = vals + r1 + 3 * sl, *v2 = vals + r2 + 3 * sl;
            y0 = fma(v0[0], x0, fma(v0[1], x1, fma(v0[2], x2, y0)));
            y1 = fma(v1[0], x0, fma(v1[1], x1, fma(v1[2], x2, y1)));
            y2 = fma(v2[0], x0, fma(v2[1], x1, fma(v2[2], x2, y2)));
        }
    }
#pragma unroll
    for (int o = NB / 2; o > 0; o >>= 1) {
        y0 += __shfl_down_sync(0xffffffffu, y0, o, NB);
        y1 += __shfl_down_sync(0xffffffffu, y1, o, NB);
        y2 += __shfl_down_sync(0xffffffffu, y2, o, NB);
    }
}

// (s, c) += (vh + vl) * (ph + pl), dropping vl*pl (2^-48 relative)
__device__ __forceinline__ void df_mac2(float2 v, float ph, float pl, float &s, float &c) {
    const float prod = v.x * ph;
    const float perr = fmaf(v.x, ph, -prod);
    float t, e;
    two_sum(s, prod, t, e);
    s = t;
    c += e + fmaf(v.x, pl, fmaf(v.y, ph, perr));
}

__device__ __forceinline__ void pair_mac(float v, float ph, float pl, float &s, float &c) { df_mac(v, ph, pl, s, c); }
__device__ __forceinline__ void pair_mac(float2 v, float ph, float pl, float &s, float &c) { df_mac2(v, ph, pl, s, c); }

// Node-block product rows of node `node` as unevaluated float pairs (s_i + c_i), summed over the
// NB lanes of the group; lane sub == 0 holds the totals. No FP64 instruction: on GB300 each one
// occupies the FP64 pipe for a whole warp, even with one lane active.
template <int NB, class VT>
__device__ __forceinline__ void node_block_pair(const int32_t *indptr, const int32_t *indices, const VT *vals,
                                                const PcgState &st, int64_t node, bool valid, int sub, float *sh,
                                                float *sc) {
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
    if (valid) {
        const int r0 = indptr[3 * node], r1 = indptr[3 * node + 1], r2 = indptr[3 * node + 2];
        const int nb = (r1 - r0) / 3;
        for (int sl = sub; sl < nb; sl += NB) {
            const int m3 = indices[r0 + 3 * sl];
            const float h0 = st.ph[m3], h1 = st.ph[m3 + 1], h2 = st.ph[m3 + 2];
            const float l0 = st.pl[m3], l1 = st.pl[m3 + 1], l2 = st.pl[m3 + 2];
            const VT *v0 = vals + r0 + 3 * sl, *v1 = vals + r1 + 3 * sl, *v2 = vals + r2 + 3 * sl;
            pair_mac(v0[0], h0, l0, s0, c0); pair_mac(v0[1], h1, l1, s0, c0); pair_mac(v0[2], h2, l2, s0, c0);
            pair_mac(v1[0], h0, l0, s1, c1); pair_mac(v1[1], h1, l1, s1, c1); pair_mac(v1[2], h2, l2, s1, c1);
            pair_mac(v2[0], h0, l0, s2, c2); pair_mac(v2[1], h1, l1, s2, c2); pair_mac(v2[2], h2, l2, s2, c2);
        }
    }
#pragma unroll
    for (int o = NB / 2; o > 0; o >>= 1) {
        float t, e;
        two_sum(s0, __shfl_down_sync(0xffffffffu, s0, o, NB), t, e);
        c0 += e + __shfl_down_sync(0xffffffffu, c0, o, NB);
        s0 = t;
        two_sum(s1, __shfl_down_sync(0xffffffffu, s1, o, NB), t, e);
        c1 += e + __shfl_down_sync(0xffffffffu, c1, o, NB);
        s1 = t;
        two_sum(s2, __shfl_down_sync(0xffffffffu, s2, o, NB), t, e);
        c2 += e + __shfl_down_sync(0xffffffffu, c2, o, NB);
        s2 = t;
    }
    sh[0] = s0; sh[1] = s1; sh[2] = s2;
    sc[0] = c0; sc[1] = c1; sc[2] = c2;
}

__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(float v) { return (double)v; }
__device__ __forceinline__ double to_d(float2 v) { return (double)v.x + (double)v.y; }

// FP64 values -> float pairs hi + lo (hi = RN(v), lo = RN(v - hi)), nnz = indptr[n]
__global__ void __launch_bounds__(PCG_NT) split_values(const int32_t *indptr, int64_t n, const double *v,
                                                       float2 *out) {
    const int64_t nnz = indptr[n];
    for (int64_t i = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * PCG_NT) {
        const double x = v[i];
        const float h = (float)x;
        out[i] = make_float2(h, (float)(x - (double)h));
    }
}

// pattern check for the node-block product: rows 3n, 3n+1, 3n+2 hold the same columns, in runs
// 3m, 3m+1, 3m+2 (one warp per node)
__global__ void pcg_check_blocks(const int32_t *indptr, const int32_t *indices, int64_t nnode, int *bad) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t m = warp; m < nnode; m += nwarps) {
        const int r0 = indptr[3 * m], r1 = indptr[3 * m + 1], r2 = indptr[3 * m + 2], r3 = indptr[3 * m + 3];
        const int l0 = r1 - r0;
        bool ok = (r2 - r1 == l0) && (r3 - r2 == l0) && (l0 % 3 == 0);
        if (ok)
            for (int t = lane; t < l0; t += 32) {
                const int c = indices[r0 + t];
                ok = ok && (indices[r1 + t] == c) && (indices[r2 + t] == c) && (c % 3 == t % 3) &&
                     (t % 3 == 0 || indices[r0 + t - 1] == c - 1);
            }
        if (!ok) atomicOr(bad, 8);
    }
}

// Dot products of the iteration are accumulated with one FP64 atomic add per block into scalar
// slots: acc[0] = p.q, acc[1 + (k & 1)] = r.z of iterate k (double-buffered), acc[3] = r.r.
// Each kernel zeroes the slot the next kernel accumulates into, after every reader is done.

// K1: q = mask(K p), p.q; zeroes r.z of iterate k+1 and r.r for K2
template <class VT, bool NODEBLK, int NB = 8>
__global__ void __launch_bounds__(PCG_NT) pcg_k1(const int32_t *indptr, const int32_t *indices, const VT *vals,
                                                 const int8_t *fixed, int64_t n, PcgState s) {
    if (s.done[0]) return;
    const int k = s.done[3];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s.acc[1 + ((k + 1) & 1)] = 0.0;
        s.acc[3] = 0.0;
    }
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)PCG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * PCG_NT) >> 5;
    double pq = 0.0;
    constexpr bool PAIR = !std::is_same<VT, double>::value;
    if constexpr (NODEBLK && PAIR) {  // float-pair products: q and p.q stay float pairs (FP32 pipe only)
        const int grp = lane / NB, sub = lane % NB;
        const int64_t nnode = n / 3;
        float pqs = 0.f, pqc = 0.f;
        for (int64_t base = warp * (32 / NB); base < nnode; base += nwarps * (32 / NB)) {
            const int64_t m = base + grp;
            float sh[3], sc[3];
            node_block_pair<NB>(indptr, indices, vals, s, m, m < nnode, sub, sh, sc);
            if (sub == 0 && m < nnode) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int64_t d = 3 * m + i;
                    float h = 0.f, l = 0.f;
                    if (!fixed[d]) {  // renormalised pair
                        h = sh[i] + sc[i];
                        l = sc[i] - (h - sh[i]);
                    }
                    s.qh[d] = h;
                    s.ql[d] = l;
                    df_mac2(make_float2(h, l), s.ph[d], s.pl[d], pqs, pqc);
                }
            }
        }
        pq = (double)pqs + (double)pqc;  // once per thread
    } else if constexpr (NODEBLK) {
        const int grp = lane / NB, sub = lane % NB;
        const int64_t nnode = n / 3;
        for (int64_t base = warp * (32 / NB); base < nnode; base += nwarps * (32 / NB)) {
            const int64_t m = base + grp;
            double y0, y1, y2;
            node_block_row<NB>(indptr, indices, vals, s, m, m < nnode, sub, y0, y1, y2);
            if (sub == 0 && m < nnode) {
                const double q0 = fixed[3 * m] ? 0.0 : y0, q1 = fixed[3 * m + 1] ? 0.0 : y1,
                             q2 = fixed[3 * m + 2] ? 0.0 : y2;
                s.q[3 * m] = q0;
                s.q[3 * m + 1] = q1;
                s.q[3 * m + 2] = q2;
                pq = fma(s.p[3 * m], q0, fma(s.p[3 * m + 1], q1, fma(s.p[3 * m + 2], q2, pq)));
            }
        }
    } else {
        for (int64_t row = warp; row < n; row += nwarps) {
            double acc = 0.0;
            const int end = indptr[row + 1];
            for (int kk = indptr[row] + lane; kk < end; kk += 32) acc = fma(to_d(vals[kk]), s.p[indices[kk]], acc);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) {
                const double qv = fixed[row] ? 0.0 : acc;
                s.q[row] = qv;
                pq = fma(s.p[row], qv, pq);
            }
        }
    }
    block_atomic_add(pq, s.acc + 0);
}

// K2: alpha = rz_k / p.q, x += alpha p, r -= alpha q, z = B^-1 r, r.z and r.r. One thread per
// dof, 30 lanes of a warp = 10 nodes; a node's three residual entries meet through shuffles.
__global__ void __launch_bounds__(PCG_NT) pcg_k2(int64_t nnode, double *x, PcgState s, int qpair) {
    // one read of the done flag and one division per CTA (FP64 division is a long FP64-pipe
    // sequence); the flag read by one thread keeps the early return uniform across the CTA
    __shared__ double s_alpha;
    __shared__ int s_done;
    const int k = s.done[3];
    if (threadIdx.x == 0) {
        s_done = s.done[0];
        s_alpha = s_done ? 0.0 : s.acc[1 + (k & 1)] / s.acc[0];
    }
    __syncthreads();
    if (s_done) return;
    const double alpha = s_alpha;
    const int lane = threadIdx.x & 31, ln = lane / 3, i = lane % 3, l0 = 3 * ln;
    const int64_t warp = (blockIdx.x * (int64_t)PCG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * PCG_NT) >> 5;
    double rzn = 0.0, rr = 0.0;
    for (int64_t base = warp * 10; base < nnode; base += nwarps * 10) {  // warp-uniform trip count
        const int64_t m = base + ln;
        const bool valid = lane < 30 && m < nnode;
        const int64_t d = 3 * m + i;
        double rv = 0.0;
        if (valid) {
            x[d] = fma(alpha, s.p[d], x[d]);
            const double qd = qpair ? (double)s.qh[d] + (double)s.ql[d] : s.q[d];
            rv = fma(-alpha, qd, s.r[d]);
            s.r[d] = rv;
        }
        const double r0 = __shfl_sync(0xffffffffu, rv, l0);
        const double r1 = __shfl_sync(0xffffffffu, rv, (l0 + 1) & 31);
        const double r2 = __shfl_sync(0xffffffffu, rv, (l0 + 2) & 31);
        if (valid) {
            const double *B = s.Binv + m * 9 + i * 3;
            const double z = fma(B[0], r0, fma(B[1], r1, B[2] * r2));
            s.z[d] = z;
            rzn = fma(rv, z, rzn);
            rr = fma(rv, rv, rr);
        }
    }
    block_atomic_add(rzn, s.acc + 1 + ((k + 1) & 1));
    block_atomic_add(rr, s.acc + 3);
}

// K3: beta = rz_{k+1} / rz_k, p = z + beta p; zeroes p.q for the next K1
__global__ void __launch_bounds__(PCG_NT) pcg_k3(int64_t n, int split, PcgState s) {
    // one thread reads the done flag for the whole CTA, so every thread takes the same branch
    __shared__ double s_beta;
    __shared__ int s_done;
    const int k = s.done[3];
    if (threadIdx.x == 0) {
        s_done = s.done[0];
        s_beta = s_done ? 0.0 : s.acc[1 + ((k + 1) & 1)] / s.acc[1 + (k & 1)];
    }
    __syncthreads();
    if (s_done) return;
    const double beta = s_beta;
    for (int64_t d = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; d < n; d += (int64_t)gridDim.x * PCG_NT) {
        const double pv = fma(beta, s.p[d], s.z[d]);
        s.p[d] = pv;
        if (split) split_store(s, d, pv);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) s.acc[0] = 0.0;  // p.q of the next iterate (K2 has read it)
}

// The end of an iteration (one thread): the convergence test on r.r, the iteration index, and,
// when the iteration runs as the body of a conditional WHILE node of a CUDA graph, the loop
// condition -- continue while not converged and fewer than maxiter iterations have run.
__global__ void pcg_tail(double tol2, int64_t maxiter, PcgState s, cudaGraphConditionalHandle h, int cond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int *d = s.done;
    if (!d[0]) {
        const int k = d[3];
        const double rr = s.acc[3];
        if (rr <= tol2) {
            d[0] = 1;
            d[1] = k + 1;
        } else if (!isfinite(rr)) {
            d[0] = 1;
            d[1] = k + 1;
            d[2] |= 4;
        }
        d[3] = k + 1;
    }
    if (cond) cudaGraphSetConditional(h, (!d[0] && (int64_t)d[3] < maxiter) ? 1u : 0u);
}

// Float-pair iteration (with the float-pair products): x, r, z, p and the block inverses as
// unevaluated float pairs, every update on the FP32 pipe (~2^-46 relative per operation); the
// FP64 pipe, which bounds pcg_k2 / pcg_k3 on GB300, only forms one partial dot product per thread.

// x, r, z (FP64, from pcg_init / pcg_init2) and B^-1 -> float pairs
__global__ void __launch_bounds__(PCG_NT) pcg_to_pairs(int64_t n, const double *x, PcgState s) {
    for (int64_t d = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; d < n; d += (int64_t)gridDim.x * PCG_NT) {
        const FloatPair xv(x[d]), rv(s.r[d]), zv(s.z[d]);
        s.xh[d] = xv.h; s.xl[d] = xv.l;
        s.rh[d] = rv.h; s.rl[d] = rv.l;
        s.zh[d] = zv.h; s.zl[d] = zv.l;
        for (int k = 0; k < 3; ++k) {
            const FloatPair bv(s.Binv[d * 3 + k]);
            s.Bh[d * 3 + k] = bv.h;
            s.Bl[d * 3 + k] = bv.l;
        }
    }
}

// x (float pairs) -> x (FP64), at the end of a solve
__global__ void __launch_bounds__(PCG_NT) pcg_from_pairs(int64_t n, double *x, PcgState s) {
    for (int64_t d = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; d < n; d += (int64_t)gridDim.x * PCG_NT)
        x[d] = (double)s.xh[d] + (double)s.xl[d];
}

// K2 in float pairs: x += alpha p, r -= alpha q, z = B^-1 r, r.z and r.r (layout as pcg_k2)
__global__ void __launch_bounds__(PCG_NT) pcg_k2_pair(int64_t nnode, PcgState s) {
    __shared__ double s_alpha;
    __shared__ int s_done;
    const int k = s.done[3];
    if (threadIdx.x == 0) {
        s_done = s.done[0];
        s_alpha = s_done ? 0.0 : s.acc[1 + (k & 1)] / s.acc[0];
    }
    __syncthreads();
    if (s_done) return;
    const FloatPair alpha(s_alpha), nalpha(-s_alpha);
    const int lane = threadIdx.x & 31, ln = lane / 3, i = lane % 3, l0 = 3 * ln;
    const int64_t warp = (blockIdx.x * (int64_t)PCG_NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * PCG_NT) >> 5;
    FloatPair rz(0.f, 0.f), rr(0.f, 0.f);
    for (int64_t base = warp * 10; base < nnode; base += nwarps * 10) {  // warp-uniform trip count
        const int64_t m = base + ln;
        const bool valid = lane < 30 && m < nnode;
        const int64_t d = 3 * m + i;
        FloatPair rv(0.f, 0.f);
        if (valid) {
            const FloatPair p(s.ph[d], s.pl[d]), q(s.qh[d], s.ql[d]);
            const FloatPair xv = fma(alpha, p, FloatPair(s.xh[d], s.xl[d]));
            s.xh[d] = xv.h;
            s.xl[d] = xv.l;
            rv = fma(nalpha, q, FloatPair(s.rh[d], s.rl[d]));
            s.rh[d] = rv.h;
            s.rl[d] = rv.l;
        }
        FloatPair r3[3];
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r3[j] = FloatPair(__shfl_sync(0xffffffffu, rv.h, (l0 + j) & 31), __shfl_sync(0xffffffffu, rv.l, (l0 + j) & 31));
        if (valid) {
            const int64_t b = m * 9 + i * 3;
            FloatPair z = FloatPair(s.Bh[b], s.Bl[b]) * r3[0];
            z = fma(FloatPair(s.Bh[b + 1], s.Bl[b + 1]), r3[1], z);
            z = fma(FloatPair(s.Bh[b + 2], s.Bl[b + 2]), r3[2], z);
            s.zh[d] = z.h;
            s.zl[d] = z.l;
            rz = fma(rv, z, rz);
            rr = fma(rv, rv, rr);
        }
    }
    block_atomic_add(fpair::to_double(rz), s.acc + 1 + ((k + 1) & 1));
    block_atomic_add(fpair::to_double(rr), s.acc + 3);
}

// K3 in float pairs: p = z + beta p (written straight as the product's float pair), convergence
__global__ void __launch_bounds__(PCG_NT) pcg_k3_pair(int64_t n, PcgState s) {
    __shared__ double s_beta;
    __shared__ int s_done;
    const int k = s.done[3];
    if (threadIdx.x == 0) {
        s_done = s.done[0];
        s_beta = s_done ? 0.0 : s.acc[1 + ((k + 1) & 1)] / s.acc[1 + (k & 1)];
    }
    __syncthreads();
    if (s_done) return;
    const FloatPair beta(s_beta);
    for (int64_t d = blockIdx.x * (int64_t)PCG_NT + threadIdx.x; d < n; d += (int64_t)gridDim.x * PCG_NT) {
        const FloatPair pv = fma(beta, FloatPair(s.ph[d], s.pl[d]), FloatPair(s.zh[d], s.zl[d]));
        s.ph[d] = pv.h;
        s.pl[d] = pv.l;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) s.acc[0] = 0.0;  // p.q of the next iterate (K2 has read it)
}

// Resident blocks of a kernel over the whole GPU (one wave), for grid sizes of the grid-stride
// kernels.
template <auto Kernel>
static int64_t resident_blocks() {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kernel, PCG_NT, 0);
    return (int64_t)std::max(1, sms) * std::max(1, per_sm);
}

// K1 launch for a value type and lanes per node; grid = one wave, or fewer blocks if the nodes
// run out first
template <class MT, int NB>
static void launch_k1(const int32_t *indptr, const int32_t *indices, const MT *vals, const int8_t *fixed, int64_t n,
                      const PcgState &s, cudaStream_t st) {
    static thread_local int64_t wave[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int64_t &w = wave[dev & 63];
    if (w == 0) w = resident_blocks<pcg_k1<MT, true, NB>>();
    const int64_t nodes_per_block = (PCG_NT / 32) * (32 / NB);
    const int64_t need = (n / 3 + nodes_per_block - 1) / nodes_per_block;
    pcg_k1<MT, true, NB><<<(unsigned)std::max<int64_t>(1, std::min(need, w)), PCG_NT, 0, st>>>(indptr, indices, vals,
                                                                                              fixed, n, s);
}

template <class MT>
static void launch_k1_nb(int nb, const int32_t *indptr, const int32_t *indices, const MT *vals, const int8_t *fixed,
                         int64_t n, const PcgState &s, cudaStream_t st) {
    switch (nb) {
        case 4: launch_k1<MT, 4>(indptr, indices, vals, fixed, n, s, st); break;
        case 16: launch_k1<MT, 16>(indptr, indices, vals, fixed, n, s, st); break;
        case 32: launch_k1<MT, 32>(indptr, indices, vals, fixed, n, s, st); break;
        default: launch_k1<MT, 8>(indptr, indices, vals, fixed, n, s, st); break;
    }
}

// Lanes per node of the node-block product, picked by timing two products with each choice on
// the first solve of a matrix shape (device, rows, nonzeros, value type) and cached. The timed
// launches only write q and the p.q slot, which the caller resets afterwards.
struct LaneKey {
    int dev, kind;
    int64_t n, nnz;
};
static std::mutex g_lane_mutex;
static std::vector<std::pair<LaneKey, int>> g_lane_cache;

template <class MT>
static int pick_lanes(const int32_t *indptr, const int32_t *indices, const MT *vals, const int8_t *fixed, int64_t n,
                      int64_t nnz, int kind, const PcgState &s, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lock(g_lane_mutex);
        for (auto &e : g_lane_cache)
            if (e.first.dev == dev && e.first.kind == kind && e.first.n == n && e.first.nnz == nnz) return e.second;
    }
    int best = 8;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return best;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return best;
    }
    for (int nb : {4, 8, 16, 32}) {
        launch_k1_nb<MT>(nb, indptr, indices, vals, fixed, n, s, st);  // first touch
        cudaEventRecord(e0, st);
        for (int r = 0; r < 2; ++r) launch_k1_nb<MT>(nb, indptr, indices, vals, fixed, n, s, st);
        cudaEventRecord(e1, st);
        float ms = 0.f;
        if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
            ms < best_ms) {
            best_ms = ms;
            best = nb;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(g_lane_mutex);
    g_lane_cache.push_back({LaneKey{dev, kind, n, nnz}, best});
    return best;
}

// The PCG iterations as one CUDA graph: a conditional WHILE node whose body -- captured from
// `iteration` on a private stream -- is one iteration, its last kernel setting the condition.
// Launched on `st`; the host waits only for the final result. Returns the executable graph (to be
// destroyed after the stream has synchronised), or nullptr when the graph cannot be built, in
// which case nothing was enqueued and the caller iterates from the host.
static std::atomic<int> g_device_loop{1};

template <class Iter>
static cudaGraphExec_t device_loop(cudaStream_t st, Iter &&iteration) {
    static std::mutex m;
    static cudaStream_t cs[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    {
        std::lock_guard<std::mutex> g(m);
        if (!cs[dev & 63] && cudaStreamCreateWithFlags(&cs[dev & 63], cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (cudaGraphCreate(&graph, 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    bool ok = false;
    do {
        cudaGraphConditionalHandle h;
        if (cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault) != cudaSuccess) break;
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if (cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np) != cudaSuccess) break;
        cudaGraph_t body = np.conditional.phGraph_out[0];
        if (cudaStreamBeginCaptureToGraph(cs[dev & 63], body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            break;
        iteration(cs[dev & 63], h, 1);
        cudaGraph_t captured = nullptr;
        if (cudaStreamEndCapture(cs[dev & 63], &captured) != cudaSuccess) break;
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            exec = nullptr;
            break;
        }
        ok = cudaGraphLaunch(exec, st) == cudaSuccess;
    } while (false);
    cudaGraphDestroy(graph);
    if (!ok) {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        cudaGetLastError();
    }
    return exec;
}

template <class VT>
static int bj_pcg(const int32_t *indptr, const int32_t *indices, const VT *vals, int64_t n, const int8_t *fixed,
                  const double *b, double *x, double rtol, int64_t maxiter, void *ws, size_t ws_bytes,
                  int64_t *iters, double *relres, cudaStream_t st, bool split = false) {
    if (!indptr || !indices || !vals || !fixed || !b || !x || !iters || !relres || n <= 0 || n % 3) return FL_ERR_ARG;
    int32_t nnz32 = 0;
    FL_CUDA_TRY(cudaMemcpyAsync(&nnz32, indptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FL_CUDA_TRY(cudaStreamSynchronize(st));
    if (nnz32 < 0) return FL_ERR_ARG;
    // the split copy is sized by the matrix
    if (pcg_layout(n, split ? nnz32 : 0, nullptr, nullptr) > ws_bytes || !ws) return FL_ERR_CAPACITY;
    PcgState s;
    float2 *vsplit = nullptr;
    pcg_layout(n, split ? nnz32 : 0, &s, (char *)ws, &vsplit);
    const int64_t nnode = n / 3;
    const unsigned g_rows = (unsigned)std::min<int64_t>((n + (PCG_NT / 32) - 1) / (PCG_NT / 32), 152 * 16);
    const unsigned g_nodes = (unsigned)std::min<int64_t>((nnode + PCG_NT - 1) / PCG_NT, 152 * 16);
    const unsigned g_dofs = (unsigned)std::min<int64_t>((n + PCG_NT - 1) / PCG_NT, 152 * 16);
    static thread_local int64_t k2_wave[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (k2_wave[dev & 63] == 0) k2_wave[dev & 63] = resident_blocks<pcg_k2>();
    const int64_t k2_need = ((nnode + 9) / 10 + PCG_NT / 32 - 1) / (PCG_NT / 32);
    const unsigned g_k2 = (unsigned)std::max<int64_t>(1, std::min(k2_need, k2_wave[dev & 63]));
    FL_CUDA_TRY(cudaMemsetAsync(s.done, 0, sizeof(int) * 4, st));
    FL_CUDA_TRY(cudaMemsetAsync(s.acc, 0, sizeof(double) * 8, st));
    bj_setup<<<g_nodes, PCG_NT, 0, st>>>(indptr, indices, vals, fixed, nnode, s.Binv, s.done + 2);
    pcg_check_blocks<<<g_rows, PCG_NT, 0, st>>>(indptr, indices, nnode, s.done + 2);
    pcg_init<<<g_rows, PCG_NT, 0, st>>>(indptr, indices, vals, fixed, b, x, n, s);
    pcg_init2<<<g_nodes, PCG_NT, 0, st>>>(nnode, s);
    double hacc[8];
    int err = 0;
    FL_CUDA_TRY(cudaMemcpyAsync(hacc, s.acc, sizeof(hacc), cudaMemcpyDeviceToHost, st));
    FL_CUDA_TRY(cudaMemcpyAsync(&err, s.done + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
    FL_CUDA_TRY(cudaStreamSynchronize(st));
    if (err & 3) return FL_ERR_ARG;  // pattern without diagonal blocks, or a singular block
    const bool nodeblk = !(err & 8);
    split = split && nodeblk;  // the float-pair product is the node-block one
    const double b2 = hacc[4];
    if (b2 == 0.0) {  // zero right-hand side: x unchanged is the solution
        *iters = 0;
        *relres = 0.0;
        return FL_OK;
    }
    if (split) split_values<<<g_dofs, PCG_NT, 0, st>>>(indptr, n, (const double *)vals, vsplit);
    int nb = 8;
    if (nodeblk) {
        nb = split ? pick_lanes<float2>(indptr, indices, vsplit, fixed, n, nnz32, 2, s, st)
                   : pick_lanes<VT>(indptr, indices, vals, fixed, n, nnz32, (int)sizeof(VT), s, st);
        FL_CUDA_TRY(cudaMemsetAsync(s.acc, 0, sizeof(double), st));  // p.q of the timed products
    }
    const double tol2 = rtol * rtol * b2;
    // with the float-pair products the iteration vectors are float pairs too
    const bool pairs = nodeblk && (split || sizeof(VT) == 4);
    if (pairs) pcg_to_pairs<<<g_dofs, PCG_NT, 0, st>>>(n, x, s);
    int hd[4] = {0, 0, 0, 0};
    // one iteration: K1, K2, K3 and the tail (convergence test, iteration index, loop condition)
    auto iteration = [&](cudaStream_t q, cudaGraphConditionalHandle h, int cond) {
        if (split) launch_k1_nb<float2>(nb, indptr, indices, vsplit, fixed, n, s, q);
        else if (nodeblk) launch_k1_nb<VT>(nb, indptr, indices, vals, fixed, n, s, q);
        else pcg_k1<VT, false><<<g_rows, PCG_NT, 0, q>>>(indptr, indices, vals, fixed, n, s);
        if (pairs) {
            pcg_k2_pair<<<g_k2, PCG_NT, 0, q>>>(nnode, s);
            pcg_k3_pair<<<g_dofs, PCG_NT, 0, q>>>(n, s);
        } else {
            pcg_k2<<<g_k2, PCG_NT, 0, q>>>(nnode, x, s, 0);
            pcg_k3<<<g_dofs, PCG_NT, 0, q>>>(n, 0, s);
        }
        pcg_tail<<<1, 32, 0, q>>>(tol2, maxiter, s, h, cond);
    };
    // the whole loop on the device (a conditional WHILE node), or host-driven with a poll of the
    // done flag every PCG_CHECK iterations
    cudaGraphExec_t loop = nullptr;
    if (maxiter > 0 && g_device_loop.load()) loop = device_loop(st, iteration);
    if (!loop) {
        int64_t k = 0;
        while (k < maxiter) {
            const int64_t kend = std::min<int64_t>(maxiter, k + PCG_CHECK);
            for (; k < kend; ++k) iteration(st, cudaGraphConditionalHandle{}, 0);
            FL_CUDA_TRY(cudaGetLastError());
            FL_CUDA_TRY(cudaMemcpyAsync(hd, s.done, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
            FL_CUDA_TRY(cudaStreamSynchronize(st));
            if (hd[0]) break;
        }
    }
    if (pairs) pcg_from_pairs<<<g_dofs, PCG_NT, 0, st>>>(n, x, s);
    FL_CUDA_TRY(cudaMemcpyAsync(hacc, s.acc, sizeof(hacc), cudaMemcpyDeviceToHost, st));
    FL_CUDA_TRY(cudaMemcpyAsync(hd, s.done, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
    const cudaError_t se = cudaStreamSynchronize(st);
    if (loop) cudaGraphExecDestroy(loop);
    if (se != cudaSuccess) return FL_ERR_CUDA;
    *iters = hd[0] ? hd[1] : maxiter;
    *relres = sqrt(hacc[3] / b2);
    if (hd[2] & 4) return FL_ERR_ARG;  // breakdown: non-finite residual
    return FL_OK;
}

}  // namespace fl

extern "C" {

int fl_SetPCGDeviceLoop(int enable) {
    if (enable != 0 && enable != 1) return FL_ERR_ARG;
    fl::g_device_loop.store(enable);
    return FL_OK;
}

int fl_GetPCGDeviceLoop(void) { return fl::g_device_loop.load(); }

size_t fl_BlockJacobiPCG_workspace_size(int64_t nrows, int64_t nnz, int value_bits) {
    return fl::pcg_layout(nrows, value_bits == FL_PCG_F64_SPLIT ? nnz : 0, nullptr, nullptr);
}

int fl_BlockJacobiPCG(const int32_t *indptr, const int32_t *indices, const void *values, int value_bits,
                      int64_t nrows, const int8_t *fixed, const double *b, double *x, double rtol, int64_t maxiter,
                      void *workspace, size_t workspace_bytes, int64_t *iterations, double *relres,
                      fl_stream_t stream) {
    if (value_bits == FL_PCG_F64 || value_bits == FL_PCG_F64_SPLIT)
        return fl::bj_pcg(indptr, indices, (const double *)values, nrows, fixed, b, x, rtol, maxiter, workspace,
                          workspace_bytes, iterations, relres, (cudaStream_t)stream, value_bits == FL_PCG_F64_SPLIT);
    if (value_bits == FL_PCG_F32)
        return fl::bj_pcg(indptr, indices, (const float *)values, nrows, fixed, b, x, rtol, maxiter, workspace,
                          workspace_bytes, iterations, relres, (cudaStream_t)stream);
    return FL_ERR_ARG;
}

}  // extern "C"
