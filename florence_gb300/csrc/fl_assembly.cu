// fl_assembly.cu -- FP64 tangent + residual assembly for the displacement formulation
// (replaces _GlobalAssemblyDF_, Florence/FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDF_.h:8-176).
//
// Two kernels per chunk of elements:
//  A. qp_kernel, one thread per (element, Gauss point): kinematics, material, and the tangent
//     pulled back to the reference element
//        Ahat[(i,d),(k,e)] = detJ sum_{j,l} G[j][d] A_ijkl G[l][e],  A_ijkl = c_ijkl + d_ik sigma_jl
//     (constitutive + geometric stiffness folded into one tensor, G = (dx/dxi)^{-1}; Ahat is
//     symmetric, 45 values), and S[i][d] = detJ sum_j sigma_ij G[j][d] for the residual. Written to
//     a scratch array Q[54][chunk Gauss points] (structure of arrays: coalesced stores and loads;
//     a chunk is sized to stay in L2).
//  B. contract_kernel, EPC elements per CTA:
//        K_e[(a,i),(b,k)] = sum_g sum_{d,e} Jm[d][a][g] Ahat_g[(i,d),(k,e)] Jm[e][b][g]
//     U_g[b][(i,d),k] = sum_e Ahat_g[(i,d),(k,e)] Jm[e][b][g] is built cooperatively in shared
//     memory per Gauss-point chunk, then each stiffness entry costs 3 FMAs per Gauss point. Only
//     node blocks a <= b are formed (K_e is symmetric), 9 register accumulators per block, blocks
//     ordered b-major so a warp mostly reads the same U row (shared-memory broadcast). Scatter:
//     triplets, CSR through the reference's element-to-nonzero maps, or CSR by binary search in
//     the row; residual t[(a,i)] = sum_g sum_d Jm[d][a][g] S_g[i][d] into T.
// The FP64 pipe bounds both kernels (GB300 has a reduced FP64 rate); the design minimises FP64
// instructions (fused multiply-adds throughout) and keeps kernel B's register footprint small
// so several CTAs share an SM and hide the per-chunk barriers.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include "fl_common.cuh"
#include "fl_tc.cuh"

namespace fl {

// contraction kernel: TPE threads per element, EPC elements per CTA, MAXB node blocks per thread
// per pass, MINB resident CTAs per SM requested from the compiler; the float-pair arithmetic
// needs more registers per accumulator update and has its own MAXB_DF / MINB_DF (same TPE/EPC,
// so the host-side chunking and shared-memory sizes are shared)
template <int NPE>
struct AsmCfg;
template <> struct AsmCfg<4> { static constexpr int TPE = 32, EPC = 8, MAXB = 1, MINB = 4, MAXB_DF = 1, MINB_DF = 4; };
template <> struct AsmCfg<8> { static constexpr int TPE = 32, EPC = 8, MAXB = 2, MINB = 4, MAXB_DF = 2, MINB_DF = 2; };
template <> struct AsmCfg<10> { static constexpr int TPE = 64, EPC = 4, MAXB = 1, MINB = 4, MAXB_DF = 1, MINB_DF = 4; };
template <> struct AsmCfg<20> { static constexpr int TPE = 128, EPC = 2, MAXB = 2, MINB = 4, MAXB_DF = 2, MINB_DF = 2; };
template <> struct AsmCfg<27> { static constexpr int TPE = 384, EPC = 1, MAXB = 1, MINB = 2, MAXB_DF = 1, MINB_DF = 2; };
template <> struct AsmCfg<35> { static constexpr int TPE = 320, EPC = 1, MAXB = 2, MINB = 2, MAXB_DF = 2, MINB_DF = 2; };
template <> struct AsmCfg<64> { static constexpr int TPE = 416, EPC = 1, MAXB = 5, MINB = 1, MAXB_DF = 3, MINB_DF = 1; };
template <> struct AsmCfg<125> { static constexpr int TPE = 512, EPC = 1, MAXB = 4, MINB = 1, MAXB_DF = 3, MINB_DF = 1; };

constexpr int QSTRIDE = 54;    // 45 symmetric Ahat entries + 9 residual entries per Gauss point
constexpr int QSM = 45;        // entries per Gauss point held in shared memory (the tangent part)
constexpr int QP_THREADS = 128;
constexpr size_t CHUNK_BYTES = (size_t)64 << 20;  // scratch per chunk: L2-resident between A and B

struct AsmArgs {
    const double *points;
    const uint64_t *elements;
    const double *Eulerx;
    const double *Jm;
    const double *w;
    int64_t nelem, nnode;
    int nq, update, mode, qc;  // mode: 0 triplets, 1 CSR via maps, 2 CSR via row search
    int32_t *I, *J;
    double *V, *T;
    const int32_t *indptr, *indices, *dl, *dg;
    MatParams mp;
    const double *eparams;  // optional per-element material parameters [nelem][3] (overrides mp)
    int *flags;
    double *Q;       // scratch [QSTRIDE][ldq]
    const float *Jmf;  // FP32 copy of Jm (the split-BF16 tangent's operand), or null
    int utab;          // split-BF16 kernel: 1 = the element's U table is built in shared memory first
    int64_t e0, ne;  // element chunk [e0, e0+ne)
    int64_t ldq;     // leading dimension of Q (>= ne*nq)
};

// Position of `col` in CSR row `row` (sorted columns) relative to the row start, -1 if absent.
__device__ __forceinline__ int row_search(const int32_t *indptr, const int32_t *indices, int row, int col) {
    const int r0 = indptr[row], r1 = indptr[row + 1];
    int lo = r0, hi = r1;
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (col < indices[mid]) hi = mid; else lo = mid;
    }
    return (lo < r1 && indices[lo] == col) ? lo - r0 : -1;
}

// CSR position of dof entry (3*nr + ri, 3*nc + ci) given the offset `off` of column 3*nc in row
// 3*nr (a node-block CSR: the three rows of a node share one column pattern, so the entry sits at
// indptr[3*nr + ri] + off + ci). The position is verified against `indices`; when it does not
// match (a CSR without node blocks) the row is searched. -1 if the entry is absent.
__device__ __forceinline__ int64_t block_entry(const int32_t *indptr, const int32_t *indices, int nr, int nc, int ri,
                                               int ci, int off) {
    const int row = 3 * nr + ri, col = 3 * nc + ci;
    if (off >= 0) {
        const int p = indptr[row] + off + ci;
        if (p < indptr[row + 1] && indices[p] == col) return p;
    }
    const int o = row_search(indptr, indices, row, col);
    return o < 0 ? -1 : (int64_t)indptr[row] + o;
}

// index of (I,K), I,K in 0..8, in the packed upper triangle of a symmetric 9x9
__host__ __device__ __forceinline__ constexpr int sym9(int I, int K) {
    return (I < K ? I : K) * 9 - ((I < K ? I : K) * ((I < K ? I : K) - 1)) / 2 + ((I < K ? K : I) - (I < K ? I : K));
}

// ------------------------------------------------------------------------------------------------
// A. Gauss-point data
// ------------------------------------------------------------------------------------------------
template <int NPE, int MAT>
__global__ void __launch_bounds__(QP_THREADS) qp_kernel(const AsmArgs A) {
    const int64_t t = (int64_t)blockIdx.x * QP_THREADS + threadIdx.x;
    const int nq = A.nq;
    int flag = 0;
    if (t < A.ne * nq) {
        const int64_t e = A.e0 + t / nq;
        const int g = (int)(t % nq);
        const uint64_t *el = A.elements + e * NPE;
        auto jm = [&](int d, int a) { return __ldg(A.Jm + ((size_t)d * NPE + a) * nq + g); };
        auto coords = [&](int a, double &X0, double &X1, double &X2, double &x0, double &x1, double &x2) {
            uint64_t nd = __ldg(el + a);
            if (nd >= (uint64_t)A.nnode) {
                flag |= FL_FLAG_BAD_INDEX;
                nd = 0;
            }
            X0 = __ldg(A.points + nd * 3); X1 = __ldg(A.points + nd * 3 + 1); X2 = __ldg(A.points + nd * 3 + 2);
            x0 = __ldg(A.Eulerx + nd * 3); x1 = __ldg(A.Eulerx + nd * 3 + 1); x2 = __ldg(A.Eulerx + nd * 3 + 2);
        };
        double G[9], F[9];
        const double detJ = kinematics_fn<NPE>(jm, coords, __ldg(A.w + g), A.update, G, F);
        double sig[6], b[6], J, c1, c2, cbb;
        MatParams mp = A.mp;
        if (A.eparams) mp = MatParams{__ldg(A.eparams + e * 3), __ldg(A.eparams + e * 3 + 1), __ldg(A.eparams + e * 3 + 2)};
        ExtraTangent ex;
        material<MAT>(F, mp, sig, b, J, c1, c2, cbb, &ex);
        if (!(J > 0.0)) flag |= FL_FLAG_NONPOSITIVE_J;
        constexpr bool NIMR = MAT == NEARLYINCOMPRESSIBLEMR;
        // GG = G^T G, GsG = G^T sigma G, bG = b G, GbG = G^T b G, gG = g G, GgG = G^T g G
        double GG[9], GsG[9], sG[9], bG[9], GbG[9], gG[9], GgG[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                sG[i * 3 + d] = fma(sig[s6(i, 0)], G[0 * 3 + d], fma(sig[s6(i, 1)], G[1 * 3 + d], sig[s6(i, 2)] * G[2 * 3 + d]));
                if (MAT == MOONEYRIVLIN || NIMR)
                    bG[i * 3 + d] = fma(b[s6(i, 0)], G[0 * 3 + d], fma(b[s6(i, 1)], G[1 * 3 + d], b[s6(i, 2)] * G[2 * 3 + d]));
                if (NIMR)
                    gG[i * 3 + d] = fma(ex.g[s6(i, 0)], G[0 * 3 + d], fma(ex.g[s6(i, 1)], G[1 * 3 + d], ex.g[s6(i, 2)] * G[2 * 3 + d]));
            }
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int e2 = d; e2 < 3; ++e2) {
                GG[d * 3 + e2] = fma(G[d], G[e2], fma(G[3 + d], G[3 + e2], G[6 + d] * G[6 + e2]));
                // no geometric stiffness for the linear elastic material (the reference builds that
                // assembler without it, AOT_Assembler.py:74-81)
                GsG[d * 3 + e2] = MAT == LINEARELASTIC ? 0.0 : fma(G[d], sG[e2], fma(G[3 + d], sG[3 + e2], G[6 + d] * sG[6 + e2]));
                if (MAT == MOONEYRIVLIN) GbG[d * 3 + e2] = fma(G[d], bG[e2], fma(G[3 + d], bG[3 + e2], G[6 + d] * bG[6 + e2]));
                if (NIMR) GgG[d * 3 + e2] = fma(G[d], gG[e2], fma(G[3 + d], gG[3 + e2], G[6 + d] * gG[6 + e2]));
            }
        // Ahat[(i,d),(k,e)] = detJ [ d_ik (c1 GG + GsG)[d][e] + c1 G[k][d] G[i][e] + c2 G[i][d] G[k][e]
        //                          + cbb (2 bG[i][d] bG[k][e] - b_ik GbG[d][e] - bG[k][d] bG[i][e]) ]
        double *q = A.Q + t;
        const int64_t ld = A.ldq;
#pragma unroll
        for (int I = 0; I < 9; ++I)
#pragma unroll
            for (int K = I; K < 9; ++K) {
                const int i = I / 3, d = I % 3, k = K / 3, e2 = K % 3;
                const int dd = d < e2 ? d : e2, ee = d < e2 ? e2 : d;
                double v = fma(c1 * G[k * 3 + d], G[i * 3 + e2], c2 * G[i * 3 + d] * G[k * 3 + e2]);
                if (i == k) v = fma(c1, GG[dd * 3 + ee], v + GsG[dd * 3 + ee]);
                if (MAT == MOONEYRIVLIN)
                    v = fma(cbb, fma(2.0 * bG[i * 3 + d], bG[k * 3 + e2], -fma(b[s6(i, k)], GbG[dd * 3 + ee], bG[k * 3 + d] * bG[i * 3 + e2])), v);
                if (NIMR) {
                    // kbI (bG_id G_ke + G_id bG_ke) + kgI (gG_id G_ke + G_id gG_ke) + kgg gG_id gG_ke
                    // + kg4 (g_ik GG_de + gG_ie G_kd + gG_kd G_ie + d_ik GgG_de)
                    v = fma(ex.kbI, fma(bG[i * 3 + d], G[k * 3 + e2], G[i * 3 + d] * bG[k * 3 + e2]), v);
                    v = fma(ex.kgI, fma(gG[i * 3 + d], G[k * 3 + e2], G[i * 3 + d] * gG[k * 3 + e2]), v);
                    v = fma(ex.kgg, gG[i * 3 + d] * gG[k * 3 + e2], v);
                    double t4 = fma(ex.g[s6(i, k)], GG[dd * 3 + ee], fma(gG[i * 3 + e2], G[k * 3 + d], gG[k * 3 + d] * G[i * 3 + e2]));
                    if (i == k) t4 += GgG[dd * 3 + ee];
                    v = fma(ex.kg4, t4, v);
                }
                q[sym9(I, K) * ld] = detJ * v;
            }
#pragma unroll
        for (int k = 0; k < 9; ++k) q[(45 + k) * ld] = detJ * sG[k];  // S[i][d]
    }
    if (flag && A.flags) atomicOr(A.flags, flag);
}

// ------------------------------------------------------------------------------------------------
// B. contraction + scatter
//
// Arithmetic of the contraction (template parameter DF):
//  false: FP64 fused multiply-adds.
//  true:  float pairs on the FP32 pipe. Every operand is held as hi + lo (hi = RN_f32(x),
//         lo = RN_f32(x - hi)); a product is formed error-free in its leading part
//         (p = ah*bh, e = fma(ah, bh, -p)) plus the cross terms ah*bl + al*bh, and added to the
//         accumulator with Knuth's two-sum, the rounding error carried in the low word. The
//         relative error of one multiply-add is about 2^-46 (the dropped al*bl and the low word's
//         own rounding), so the element matrix is FP64-accurate to ~1e-14 relative while the
//         work runs at the FP32 rate, 64x GB300's FP64 rate. The residual stays FP64.
// ------------------------------------------------------------------------------------------------
template <bool DF>
struct Arith;

template <>
struct Arith<false> {
    using S = double;  // shared-memory operand
    struct Acc {
        double v;
    };
    static __device__ __forceinline__ S split(double x) { return x; }
    static __device__ __forceinline__ void zero(Acc &a) { a.v = 0.0; }
    static __device__ __forceinline__ void mac(Acc &a, S x, S y) { a.v = fma(x, y, a.v); }
    static __device__ __forceinline__ double value(const Acc &a) { return a.v; }
    static __device__ __forceinline__ S store(const Acc &a) { return a.v; }
};

template <>
struct Arith<true> {
    using S = float2;
    struct Acc {
        float h, l;
    };
    static __device__ __forceinline__ S split(double x) {
        const float h = (float)x;
        return make_float2(h, (float)(x - (double)h));
    }
    static __device__ __forceinline__ void zero(Acc &a) { a.h = a.l = 0.f; }
    static __device__ __forceinline__ void mac(Acc &a, S x, S y) {
        const float p = x.x * y.x;
        const float pe = fmaf(x.x, y.y, fmaf(x.y, y.x, fmaf(x.x, y.x, -p)));
        const float s = a.h + p;
        const float bv = s - a.h;
        const float e = (a.h - (s - bv)) + (p - bv);
        a.h = s;
        a.l += e + pe;
    }
    static __device__ __forceinline__ double value(const Acc &a) { return (double)a.h + (double)a.l; }
    static __device__ __forceinline__ S store(const Acc &a) {  // renormalised pair
        const float h = a.h + a.l;
        return make_float2(h, a.l - (h - a.h));
    }
};

template <int NPE, bool DF>
__global__ void __launch_bounds__(AsmCfg<NPE>::TPE * AsmCfg<NPE>::EPC, DF ? AsmCfg<NPE>::MINB_DF : AsmCfg<NPE>::MINB)
    contract_kernel(const AsmArgs A) {
    using AR = Arith<DF>;
    using S = typename AR::S;
    using Acc = typename AR::Acc;
    constexpr int TPE = AsmCfg<NPE>::TPE, EPC = AsmCfg<NPE>::EPC;
    constexpr int MAXB = DF ? AsmCfg<NPE>::MAXB_DF : AsmCfg<NPE>::MAXB;
    constexpr int NT = TPE * EPC, NDOF = 3 * NPE, NBLK = NPE * (NPE + 1) / 2;
    constexpr int PER_PASS = TPE * MAXB, NPASS = (NBLK + PER_PASS - 1) / PER_PASS;
    static_assert(sizeof(S) == sizeof(double), "shared-memory layout assumes 8-byte operands");
    const int nq = A.nq, QC = A.qc;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    S *Qs = reinterpret_cast<S *>(smem_raw);                                 // [EPC][nq][QSM]
    S *Jc = Qs + (size_t)EPC * nq * QSM;                                     // [QC][NPE][3]
    S *Us = Jc + (size_t)QC * NPE * 3;                                       // [EPC][QC][NPE][27]
    double *Ss = reinterpret_cast<double *>(Us + (size_t)EPC * QC * NPE * 27);  // [EPC][nq][9] residual part
    int *nodes = reinterpret_cast<int *>(Ss + (size_t)EPC * nq * 9);          // [EPC][NPE]
    int *inv = nodes + EPC * NPE;                                            // [EPC][NDOF]
    __shared__ int s_flag;
    __shared__ int64_t s_nnz;

    const int tid = threadIdx.x, slot = tid / TPE, lt = tid % TPE;
    const int64_t el = (int64_t)blockIdx.x * EPC + slot;  // element within the chunk
    const int64_t e = A.e0 + el;
    const bool active = el < A.ne;
    int flag = 0;
    if (tid == 0) {
        s_flag = 0;
        s_nnz = (A.mode != 0) ? (int64_t)A.indptr[3 * A.nnode] : 0;
    }

    const int64_t cap = (int64_t)NDOF * NDOF;
    const double *qg = A.Q + el * nq;  // this element's Gauss-point data, Q[k][el*nq + g]
    if (active) {
        for (int a = lt; a < NPE; a += TPE) {
            uint64_t nd = A.elements[e * NPE + a];
            if (nd >= (uint64_t)A.nnode) {
                flag |= FL_FLAG_BAD_INDEX;
                nd = 0;
            }
            nodes[slot * NPE + a] = (int)nd;
        }
        if (A.mode == 1) {
            // invert the element's dof permutation carried by data_local_indices:
            // dl[e*cap + i*NDOF + j] = perm[i]*NDOF + perm[j]  ->  inv[perm[i]] = i
            for (int i = lt; i < NDOF; i += TPE) {
                const int v = A.dl[e * cap + (int64_t)i * NDOF];
                const int p = v / NDOF;
                if (v < 0 || p >= NDOF) flag |= FL_FLAG_BAD_INDEX;
                else inv[slot * NDOF + p] = i;
            }
        }
        // Gauss-point data -> tangent part Qs[slot][g][k] (operand format), residual part
        // Ss[slot][g][k] (FP64)
        for (int idx = lt; idx < nq * QSTRIDE; idx += TPE) {
            const int k = idx / nq, g = idx % nq;
            const double v = qg[k * A.ldq + g];
            if (k < QSM) Qs[((size_t)slot * nq + g) * QSM + k] = AR::split(v);
            else Ss[((size_t)slot * nq + g) * 9 + (k - QSM)] = v;
        }
    }
    __syncthreads();

    // residual t[(a,i)] = sum_g sum_d Jm[d][a][g] S_g[i][d], FP64
    if (active && A.update) {
        for (int r = lt; r < NDOF; r += TPE) {
            const int a = r / 3, i = r % 3;
            double t = 0.0;
            const double *qs = Ss + (size_t)slot * nq * 9 + i * 3;
            for (int g = 0; g < nq; ++g, qs += 9) {
                t = fma(__ldg(A.Jm + (size_t)a * nq + g), qs[0], t);
                t = fma(__ldg(A.Jm + ((size_t)NPE + a) * nq + g), qs[1], t);
                t = fma(__ldg(A.Jm + ((size_t)2 * NPE + a) * nq + g), qs[2], t);
            }
            atomicAdd(A.T + 3 * (int64_t)nodes[slot * NPE + a] + i, t);
        }
    }

    // stiffness, in passes over the node blocks (a <= b, b-major)
    for (int pass = 0; pass < NPASS; ++pass) {
        Acc acc[MAXB][9];
        int ba[MAXB], bb[MAXB];
#pragma unroll
        for (int m = 0; m < MAXB; ++m) {
            const int blk = pass * PER_PASS + m * TPE + lt;
            int b = (int)((sqrtf(8.0f * blk + 1.0f) - 1.0f) * 0.5f);
            while (b * (b + 1) / 2 > blk) --b;
            while ((b + 1) * (b + 2) / 2 <= blk) ++b;
            ba[m] = blk < NBLK ? blk - b * (b + 1) / 2 : -1;
            bb[m] = b;
#pragma unroll
            for (int k = 0; k < 9; ++k) AR::zero(acc[m][k]);
        }
        for (int c0 = 0; c0 < nq; c0 += QC) {
            const int qc = min(QC, nq - c0);
            for (int idx = tid; idx < qc * NPE * 3; idx += NT) {
                const int q = idx / (NPE * 3), r = idx % (NPE * 3), a = r / 3, d = r % 3;
                Jc[idx] = AR::split(__ldg(A.Jm + ((size_t)d * NPE + a) * nq + c0 + q));
            }
            __syncthreads();
            if (active) {
                // U_g[b][(i,d),k], one entry per work item (balanced over the CTA's threads; the
                // tensor index varies across a warp, so it is computed, not unrolled)
                for (int idx = lt; idx < qc * NPE * 27; idx += TPE) {
                    const int q = idx / (NPE * 27), r = idx % (NPE * 27), b = r / 27, s = r % 27;
                    const int I = s / 3, k = s % 3;  // s = (i*3+d)*3 + k, I = i*3+d
                    const S *qq = Qs + ((size_t)slot * nq + c0 + q) * QSM;
                    const S *jb = Jc + (q * NPE + b) * 3;
                    Acc u;
                    AR::zero(u);
                    AR::mac(u, qq[sym9(I, k * 3 + 2)], jb[2]);
                    AR::mac(u, qq[sym9(I, k * 3 + 1)], jb[1]);
                    AR::mac(u, qq[sym9(I, k * 3 + 0)], jb[0]);
                    Us[(((size_t)slot * QC + q) * NPE + b) * 27 + s] = AR::store(u);
                }
            }
            __syncthreads();
            if (active) {
                for (int q = 0; q < qc; ++q) {
#pragma unroll
                    for (int m = 0; m < MAXB; ++m) {
                        if (ba[m] < 0) continue;
                        const S *ja = Jc + (q * NPE + ba[m]) * 3;
                        const S j0 = ja[0], j1 = ja[1], j2 = ja[2];
                        const S *u = Us + (((size_t)slot * QC + q) * NPE + bb[m]) * 27;
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int k = 0; k < 3; ++k) {
                                AR::mac(acc[m][i * 3 + k], j0, u[(i * 3 + 0) * 3 + k]);
                                AR::mac(acc[m][i * 3 + k], j1, u[(i * 3 + 1) * 3 + k]);
                                AR::mac(acc[m][i * 3 + k], j2, u[(i * 3 + 2) * 3 + k]);
                            }
                    }
                }
            }
            __syncthreads();
        }
        // scatter this pass's blocks
        if (active) {
#pragma unroll
            for (int m = 0; m < MAXB; ++m) {
                if (ba[m] < 0) continue;
                const int a = ba[m], b = bb[m];
                const int na = nodes[slot * NPE + a], nb = nodes[slot * NPE + b];
                if (A.mode == 2) {  // one row search per node block and mirror
                    for (int mirror = 0; mirror < (a == b ? 1 : 2); ++mirror) {
                        const int nr = mirror ? nb : na, nc = mirror ? na : nb;
                        const int off = row_search(A.indptr, A.indices, 3 * nr, 3 * nc);
#pragma unroll
                        for (int ri = 0; ri < 3; ++ri)
#pragma unroll
                            for (int ci = 0; ci < 3; ++ci) {
                                const double v = AR::value(mirror ? acc[m][ci * 3 + ri] : acc[m][ri * 3 + ci]);
                                const int64_t pos = block_entry(A.indptr, A.indices, nr, nc, ri, ci, off);
                                if (pos >= 0 && pos < s_nnz) atomicAdd(A.V + pos, v);
                                else flag |= FL_FLAG_BAD_INDEX;
                            }
                    }
                    continue;
                }
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const double v = AR::value(acc[m][i * 3 + k]);
                        const int r = 3 * a + i, c = 3 * b + k;
                        const int gr = 3 * na + i, gc = 3 * nb + k;
                        for (int mirror = 0; mirror < (a == b ? 1 : 2); ++mirror) {
                            const int rr = mirror ? c : r, cc = mirror ? r : c;
                            const int grr = mirror ? gc : gr, gcc = mirror ? gr : gc;
                            if (A.mode == 0) {
                                const int64_t o = e * cap + (int64_t)rr * NDOF + cc;
                                A.I[o] = grr;
                                A.J[o] = gcc;
                                A.V[o] = v;
                            } else {  // mode 1
                                const int ir = inv[slot * NDOF + rr], ic = inv[slot * NDOF + cc];
                                const int64_t pos = ((unsigned)ir < (unsigned)NDOF && (unsigned)ic < (unsigned)NDOF)
                                                        ? (int64_t)A.dg[e * cap + (int64_t)ir * NDOF + ic] : -1;
                                if (pos >= 0 && pos < s_nnz) atomicAdd(A.V + pos, v);
                                else flag |= FL_FLAG_BAD_INDEX;
                            }
                        }
                    }
            }
        }
    }
    if (flag) atomicOr(&s_flag, flag);
    __syncthreads();
    if (tid == 0 && s_flag && A.flags) atomicOr(A.flags, s_flag);
}

// Tuning table: Gauss points per shared-memory chunk of the contraction kernel, per
// (nodes per element, Gauss points), set by fl_SetAssemblyTuning (the autotuner); 0 = default.
constexpr int TUNE_SLOTS = 64;
struct TuneEntry { int npe, nq, qc; };
static TuneEntry g_tune[TUNE_SLOTS];
static std::mutex g_tune_mutex;

static int tuned_qc(int npe, int nq) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    for (int i = 0; i < TUNE_SLOTS; ++i)
        if (g_tune[i].npe == npe && g_tune[i].nq == nq) return g_tune[i].qc;
    return 0;
}

template <int NPE>
static int asm_qc(int nq) {
    constexpr int EPC = AsmCfg<NPE>::EPC;
    int qc = tuned_qc(NPE, nq);
    if (qc <= 0) qc = 32768 / (EPC * NPE * 27 * 8);
    if (qc < 1) qc = 1;
    if (qc > nq) qc = nq;
    return qc;
}

template <int NPE>
static size_t asm_smem_bytes(int nq, int qc) {
    constexpr int EPC = AsmCfg<NPE>::EPC;
    return sizeof(double) * ((size_t)EPC * nq * QSM + (size_t)qc * NPE * 3 + (size_t)EPC * qc * NPE * 27 +
                             (size_t)EPC * nq * 9) +
           sizeof(int) * ((size_t)EPC * NPE + (size_t)EPC * 3 * NPE);
}

// Elements per chunk for a scratch of `bytes` (a multiple of the CTA's element count).
static int64_t chunk_elements(size_t bytes, int nq, int epc) {
    int64_t ce = (int64_t)(bytes / (sizeof(double) * QSTRIDE * (size_t)nq));
    return ce - ce % epc;
}

// Arithmetic of the contraction kernel (fl_SetAssemblyArithmetic): float pairs by default, the
// faster of the two on GB300, within the FP64 path's accuracy bar
static std::atomic<int> g_arith{FL_ARITH_FLOAT_PAIR};

// Runs A and B over [0, nelem) in chunks of at most `chunk` elements through scratch Q.
template <int NPE, int MAT, bool DF>
static int run_chunks_t(AsmArgs A, double *Q, int64_t chunk, cudaStream_t stream) {
    constexpr int EPC = AsmCfg<NPE>::EPC, NT = AsmCfg<NPE>::TPE * EPC;
    A.qc = asm_qc<NPE>(A.nq);
    const size_t smem = asm_smem_bytes<NPE>(A.nq, A.qc);
    if (smem > 227 * 1024) return FL_ERR_UNSUPPORTED;
    { const int st = ensure_smem<contract_kernel<NPE, DF>>(smem); if (st != FL_OK) return st; }
    A.Q = Q;
    A.ldq = chunk * A.nq;
    for (int64_t e0 = 0; e0 < A.nelem; e0 += chunk) {
        A.e0 = e0;
        A.ne = A.nelem - e0 < chunk ? A.nelem - e0 : chunk;
        const int64_t nqp = A.ne * A.nq;
        qp_kernel<NPE, MAT><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
        contract_kernel<NPE, DF><<<(unsigned)((A.ne + EPC - 1) / EPC), NT, smem, stream>>>(A);
    }
    return launch_status();
}

template <int NPE, int MAT>
static int run_chunks(AsmArgs A, double *Q, int64_t chunk, cudaStream_t stream) {
    if (g_arith.load() == FL_ARITH_FLOAT_PAIR) return run_chunks_t<NPE, MAT, true>(A, Q, chunk, stream);
    return run_chunks_t<NPE, MAT, false>(A, Q, chunk, stream);
}

template <int NPE, int MAT>
static int launch_asm(AsmArgs A, double *scratch, size_t scratch_bytes, cudaStream_t stream) {
    constexpr int EPC = AsmCfg<NPE>::EPC;
    if (A.nelem == 0) return FL_OK;
    if (scratch) {  // caller-provided scratch
        const int64_t chunk = chunk_elements(scratch_bytes, A.nq, EPC);
        if (chunk < EPC) return FL_ERR_CAPACITY;
        return run_chunks<NPE, MAT>(A, scratch, chunk, stream);
    }
    int64_t chunk = chunk_elements(CHUNK_BYTES, A.nq, EPC);
    if (chunk > A.nelem) chunk = A.nelem + (EPC - A.nelem % EPC) % EPC;
    double *Q = nullptr;
    FL_CUDA_TRY(cudaMallocAsync((void **)&Q, sizeof(double) * QSTRIDE * (size_t)A.nq * chunk, stream));
    const int st = run_chunks<NPE, MAT>(A, Q, chunk, stream);
    const cudaError_t fe = cudaFreeAsync(Q, stream);
    if (st != FL_OK) return st;
    return fe == cudaSuccess ? FL_OK : FL_ERR_CUDA;
}

template <int MAT>
static int dispatch_asm(int npe, const AsmArgs &A, double *scratch, size_t scratch_bytes, cudaStream_t s) {
    switch (npe) {
        case 4: return launch_asm<4, MAT>(A, scratch, scratch_bytes, s);
        case 8: return launch_asm<8, MAT>(A, scratch, scratch_bytes, s);
        case 10: return launch_asm<10, MAT>(A, scratch, scratch_bytes, s);
        case 20: return launch_asm<20, MAT>(A, scratch, scratch_bytes, s);
        case 27: return launch_asm<27, MAT>(A, scratch, scratch_bytes, s);
        case 35: return launch_asm<35, MAT>(A, scratch, scratch_bytes, s);
        case 64: return launch_asm<64, MAT>(A, scratch, scratch_bytes, s);
        case 125: return launch_asm<125, MAT>(A, scratch, scratch_bytes, s);
        default: return FL_ERR_UNSUPPORTED;
    }
}

// Argument checks and mode selection shared by the entry points. scratch == nullptr: the
// scratch is taken from the stream-ordered allocator for the duration of the call.
int global_assembly_df(int mat, const double *points, const uint64_t *elements, const double *Eulerx,
                       const double *Jm, const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss,
                       int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t H_VoigtSize,
                       int64_t requires_geometry_update, int32_t *I_stiff, int32_t *J_stiff, double *V_stiff,
                       double *T, int recompute_sparsity_pattern, int squeeze_sparsity_pattern,
                       const int32_t *data_local_indices, const int32_t *data_global_indices, MatParams mp,
                       int *flags, double *scratch, size_t scratch_bytes, cudaStream_t stream,
                       const double *eparams = nullptr) {
    if (ndim != 3 || nvar != 3 || H_VoigtSize != 6) return FL_ERR_ARG;
    if (nelem < 0 || nnode <= 0) return FL_ERR_ARG;
    if (ngauss <= 0 || ngauss > 343) return FL_ERR_UNSUPPORTED;
    if (3 * nnode + 2 > INT32_MAX) return FL_ERR_UNSUPPORTED;
    if (mat != NEOHOOKEAN && mat != MOONEYRIVLIN && mat != NEARLYINCOMPRESSIBLEMR && mat != LINEARELASTIC)
        return FL_ERR_UNSUPPORTED;
    if (nelem == 0) return FL_OK;  // nothing is read or written
    if (!points || !elements || !Eulerx || !Jm || !AllGauss || !V_stiff || !T) return FL_ERR_ARG;
    AsmArgs A;
    A.points = points;
    A.elements = elements;
    A.Eulerx = Eulerx;
    A.Jm = Jm;
    A.Jmf = nullptr;
    A.utab = 0;
    A.w = AllGauss;
    A.nelem = nelem;
    A.nnode = nnode;
    A.nq = (int)ngauss;
    A.update = requires_geometry_update ? 1 : 0;
    A.I = nullptr;
    A.J = nullptr;
    A.V = V_stiff;
    A.T = T;
    A.indptr = A.indices = A.dl = A.dg = nullptr;
    A.mp = mp;
    A.eparams = eparams;
    A.flags = flags;
    A.Q = nullptr;
    A.e0 = A.ne = A.ldq = 0;
    A.qc = 1;
    if (recompute_sparsity_pattern) {
        if (!I_stiff || !J_stiff) return FL_ERR_ARG;
        A.mode = 0;
        A.I = I_stiff;
        A.J = J_stiff;
    } else {
        // the reference's wrapper passes indptr in I_stiff and indices in J_stiff
        if (!I_stiff || !J_stiff) return FL_ERR_ARG;
        A.indptr = I_stiff;
        A.indices = J_stiff;
        if (squeeze_sparsity_pattern) {
            A.mode = 2;
        } else {
            if (!data_local_indices || !data_global_indices) return FL_ERR_ARG;
            A.mode = 1;
            A.dl = data_local_indices;
            A.dg = data_global_indices;
        }
    }
    switch (mat) {
        case NEOHOOKEAN: return dispatch_asm<NEOHOOKEAN>((int)nodeperelem, A, scratch, scratch_bytes, stream);
        case MOONEYRIVLIN: return dispatch_asm<MOONEYRIVLIN>((int)nodeperelem, A, scratch, scratch_bytes, stream);
        case NEARLYINCOMPRESSIBLEMR:
            return dispatch_asm<NEARLYINCOMPRESSIBLEMR>((int)nodeperelem, A, scratch, scratch_bytes, stream);
        default: return dispatch_asm<LINEARELASTIC>((int)nodeperelem, A, scratch, scratch_bytes, stream);
    }
}

// Material of a C-ABI material number and its parameters from the reference's argument names:
// neo-Hookean and linear elastic (mu, lamb), Mooney-Rivlin (mu1, mu2, lamb), nearly incompressible
// Mooney-Rivlin (alpha, beta, kappa) = (mu1, mu2, lamb) (AOT_Assembler.py:62-71).
static int material_of(int material_number, double mu, double mu1, double mu2, double lamb, int *mat, MatParams *mp) {
    switch (material_number) {
        case FL_MATERIAL_NEOHOOKEAN: *mat = NEOHOOKEAN; *mp = {mu, lamb, 0.0}; return FL_OK;
        case FL_MATERIAL_MOONEYRIVLIN: *mat = MOONEYRIVLIN; *mp = {mu1, mu2, lamb}; return FL_OK;
        case FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN: *mat = NEARLYINCOMPRESSIBLEMR; *mp = {mu1, mu2, lamb}; return FL_OK;
        case FL_MATERIAL_LINEARELASTIC: *mat = LINEARELASTIC; *mp = {mu, lamb, 0.0}; return FL_OK;
        default: return FL_ERR_UNSUPPORTED;
    }
}

// ------------------------------------------------------------------------------------------------
// C. Mixed-precision contraction on the tensor cores (inexact-Newton Jacobian).
//
// Per element, K^T[(i,b,k), a] = sum_{(g,d)} U^T[(i,b,k),(g,d)] L[(g,d), a] with
// U_g[(i,d),(b,k)] = sum_e Ahat_g[(i,d),(k,e)] Jm[e][b][g] (from the FP64 Gauss-point data, formed
// in FP32) and L[(g,d), a] = Jm[d][a][g]. Both operands are split into three BF16 terms
// (x = hi + mid + lo, 24 significant bits together) and multiplied as the six products whose
// order is at least 2^-16 (hi*hi, hi*mid, mid*hi, hi*lo, lo*hi, mid*mid) with FP32 accumulation
// (mma.sync m16n8k16 bf16): the tangent to about FP32 accuracy (~1e-7 relative), enough for
// Newton to keep its FP64 iteration count on ill-conditioned problems (a two-term split, ~1e-5,
// slows Newton down). The result goes to FP32 CSR values (the Jacobian the PCG applies); the residual is
// formed in FP64 exactly as in contract_kernel. Rows are processed in chunks of MX_MC and the
// reduction dimension in chunks of MX_KC, so any element order fits in shared memory.
// ------------------------------------------------------------------------------------------------
constexpr int MX_NT = 128, MX_MC = 64, MX_KC = 96;

// x = hi + mid + lo, three BF16 terms with 8 significant bits each (FP32's 24 bits)
__device__ __forceinline__ void bf16_split3(float v, __nv_bfloat16 &hi, __nv_bfloat16 &mid, __nv_bfloat16 &lo) {
    hi = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(hi);
    mid = __float2bfloat16_rn(r1);
    lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void to_float(const double *a, float *b, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// reduction-chunk width of the split-BF16 kernel: the padded 3*nq, at most MX_KC (the operand
// buffers are sized by it, so short reductions leave room for more resident CTAs)
__host__ __device__ inline int mixed_kc(int nq) {
    const int kp = (3 * nq + 15) / 16 * 16;
    return kp < MX_KC ? kp : MX_KC;
}

// shared memory of the split-BF16 kernel without the U table (16-byte multiple)
template <int NPE>
__host__ __device__ inline size_t mixed_base_bytes(int nq) {
    constexpr int NP = (NPE + 7) / 8 * 8;
    const int ast = mixed_kc(nq) + 8;
    const size_t b = sizeof(float) * (((size_t)nq * QSM + 3) / 4 * 4) +
                     sizeof(__nv_bfloat16) * 3 * ((size_t)MX_MC * ast + (size_t)NP * ast) +
                     sizeof(int) * (NPE + 3 * NPE) + sizeof(int16_t) * NPE * NPE;
    return (b + 15) / 16 * 16;
}

template <int NPE>
__global__ void __launch_bounds__(MX_NT) contract_mixed_kernel(const AsmArgs A, float *V32) {
    constexpr int NDOF = 3 * NPE, M = 9 * NPE, NP = (NPE + 7) / 8 * 8, NT8 = NP / 8;
    const int nq = A.nq, K = 3 * nq;
    const int KC = mixed_kc(nq), AST = KC + 8;  // chunk width and padded row stride (bf16) of the operands
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *Qs = reinterpret_cast<float *>(smem_raw);                                // [nq][QSM]
    __nv_bfloat16 *Ah = reinterpret_cast<__nv_bfloat16 *>(Qs + ((size_t)nq * QSM + 3) / 4 * 4);  // [3][MX_MC][AST]
    __nv_bfloat16 *Am = Ah + MX_MC * AST;
    __nv_bfloat16 *Al = Am + MX_MC * AST;
    __nv_bfloat16 *Bh = Al + MX_MC * AST;                                            // [3][NP][AST]
    __nv_bfloat16 *Bm = Bh + NP * AST;
    __nv_bfloat16 *Bl = Bm + NP * AST;
    int *nodes = reinterpret_cast<int *>(Bl + NP * AST);                             // [NPE]
    int *inv = nodes + NPE;                                                          // [NDOF]
    int16_t *boff = reinterpret_cast<int16_t *>(inv + NDOF);                         // [NPE][NPE]
    float *Ut = reinterpret_cast<float *>(smem_raw + mixed_base_bytes<NPE>(nq));      // [nq][NPE][27] if utab
    __shared__ int s_flag;
    __shared__ int64_t s_nnz;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
    const int64_t cap = (int64_t)NDOF * NDOF;
    int flag = 0;
    if (tid == 0) {
        s_flag = 0;
        s_nnz = (int64_t)A.indptr[3 * A.nnode];
    }
    for (int64_t el = blockIdx.x; el < A.ne; el += gridDim.x) {
        const int64_t e = A.e0 + el;
        __syncthreads();  // previous element done with the shared buffers
        for (int a = tid; a < NPE; a += MX_NT) {
            uint64_t nd = A.elements[e * NPE + a];
            if (nd >= (uint64_t)A.nnode) {
                flag |= FL_FLAG_BAD_INDEX;
                nd = 0;
            }
            nodes[a] = (int)nd;
        }
        if (A.dl)
            for (int i = tid; i < NDOF; i += MX_NT) {
                const int v = A.dl[e * cap + (int64_t)i * NDOF];
                const int p = v / NDOF;
                if (v < 0 || p >= NDOF) flag |= FL_FLAG_BAD_INDEX;
                else inv[p] = i;
            }
        const double *q = A.Q + el * nq;
        for (int idx = tid; idx < nq * QSM; idx += MX_NT) {
            const int k = idx / nq, g = idx % nq;
            Qs[(size_t)g * QSM + k] = (float)q[k * A.ldq + g];
        }
        __syncthreads();
        if (!A.dl)  // offset of column node b in row node a; consecutive threads share a row
            for (int idx = tid; idx < NPE * NPE; idx += MX_NT) {
                const int off = row_search(A.indptr, A.indices, 3 * nodes[idx / NPE], 3 * nodes[idx % NPE]);
                boff[idx] = (int16_t)(off >= 0 && off < 32768 ? off : -1);
            }
        // residual in FP64
        if (A.update) {
            for (int r = tid; r < NDOF; r += MX_NT) {
                const int a = r / 3, i = r % 3;
                double t = 0.0;
                const double *qs = q + (size_t)(45 + i * 3) * A.ldq;  // S from the L2-resident scratch
                for (int g = 0; g < nq; ++g) {
                    t = fma(__ldg(A.Jm + (size_t)a * nq + g), qs[g], t);
                    t = fma(__ldg(A.Jm + ((size_t)NPE + a) * nq + g), qs[A.ldq + g], t);
                    t = fma(__ldg(A.Jm + ((size_t)2 * NPE + a) * nq + g), qs[2 * A.ldq + g], t);
                }
                atomicAdd(A.T + 3 * (int64_t)nodes[a] + i, t);
            }
        }
        if (A.utab)  // U_g[b][(i,d),k] of the whole element: all 27 entries of one (g, b) per work item,
                     // compile-time tensor indices, no divergence
            for (int it = tid; it < nq * NPE; it += MX_NT) {
                const int g = it / NPE, b = it % NPE;
                const float *qq = Qs + (size_t)g * QSM;
                const float j0 = __ldg(A.Jmf + (size_t)b * nq + g), j1 = __ldg(A.Jmf + ((size_t)NPE + b) * nq + g),
                            j2 = __ldg(A.Jmf + ((size_t)2 * NPE + b) * nq + g);
                float *uo = Ut + ((size_t)g * NPE + b) * 27;
#pragma unroll
                for (int II = 0; II < 9; ++II)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        uo[II * 3 + k] = fmaf(qq[sym9(II, k * 3 + 0)], j0,
                                              fmaf(qq[sym9(II, k * 3 + 1)], j1, qq[sym9(II, k * 3 + 2)] * j2));
            }
        for (int m0 = 0; m0 < M; m0 += MX_MC) {
            float acc[NT8][4];
#pragma unroll
            for (int t = 0; t < NT8; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
            for (int k0 = 0; k0 < K; k0 += KC) {
                const int kc = min(KC, K - k0), kcp = (kc + 15) / 16 * 16;
                __syncthreads();  // previous chunk's MMAs done
                // A chunk: rows r = m0 + rr -> (i, b, k) with r = (i*NPE + b)*3 + k; cols c = k0 + cc -> (g, d)
                for (int idx = tid; idx < MX_MC * kcp; idx += MX_NT) {
                    const int rr = idx / kcp, cc = idx % kcp, r = m0 + rr, c = k0 + cc;
                    float v = 0.f;
                    if (r < M && cc < kc) {
                        const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
                        const int g = c / 3, d = c % 3, I = i * 3 + d;
                        if (A.utab) {
                            v = Ut[((size_t)g * NPE + b) * 27 + I * 3 + k];
                        } else {
                            const float *qq = Qs + (size_t)g * QSM;  // U in FP32: the tangent's target accuracy
                            v = fmaf(qq[sym9(I, k * 3 + 0)], __ldg(A.Jmf + ((size_t)0 * NPE + b) * nq + g),
                                     fmaf(qq[sym9(I, k * 3 + 1)], __ldg(A.Jmf + ((size_t)1 * NPE + b) * nq + g),
                                          qq[sym9(I, k * 3 + 2)] * __ldg(A.Jmf + ((size_t)2 * NPE + b) * nq + g)));
                        }
                    }
                    bf16_split3(v, Ah[rr * AST + cc], Am[rr * AST + cc], Al[rr * AST + cc]);
                }
                // B chunk, stored [n][k]: B[(g,d), a] = Jm[d][a][g]
                for (int idx = tid; idx < NP * kcp; idx += MX_NT) {
                    const int n = idx / kcp, cc = idx % kcp, c = k0 + cc;
                    float v = 0.f;
                    if (n < NPE && cc < kc) v = __ldg(A.Jmf + ((size_t)(c % 3) * NPE + n) * nq + c / 3);
                    bf16_split3(v, Bh[n * AST + cc], Bm[n * AST + cc], Bl[n * AST + cc]);
                }
                __syncthreads();
                // warp w: m-tile w of the chunk (16 rows), all n-tiles
                const int mr = warp * 16;
                for (int ks = 0; ks < kcp; ks += 16) {
                    uint32_t ah[4], am[4], al[4];
                    const int c0 = ks + tig * 2;
                    auto ldA = [&](const __nv_bfloat16 *X, uint32_t *f) {
                        f[0] = *reinterpret_cast<const uint32_t *>(X + (mr + gid) * AST + c0);
                        f[1] = *reinterpret_cast<const uint32_t *>(X + (mr + gid + 8) * AST + c0);
                        f[2] = *reinterpret_cast<const uint32_t *>(X + (mr + gid) * AST + c0 + 8);
                        f[3] = *reinterpret_cast<const uint32_t *>(X + (mr + gid + 8) * AST + c0 + 8);
                    };
                    ldA(Ah, ah);
                    ldA(Am, am);
                    ldA(Al, al);
#pragma unroll
                    for (int t = 0; t < NT8; ++t) {
                        uint32_t bh[2], bm[2], bl[2];
                        const int n = t * 8 + gid;
                        bh[0] = *reinterpret_cast<const uint32_t *>(Bh + n * AST + c0);
                        bh[1] = *reinterpret_cast<const uint32_t *>(Bh + n * AST + c0 + 8);
                        bm[0] = *reinterpret_cast<const uint32_t *>(Bm + n * AST + c0);
                        bm[1] = *reinterpret_cast<const uint32_t *>(Bm + n * AST + c0 + 8);
                        bl[0] = *reinterpret_cast<const uint32_t *>(Bl + n * AST + c0);
                        bl[1] = *reinterpret_cast<const uint32_t *>(Bl + n * AST + c0 + 8);
                        // smallest terms first
                        mma_bf16(acc[t], am, bm);
                        mma_bf16(acc[t], al, bh);
                        mma_bf16(acc[t], ah, bl);
                        mma_bf16(acc[t], am, bh);
                        mma_bf16(acc[t], ah, bm);
                        mma_bf16(acc[t], ah, bh);
                    }
                }
            }
            // scatter: C[r, a] = K_e[(a,i),(b,k)]
#pragma unroll
            for (int t = 0; t < NT8; ++t)
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int r = m0 + warp * 16 + gid + (h >> 1) * 8, a = t * 8 + tig * 2 + (h & 1);
                    if (r >= M || a >= NPE) continue;
                    const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
                    int64_t pos = -1;
                    if (A.dl) {
                        const int ir = inv[3 * a + i], ic = inv[3 * b + k];
                        if ((unsigned)ir < (unsigned)NDOF && (unsigned)ic < (unsigned)NDOF)
                            pos = (int64_t)A.dg[e * cap + (int64_t)ir * NDOF + ic];
                    } else {
                        pos = block_entry(A.indptr, A.indices, nodes[a], nodes[b], i, k, boff[a * NPE + b]);
                    }
                    if (pos >= 0 && pos < s_nnz) atomicAdd(V32 + pos, acc[t][h]);
                    else flag |= FL_FLAG_BAD_INDEX;
                }
        }
    }
    if (flag) atomicOr(&s_flag, flag);
    __syncthreads();
    if (tid == 0 && s_flag && A.flags) atomicOr(A.flags, s_flag);
}

// ------------------------------------------------------------------------------------------------
// D. The split-BF16 tangent on the fifth-generation tensor cores (tcgen05). Same operands and
// products as contract_mixed_kernel, organised for the tensor core: per element and 128-row tile
// of K^T[(i,b,k), a], the three BF16 terms of U (A operand, 128 x KC) and of Jm (B operand,
// NB x KC, NB = NPE padded to 16) are written to shared memory in the K-major core-matrix layout;
// one thread issues the six products per 16-wide K step as tcgen05.mma into an FP32 accumulator
// in tensor memory and commits them to an mbarrier; after the last K chunk each warp reads its 32
// accumulator rows with tcgen05.ld and scatters them. The B operand depends only on the element
// type: with a single K chunk it is built once per CTA. Waits are bounded (on expiry the element
// is skipped and FL_FLAG_BAD_INDEX raised, so the call reports an error).
// ------------------------------------------------------------------------------------------------
constexpr int TC_MT = 128;
constexpr long long TC_WAIT = 1ll << 22;

template <int NPE>
__host__ __device__ constexpr int tc_nb() { return (NPE + 15) / 16 * 16; }

template <int NPE>
__host__ __device__ constexpr int tc_tmem_cols() {
    const int n = (tc_nb<NPE>() + 31) / 32 * 32;
    return n <= 32 ? 32 : (n <= 64 ? 64 : (n <= 128 ? 128 : 256));
}

// shared memory: Qs float [nq][QSM] | A terms 3 x [128][KC] bf16 | B terms 3 x [NB][KC] bf16 |
// nodes, inv, boff
template <int NPE>
__host__ __device__ inline size_t tc_smem_bytes(int nq) {
    const int kc = mixed_kc(nq);
    const size_t b = sizeof(float) * (((size_t)nq * QSM + 31) / 32 * 32) +
                     sizeof(__nv_bfloat16) * 3 * ((size_t)TC_MT * kc + (size_t)tc_nb<NPE>() * kc) +
                     sizeof(int) * (NPE + 3 * NPE) + sizeof(int16_t) * NPE * NPE;
    return (b + 127) / 128 * 128;
}

template <int NPE>
__global__ void __launch_bounds__(128) contract_tc_kernel(const AsmArgs A, float *V32) {
    constexpr int NDOF = 3 * NPE, M = 9 * NPE, NB = (NPE + 15) / 16 * 16;
    const int nq = A.nq, K = 3 * nq, KC = mixed_kc(nq);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *Qs = reinterpret_cast<float *>(smem_raw);  // [nq][QSM]
    __nv_bfloat16 *At[3], *Bt[3];
    At[0] = reinterpret_cast<__nv_bfloat16 *>(smem_raw + sizeof(float) * (((size_t)nq * QSM + 31) / 32 * 32));
    At[1] = At[0] + TC_MT * KC;
    At[2] = At[1] + TC_MT * KC;
    Bt[0] = At[2] + TC_MT * KC;
    Bt[1] = Bt[0] + NB * KC;
    Bt[2] = Bt[1] + NB * KC;
    int *nodes = reinterpret_cast<int *>(Bt[2] + NB * KC);  // [NPE]
    int *inv = nodes + NPE;                                 // [NDOF]
    int16_t *boff = reinterpret_cast<int16_t *>(inv + NDOF);  // [NPE][NPE]
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t taddr_s;
    __shared__ int s_flag;
    __shared__ int64_t s_nnz;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t cap = (int64_t)NDOF * NDOF;
    constexpr int TCOLS = tc_tmem_cols<NPE>();
    int flag = 0;
    uint32_t phase = 0;
    if (tid == 0) {
        s_flag = 0;
        s_nnz = (int64_t)A.indptr[3 * A.nnode];
        tc::mbar_init(&mbar, 1);
    }
    if (warp == 0) tc::tmem_alloc(&taddr_s, TCOLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = taddr_s;
    const uint32_t idesc = tc::idesc_bf16_f32(TC_MT, NB);
    const uint32_t sbo = (uint32_t)(KC / 8) * 128;
    const bool b_once = K <= KC;  // one K chunk: the Jm operand is built once per CTA
    bool b_built = false;
    bool ok = true;

    auto build_b = [&](int k0, int kc) {
        for (int idx = tid; idx < NB * KC; idx += 128) {
            const int n = idx / KC, cc = idx % KC, c = k0 + cc;
            float v = 0.f;
            if (n < NPE && cc < kc) v = __ldg(A.Jmf + ((size_t)(c % 3) * NPE + n) * nq + c / 3);
            const uint32_t off = tc::kmajor_offset(n, cc, KC) / 2;
            bf16_split3(v, Bt[0][off], Bt[1][off], Bt[2][off]);
        }
    };

    for (int64_t el = blockIdx.x; el < A.ne && ok; el += gridDim.x) {
        const int64_t e = A.e0 + el;
        __syncthreads();  // previous element done with the shared buffers
        for (int a = tid; a < NPE; a += 128) {
            uint64_t nd = A.elements[e * NPE + a];
            if (nd >= (uint64_t)A.nnode) {
                flag |= FL_FLAG_BAD_INDEX;
                nd = 0;
            }
            nodes[a] = (int)nd;
        }
        if (A.dl)
            for (int i = tid; i < NDOF; i += 128) {
                const int v = A.dl[e * cap + (int64_t)i * NDOF];
                const int p = v / NDOF;
                if (v < 0 || p >= NDOF) flag |= FL_FLAG_BAD_INDEX;
                else inv[p] = i;
            }
        const double *q = A.Q + el * nq;
        for (int idx = tid; idx < nq * QSM; idx += 128) {
            const int k = idx / nq, g = idx % nq;
            Qs[(size_t)g * QSM + k] = (float)q[k * A.ldq + g];
        }
        __syncthreads();
        if (!A.dl)  // offset of column node b in row node a; consecutive threads share a row
            for (int idx = tid; idx < NPE * NPE; idx += 128) {
                const int off = row_search(A.indptr, A.indices, 3 * nodes[idx / NPE], 3 * nodes[idx % NPE]);
                boff[idx] = (int16_t)(off >= 0 && off < 32768 ? off : -1);
            }
        // residual in FP64
        if (A.update) {
            for (int r = tid; r < NDOF; r += 128) {
                const int a = r / 3, i = r % 3;
                double t = 0.0;
                const double *qs = q + (size_t)(45 + i * 3) * A.ldq;
                for (int g = 0; g < nq; ++g) {
                    t = fma(__ldg(A.Jm + (size_t)a * nq + g), qs[g], t);
                    t = fma(__ldg(A.Jm + ((size_t)NPE + a) * nq + g), qs[A.ldq + g], t);
                    t = fma(__ldg(A.Jm + ((size_t)2 * NPE + a) * nq + g), qs[2 * A.ldq + g], t);
                }
                atomicAdd(A.T + 3 * (int64_t)nodes[a] + i, t);
            }
        }
        for (int m0 = 0; m0 < M; m0 += TC_MT) {
            for (int k0 = 0; k0 < K; k0 += KC) {
                const int kc = min(KC, K - k0);
                // operands of this chunk (the previous chunk's MMAs completed: waited below)
                for (int idx = tid; idx < TC_MT * KC; idx += 128) {
                    const int rr = idx / KC, cc = idx % KC, r = m0 + rr, c = k0 + cc;
                    float v = 0.f;
                    if (r < M && cc < kc) {
                        const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
                        const int g = c / 3, d = c % 3, I = i * 3 + d;
                        const float *qq = Qs + (size_t)g * QSM;  // U in FP32: the tangent's target accuracy
                        v = fmaf(qq[sym9(I, k * 3 + 0)], __ldg(A.Jmf + ((size_t)0 * NPE + b) * nq + g),
                                 fmaf(qq[sym9(I, k * 3 + 1)], __ldg(A.Jmf + ((size_t)1 * NPE + b) * nq + g),
                                      qq[sym9(I, k * 3 + 2)] * __ldg(A.Jmf + ((size_t)2 * NPE + b) * nq + g)));
                    }
                    const uint32_t off = tc::kmajor_offset(rr, cc, KC) / 2;
                    bf16_split3(v, At[0][off], At[1][off], At[2][off]);
                }
                if (!b_once || !b_built) {
                    build_b(k0, kc);
                    b_built = true;
                }
                tc::fence_async_smem();
                tc::fence_before_sync();
                __syncthreads();
                tc::fence_after_sync();
                if (tid == 0) {
                    // the six products of order >= 2^-16, smallest first (term 0 = hi, 1 = mid, 2 = lo)
                    const int pa[6] = {1, 2, 0, 1, 0, 0}, pb[6] = {1, 0, 2, 0, 1, 0};
                    for (int ks = 0; ks < KC / 16; ++ks) {
                        if (16 * ks >= kc) break;
                        for (int t = 0; t < 6; ++t) {
                            const uint64_t da = tc::smem_desc(At[pa[t]] + ks * 16 * 8, 128, sbo);
                            const uint64_t db = tc::smem_desc(Bt[pb[t]] + ks * 16 * 8, 128, sbo);
                            tc::mma_bf16(taddr, da, db, idesc, k0 > 0 || ks > 0 || t > 0);
                        }
                    }
                    tc::mma_commit(&mbar);
                }
                ok = __syncthreads_and(tc::mbar_wait(&mbar, phase & 1, TC_WAIT)) != 0;  // uniform in the CTA
                ++phase;
                tc::fence_after_sync();
                if (!ok) break;
            }
            if (!ok) {
                flag |= FL_FLAG_BAD_INDEX;  // reported as an error by the caller
                break;
            }
            // read back: warp w holds rows m0 + 32 w + lane of the tile
            const int r = m0 + 32 * warp + lane;
            const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
#pragma unroll 1
            for (int c0 = 0; c0 < NB; c0 += 32) {
                float v[32];
                tc::tmem_ld32(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
                if (r >= M) continue;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int a = c0 + j;  // C[r, a] = K_e[(a,i),(b,k)]
                    if (a >= NPE) continue;
                    int64_t pos = -1;
                    if (A.dl) {
                        const int ir = inv[3 * a + i], ic = inv[3 * b + k];
                        if ((unsigned)ir < (unsigned)NDOF && (unsigned)ic < (unsigned)NDOF)
                            pos = (int64_t)A.dg[e * cap + (int64_t)ir * NDOF + ic];
                    } else {
                        pos = block_entry(A.indptr, A.indices, nodes[a], nodes[b], i, k, boff[a * NPE + b]);
                    }
                    if (pos >= 0 && pos < s_nnz) atomicAdd(V32 + pos, v[j]);
                    else flag |= FL_FLAG_BAD_INDEX;
                }
            }
            tc::fence_before_sync();
            __syncthreads();  // every warp has read the accumulator before the next tile's MMAs
            tc::fence_after_sync();
        }
    }
    if (flag) atomicOr(&s_flag, flag);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, TCOLS);
    if (tid == 0 && s_flag && A.flags) atomicOr(A.flags, s_flag);
}

template <int NPE>
static size_t mixed_smem_bytes(int nq, bool utab) {
    return mixed_base_bytes<NPE>(nq) + (utab ? sizeof(float) * (size_t)nq * NPE * 27 : 0);
}

template <int NPE, int MAT>
static int launch_mixed(AsmArgs A, float *V32, cudaStream_t stream) {
    if (A.nelem == 0) return FL_OK;
    A.utab = 0;
    const size_t smem = tc_smem_bytes<NPE>(A.nq);
    if (smem > 227 * 1024) return FL_ERR_UNSUPPORTED;
    { const int st = ensure_smem<contract_tc_kernel<NPE>>(smem); if (st != FL_OK) return st; }
    int64_t chunk = chunk_elements(CHUNK_BYTES, A.nq, 1);
    if (chunk > A.nelem) chunk = A.nelem;
    double *Q = nullptr;  // Gauss-point scratch, then the FP32 copy of Jm
    const size_t qbytes = (sizeof(double) * QSTRIDE * (size_t)A.nq * chunk + 255) & ~(size_t)255;
    const int64_t njm = (int64_t)3 * NPE * A.nq;
    FL_CUDA_TRY(cudaMallocAsync((void **)&Q, qbytes + sizeof(float) * (size_t)njm, stream));
    A.Q = Q;
    A.ldq = chunk * A.nq;
    float *Jmf = reinterpret_cast<float *>(reinterpret_cast<char *>(Q) + qbytes);
    to_float<<<(unsigned)((njm + 255) / 256), 256, 0, stream>>>(A.Jm, Jmf, njm);
    A.Jmf = Jmf;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int64_t e0 = 0; e0 < A.nelem; e0 += chunk) {
        A.e0 = e0;
        A.ne = A.nelem - e0 < chunk ? A.nelem - e0 : chunk;
        const int64_t nqp = A.ne * A.nq;
        qp_kernel<NPE, MAT><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
        const int64_t grid = std::min<int64_t>(A.ne, (int64_t)sms * 8);
        contract_tc_kernel<NPE><<<(unsigned)grid, 128, smem, stream>>>(A, V32);
    }
    const int st = launch_status();
    const cudaError_t fe = cudaFreeAsync(Q, stream);
    if (st != FL_OK) return st;
    return fe == cudaSuccess ? FL_OK : FL_ERR_CUDA;
}

template <int MAT>
static int mixed_dispatch(int npe, const AsmArgs &A, float *V32, cudaStream_t s) {
    switch (npe) {
        case 4: return launch_mixed<4, MAT>(A, V32, s);
        case 8: return launch_mixed<8, MAT>(A, V32, s);
        case 10: return launch_mixed<10, MAT>(A, V32, s);
        case 20: return launch_mixed<20, MAT>(A, V32, s);
        case 27: return launch_mixed<27, MAT>(A, V32, s);
        case 35: return launch_mixed<35, MAT>(A, V32, s);
        case 64: return launch_mixed<64, MAT>(A, V32, s);
        case 125: return launch_mixed<125, MAT>(A, V32, s);
        default: return FL_ERR_UNSUPPORTED;
    }
}

// ------------------------------------------------------------------------------------------------
// Allocation-free variant. Its Gauss-point scratch is this file-scope device array (every GPU that
// loads the library holds it until the process exits). Host code cannot use the array's name as
// a device address, so the address is looked up once per device with cudaGetSymbolAddress and
// cached. Every call shares the array: the Gauss-point kernel writes every entry the contraction
// kernel reads, so nothing needs clearing between calls, but calls that overlap on the GPU (other
// streams, other host threads) race on it.
// ------------------------------------------------------------------------------------------------
static __device__ __align__(256) double g_noalloc_scratch[FL_NOALLOC_SCRATCH_BYTES / sizeof(double)];

constexpr int NOALLOC_MAX_DEVICES = 256;
static void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(double **out) {
    int dev = 0;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return FL_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FL_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    *out = (double *)g_noalloc_ptr[dev];
    return FL_OK;
}

}  // namespace fl

extern "C" {

int fl_GlobalAssemblyDF_noalloc(int material_number, FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mu3; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e;
    (void)anisotropic_orientations;
    fl::MatParams mp;
    int mat = 0;
    if (fl::material_of(material_number, mu, mu1, mu2, lamb, &mat, &mp) != FL_OK) return FL_ERR_UNSUPPORTED;
    if (ngauss <= 0 || ngauss > 343 || nelem < 0) return FL_ERR_ARG;
    // the whole mesh must fit the array in one pass: nelem * ngauss Gauss points of 54 doubles
    if ((double)nelem * (double)ngauss * fl::QSTRIDE * sizeof(double) > (double)FL_NOALLOC_SCRATCH_BYTES)
        return FL_ERR_CAPACITY;
    if (nelem == 0) return FL_OK;
    double *scratch = nullptr;
    const int st = fl::noalloc_scratch(&scratch);
    if (st != FL_OK) return st;
    return fl::global_assembly_df(mat, points, elements, Eulerx, Jm, AllGauss, ndim, nvar, ngauss, nelem, nodeperelem,
                                  nnode, H_VoigtSize, requires_geometry_update, I_stiff, J_stiff, V_stiff, T,
                                  recompute_sparsity_pattern, squeeze_sparsity_pattern, data_local_indices,
                                  data_global_indices, mp, flags, scratch, FL_NOALLOC_SCRATCH_BYTES,
                                  (cudaStream_t)stream);
}

int fl_GlobalAssemblyDF_Mixed(int material_number, const double *points, const uint64_t *elements,
                              const double *Eulerx, const double *Jm, const double *AllGauss, int64_t ngauss,
                              int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t requires_geometry_update,
                              const int32_t *indptr, const int32_t *indices, const int32_t *data_local_indices,
                              const int32_t *data_global_indices, float *V_stiff, double *T, double mu, double mu1,
                              double mu2, double lamb, const double *element_params, int *flags,
                              fl_stream_t stream) {
    if (nelem < 0 || nnode <= 0 || ngauss <= 0 || ngauss > 343) return FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    const bool maps = data_local_indices && data_global_indices;
    if (!points || !elements || !Eulerx || !Jm || !AllGauss || !indptr || !V_stiff || !T) return FL_ERR_ARG;
    if (!maps && !indices) return FL_ERR_ARG;
    if (3 * nnode + 2 > INT32_MAX) return FL_ERR_UNSUPPORTED;
    fl::AsmArgs A;
    A.points = points;
    A.elements = elements;
    A.Eulerx = Eulerx;
    A.Jm = Jm;
    A.Jmf = nullptr;
    A.utab = 0;
    A.w = AllGauss;
    A.nelem = nelem;
    A.nnode = nnode;
    A.nq = (int)ngauss;
    A.update = requires_geometry_update ? 1 : 0;
    A.mode = 1;
    A.qc = 1;
    A.I = A.J = nullptr;
    A.V = nullptr;
    A.T = T;
    A.indptr = indptr;
    A.indices = indices;
    A.dl = maps ? data_local_indices : nullptr;
    A.dg = maps ? data_global_indices : nullptr;
    A.eparams = element_params;
    A.flags = flags;
    A.Q = nullptr;
    A.e0 = A.ne = A.ldq = 0;
    int mat = 0;
    if (fl::material_of(material_number, mu, mu1, mu2, lamb, &mat, &A.mp) != FL_OK) return FL_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    switch (mat) {
        case fl::NEOHOOKEAN: return fl::mixed_dispatch<fl::NEOHOOKEAN>((int)nodeperelem, A, V_stiff, s);
        case fl::MOONEYRIVLIN: return fl::mixed_dispatch<fl::MOONEYRIVLIN>((int)nodeperelem, A, V_stiff, s);
        case fl::NEARLYINCOMPRESSIBLEMR:
            return fl::mixed_dispatch<fl::NEARLYINCOMPRESSIBLEMR>((int)nodeperelem, A, V_stiff, s);
        default: return fl::mixed_dispatch<fl::LINEARELASTIC>((int)nodeperelem, A, V_stiff, s);
    }
}

int fl_GlobalAssemblyDF_Batched(int material_number, const double *points, const uint64_t *elements,
                                const double *Eulerx, const double *Jm, const double *AllGauss, int64_t ngauss,
                                int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t requires_geometry_update,
                                const double *element_params, const int32_t *indptr, const int32_t *indices,
                                const int32_t *data_local_indices, const int32_t *data_global_indices,
                                double *V_stiff, double *T, int *flags, fl_stream_t stream) {
    if (!element_params && nelem > 0) return FL_ERR_ARG;
    const int squeeze = (data_local_indices == nullptr || data_global_indices == nullptr) ? 1 : 0;
    int mat = 0;
    fl::MatParams unused;
    if (fl::material_of(material_number, 0, 0, 0, 0, &mat, &unused) != FL_OK) return FL_ERR_UNSUPPORTED;
    return fl::global_assembly_df(mat, points, elements, Eulerx, Jm, AllGauss, 3, 3, ngauss, nelem, nodeperelem, nnode,
                                  6, requires_geometry_update, const_cast<int32_t *>(indptr),
                                  const_cast<int32_t *>(indices), V_stiff, T, 0, squeeze, data_local_indices,
                                  data_global_indices, fl::MatParams{0, 0, 0}, flags, nullptr, 0, (cudaStream_t)stream,
                                  element_params);
}

int fl_SetAssemblyArithmetic(int arithmetic) {
    if (arithmetic != FL_ARITH_FP64 && arithmetic != FL_ARITH_FLOAT_PAIR) return FL_ERR_ARG;
    fl::g_arith.store(arithmetic);
    return FL_OK;
}

int fl_GetAssemblyArithmetic(void) { return fl::g_arith.load(); }

int fl_SetAssemblyTuning(int64_t nodeperelem, int64_t ngauss, int gauss_chunk) {
    std::lock_guard<std::mutex> lock(fl::g_tune_mutex);
    int freeslot = -1;
    for (int i = 0; i < fl::TUNE_SLOTS; ++i) {
        if (fl::g_tune[i].npe == nodeperelem && fl::g_tune[i].nq == ngauss) {
            fl::g_tune[i].qc = gauss_chunk;
            return FL_OK;
        }
        if (freeslot < 0 && fl::g_tune[i].npe == 0) freeslot = i;
    }
    if (freeslot < 0) return FL_ERR_CAPACITY;
    fl::g_tune[freeslot] = fl::TuneEntry{(int)nodeperelem, (int)ngauss, gauss_chunk};
    return FL_OK;
}

const char *fl_status_string(int status) {
    switch (status) {
        case FL_OK: return "ok";
        case FL_ERR_ARG: return "invalid argument";
        case FL_ERR_UNSUPPORTED: return "unsupported element size, Gauss point count or material";
        case FL_ERR_CUDA: return "CUDA error";
        case FL_ERR_MESH: return "mesh rejected: a node belongs to no element";
        case FL_ERR_CAPACITY: return "output or workspace buffer too small";
        default: return "unknown status";
    }
}

int fl_GlobalAssemblyDF__NeoHookean_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mu1; (void)mu2; (void)mu3; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3;
    (void)eps_e; (void)anisotropic_orientations;
    fl::MatParams mp{mu, lamb, 0.0};
    return fl::global_assembly_df(fl::NEOHOOKEAN, points, elements, Eulerx, Jm, AllGauss, ndim, nvar, ngauss, nelem,
                                  nodeperelem, nnode, H_VoigtSize, requires_geometry_update, I_stiff, J_stiff, V_stiff, T,
                                  recompute_sparsity_pattern, squeeze_sparsity_pattern, data_local_indices,
                                  data_global_indices, mp, flags, nullptr, 0, (cudaStream_t)stream);
}

int fl_GlobalAssemblyDF__NearlyIncompressibleMooneyRivlin_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mu; (void)mu3; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e;
    (void)anisotropic_orientations;
    fl::MatParams mp{mu1, mu2, lamb};  // (alpha, beta, kappa)
    return fl::global_assembly_df(fl::NEARLYINCOMPRESSIBLEMR, points, elements, Eulerx, Jm, AllGauss, ndim, nvar,
                                  ngauss, nelem, nodeperelem, nnode, H_VoigtSize, requires_geometry_update, I_stiff,
                                  J_stiff, V_stiff, T, recompute_sparsity_pattern, squeeze_sparsity_pattern,
                                  data_local_indices, data_global_indices, mp, flags, nullptr, 0, (cudaStream_t)stream);
}

int fl_GlobalAssemblyDF__LinearElastic_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mu1; (void)mu2; (void)mu3; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3;
    (void)eps_e; (void)anisotropic_orientations;
    fl::MatParams mp{mu, lamb, 0.0};
    return fl::global_assembly_df(fl::LINEARELASTIC, points, elements, Eulerx, Jm, AllGauss, ndim, nvar, ngauss,
                                  nelem, nodeperelem, nnode, H_VoigtSize, requires_geometry_update, I_stiff, J_stiff,
                                  V_stiff, T, recompute_sparsity_pattern, squeeze_sparsity_pattern, data_local_indices,
                                  data_global_indices, mp, flags, nullptr, 0, (cudaStream_t)stream);
}

int fl_GlobalAssemblyDF__MooneyRivlin_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mu; (void)mu3; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e;
    (void)anisotropic_orientations;
    fl::MatParams mp{mu1, mu2, lamb};
    return fl::global_assembly_df(fl::MOONEYRIVLIN, points, elements, Eulerx, Jm, AllGauss, ndim, nvar, ngauss, nelem,
                                  nodeperelem, nnode, H_VoigtSize, requires_geometry_update, I_stiff, J_stiff, V_stiff, T,
                                  recompute_sparsity_pattern, squeeze_sparsity_pattern, data_local_indices,
                                  data_global_indices, mp, flags, nullptr, 0, (cudaStream_t)stream);
}

}  // extern "C"
