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
#include "fl_reftensor.cuh"
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
    const double *orient;   // fibre direction per element [nelem][3] (transversely isotropic material)
    // float-pair kinematics (optional): per node X hi, X lo, u hi, u lo [nnode][12] floats, and
    // the shape-function gradients as pairs [3][npe][nq]
    const float *npair;
    const float2 *jmp;
    int *flags;
    const int32_t *boff;  // optional per-element block offsets [nelem][npe][npe] (fl_ElementBlockOffsets)
    const double *geo = nullptr;  // optional reference geometry [10][nelem * nq] (fl_ReferenceGeometry)
    double *Q;       // scratch [QSTRIDE][ldq]
    float *Qf;       // split-BF16 path: FP32 tangent part [45][ldq] (Q then holds S [9][ldq])
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

// Pulled-back tangent of one Gauss point in arithmetic T from the FP64 kinematics and material:
// Ahat[(i,d),(k,e)] = detJ [ d_ik (c1 GG + GsG)[d][e] + c1 G[k][d] G[i][e] + c2 G[i][d] G[k][e]
//                          + cbb (2 bG[i][d] bG[k][e] - b_ik GbG[d][e] - bG[k][d] bG[i][e]) ] (+ the
// nearly incompressible material's terms), handed to out.put(sym9(I, K), value), I = 3 i + d,
// K = 3 k + e
template <typename T, int MAT, class OUT>
__device__ __forceinline__ void pulled_back_tangent(const double *Gd, const double *sigd, const double *bd,
                                                    const ExtraTangent &exd, double c1d, double c2d, double cbbd,
                                                    double detJd, const OUT &out) {
    constexpr bool NIMR = MAT == NEARLYINCOMPRESSIBLEMR;
    constexpr bool BB = MAT == MOONEYRIVLIN || MAT == ANISOTROPICMR1;    // the cbb (b b) terms
    constexpr bool GT = NIMR || MAT == ANISOTROPICMR1;                    // the g terms (kgI, kg4)
    T G[9], sig[6], b[6], g6[6];
#pragma unroll
    for (int i = 0; i < 9; ++i) G[i] = (T)Gd[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        sig[i] = (T)sigd[i];
        b[i] = (T)bd[i];
        g6[i] = (T)exd.g[i];
    }
    const T c1 = (T)c1d, c2 = (T)c2d, cbb = (T)cbbd, detJ = (T)detJd;
    const T kbI = (T)exd.kbI, kgI = (T)exd.kgI, kgg = (T)exd.kgg, kg4 = (T)exd.kg4;
    // GG = G^T G, GsG = G^T sigma G, bG = b G, GbG = G^T b G, gG = g G, GgG = G^T g G
    T GG[9], GsG[9], sG[9], bG[9], GbG[9], gG[9], GgG[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            sG[i * 3 + d] = fma(sig[s6(i, 0)], G[0 * 3 + d], fma(sig[s6(i, 1)], G[1 * 3 + d], sig[s6(i, 2)] * G[2 * 3 + d]));
            if (BB || NIMR)
                bG[i * 3 + d] = fma(b[s6(i, 0)], G[0 * 3 + d], fma(b[s6(i, 1)], G[1 * 3 + d], b[s6(i, 2)] * G[2 * 3 + d]));
            if (GT)
                gG[i * 3 + d] = fma(g6[s6(i, 0)], G[0 * 3 + d], fma(g6[s6(i, 1)], G[1 * 3 + d], g6[s6(i, 2)] * G[2 * 3 + d]));
        }
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int e2 = d; e2 < 3; ++e2) {
            GG[d * 3 + e2] = fma(G[d], G[e2], fma(G[3 + d], G[3 + e2], G[6 + d] * G[6 + e2]));
            // no geometric stiffness for the linear elastic material (the reference builds that
            // assembler without it, AOT_Assembler.py:74-81)
            GsG[d * 3 + e2] = MAT == LINEARELASTIC ? (T)0 : fma(G[d], sG[e2], fma(G[3 + d], sG[3 + e2], G[6 + d] * sG[6 + e2]));
            if (BB) GbG[d * 3 + e2] = fma(G[d], bG[e2], fma(G[3 + d], bG[3 + e2], G[6 + d] * bG[6 + e2]));
            if (GT) GgG[d * 3 + e2] = fma(G[d], gG[e2], fma(G[3 + d], gG[3 + e2], G[6 + d] * gG[6 + e2]));
        }
#pragma unroll
    for (int I = 0; I < 9; ++I)
#pragma unroll
        for (int K = I; K < 9; ++K) {
            const int i = I / 3, d = I % 3, k = K / 3, e2 = K % 3;
            const int dd = d < e2 ? d : e2, ee = d < e2 ? e2 : d;
            T v = fma(c1 * G[k * 3 + d], G[i * 3 + e2], c2 * G[i * 3 + d] * G[k * 3 + e2]);
            if (i == k) v = fma(c1, GG[dd * 3 + ee], v + GsG[dd * 3 + ee]);
            if (BB)
                v = fma(cbb, fma((T)2 * bG[i * 3 + d], bG[k * 3 + e2], -fma(b[s6(i, k)], GbG[dd * 3 + ee], bG[k * 3 + d] * bG[i * 3 + e2])), v);
            if (GT) {
                // kbI (bG_id G_ke + G_id bG_ke) + kgI (gG_id G_ke + G_id gG_ke) + kgg gG_id gG_ke
                // + kg4 (g_ik GG_de + gG_ie G_kd + gG_kd G_ie + d_ik GgG_de)
                if (NIMR) v = fma(kbI, fma(bG[i * 3 + d], G[k * 3 + e2], G[i * 3 + d] * bG[k * 3 + e2]), v);
                v = fma(kgI, fma(gG[i * 3 + d], G[k * 3 + e2], G[i * 3 + d] * gG[k * 3 + e2]), v);
                if (NIMR) v = fma(kgg, gG[i * 3 + d] * gG[k * 3 + e2], v);
                T t4 = fma(g6[s6(i, k)], GG[dd * 3 + ee], fma(gG[i * 3 + e2], G[k * 3 + d], gG[k * 3 + d] * G[i * 3 + e2]));
                if (i == k) t4 += GgG[dd * 3 + ee];
                v = fma(kg4, t4, v);
            }
            out.put(sym9(I, K), detJ * v);
        }
}

// Gauss-point tangent writers: FP64, FP32, or a float pair hi + lo
struct QOutF64 {
    double *q;
    int64_t ld;
    __device__ void put(int p, double v) const { q[p * ld] = v; }
};
struct QOutF32 {
    float *q;
    int64_t ld;
    __device__ void put(int p, float v) const { q[p * ld] = v; }
};
struct QOutDF {
    float *h, *l;
    int64_t ld;
    float *amax;  // the largest |hi| written (a register of the caller once inlined)
    __device__ void put(int p, FloatPair v) const {
        h[p * ld] = v.h;
        l[p * ld] = v.l;
        *amax = v.h == v.h ? fmaxf(*amax, fabsf(v.h)) : INFINITY;  // NaN: an overflow met inf - inf
    }
};

// Float pairs keep ~2^-46 of their value while the low word stays a normal FP32 number and the
// high word far from overflow: a Gauss point whose largest tangent entry (or stress factor) lies
// outside [2^-78, 2^120] is reported (FL_FLAG_PAIR_RANGE) so that the caller can assemble in FP64.
__device__ __forceinline__ bool pair_out_of_range(float amax) {
    return amax > 0x1p120f || (amax > 0.f && amax < 0x1p-78f);
}

// Gauss-point output layout: FP64 [54][ldq] in Q; FP32 tangent [45][ldq] in Qf with S [9][ldq]
// in Q; the tangent formed in float-pair arithmetic (hi [45][ldq] then lo [45][ldq]) in Qf with
// S [9][ldq] in Q; the float-pair tangent with S as float pairs too (Sh [9][ldq], Sl [9][ldq] floats
// in S's 72 bytes per point) for the reference-tensor contraction
enum { QOUT_F64 = 0, QOUT_F32 = 1, QOUT_DF = 2, QOUT_RT = 3 };

// QOUT: layout of the Gauss-point data (QOUT_F64 for the FP64 contraction, QOUT_F32 for the
// split-BF16 Jacobian, QOUT_DF for the float-pair and tensor-core contractions); the kinematics,
// the material law and S are FP64 in every layout
template <int NPE, int MAT, int QOUT = QOUT_F64>
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
        double detJ;
        if (A.geo && !A.npair) {  // the reference configuration's part from the per-mesh table
            const int64_t gi = e * nq + g, gs = A.nelem * (int64_t)nq;
            double iPX[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) iPX[k] = __ldg(A.geo + k * gs + gi);
            const double detX = __ldg(A.geo + 9 * gs + gi);
            auto xcoords = [&](int a, double &x0, double &x1, double &x2) {
                uint64_t nd = __ldg(el + a);
                if (nd >= (uint64_t)A.nnode) {
                    flag |= FL_FLAG_BAD_INDEX;
                    nd = 0;
                }
                x0 = __ldg(A.Eulerx + nd * 3); x1 = __ldg(A.Eulerx + nd * 3 + 1); x2 = __ldg(A.Eulerx + nd * 3 + 2);
            };
            detJ = kinematics_ref<NPE>(jm, xcoords, iPX, detX, __ldg(A.w + g), A.update, G, F);
        } else if (A.npair) {  // coordinate sums as float pairs (FP32 pipe)
            auto jp = [&](int d, int a) {
                const float2 v = __ldg(A.jmp + ((size_t)d * NPE + a) * nq + g);
                return FloatPair(v.x, v.y);
            };
            auto nodep = [&](int a, FloatPair *X, FloatPair *U) {
                uint64_t nd = __ldg(el + a);
                if (nd >= (uint64_t)A.nnode) {
                    flag |= FL_FLAG_BAD_INDEX;
                    nd = 0;
                }
                const float4 *q = reinterpret_cast<const float4 *>(A.npair + nd * 12);
                const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
                X[0] = FloatPair(q0.x, q1.y); X[1] = FloatPair(q0.y, q1.z); X[2] = FloatPair(q0.z, q1.w);
                U[0] = FloatPair(q0.w, q2.y); U[1] = FloatPair(q1.x, q2.z); U[2] = FloatPair(q2.x, q2.w);
            };
            detJ = kinematics_pair<NPE>(jp, nodep, __ldg(A.w + g), A.update, G, F);
        } else {
            detJ = kinematics_fn<NPE>(jm, coords, __ldg(A.w + g), A.update, G, F);
        }
        double sig[6], b[6], J, c1, c2, cbb;
        MatParams mp = A.mp;
        if (A.eparams) mp = MatParams{__ldg(A.eparams + e * 3), __ldg(A.eparams + e * 3 + 1), __ldg(A.eparams + e * 3 + 2), 0.0};
        ExtraTangent ex;
        material<MAT>(F, mp, sig, b, J, c1, c2, cbb, &ex, A.orient ? A.orient + e * 3 : nullptr);
        if (!(J > 0.0)) flag |= FL_FLAG_NONPOSITIVE_J;
        const int64_t ld = A.ldq;
        double *q = A.Q + t;
        // S[i][d] = detJ sum_j sigma_ij G[j][d], the residual's Gauss-point factor, in FP64
        double *qs = QOUT != QOUT_F64 ? q : q + 45 * ld;
        float amax = 0.f;  // largest magnitude held as float pairs
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double sv =
                    detJ * fma(sig[s6(i, 0)], G[0 * 3 + d], fma(sig[s6(i, 1)], G[1 * 3 + d], sig[s6(i, 2)] * G[2 * 3 + d]));
                if constexpr (QOUT == QOUT_RT) {
                    const FloatPair sp(sv);
                    float *sf = reinterpret_cast<float *>(A.Q) + t;
                    sf[(i * 3 + d) * ld] = sp.h;
                    sf[(9 + i * 3 + d) * ld] = sp.l;
                    amax = sp.h == sp.h ? fmaxf(amax, fabsf(sp.h)) : INFINITY;
                } else {
                    qs[(i * 3 + d) * ld] = sv;
                }
            }
        if constexpr (QOUT == QOUT_F32)
            pulled_back_tangent<float, MAT>(G, sig, b, ex, c1, c2, cbb, detJ, QOutF32{A.Qf + t, ld});
        else if constexpr (QOUT == QOUT_DF || QOUT == QOUT_RT)
            pulled_back_tangent<FloatPair, MAT>(G, sig, b, ex, c1, c2, cbb, detJ,
                                                QOutDF{A.Qf + t, A.Qf + 45 * ld + t, ld, &amax});
        else
            pulled_back_tangent<double, MAT>(G, sig, b, ex, c1, c2, cbb, detJ, QOutF64{q, ld});
        if ((QOUT == QOUT_DF || QOUT == QOUT_RT) && pair_out_of_range(amax)) flag |= FL_FLAG_PAIR_RANGE;
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
            if constexpr (DF) {
                if (A.Qf) {  // the Gauss-point kernel wrote the tangent as float pairs
                    const size_t col = (size_t)el * nq + g;
                    if (k < QSM)
                        Qs[((size_t)slot * nq + g) * QSM + k] =
                            make_float2(A.Qf[(size_t)k * A.ldq + col], A.Qf[(size_t)(QSM + k) * A.ldq + col]);
                    else
                        Ss[((size_t)slot * nq + g) * 9 + (k - QSM)] = A.Q[(size_t)(k - QSM) * A.ldq + col];
                    continue;
                }
            }
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

// Arithmetic of the contraction (fl_SetAssemblyArithmetic): by default the reference-tensor GEMMs
// on the tensor cores where they apply, float pairs on the FP32 pipe elsewhere; FP64 multiply-adds
// only when asked for
static std::atomic<int> g_arith{FL_ARITH_REFERENCE_TENSOR};

// Float-pair kinematics inputs, once per assembly call: per node the reference coordinates X and
// the displacement u = x - X (formed in FP64) as float pairs, 12 floats in three float4 words
// (Xh0 Xh1 Xh2 Uh0 | Uh1 Xl0 Xl1 Xl2 | Uh2 Ul0 Ul1 Ul2), and the shape-function gradients as
// (hi, lo) pairs.
__global__ void node_pairs_kernel(const double *points, const double *Eulerx, int64_t nnode, float *out) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nnode) return;
    FloatPair X[3], U[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double xv = points[n * 3 + k];
        X[k] = FloatPair(xv);
        U[k] = FloatPair(Eulerx[n * 3 + k] - xv);
    }
    float4 *o = reinterpret_cast<float4 *>(out + n * 12);
    o[0] = make_float4(X[0].h, X[1].h, X[2].h, U[0].h);
    o[1] = make_float4(U[1].h, X[0].l, X[1].l, X[2].l);
    o[2] = make_float4(U[2].h, U[0].l, U[1].l, U[2].l);
}

__global__ void jm_pairs_kernel(const double *Jm, float2 *out, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const FloatPair v(Jm[i]);
    out[i] = make_float2(v.h, v.l);
}

// The reference configuration's part of the kinematics per (element, Gauss point): (dX/dxi)^-1 and
// det(dX/dxi), as kinematics_fn forms them (the same sums in the same order), into
// geo[10][nelem * nq]; constant for a mesh.
template <int NPE>
__global__ void __launch_bounds__(QP_THREADS) reference_geometry_kernel(const double *points, const uint64_t *elements,
                                                                         const double *Jm, int64_t nelem, int nq,
                                                                         int64_t nnode, double *geo, int *flags) {
    const int64_t t = (int64_t)blockIdx.x * QP_THREADS + threadIdx.x;
    if (t >= nelem * nq) return;
    const int64_t e = t / nq;
    const int g = (int)(t % nq);
    const uint64_t *el = elements + e * NPE;
    double PX[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) PX[k] = 0.0;
    int flag = 0;
#pragma unroll 4
    for (int a = 0; a < NPE; ++a) {
        const double j0 = __ldg(Jm + ((size_t)0 * NPE + a) * nq + g), j1 = __ldg(Jm + ((size_t)1 * NPE + a) * nq + g),
                     j2 = __ldg(Jm + ((size_t)2 * NPE + a) * nq + g);
        uint64_t nd = __ldg(el + a);
        if (nd >= (uint64_t)nnode) {
            flag |= FL_FLAG_BAD_INDEX;
            nd = 0;
        }
        const double X0 = __ldg(points + nd * 3), X1 = __ldg(points + nd * 3 + 1), X2 = __ldg(points + nd * 3 + 2);
        PX[0] += j0 * X0; PX[1] += j0 * X1; PX[2] += j0 * X2;
        PX[3] += j1 * X0; PX[4] += j1 * X1; PX[5] += j1 * X2;
        PX[6] += j2 * X0; PX[7] += j2 * X1; PX[8] += j2 * X2;
    }
    double iPX[9];
    const double detX = inv3(PX, iPX);
    const int64_t gs = nelem * (int64_t)nq;
#pragma unroll
    for (int k = 0; k < 9; ++k) geo[k * gs + t] = iPX[k];
    geo[9 * gs + t] = detX;
    if (flag && flags) atomicOr(flags, flag);
}

static size_t pair_prep_bytes(int64_t nnode, int npe, int nq) {
    return ((sizeof(float) * 12 * (size_t)nnode + 255) & ~(size_t)255) +
           ((sizeof(float2) * 3 * (size_t)npe * nq + 255) & ~(size_t)255);
}

// fills the float-pair kinematics inputs at `base` (pair_prep_bytes long) and points A at them
static void pair_prep(AsmArgs &A, int npe, char *base, cudaStream_t stream) {
    float *np = reinterpret_cast<float *>(base);
    float2 *jp = reinterpret_cast<float2 *>(base + ((sizeof(float) * 12 * (size_t)A.nnode + 255) & ~(size_t)255));
    const int64_t nj = (int64_t)3 * npe * A.nq;
    node_pairs_kernel<<<(unsigned)((A.nnode + 255) / 256), 256, 0, stream>>>(A.points, A.Eulerx, A.nnode, np);
    jm_pairs_kernel<<<(unsigned)((nj + 255) / 256), 256, 0, stream>>>(A.Jm, jp, nj);
    A.npair = np;
    A.jmp = jp;
}

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
    // float pairs: the Gauss-point kernel forms the tangent in float-pair arithmetic and writes it
    // as hi [45][ldq] + lo [45][ldq] after S [9][ldq] (the same 432 bytes per Gauss point)
    A.Qf = DF ? reinterpret_cast<float *>(Q + (size_t)9 * A.ldq) : nullptr;
    for (int64_t e0 = 0; e0 < A.nelem; e0 += chunk) {
        A.e0 = e0;
        A.ne = A.nelem - e0 < chunk ? A.nelem - e0 : chunk;
        const int64_t nqp = A.ne * A.nq;
        if (DF)
            qp_kernel<NPE, MAT, QOUT_DF><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
        else
            qp_kernel<NPE, MAT><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
        contract_kernel<NPE, DF><<<(unsigned)((A.ne + EPC - 1) / EPC), NT, smem, stream>>>(A);
    }
    return launch_status();
}

template <int NPE, int MAT>
static int run_chunks(AsmArgs A, double *Q, int64_t chunk, cudaStream_t stream) {
    if (g_arith.load() == FL_ARITH_FP64) return run_chunks_t<NPE, MAT, false>(A, Q, chunk, stream);
    return run_chunks_t<NPE, MAT, true>(A, Q, chunk, stream);
}

template <int NPE, int MAT>
static int launch_oz(AsmArgs A, cudaStream_t stream);
template <int NPE>
static bool oz_supported(int nq);

// FP64 tangent as tensor-core GEMMs against the reference tensor (fl_reftensor.cu): the Gauss-point
// kernel writes the float-pair layout (float-pair kinematics) for a chunk of elements, the
// contraction kernel reads it tile by tile. Scratch from the stream-ordered allocator: the chunk's
// Gauss-point data (432 bytes per point, chunks of at most 512 MB), the float-pair kinematics
// inputs, the reference tensor's digit planes and, unless the caller supplies them, the block
// offsets of the pattern.
constexpr size_t RT_CHUNK_BYTES = (size_t)512 << 20;

// Freed stream-ordered memory is returned to the device at synchronisation points only above the
// pool's release threshold (0 by default): a Newton or time loop that synchronises between
// assembly calls would otherwise unmap and map its scratch again every call. Raised once per
// device to `bytes` on the device's current pool (a setting of this process only).
static void keep_pool_reserve(uint64_t bytes) {
    static std::mutex m;
    static bool done[256];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return;
    std::lock_guard<std::mutex> g(m);
    if (done[dev]) return;
    done[dev] = true;
    cudaMemPool_t pool;
    if (cudaDeviceGetMemPool(&pool, dev) != cudaSuccess) return;
    uint64_t cur = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur) == cudaSuccess && cur < bytes)
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &bytes);
}

template <int NPE, int MAT>
static int launch_rt(AsmArgs A, cudaStream_t stream) {
    if (A.nelem == 0) return FL_OK;
    int64_t chunk = std::max<int64_t>(1, (int64_t)(RT_CHUNK_BYTES / ((size_t)QSTRIDE * sizeof(double) * A.nq)));
    if (chunk > A.nelem) chunk = A.nelem;
    // the contraction stages the Gauss-point data with 16-byte loads: rows of a multiple of 4 floats
    const int64_t ldq = (chunk * A.nq + 3) / 4 * 4;
    const size_t qbytes = ((size_t)QSTRIDE * sizeof(double) * ldq + 255) & ~(size_t)255;
    const size_t pbytes = (pair_prep_bytes(A.nnode, NPE, A.nq) + 255) & ~(size_t)255;
    const size_t phibytes = rt_phi_bytes(NPE, A.nq);
    const size_t obytes = A.boff ? 0 : ((sizeof(int32_t) * (size_t)NPE * NPE * A.nelem + 255) & ~(size_t)255);
    keep_pool_reserve((uint64_t)2 << 30);
    char *base = nullptr;
    FL_CUDA_TRY(cudaMallocAsync((void **)&base, qbytes + pbytes + phibytes + obytes, stream));
    int st = FL_OK;
    do {
        A.Q = reinterpret_cast<double *>(base);
        A.ldq = ldq;
        A.Qf = reinterpret_cast<float *>(A.Q + (size_t)9 * A.ldq);
        pair_prep(A, NPE, base + qbytes, stream);
        // FP64 kinematics: float-pair coordinate sums lose ~2^-46 of sum |Jm X| to cancellation,
        // which the inverse Jacobian of a sliver element amplifies past the FP64 bar (measured
        // 1.8e-11 against 6.4e-13 on the Delaunay beam); the float-pair shape-function gradients
        // still serve the residual
        A.npair = nullptr;
        void *phi = base + qbytes + pbytes;
        if ((st = rt_build_phi(A.Jm, NPE, A.nq, phi, stream)) != FL_OK) break;
        const int32_t *boff = A.boff;
        if (!boff) {
            int32_t *ob = reinterpret_cast<int32_t *>(base + qbytes + pbytes + phibytes);
            if ((st = rt_block_offsets(A.elements, A.nelem, NPE, A.nnode, A.indptr, A.indices, ob, A.flags, stream)) !=
                FL_OK)
                break;
            boff = ob;
        }
        RtArgs R;
        R.Qh = A.Qf;
        R.Ql = A.Qf + (size_t)45 * A.ldq;
        R.Sp = reinterpret_cast<const float *>(A.Q);
        R.ldq = A.ldq;
        R.nq = A.nq;
        R.update = A.update;
        R.elements = A.elements;
        R.nnode = A.nnode;
        R.indptr = A.indptr;
        R.indices = A.indices;
        R.boff = boff;
        R.jmp = A.jmp;
        R.phi = phi;
        R.phiexp = rt_phi_exponents(phi, NPE, A.nq);
        R.V = A.V;
        R.T = A.T;
        R.flags = A.flags;
        for (int64_t e0 = 0; e0 < A.nelem && st == FL_OK; e0 += chunk) {
            A.e0 = e0;
            A.ne = A.nelem - e0 < chunk ? A.nelem - e0 : chunk;
            const int64_t nqp = A.ne * A.nq;
            qp_kernel<NPE, MAT, QOUT_RT><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
            R.e0 = e0;
            R.ne = A.ne;
            st = rt_contract(R, NPE, stream);
        }
    } while (false);
    if (st == FL_OK) st = launch_status();
    const cudaError_t fe = cudaFreeAsync(base, stream);
    if (st != FL_OK) return st;
    return fe == cudaSuccess ? FL_OK : FL_ERR_CUDA;
}

template <int NPE, int MAT>
static int launch_asm(AsmArgs A, double *scratch, size_t scratch_bytes, cudaStream_t stream) {
    constexpr int EPC = AsmCfg<NPE>::EPC;
    if (A.nelem == 0) return FL_OK;
    // FP64 tangent as tensor-core GEMMs against the reference tensor: CSR output, its own
    // scratch, element types it supports
    if (g_arith.load() == FL_ARITH_REFERENCE_TENSOR && !scratch && A.mode != 0 && rt_supported(NPE, A.nq))
        return launch_rt<NPE, MAT>(A, stream);
    // FP64 tangent on the tensor cores: CSR output, its own scratch, elements it supports
    if (g_arith.load() == FL_ARITH_TENSOR && !scratch && A.mode != 0 && oz_supported<NPE>(A.nq))
        return launch_oz<NPE, MAT>(A, stream);
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
                       const double *eparams = nullptr, const double *orient = nullptr,
                       const int32_t *boff = nullptr, const double *geo = nullptr) {
    if (ndim != 3 || nvar != 3 || H_VoigtSize != 6) return FL_ERR_ARG;
    if (nelem < 0 || nnode <= 0) return FL_ERR_ARG;
    if (ngauss <= 0 || ngauss > 343) return FL_ERR_UNSUPPORTED;
    if (3 * nnode + 2 > INT32_MAX) return FL_ERR_UNSUPPORTED;
    if (mat != NEOHOOKEAN && mat != MOONEYRIVLIN && mat != NEARLYINCOMPRESSIBLEMR && mat != LINEARELASTIC &&
        mat != ANISOTROPICMR1)
        return FL_ERR_UNSUPPORTED;
    if (mat == ANISOTROPICMR1 && eparams) return FL_ERR_UNSUPPORTED;  // per-element parameters: 3 values
    if (nelem == 0) return FL_OK;  // nothing is read or written
    if (!points || !elements || !Eulerx || !Jm || !AllGauss || !V_stiff || !T) return FL_ERR_ARG;
    if (mat == ANISOTROPICMR1 && !orient) return FL_ERR_ARG;  // the fibre directions are required
    AsmArgs A;
    A.points = points;
    A.elements = elements;
    A.Eulerx = Eulerx;
    A.Jm = Jm;
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
    A.Qf = nullptr;
    A.orient = mat == ANISOTROPICMR1 ? orient : nullptr;
    A.npair = nullptr;
    A.jmp = nullptr;
    A.boff = boff;
    A.geo = geo;
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
        case ANISOTROPICMR1: return dispatch_asm<ANISOTROPICMR1>((int)nodeperelem, A, scratch, scratch_bytes, stream);
        default: return dispatch_asm<LINEARELASTIC>((int)nodeperelem, A, scratch, scratch_bytes, stream);
    }
}

// Material of a C-ABI material number and its parameters from the reference's argument names:
// neo-Hookean and linear elastic (mu, lamb), Mooney-Rivlin (mu1, mu2, lamb), nearly incompressible
// Mooney-Rivlin (alpha, beta, kappa) = (mu1, mu2, lamb), transversely isotropic Mooney-Rivlin
// (mu1, mu2, lamb, mu3) (AOT_Assembler.py:62-75, 110-115).
static int material_of(int material_number, double mu, double mu1, double mu2, double lamb, int *mat, MatParams *mp,
                       double mu3 = 0.0) {
    switch (material_number) {
        case FL_MATERIAL_NEOHOOKEAN: *mat = NEOHOOKEAN; *mp = {mu, lamb, 0.0}; return FL_OK;
        case FL_MATERIAL_MOONEYRIVLIN: *mat = MOONEYRIVLIN; *mp = {mu1, mu2, lamb}; return FL_OK;
        case FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN: *mat = NEARLYINCOMPRESSIBLEMR; *mp = {mu1, mu2, lamb}; return FL_OK;
        case FL_MATERIAL_LINEARELASTIC: *mat = LINEARELASTIC; *mp = {mu, lamb, 0.0}; return FL_OK;
        case FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1: *mat = ANISOTROPICMR1; *mp = {mu1, mu2, lamb, mu3}; return FL_OK;
        default: return FL_ERR_UNSUPPORTED;
    }
}

// ------------------------------------------------------------------------------------------------
// C. Mixed-precision (split-BF16) tangent: shared pieces. The Jacobian is formed on the tensor
// cores (section D) with both operands split into three BF16 terms (x = hi + mid + lo, 24
// significant bits together) and multiplied as the six products whose order is at least 2^-16
// with FP32 accumulation: the tangent to about FP32 accuracy, enough for Newton on
// ill-conditioned problems (a two-term split, ~1e-5, slows Newton down). The residual is formed
// in FP64 exactly as in contract_kernel.
// ------------------------------------------------------------------------------------------------
constexpr int MX_KC = 96;  // widest reduction chunk

// reduction-chunk width of the split-BF16 kernel: the padded 3*nq, at most MX_KC (the operand
// buffers are sized by it, so short reductions leave room for more resident CTAs)
__host__ __device__ inline int mixed_kc(int nq) {
    const int kp = (3 * nq + 15) / 16 * 16;
    return kp < MX_KC ? kp : MX_KC;
}

// ------------------------------------------------------------------------------------------------
// D. The split-BF16 tangent on the fifth-generation tensor cores (tcgen05).
//
//    K^T[(i,b,k), a] = sum_(g,d) U[(i,b,k),(g,d)] Jm[d][a][g],
//    U[(i,b,k),(g,d)] = sum_e Ahat_g[(i,d),(k,e)] Jm[e][b][g]
//
// One work item = (element, group of 128-row tiles of K^T). Per reduction chunk of KC columns
// (g,d), the CTA writes the three BF16 terms of U (A operand, rows of the tile group x KC) and of
// Jm (B operand, NB x KC, NB = NPE padded to 16) to shared memory in the K-major core-matrix
// layout; one thread issues, per tile and 16-wide K step, the six products as tcgen05.mma into
// that tile's FP32 accumulator in tensor memory and commits them to an mbarrier. After the last
// chunk the eight warps read the accumulators with tcgen05.ld (warps w and w + 4 share tensor-
// memory lanes 32 (w % 4) .. + 31 and split the tiles between them) and scatter them.
//
// The U build is the kernel's main work: each thread forms 8 consecutive columns of one row (one
// 16-byte row of a core matrix) from float4 rows of the pulled-back tangent
// Qx[g][(i,d)][k] = (Ahat[(i,d),(k,0..2)], 0) in shared memory and float4 rows
// J4[g][b] = (Jm[0..2][b][g], 0) (read-only cache), splits them into packed BF16 pairs and stores
// the three terms as 16-byte words. The B operand depends only on the element type: with one K
// chunk it is built once per CTA. Waits are bounded (on expiry the CTA stops and raises
// FL_FLAG_BAD_INDEX, which the call reports as an error).
// ------------------------------------------------------------------------------------------------
constexpr int TC_MT = 128;       // rows per tile (the MMA's M)
constexpr int TC_THREADS = 256;  // eight warps
constexpr long long TC_WAIT = 1ll << 22;

template <int NPE>
__host__ __device__ constexpr int tc_nb() { return (NPE + 15) / 16 * 16; }
template <int NPE>
__host__ __device__ constexpr int tc_ntiles() { return (9 * NPE + TC_MT - 1) / TC_MT; }
// tensor-memory columns per tile accumulator (read back 32 at a time)
template <int NPE>
__host__ __device__ constexpr int tc_colw() { return (tc_nb<NPE>() + 31) / 32 * 32; }

// valid rows of K^T per (tile, tensor-memory lane quarter): the 9 NPE rows are spread evenly over
// the 4 lane quarters of every tile, so each warp reads back an equal share
template <int NPE>
__host__ __device__ constexpr int tc_rpl() { return (9 * NPE + 4 * tc_ntiles<NPE>() - 1) / (4 * tc_ntiles<NPE>()); }

// Gauss-point values prefetched into registers per thread for the next work item (the 54 nq
// values of an element when they fit, else loaded when needed)
constexpr int TC_PF = 4;

// shared memory: Qr double [9][nq] | Qx float4 [nq][27] | A terms 3 x [tg * 128][KC] bf16 |
// B terms 3 x [NB][KC] bf16 | nodes, inv, boff
// (with the element's map block [9 NPE^2] int after them when it is staged)
template <int NPE>
__host__ __device__ inline size_t tc_map_offset(int nq, int kc, int tg) {
    const size_t b = (sizeof(double) * 9 * (size_t)nq + 15) / 16 * 16 + sizeof(float4) * 27 * (size_t)nq +
                     sizeof(__nv_bfloat16) * 3 * ((size_t)tg * TC_MT * kc + (size_t)tc_nb<NPE>() * kc) +
                     sizeof(int) * (NPE + 3 * NPE) + sizeof(int16_t) * NPE * NPE;
    return (b + 15) / 16 * 16;
}
template <int NPE>
__host__ __device__ inline size_t tc_smem_bytes(int nq, int kc, int tg, bool stage = false) {
    const size_t b = tc_map_offset<NPE>(nq, kc, tg) + (stage ? sizeof(int) * 9 * (size_t)NPE * NPE : 0);
    return (b + 127) / 128 * 128;
}

// asynchronous global -> shared copies (cp.async; 16 bytes needs both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// J4[g][b] = (Jm[0][b][g], Jm[1][b][g], Jm[2][b][g], 0) for g < nq, zero rows for nq <= g < nq + 4
__global__ void jm_float4(const double *Jm, float4 *J4, int npe, int nq) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (nq + 4) * npe) return;
    const int g = t / npe, b = t % npe;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g < nq) {
        v.x = (float)Jm[((size_t)0 * npe + b) * nq + g];
        v.y = (float)Jm[((size_t)1 * npe + b) * nq + g];
        v.z = (float)Jm[((size_t)2 * npe + b) * nq + g];
    }
    J4[t] = v;
}

__device__ __forceinline__ float dot3(const float4 &q, const float4 &j) { return fmaf(q.x, j.x, fmaf(q.y, j.y, q.z * j.z)); }

// three-term split of 8 values into packed BF16 pairs (element t in half t % 2 of word t / 2)
__device__ __forceinline__ void split8(const float (&v)[8], uint4 &H, uint4 &Mi, uint4 &L) {
    uint32_t h[4], m[4], l[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * p], v[2 * p + 1]);
        const float2 hf = __bfloat1622float2(h2);
        const float r0 = v[2 * p] - hf.x, r1 = v[2 * p + 1] - hf.y;
        const __nv_bfloat162 m2 = __floats2bfloat162_rn(r0, r1);
        const float2 mf = __bfloat1622float2(m2);
        const __nv_bfloat162 l2 = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);
        h[p] = *reinterpret_cast<const uint32_t *>(&h2);
        m[p] = *reinterpret_cast<const uint32_t *>(&m2);
        l[p] = *reinterpret_cast<const uint32_t *>(&l2);
    }
    H = make_uint4(h[0], h[1], h[2], h[3]);
    Mi = make_uint4(m[0], m[1], m[2], m[3]);
    L = make_uint4(l[0], l[1], l[2], l[3]);
}

// U at columns c0 .. c0 + 7 (c = 3 g + d, c0 = 3 g0 + D0) of row (i, b, k), all below K
template <int NPE, int D0>
__device__ __forceinline__ void u_row8(const float4 *qx, const float4 *J4, int g0, int i, int b, int k,
                                       float (&v)[8]) {
    float4 j[4];
#pragma unroll
    for (int s = 0; s < (D0 + 7) / 3 + 1; ++s) j[s] = __ldg(J4 + (size_t)(g0 + s) * NPE + b);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int gg = (D0 + t) / 3, dd = (D0 + t) % 3;
        v[t] = dot3(qx[(g0 + gg) * 27 + 9 * i + 3 * dd + k], j[gg]);
    }
}

// (I, K), I <= K, of entry p of the packed upper triangle of a symmetric 9x9 (sym9's inverse)
struct SymPairs {
    unsigned char I[45], K[45];
};
__host__ __device__ constexpr SymPairs make_sym_pairs() {
    SymPairs t{};
    int p = 0;
    for (int I = 0; I < 9; ++I)
        for (int K = I; K < 9; ++K) {
            t.I[p] = (unsigned char)I;
            t.K[p] = (unsigned char)K;
            ++p;
        }
    return t;
}
__constant__ SymPairs c_sym = make_sym_pairs();

// n / d for n, d < 2^16 (n d < 2^32) by one high multiply with m = ceil(2^32 / d), d >= 2
__device__ __forceinline__ int fastdiv(int n, uint32_t m) { return (int)__umulhi((uint32_t)n, m); }

template <int NPE>
__global__ void __launch_bounds__(TC_THREADS, 2)
    contract_tc_kernel(const AsmArgs A, const float4 *__restrict__ J4, float *V32, int KC, int tg, int tcols,
                       int stage) {
    constexpr int NDOF = 3 * NPE, M = 9 * NPE, NB = tc_nb<NPE>(), NT = tc_ntiles<NPE>(), CW = tc_colw<NPE>();
    constexpr int RPL = tc_rpl<NPE>(), RPL8 = (RPL + 7) / 8 * 8;
    const int nq = A.nq, K = 3 * nq;
    const int ngrp = (NT + tg - 1) / tg;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *Qr = reinterpret_cast<double *>(smem_raw);  // [9][nq] residual part
    float4 *Qx = reinterpret_cast<float4 *>(smem_raw + (sizeof(double) * 9 * (size_t)nq + 15) / 16 * 16);  // [nq][27]
    __nv_bfloat16 *At[3], *Bt[3];
    At[0] = reinterpret_cast<__nv_bfloat16 *>(Qx + 27 * nq);
    At[1] = At[0] + (size_t)tg * TC_MT * KC;
    At[2] = At[1] + (size_t)tg * TC_MT * KC;
    Bt[0] = At[2] + (size_t)tg * TC_MT * KC;
    Bt[1] = Bt[0] + NB * KC;
    Bt[2] = Bt[1] + NB * KC;
    int *nodes = reinterpret_cast<int *>(Bt[2] + NB * KC);  // [NPE]
    int *inv = nodes + NPE;                                 // [NDOF]
    int16_t *boff = reinterpret_cast<int16_t *>(inv + NDOF);  // [NPE][NPE]
    // the element's block of the local-to-global map [NDOF][NDOF], copied asynchronously
    int *dgs = reinterpret_cast<int *>(smem_raw + tc_map_offset<NPE>(nq, KC, tg));
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t taddr_s;
    __shared__ int s_flag;
    __shared__ int64_t s_nnz;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t cap = (int64_t)NDOF * NDOF;
    const int64_t nwork = A.ne * ngrp;
    const bool staged = stage && A.dg;
    const bool wide = staged && (cap & 3) == 0 && ((uintptr_t)A.dg & 15) == 0;  // 16-byte copies
    const bool pf = 54 * nq <= TC_THREADS * TC_PF;  // Gauss-point values fit the prefetch registers
    int flag = 0;
    uint32_t phase = 0;
    if (tid == 0) {
        s_flag = 0;
        s_nnz = (int64_t)A.indptr[3 * A.nnode];
        tc::mbar_init(&mbar, 1);
    }
    if (warp == 0) tc::tmem_alloc(&taddr_s, (uint32_t)tcols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = taddr_s;
    const uint32_t idesc = tc::idesc_bf16_f32(TC_MT, NB);
    const uint32_t sbo = (uint32_t)(KC / 8) * 128;
    const bool b_once = K <= KC;  // one K chunk: the Jm operand is built once per CTA
    bool b_built = false;
    bool ok = true;

    // per-element inputs of work item w, loaded into registers ahead of use: node tid, entry tid of
    // the first column of the local-to-sorted map, and the element's Gauss-point values
    uint64_t pq[TC_PF];  // raw bits: a float (tangent part) or a double (residual part)
    int pslot[TC_PF];    // (value p << 16) | Gauss point g of register slot j, -1 if unused
#pragma unroll
    for (int j = 0; j < TC_PF; ++j) {
        const int idx = tid + TC_THREADS * j;
        pslot[j] = pf && idx < 54 * nq ? ((idx / nq) << 16) | (idx % nq) : -1;
    }
    uint64_t pnode = 0;
    int pdl = 0;
    // Gauss-point value p (0..44 the FP32 tangent part in A.Qf, 45..53 the FP64 residual part in
    // A.Q) of point g of element el, as raw bits
    auto load_q = [&](int p, int g, int64_t el) -> uint64_t {
        const size_t col = (size_t)el * nq + g;
        return p < 45 ? (uint64_t)__float_as_uint(A.Qf[(size_t)p * A.ldq + col])
                      : (uint64_t)__double_as_longlong(A.Q[(size_t)(p - 45) * A.ldq + col]);
    };
    auto prefetch = [&](int64_t w) {
        if (w >= nwork) return;
        const int64_t el = w / ngrp, e = A.e0 + el;
        if (tid < NPE) pnode = A.elements[e * NPE + tid];
        if (A.dl && tid < NDOF) pdl = A.dl[e * cap + (int64_t)tid * NDOF];
#pragma unroll
        for (int j = 0; j < TC_PF; ++j)
            if (pslot[j] >= 0) pq[j] = load_q(pslot[j] >> 16, pslot[j] & 0xffff, el);
    };
    auto put_q = [&](int p, int g, uint64_t bits) {
        if (p >= 45) {
            Qr[(p - 45) * nq + g] = __longlong_as_double((long long)bits);
            return;
        }
        const float v = __uint_as_float((uint32_t)bits);
        const int I = c_sym.I[p], Kc = c_sym.K[p];
        float *qx = reinterpret_cast<float *>(Qx + (size_t)g * 27);
        qx[(I * 3 + Kc / 3) * 4 + Kc % 3] = v;
        if (Kc != I) qx[(Kc * 3 + I / 3) * 4 + I % 3] = v;
    };
    // MMA rows whose lane is past RPL8 hold zeros for every work item: written once
    for (int idx = tid; idx < tg * TC_MT * (KC / 8); idx += TC_THREADS) {
        const int rr = idx % (tg * TC_MT), cg = idx / (tg * TC_MT);
        if ((rr & 31) < RPL8) continue;
        const uint32_t off = tc::kmajor_offset(rr, 8 * cg, KC) / 2;
        *reinterpret_cast<uint4 *>(At[0] + off) = make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4 *>(At[1] + off) = make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4 *>(At[2] + off) = make_uint4(0, 0, 0, 0);
    }
    prefetch(blockIdx.x);

    for (int64_t w = blockIdx.x; w < nwork && ok; w += gridDim.x) {
        const int64_t el = w / ngrp, e = A.e0 + el;
        const int grp = (int)(w % ngrp);
        const int t0 = grp * tg, tn = min(tg, NT - t0);
        __syncthreads();  // previous work item done with the shared buffers
        for (int a = tid; a < NPE; a += TC_THREADS) {  // entry tid was prefetched
            uint64_t nd = a == tid ? pnode : A.elements[e * NPE + a];
            if (nd >= (uint64_t)A.nnode) {
                flag |= FL_FLAG_BAD_INDEX;
                nd = 0;
            }
            nodes[a] = (int)nd;
        }
        if (A.dl)
            for (int i = tid; i < NDOF; i += TC_THREADS) {
                const int v = i == tid ? pdl : A.dl[e * cap + (int64_t)i * NDOF];
                const int p = v / NDOF;
                if (v < 0 || p >= NDOF) flag |= FL_FLAG_BAD_INDEX;
                else inv[p] = i;
            }
        if (pf) {
#pragma unroll
            for (int j = 0; j < TC_PF; ++j)
                if (pslot[j] >= 0) put_q(pslot[j] >> 16, pslot[j] & 0xffff, pq[j]);
        } else {
            for (int idx = tid; idx < 54 * nq; idx += TC_THREADS) put_q(idx / nq, idx % nq, load_q(idx / nq, idx % nq, el));
        }
        __syncthreads();
        if (staged) {  // map block of this element, needed at the read-back
            const int *src = A.dg + e * cap;
            if (wide)
                for (int i = 4 * tid; i < cap; i += 4 * TC_THREADS) cp_async16(dgs + i, src + i);
            else
                for (int i = tid; i < cap; i += TC_THREADS) cp_async4(dgs + i, src + i);
            cp_async_commit();
        }
        prefetch(w + gridDim.x);  // next item's inputs, in flight during this item
        if (!A.dl)  // offset of column node b in row node a; consecutive threads share a row
            for (int idx = tid; idx < NPE * NPE; idx += TC_THREADS) {
                const int off = row_search(A.indptr, A.indices, 3 * nodes[idx / NPE], 3 * nodes[idx % NPE]);
                boff[idx] = (int16_t)(off >= 0 && off < 32768 ? off : -1);
            }
        // residual in FP64 (first tile group only): four threads per dof, each a quarter of the
        // Gauss points, combined by shuffles (the loop trip count is uniform across the CTA)
        if (A.update && grp == 0) {
            for (int base = 0; base < 4 * NDOF; base += TC_THREADS) {
                const int idx = base + tid, r = idx >> 2, part = idx & 3;
                double t = 0.0;
                if (r < NDOF) {
                    const int a = r / 3, i = r % 3;
                    for (int g = part; g < nq; g += 4) {
                        t = fma(__ldg(A.Jm + (size_t)a * nq + g), Qr[(i * 3) * nq + g], t);
                        t = fma(__ldg(A.Jm + ((size_t)NPE + a) * nq + g), Qr[(i * 3 + 1) * nq + g], t);
                        t = fma(__ldg(A.Jm + ((size_t)2 * NPE + a) * nq + g), Qr[(i * 3 + 2) * nq + g], t);
                    }
                }
                t += __shfl_xor_sync(0xffffffffu, t, 1);
                t += __shfl_xor_sync(0xffffffffu, t, 2);
                if (r < NDOF && part == 0) atomicAdd(A.T + 3 * (int64_t)nodes[r / 3] + r % 3, t);
            }
        }
        for (int k0 = 0; k0 < K; k0 += KC) {
            const int kc = min(KC, K - k0);
            // A operand: item = (row rl of the tile group, 8-column group cg); consecutive threads
            // take consecutive rows and each quarter warp stores one 128-byte core matrix. Row
            // rl = q RPL8 + l (q = 4 t + s, RPL8 = RPL padded to 8) sits at MMA row rr = 32 q + l
            // (tile t0 + t, lane quarter s, lane l) and holds row r = (4 t0 + q) RPL + l of K^T
            // when l < RPL and r < M, else zeros; lanes l >= RPL8 were zeroed at the start
            const int nrg = tn * 4 * RPL8;
            const uint32_t mg = 0xFFFFFFFFu / (uint32_t)nrg + 1u;
            for (int idx = tid; idx < nrg * (KC / 8); idx += TC_THREADS) {
                const int cg = fastdiv(idx, mg), rl = idx - cg * nrg, c0 = k0 + 8 * cg;
                const int q4 = rl / RPL8, l = rl - q4 * RPL8, rr = 32 * q4 + l, r = (4 * t0 + q4) * RPL + l;
                const bool live = l < RPL && r < M;
                float v[8];
                if (live && c0 + 8 <= K) {
                    const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
                    const int g0 = c0 / 3;
                    switch (c0 - 3 * g0) {
                        case 0: u_row8<NPE, 0>(Qx, J4, g0, i, b, k, v); break;
                        case 1: u_row8<NPE, 1>(Qx, J4, g0, i, b, k, v); break;
                        default: u_row8<NPE, 2>(Qx, J4, g0, i, b, k, v); break;
                    }
                } else {
                    const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        const int c = c0 + t;
                        v[t] = 0.f;
                        if (live && c < K) {
                            const int g = c / 3, d = c % 3;
                            v[t] = dot3(Qx[(size_t)g * 27 + 9 * i + 3 * d + k], __ldg(J4 + (size_t)g * NPE + b));
                        }
                    }
                }
                uint4 h, m, lo;
                split8(v, h, m, lo);
                const uint32_t off = tc::kmajor_offset(rr, 8 * cg, KC) / 2;
                *reinterpret_cast<uint4 *>(At[0] + off) = h;
                *reinterpret_cast<uint4 *>(At[1] + off) = m;
                *reinterpret_cast<uint4 *>(At[2] + off) = lo;
            }
            if (!b_once || !b_built) {  // B operand: Jm[d][n][g] at column c = 3 g + d
                for (int idx = tid; idx < NB * (KC / 8); idx += TC_THREADS) {
                    const int n = idx % NB, cg = idx / NB, c0 = k0 + 8 * cg;
                    float v[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        const int c = c0 + t;
                        v[t] = 0.f;
                        if (n < NPE && c < K) {
                            const float4 jj = __ldg(J4 + (size_t)(c / 3) * NPE + n);
                            const int d = c % 3;
                            v[t] = d == 0 ? jj.x : (d == 1 ? jj.y : jj.z);
                        }
                    }
                    uint4 h, m, lo;
                    split8(v, h, m, lo);
                    const uint32_t off = tc::kmajor_offset(n, 8 * cg, KC) / 2;
                    *reinterpret_cast<uint4 *>(Bt[0] + off) = h;
                    *reinterpret_cast<uint4 *>(Bt[1] + off) = m;
                    *reinterpret_cast<uint4 *>(Bt[2] + off) = lo;
                }
                b_built = true;
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
                // per tile, the six products of order >= 2^-16, smallest first (0 = hi, 1 = mid,
                // 2 = lo); a descriptor's start-address field counts 16-byte units, so the next
                // K step (two core matrices, 256 bytes) adds 16 and the next tile (256 KC bytes) 16 KC
                const int pa[6] = {1, 2, 0, 1, 0, 0}, pb[6] = {1, 0, 2, 0, 1, 0};
                uint64_t da0[3], db0[3];
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    da0[p] = tc::smem_desc(At[p], 128, sbo);
                    db0[p] = tc::smem_desc(Bt[p], 128, sbo);
                }
                for (int t = 0; t < tn; ++t)
                    for (int ks = 0; 16 * ks < kc; ++ks)
#pragma unroll
                        for (int p = 0; p < 6; ++p)
                            tc::mma_bf16(taddr + (uint32_t)(t * CW), da0[pa[p]] + (uint64_t)(t * 16 * KC + 16 * ks),
                                         db0[pb[p]] + (uint64_t)(16 * ks), idesc, k0 > 0 || ks > 0 || p > 0);
                tc::mma_commit(&mbar);
            }
            if (staged && k0 + KC >= K) cp_async_wait_all();  // own map copies landed
            // warp 0 polls the barrier, the others wait at the CTA barrier; uniform result
            ok = __syncthreads_and(warp == 0 ? tc::mbar_wait(&mbar, phase & 1, TC_WAIT) : true) != 0;
            ++phase;
            tc::fence_after_sync();
            if (!ok) break;
        }
        if (!ok) {
            flag |= FL_FLAG_BAD_INDEX;  // reported as an error by the caller
            break;
        }
        // read back: units of (tile, 16 columns), alternating between warps w and w + 4, which
        // share tensor-memory lane quarter w % 4
        const int sub = warp & 3, half = warp >> 2;
        constexpr int CB = NB / 16;
        for (int u = half; u < tn * CB; u += 2) {
            const int t = u / CB, c0 = (u % CB) * 16;
            float v[16];
            tc::tmem_ld16(taddr + ((uint32_t)(32 * sub) << 16) + (uint32_t)(t * CW + c0), v);
            const int r = ((t0 + t) * 4 + sub) * RPL + lane;
            if (lane >= RPL || r >= M) continue;
            const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
            if (A.dl) {  // positions first (independent loads in flight together), then the adds
                const int ic = inv[3 * b + k];
                int64_t pos[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int a = c0 + j;
                    pos[j] = -1;
                    if (a < NPE) {
                        const int ir = inv[3 * a + i];
                        if ((unsigned)ir < (unsigned)NDOF && (unsigned)ic < (unsigned)NDOF)
                            pos[j] = staged ? (int64_t)dgs[ir * NDOF + ic] : (int64_t)A.dg[e * cap + (int64_t)ir * NDOF + ic];
                    }
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (c0 + j >= NPE) continue;
                    if (pos[j] >= 0 && pos[j] < s_nnz) atomicAdd(V32 + pos[j], v[j]);
                    else flag |= FL_FLAG_BAD_INDEX;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int a = c0 + j;  // C[r, a] = K_e[(a,i),(b,k)]
                    if (a >= NPE) continue;
                    const int64_t pos = block_entry(A.indptr, A.indices, nodes[a], nodes[b], i, k, boff[a * NPE + b]);
                    if (pos >= 0 && pos < s_nnz) atomicAdd(V32 + pos, v[j]);
                    else flag |= FL_FLAG_BAD_INDEX;
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();  // every warp has read the accumulators before the next item's MMAs
        tc::fence_after_sync();
    }
    cp_async_wait_all();  // no copy outstanding at exit
    if (!ok)  // give MMAs still in flight a second bounded wait before the tensor memory is freed
        (void)__syncthreads_and(warp == 0 ? tc::mbar_wait(&mbar, (phase - 1) & 1, TC_WAIT) : true);
    if (flag) atomicOr(&s_flag, flag);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, (uint32_t)tcols);
    if (tid == 0 && s_flag && A.flags) atomicOr(A.flags, s_flag);
}

// Tiling of the split-BF16 kernel (fl_SetTensorCoreTiling): 0 = automatic
static std::atomic<int> g_tc_tg{0}, g_tc_kc{0};

struct TcPlan {
    int kc, tg, tcols;
    size_t smem;
    int stage;  // the element's map block is staged in shared memory
};

// Plan: reduction chunk kc (a multiple of 16, at most MX_KC) and tile group tg (tiles per work
// item, tensor memory tg * CW <= 256 columns). First choice: the padded 3 nq as kc with the most
// tiles that leave room for two CTAs per SM; else the widest kc, then the most tiles, that fit one
// CTA. fl_SetTensorCoreTiling fixes either.
template <int NPE>
static TcPlan tc_plan(int nq) {
    constexpr int NT = tc_ntiles<NPE>(), CW = tc_colw<NPE>();
    const int kc_req = g_tc_kc.load(), tg_req = g_tc_tg.load();
    const int kc_nat = kc_req > 0 ? std::min((kc_req + 15) / 16 * 16, MX_KC) : mixed_kc(nq);
    const size_t limit[2] = {113 * 1024, 227 * 1024};
    for (int pass = 0; pass < 2; ++pass)
        for (int kc = kc_nat; kc >= 16; kc -= 16) {
            if ((pass == 0 || kc_req > 0) && kc != kc_nat) break;
            for (int tg = tg_req > 0 ? std::min(tg_req, NT) : NT; tg >= 1; --tg) {
                if (tg_req > 0 && tg != std::min(tg_req, NT)) break;
                if (tg * CW > 256) continue;
                const size_t s = tc_smem_bytes<NPE>(nq, kc, tg);
                if (s > limit[pass]) continue;
                int cols = 32;
                while (cols < tg * CW) cols *= 2;
                const size_t s2 = tc_smem_bytes<NPE>(nq, kc, tg, true);
                return s2 <= limit[pass] ? TcPlan{kc, tg, cols, s2, 1} : TcPlan{kc, tg, cols, s, 0};
            }
        }
    return TcPlan{0, 0, 0, 0, 0};
}

// Resident CTAs per SM of the split-BF16 kernel, from its shared memory (with the largest
// shared-memory carveout requested), registers and tensor-memory columns (512 per SM)
static int tc_ctas_per_sm(const void *kernel, const TcPlan &P) {
    int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return 1;
    const size_t per_cta = P.smem + fa.sharedSizeBytes + (size_t)reserved;
    int n = (int)((size_t)smem_sm / per_cta);
    const int regs = (fa.numRegs + 7) / 8 * 8;
    if (regs > 0) n = std::min(n, regs_sm / (TC_THREADS * regs));
    n = std::min(n, 512 / P.tcols);
    return std::max(1, std::min(n, 8));
}

template <int NPE, int MAT>
static int launch_mixed(AsmArgs A, float *V32, cudaStream_t stream) {
    if (A.nelem == 0) return FL_OK;
    const TcPlan P = tc_plan<NPE>(A.nq);
    if (P.tg == 0) return FL_ERR_UNSUPPORTED;
    { const int st = ensure_smem<contract_tc_kernel<NPE>>(P.smem); if (st != FL_OK) return st; }
    // Gauss-point scratch per chunk: S [9][ldq] FP64, the tangent part [45][ldq] FP32 (252 bytes
    // per point, the chunk sized like the FP64 path's to stay in L2), then the float4 table of Jm
    int64_t chunk = std::max<int64_t>(1, (int64_t)(CHUNK_BYTES / ((9 * sizeof(double) + 45 * sizeof(float)) * (size_t)A.nq)));
    if (chunk > A.nelem) chunk = A.nelem;
    const size_t sbytes = (sizeof(double) * 9 * (size_t)A.nq * chunk + 255) & ~(size_t)255;
    const size_t fbytes = (sizeof(float) * 45 * (size_t)A.nq * chunk + 255) & ~(size_t)255;
    const int64_t nj4 = (int64_t)(A.nq + 4) * NPE;
    double *Q = nullptr;
    const size_t j4bytes = (sizeof(float4) * (size_t)nj4 + 255) & ~(size_t)255;
    FL_CUDA_TRY(cudaMallocAsync((void **)&Q, sbytes + fbytes + j4bytes + pair_prep_bytes(A.nnode, NPE, A.nq), stream));
    A.Q = Q;
    A.Qf = reinterpret_cast<float *>(reinterpret_cast<char *>(Q) + sbytes);
    A.ldq = chunk * A.nq;
    float4 *J4 = reinterpret_cast<float4 *>(reinterpret_cast<char *>(Q) + sbytes + fbytes);
    pair_prep(A, NPE, reinterpret_cast<char *>(Q) + sbytes + fbytes + j4bytes, stream);
    jm_float4<<<(unsigned)((nj4 + 255) / 256), 256, 0, stream>>>(A.Jm, J4, NPE, A.nq);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int occ = tc_ctas_per_sm(reinterpret_cast<const void *>(contract_tc_kernel<NPE>), P);
    const int ngrp = (tc_ntiles<NPE>() + P.tg - 1) / P.tg;
    for (int64_t e0 = 0; e0 < A.nelem; e0 += chunk) {
        A.e0 = e0;
        A.ne = A.nelem - e0 < chunk ? A.nelem - e0 : chunk;
        const int64_t nqp = A.ne * A.nq;
        qp_kernel<NPE, MAT, QOUT_F32><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
        const int64_t grid = std::min<int64_t>(A.ne * ngrp, (int64_t)sms * occ);
        contract_tc_kernel<NPE><<<(unsigned)grid, TC_THREADS, P.smem, stream>>>(A, J4, V32, P.kc, P.tg, P.tcols,
                                                                                 P.stage);
    }
    const int st = launch_status();
    const cudaError_t fe = cudaFreeAsync(Q, stream);
    if (st != FL_OK) return st;
    return fe == cudaSuccess ? FL_OK : FL_ERR_CUDA;
}

// ------------------------------------------------------------------------------------------------
// E. The FP64 tangent on the tensor cores (FL_ARITH_TENSOR).
//
// The same contraction as section D, to FP64 accuracy: both operands are scaled by a power of two
// (per element for U, from max|Ahat| times the largest column sum of |Jm|; per element type for Jm)
// and written as six signed base-256 digits, x = 2^e (d0 + d1 2^-8 + ... + d5 2^-40) / 128, every
// digit an integer of at most 8 bits, held exactly in BF16. The products of digit pairs (i, j)
// are summed per level w = i + j < 6 in an FP32 tensor-memory accumulator of their own: 21 MMAs
// per tile and 16-wide K step. Digits 0-2 are at most 128 in magnitude, so a product is at most
// 2^14 and the levels 0-2 (the ones whose rounding would show at 1e-12) sum exactly as long as
// 3 K 2^14 < 2^24; the levels 3-5 weigh 2^-24 and less. The read-back recombines the levels in
// float-pair arithmetic (Horner in 2^-8 from level 5), scales by 2^(eU + eJ - 14) and adds the
// FP64 value into V. U itself is formed in float-pair arithmetic from Ahat and Jm as float pairs
// (the Gauss-point kernel writes Ahat as hi + lo), ~2^-46 relative; the residual is FP64.
// One tile per work item (the six accumulators of a 32-column tile take 192 tensor-memory
// columns), reduction chunks of KC columns, the Jm digits built once per CTA for the whole K.
// ------------------------------------------------------------------------------------------------
constexpr int OZ_DIG = 6;
constexpr int OZ_THREADS = 256;

__device__ __forceinline__ void oz_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// six signed digits of the float pair (h, l), |h + l| <= 128: h + l = d0 + d1/256 + ... + d5/256^5
// up to ~2^-40 (digits 0-2 within [-128, 128], digits 3-5 within [-193, 193])
__device__ __forceinline__ void oz_digits(float h, float l, float (&d)[OZ_DIG]) {
    d[0] = rintf(h);
    float r = h - d[0];  // exact: |r| <= 1/2 and a multiple of ulp(h)
    d[1] = rintf(r * 256.f);
    r = r * 256.f - d[1];
    d[2] = rintf(r * 256.f);
    r = r * 256.f - d[2];
    float t, te;
    oz_two_sum(r * 256.f, l * 16777216.f, t, te);  // the rest of h and all of l, in units of digit 3
    d[3] = rintf(t);
    r = t - d[3];
    d[4] = rintf(r * 256.f);
    r = r * 256.f - d[4];
    d[5] = rintf(r * 256.f + te * 256.f);
}

// U entry sum_l (qh_l + ql_l)(jh_l + jl_l) as a float pair (ql jl dropped, ~2^-48 relative)
__device__ __forceinline__ void oz_dot3(const float4 &qh, const float4 &ql, const float4 &jh, const float4 &jl,
                                        float &h, float &l) {
    const float p0 = qh.x * jh.x, e0 = fmaf(qh.x, jh.x, -p0) + fmaf(qh.x, jl.x, ql.x * jh.x);
    const float p1 = qh.y * jh.y, e1 = fmaf(qh.y, jh.y, -p1) + fmaf(qh.y, jl.y, ql.y * jh.y);
    const float p2 = qh.z * jh.z, e2 = fmaf(qh.z, jh.z, -p2) + fmaf(qh.z, jl.z, ql.z * jh.z);
    float s, es, s2, es2;
    oz_two_sum(p0, p1, s, es);
    oz_two_sum(s, p2, s2, es2);
    const float err = (e0 + e1) + (e2 + es) + es2;
    oz_two_sum(s2, err, h, l);
}

// digit planes of 8 values (element t in half t % 2 of word t / 2): 8 x 6 digits -> 6 uint4
__device__ __forceinline__ void oz_pack8(const float (&d)[8][OZ_DIG], uint4 (&out)[OZ_DIG]) {
#pragma unroll
    for (int s = 0; s < OZ_DIG; ++s) {
        uint32_t w[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const __nv_bfloat162 b2 = __floats2bfloat162_rn(d[2 * p][s], d[2 * p + 1][s]);
            w[p] = *reinterpret_cast<const uint32_t *>(&b2);
        }
        out[s] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// digits of U at columns c0 .. c0 + 7 (c = 3 g + d, c0 = 3 g0 + D0, all below K) of row (i, b, k),
// scaled by su, packed per digit plane: w[s] holds plane s of the 8 values
template <int NPE, int D0>
__device__ __forceinline__ void oz_row8(const float4 *Qxh, const float4 *Qxl, const float4 *J4h, const float4 *J4l,
                                        int g0, int i, int b, int k, float su, uint4 (&w)[OZ_DIG]) {
    constexpr int NG = (D0 + 7) / 3 + 1;
    float4 jh[NG], jl[NG];
#pragma unroll
    for (int s = 0; s < NG; ++s) {
        jh[s] = __ldg(J4h + (size_t)(g0 + s) * NPE + b);
        jl[s] = __ldg(J4l + (size_t)(g0 + s) * NPE + b);
    }
    uint32_t pw[OZ_DIG][4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        float da[OZ_DIG], db[OZ_DIG];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int t = 2 * p + q, gg = (D0 + t) / 3, dd = (D0 + t) % 3;
            const int o = (g0 + gg) * 27 + 9 * i + 3 * dd + k;
            float h, l;
            oz_dot3(Qxh[o], Qxl[o], jh[gg], jl[gg], h, l);
            oz_digits(h * su, l * su, q == 0 ? da : db);
        }
#pragma unroll
        for (int s = 0; s < OZ_DIG; ++s) {
            const __nv_bfloat162 b2 = __floats2bfloat162_rn(da[s], db[s]);
            pw[s][p] = *reinterpret_cast<const uint32_t *>(&b2);
        }
    }
#pragma unroll
    for (int s = 0; s < OZ_DIG; ++s) w[s] = make_uint4(pw[s][0], pw[s][1], pw[s][2], pw[s][3]);
}

// Jm as float4 pairs: J4h/J4l[g][b] = (Jm[0..2][b][g] hi / lo, 0), zero rows for nq <= g < nq + 4
__global__ void jm_float4_pair(const double *Jm, float4 *J4h, float4 *J4l, int npe, int nq) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (nq + 4) * npe) return;
    const int g = t / npe, b = t % npe;
    float hv[3] = {0.f, 0.f, 0.f}, lv[3] = {0.f, 0.f, 0.f};
    if (g < nq)
        for (int d = 0; d < 3; ++d) {
            const double x = Jm[((size_t)d * npe + b) * nq + g];
            hv[d] = (float)x;
            lv[d] = (float)(x - (double)hv[d]);
        }
    J4h[t] = make_float4(hv[0], hv[1], hv[2], 0.f);
    J4l[t] = make_float4(lv[0], lv[1], lv[2], 0.f);
}

// power-of-two exponent e with 2^e > |x| (x >= 0 finite), 0 for x == 0
__device__ __forceinline__ int oz_exp_above(float x) {
    if (!(x > 0.f)) return 0;
    return ((__float_as_int(x) >> 23) & 0xff) - 127 + 1;
}
__device__ __forceinline__ float oz_pow2(int e) { return __int_as_float((127 + e) << 23); }  // |e| < 127

// shared memory: Qr double [9][nq] | Qxh, Qxl float4 [nq][27] | A digits 6 x [128][KC] bf16 |
// B digits 6 x [NB][KB] bf16 (KB = the reduction padded to whole chunks) | nodes, inv, boff | map
template <int NPE>
__host__ __device__ inline size_t oz_map_offset(int nq, int kc) {
    const int kb = (3 * nq + kc - 1) / kc * kc;
    const size_t b = (sizeof(double) * 9 * (size_t)nq + 15) / 16 * 16 + 2 * sizeof(float4) * 27 * (size_t)nq +
                     sizeof(__nv_bfloat16) * OZ_DIG * ((size_t)TC_MT * kc + (size_t)tc_nb<NPE>() * kb) +
                     sizeof(int) * (NPE + 3 * NPE) + sizeof(int16_t) * NPE * NPE;
    return (b + 15) / 16 * 16;
}
template <int NPE>
__host__ __device__ inline size_t oz_smem_bytes(int nq, int kc, bool stage) {
    const size_t b = oz_map_offset<NPE>(nq, kc) + (stage ? sizeof(int) * 9 * (size_t)NPE * NPE : 0);
    return (b + 127) / 128 * 128;
}

template <int NPE>
__global__ void __launch_bounds__(OZ_THREADS, 2)
    contract_oz_kernel(const AsmArgs A, const float4 *__restrict__ J4h, const float4 *__restrict__ J4l, int KC,
                       int tcols, int stage) {
    constexpr int NDOF = 3 * NPE, M = 9 * NPE, NB = tc_nb<NPE>(), NT = tc_ntiles<NPE>(), CW = tc_colw<NPE>();
    constexpr int RPL = tc_rpl<NPE>(), RPL8 = (RPL + 7) / 8 * 8;
    const int nq = A.nq, K = 3 * nq, KB = (K + KC - 1) / KC * KC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *Qr = reinterpret_cast<double *>(smem_raw);  // [9][nq]
    float4 *Qxh = reinterpret_cast<float4 *>(smem_raw + (sizeof(double) * 9 * (size_t)nq + 15) / 16 * 16);
    float4 *Qxl = Qxh + 27 * nq;
    __nv_bfloat16 *Ad = reinterpret_cast<__nv_bfloat16 *>(Qxl + 27 * nq);  // plane s at s * 128 * KC
    __nv_bfloat16 *Bd = Ad + (size_t)OZ_DIG * TC_MT * KC;                   // plane s at s * NB * KB
    int *nodes = reinterpret_cast<int *>(Bd + (size_t)OZ_DIG * NB * KB);
    int *inv = nodes + NPE;
    int16_t *boff = reinterpret_cast<int16_t *>(inv + NDOF);
    int *dgs = reinterpret_cast<int *>(smem_raw + oz_map_offset<NPE>(nq, KC));
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t taddr_s;
    __shared__ int s_flag, s_amax[2], s_jmax, s_jsum;
    __shared__ int64_t s_nnz;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t cap = (int64_t)NDOF * NDOF;
    const int64_t nwork = A.ne * NT;
    const bool staged = stage && A.dg;
    const bool wide = staged && (cap & 3) == 0 && ((uintptr_t)A.dg & 15) == 0;
    const bool pf = 54 * nq <= OZ_THREADS * TC_PF;
    int flag = 0;
    uint32_t phase = 0;
    if (tid == 0) {
        s_flag = 0;
        s_amax[0] = s_amax[1] = 0;
        s_jmax = s_jsum = 0;
        s_nnz = (int64_t)A.indptr[3 * A.nnode];
        tc::mbar_init(&mbar, 1);
    }
    if (warp == 0) tc::tmem_alloc(&taddr_s, (uint32_t)tcols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = taddr_s;
    const uint32_t idesc = tc::idesc_bf16_f32(TC_MT, NB);
    const uint32_t sbo_a = (uint32_t)(KC / 8) * 128, sbo_b = (uint32_t)(KB / 8) * 128;

    // Jm scale (element type): max |Jm| and the largest sum over l of |Jm[l][b][g]| (hi parts)
    for (int idx = tid; idx < nq * NPE; idx += OZ_THREADS) {
        const float4 j = __ldg(J4h + idx);
        const float ax = fabsf(j.x), ay = fabsf(j.y), az = fabsf(j.z);
        atomicMax(&s_jmax, __float_as_int(fmaxf(ax, fmaxf(ay, az))));
        atomicMax(&s_jsum, __float_as_int(ax + ay + az));
    }
    // lanes past RPL8 are zero rows of every A plane, written once
    for (int idx = tid; idx < TC_MT * (KC / 8); idx += OZ_THREADS) {
        const int rr = idx % TC_MT, cg = idx / TC_MT;
        if ((rr & 31) < RPL8) continue;
        const uint32_t off = tc::kmajor_offset(rr, 8 * cg, KC) / 2;
#pragma unroll
        for (int s = 0; s < OZ_DIG; ++s)
            *reinterpret_cast<uint4 *>(Ad + (size_t)s * TC_MT * KC + off) = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
    const float jsum = __int_as_float(s_jsum) * (1.f + 1.f / 1048576.f);
    const int eJ = oz_exp_above(__int_as_float(s_jmax) * (1.f + 1.f / 1048576.f));
    {  // B digits for the whole reduction: row n = node, column c = 3 g + d
        const float sj = oz_pow2(7 - eJ);
        for (int idx = tid; idx < NB * (KB / 8); idx += OZ_THREADS) {
            const int n = idx % NB, cg = idx / NB;
            float d[8][OZ_DIG];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int c = 8 * cg + t;
                float h = 0.f, l = 0.f;
                if (n < NPE && c < K) {
                    const float4 jh = __ldg(J4h + (size_t)(c / 3) * NPE + n), jl = __ldg(J4l + (size_t)(c / 3) * NPE + n);
                    const int dd = c % 3;
                    h = (dd == 0 ? jh.x : (dd == 1 ? jh.y : jh.z)) * sj;
                    l = (dd == 0 ? jl.x : (dd == 1 ? jl.y : jl.z)) * sj;
                }
                oz_digits(h, l, d[t]);
            }
            uint4 w[OZ_DIG];
            oz_pack8(d, w);
            const uint32_t off = tc::kmajor_offset(n, 8 * cg, KB) / 2;
#pragma unroll
            for (int s = 0; s < OZ_DIG; ++s) *reinterpret_cast<uint4 *>(Bd + (size_t)s * NB * KB + off) = w[s];
        }
    }
    bool ok = true;

    uint64_t pq[TC_PF];  // prefetched Gauss-point values: (lo << 32 | hi) of a tangent entry, or an S double
    int pslot[TC_PF];
#pragma unroll
    for (int j = 0; j < TC_PF; ++j) {
        const int idx = tid + OZ_THREADS * j;
        pslot[j] = pf && idx < 54 * nq ? ((idx / nq) << 16) | (idx % nq) : -1;
    }
    uint64_t pnode = 0;
    int pdl = 0;
    auto load_q = [&](int p, int g, int64_t el) -> uint64_t {
        const size_t col = (size_t)el * nq + g;
        if (p < 45)
            return ((uint64_t)__float_as_uint(A.Qf[(size_t)(45 + p) * A.ldq + col]) << 32) |
                   (uint64_t)__float_as_uint(A.Qf[(size_t)p * A.ldq + col]);
        return (uint64_t)__double_as_longlong(A.Q[(size_t)(p - 45) * A.ldq + col]);
    };
    auto prefetch = [&](int64_t w) {
        if (w >= nwork) return;
        const int64_t el = w / NT, e = A.e0 + el;
        if (tid < NPE) pnode = A.elements[e * NPE + tid];
        if (A.dl && tid < NDOF) pdl = A.dl[e * cap + (int64_t)tid * NDOF];
#pragma unroll
        for (int j = 0; j < TC_PF; ++j)
            if (pslot[j] >= 0) pq[j] = load_q(pslot[j] >> 16, pslot[j] & 0xffff, el);
    };
    auto put_q = [&](int p, int g, uint64_t bits, int *amax) {
        if (p >= 45) {
            Qr[(p - 45) * nq + g] = __longlong_as_double((long long)bits);
            return;
        }
        const float h = __uint_as_float((uint32_t)bits), l = __uint_as_float((uint32_t)(bits >> 32));
        atomicMax(amax, __float_as_int(fabsf(h)));
        const int I = c_sym.I[p], Kc = c_sym.K[p];
        float *qh = reinterpret_cast<float *>(Qxh + (size_t)g * 27), *ql = reinterpret_cast<float *>(Qxl + (size_t)g * 27);
        qh[(I * 3 + Kc / 3) * 4 + Kc % 3] = h;
        ql[(I * 3 + Kc / 3) * 4 + Kc % 3] = l;
        if (Kc != I) {
            qh[(Kc * 3 + I / 3) * 4 + I % 3] = h;
            ql[(Kc * 3 + I / 3) * 4 + I % 3] = l;
        }
    };
    prefetch(blockIdx.x);

    int it = 0;
    for (int64_t w = blockIdx.x; w < nwork && ok; w += gridDim.x, ++it) {
        const int64_t el = w / NT, e = A.e0 + el;
        const int t0 = (int)(w % NT);
        int *amax = &s_amax[it & 1];
        __syncthreads();  // previous work item done with the shared buffers
        if (tid == 0) s_amax[(it + 1) & 1] = 0;  // for the next item (read by nobody until then)
        for (int a = tid; a < NPE; a += OZ_THREADS) {
            uint64_t nd = a == tid ? pnode : A.elements[e * NPE + a];
            if (nd >= (uint64_t)A.nnode) {
                flag |= FL_FLAG_BAD_INDEX;
                nd = 0;
            }
            nodes[a] = (int)nd;
        }
        if (A.dl)
            for (int i = tid; i < NDOF; i += OZ_THREADS) {
                const int v = i == tid ? pdl : A.dl[e * cap + (int64_t)i * NDOF];
                const int p = v / NDOF;
                if (v < 0 || p >= NDOF) flag |= FL_FLAG_BAD_INDEX;
                else inv[p] = i;
            }
        if (pf) {
#pragma unroll
            for (int j = 0; j < TC_PF; ++j)
                if (pslot[j] >= 0) put_q(pslot[j] >> 16, pslot[j] & 0xffff, pq[j], amax);
        } else {
            for (int idx = tid; idx < 54 * nq; idx += OZ_THREADS)
                put_q(idx / nq, idx % nq, load_q(idx / nq, idx % nq, el), amax);
        }
        __syncthreads();
        if (staged) {
            const int *src = A.dg + e * cap;
            if (wide)
                for (int i = 4 * tid; i < cap; i += 4 * OZ_THREADS) cp_async16(dgs + i, src + i);
            else
                for (int i = tid; i < cap; i += OZ_THREADS) cp_async4(dgs + i, src + i);
            cp_async_commit();
        }
        prefetch(w + gridDim.x);
        if (!A.dl)
            for (int idx = tid; idx < NPE * NPE; idx += OZ_THREADS) {
                const int off = row_search(A.indptr, A.indices, 3 * nodes[idx / NPE], 3 * nodes[idx % NPE]);
                boff[idx] = (int16_t)(off >= 0 && off < 32768 ? off : -1);
            }
        if (A.update && t0 == 0) {  // residual in FP64, four threads per dof
            for (int base = 0; base < 4 * NDOF; base += OZ_THREADS) {
                const int idx = base + tid, r = idx >> 2, part = idx & 3;
                double t = 0.0;
                if (r < NDOF) {
                    const int a = r / 3, i = r % 3;
                    for (int g = part; g < nq; g += 4) {
                        t = fma(__ldg(A.Jm + (size_t)a * nq + g), Qr[(i * 3) * nq + g], t);
                        t = fma(__ldg(A.Jm + ((size_t)NPE + a) * nq + g), Qr[(i * 3 + 1) * nq + g], t);
                        t = fma(__ldg(A.Jm + ((size_t)2 * NPE + a) * nq + g), Qr[(i * 3 + 2) * nq + g], t);
                    }
                }
                t += __shfl_xor_sync(0xffffffffu, t, 1);
                t += __shfl_xor_sync(0xffffffffu, t, 2);
                if (r < NDOF && part == 0) atomicAdd(A.T + 3 * (int64_t)nodes[r / 3] + r % 3, t);
            }
        }
        const int eU = oz_exp_above(__int_as_float(*amax) * jsum);
        const float su = oz_pow2(7 - eU);
        for (int k0 = 0; k0 < K; k0 += KC) {
            const int kc = min(KC, K - k0);
            // A digits: item = (row rl of the tile, 8-column group cg), rows as in section D
            constexpr int NRG = 4 * RPL8;
            for (int idx = tid; idx < NRG * (KC / 8); idx += OZ_THREADS) {
                const int cg = idx / NRG, rl = idx - cg * NRG, c0 = k0 + 8 * cg;
                const int q4 = rl / RPL8, l8 = rl - q4 * RPL8, rr = 32 * q4 + l8, r = (4 * t0 + q4) * RPL + l8;
                const bool live = l8 < RPL && r < M;
                const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
                uint4 wv[OZ_DIG];
                if (live && c0 + 8 <= K) {
                    const int g0 = c0 / 3;
                    switch (c0 - 3 * g0) {
                        case 0: oz_row8<NPE, 0>(Qxh, Qxl, J4h, J4l, g0, i, b, k, su, wv); break;
                        case 1: oz_row8<NPE, 1>(Qxh, Qxl, J4h, J4l, g0, i, b, k, su, wv); break;
                        default: oz_row8<NPE, 2>(Qxh, Qxl, J4h, J4l, g0, i, b, k, su, wv); break;
                    }
                } else {
                    float d[8][OZ_DIG];
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        const int c = c0 + t;
                        float h = 0.f, l = 0.f;
                        if (live && c < K) {
                            const int g = c / 3, dd = c % 3;
                            oz_dot3(Qxh[(size_t)g * 27 + 9 * i + 3 * dd + k], Qxl[(size_t)g * 27 + 9 * i + 3 * dd + k],
                                    __ldg(J4h + (size_t)g * NPE + b), __ldg(J4l + (size_t)g * NPE + b), h, l);
                            h *= su;
                            l *= su;
                        }
                        oz_digits(h, l, d[t]);
                    }
                    oz_pack8(d, wv);
                }
                const uint32_t off = tc::kmajor_offset(rr, 8 * cg, KC) / 2;
#pragma unroll
                for (int s = 0; s < OZ_DIG; ++s) *reinterpret_cast<uint4 *>(Ad + (size_t)s * TC_MT * KC + off) = wv[s];
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
                // level w = i + j into accumulator w (columns w CW); the first product of a level
                // overwrites it
                uint64_t da0[OZ_DIG], db0[OZ_DIG];
#pragma unroll
                for (int s = 0; s < OZ_DIG; ++s) {
                    da0[s] = tc::smem_desc(Ad + (size_t)s * TC_MT * KC, 128, sbo_a);
                    db0[s] = tc::smem_desc(Bd + (size_t)s * NB * KB, 128, sbo_b);
                }
                for (int ks = 0; 16 * ks < kc; ++ks)
#pragma unroll
                    for (int lv = 0; lv < OZ_DIG; ++lv)
#pragma unroll
                        for (int i = 0; i <= lv; ++i)
                            tc::mma_bf16(taddr + (uint32_t)(lv * CW), da0[i] + (uint64_t)(16 * ks),
                                         db0[lv - i] + (uint64_t)(k0 + 16 * ks), idesc, k0 > 0 || ks > 0 || i > 0);
                tc::mma_commit(&mbar);
            }
            if (staged && k0 + KC >= K) cp_async_wait_all();
            ok = __syncthreads_and(warp == 0 ? tc::mbar_wait(&mbar, phase & 1, TC_WAIT) : true) != 0;
            ++phase;
            tc::fence_after_sync();
            if (!ok) break;
        }
        if (!ok) {
            flag |= FL_FLAG_BAD_INDEX;
            break;
        }
        // read back: 16-column blocks alternating between warps w and w + 4. Levels 5..3 (weights
        // 2^-40..2^-24) are combined in FP32; levels 2, 1, 0, whose sums are exact integers, join
        // as float pairs; then the scale and the FP64 add
        const int sub = warp & 3, half = warp >> 2;
        constexpr int CB = NB / 16;
        const float scale = oz_pow2(eU + eJ - 14);
        const int r = (4 * t0 + sub) * RPL + lane;
        const bool row_ok = lane < RPL && r < M;
        const int k = r % 3, b = (r / 3) % NPE, i = r / (3 * NPE);
        const int ic = A.dl && row_ok ? inv[3 * b + k] : 0;
        const uint32_t tl = taddr + ((uint32_t)(32 * sub) << 16);
#pragma unroll
        for (int u = 0; u < CB; ++u) {
            if ((u & 1) != half) continue;  // warp-uniform
            const int c0 = u * 16;
            constexpr int NV = 16;
            float hh[NV], ll[NV], v[NV];
            tc::tmem_ld16(tl + (uint32_t)(5 * CW + c0), v);
#pragma unroll
            for (int j = 0; j < NV; ++j) hh[j] = v[j];
            tc::tmem_ld16(tl + (uint32_t)(4 * CW + c0), v);
#pragma unroll
            for (int j = 0; j < NV; ++j) hh[j] = fmaf(hh[j], 1.f / 256.f, v[j]);
            tc::tmem_ld16(tl + (uint32_t)(3 * CW + c0), v);
#pragma unroll
            for (int j = 0; j < NV; ++j) {
                hh[j] = fmaf(hh[j], 1.f / 256.f, v[j]);
                ll[j] = 0.f;
            }
#pragma unroll 1
            for (int lv = 2; lv >= 0; --lv) {
                tc::tmem_ld16(tl + (uint32_t)(lv * CW + c0), v);
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    float sh, e2;
                    oz_two_sum(v[j], hh[j] * (1.f / 256.f), sh, e2);
                    ll[j] = fmaf(ll[j], 1.f / 256.f, e2);
                    hh[j] = sh;
                }
            }
            if (!row_ok) continue;
            if (A.dl) {
                int64_t pos[NV];
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    const int a = c0 + j;
                    pos[j] = -1;
                    if (a < NPE) {
                        const int ir = inv[3 * a + i];
                        if ((unsigned)ir < (unsigned)NDOF && (unsigned)ic < (unsigned)NDOF)
                            pos[j] = staged ? (int64_t)dgs[ir * NDOF + ic] : (int64_t)A.dg[e * cap + (int64_t)ir * NDOF + ic];
                    }
                }
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    if (c0 + j >= NPE) continue;
                    const double vv = (double)(hh[j] * scale) + (double)(ll[j] * scale);
                    if (pos[j] >= 0 && pos[j] < s_nnz) atomicAdd(A.V + pos[j], vv);
                    else flag |= FL_FLAG_BAD_INDEX;
                }
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    const int a = c0 + j;
                    if (a >= NPE) continue;
                    const double vv = (double)(hh[j] * scale) + (double)(ll[j] * scale);
                    const int64_t pos = block_entry(A.indptr, A.indices, nodes[a], nodes[b], i, k, boff[a * NPE + b]);
                    if (pos >= 0 && pos < s_nnz) atomicAdd(A.V + pos, vv);
                    else flag |= FL_FLAG_BAD_INDEX;
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    cp_async_wait_all();
    if (!ok) (void)__syncthreads_and(warp == 0 ? tc::mbar_wait(&mbar, (phase - 1) & 1, TC_WAIT) : true);
    if (flag) atomicOr(&s_flag, flag);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, (uint32_t)tcols);
    if (tid == 0 && s_flag && A.flags) atomicOr(A.flags, s_flag);
}

// Plan of the FP64 tensor-core kernel: one tile per item (6 accumulators of CW columns); the
// element map staged in shared memory if possible, with the widest reduction chunk (multiple of
// 16) that leaves room for two CTAs per SM, else for one.
// Unsupported (0) when the exact levels could overflow FP32 (3 K 2^14 >= 2^24) or nothing fits.
template <int NPE>
static TcPlan oz_plan(int nq) {
    constexpr int CW = tc_colw<NPE>();
    if (3 * 3 * nq * 16384.0 >= 16777216.0 || OZ_DIG * CW > 512) return TcPlan{0, 0, 0, 0, 0};
    const int kmax = std::min(MX_KC, (3 * nq + 15) / 16 * 16);
    const size_t limit[2] = {113 * 1024, 227 * 1024};
    int cols = 32;
    while (cols < OZ_DIG * CW) cols *= 2;
    for (int pass = 0; pass < 2; ++pass)
        for (int stage = 1; stage >= 0; --stage)  // the staged map first (the scatter's latency)
            for (int kc = kmax; kc >= 16; kc -= 16) {
                const size_t s = oz_smem_bytes<NPE>(nq, kc, stage != 0);
                if (s <= limit[pass]) return TcPlan{kc, 1, cols, s, stage};
            }
    return TcPlan{0, 0, 0, 0, 0};
}

template <int NPE>
static bool oz_supported(int nq) { return oz_plan<NPE>(nq).tg > 0; }

template <int NPE, int MAT>
static int launch_oz(AsmArgs A, cudaStream_t stream) {
    if (A.nelem == 0) return FL_OK;
    const TcPlan P = oz_plan<NPE>(A.nq);
    if (P.tg == 0) return FL_ERR_UNSUPPORTED;
    { const int st = ensure_smem<contract_oz_kernel<NPE>>(P.smem); if (st != FL_OK) return st; }
    // Gauss-point scratch per chunk: S [9][ldq] FP64, the tangent as float pairs [90][ldq]
    // (288 bytes per point), then the float4 pair tables of Jm
    int64_t chunk = std::max<int64_t>(1, (int64_t)(CHUNK_BYTES / ((9 * sizeof(double) + 90 * sizeof(float)) * (size_t)A.nq)));
    if (chunk > A.nelem) chunk = A.nelem;
    const size_t sbytes = (sizeof(double) * 9 * (size_t)A.nq * chunk + 255) & ~(size_t)255;
    const size_t fbytes = (sizeof(float) * 90 * (size_t)A.nq * chunk + 255) & ~(size_t)255;
    const int64_t nj4 = (int64_t)(A.nq + 4) * NPE;
    const size_t jbytes = (sizeof(float4) * (size_t)nj4 + 255) & ~(size_t)255;
    double *Q = nullptr;
    FL_CUDA_TRY(cudaMallocAsync((void **)&Q, sbytes + fbytes + 2 * jbytes + pair_prep_bytes(A.nnode, NPE, A.nq), stream));
    pair_prep(A, NPE, reinterpret_cast<char *>(Q) + sbytes + fbytes + 2 * jbytes, stream);
    A.npair = nullptr;  // FP64 kinematics: see launch_rt (sliver elements)
    A.Q = Q;
    A.Qf = reinterpret_cast<float *>(reinterpret_cast<char *>(Q) + sbytes);
    A.ldq = chunk * A.nq;
    float4 *J4h = reinterpret_cast<float4 *>(reinterpret_cast<char *>(Q) + sbytes + fbytes);
    float4 *J4l = reinterpret_cast<float4 *>(reinterpret_cast<char *>(J4h) + jbytes);
    jm_float4_pair<<<(unsigned)((nj4 + 255) / 256), 256, 0, stream>>>(A.Jm, J4h, J4l, NPE, A.nq);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int occ = tc_ctas_per_sm(reinterpret_cast<const void *>(contract_oz_kernel<NPE>), P);
    for (int64_t e0 = 0; e0 < A.nelem; e0 += chunk) {
        A.e0 = e0;
        A.ne = A.nelem - e0 < chunk ? A.nelem - e0 : chunk;
        const int64_t nqp = A.ne * A.nq;
        qp_kernel<NPE, MAT, QOUT_DF><<<(unsigned)((nqp + QP_THREADS - 1) / QP_THREADS), QP_THREADS, 0, stream>>>(A);
        const int64_t grid = std::min<int64_t>(A.ne * tc_ntiles<NPE>(), (int64_t)sms * occ);
        contract_oz_kernel<NPE><<<(unsigned)grid, OZ_THREADS, P.smem, stream>>>(A, J4h, J4l, P.kc, P.tcols, P.stage);
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
    (void)sorter; (void)rho; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e;
    fl::MatParams mp;
    int mat = 0;
    // the two materials of its contract (the others read further arrays a range-by-range caller
    // would have to offset)
    if (material_number != FL_MATERIAL_NEOHOOKEAN && material_number != FL_MATERIAL_MOONEYRIVLIN)
        return FL_ERR_UNSUPPORTED;
    if (fl::material_of(material_number, mu, mu1, mu2, lamb, &mat, &mp, mu3) != FL_OK) return FL_ERR_UNSUPPORTED;
    if (ngauss <= 0 || ngauss > 343 || nelem < 0) return FL_ERR_ARG;
    // the whole mesh must fit the array: nelem * ngauss Gauss points of 54 doubles (the kernels
    // may still process it in more than one chunk of whole contraction tiles)
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
                                  (cudaStream_t)stream, nullptr, anisotropic_orientations);
}

int fl_GlobalAssemblyDF_Mixed(int material_number, const double *points, const uint64_t *elements,
                              const double *Eulerx, const double *Jm, const double *AllGauss, int64_t ngauss,
                              int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t requires_geometry_update,
                              const int32_t *indptr, const int32_t *indices, const int32_t *data_local_indices,
                              const int32_t *data_global_indices, float *V_stiff, double *T, double mu, double mu1,
                              double mu2, double lamb, double mu3, const double *anisotropic_orientations,
                              const double *element_params, int *flags, fl_stream_t stream) {
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
    A.w = AllGauss;
    A.nelem = nelem;
    A.nnode = nnode;
    A.nq = (int)ngauss;
    A.update = requires_geometry_update ? 1 : 0;
    A.boff = nullptr;
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
    A.Qf = nullptr;
    A.orient = nullptr;
    A.npair = nullptr;
    A.jmp = nullptr;
    A.e0 = A.ne = A.ldq = 0;
    int mat = 0;
    if (fl::material_of(material_number, mu, mu1, mu2, lamb, &mat, &A.mp, mu3) != FL_OK) return FL_ERR_UNSUPPORTED;
    if (mat == fl::ANISOTROPICMR1) {
        if (!anisotropic_orientations) return FL_ERR_ARG;
        if (element_params) return FL_ERR_UNSUPPORTED;
        A.orient = anisotropic_orientations;
    }
    cudaStream_t s = (cudaStream_t)stream;
    switch (mat) {
        case fl::NEOHOOKEAN: return fl::mixed_dispatch<fl::NEOHOOKEAN>((int)nodeperelem, A, V_stiff, s);
        case fl::MOONEYRIVLIN: return fl::mixed_dispatch<fl::MOONEYRIVLIN>((int)nodeperelem, A, V_stiff, s);
        case fl::ANISOTROPICMR1: return fl::mixed_dispatch<fl::ANISOTROPICMR1>((int)nodeperelem, A, V_stiff, s);
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
    if (arithmetic != FL_ARITH_FP64 && arithmetic != FL_ARITH_FLOAT_PAIR && arithmetic != FL_ARITH_TENSOR &&
        arithmetic != FL_ARITH_REFERENCE_TENSOR)
        return FL_ERR_ARG;
    fl::g_arith.store(arithmetic);
    return FL_OK;
}

int fl_GetAssemblyArithmetic(void) { return fl::g_arith.load(); }

int fl_SetTensorCoreTiling(int tile_group, int reduction_chunk) {
    if (tile_group < 0 || tile_group > 16 || reduction_chunk < 0 || reduction_chunk > fl::MX_KC) return FL_ERR_ARG;
    fl::g_tc_tg.store(tile_group);
    fl::g_tc_kc.store(reduction_chunk);
    return FL_OK;
}

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

int fl_GlobalAssemblyDF__AnisotropicMooneyRivlin_1_(FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mu; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e;
    fl::MatParams mp{mu1, mu2, lamb, mu3};
    return fl::global_assembly_df(fl::ANISOTROPICMR1, points, elements, Eulerx, Jm, AllGauss, ndim, nvar, ngauss,
                                  nelem, nodeperelem, nnode, H_VoigtSize, requires_geometry_update, I_stiff, J_stiff,
                                  V_stiff, T, recompute_sparsity_pattern, squeeze_sparsity_pattern, data_local_indices,
                                  data_global_indices, mp, flags, nullptr, 0, (cudaStream_t)stream, nullptr,
                                  anisotropic_orientations);
}

int fl_ReferenceGeometry(const double *points, const uint64_t *elements, const double *Jm, int64_t nelem,
                         int64_t nodeperelem, int64_t ngauss, int64_t nnode, double *geometry, int *flags,
                         fl_stream_t stream) {
    if (nelem < 0 || ngauss <= 0 || nnode <= 0) return FL_ERR_ARG;
    if (nelem == 0) return FL_OK;
    if (!points || !elements || !Jm || !geometry) return FL_ERR_ARG;
    const int64_t n = nelem * ngauss;
    const unsigned grid = (unsigned)((n + fl::QP_THREADS - 1) / fl::QP_THREADS);
    cudaStream_t st = (cudaStream_t)stream;
    switch (nodeperelem) {
#define FL_GEO_CASE(NPE) \
        case NPE: fl::reference_geometry_kernel<NPE><<<grid, fl::QP_THREADS, 0, st>>>(points, elements, Jm, nelem, (int)ngauss, nnode, geometry, flags); break;
        FL_GEO_CASE(4) FL_GEO_CASE(8) FL_GEO_CASE(10) FL_GEO_CASE(20) FL_GEO_CASE(27) FL_GEO_CASE(35) FL_GEO_CASE(64)
        FL_GEO_CASE(125)
#undef FL_GEO_CASE
        default: return FL_ERR_UNSUPPORTED;
    }
    return fl::launch_status();
}

int fl_GlobalAssemblyDF_Blocks(int material_number, const int32_t *block_offsets, const double *reference_geometry,
                               FL_GLOBAL_ASSEMBLY_DF_ARGS) {
    (void)Eulerp; (void)bases; (void)local_rows_stiffness; (void)local_cols_stiffness; (void)sorted_elements;
    (void)sorter; (void)rho; (void)mue; (void)eps_1; (void)eps_2; (void)eps_3; (void)eps_e;
    fl::MatParams mp;
    int mat = 0;
    if (fl::material_of(material_number, mu, mu1, mu2, lamb, &mat, &mp, mu3) != FL_OK) return FL_ERR_UNSUPPORTED;
    return fl::global_assembly_df(mat, points, elements, Eulerx, Jm, AllGauss, ndim, nvar, ngauss, nelem, nodeperelem,
                                  nnode, H_VoigtSize, requires_geometry_update, I_stiff, J_stiff, V_stiff, T,
                                  recompute_sparsity_pattern, squeeze_sparsity_pattern, data_local_indices,
                                  data_global_indices, mp, flags, nullptr, 0, (cudaStream_t)stream, nullptr,
                                  anisotropic_orientations, block_offsets, reference_geometry);
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
