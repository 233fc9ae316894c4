// fl_reftensor.cu -- the FP64 element tangents as one tensor-core GEMM per tile of elements.
//
// The Gauss-point kernel (fl_assembly.cu) pulls the tangent back to the reference element,
//     Ahat_g[(i,d),(k,e)] = detJ sum_{j,l} G[j][d] A_ijkl G[l][e],   G = (dx/dxi)^{-1},
// so that the element matrix of the displacement formulation (_ConstitutiveStiffnessDF_.h:83-156
// plus _GeometricStiffness_.h:61-99, as _LowLevelAssemblyDF_.h:8-176 forms it) is
//     K_e[(a,i),(b,k)] = sum_{g,d,e} Jm[d][a][g] Jm[e][b][g] Ahat_g[(i,d),(k,e)].
// The shape-function gradients Jm on the reference element are the same for every element, so
// with the reference tensor Phi[(a,b),(g,d,e)] = Jm[d][a][g] Jm[e][b][g] (node pairs a <= b) this
// is a GEMM per tile of elements,
//     K[(el,i,k), (a,b)] = sum_{(g,d,e)} Ahat[(el,i,k), (g,d,e)] Phi[(a,b), (g,d,e)],
// the reference-tensor / geometry-tensor factorisation of Kirby and Logg ("A compiler for
// variational forms", ACM TOMS 32, 2006), here with the element-dependent factor being the
// pulled-back tangent itself (81 values per Gauss point, 9 nq per element row of the GEMM).
//
// FP64 accuracy on BF16 tensor cores (the Ozaki splitting, Ozaki et al., Numer. Algorithms 59,
// 2012): every row of Ahat and every column of Phi is scaled by a power of two into (-128, 128)
// and written as seven digit planes x = p0 + p1 + ... + p6 with p_s an integer multiple of 2^-8s
// of at most 128 in magnitude (8 significant bits: exact in BF16). The 28 plane products (s, t)
// with s + t <= 6 are accumulated per level L = s + t in FP32 tensor memory; a product is at most
// 2^14 times the level weight and K <= 256, so the levels 0-3 (at most 4 products each) sum
// exactly; levels 4 to 6 share the fifth accumulator (their rounding is below 2^-55 of the row
// and column scales). The truncation after level 6 is below 2^-49 K max|row| max|column|: six
// planes (2^-41) were measured too coarse for the sliver elements of a Delaunay mesh.
// The epilogue turns the five sums into one 64-bit fixed-point integer and that into the FP64
// value exactly rounded, with integer instructions only (GB300's FP64 pipe is 1/64 of FP32).
//
// Work split (one persistent CTA per SM, 544 threads):
//   warps 0-7   epilogue: per tile the residual (float pairs, atomic adds); per chunk, two warps
//               per tensor-memory lane quarter (alternate groups of 8 columns), tensor memory ->
//               FP64 entries -> atomic adds into the CSR values
//   warps 8-15  producers: per tile the node tables, block offsets, one bulk copy per row of the
//               tile's Gauss-point data, the row scales; per 16-wide K step the seven A planes
//               (two threads per row, one 8-column half each)
//   warp 16     one thread: bulk copies of the Phi planes (cp.async.bulk) and the 28 MMAs per step
// A tile is 14 elements (126 of the 128 MMA rows); the 210 node pairs of a 20-node tet run as
// three 80-column chunks (five accumulators of 80 columns fit the 512 tensor-memory columns),
// each chunk re-deriving the A planes. Every wait is bounded: a timeout sets FL_FLAG_TIMEOUT,
// all roles leave their loops, in-flight copies and MMAs are waited for (bounded) and the tensor
// memory is released.
#include <cuda_bf16.h>

#include <algorithm>

#include "fl_common.cuh"
#include "fl_reftensor.cuh"
#include "fl_reftensor_math.cuh"
#include "fl_tc.cuh"

namespace fl {

constexpr int RT_EPT = 14;                // elements per tile (9 rows each)
constexpr int RT_M = 128;                 // MMA rows
constexpr int RT_NACC = 5;                // accumulators (levels 0, 1, 2, 3, 4-6)
constexpr int RT_ACCSTRIDE = 96;          // tensor-memory columns between accumulators
constexpr int RT_TMEM_COLS = 512;
constexpr int RT_NST = 2;                 // pipeline stages
constexpr int RT_A_PLANE = RT_M * 16 * 2;                 // bytes of one A plane of a 16-wide K step
constexpr int RT_B_PLANE = RT_NB * 16 * 2;
constexpr int RT_A_BYTES = RT_DIG * RT_A_PLANE;           // 28 672
constexpr int RT_B_BYTES = RT_DIG * RT_B_PLANE;           // 17 920
constexpr int RT_STAGE = RT_A_BYTES + RT_B_BYTES;
constexpr int RT_NEPI = 256;              // epilogue threads: two warps per tensor-memory lane quarter
constexpr int RT_NPROD = 256;             // producer threads: two per A row
constexpr int RT_THREADS = RT_NEPI + RT_NPROD + 32;
constexpr int RT_MMA_WARP = (RT_NEPI + RT_NPROD) / 32;
constexpr int RT_MAX_NQ = 15;             // the tile's Gauss-point data must fit in shared memory
constexpr long long RT_WAIT_LIMIT = 1ll << 23;
constexpr int RT_MAXCOLS = 256;           // pair columns of the largest element type taken (20 nodes: 240)
constexpr int RT_MAXK = 16 * 9;           // K columns for up to 15 Gauss points (135, padded to 144)

// ------------------------------------------------------------------------------------------------
// device pieces: barriers, bulk copies, tensor-memory loads
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(mbar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(saddr(mbar)), "r"(parity)
        : "memory");
    return done != 0;
}

// phase `parity` of the mbarrier complete, waiting in hardware (the thread is suspended until the
// phase completes or about `ns` nanoseconds pass, so waiting warps take no issue slots)
__device__ __forceinline__ bool mbar_try(uint64_t *mbar, uint32_t parity, uint32_t ns) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(saddr(mbar)), "r"(parity), "r"(ns)
        : "memory");
    return done != 0;
}

// bounded wait; gives up (and raises the CTA's abort flag) after RT_WAIT_TRIES suspensions of up
// to 100 microseconds (well under a second in all), or at once when another role has aborted
constexpr int RT_WAIT_TRIES = 4000;
__device__ __forceinline__ bool rt_wait(uint64_t *mbar, uint32_t parity, volatile int *abort_flag) {
    if (mbar_test(mbar, parity)) return true;
    for (int i = 0; i < RT_WAIT_TRIES; ++i) {
        if (mbar_try(mbar, parity, 100000u)) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(mbar))
                 : "memory");
}

__device__ __forceinline__ void producers_sync() { asm volatile("bar.sync 1, 256;\n" ::: "memory"); }

// 8 consecutive FP32 columns of this warp's 32 lanes, no wait
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

// 16 consecutive FP32 columns of this warp's 32 lanes, no wait
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// per-tile tables of the epilogue (double-buffered by tile)
template <int NPE>
struct RtTables {
    int nodes[RT_EPT * NPE];
    int rs0[RT_EPT * NPE];     // indptr[3 node]
    int rlen[RT_EPT * NPE];    // length of each of the node's three rows
    int rexp[RT_M];            // row exponents
    int16_t boff[RT_EPT * NPE * NPE];
};

template <int NPE>
__host__ __device__ constexpr size_t rt_tables_bytes() { return (sizeof(RtTables<NPE>) + 127) / 128 * 128; }

// shared memory: stages | the tile's Gauss-point data (tangent hi [45][TQ], lo [45][TQ], residual
// factor hi [9][TQ], lo [9][TQ]; TQ = 14 nq) | tables x 2 | column exponents | row scales | Jm pairs
__host__ __device__ inline size_t rt_tile_bytes(int nq) {
    return ((size_t)(2 * 45 + 2 * 9) * RT_EPT * nq * sizeof(float) + 127) / 128 * 128;
}
template <int NPE>
__host__ __device__ inline size_t rt_smem_bytes(int nq) {
    return (size_t)RT_NST * RT_STAGE + rt_tile_bytes(nq) + 2 * rt_tables_bytes<NPE>() +
           (size_t)rt_chunks(NPE) * RT_NB * sizeof(int) + RT_M * sizeof(float) +
           ((size_t)3 * NPE * nq * sizeof(float2) + 127) / 128 * 128 + 256;
}

// CSR position of entry (3 nr + ri, 3 nc + ci) by binary search in the row, -1 if absent
__device__ __forceinline__ int64_t rt_search(const int32_t *indptr, const int32_t *indices, int nr, int ri, int nc,
                                             int ci) {
    const int row = 3 * nr + ri, col = 3 * nc + ci;
    int lo = indptr[row], hi = indptr[row + 1];
    const int end = hi;
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (col < indices[mid]) hi = mid; else lo = mid;
    }
    return (lo < end && indices[lo] == col) ? (int64_t)lo : -1;
}

template <int NPE>
__global__ void __launch_bounds__(RT_THREADS, 1) rt_contract_kernel(const RtArgs R) {
    constexpr int P = rt_pairs(NPE), NCH = rt_chunks(NPE);
    const int nq = R.nq, K = 9 * nq, NKS = rt_ksteps(nq), TQ = RT_EPT * nq;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *stages = smem;
    float *AH = reinterpret_cast<float *>(smem + (size_t)RT_NST * RT_STAGE);
    float *AL = AH + 45 * TQ;
    float *SH = AL + 45 * TQ;  // residual factor S_g[i][d] of the tile, hi [9][TQ] then lo [9][TQ]
    float *SL = SH + 9 * TQ;
    RtTables<NPE> *tables = reinterpret_cast<RtTables<NPE> *>(smem + (size_t)RT_NST * RT_STAGE + rt_tile_bytes(nq));
    int *colexp = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(tables) + 2 * rt_tables_bytes<NPE>());
    float *rsc = reinterpret_cast<float *>(colexp + NCH * RT_NB);
    float2 *jms = reinterpret_cast<float2 *>(rsc + RT_M);  // Jm as float pairs [3][NPE][nq]

    // fullA: the 8 producer warps wrote a stage's A planes; fullB: its Phi planes arrived (bulk
    // copy bytes); empty: the MMAs reading the stage completed; accf / acce: a chunk's
    // accumulators are complete / were read out; tblf / tble: a tile's tables are written / no
    // longer needed; fin: every MMA issued has completed
    __shared__ __align__(8) uint64_t fullA[RT_NST], fullB[RT_NST], empty_bar[RT_NST], accf_bar, acce_bar,
        tblf_bar[2], tble_bar[2], rdone_bar, stage_bar, fin_bar;
    __shared__ uint32_t taddr_s;
    __shared__ volatile int s_abort;
    __shared__ int s_flag;
    __shared__ int64_t s_nnz;
    // index tables: node pair (a, b) of each pair column; Gauss point and (d, e) of each K column;
    // per row (el, i, k) the offset of its tangent entries (3i + d, 3k + e) in the tile data
    __shared__ int8_t pair_a[RT_MAXCOLS], pair_b[RT_MAXCOLS];
    __shared__ uint8_t k_g[RT_MAXK], k_de[RT_MAXK];
    __shared__ int16_t row_off[RT_M][9];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (R.ne + RT_EPT - 1) / RT_EPT;
    const int64_t mine = (int64_t)blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t total_steps = mine * NCH * NKS;

    if (tid == 0) {
        for (int s = 0; s < RT_NST; ++s) {
            tc::mbar_init(&fullA[s], RT_NPROD / 32);
            tc::mbar_init(&fullB[s], 1);
            tc::mbar_init(&empty_bar[s], 1);
        }
        tc::mbar_init(&accf_bar, 1);
        tc::mbar_init(&acce_bar, RT_NEPI / 32);
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tblf_bar[b], RT_NPROD / 32);
            tc::mbar_init(&tble_bar[b], RT_NEPI / 32);
        }
        tc::mbar_init(&rdone_bar, RT_NEPI / 32);  // the epilogue warps read the tile's residual factors
        tc::mbar_init(&stage_bar, 1);  // the tile's Gauss-point data landed (bulk copy bytes)
        tc::mbar_init(&fin_bar, 1);
        s_abort = 0;
        s_flag = 0;
        s_nnz = (int64_t)R.indptr[3 * R.nnode];
    }
    for (int n = tid; n < NCH * RT_NB; n += RT_THREADS) {
        colexp[n] = R.phiexp[n];
        int a = 0, b = 0;
        if (n < P) rt_pair(n, a, b);
        pair_a[n] = (int8_t)a;
        pair_b[n] = (int8_t)b;
    }
    for (int kk = tid; kk < NKS * 16; kk += RT_THREADS) {
        k_g[kk] = (uint8_t)(kk < K ? kk / 9 : 0);
        k_de[kk] = (uint8_t)(kk < K ? kk % 9 : 0);
    }
    if (tid < RT_M) {
        const int el = tid / 9, i = (tid % 9) / 3, k = tid % 3;
        for (int de = 0; de < 9; ++de)
            row_off[tid][de] = (int16_t)(tid < 9 * RT_EPT ? rt_sym9(3 * i + de / 3, 3 * k + de % 3) * TQ + el * nq : 0);
    }
    for (int n = tid; n < 3 * NPE * nq; n += RT_THREADS) jms[n] = R.jmp[n];
    if (warp == RT_MMA_WARP) tc::tmem_alloc(&taddr_s, RT_TMEM_COLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = taddr_s;
    int flag = 0;

    if (warp >= RT_NEPI / 32 && warp < RT_MMA_WARP) {
        // ---------------------------------------------------------------------------- producers
        const int p = tid - RT_NEPI;
        bool stage_pending = false;  // (thread p == 0) a bulk copy of tile data not yet waited for
        uint32_t stage_parity = 0;
        int64_t gs = 0;
        for (int64_t it = 0; it < mine && !s_abort; ++it) {
            const int64_t tile = blockIdx.x + it * (int64_t)gridDim.x;
            const int buf = (int)(it & 1);
            const int64_t el0 = tile * RT_EPT;  // chunk-local index of the tile's first element
            RtTables<NPE> &tb = tables[buf];
            // the tile data are overwritten once the epilogue has formed the previous tile's residual
            if (it >= 1 && !rt_wait(&rdone_bar, (uint32_t)((it - 1) & 1), &s_abort)) break;
            producers_sync();  // every producer is past the previous tile's K steps
            // the tile's Gauss-point data: 108 rows (tangent hi, lo; residual factor hi, lo) of TQ
            // floats; as one bulk copy per row when the rows are 16-byte aligned (an even number of
            // Gauss points), overlapping the table loads, else with plain loads
            const int64_t c0 = el0 * nq, cend = R.ne * nq;
            auto row_src = [&](int row) -> const float * {
                return row < 45 ? R.Qh + (size_t)row * R.ldq
                       : row < 90 ? R.Ql + (size_t)(row - 45) * R.ldq
                                  : R.Sp + (size_t)(row - 90) * R.ldq;
            };
            const bool bulk = (TQ & 3) == 0;
            if (bulk && p == 0) {
                const int64_t avail = R.ldq - c0;  // the rows' floats from c0 to the end of the row
                const uint32_t nb = (uint32_t)((avail < TQ ? avail : TQ) * 4) & ~15u;
                tc::fence_async_smem();  // the previous tile's generic reads of the buffer come first
                mbar_arrive_tx(&stage_bar, 108u * nb);
                if (nb)
                    for (int row = 0; row < 108; ++row) bulk_g2s(AH + (size_t)row * TQ, row_src(row) + c0, nb, &stage_bar);
                stage_pending = true;
                stage_parity = (uint32_t)(it & 1);
            }
            if (it >= 2 && !rt_wait(&tble_bar[buf], (uint32_t)(((it - 2) >> 1) & 1), &s_abort)) break;
            for (int idx = p; idx < RT_EPT * NPE; idx += RT_NPROD) {
                const int64_t e = el0 + idx / NPE;
                int node = -1, r0 = 0, rl = 0;
                if (e < R.ne) {
                    const uint64_t nd = R.elements[(R.e0 + e) * NPE + idx % NPE];
                    if (nd < (uint64_t)R.nnode) {
                        node = (int)nd;
                        r0 = R.indptr[3 * node];
                        rl = R.indptr[3 * node + 1] - r0;
                    } else {
                        flag |= FL_FLAG_BAD_INDEX;
                    }
                }
                tb.nodes[idx] = node;
                tb.rs0[idx] = r0;
                tb.rlen[idx] = rl;
            }
            for (int idx = p; idx < RT_EPT * NPE * NPE; idx += RT_NPROD) {
                const int64_t e = el0 + idx / (NPE * NPE);
                int v = -1;
                if (e < R.ne) v = R.boff[(R.e0 + e) * (NPE * NPE) + idx % (NPE * NPE)];
                tb.boff[idx] = (int16_t)(v >= 0 && v < 32768 ? v : -1);
            }
            if (bulk) {
                if (!rt_wait(&stage_bar, (uint32_t)(it & 1), &s_abort)) break;
                if (p == 0) stage_pending = false;
            } else {
                for (int idx = p; idx < 108 * TQ; idx += RT_NPROD) {
                    const int row = idx / TQ, c = idx % TQ;
                    AH[idx] = c0 + c < cend ? row_src(row)[c0 + c] : 0.f;
                }
            }
            producers_sync();
            {   // row scales: the largest |hi| of each row over (g, d, e), RT_NPROD / 128 threads per row
                constexpr int TPR = RT_NPROD / RT_M;
                const int r = p / TPR, hf = p % TPR;
                float mx = 0.f;
                if (r < 9 * RT_EPT)
                    for (int de = hf; de < 9; de += TPR) {
                        const float *src = AH + row_off[r][de];
#pragma unroll 2
                        for (int g = 0; g < nq; ++g) mx = fmaxf(mx, fabsf(src[g]));
                    }
                if (TPR == 2) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
                if (hf == 0) {
                    int E;
                    float sc;
                    rt_row_scale(mx, E, sc);
                    tb.rexp[r] = E;
                    rsc[r] = sc;
                }
            }
            producers_sync();  // row scales visible to every producer
            if (lane == 0) mbar_arrive(&tblf_bar[buf]);
            // A planes, chunk by chunk (the same planes for every chunk of the tile)
            const int r = p & (RT_M - 1);  // the row; its 8-column halves of each K step from kg0 by KGS
            const int kg0 = p / RT_M, KGS = RT_NPROD / RT_M;
            const int el = r / 9;
            const bool rowok = r < 9 * RT_EPT && el0 + el < R.ne;
            const float sc = rowok ? rsc[r] : 0.f;
            for (int c = 0; c < NCH && !s_abort; ++c)
                for (int j = 0; j < NKS; ++j, ++gs) {
                    const int s = (int)(gs % RT_NST);
                    const int64_t u = gs / RT_NST;
                    if (u > 0 && !rt_wait(&empty_bar[s], (uint32_t)((u - 1) & 1), &s_abort)) break;
#pragma unroll 1
                    for (int kg = kg0; kg < 2; kg += KGS) {
                    float dg[8][RT_DIG];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int kk = 16 * j + 8 * kg + q;
                        float h = 0.f, l = 0.f;
                        if (rowok && kk < K) {
                            const int src = row_off[r][k_de[kk]] + k_g[kk];
                            h = AH[src];
                            l = AL[src];
                        }
                        rt_digits(h, l, sc, dg[q]);
                    }
                    unsigned char *ab = stages + (size_t)s * RT_STAGE + kmaj16(r, 8 * kg);
#pragma unroll
                    for (int t = 0; t < RT_DIG; ++t) {
                        const uint4 w = make_uint4(pack_bf16(dg[0][t], dg[1][t]), pack_bf16(dg[2][t], dg[3][t]),
                                                   pack_bf16(dg[4][t], dg[5][t]), pack_bf16(dg[6][t], dg[7][t]));
                        *reinterpret_cast<uint4 *>(ab + (size_t)t * RT_A_PLANE) = w;
                    }
                    }
                    tc::fence_async_smem();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&fullA[s]);
                }
        }
        // an aborted run can leave a bulk copy of tile data in flight: wait for it (bounded) before
        // the CTA's shared memory is released
        if (stage_pending) tc::mbar_wait(&stage_bar, stage_parity, RT_WAIT_LIMIT);
    } else if (warp == RT_MMA_WARP) {
        // ---------------------------------------------------------------------------- MMA issue
        if (lane == 0 && total_steps > 0) {
            const uint32_t idesc = tc::idesc_bf16_f32(RT_M, RT_NB);
            const unsigned char *phi = reinterpret_cast<const unsigned char *>(R.phi);
            int64_t issued = 0;  // bulk copies issued
            auto issue_b = [&](int64_t q) {
                const int s = (int)(q % RT_NST);
                const int64_t cq = (q / NKS) % NCH, jq = q % NKS;
                mbar_arrive_tx(&fullB[s], RT_B_BYTES);
                bulk_g2s(stages + (size_t)s * RT_STAGE + RT_A_BYTES, phi + (size_t)(cq * NKS + jq) * RT_B_BYTES,
                         RT_B_BYTES, &fullB[s]);
                issued = q + 1;
            };
            for (int64_t q = 0; q < RT_NST - 1 && q < total_steps; ++q) issue_b(q);
            int64_t cc = 0;
            for (int64_t gs = 0; gs < total_steps; ++gs) {
                const int j = (int)(gs % NKS);
                if (j == 0 && cc > 0 && !rt_wait(&acce_bar, (uint32_t)((cc - 1) & 1), &s_abort)) break;
                const int s = (int)(gs % RT_NST);
                const uint32_t par = (uint32_t)((gs / RT_NST) & 1);
                if (!rt_wait(&fullB[s], par, &s_abort) || !rt_wait(&fullA[s], par, &s_abort)) break;
                tc::fence_after_sync();
                const unsigned char *st = stages + (size_t)s * RT_STAGE;
                bool fresh[RT_NACC];
#pragma unroll
                for (int L = 0; L < RT_NACC; ++L) fresh[L] = (j == 0);
#pragma unroll
                for (int sa = 0; sa < RT_DIG; ++sa)
#pragma unroll
                    for (int sb = 0; sb < RT_DIG - sa; ++sb) {
                        const int L = sa + sb < RT_NACC - 1 ? sa + sb : RT_NACC - 1;
                        const uint64_t da = tc::smem_desc(st + (size_t)sa * RT_A_PLANE, 128, 256);
                        const uint64_t db = tc::smem_desc(st + RT_A_BYTES + (size_t)sb * RT_B_PLANE, 128, 256);
                        tc::mma_bf16(taddr + (uint32_t)(L * RT_ACCSTRIDE), da, db, idesc, !fresh[L]);
                        fresh[L] = false;
                    }
                tc::mma_commit(&empty_bar[s]);
                if (j == NKS - 1) {
                    tc::mma_commit(&accf_bar);
                    ++cc;
                }
                const int64_t q = gs + RT_NST - 1;  // the next Phi stage to fetch: its stage held step gs - 1
                if (q < total_steps) {
                    const int sq = (int)(q % RT_NST);
                    const int64_t uq = q / RT_NST;
                    if (uq > 0 && !rt_wait(&empty_bar[sq], (uint32_t)((uq - 1) & 1), &s_abort)) break;
                    issue_b(q);
                }
            }
            // before the tensor memory is released: every MMA issued has completed, and every bulk
            // copy issued has landed (bounded waits; only an aborted run has copies outstanding)
            tc::mma_commit(&fin_bar);
            tc::mbar_wait(&fin_bar, 0, RT_WAIT_LIMIT);
            for (int64_t q = std::max<int64_t>(0, issued - RT_NST); q < issued; ++q)
                tc::mbar_wait(&fullB[q % RT_NST], (uint32_t)((q / RT_NST) & 1), RT_WAIT_LIMIT);
        }
    } else {
        // ---------------------------------------------------------------------------- epilogue
        // warp w reads tensor-memory lanes 32 (w % 4) .. + 31 (its rows) and the column groups of 8
        // whose index has the parity w / 4
        const int quarter = warp & 3, half = warp >> 2;
        const int r = 32 * quarter + lane;
        const int el = r / 9, i = (r % 9) / 3, k = r % 3;
        const uint32_t trow = taddr + ((uint32_t)(32 * quarter) << 16);
        int64_t cc = 0;
        for (int64_t it = 0; it < mine && !s_abort; ++it) {
            const int64_t tile = blockIdx.x + it * (int64_t)gridDim.x;
            const int buf = (int)(it & 1);
            const RtTables<NPE> &tb = tables[buf];
            if (!rt_wait(&tblf_bar[buf], (uint32_t)((it >> 1) & 1), &s_abort)) break;
            if (R.update) {  // residual t[(a,i)] = sum_g sum_d Jm[d][a][g] S_g[i][d] in float pairs
                for (int idx = tid; idx < RT_EPT * NPE * 3; idx += RT_NEPI) {
                    const int re = idx / (NPE * 3), a = (idx % (NPE * 3)) / 3, ri = idx % 3;
                    const int node = tb.nodes[re * NPE + a];
                    if (tile * RT_EPT + re >= R.ne || node < 0) continue;
                    FloatPair t(0.f, 0.f);
                    for (int g = 0; g < nq; ++g)
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            const float2 j = jms[(d * NPE + a) * nq + g];
                            const int o = (ri * 3 + d) * TQ + re * nq + g;
                            t = fma(FloatPair(j.x, j.y), FloatPair(SH[o], SL[o]), t);
                        }
                    atomicAdd(R.T + 3 * (int64_t)node + ri, to_double(t));
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&rdone_bar);
            const bool rv = r < 9 * RT_EPT && tile * RT_EPT + el < R.ne;
            const int Er = tb.rexp[r];
            bool ok = true;
            for (int c = 0; c < NCH; ++c, ++cc) {
                if (!rt_wait(&accf_bar, (uint32_t)(cc & 1), &s_abort)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
#pragma unroll 1
                for (int cg = half; cg < RT_NB / 8; cg += 2) {
                    uint32_t v[RT_NACC][8];
#pragma unroll
                    for (int L = 0; L < RT_NACC; ++L)
                        tmem_ld8_nowait(trow + (uint32_t)(L * RT_ACCSTRIDE + 8 * cg), v[L]);
                    tmem_wait_ld();
                    if (cg + 2 >= RT_NB / 8) {  // this warp's last columns of the chunk are read
                        tc::fence_before_sync();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&acce_bar);
                    }
                    if (!rv) continue;
                    const int64_t nnz = s_nnz;
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj) {
                        const int n = c * RT_NB + cg * 8 + jj;
                        if (n >= P) continue;
                        const int a = pair_a[n], b = pair_b[n];
                        const int na = tb.nodes[el * NPE + a], nb = tb.nodes[el * NPE + b];
                        if (na < 0 || nb < 0) continue;
                        const double val = rt_combine(__uint_as_float(v[0][jj]), __uint_as_float(v[1][jj]),
                                                      __uint_as_float(v[2][jj]), __uint_as_float(v[3][jj]),
                                                      __uint_as_float(v[4][jj]), Er + colexp[n] - 14);
                        const int o1 = tb.boff[(el * NPE + a) * NPE + b];
                        int64_t pos = o1 >= 0 ? (int64_t)tb.rs0[el * NPE + a] + i * tb.rlen[el * NPE + a] + o1 + k
                                              : rt_search(R.indptr, R.indices, na, i, nb, k);
                        if (pos >= 0 && pos < nnz) atomicAdd(R.V + pos, val);
                        else flag |= FL_FLAG_BAD_INDEX;
                        if (a != b) {
                            const int o2 = tb.boff[(el * NPE + b) * NPE + a];
                            pos = o2 >= 0 ? (int64_t)tb.rs0[el * NPE + b] + k * tb.rlen[el * NPE + b] + o2 + i
                                          : rt_search(R.indptr, R.indices, nb, k, na, i);
                            if (pos >= 0 && pos < nnz) atomicAdd(R.V + pos, val);
                            else flag |= FL_FLAG_BAD_INDEX;
                        }
                    }
                }
            }
            if (!ok) break;
            __syncwarp();
            if (lane == 0) mbar_arrive(&tble_bar[buf]);
        }
    }

    if (flag) atomicOr(&s_flag, flag);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && (s_flag || s_abort) && R.flags) atomicOr(R.flags, s_flag | (s_abort ? FL_FLAG_TIMEOUT : 0));
    if (warp == RT_MMA_WARP) tc::tmem_dealloc(taddr, RT_TMEM_COLS);
}

// Phi digit planes: one block per pair column n (all NCH * 80, padding columns zero), FP64
// products Jm[d][a][g] Jm[e][b][g], scaled by 2^(7 - F), F the column's exponent, and split into six
// planes q_t (multiples of 2^-8t, at most 128 * 2^-8t in magnitude); stored per (chunk, K step) as
// six 80 x 16 K-major planes, the layout one bulk copy moves into a stage.
__global__ void rt_phi_kernel(const double *Jm, int npe, int nq, __nv_bfloat16 *phi, int *phiexp) {
    const int n = blockIdx.x, P = rt_pairs(npe), K = 9 * nq, NKS = rt_ksteps(nq);
    __shared__ double s_max[256];
    int a = 0, b = 0;
    if (n < P) rt_pair(n, a, b);
    auto val = [&](int kk) -> double {
        if (n >= P || kk >= K) return 0.0;
        const int g = kk / 9, d = (kk % 9) / 3, e = kk % 3;
        return Jm[((size_t)d * npe + a) * nq + g] * Jm[((size_t)e * npe + b) * nq + g];
    };
    double mx = 0.0;
    for (int kk = threadIdx.x; kk < K; kk += blockDim.x) mx = fmax(mx, fabs(val(kk)));
    s_max[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + w]);
        __syncthreads();
    }
    int F = 0;
    if (s_max[0] > 0.0) frexp(s_max[0], &F);  // s_max < 2^F
    if (threadIdx.x == 0) phiexp[n] = F;
    const int c = n / RT_NB, nl = n % RT_NB;
    for (int kk = threadIdx.x; kk < NKS * 16; kk += blockDim.x) {
        float q[RT_DIG];
        rt_digits_f64(ldexp(val(kk), 7 - F), q);
        unsigned char *base = reinterpret_cast<unsigned char *>(phi) + (size_t)(c * NKS + kk / 16) * RT_B_BYTES;
        for (int t = 0; t < RT_DIG; ++t)
            *reinterpret_cast<__nv_bfloat16 *>(base + (size_t)t * RT_B_PLANE + kmaj16(nl, kk % 16)) =
                __float2bfloat16_rn(q[t]);
    }
}

// Block offsets: for element e and nodes (a, b), the offset of column 3 node_b in row 3 node_a
// when the node block is where a node-blocked CSR puts it (the three rows of a node of equal
// length and consecutive, the block's nine entries at row start + i length + offset + k), else -1
// (the contraction then searches each entry's row).
__global__ void rt_boff_kernel(const uint64_t *elements, int64_t nelem, int npe, int64_t nnode,
                               const int32_t *indptr, const int32_t *indices, int32_t *out, int *flags) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)npe * npe;
    if (t >= nelem * per) return;
    const int64_t e = t / per;
    const int a = (int)((t % per) / npe), b = (int)(t % npe);
    const uint64_t na = elements[e * npe + a], nb = elements[e * npe + b];
    if (na >= (uint64_t)nnode || nb >= (uint64_t)nnode) {
        out[t] = -1;
        if (flags) atomicOr(flags, FL_FLAG_BAD_INDEX);
        return;
    }
    const int row = 3 * (int)na, col = 3 * (int)nb;
    const int r0 = indptr[row], len = indptr[row + 1] - r0;
    int lo = r0, hi = r0 + len;
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (col < indices[mid]) hi = mid; else lo = mid;
    }
    int off = (len > 0 && indices[lo] == col) ? lo - r0 : -1;
    for (int i = 0; i < 3 && off >= 0; ++i) {
        if (indptr[row + i] != r0 + i * len || indptr[row + i + 1] - indptr[row + i] != len || off + 2 >= len) {
            off = -1;
            break;
        }
        for (int k = 0; k < 3; ++k)
            if (indices[r0 + i * len + off + k] != col + k) off = -1;
    }
    out[t] = off;
}

template <int NPE>
static int rt_launch_t(const RtArgs &R, cudaStream_t stream) {
    const size_t smem = rt_smem_bytes<NPE>(R.nq);
    { const int st = ensure_smem<rt_contract_kernel<NPE>>(smem); if (st != FL_OK) return st; }
    int dev = 0, sms = 0;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    FL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t ntiles = (R.ne + RT_EPT - 1) / RT_EPT;
    const int64_t grid = std::min<int64_t>(ntiles, sms);
    if (grid <= 0) return FL_OK;
    rt_contract_kernel<NPE><<<(unsigned)grid, RT_THREADS, smem, stream>>>(R);
    return launch_status();
}

bool rt_supported(int npe, int nq) {
    if (nq < 1 || nq > RT_MAX_NQ) return false;
    switch (npe) {
        case 4: case 8: case 10: case 20: return true;
        default: return false;
    }
}

size_t rt_phi_bytes(int npe, int nq) {
    const size_t planes = (size_t)rt_chunks(npe) * rt_ksteps(nq) * RT_B_BYTES;
    return (planes + 255) / 256 * 256 + ((size_t)rt_chunks(npe) * RT_NB * sizeof(int) + 255) / 256 * 256;
}

const int *rt_phi_exponents(const void *buf, int npe, int nq) {
    const size_t planes = (size_t)rt_chunks(npe) * rt_ksteps(nq) * RT_B_BYTES;
    return reinterpret_cast<const int *>(reinterpret_cast<const unsigned char *>(buf) + (planes + 255) / 256 * 256);
}

int rt_build_phi(const double *Jm, int npe, int nq, void *buf, cudaStream_t stream) {
    if (!rt_supported(npe, nq)) return FL_ERR_UNSUPPORTED;
    rt_phi_kernel<<<(unsigned)(rt_chunks(npe) * RT_NB), 128, 0, stream>>>(
        Jm, npe, nq, reinterpret_cast<__nv_bfloat16 *>(buf), const_cast<int *>(rt_phi_exponents(buf, npe, nq)));
    return launch_status();
}

int rt_block_offsets(const uint64_t *elements, int64_t nelem, int npe, int64_t nnode, const int32_t *indptr,
                     const int32_t *indices, int32_t *out, int *flags, cudaStream_t stream) {
    const int64_t n = nelem * (int64_t)npe * npe;
    if (n == 0) return FL_OK;
    rt_boff_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(elements, nelem, npe, nnode, indptr, indices, out,
                                                                     flags);
    return launch_status();
}

int rt_contract(const RtArgs &R, int npe, cudaStream_t stream) {
    if (!rt_supported(npe, R.nq)) return FL_ERR_UNSUPPORTED;
    switch (npe) {
        case 4: return rt_launch_t<4>(R, stream);
        case 8: return rt_launch_t<8>(R, stream);
        case 10: return rt_launch_t<10>(R, stream);
        case 20: return rt_launch_t<20>(R, stream);
        default: return FL_ERR_UNSUPPORTED;
    }
}

}  // namespace fl

extern "C" int fl_ElementBlockOffsets(const uint64_t *elements, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                                      const int32_t *indptr, const int32_t *indices, int32_t *block_offsets,
                                      int *flags, fl_stream_t stream) {
    if (nelem < 0 || nodeperelem <= 0 || nodeperelem > 181 || nnode <= 0) return FL_ERR_ARG;
    if (3 * nnode + 2 > INT32_MAX) return FL_ERR_UNSUPPORTED;
    if (nelem == 0) return FL_OK;
    if (!elements || !indptr || !indices || !block_offsets) return FL_ERR_ARG;
    return fl::rt_block_offsets(elements, nelem, (int)nodeperelem, nnode, indptr, indices, block_offsets, flags,
                                (cudaStream_t)stream);
}
