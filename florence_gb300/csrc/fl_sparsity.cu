// fl_sparsity.cu -- device construction of the global CSR pattern and of the reference's
// element-to-nonzero maps, bit-identical to ComputeSparsityPattern
// (Florence/FiniteElements/Assembly/_Assembly_/ComputeSparsityPattern.pyx:44-112 and
//  ComputeSparsityPattern.h:22-125):
//   - row nvar*n+j of node n lists, for every node m adjacent to n (sharing an element, n itself
//     included) in increasing order, the columns nvar*m+0 .. nvar*m+nvar-1;
//   - data_global_indices[e*cap + i*ndof + j] is the CSR position of (row rc[i], column rc[j]) and
//     data_local_indices[e*cap + i*ndof + j] = rcl[i]*ndof + rcl[j], where rc/rcl enumerate the
//     element's dofs in increasing node order (rc = global dof, rcl = local dof).
// Steps: node incidence counts -> scan -> incidence lists; per node a CTA gathers the nodes of
// its elements into shared memory, bitonic-sorts them and counts/writes the distinct ones; a
// scan of the per-node counts gives indptr; per element a CTA ranks its nodes and binary-searches
// each dof pair in its row.
#include <algorithm>

#include "fl_common.cuh"
#include "fl_scan.cuh"

namespace fl {

constexpr int SP_MAX_CAND = 16384;  // candidate neighbour entries per node held in shared memory

struct SpWork {
    int32_t *cnt;     // [nnode+1] incidence counts, then exclusive scan (starts)
    int32_t *cursor;  // [nnode]
    int32_t *list;    // [nelem*npe] incident elements per node
    int64_t *nbr;     // [nnode+1] distinct neighbours per node, then exclusive scan
    int64_t *bsum;    // [scan block sums]
    int32_t *info;    // [4]: error bits, max incidence degree
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t sp_layout(int64_t nelem, int64_t npe, int64_t nnode, SpWork *w, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    const int64_t nb = (nnode + 1 + SCAN_ITEMS - 1) / SCAN_ITEMS + 1;
    SpWork t;
    t.cnt = (int32_t *)take(sizeof(int32_t) * (nnode + 1));
    t.cursor = (int32_t *)take(sizeof(int32_t) * nnode);
    t.list = (int32_t *)take(sizeof(int32_t) * nelem * npe);
    t.nbr = (int64_t *)take(sizeof(int64_t) * (nnode + 1));
    t.bsum = (int64_t *)take(sizeof(int64_t) * (nb + SCAN_ITEMS));
    t.info = (int32_t *)take(sizeof(int32_t) * 4);
    if (w) *w = t;
    return off;
}

__global__ void sp_count(const int64_t *el, int64_t n, int64_t nnode, int32_t *cnt, int32_t *info) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t nd = el[k];
        if (nd < 0 || nd >= nnode) atomicOr(info, 1);
        else atomicAdd(cnt + nd, 1);
    }
}

// node starts, zero-degree check, maximum degree (cnt already scanned into starts; degrees are
// the differences)
__global__ void sp_degree_check(const int32_t *start, int64_t nnode, int32_t *info) {
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nnode; n += (int64_t)gridDim.x * blockDim.x) {
        const int deg = start[n + 1] - start[n];
        if (deg == 0) atomicOr(info, 2);
        atomicMax(info + 1, deg);
    }
}

__global__ void sp_fill_lists(const int64_t *el, int64_t n, int64_t npe, const int32_t *start, int32_t *cursor,
                              int32_t *list) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t nd = el[k];
        const int pos = atomicAdd(cursor + nd, 1);
        list[start[nd] + pos] = (int32_t)(k / npe);
    }
}

constexpr int SP_NT = 128;

// CTA per node: the nodes of its elements are bitonic-sorted in shared memory (a power-of-two
// buffer sized for this node's own candidate count), first occurrences are flagged, and a block
// scan of per-thread segment counts gives every distinct neighbour its rank. Returns the number
// of distinct neighbours; if out != nullptr, writes the sorted distinct neighbours to out[rank].
__device__ int node_neighbours(const int64_t *el, int64_t npe, const int32_t *start, const int32_t *list, int64_t n,
                               int32_t *buf, int32_t *out) {
    __shared__ int warp_tot[SP_NT / 32];
    const int s0 = start[n], deg = start[n + 1] - s0;
    const int m = deg * (int)npe;
    int capc = 32;
    while (capc < m) capc <<= 1;
    for (int i = threadIdx.x; i < capc; i += SP_NT) {
        if (i < m) buf[i] = (int32_t)el[(int64_t)list[s0 + i / (int)npe] * npe + i % (int)npe];
        else buf[i] = INT32_MAX;
    }
    __syncthreads();
    for (int k = 2; k <= capc; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < capc; i += SP_NT) {
                const int p = i ^ j;
                if (p > i) {
                    const int32_t a = buf[i], b = buf[p];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        buf[i] = b;
                        buf[p] = a;
                    }
                }
            }
            __syncthreads();
        }
    // contiguous segment per thread; first occurrences among the m real keys
    const int per = (m + SP_NT - 1) / SP_NT;
    const int lo = threadIdx.x * per, hi = min(m, lo + per);
    int c = 0;
    for (int i = lo; i < hi; ++i) c += (i == 0 || buf[i] != buf[i - 1]);
    // block exclusive scan of c
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    int base = 0, total = 0;
    for (int w = 0; w < SP_NT / 32; ++w) {
        if (w < wid) base += warp_tot[w];
        total += warp_tot[w];
    }
    if (out) {
        int r = base + incl - c;
        for (int i = lo; i < hi; ++i)
            if (i == 0 || buf[i] != buf[i - 1]) out[r++] = buf[i];
    }
    __syncthreads();  // buf and warp_tot are reused by the caller's next node
    return total;
}

__global__ void __launch_bounds__(SP_NT) sp_count_neighbours(const int64_t *el, int64_t npe, const int32_t *start,
                                                             const int32_t *list, int64_t *nbr) {
    extern __shared__ int32_t sbuf[];
    const int64_t n = blockIdx.x;
    const int count = node_neighbours(el, npe, start, list, n, sbuf, nullptr);
    if (threadIdx.x == 0) nbr[n] = count;
}

__global__ void __launch_bounds__(SP_NT) sp_write_rows(const int64_t *el, int64_t npe, const int32_t *start,
                                                       const int32_t *list, int capc, const int64_t *off, int64_t nvar,
                                                       int32_t *indptr, int32_t *indices) {
    extern __shared__ int32_t sbuf[];
    int32_t *buf = sbuf, *uniq = sbuf + capc;
    const int64_t n = blockIdx.x;
    const int cnt = node_neighbours(el, npe, start, list, n, buf, uniq);
    __syncthreads();
    const int64_t base = off[n] * nvar * nvar;
    const int64_t rowlen = (int64_t)cnt * nvar;
    // row nvar*n+j: columns nvar*uniq[k]+l in order (k-major, then l)
    for (int64_t t = threadIdx.x; t < nvar * rowlen; t += SP_NT) {
        const int64_t j = t / rowlen, r = t % rowlen, k = r / nvar, l = r % nvar;
        indices[base + j * rowlen + r] = (int32_t)(nvar * uniq[k] + l);
    }
    if (threadIdx.x < nvar) indptr[n * nvar + threadIdx.x] = (int32_t)(base + threadIdx.x * rowlen);
}

__global__ void sp_last_indptr(int32_t *indptr, int64_t nrows, const int64_t *off, int64_t nnode, int64_t nvar) {
    indptr[nrows] = (int32_t)(off[nnode] * nvar * nvar);
}

// data maps: CTA per element
__global__ void sp_data_maps(const int64_t *el, int64_t npe, int64_t nvar, const int32_t *indptr, const int32_t *indices,
                             int32_t *dl, int32_t *dg) {
    extern __shared__ int32_t sm[];
    const int NPE = (int)npe, NDOF = (int)(npe * nvar);
    int32_t *nodes = sm, *sorter = sm + NPE, *rc = sm + 2 * NPE, *rcl = rc + NDOF;
    const int64_t e = blockIdx.x;
    for (int k = threadIdx.x; k < NPE; k += blockDim.x) nodes[k] = (int32_t)el[e * npe + k];
    __syncthreads();
    for (int k = threadIdx.x; k < NPE; k += blockDim.x) {
        int r = 0;  // rank of node k (ties broken by position, like a stable argsort)
        for (int m = 0; m < NPE; ++m) r += (nodes[m] < nodes[k]) || (nodes[m] == nodes[k] && m < k);
        sorter[r] = k;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NDOF; i += blockDim.x) {
        const int s = sorter[i / (int)nvar], c = i % (int)nvar;
        rc[i] = (int32_t)(nvar * nodes[s] + c);
        rcl[i] = (int32_t)(s * nvar + c);
    }
    __syncthreads();
    const int64_t cap = (int64_t)NDOF * NDOF;
    for (int64_t idx = threadIdx.x; idx < cap; idx += blockDim.x) {
        const int i = (int)(idx / NDOF), j = (int)(idx % NDOF);
        const int row = rc[i], col = rc[j];
        int lo = indptr[row], hi = indptr[row + 1];
        while (hi - lo > 1) {
            const int mid = lo + (hi - lo) / 2;
            if (col < indices[mid]) hi = mid; else lo = mid;
        }
        dg[e * cap + idx] = lo;
        dl[e * cap + idx] = rcl[i] * NDOF + rcl[j];
    }
}

static int compute_sparsity(const int64_t *elements, int64_t nelem, int64_t npe, int64_t nnode, int64_t nvar,
                            int32_t *indptr, int32_t *indices, int64_t cap_indices, int64_t *nnz_out, int32_t *dl,
                            int32_t *dg, void *workspace, size_t ws_bytes, cudaStream_t s) {
    if (!elements || !indptr || !nnz_out || !workspace || nelem <= 0 || npe <= 0 || nnode <= 0 || nvar <= 0)
        return FL_ERR_ARG;
    if ((dl == nullptr) != (dg == nullptr)) return FL_ERR_ARG;
    if (nnode * nvar + 1 > INT32_MAX) return FL_ERR_UNSUPPORTED;
    SpWork w;
    if (sp_layout(nelem, npe, nnode, nullptr, nullptr) > ws_bytes) return FL_ERR_CAPACITY;
    sp_layout(nelem, npe, nnode, &w, (char *)workspace);
    const int64_t n = nelem * npe;
    FL_CUDA_TRY(cudaMemsetAsync(w.cnt, 0, sizeof(int32_t) * (nnode + 1), s));
    FL_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, sizeof(int32_t) * nnode, s));
    FL_CUDA_TRY(cudaMemsetAsync(w.info, 0, sizeof(int32_t) * 4, s));
    const unsigned g1 = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
    sp_count<<<g1, 256, 0, s>>>(elements, n, nnode, w.cnt, w.info);
    int32_t hinfo[4];
    FL_CUDA_TRY(cudaMemcpyAsync(hinfo, w.info, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    if (hinfo[0] & 1) return FL_ERR_ARG;  // node id out of range
    exclusive_scan<int32_t, int32_t>(w.cnt, w.cnt, nnode + 1, w.bsum, s);
    const unsigned g2 = (unsigned)std::min<int64_t>((nnode + 255) / 256, 152 * 16);
    sp_degree_check<<<g2, 256, 0, s>>>(w.cnt, nnode, w.info);
    FL_CUDA_TRY(cudaMemcpyAsync(hinfo, w.info, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    if (hinfo[0] & 2) return FL_ERR_MESH;
    const int64_t maxcand = (int64_t)hinfo[1] * npe;
    if (maxcand > SP_MAX_CAND) return FL_ERR_UNSUPPORTED;
    int capc = 32;
    while (capc < maxcand) capc <<= 1;
    sp_fill_lists<<<g1, 256, 0, s>>>(elements, n, npe, w.cnt, w.cursor, w.list);
    const size_t shm = sizeof(int32_t) * 2 * capc;  // sort buffer + distinct neighbours
    if (shm > 48 * 1024) {
        FL_CUDA_TRY(cudaFuncSetAttribute(sp_count_neighbours, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        FL_CUDA_TRY(cudaFuncSetAttribute(sp_write_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    }
    sp_count_neighbours<<<(unsigned)nnode, SP_NT, shm, s>>>(elements, npe, w.cnt, w.list, w.nbr);
    FL_CUDA_TRY(cudaMemsetAsync(w.nbr + nnode, 0, sizeof(int64_t), s));
    exclusive_scan<int64_t, int64_t>(w.nbr, w.nbr, nnode + 1, w.bsum, s);
    int64_t total_nodes_pairs = 0;
    FL_CUDA_TRY(cudaMemcpyAsync(&total_nodes_pairs, w.nbr + nnode, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    const int64_t nnz = total_nodes_pairs * nvar * nvar;
    *nnz_out = nnz;
    if (nnz > INT32_MAX) return FL_ERR_UNSUPPORTED;
    if (!indices || cap_indices < nnz) return FL_ERR_CAPACITY;
    sp_write_rows<<<(unsigned)nnode, SP_NT, shm, s>>>(elements, npe, w.cnt, w.list, capc, w.nbr, nvar, indptr, indices);
    sp_last_indptr<<<1, 1, 0, s>>>(indptr, nnode * nvar, w.nbr, nnode, nvar);
    if (dl) {
        const int ndof = (int)(npe * nvar);
        const size_t shm2 = sizeof(int32_t) * (2 * npe + 2 * ndof);
        sp_data_maps<<<(unsigned)nelem, 256, shm2, s>>>(elements, npe, nvar, indptr, indices, dl, dg);
    }
    return launch_status();
}

}  // namespace fl

extern "C" {

size_t fl_ComputeSparsityPattern_workspace_size(int64_t nelem, int64_t nodeperelem, int64_t nnode) {
    return fl::sp_layout(nelem, nodeperelem, nnode, nullptr, nullptr);
}

int fl_ComputeSparsityPattern(const int64_t *elements, int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t nvar,
                              int32_t *indptr, int32_t *indices, int64_t indices_capacity, int64_t *nnz,
                              int32_t *data_local_indices, int32_t *data_global_indices, void *workspace,
                              size_t workspace_bytes, fl_stream_t stream) {
    return fl::compute_sparsity(elements, nelem, nodeperelem, nnode, nvar, indptr, indices, indices_capacity, nnz,
                                data_local_indices, data_global_indices, workspace, workspace_bytes,
                                (cudaStream_t)stream);
}

}  // extern "C"
