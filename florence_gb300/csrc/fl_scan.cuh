// fl_scan.cuh -- device exclusive prefix sum over int32/int64 counts (three kernels: per-block
// totals, a one-CTA scan of the totals, a per-block scan that adds the block's offset), used by
// the sparsity-pattern and mesh-generation passes. `bsum` needs ceil(n / SCAN_ITEMS) int64 slots.
#pragma once
#include <cstdint>

namespace fl {
namespace {

constexpr int SCAN_ITEMS = 2048, SCAN_THREADS = 512;

template <class T>
__global__ void scan_totals(const T *in, int64_t n, int64_t *bsum) {
    __shared__ int64_t red[SCAN_THREADS];
    const int64_t base = (int64_t)blockIdx.x * SCAN_ITEMS;
    int64_t s = 0;
    for (int i = threadIdx.x; i < SCAN_ITEMS; i += SCAN_THREADS)
        if (base + i < n) s += (int64_t)in[base + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = SCAN_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = red[0];
}

__global__ void scan_block_sums(int64_t *bsum, int64_t nb) {
    // single CTA: exclusive scan of nb block totals, chunk by chunk
    __shared__ int64_t buf[SCAN_THREADS];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t c0 = 0; c0 < nb; c0 += SCAN_THREADS) {
        const int64_t i = c0 + threadIdx.x;
        const int64_t v = i < nb ? bsum[i] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < SCAN_THREADS; o <<= 1) {
            int64_t t = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == SCAN_THREADS - 1) carry += buf[threadIdx.x];
        __syncthreads();
    }
}

template <class TIN, class TOUT>
__global__ void scan_apply(const TIN *in, TOUT *out, int64_t n, const int64_t *bsum) {
    // each thread scans SCAN_ITEMS/SCAN_THREADS consecutive items
    constexpr int PER = SCAN_ITEMS / SCAN_THREADS;
    __shared__ int64_t buf[SCAN_THREADS];
    const int64_t base = (int64_t)blockIdx.x * SCAN_ITEMS + (int64_t)threadIdx.x * PER;
    int64_t v[PER], s = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        v[k] = base + k < n ? (int64_t)in[base + k] : 0;
        s += v[k];
    }
    buf[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < SCAN_THREADS; o <<= 1) {
        int64_t t = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
        __syncthreads();
        buf[threadIdx.x] += t;
        __syncthreads();
    }
    int64_t run = bsum[blockIdx.x] + buf[threadIdx.x] - s;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        if (base + k < n) out[base + k] = (TOUT)run;
        run += v[k];
    }
}

template <class TIN, class TOUT>
void exclusive_scan(const TIN *in, TOUT *out, int64_t n, int64_t *bsum, cudaStream_t s) {
    const int64_t nb = (n + SCAN_ITEMS - 1) / SCAN_ITEMS;
    scan_totals<TIN><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, bsum);
    scan_block_sums<<<1, SCAN_THREADS, 0, s>>>(bsum, nb);
    scan_apply<TIN, TOUT><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, bsum);
}

}  // namespace
}  // namespace fl
