// fl_reftensor.cuh -- the FP64 tangent as one tensor-core GEMM per tile of elements against the
// element-independent reference tensor (fl_reftensor.cu). Shared between the assembly driver
// (fl_assembly.cu) and the kernel's translation unit.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace fl {

// One chunk of elements whose Gauss-point data the Gauss-point kernel wrote as float pairs: the
// residual factor S (hi [9][ldq] then lo [9][ldq]) and the pulled-back tangent hi [45][ldq], lo
// [45][ldq], column (e - e0) * nq + g for element e of the chunk and Gauss point g; ldq a multiple of
// 4 and every array 16-byte aligned (the contraction stages them with 16-byte loads).
struct RtArgs {
    const float *Qh, *Ql;
    const float *Sp;
    int64_t ldq;
    int64_t e0, ne;            // the chunk: mesh elements [e0, e0 + ne)
    int nq, update;            // update: form the residual (requires_geometry_update)
    const uint64_t *elements;  // [nelem][npe]
    int64_t nnode;
    const int32_t *indptr, *indices;  // the CSR pattern (its size indptr[3 nnode] bounds the scatter)
    const int32_t *boff;       // [nelem][npe][npe] column offset of node b's block in node a's rows, -1: search
    const float2 *jmp;         // Jm as float pairs [3][npe][nq] (residual)
    const void *phi;           // digit planes of the reference tensor (rt_build_phi)
    const int *phiexp;         // per pair column: F with max |phi| < 2^F
    double *V, *T;
    int *flags;
};

bool rt_supported(int npe, int nq);                      // element types / Gauss-point counts the kernel takes
size_t rt_phi_bytes(int npe, int nq);                    // digit planes + exponents, 256-byte aligned
int rt_build_phi(const double *Jm, int npe, int nq, void *buf, cudaStream_t s);  // fills rt_phi_bytes at buf
const int *rt_phi_exponents(const void *buf, int npe, int nq);                   // the exponents inside buf
int rt_block_offsets(const uint64_t *elements, int64_t nelem, int npe, int64_t nnode, const int32_t *indptr,
                     const int32_t *indices, int32_t *out, int *flags, cudaStream_t s);
int rt_contract(const RtArgs &R, int npe, cudaStream_t s);

}  // namespace fl
