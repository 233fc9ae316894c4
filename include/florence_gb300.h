/*
 * florence_gb300.h -- C ABI of the GB300 (sm_103a) displacement-formulation assembly engine.
 *
 * Every pointer argument named like an array is a DEVICE pointer (memory of the current CUDA
 * device) unless its comment says "host". Sizes are element counts. Every entry point is
 * asynchronous on `stream` unless its comment says it synchronises, and returns an int status
 * (FL_OK == 0). Outputs that the reference accumulates into (V, T, M) are accumulated (+=) here
 * too: the caller zero-initialises them, as the reference's Cython wrappers do.
 *
 * The entry points replace these reference interfaces (paths inside the Florence repository):
 *   fl_ComputeSparsityPattern          FiniteElements/Assembly/_Assembly_/ComputeSparsityPattern.pyx:44-112
 *                                      (+ _ComputeSparsityPattern_ / _ComputeDataIndices_, ComputeSparsityPattern.h:22-125)
 *   fl_GlobalAssemblyDF__NeoHookean_   _GlobalAssemblyDF_ monomorphised for _NeoHookean_ by AOT_Assembler.py:36-118,
 *   fl_GlobalAssemblyDF__MooneyRivlin_ FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDF_.h:8-47 (signature),
 *                                      called from _LowLevelAssemblyDF_.pyx:115-154
 *   fl_GlobalAssemblyExplicit_DF_DPF_  FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyExplicit_DF_DPF_.h:728-829
 *                                      (signature), called from _LowLevelAssemblyExplicit_DF_DPF_.pyx:123-152
 *   fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_, _106_, _105_, _101_, _0_, fl_GlobalAssemblyDPF__SteinmannModel_,
 *   fl_GlobalAssemblyDPF__Piezoelectric_100_
 *                                      FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDPF_.h:8-198 (signature),
 *                                      called from _LowLevelAssemblyDPF_.pyx:53-160
 *   fl_LumpedMass, fl_ConsistentMass   VariationalPrinciple/_Mass_/_MassIntegrand_.h:249-400 (mass_type 0 / 1),
 *                                      called from _MassIntegrand_.pyx:192-348 (__TotalConstantMassIntegrand__)
 *   fl_RaiseTetOrder                   the tet branch of Mesh.GetHighOrderMesh (MeshGeneration/Mesh.py:1339-1410),
 *                                      HighOrderMeshTet_SEMISTABLE (HigherOrderMeshing/HigherOrderMeshingTet.py:19-135)
 */
#ifndef FLORENCE_GB300_H
#define FLORENCE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without pulling in the CUDA headers (identical type) */
typedef struct CUstream_st *fl_stream_t;

/* status codes */
#define FL_OK 0
#define FL_ERR_ARG 1           /* invalid argument (null pointer, unsupported ndim/nvar, bad size) */
#define FL_ERR_UNSUPPORTED 2   /* valid but not built: nodes per element, Gauss points or material */
#define FL_ERR_CUDA 3          /* a CUDA runtime call or kernel launch failed */
#define FL_ERR_MESH 4          /* mesh rejected: a node belongs to no element (the reference fails too) */
#define FL_ERR_CAPACITY 5      /* an output or workspace buffer is smaller than required */

/* bits OR-ed into the optional device word `flags` by the assembly kernels */
#define FL_FLAG_NONPOSITIVE_J 1 /* det F <= 0 at some Gauss point; results are still written */
#define FL_FLAG_BAD_INDEX 2     /* an element node id or a map entry is out of range; the entry was skipped */
#define FL_FLAG_TIMEOUT 4       /* a bounded wait inside a tensor-core kernel gave up; outputs incomplete */
#define FL_FLAG_CAPACITY 16     /* fl_CoarsePCG: a CTA's share of the rows does not fit its shared memory;
                                 * nothing was solved */
#define FL_FLAG_PAIR_RANGE 8    /* a Gauss point's pulled-back tangent (or, with FL_ARITH_REFERENCE_TENSOR,
                                 * its stress factor) has its largest magnitude outside [2^-78, 2^120]:
                                 * the float pairs these arithmetics hold it in (FP32 exponent range) may
                                 * have lost digits. The values are written; assemble again with
                                 * FL_ARITH_FP64 (the Python drop-ins do this by themselves) */

/* material numbers of the explicit entry point (_LowLevelAssemblyExplicit_DF_DPF_.pyx:72-109) */
#define FL_MATERIAL_NEOHOOKEAN 1
#define FL_MATERIAL_MOONEYRIVLIN 2
#define FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN 3
#define FL_MATERIAL_LINEARELASTIC 10
/* the transversely isotropic Mooney-Rivlin law (implicit entry points only; the reference's
 * explicit dispatcher has no number for it) */
#define FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1 11

const char *fl_status_string(int status);

/* ------------------------------------------------------------------------------------------
 * Sparsity pattern of the global tangent: node adjacency expanded by nvar x nvar blocks, rows
 * sorted, plus the reference's element-to-nonzero maps. Bit-identical to the reference.
 *   elements        [nelem * nodeperelem] node ids (int64)
 *   indptr          out [nnode*nvar + 1]
 *   indices         out [indices_capacity]; the pattern needs nnz entries
 *   nnz             host out: number of nonzeros
 *   data_local_indices, data_global_indices
 *                   out [nelem * (nvar*nodeperelem)^2] or both NULL (the reference's squeeze mode)
 *   workspace       device scratch of fl_ComputeSparsityPattern_workspace_size() bytes
 * Synchronises `stream` once (to read nnz). Returns FL_ERR_CAPACITY with *nnz set when
 * indices_capacity < nnz (call again with a larger buffer).
 * ------------------------------------------------------------------------------------------ */
size_t fl_ComputeSparsityPattern_workspace_size(int64_t nelem, int64_t nodeperelem, int64_t nnode);
int fl_ComputeSparsityPattern(const int64_t *elements, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                              int64_t nvar, int32_t *indptr, int32_t *indices, int64_t indices_capacity,
                              int64_t *nnz, int32_t *data_local_indices, int32_t *data_global_indices,
                              void *workspace, size_t workspace_bytes, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * High-order tet mesh from a linear one (the tet branch of GetHighOrderMesh). `pattern` (HOST,
 * [nodeperelem * 4]) holds the barycentric coordinates of the high-order element's local nodes
 * with respect to its four vertices, e.g. the reference element's node layout. A local node
 * belongs to the vertices whose weight exceeds 1e-10 (a vertex, an edge, a face or the
 * interior); nodes of shared edges and faces are merged when their weights, read in increasing
 * global-vertex order and rounded to 1e-6, agree. Output: the same mesh as the reference's up to
 * a permutation of node numbers; the numbering is the lexicographic order of (entity size,
 * global vertex ids ascending, weights in that order): used vertices first (in id order), then
 * edge, face and interior nodes. Positions are the weighted sums of the vertex coordinates.
 *   points          [nvert * 3] linear vertices
 *   elements        [nelem * 4] linear tets (int64 vertex ids)
 *   out_points      out [points_capacity * 3]
 *   nnode           host out: number of nodes of the high-order mesh
 *   out_elements    out [nelem * nodeperelem] (int64 node ids)
 *   workspace       device scratch of fl_RaiseTetOrder_workspace_size() bytes (about 96 B per
 *                   element + 40 B per vertex)
 * Synchronises `stream` twice. Returns FL_ERR_CAPACITY with *nnode set when
 * points_capacity < nnode (or out_points is NULL): call again with a larger buffer.
 * FL_ERR_ARG for a vertex id out of range, FL_ERR_MESH for an element that repeats a vertex,
 * FL_ERR_UNSUPPORTED for a layout whose shared nodes cannot be matched from both sides (weights
 * not symmetric under the permutations of an edge's or face's vertices) or nodeperelem > 35.
 * fl_TetNodeLayout (host only, no CUDA call) classifies a pattern the same way and returns
 * counts[0..2] = nodes inside one edge, inside one face, inside the element.
 * ------------------------------------------------------------------------------------------ */
int fl_TetNodeLayout(const double *pattern, int64_t nodeperelem, int64_t *counts);
size_t fl_RaiseTetOrder_workspace_size(int64_t nelem, int64_t nvert);
int fl_RaiseTetOrder(const double *points, int64_t nvert, const int64_t *elements, int64_t nelem,
                     const double *pattern, int64_t nodeperelem, double *out_points, int64_t points_capacity,
                     int64_t *nnode, int64_t *out_elements, void *workspace, size_t workspace_bytes,
                     fl_stream_t stream);
/* fl_RaiseHexOrder: the hex branch of Mesh.GetHighOrderMesh (MeshGeneration/Mesh.py:1388-1389 ->
 * HigherOrderMeshing/HigherOrderMeshingHex.py:19-135, HighOrderMeshHex) on the device, with the
 * same arguments and behaviour as fl_RaiseTetOrder except:
 *   elements        [nelem * 8] linear hexes (int64 vertex ids, the reference's hex vertex order)
 *   pattern         [nodeperelem * 3] reference coordinates in [-1, 1]^3 of the high-order
 *                   element's local nodes, its first 8 nodes the vertices in the order of the
 *                   linear element's columns (the reference's node arrangement); a node's weights
 *                   are the trilinear shape functions of the 8 vertices at it
 *   workspace       fl_RaiseHexOrder_workspace_size() bytes (about 180 B per element + 40 B per
 *                   vertex)
 * FL_ERR_UNSUPPORTED for a layout that is not vertex / edge / face / interior nodes symmetric
 * under the edge swaps and the square's symmetries, or nodeperelem > 125 (p = 4).
 * fl_HexNodeLayout (host only) classifies a pattern the same way (counts as fl_TetNodeLayout). */
int fl_HexNodeLayout(const double *pattern, int64_t nodeperelem, int64_t *counts);
size_t fl_RaiseHexOrder_workspace_size(int64_t nelem, int64_t nvert);
int fl_RaiseHexOrder(const double *points, int64_t nvert, const int64_t *elements, int64_t nelem,
                     const double *pattern, int64_t nodeperelem, double *out_points, int64_t points_capacity,
                     int64_t *nnode, int64_t *out_elements, void *workspace, size_t workspace_bytes,
                     fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Implicit assembly of the tangent stiffness and the internal-force residual (FP64), one
 * entry per material, argument list of the reference's _GlobalAssemblyDF_<Mat> plus `flags`
 * and `stream`:
 *   points [nnode*3], elements [nelem*nodeperelem] (uint64), Eulerx [nnode*3],
 *   Jm [ndim*nodeperelem*ngauss] (reference-element gradients, d-major then node then point),
 *   AllGauss [ngauss] (weights). Eulerp, bases, local_rows_stiffness, local_cols_stiffness,
 *   sorted_elements, sorter and anisotropic_orientations are accepted for signature parity and
 *   not read (the kernel derives what they carry).
 *   recompute_sparsity_pattern = 1: triplets, I_stiff/J_stiff/V_stiff of nelem*ndof^2 entries,
 *     entry elem*ndof^2 + r*ndof + c holds (global row of local dof r, global column of c, K_e[r][c]).
 *   recompute_sparsity_pattern = 0: CSR values V_stiff[nnz] += , with I_stiff = indptr and
 *     J_stiff = indices (as the reference's wrapper passes them), through data_local_indices /
 *     data_global_indices, or, if squeeze_sparsity_pattern = 1, by binary search in each row.
 *   T [nnode*3] += residual (internal traction) when requires_geometry_update == 1.
 *   ndim and nvar must be 3 and H_VoigtSize 6. flags: optional device int (FL_FLAG_* bits OR-ed in).
 * Supported nodeperelem: 4, 8, 10, 20, 27, 35, 64, 125 (tet p=1..4, hex p=1..4); ngauss <= 343.
 * ------------------------------------------------------------------------------------------ */
#define FL_GLOBAL_ASSEMBLY_DF_ARGS                                                                          \
    const double *points, const uint64_t *elements, const double *Eulerx, const double *Eulerp,            \
        const double *bases, const double *Jm, const double *AllGauss, int64_t ndim, int64_t nvar,          \
        int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t H_VoigtSize,             \
        int64_t requires_geometry_update, const int64_t *local_rows_stiffness,                              \
        const int64_t *local_cols_stiffness, int32_t *I_stiff, int32_t *J_stiff, double *V_stiff,           \
        double *T, int recompute_sparsity_pattern, int squeeze_sparsity_pattern,                            \
        const int32_t *data_local_indices, const int32_t *data_global_indices,                              \
        const uint64_t *sorted_elements, const int64_t *sorter, double rho, double mu, double mu1,          \
        double mu2, double mu3, double mue, double lamb, double eps_1, double eps_2, double eps_3,          \
        double eps_e, const double *anisotropic_orientations, int *flags, fl_stream_t stream

int fl_GlobalAssemblyDF__NeoHookean_(FL_GLOBAL_ASSEMBLY_DF_ARGS);   /* mu, lamb */
int fl_GlobalAssemblyDF__MooneyRivlin_(FL_GLOBAL_ASSEMBLY_DF_ARGS); /* mu1, mu2, lamb */
/* The same for the two other isotropic low-level DF materials of the reference
 * (AOT_Assembler.py:8-14): _GlobalAssemblyDF__NearlyIncompressibleMooneyRivlin_ (parameters
 * alpha, beta, kappa passed as mu1, mu2, lamb; _NearlyIncompressibleMooneyRivlin_.h:26-90) and
 * _GlobalAssemblyDF__LinearElastic_ (mu, lamb; _LinearElastic_.h:26-60; built without the geometric
 * stiffness, AOT_Assembler.py:74-81). */
int fl_GlobalAssemblyDF__NearlyIncompressibleMooneyRivlin_(FL_GLOBAL_ASSEMBLY_DF_ARGS);
int fl_GlobalAssemblyDF__LinearElastic_(FL_GLOBAL_ASSEMBLY_DF_ARGS);
/* _GlobalAssemblyDF__AnisotropicMooneyRivlin_1_ (AOT_Assembler.py:8-14, 72-75, 113-114): the
 * transversely isotropic Mooney-Rivlin law of _AnisotropicMooneyRivlin_1_.h:31-88 with parameters
 * mu1, mu2, mu3, lamb and one fibre direction per element, anisotropic_orientations [nelem][3]
 * (device, required: FL_ERR_ARG if null). */
int fl_GlobalAssemblyDF__AnisotropicMooneyRivlin_1_(FL_GLOBAL_ASSEMBLY_DF_ARGS);

/* ------------------------------------------------------------------------------------------
 * Allocation-free tangent + residual assembly. No counterpart in the reference (its assembly
 * runs on the CPU and mallocs its own work arrays).
 *
 * For callers that cannot allocate device memory while they run: cudaMalloc and cudaFree may
 * synchronise the whole device and can fail under memory pressure, so an application that
 * reserves its device memory once at start-up -- its own pool allocator handing out every byte,
 * or a Newton / time-stepping loop that must not stall or fail half-way -- cannot let an
 * assembly call allocate. fl_GlobalAssemblyDF__<Mat>_ takes its Gauss-point scratch from the
 * stream-ordered allocator on every call; this entry point instead uses a fixed array of
 * FL_NOALLOC_SCRATCH_BYTES (32 MiB) that the library places in device memory when it is loaded
 * (every GPU that loads the library holds it until the process exits). It calls no cudaMalloc,
 * cudaFree or other allocating routine. The caller still passes every input and output.
 *
 * Same arguments and results as fl_GlobalAssemblyDF__NeoHookean_ / __MooneyRivlin_, preceded by
 * material_number (FL_MATERIAL_NEOHOOKEAN: mu, lamb; FL_MATERIAL_MOONEYRIVLIN: mu1, mu2, lamb; any
 * other material number returns FL_ERR_UNSUPPORTED).
 * Limit: nelem * ngauss * 432 bytes (54 doubles per Gauss point) must fit in
 * FL_NOALLOC_SCRATCH_BYTES, e.g. up to 621 hex p=2 elements with 125 Gauss points or 5 548 tet
 * p=3 elements with 14; larger meshes return FL_ERR_CAPACITY without launching anything. Such a
 * mesh can be assembled in consecutive element ranges, because the outputs accumulate: pass
 * elements + e0*nodeperelem, nelem = range length and, in CSR mode, data_local_indices and
 * data_global_indices + e0*ndof^2 (triplet mode: I/J/V_stiff + e0*ndof^2).
 * The first call on each device looks up the array's device address (cudaGetSymbolAddress, with
 * that device current); make that first call before any stream capture. Every call uses the same
 * array and leaves its contents behind; each call writes all the scratch it reads, so nothing
 * has to be cleared, but calls that overlap on the GPU (different streams or host threads) race
 * on the array and must be serialised by the caller.
 * ------------------------------------------------------------------------------------------ */
#define FL_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
int fl_GlobalAssemblyDF_noalloc(int material_number, FL_GLOBAL_ASSEMBLY_DF_ARGS);

/* ------------------------------------------------------------------------------------------
 * Mixed-precision tangent for inexact Newton: the tangent of fl_GlobalAssemblyDF__<Mat>_ with its
 * dense per-element contraction on the tensor cores (split-BF16, three products, FP32
 * accumulation) written to FP32 CSR values V_stiff[nnz] (+=), and the residual T[nnode*3] (+=)
 * in FP64 exactly as the FP64 entry points form it. Kinematics and the constitutive update stay
 * FP64. No reference counterpart: the reference assembles only in FP64
 * (_LowLevelAssemblyDF_.h:8-176); this is the Jacobian fl_BlockJacobiPCG applies with
 * value_bits = 32. CSR through the reference's element-to-nonzero maps, or, with both map
 * pointers NULL, by binary search in the rows of indptr/indices.
 * material_number: FL_MATERIAL_NEOHOOKEAN (mu, lamb), FL_MATERIAL_MOONEYRIVLIN (mu1, mu2, lamb),
 * FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN (alpha, beta, kappa as mu1, mu2, lamb),
 * FL_MATERIAL_LINEARELASTIC (mu, lamb) or FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1 (mu1, mu2, lamb, mu3
 * and anisotropic_orientations [nelem][3], required for it and ignored otherwise);
 * element_params [nelem][3] (optional) overrides (p0, p1, p2) per element, as in
 * fl_GlobalAssemblyDF_Batched (not for the transversely isotropic law).
 * ------------------------------------------------------------------------------------------ */
int fl_GlobalAssemblyDF_Mixed(int material_number, const double *points, const uint64_t *elements,
                              const double *Eulerx, const double *Jm, const double *AllGauss, int64_t ngauss,
                              int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t requires_geometry_update,
                              const int32_t *indptr, const int32_t *indices, const int32_t *data_local_indices,
                              const int32_t *data_global_indices, float *V_stiff, double *T, double mu, double mu1,
                              double mu2, double lamb, double mu3, const double *anisotropic_orientations,
                              const double *element_params, int *flags, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Batched assembly of many independent meshes: the caller concatenates the instances of one
 * element type into one mesh with disjoint node ranges (the CSR tangent is then the direct sum of
 * the instances' tangents) and gives every element its own material parameters,
 * element_params[nelem][3] = (mu, lamb, 0) for FL_MATERIAL_NEOHOOKEAN or (mu1, mu2, lamb) for
 * FL_MATERIAL_MOONEYRIVLIN. CSR values V_stiff[nnz] (+=) through the element-to-nonzero maps, or,
 * with both map pointers NULL, by binary search in each row (no per-element maps: the memory of
 * large batches); residual T (+=). No reference counterpart: the reference assembles one mesh per
 * call (_LowLevelAssemblyDF_.h:8-176); its DetachedParallelFEMSolver
 * (Solver/DetachedParallelFEMSolver.py:11-248) runs independent problems as separate processes.
 * ------------------------------------------------------------------------------------------ */
int fl_GlobalAssemblyDF_Batched(int material_number, const double *points, const uint64_t *elements,
                                const double *Eulerx, const double *Jm, const double *AllGauss, int64_t ngauss,
                                int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t requires_geometry_update,
                                const double *element_params, const int32_t *indptr, const int32_t *indices,
                                const int32_t *data_local_indices, const int32_t *data_global_indices,
                                double *V_stiff, double *T, int *flags, fl_stream_t stream);

/* Autotuner hook: Gauss points per shared-memory chunk of the FP64 contraction kernel for one
 * (nodeperelem, ngauss) pair (0 restores the default). Applies to every later FP64 assembly call
 * in the process. FL_ERR_CAPACITY when the table (64 pairs) is full. */
int fl_SetAssemblyTuning(int64_t nodeperelem, int64_t ngauss, int gauss_chunk);

/* Arithmetic of the stiffness contraction in every later FP64-valued assembly call of the process
 * (no reference counterpart; the reference contracts in FP64). FL_ARITH_FP64: FP64 fused
 * multiply-adds. FL_ARITH_FLOAT_PAIR: each operand held as an unevaluated pair of
 * floats (hi + lo), products formed error-free in their leading part and summed with a
 * compensated two-sum on the FP32 pipe, ~2^-46 relative per multiply-add (element matrices
 * within ~1e-14 of FP64), about 1.6x faster on GB300, whose FP64 rate is 1/64 of its FP32 rate. The kinematics, the material law, the residual and the scatter stay FP64
 * in both. FL_ERR_ARG for other values. */
#define FL_ARITH_FP64 0
#define FL_ARITH_FLOAT_PAIR 1
/* FL_ARITH_TENSOR: the contraction on the tensor cores with both operands scaled and split into
 * six signed 8-bit digits held exactly in BF16, digit products summed per weight level in FP32
 * (the three leading levels exactly), recombined as float pairs and added in FP64: element
 * matrices within ~1e-13 of FP64. Applies to CSR outputs (maps or squeeze) without a
 * caller-provided scratch, for element types whose reduction fits (3 * 3 * ngauss * 2^14 < 2^24);
 * other calls use the float-pair contraction. */
#define FL_ARITH_TENSOR 2
/* FL_ARITH_REFERENCE_TENSOR: every element matrix of a tile of 14 elements as one tensor-core GEMM
 * of the pulled-back tangents [(element, i, k) x (Gauss point, d, e)] against the element-type
 * constant reference tensor Phi[(a, b) x (Gauss point, d, e)] = Jm[d][a][g] Jm[e][b][g] (node
 * pairs a <= b), both operands split into seven BF16 digit planes (28 plane products, five FP32
 * tensor-memory accumulators, the leading four levels exact), recombined exactly into FP64 with
 * integer instructions: element matrices within ~1e-14 of FP64. The kinematics and the material
 * law run in FP64, the tangent's pull-back and the residual as float pairs. Applies to CSR
 * outputs (maps or squeeze) without a caller-provided scratch, for 4-, 8-, 10- and 20-node
 * elements with at most 15 Gauss points; other calls use the float-pair contraction. The
 * default. */
#define FL_ARITH_REFERENCE_TENSOR 3
int fl_SetAssemblyArithmetic(int arithmetic);
int fl_GetAssemblyArithmetic(void);

/* Per-element block offsets of a node-blocked CSR pattern (no reference counterpart: the
 * reference's element-to-nonzero maps, ComputeSparsityPattern.h:67-125, hold one position per
 * element matrix entry; this holds one per node pair, 9x fewer): block_offsets[e][a][b]
 * (nelem * nodeperelem^2 int32, device) = the offset of column 3 * elements[e][b] within row
 * 3 * elements[e][a] when the 3x3 node block sits where a node-blocked CSR puts it (the node's three
 * rows of equal length and consecutive, the block's entries at indptr[3 n] + i * rowlength +
 * offset + k), else -1. Built once per mesh for fl_GlobalAssemblyDF_Blocks. flags: optional
 * device int, FL_FLAG_BAD_INDEX for an out-of-range node id. No synchronisation. */
int fl_ElementBlockOffsets(const uint64_t *elements, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                           const int32_t *indptr, const int32_t *indices, int32_t *block_offsets, int *flags,
                           fl_stream_t stream);

/* The reference configuration's part of the kinematics (no reference counterpart; the reference
 * recomputes it in every call, _KinematicMeasures_.h:64-99): per element and Gauss point the
 * inverse of dX/dxi = sum_a Jm[.][a][g] X_a (9 values, row-major) and its determinant, into
 * geometry[10][nelem * ngauss] (device FP64, element-major within each row: index e * ngauss + g).
 * Constant for a mesh; the assembly given it (fl_GlobalAssemblyDF_Blocks) forms only the current
 * configuration's sums, with results identical to recomputing it. flags: optional device int,
 * FL_FLAG_BAD_INDEX for an out-of-range node id. No synchronisation. */
int fl_ReferenceGeometry(const double *points, const uint64_t *elements, const double *Jm, int64_t nelem,
                         int64_t nodeperelem, int64_t ngauss, int64_t nnode, double *geometry, int *flags,
                         fl_stream_t stream);

/* fl_GlobalAssemblyDF__<Mat>_ with per-mesh data supplied by a caller that keeps the mesh on the
 * device between calls (no reference counterpart): the block offsets (fl_ElementBlockOffsets; in
 * CSR mode with FL_ARITH_REFERENCE_TENSOR the contraction scatters through them instead of building
 * them in the call) and the reference geometry (fl_ReferenceGeometry, computed for the same points,
 * elements and Jm). Same arguments and results otherwise, preceded by material_number
 * (FL_MATERIAL_*), block_offsets and reference_geometry (each may be NULL). */
int fl_GlobalAssemblyDF_Blocks(int material_number, const int32_t *block_offsets, const double *reference_geometry,
                               FL_GLOBAL_ASSEMBLY_DF_ARGS);

/* Tiling of the split-BF16 tensor-core tangent (fl_GlobalAssemblyDF_Mixed; no reference
 * counterpart) for every later call of the process: tile_group = 128-row tiles of the element's
 * transposed stiffness per work item (1..16), reduction_chunk = (Gauss point, direction) columns
 * per tensor-core round (a multiple of 16 up to 96). 0 = automatic (the default). A choice whose
 * shared or tensor memory does not fit makes later calls return FL_ERR_UNSUPPORTED. FL_ERR_ARG
 * outside the ranges. */
int fl_SetTensorCoreTiling(int tile_group, int reduction_chunk);

/* ------------------------------------------------------------------------------------------
 * Explicit (matrix-free) internal force, T[nnode*nvar] += sum_e sum_g detJ (grad N_a . sigma).
 * Argument list of the reference's _GlobalAssemblyExplicit_DF_DPF_ plus flags and stream.
 * formulation_number must be 0 (mechanics), material_number FL_MATERIAL_NEOHOOKEAN (mu, lamb)
 * or FL_MATERIAL_MOONEYRIVLIN (mu1, mu2, lamb). Unused pointers may be NULL.
 * ------------------------------------------------------------------------------------------ */
int fl_GlobalAssemblyExplicit_DF_DPF_(const double *points, const uint64_t *elements, const double *Eulerx,
                                      const double *Eulerp, const double *bases, const double *Jm,
                                      const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss,
                                      int64_t nelem, int64_t nodeperelem, int64_t nnode, int64_t H_VoigtSize,
                                      int64_t requires_geometry_update, double *T, double rho, double mu,
                                      double mu1, double mu2, double mu3, double mue, double lamb, double eps_1,
                                      double eps_2, double eps_3, double eps_e,
                                      const double *anisotropic_orientations, int material_number,
                                      int formulation_number, int *flags, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Displacement-potential (electromechanics) assembly, nvar 4 (three displacements and the electric
 * potential per node, global dof 4 n + v), H_VoigtSize 9: the reference's _GlobalAssemblyDPF_
 * (FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDPF_.h:8-198) as AOT_Assembler.py:125-175
 * monomorphises it for _IsotropicElectroMechanics_108_, _106_, _105_, _101_, _0_, _SteinmannModel_ and
 * _Piezoelectric_100_, called from
 * _LowLevelAssemblyDPF_.pyx:53-160. Same argument list and scatter modes as the DF entries:
 * recompute_sparsity_pattern -> triplets (I_stiff, J_stiff, V_stiff [nelem*(4 npe)^2]); else
 * I_stiff = indptr [4 nnode + 1], J_stiff = indices, V_stiff [nnz] += at the positions the maps
 * name (found, as with squeeze_sparsity_pattern, by one search per row of a node pair's 4 x 4 block:
 * the tangent is formed per node pair a <= b and mirrored, being symmetric). Eulerp [nnode] is the
 * electric potential; T [4 nnode] +=. The maps mode reads indptr[4 nnode] once (one
 * synchronisation). flags: optional device int
 * (FL_FLAG_* bits). FL_ERR_UNSUPPORTED when an element's Gauss-point data do not fit in shared
 * memory (more than about 64 nodes x 64 points).
 * ------------------------------------------------------------------------------------------ */
int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_(FL_GLOBAL_ASSEMBLY_DF_ARGS); /* mu1, mu2, lamb, eps_2 */
int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_101_(FL_GLOBAL_ASSEMBLY_DF_ARGS); /* mu, lamb, eps_1 */
int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_0_(FL_GLOBAL_ASSEMBLY_DF_ARGS);   /* mu, lamb, eps_1 */
int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_106_(FL_GLOBAL_ASSEMBLY_DF_ARGS); /* mu1, mu2, lamb, eps_1, eps_2 */
int fl_GlobalAssemblyDPF__IsotropicElectroMechanics_105_(FL_GLOBAL_ASSEMBLY_DF_ARGS); /* mu1, mu2, lamb, eps_1, eps_2 */
int fl_GlobalAssemblyDPF__SteinmannModel_(FL_GLOBAL_ASSEMBLY_DF_ARGS); /* mu, lamb, c1 as eps_3, c2 as eps_2, eps_1 */
/* mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3; anisotropic_orientations [nelem*3] required (one fibre
 * direction per element) */
int fl_GlobalAssemblyDPF__Piezoelectric_100_(FL_GLOBAL_ASSEMBLY_DF_ARGS);

/* ------------------------------------------------------------------------------------------
 * Lumped (row-sum) mass: M[nnode*nvar] += row sums of sum_g rho N N^T w_g |det dX/dxi|.
 * bases [nodeperelem*ngauss] (node-major), Jm and AllGauss as above. flags: optional device int.
 * ------------------------------------------------------------------------------------------ */
int fl_LumpedMass(const double *points, const uint64_t *elements, const double *bases, const double *Jm,
                  const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss, int64_t nelem,
                  int64_t nodeperelem, int64_t nnode, double rho, double *M, int *flags, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Consistent mass (mass_type 1 of _GenericConstantMassIntegrand_, _MassIntegrand_.h:249-400,
 * scattered as its fill_global_data, :68-178): element mass sum_g rho N_a N_b w_g |det dX/dxi|
 * on the nvar diagonal of every node pair.
 *   recompute_sparsity_pattern != 0: triplets I_mass, J_mass, V_mass [nelem*(nvar*nodeperelem)^2]
 *     written in element-local order (entry e*ndof^2 + r*ndof + c, zeros off the nvar diagonal);
 *   else squeeze_sparsity_pattern != 0: V_mass[nnz] += by searching each CSR row (indptr, indices);
 *   else: V_mass[nnz] += through the element-to-nonzero maps (data_local_indices,
 *     data_global_indices, [nelem*(nvar*nodeperelem)^2] each).
 * nvar 1..4 (the mass acts on every field, as in the reference). flags: optional device int,
 * FL_FLAG_BAD_INDEX when a node id or map entry is out of range (the entry is skipped).
 * ------------------------------------------------------------------------------------------ */
int fl_ConsistentMass(const double *points, const uint64_t *elements, const double *bases, const double *Jm,
                      const double *AllGauss, int64_t ndim, int64_t nvar, int64_t ngauss, int64_t nelem,
                      int64_t nodeperelem, int64_t nnode, double rho, int recompute_sparsity_pattern,
                      int squeeze_sparsity_pattern, const int32_t *indptr, const int32_t *indices, int64_t nnz,
                      const int32_t *data_local_indices, const int32_t *data_global_indices, int32_t *I_mass,
                      int32_t *J_mass, double *V_mass, int *flags, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Explicit central-difference dynamics (the lumped-mass loop of
 * ExplicitStructuralDynamicIntegrator.Solver, TimeIntegrators/ExplicitStructuralDynamicIntegrator.py:28-245).
 *
 * fl_ReferenceGradients: grad0 [nelem][ngauss][nodeperelem][3] (FP32) = dN_a/dX at each Gauss
 *   point and dV [nelem][ngauss] (FP32) = w |det dX/dxi|, once per mesh, for fl_InternalForceF32.
 * fl_InternalForceF32: T [nnode*3] (FP32) += internal force at displacement u [nnode*3] (FP64
 *   state, converted per element), computed and accumulated in FP32 in the total-Lagrangian form
 *   (first Piola stress from H = grad_0 u without forming I + H, so small strains keep FP32's
 *   relative precision). The FP32 counterpart of fl_GlobalAssemblyExplicit_DF_DPF_ (same
 *   quantity). Neo-Hookean only (mu, lamb); ngauss <= 32.
 * fl_CentralDifferenceUpdate: on free dofs a = (Fext - T) / M (Minv given, Fext may be NULL),
 *   v += dt a, u += dt v -- the leapfrog form of the reference's lumped update
 *   (ExplicitStructuralDynamicIntegrator.py:131-139). T is FP64, or FP32 when T_is_f32 != 0.
 * fl_StrainEnergy: *energy += sum_e sum_g W(F) w |det dX/dxi| at Eulerx (neo-Hookean
 *   W = mu/2 (tr C - 3) - mu ln J + lamb/2 (J-1)^2, MaterialLibrary/NeoHookean.py:70-80; the
 *   reference sums it in DisplacementFormulation.GetEnergy, DisplacementFormulation.py:326-371).
 * ------------------------------------------------------------------------------------------ */
int fl_ReferenceGradients(const double *points, const uint64_t *elements, const double *Jm, const double *AllGauss,
                          int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode, float *grad0,
                          float *dV, int *flags, fl_stream_t stream);
int fl_InternalForceF32(const uint64_t *elements, const double *u, const float *grad0, const float *dV,
                        int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode, int material_number,
                        double mu, double lamb, float *T, int *flags, fl_stream_t stream);
/* Float-pair variant (no reference counterpart): the same total-Lagrangian neo-Hookean force with
 * every quantity carried as an unevaluated pair of floats on the FP32 pipe (~2^-46 relative per
 * operation, FP64-level results). fl_ReferenceGradientsPair writes dN_a/dX as grad0_hi + grad0_lo
 * (FP32 arrays, layout of grad0 above) and dV in FP64; fl_InternalForcePair accumulates
 * T [nnode*3] (FP64) +=. ngauss <= 32. */
int fl_ReferenceGradientsPair(const double *points, const uint64_t *elements, const double *Jm,
                              const double *AllGauss, int64_t ngauss, int64_t nelem, int64_t nodeperelem,
                              int64_t nnode, float *grad0_hi, float *grad0_lo, double *dV, int *flags,
                              fl_stream_t stream);
int fl_InternalForcePair(const uint64_t *elements, const double *u, const float *grad0_hi, const float *grad0_lo,
                         const double *dV, int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                         int material_number, double mu, double lamb, double *T, int *flags, fl_stream_t stream);
int fl_CentralDifferenceUpdate(int64_t n, double dt, const void *T, int T_is_f32, const double *Fext,
                               const double *Minv, const int8_t *fixed, double *u, double *v, fl_stream_t stream);
int fl_StrainEnergy(const double *points, const uint64_t *elements, const double *Eulerx, const double *Jm,
                    const double *AllGauss, int64_t ngauss, int64_t nelem, int64_t nodeperelem, int64_t nnode,
                    int material_number, double mu, double lamb, double *energy, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Newton's linear step: K_ff x_f = b_f by conjugate gradients with a 3x3 nodal block-Jacobi
 * preconditioner, FP64, on the assembled CSR tangent (replaces the reduce-and-solve of
 * NewtonRaphson, Solver/FEMSolver.py:951-954: BoundaryCondition.GetReducedMatrices,
 * BoundaryCondition.py:842-857, and LinearSolver.Solve, Solver/LinearSolver.py:208-330).
 *   indptr/indices/values  CSR of K [nrows x nrows], nrows = 3 * nodes, every 3x3 diagonal block
 *                          present in the pattern (true for assembled tangents); value_bits:
 *                          FL_PCG_F64        FP64 values, FP64 products
 *                          FL_PCG_F64_SPLIT  FP64 values, split once per solve into float pairs
 *                                            (hi + lo) in the workspace; products in float-pair
 *                                            arithmetic on the FP32 pipe (~2^-44 relative)
 *                          FL_PCG_F32        FP32 values (an inexact-Newton Jacobian), float-pair
 *                                            products
 *                          the vectors, dot products and the preconditioner are FP64 in all three
 *   fixed [nrows]          1 for Dirichlet dofs: their rows and columns are left out (masking)
 *   b [nrows]              right-hand side (fixed entries ignored)
 *   x [nrows]              in: initial guess with zero fixed entries; out: solution
 *   stop when |r| <= rtol |b| (free dofs) or after maxiter iterations; iterations and relres
 *   (host out) report where it stopped. workspace: fl_BlockJacobiPCG_workspace_size(nrows, nnz,
 *   value_bits) bytes.
 * The iterations run on the device as one CUDA graph: a conditional WHILE node whose body is one
 * iteration (three kernels and a one-thread tail that tests convergence and sets the loop
 * condition), so the host waits once per solve. With fl_SetPCGDeviceLoop(0), or where the graph
 * cannot be built, the host launches the iterations and synchronises every 16 of them to test
 * convergence. FL_ERR_ARG on a missing or singular diagonal block or a non-finite residual.
 * ------------------------------------------------------------------------------------------ */
int fl_SetPCGDeviceLoop(int enable);
int fl_GetPCGDeviceLoop(void);
#define FL_PCG_F64 64
#define FL_PCG_F32 32
#define FL_PCG_F64_SPLIT 6432
/* ------------------------------------------------------------------------------------------
 * Pieces of the two-level p-multigrid preconditioner of Newton's linear step on high-order
 * tetrahedra (florence_gb300/multigrid.py). No reference counterpart: the reference solves the
 * reduced system with a direct or a scipy iterative solver (Solver/LinearSolver.py:153-330).
 * All pointers are device pointers; nothing synchronises.
 *
 * fl_NodalTransfer: y[3r + i] (=, or += with accumulate) sum_{k = ptr[r]}^{ptr[r+1]-1} w[k]
 *   x[3 cols[k] + i] for the nrows node rows (a prolongation from vertex values to the nodes of
 *   the high-order elements, or its transpose, the restriction).
 * fl_MaskedMatVec: y = K_ff x on the rows of an FP64 CSR matrix, rows and columns of fixed dofs
 *   (fixed[dof] != 0) masked; with b non-NULL y = b - K_ff x instead (y = 0 on fixed rows).
 * fl_MaskedMatVecBlocks: the same product for a node-blocked pattern (the three rows of a node list
 *   the same nodes, three columns each: every assembled tangent's pattern), one warp per node and
 *   one column index per 3x3 block; x must be zero on fixed dofs. fl_MaskedMatVecBlocksF32: with
 *   FP32 values (FP32 products and sums), for smoothers. fl_MaskedMatVecBlocksPair: with the
 *   values and x as float pairs (hi, lo interleaved, from fl_SplitPairs), ~2^-44 relative, on the
 *   FP32 pipe. fl_SplitPairs: pairs[2i], pairs[2i + 1] = hi, lo of v[i].
 * fl_BlockJacobiInverse: Binv[n][9] = inverse of each node's 3x3 diagonal block, fixed rows and
 *   columns replaced by the identity (FL_FLAG_BAD_INDEX in flags for a missing or singular block).
 * fl_BlockJacobiApply: z (=, or +=) omega Binv r per node, 0 on fixed dofs.
 * fl_CoarsePCG: x = the block-Jacobi PCG solution of K_ff x = b_f from x = 0 (Binv from
 *   fl_BlockJacobiInverse of the same matrix; a node-blocked pattern as fl_MaskedMatVecBlocks
 *   takes), stopped at |r| <= rtol |b_f| or after maxiter
 *   iterations, in ONE cooperative launch (every CTA resident, grid barriers between the three
 *   phases of an iteration, bounded waits): for small systems, whose iterations would otherwise
 *   be bound by kernel boundaries. workspace: fl_CoarsePCG_workspace_size(nrows) bytes.
 *   iterations (optional, device int64): the iteration count is ADDED to it; relres (optional,
 *   device double): |r| / |b_f| at the end; flags (optional, device int): FL_FLAG_TIMEOUT when a
 *   barrier wait gave up, FL_FLAG_BAD_INDEX when p.K_ff p <= 0, FL_FLAG_CAPACITY (nothing solved)
 *   when the rows of one SM's share of the nodes exceed its 200 KB of shared memory, where they
 *   stay for the whole solve (about 16 k nodes on 152 SMs). FL_ERR_UNSUPPORTED without
 *   cooperative launch. Nothing synchronises.
 * ------------------------------------------------------------------------------------------ */
int fl_NodalTransfer(int64_t nrows, const int32_t *ptr, const int32_t *cols, const double *weights, const double *x,
                     double *y, int accumulate, fl_stream_t stream);
int fl_MaskedMatVec(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nrows,
                    const int8_t *fixed, const double *x, const double *b, double *y, fl_stream_t stream);
int fl_MaskedMatVecBlocks(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nrows,
                          const int8_t *fixed, const double *x, const double *b, double *y, fl_stream_t stream);
int fl_MaskedMatVecBlocksF32(const int32_t *indptr, const int32_t *indices, const float *values, int64_t nrows,
                             const int8_t *fixed, const double *x, const double *b, double *y, fl_stream_t stream);
int fl_SplitPairs(int64_t n, const double *v, float *pairs, fl_stream_t stream);
/* fl_MaskedMatMatBlocksF32: Y = K_ff X for ncolumns (32, 64 or 128) columns at once, X and Y
 * row-major [nrows][ncolumns] FP32, FP32 values of a node-blocked pattern; X zero on fixed dofs.
 * For projections onto a reduced basis (the warm start's Galerkin correction). */
int fl_MaskedMatMatBlocksF32(const int32_t *indptr, const int32_t *indices, const float *values, int64_t nrows,
                             const int8_t *fixed, const float *X, float *Y, int64_t ncolumns, fl_stream_t stream);
int fl_MaskedMatVecBlocksPair(const int32_t *indptr, const int32_t *indices, const float *value_pairs, int64_t nrows,
                              const int8_t *fixed, const float *x_pairs, const double *b, double *y,
                              fl_stream_t stream);
int fl_BlockJacobiInverse(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nnode,
                          const int8_t *fixed, double *Binv, int *flags, fl_stream_t stream);
int fl_BlockJacobiApply(int64_t nnode, const double *Binv, const int8_t *fixed, double omega, const double *r,
                        double *z, int accumulate, fl_stream_t stream);
size_t fl_CoarsePCG_workspace_size(int64_t nrows);
int fl_CoarsePCG(const int32_t *indptr, const int32_t *indices, const double *values, int64_t nrows,
                 const int8_t *fixed, const double *Binv, const double *b, double *x, double rtol, int64_t maxiter,
                 void *workspace, size_t workspace_bytes, int64_t *iterations, double *relres, int *flags,
                 fl_stream_t stream);

size_t fl_BlockJacobiPCG_workspace_size(int64_t nrows, int64_t nnz, int value_bits);
int fl_BlockJacobiPCG(const int32_t *indptr, const int32_t *indices, const void *values, int value_bits,
                      int64_t nrows, const int8_t *fixed, const double *b, double *x, double rtol, int64_t maxiter,
                      void *workspace, size_t workspace_bytes, int64_t *iterations, double *relres,
                      fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Learned Newton warm start (no reference counterpart: the reference starts every increment
 * from the previous one, Solver/FEMSolver.py:841-929). An MLP 3 -> 256 -> 256 -> 64 with GELU
 * maps (load, material) parameters to the coefficients of the displacement in a 64-mode POD
 * basis. BF16 arithmetic (GEMM operands rounded to BF16, FP32 accumulation), FP32 master
 * parameters: params [fl_MLP_num_params()] = W1[3][256], b1[256], W2[256][256], b2[256],
 * W3[256][64], b3[64] (row-major, y = x W + b). x [batch][3], y/target [batch][64], FP32.
 * fl_MLPForward: y = net(x). fl_MLPGradients: grads [num_params] = dL/dparams and *loss (device,
 * optional) = L for L = sum (y - target)^2 / (2 batch 64). fl_MLPAdamStep: Adam update of params
 * (m, v [num_params] state, step >= 1). workspace: fl_MLP_workspace_size(batch) bytes.
 * ------------------------------------------------------------------------------------------ */
int64_t fl_MLP_num_params(void);
size_t fl_MLP_workspace_size(int64_t batch);
int fl_MLPForward(const float *params, const float *x, int64_t batch, float *y, void *workspace, size_t ws_bytes,
                  fl_stream_t stream);
int fl_MLPGradients(const float *params, const float *x, const float *target, int64_t batch, float *grads,
                    float *loss, void *workspace, size_t ws_bytes, fl_stream_t stream);
int fl_MLPAdamStep(float *params, const float *grads, float *m, float *v, int64_t step, float lr, float beta1,
                   float beta2, float eps, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Measurement helpers: device time of independent FMA chains over the whole GPU, used to measure
 * the FP64 and FP32 roofs that the assembly kernels are bound by (FP64 arithmetic, and the
 * float-pair arithmetic on the FP32 pipe). Synchronise the stream. gflops (host out) = achieved
 * GFLOP/s (2 flops per FMA).
 * ------------------------------------------------------------------------------------------ */
int fl_measure_fp64_peak(double *gflops, fl_stream_t stream);
int fl_measure_fp32_peak(double *gflops, fl_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * External forces, F[nnode*3] += (device arrays). AssembleExternalTractionForces
 * (Assembly.py:451-514): for every face f with neumann_flags[f] != 0 (all faces if the flags are
 * NULL), F[(faces[f][a], i)] += applied_neumann[f][i] * sum_g Bases[a][g] w_g, the reference's
 * parent-face weights; with Jm_face [2][nodeperface][ngauss] (the face basis gradients) and the
 * points, w_g is multiplied by |dX/dxi x dX/deta| (the physical face). AssembleBodyForces
 * (Assembly.py:516-560): F[(elements[e][a], z)] -= rho * sum_g Bases[a][g] w_g for every element.
 * flags: device int, FL_FLAG_BAD_INDEX when a node id is out of range. No synchronisation.
 * ------------------------------------------------------------------------------------------ */
int fl_AssembleExternalTractionForces(const uint64_t *faces, int64_t nface, int64_t nodeperface,
                                      const uint8_t *neumann_flags, const double *applied_neumann,
                                      const double *Bases, const double *AllGauss, int64_t ngauss,
                                      const double *points, const double *Jm_face, int64_t nnode, double *F,
                                      int *flags, fl_stream_t stream);
int fl_AssembleBodyForces(const uint64_t *elements, int64_t nelem, int64_t nodeperelem, const double *Bases,
                          const double *AllGauss, int64_t ngauss, double rho, int64_t nnode, double *F, int *flags,
                          fl_stream_t stream);

/* Self-test of the tcgen05 tensor-core path (no reference counterpart): D [128 x 32] (FP32,
 * row-major) = A [128 x 48] * B [32 x 48]^T with BF16 A and B (row-major, device pointers), one
 * CTA, operands in shared memory, accumulator in tensor memory. *status (device) gets bit 1 if
 * the completion wait timed out. */
int fl_TensorCoreSelfTest(const void *A_bf16, const void *B_bf16, float *D, int *status, fl_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
