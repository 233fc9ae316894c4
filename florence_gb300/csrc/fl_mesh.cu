// fl_mesh.cu -- device generation of a high-order tet mesh from a linear one: the node placement
// and duplicate removal that Mesh.GetHighOrderMesh does for tets
// (Florence/MeshGeneration/Mesh.py:1339-1410 -> HighOrderMeshTet_SEMISTABLE,
//  HigherOrderMeshing/HigherOrderMeshingTet.py:19-135).
//
// The reference places every element's non-vertex nodes independently and then merges
// coincident points by rounding their coordinates and sorting them. Here the merge is
// topological: a local node is classified by the vertices that carry a nonzero barycentric weight
// (1 vertex, 2 an edge, 3 a face, 4 the interior), and nodes on a shared edge or face are the same
// node when their weights, listed in increasing global-vertex order, are the same. The result is
// the reference's mesh up to a permutation of the node numbers. The numbering itself is the
// lexicographic order of the keys (entity size, global vertices ascending, weights in that order)
// -- vertices first, then edges, faces and element interiors -- which the host builder
// (florence_gb300/meshes.py, raise_tet_order) also produces, so the two agree node for node.
//
// Steps: per-vertex incidence lists (counts, scan, fill); a warp per vertex collects the edges and
// faces it owns (the vertex is their smallest id), removes repeats and ranks the distinct ones in
// shared memory, once to count and, after scans of the counts, once to write into every element
// the number of each of its local edges and faces, marked where the element is the smallest one
// holding the entity; a CTA per tile of 32 elements, one warp per entity slot, then numbers the
// local nodes and -- in the marked element only, so that exactly one thread writes each node --
// computes their positions from the barycentric weights.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fl_common.cuh"
#include "fl_scan.cuh"

namespace fl {

constexpr int HM_MAX_NPE = 35;   // up to p = 4
constexpr int HM_MAX_EDGE = 8;   // nodes inside one edge
constexpr int HM_MAX_FACE = 16;  // nodes inside one face
constexpr double HM_NZ_TOL = 1e-10;
constexpr double HM_QSCALE = 1e6;
constexpr int HM_NT = 256;

// local node layout of the high-order tet, classified on the host
struct HmPattern {
    int npe, ne, nf, ni;
    double lam[HM_MAX_NPE][4];  // barycentric weights of the local nodes
    int kind[HM_MAX_NPE];       // vertices carrying the node: 1 vertex, 2 edge, 3 face, 4 interior
    int loc[HM_MAX_NPE][3];     // those local vertices, ascending (interior nodes: rank among them)
    int q[HM_MAX_NPE][3];       // their weights, rounded to 1e-6
    int qe[HM_MAX_EDGE];        // distinct first weights of an edge's nodes, ascending
    int qf[HM_MAX_FACE][2];     // distinct (first, second) weights of a face's nodes, ascending
    int vnode[4];                   // local node of each vertex
    int enode[6][HM_MAX_EDGE];      // local nodes inside each local edge (TET_EDGES order)
    int fnode[4][HM_MAX_FACE];      // local nodes inside each local face (TET_FACES order)
    int inode[HM_MAX_NPE];          // interior local nodes, ascending
};

static const int TET_EDGES[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
static const int TET_FACES[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

__constant__ int TET_EDGES_D[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
__constant__ int TET_FACES_D[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

// index in TET_EDGES of the edge between local vertices a < b
__host__ __device__ inline int hm_edge_id(int a, int b) { return a * (5 - a) / 2 + b - 1; }

// FL_OK, or FL_ERR_UNSUPPORTED when the layout is not one that shared entities can number
// consistently from either side (weights not symmetric under the vertex permutations of an edge
// or face, different node counts per edge or face, two nodes of one entity with equal keys)
static int classify_pattern(const double *lam, int64_t npe, HmPattern *P) {
    if (!lam || npe < 4 || npe > HM_MAX_NPE) return npe > HM_MAX_NPE ? FL_ERR_UNSUPPORTED : FL_ERR_ARG;
    *P = HmPattern{};
    P->npe = (int)npe;
    int nvtx[4] = {0, 0, 0, 0}, nint = 0;
    std::vector<std::pair<int, int>> edge_nodes[6];          // (q of lower local vertex, q of upper)
    std::vector<std::vector<int>> face_nodes[4];             // (q_i, q_j, q_k) in local order
    for (int a = 0; a < npe; ++a) {
        int cnt = 0, idx[4] = {0, 0, 0, 0}, qq[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; ++k) {
            const double v = lam[a * 4 + k];
            if (!std::isfinite(v)) return FL_ERR_ARG;
            P->lam[a][k] = v;
            if (std::fabs(v) > HM_NZ_TOL) {
                idx[cnt] = k;
                qq[cnt] = (int)std::nearbyint(v * HM_QSCALE);  // round half to even, as numpy.round
                ++cnt;
            }
        }
        if (cnt == 0) return FL_ERR_UNSUPPORTED;
        P->kind[a] = cnt;
        for (int i = 0; i < 3; ++i) {
            P->loc[a][i] = i < cnt ? idx[i] : 0;
            P->q[a][i] = i < cnt ? qq[i] : 0;
        }
        if (cnt == 1) {
            ++nvtx[idx[0]];
        } else if (cnt == 2) {
            for (int s = 0; s < 6; ++s)
                if (TET_EDGES[s][0] == idx[0] && TET_EDGES[s][1] == idx[1]) edge_nodes[s].push_back({qq[0], qq[1]});
        } else if (cnt == 3) {
            for (int s = 0; s < 4; ++s)
                if (TET_FACES[s][0] == idx[0] && TET_FACES[s][1] == idx[1] && TET_FACES[s][2] == idx[2])
                    face_nodes[s].push_back({qq[0], qq[1], qq[2]});
        } else {
            P->loc[a][0] = nint++;
        }
    }
    for (int k = 0; k < 4; ++k)
        if (nvtx[k] != 1) return FL_ERR_UNSUPPORTED;
    // edges: the first weights seen from either end must be the same distinct set on every edge
    std::vector<int> ref_e;
    for (int s = 0; s < 6; ++s) {
        std::vector<int> fwd, rev;
        for (auto &w : edge_nodes[s]) {
            fwd.push_back(w.first);
            rev.push_back(w.second);
        }
        std::sort(fwd.begin(), fwd.end());
        std::sort(rev.begin(), rev.end());
        if (fwd != rev || std::adjacent_find(fwd.begin(), fwd.end()) != fwd.end()) return FL_ERR_UNSUPPORTED;
        if (s == 0) ref_e = fwd;
        else if (fwd != ref_e) return FL_ERR_UNSUPPORTED;
    }
    if (ref_e.size() > (size_t)HM_MAX_EDGE) return FL_ERR_UNSUPPORTED;
    // faces: the weight triples must be closed under the six vertex permutations, the same on
    // every face, and told apart by their first two weights
    std::vector<std::vector<int>> ref_f;
    for (int s = 0; s < 4; ++s) {
        std::vector<std::vector<int>> set = face_nodes[s];
        std::sort(set.begin(), set.end());
        for (auto &t : set) {
            std::vector<int> p = t;
            std::sort(p.begin(), p.end());
            do {
                if (!std::binary_search(set.begin(), set.end(), p)) return FL_ERR_UNSUPPORTED;
            } while (std::next_permutation(p.begin(), p.end()));
        }
        for (size_t i = 1; i < set.size(); ++i)
            if (set[i][0] == set[i - 1][0] && set[i][1] == set[i - 1][1]) return FL_ERR_UNSUPPORTED;
        if (s == 0) ref_f = set;
        else if (set != ref_f) return FL_ERR_UNSUPPORTED;
    }
    if (ref_f.size() > (size_t)HM_MAX_FACE) return FL_ERR_UNSUPPORTED;
    P->ne = (int)ref_e.size();
    P->nf = (int)ref_f.size();
    P->ni = nint;
    for (int i = 0; i < P->ne; ++i) P->qe[i] = ref_e[i];
    for (int i = 0; i < P->nf; ++i) {
        P->qf[i][0] = ref_f[i][0];
        P->qf[i][1] = ref_f[i][1];
    }
    // local nodes per entity, in local-node order
    int ce[6] = {0, 0, 0, 0, 0, 0}, cf[4] = {0, 0, 0, 0};
    for (int a = 0; a < npe; ++a) {
        const int *l = P->loc[a];
        if (P->kind[a] == 1) {
            P->vnode[l[0]] = a;
        } else if (P->kind[a] == 2) {
            const int s = hm_edge_id(l[0], l[1]);
            P->enode[s][ce[s]++] = a;
        } else if (P->kind[a] == 3) {
            const int s = 3 - (6 - l[0] - l[1] - l[2]);  // the face without vertex m is face 3 - m
            P->fnode[s][cf[s]++] = a;
        } else {
            P->inode[l[0]] = a;
        }
    }
    return FL_OK;
}

struct HmWork {
    int32_t *cnt;     // [nvert+1] incidence counts, then their exclusive scan (list starts)
    int32_t *cursor;  // [nvert]
    int32_t *list;    // [4*nelem] elements holding each vertex
    int32_t *vmin;    // [nvert] smallest element holding the vertex (-1: unused)
    int64_t *vrank;   // [nvert+1] used flags, then the node numbers of the used vertices
    int64_t *ecnt;    // [nvert+1] distinct edges each vertex owns, then the first edge number of each
    int64_t *fcnt;    // [nvert+1] distinct faces each vertex owns, then the first face number of each
    int64_t *eedge;   // [6*nelem] edge number << 1 | (this element is the smallest holding it)
    int64_t *eface;   // [4*nelem] face number << 1 | (this element is the smallest holding it)
    int64_t *bsum;    // scan block sums
    int32_t *info;    // [4]: error bits (1 vertex id out of range, 2 repeated vertex), maximum degree
};

static size_t hm_align(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t hm_layout(int64_t nelem, int64_t nvert, HmWork *w, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += hm_align(bytes);
        return p;
    };
    const int64_t nb = (nvert + 1 + SCAN_ITEMS - 1) / SCAN_ITEMS + 1;
    HmWork t;
    t.cnt = (int32_t *)take(sizeof(int32_t) * (nvert + 1));
    t.cursor = (int32_t *)take(sizeof(int32_t) * nvert);
    t.list = (int32_t *)take(sizeof(int32_t) * 4 * nelem);
    t.vmin = (int32_t *)take(sizeof(int32_t) * nvert);
    t.vrank = (int64_t *)take(sizeof(int64_t) * (nvert + 1));
    t.ecnt = (int64_t *)take(sizeof(int64_t) * (nvert + 1));
    t.fcnt = (int64_t *)take(sizeof(int64_t) * (nvert + 1));
    t.eedge = (int64_t *)take(sizeof(int64_t) * 6 * nelem);
    t.eface = (int64_t *)take(sizeof(int64_t) * 4 * nelem);
    t.bsum = (int64_t *)take(sizeof(int64_t) * (nb + SCAN_ITEMS));
    t.info = (int32_t *)take(sizeof(int32_t) * 4);
    if (w) *w = t;
    return off;
}

__global__ void hm_count(const int64_t *el, int64_t nelem, int64_t nvert, int32_t *cnt, int32_t *info) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelem; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t g[4];
        bool in_range = true;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            g[k] = el[e * 4 + k];
            in_range &= g[k] >= 0 && g[k] < nvert;
        }
        if (!in_range) {
            atomicOr(info, 1);
            continue;
        }
        if (g[0] == g[1] || g[0] == g[2] || g[0] == g[3] || g[1] == g[2] || g[1] == g[3] || g[2] == g[3]) {
            atomicOr(info, 2);
            continue;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) atomicAdd(cnt + g[k], 1);
    }
}

__global__ void hm_max_degree(const int32_t *start, int64_t nvert, int32_t *info) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvert; v += (int64_t)gridDim.x * blockDim.x)
        atomicMax(info + 1, start[v + 1] - start[v]);
}

__global__ void hm_fill(const int64_t *el, int64_t nelem, const int32_t *start, int32_t *cursor, int32_t *list) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelem; e += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t v = el[e * 4 + k];
            list[start[v] + atomicAdd(cursor + v, 1)] = (int32_t)e;
        }
}

// shared-memory bytes one warp needs for `cap` candidate edges and faces
__host__ __device__ inline size_t hm_warp_bytes(int cap) { return ((size_t)cap * 24 + 15) & ~(size_t)15; }

// warp per vertex v: the edges (v, w > v) and faces (v, b, c), v < b < c, of its elements. A
// candidate represents its entity when no other candidate of the entity comes from a smaller
// element; the rank of its other vertices among the representatives numbers the entity within
// v's. COUNT: per-vertex totals, used flag and smallest element. WRITE: every element's number
// for each of its local edges and faces that v owns, with the smallest-element mark.
template <bool WRITE>
__global__ void __launch_bounds__(HM_NT) hm_owned(const int64_t *el, int64_t nvert, int cap, int warps, HmWork w) {
    extern __shared__ __align__(16) unsigned char hm_smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t v = (int64_t)blockIdx.x * warps + wid;
    if (wid >= warps || v >= nvert) return;  // warp-uniform: no block-wide barrier follows
    unsigned char *base = hm_smem + (size_t)wid * hm_warp_bytes(cap);
    uint64_t *fkey = (uint64_t *)base;
    int32_t *ew = (int32_t *)(fkey + cap);
    int32_t *ee = ew + cap;
    int32_t *fe = ee + cap;
    uint8_t *erep = (uint8_t *)(fe + cap);
    uint8_t *frep = erep + cap;
    uint8_t *es = frep + cap;  // local edge of the candidate in its element
    uint8_t *fs = es + cap;    // local face

    const int s0 = w.cnt[v], deg = w.cnt[v + 1] - s0;
    int me = 0, mf = 0, emn = INT32_MAX;
    for (int t0 = 0; t0 < deg; t0 += 32) {
        const int t = t0 + lane;
        int ce = 0, cf = 0, e = -1;
        int ow[3] = {0, 0, 0}, os[3] = {0, 0, 0}, fsl[3] = {0, 0, 0};
        uint64_t of[3] = {0, 0, 0};
        if (t < deg) {
            e = w.list[s0 + t];
            emn = min(emn, e);
            int64_t o[3] = {0, 0, 0};
            int lo[3] = {0, 0, 0}, kv = 0, no = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int64_t g = el[(int64_t)e * 4 + k];
                if (g == v) {
                    kv = k;
                } else if (no < 3) {
                    o[no] = g;
                    lo[no] = k;
                    ++no;
                }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
                if (o[i] > v) {
                    ow[ce] = (int)o[i];
                    os[ce] = hm_edge_id(min(kv, lo[i]), max(kv, lo[i]));
                    ++ce;
                }
            const int pi[3] = {0, 0, 1}, pj[3] = {1, 2, 2}, px[3] = {2, 1, 0};
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                const int64_t b = o[pi[s]], c = o[pj[s]];
                if (b > v && c > v) {
                    of[cf] = ((uint64_t)min(b, c) << 32) | (uint64_t)max(b, c);
                    fsl[cf] = 3 - lo[px[s]];  // the face without local vertex m is face 3 - m
                    ++cf;
                }
            }
        }
        int ie = ce, jf = cf;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int te = __shfl_up_sync(0xffffffffu, ie, off), tf = __shfl_up_sync(0xffffffffu, jf, off);
            if (lane >= off) {
                ie += te;
                jf += tf;
            }
        }
        const int tot_e = __shfl_sync(0xffffffffu, ie, 31), tot_f = __shfl_sync(0xffffffffu, jf, 31);
        const int pe = me + ie - ce, pf = mf + jf - cf;
        for (int i = 0; i < ce; ++i) {
            ew[pe + i] = ow[i];
            ee[pe + i] = e;
            es[pe + i] = (uint8_t)os[i];
        }
        for (int i = 0; i < cf; ++i) {
            fkey[pf + i] = of[i];
            fe[pf + i] = e;
            fs[pf + i] = (uint8_t)fsl[i];
        }
        me += tot_e;
        mf += tot_f;
    }
    __syncwarp();
    int nrep_e = 0, nrep_f = 0;
    for (int i = lane; i < me; i += 32) {
        const int wi = ew[i], ei = ee[i];
        bool rep = true;
        for (int j = 0; j < me; ++j)
            if (ew[j] == wi && ee[j] < ei) {
                rep = false;
                break;
            }
        erep[i] = rep;
        nrep_e += rep;
    }
    for (int i = lane; i < mf; i += 32) {
        const uint64_t ki = fkey[i];
        const int ei = fe[i];
        bool rep = true;
        for (int j = 0; j < mf; ++j)
            if (fkey[j] == ki && fe[j] < ei) {
                rep = false;
                break;
            }
        frep[i] = rep;
        nrep_f += rep;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        nrep_e += __shfl_xor_sync(0xffffffffu, nrep_e, off);
        nrep_f += __shfl_xor_sync(0xffffffffu, nrep_f, off);
        emn = min(emn, __shfl_xor_sync(0xffffffffu, emn, off));
    }
    if (!WRITE) {
        if (lane == 0) {
            w.ecnt[v] = nrep_e;
            w.fcnt[v] = nrep_f;
            w.vrank[v] = deg > 0;
            w.vmin[v] = deg > 0 ? emn : -1;
        }
        return;
    }
    __syncwarp();
    const int64_t eb = w.ecnt[v], fb = w.fcnt[v];
    for (int i = lane; i < me; i += 32) {
        const int wi = ew[i];
        int r = 0;
        for (int j = 0; j < me; ++j) r += erep[j] && ew[j] < wi;
        w.eedge[(int64_t)ee[i] * 6 + es[i]] = ((eb + r) << 1) | (int64_t)erep[i];
    }
    for (int i = lane; i < mf; i += 32) {
        const uint64_t ki = fkey[i];
        int r = 0;
        for (int j = 0; j < mf; ++j) r += frep[j] && fkey[j] < ki;
        w.eface[(int64_t)fe[i] * 4 + fs[i]] = ((fb + r) << 1) | (int64_t)frep[i];
    }
}

// the weighted vertex sum of local node a (vertex order, separately rounded products and sums)
__device__ __forceinline__ void hm_position(const HmPattern &P, int a, const double *X, const int64_t *g,
                                            double *out) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double s = __dmul_rn(P.lam[a][0], X[g[0] * 3 + d]);
#pragma unroll
        for (int k = 1; k < 4; ++k) s = __dadd_rn(s, __dmul_rn(P.lam[a][k], X[g[k] * 3 + d]));
        out[d] = s;
    }
}

constexpr int HM_SLOTS = 15;  // per element: 4 vertices, 6 edges, 4 faces, the interior
constexpr int HM_TILE = 32;   // elements per tile: one lane each, one warp per slot

// CTA of HM_SLOTS warps per tile of 32 elements: warp `slot` numbers the local nodes of that
// entity (vertex 0-3, edge 0-5, face 0-3, interior) in each lane's element, so every read of the
// layout table is warp-uniform; positions are written where the element is the smallest holding
// the entity; the tile's element rows are gathered in shared memory and stored contiguously.
__global__ void __launch_bounds__(HM_SLOTS * 32) hm_nodes(const double *X, const int64_t *el, int64_t nelem,
                                                          const __grid_constant__ HmPattern P, HmWork w,
                                                          int64_t nv, int64_t nedge, int64_t nface, double *outX,
                                                          int64_t *outE) {
    __shared__ int64_t rows[HM_TILE * HM_MAX_NPE];
    const int slot = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t base_e = nv, base_f = nv + nedge * P.ne, base_i = base_f + nface * P.nf;
    for (int64_t t0 = (int64_t)blockIdx.x * HM_TILE; t0 < nelem; t0 += (int64_t)gridDim.x * HM_TILE) {
        const int64_t e = t0 + lane;
        int64_t *row = rows + lane * P.npe;
        if (e < nelem) {
            int64_t g[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) g[k] = el[e * 4 + k];
            if (slot < 4) {
                const int64_t v = g[slot];
                const int a = P.vnode[slot];
                const int64_t id = w.vrank[v];
                row[a] = id;
                if (w.vmin[v] == (int32_t)e) hm_position(P, a, X, g, outX + id * 3);
            } else if (slot < 10) {
                const int s = slot - 4;
                const int64_t code = w.eedge[e * 6 + s];
                const bool fwd = g[TET_EDGES_D[s][0]] < g[TET_EDGES_D[s][1]];
                for (int t = 0; t < P.ne; ++t) {
                    const int a = P.enode[s][t];
                    const int qa = fwd ? P.q[a][0] : P.q[a][1];
                    int r = 0;
                    for (int i = 0; i < P.ne; ++i)
                        if (P.qe[i] == qa) r = i;
                    const int64_t id = base_e + (code >> 1) * P.ne + r;
                    row[a] = id;
                    if (code & 1) hm_position(P, a, X, g, outX + id * 3);
                }
            } else if (slot < 14) {
                const int s = slot - 10;
                const int64_t code = w.eface[e * 4 + s];
                const int64_t g0 = g[TET_FACES_D[s][0]], g1 = g[TET_FACES_D[s][1]], g2 = g[TET_FACES_D[s][2]];
                // rank in increasing global order of each of the face's three local vertices
                const int r0 = (g0 > g1) + (g0 > g2), r1 = (g1 > g0) + (g1 > g2), r2 = (g2 > g0) + (g2 > g1);
                for (int t = 0; t < P.nf; ++t) {
                    const int a = P.fnode[s][t];
                    int qs[3];
                    qs[r0] = P.q[a][0];
                    qs[r1] = P.q[a][1];
                    qs[r2] = P.q[a][2];
                    int r = 0;
                    for (int i = 0; i < P.nf; ++i)
                        if (P.qf[i][0] == qs[0] && P.qf[i][1] == qs[1]) r = i;
                    const int64_t id = base_f + (code >> 1) * P.nf + r;
                    row[a] = id;
                    if (code & 1) hm_position(P, a, X, g, outX + id * 3);
                }
            } else {
                for (int t = 0; t < P.ni; ++t) {
                    const int a = P.inode[t];
                    const int64_t id = base_i + e * P.ni + t;
                    row[a] = id;
                    hm_position(P, a, X, g, outX + id * 3);
                }
            }
        }
        __syncthreads();
        const int n = (int)min((int64_t)HM_TILE, nelem - t0) * P.npe;
        for (int i = threadIdx.x; i < n; i += blockDim.x) outE[t0 * P.npe + i] = rows[i];
        __syncthreads();
    }
}

static unsigned hm_grid(int64_t n, int threads) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16));
}

static int raise_tet_order(const double *X, int64_t nvert, const int64_t *el, int64_t nelem, const double *pattern,
                           int64_t npe, double *outX, int64_t cap_points, int64_t *nnode_out, int64_t *outE,
                           void *workspace, size_t ws_bytes, cudaStream_t s) {
    if (!X || !el || !pattern || !nnode_out || !outE || !workspace || nelem <= 0 || nvert <= 0) return FL_ERR_ARG;
    if (nelem > INT32_MAX || nvert >= INT32_MAX) return FL_ERR_UNSUPPORTED;
    HmPattern P;
    const int pst = classify_pattern(pattern, npe, &P);
    if (pst != FL_OK) return pst;
    if (hm_layout(nelem, nvert, nullptr, nullptr) > ws_bytes) return FL_ERR_CAPACITY;
    HmWork w;
    hm_layout(nelem, nvert, &w, (char *)workspace);
    FL_CUDA_TRY(cudaMemsetAsync(w.cnt, 0, sizeof(int32_t) * (nvert + 1), s));
    FL_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, sizeof(int32_t) * nvert, s));
    FL_CUDA_TRY(cudaMemsetAsync(w.info, 0, sizeof(int32_t) * 4, s));
    hm_count<<<hm_grid(nelem, 256), 256, 0, s>>>(el, nelem, nvert, w.cnt, w.info);
    exclusive_scan<int32_t, int32_t>(w.cnt, w.cnt, nvert + 1, w.bsum, s);
    hm_max_degree<<<hm_grid(nvert, 256), 256, 0, s>>>(w.cnt, nvert, w.info);
    int32_t hinfo[4];
    FL_CUDA_TRY(cudaMemcpyAsync(hinfo, w.info, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    if (hinfo[0] & 1) return FL_ERR_ARG;   // vertex id out of range
    if (hinfo[0] & 2) return FL_ERR_MESH;  // an element repeats a vertex
    const int cap = std::max(1, 3 * hinfo[1]);
    const size_t per_warp = hm_warp_bytes(cap);
    const size_t smem_budget = 96 * 1024;
    if (per_warp > 200 * 1024) return FL_ERR_UNSUPPORTED;  // a vertex in more than ~2800 elements
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(HM_NT / 32, smem_budget / per_warp));
    const size_t smem = per_warp * warps;
    if (smem > 48 * 1024) {
        FL_CUDA_TRY(cudaFuncSetAttribute(hm_owned<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FL_CUDA_TRY(cudaFuncSetAttribute(hm_owned<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    hm_fill<<<hm_grid(nelem, 256), 256, 0, s>>>(el, nelem, w.cnt, w.cursor, w.list);
    const unsigned gv = (unsigned)((nvert + warps - 1) / warps);
    hm_owned<false><<<gv, 32 * warps, smem, s>>>(el, nvert, cap, warps, w);
    FL_CUDA_TRY(cudaMemsetAsync(w.vrank + nvert, 0, sizeof(int64_t), s));
    FL_CUDA_TRY(cudaMemsetAsync(w.ecnt + nvert, 0, sizeof(int64_t), s));
    FL_CUDA_TRY(cudaMemsetAsync(w.fcnt + nvert, 0, sizeof(int64_t), s));
    exclusive_scan<int64_t, int64_t>(w.vrank, w.vrank, nvert + 1, w.bsum, s);
    exclusive_scan<int64_t, int64_t>(w.ecnt, w.ecnt, nvert + 1, w.bsum, s);
    exclusive_scan<int64_t, int64_t>(w.fcnt, w.fcnt, nvert + 1, w.bsum, s);
    int64_t tot[3];
    FL_CUDA_TRY(cudaMemcpyAsync(tot + 0, w.vrank + nvert, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaMemcpyAsync(tot + 1, w.ecnt + nvert, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaMemcpyAsync(tot + 2, w.fcnt + nvert, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    const int64_t nnode = tot[0] + tot[1] * P.ne + tot[2] * P.nf + nelem * P.ni;
    *nnode_out = nnode;
    if (!outX || cap_points < nnode) return FL_ERR_CAPACITY;
    hm_owned<true><<<gv, 32 * warps, smem, s>>>(el, nvert, cap, warps, w);
    const unsigned gn = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((nelem + HM_TILE - 1) / HM_TILE, 152 * 8));
    hm_nodes<<<gn, HM_SLOTS * 32, 0, s>>>(X, el, nelem, P, w, tot[0], tot[1], tot[2], outX, outE);
    return launch_status();
}

}  // namespace fl

extern "C" {

int fl_TetNodeLayout(const double *pattern, int64_t nodeperelem, int64_t *counts) {
    if (!counts) return FL_ERR_ARG;
    fl::HmPattern P;
    const int st = fl::classify_pattern(pattern, nodeperelem, &P);
    if (st != FL_OK) return st;
    counts[0] = P.ne;
    counts[1] = P.nf;
    counts[2] = P.ni;
    return FL_OK;
}

size_t fl_RaiseTetOrder_workspace_size(int64_t nelem, int64_t nvert) {
    return fl::hm_layout(nelem, nvert, nullptr, nullptr);
}

int fl_RaiseTetOrder(const double *points, int64_t nvert, const int64_t *elements, int64_t nelem,
                     const double *pattern, int64_t nodeperelem, double *out_points, int64_t points_capacity,
                     int64_t *nnode, int64_t *out_elements, void *workspace, size_t workspace_bytes,
                     fl_stream_t stream) {
    return fl::raise_tet_order(points, nvert, elements, nelem, pattern, nodeperelem, out_points, points_capacity,
                               nnode, out_elements, workspace, workspace_bytes, (cudaStream_t)stream);
}

}  // extern "C"
