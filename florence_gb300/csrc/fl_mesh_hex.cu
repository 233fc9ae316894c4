// fl_mesh_hex.cu -- device generation of a high-order hex mesh from a linear one: the node placement
// and duplicate removal that Mesh.GetHighOrderMesh does for hexes
// (Florence/MeshGeneration/Mesh.py:1388-1389 -> HighOrderMeshHex,
//  HigherOrderMeshing/HigherOrderMeshingHex.py:19-135).
//
// The reference places every element's non-vertex nodes at the trilinear map of the reference
// element's node layout and then merges coincident points by rounding their coordinates and
// sorting them. Here, as for tets (fl_mesh.cu), the merge is topological: a local node belongs to
// the vertices whose trilinear weight is nonzero (1 vertex, 2 an edge, 4 a face, 8 the interior),
// and two elements' nodes on a shared edge or face are the same node when their weights, listed
// in increasing global-vertex order, are the same. The numbering is the lexicographic order of
// the keys (entity size, global vertices ascending, weights in that order): vertices first, then
// edges, faces and element interiors, which the host builder (florence_gb300/meshes.py,
// raise_hex_order) also produces, so the two agree node for node. The result is the reference's
// mesh up to a permutation of the node numbers.
//
// Steps: per-vertex incidence lists (counts, scan, fill); a warp per vertex collects the edges
// (v, w > v) and the faces whose smallest vertex is v from its elements, removes repeats and ranks
// the distinct ones in shared memory, once to count and, after scans of the counts, once to write
// into every element the number of each of its local edges and faces, marked where the element is
// the smallest one holding the entity; a CTA per tile of 32 elements, one warp per entity slot (8
// vertices, 12 edges, 6 faces, the interior), then numbers the local nodes and -- in the marked
// element only, so that exactly one thread writes each node -- computes their positions.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fl_common.cuh"
#include "fl_scan.cuh"

namespace fl {

constexpr int HX_MAX_NPE = 125;  // up to p = 4
constexpr int HX_MAX_EDGE = 3;   // nodes inside one edge
constexpr int HX_MAX_FACE = 9;   // nodes inside one face
constexpr double HX_NZ_TOL = 1e-10;
constexpr double HX_QSCALE = 1e6;
constexpr int HX_NT = 256;

// local node layout of the high-order hex, classified on the host (the first 8 local nodes are the
// vertices, in the order of the linear element's columns)
struct HxPattern {
    int npe, ne, nf, ni;
    double w[HX_MAX_NPE][8];   // trilinear weights of the local nodes at the 8 vertices
    int q[HX_MAX_NPE][8];      // the same rounded to 1e-6 (0 where the weight is zero)
    int edge_v[12][2];         // local vertices of each edge
    int face_v[6][4];          // local vertices of each face (cyclic order)
    int vedge[8][3];           // the 3 edges at each vertex
    int vface[8][3];           // the 3 faces at each vertex
    int enode[12][HX_MAX_EDGE];
    int fnode[6][HX_MAX_FACE];
    int inode[HX_MAX_NPE];
};

// FL_OK, or FL_ERR_UNSUPPORTED when the layout is not one that shared entities can number
// consistently from either side
static int classify_hex_pattern(const double *xi, int64_t npe, HxPattern *P) {
    if (!xi || npe < 8) return FL_ERR_ARG;
    if (npe > HX_MAX_NPE) return FL_ERR_UNSUPPORTED;
    *P = HxPattern{};
    P->npe = (int)npe;
    int sg[8][3];
    for (int k = 0; k < 8; ++k)
        for (int d = 0; d < 3; ++d) {
            const double v = xi[k * 3 + d];
            if (!std::isfinite(v) || std::fabs(std::fabs(v) - 1.0) > 1e-9) return FL_ERR_UNSUPPORTED;
            sg[k][d] = v > 0 ? 1 : -1;
        }
    for (int k = 0; k < 8; ++k)
        for (int j = 0; j < k; ++j)
            if (sg[j][0] == sg[k][0] && sg[j][1] == sg[k][1] && sg[j][2] == sg[k][2]) return FL_ERR_UNSUPPORTED;
    // edges: vertex pairs that differ in one sign; faces: the 4 vertices sharing one sign
    int ne = 0;
    for (int a = 0; a < 8; ++a)
        for (int b = a + 1; b < 8; ++b) {
            int diff = 0;
            for (int d = 0; d < 3; ++d) diff += sg[a][d] != sg[b][d];
            if (diff == 1) {
                P->edge_v[ne][0] = a;
                P->edge_v[ne][1] = b;
                ++ne;
            }
        }
    int nf = 0;
    for (int d = 0; d < 3; ++d)
        for (int s = -1; s <= 1; s += 2) {
            int vs[4], n = 0;
            for (int k = 0; k < 8; ++k)
                if (sg[k][d] == s) vs[n++] = k;
            // cyclic order in the face's plane: (-,-), (+,-), (+,+), (-,+) of its two free signs
            const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
            const int want[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
            for (int c = 0; c < 4; ++c)
                for (int i = 0; i < 4; ++i)
                    if (sg[vs[i]][d1] == want[c][0] && sg[vs[i]][d2] == want[c][1]) P->face_v[nf][c] = vs[i];
            ++nf;
        }
    for (int k = 0; k < 8; ++k) {
        int ce = 0, cf = 0;
        for (int s = 0; s < 12; ++s)
            if (P->edge_v[s][0] == k || P->edge_v[s][1] == k) P->vedge[k][ce++] = s;
        for (int f = 0; f < 6; ++f)
            for (int c = 0; c < 4; ++c)
                if (P->face_v[f][c] == k) P->vface[k][cf++] = f;
        if (ce != 3 || cf != 3) return FL_ERR_UNSUPPORTED;
    }
    // weights and kinds
    int cnt_e[12] = {}, cnt_f[6] = {}, nint = 0;
    for (int a = 0; a < npe; ++a) {
        int nz = 0, vs[8];
        for (int k = 0; k < 8; ++k) {
            double w = 1.0;
            for (int d = 0; d < 3; ++d) {
                const double x = xi[a * 3 + d];
                if (!std::isfinite(x)) return FL_ERR_ARG;
                w *= 0.5 * (1.0 + sg[k][d] * x);
            }
            if (std::fabs(w) <= HX_NZ_TOL) w = 0.0;
            P->w[a][k] = w;
            P->q[a][k] = (int)std::nearbyint(w * HX_QSCALE);
            if (w != 0.0) vs[nz++] = k;
        }
        if (a < 8) {
            if (nz != 1 || vs[0] != a) return FL_ERR_UNSUPPORTED;  // the vertices come first, in order
            continue;
        }
        if (nz == 2) {
            int s = -1;
            for (int t = 0; t < 12; ++t)
                if (P->edge_v[t][0] == vs[0] && P->edge_v[t][1] == vs[1]) s = t;
            if (s < 0 || cnt_e[s] >= HX_MAX_EDGE) return FL_ERR_UNSUPPORTED;
            P->enode[s][cnt_e[s]++] = a;
        } else if (nz == 4) {
            int f = -1;
            for (int t = 0; t < 6; ++t) {
                int hit = 0;
                for (int c = 0; c < 4; ++c)
                    for (int i = 0; i < 4; ++i) hit += P->face_v[t][c] == vs[i];
                if (hit == 4) f = t;
            }
            if (f < 0 || cnt_f[f] >= HX_MAX_FACE) return FL_ERR_UNSUPPORTED;
            P->fnode[f][cnt_f[f]++] = a;
        } else if (nz == 8) {
            P->inode[nint++] = a;
        } else {
            return FL_ERR_UNSUPPORTED;  // a node that is neither on a vertex, an edge, a face nor inside
        }
    }
    for (int s = 1; s < 12; ++s)
        if (cnt_e[s] != cnt_e[0]) return FL_ERR_UNSUPPORTED;
    for (int f = 1; f < 6; ++f)
        if (cnt_f[f] != cnt_f[0]) return FL_ERR_UNSUPPORTED;
    P->ne = cnt_e[0];
    P->nf = cnt_f[0];
    P->ni = nint;
    // symmetry: the weight pairs of an edge's nodes are closed under swapping its ends, and the
    // weight 4-tuples of a face's nodes (cyclic order) under the square's eight symmetries, with no
    // two nodes of an entity alike -- otherwise two elements could disagree about a shared node
    for (int s = 0; s < 12; ++s) {
        std::vector<std::pair<int, int>> set;
        for (int t = 0; t < P->ne; ++t) {
            const int a = P->enode[s][t];
            set.push_back({P->q[a][P->edge_v[s][0]], P->q[a][P->edge_v[s][1]]});
        }
        std::sort(set.begin(), set.end());
        if (std::adjacent_find(set.begin(), set.end()) != set.end()) return FL_ERR_UNSUPPORTED;
        for (auto &p : set)
            if (!std::binary_search(set.begin(), set.end(), std::make_pair(p.second, p.first))) return FL_ERR_UNSUPPORTED;
    }
    for (int f = 0; f < 6; ++f) {
        std::vector<std::vector<int>> set;
        for (int t = 0; t < P->nf; ++t) {
            const int a = P->fnode[f][t];
            std::vector<int> v(4);
            for (int c = 0; c < 4; ++c) v[c] = P->q[a][P->face_v[f][c]];
            set.push_back(v);
        }
        std::sort(set.begin(), set.end());
        if (std::adjacent_find(set.begin(), set.end()) != set.end()) return FL_ERR_UNSUPPORTED;
        for (auto &v : set)
            for (int r = 0; r < 4; ++r)
                for (int m = 0; m < 2; ++m) {  // rotation by r, mirrored when m
                    std::vector<int> u(4);
                    for (int c = 0; c < 4; ++c) u[c] = v[m ? (4 - c + r) % 4 : (c + r) % 4];
                    if (!std::binary_search(set.begin(), set.end(), u)) return FL_ERR_UNSUPPORTED;
                }
    }
    return FL_OK;
}

struct HxWork {
    int32_t *cnt;     // [nvert+1] incidence counts, then their exclusive scan (list starts)
    int32_t *cursor;  // [nvert]
    int32_t *list;    // [8*nelem] elements holding each vertex
    int32_t *vmin;    // [nvert] smallest element holding the vertex (-1: unused)
    int64_t *vrank;   // [nvert+1] used flags, then the node numbers of the used vertices
    int64_t *ecnt;    // [nvert+1] distinct edges each vertex owns, then the first edge number of each
    int64_t *fcnt;    // [nvert+1] distinct faces each vertex owns, then the first face number of each
    int64_t *eedge;   // [12*nelem] edge number << 1 | (this element is the smallest holding it)
    int64_t *eface;   // [6*nelem] face number << 1 | (this element is the smallest holding it)
    int64_t *bsum;    // scan block sums
    int32_t *info;    // [4]: error bits (1 vertex id out of range, 2 repeated vertex), maximum degree
};

static size_t hx_align(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t hx_layout(int64_t nelem, int64_t nvert, HxWork *w, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += hx_align(bytes);
        return p;
    };
    const int64_t nb = (nvert + 1 + SCAN_ITEMS - 1) / SCAN_ITEMS + 1;
    HxWork t;
    t.cnt = (int32_t *)take(sizeof(int32_t) * (nvert + 1));
    t.cursor = (int32_t *)take(sizeof(int32_t) * nvert);
    t.list = (int32_t *)take(sizeof(int32_t) * 8 * nelem);
    t.vmin = (int32_t *)take(sizeof(int32_t) * nvert);
    t.vrank = (int64_t *)take(sizeof(int64_t) * (nvert + 1));
    t.ecnt = (int64_t *)take(sizeof(int64_t) * (nvert + 1));
    t.fcnt = (int64_t *)take(sizeof(int64_t) * (nvert + 1));
    t.eedge = (int64_t *)take(sizeof(int64_t) * 12 * nelem);
    t.eface = (int64_t *)take(sizeof(int64_t) * 6 * nelem);
    t.bsum = (int64_t *)take(sizeof(int64_t) * (nb + SCAN_ITEMS));
    t.info = (int32_t *)take(sizeof(int32_t) * 4);
    if (w) *w = t;
    return off;
}

__global__ void hx_count(const int64_t *el, int64_t nelem, int64_t nvert, int32_t *cnt, int32_t *info) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelem; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t g[8];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            g[k] = el[e * 8 + k];
            ok &= g[k] >= 0 && g[k] < nvert;
        }
        if (!ok) {
            atomicOr(info, 1);
            continue;
        }
        bool rep = false;
#pragma unroll
        for (int k = 0; k < 8; ++k)
#pragma unroll
            for (int j = 0; j < k; ++j) rep |= g[j] == g[k];
        if (rep) {
            atomicOr(info, 2);
            continue;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) atomicAdd(cnt + g[k], 1);
    }
}

__global__ void hx_max_degree(const int32_t *start, int64_t nvert, int32_t *info) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvert; v += (int64_t)gridDim.x * blockDim.x)
        atomicMax(info + 1, start[v + 1] - start[v]);
}

__global__ void hx_fill(const int64_t *el, int64_t nelem, const int32_t *start, int32_t *cursor, int32_t *list) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelem; e += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int64_t v = el[e * 8 + k];
            list[start[v] + atomicAdd(cursor + v, 1)] = (int32_t)e;
        }
}

// shared-memory bytes one warp needs for `cap` candidate edges and `cap` candidate faces
__host__ __device__ inline size_t hx_warp_bytes(int cap) { return ((size_t)cap * 30 + 15) & ~(size_t)15; }

__device__ __forceinline__ bool hx_less3(const int32_t *a, const int32_t *b) {
    return a[0] != b[0] ? a[0] < b[0] : a[1] != b[1] ? a[1] < b[1] : a[2] < b[2];
}

// warp per vertex v: the edges (v, w > v) and the faces whose smallest vertex is v (keyed by their
// other three vertices, ascending) of v's elements. A candidate represents its entity when no other
// candidate of the entity comes from a smaller element; the rank of its key among the
// representatives numbers the entity within v's. COUNT: per-vertex totals, used flag, smallest
// element. WRITE: every element's number for each of its local edges and faces that v owns, with
// the smallest-element mark.
template <bool WRITE>
__global__ void __launch_bounds__(HX_NT) hx_owned(const int64_t *el, int64_t nvert, int cap, int warps,
                                                  const __grid_constant__ HxPattern P, HxWork w) {
    extern __shared__ __align__(16) unsigned char hx_smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t v = (int64_t)blockIdx.x * warps + wid;
    if (wid >= warps || v >= nvert) return;  // warp-uniform: no block-wide barrier follows
    unsigned char *base = hx_smem + (size_t)wid * hx_warp_bytes(cap);
    int32_t *fk = (int32_t *)base;  // [3 cap] face keys
    int32_t *ew = fk + 3 * cap;     // [cap] edge keys
    int32_t *ee = ew + cap;         // [cap] element of the edge candidate
    int32_t *fe = ee + cap;         // [cap] element of the face candidate
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
        int32_t fkey[3][3] = {};
        if (t < deg) {
            e = w.list[s0 + t];
            emn = min(emn, e);
            int64_t g[8];
            int kv = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                g[k] = el[(int64_t)e * 8 + k];
                if (g[k] == v) kv = k;
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int s = P.vedge[kv][i];
                const int ko = P.edge_v[s][0] == kv ? P.edge_v[s][1] : P.edge_v[s][0];
                if (g[ko] > v) {
                    ow[ce] = (int)g[ko];
                    os[ce] = s;
                    ++ce;
                }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int f = P.vface[kv][i];
                int32_t o[3];
                int no = 0;
                bool owner = true;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int64_t gc = g[P.face_v[f][c]];
                    if (gc == v) continue;
                    owner &= gc > v;
                    if (no < 3) o[no++] = (int32_t)gc;
                }
                if (owner && no == 3) {
                    // the other three vertices ascending
                    if (o[0] > o[1]) { const int32_t x = o[0]; o[0] = o[1]; o[1] = x; }
                    if (o[1] > o[2]) { const int32_t x = o[1]; o[1] = o[2]; o[2] = x; }
                    if (o[0] > o[1]) { const int32_t x = o[0]; o[0] = o[1]; o[1] = x; }
                    fkey[cf][0] = o[0];
                    fkey[cf][1] = o[1];
                    fkey[cf][2] = o[2];
                    fsl[cf] = f;
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
            fk[3 * (pf + i)] = fkey[i][0];
            fk[3 * (pf + i) + 1] = fkey[i][1];
            fk[3 * (pf + i) + 2] = fkey[i][2];
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
        const int32_t *ki = fk + 3 * i;
        const int ei = fe[i];
        bool rep = true;
        for (int j = 0; j < mf; ++j) {
            const int32_t *kj = fk + 3 * j;
            if (kj[0] == ki[0] && kj[1] == ki[1] && kj[2] == ki[2] && fe[j] < ei) {
                rep = false;
                break;
            }
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
        w.eedge[(int64_t)ee[i] * 12 + es[i]] = ((eb + r) << 1) | (int64_t)erep[i];
    }
    for (int i = lane; i < mf; i += 32) {
        const int32_t *ki = fk + 3 * i;
        int r = 0;
        for (int j = 0; j < mf; ++j) r += frep[j] && hx_less3(fk + 3 * j, ki);
        w.eface[(int64_t)fe[i] * 6 + fs[i]] = ((fb + r) << 1) | (int64_t)frep[i];
    }
}

// the weighted vertex sum of local node a (vertex order, separately rounded products and sums)
__device__ __forceinline__ void hx_position(const HxPattern &P, int a, const double *X, const int64_t *g,
                                            double *out) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double s = __dmul_rn(P.w[a][0], X[g[0] * 3 + d]);
#pragma unroll
        for (int k = 1; k < 8; ++k) s = __dadd_rn(s, __dmul_rn(P.w[a][k], X[g[k] * 3 + d]));
        out[d] = s;
    }
}

constexpr int HX_SLOTS = 27;  // per element: 8 vertices, 12 edges, 6 faces, the interior
constexpr int HX_TILE = 32;   // elements per tile: one lane each, one warp per slot

// CTA of HX_SLOTS warps per tile of 32 elements: warp `slot` numbers the local nodes of that entity
// in each lane's element (every read of the layout table warp-uniform); positions are written where
// the element is the smallest holding the entity; the tile's element rows are gathered in shared
// memory and stored contiguously. Within an edge or face, a node's number is the rank of its
// weights, listed in increasing global-vertex order, among those of the entity's nodes.
__global__ void __launch_bounds__(HX_SLOTS * 32) hx_nodes(const double *X, const int64_t *el, int64_t nelem,
                                                          const __grid_constant__ HxPattern P, HxWork w, int64_t nv,
                                                          int64_t nedge, int64_t nface, double *outX, int64_t *outE) {
    __shared__ int64_t rows[HX_TILE * HX_MAX_NPE];
    const int slot = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t base_e = nv, base_f = nv + nedge * P.ne, base_i = base_f + nface * P.nf;
    for (int64_t t0 = (int64_t)blockIdx.x * HX_TILE; t0 < nelem; t0 += (int64_t)gridDim.x * HX_TILE) {
        const int64_t e = t0 + lane;
        int64_t *row = rows + lane * P.npe;
        if (e < nelem) {
            int64_t g[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) g[k] = el[e * 8 + k];
            if (slot < 8) {
                const int64_t v = g[slot];
                const int64_t id = w.vrank[v];
                row[slot] = id;
                if (w.vmin[v] == (int32_t)e) hx_position(P, slot, X, g, outX + id * 3);
            } else if (slot < 20) {
                const int s = slot - 8;
                const int64_t code = w.eedge[e * 12 + s];
                const int l0 = P.edge_v[s][0], l1 = P.edge_v[s][1];
                const int lo = g[l0] < g[l1] ? l0 : l1, hi = lo == l0 ? l1 : l0;
                for (int t = 0; t < P.ne; ++t) {
                    const int a = P.enode[s][t];
                    const int qa = P.q[a][lo], qb = P.q[a][hi];
                    int r = 0;
                    for (int u = 0; u < P.ne; ++u) {
                        const int b = P.enode[s][u];
                        const int pa = P.q[b][lo], pb = P.q[b][hi];
                        r += pa < qa || (pa == qa && pb < qb);
                    }
                    const int64_t id = base_e + (code >> 1) * P.ne + r;
                    row[a] = id;
                    if (code & 1) hx_position(P, a, X, g, outX + id * 3);
                }
            } else if (slot < 26) {
                const int f = slot - 20;
                const int64_t code = w.eface[e * 6 + f];
                // the face's local vertices in increasing global order
                int ord[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int lc = P.face_v[f][c];
                    int r = 0;
#pragma unroll
                    for (int c2 = 0; c2 < 4; ++c2) r += g[P.face_v[f][c2]] < g[lc];
                    ord[r] = lc;
                }
                for (int t = 0; t < P.nf; ++t) {
                    const int a = P.fnode[f][t];
                    int r = 0;
                    for (int u = 0; u < P.nf; ++u) {
                        const int b = P.fnode[f][u];
                        int cmp = 0;  // tuple(b) < tuple(a) ?
#pragma unroll
                        for (int c = 0; c < 4; ++c)
                            if (cmp == 0 && P.q[b][ord[c]] != P.q[a][ord[c]]) cmp = P.q[b][ord[c]] < P.q[a][ord[c]] ? 1 : 2;
                        r += cmp == 1;
                    }
                    const int64_t id = base_f + (code >> 1) * P.nf + r;
                    row[a] = id;
                    if (code & 1) hx_position(P, a, X, g, outX + id * 3);
                }
            } else {
                for (int t = 0; t < P.ni; ++t) {
                    const int a = P.inode[t];
                    const int64_t id = base_i + e * P.ni + t;
                    row[a] = id;
                    hx_position(P, a, X, g, outX + id * 3);
                }
            }
        }
        __syncthreads();
        const int n = (int)min((int64_t)HX_TILE, nelem - t0) * P.npe;
        for (int i = threadIdx.x; i < n; i += blockDim.x) outE[t0 * P.npe + i] = rows[i];
        __syncthreads();
    }
}

static unsigned hx_grid(int64_t n, int threads) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16));
}

static int raise_hex_order(const double *X, int64_t nvert, const int64_t *el, int64_t nelem, const double *pattern,
                           int64_t npe, double *outX, int64_t cap_points, int64_t *nnode_out, int64_t *outE,
                           void *workspace, size_t ws_bytes, cudaStream_t s) {
    if (!X || !el || !pattern || !nnode_out || !outE || !workspace || nelem <= 0 || nvert <= 0) return FL_ERR_ARG;
    if (nelem > INT32_MAX / 8 || nvert >= INT32_MAX) return FL_ERR_UNSUPPORTED;
    HxPattern P;
    const int pst = classify_hex_pattern(pattern, npe, &P);
    if (pst != FL_OK) return pst;
    if (hx_layout(nelem, nvert, nullptr, nullptr) > ws_bytes) return FL_ERR_CAPACITY;
    HxWork w;
    hx_layout(nelem, nvert, &w, (char *)workspace);
    FL_CUDA_TRY(cudaMemsetAsync(w.cnt, 0, sizeof(int32_t) * (nvert + 1), s));
    FL_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, sizeof(int32_t) * nvert, s));
    FL_CUDA_TRY(cudaMemsetAsync(w.info, 0, sizeof(int32_t) * 4, s));
    hx_count<<<hx_grid(nelem, 256), 256, 0, s>>>(el, nelem, nvert, w.cnt, w.info);
    exclusive_scan<int32_t, int32_t>(w.cnt, w.cnt, nvert + 1, w.bsum, s);
    hx_max_degree<<<hx_grid(nvert, 256), 256, 0, s>>>(w.cnt, nvert, w.info);
    int32_t hinfo[4];
    FL_CUDA_TRY(cudaMemcpyAsync(hinfo, w.info, sizeof(hinfo), cudaMemcpyDeviceToHost, s));
    FL_CUDA_TRY(cudaStreamSynchronize(s));
    if (hinfo[0] & 1) return FL_ERR_ARG;   // vertex id out of range
    if (hinfo[0] & 2) return FL_ERR_MESH;  // an element repeats a vertex
    const int cap = std::max(1, 3 * hinfo[1]);
    const size_t per_warp = hx_warp_bytes(cap);
    const size_t smem_budget = 96 * 1024;
    if (per_warp > 200 * 1024) return FL_ERR_UNSUPPORTED;  // a vertex in more than ~2 000 elements
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(HX_NT / 32, smem_budget / per_warp));
    const size_t smem = per_warp * warps;
    if (smem > 48 * 1024) {
        FL_CUDA_TRY(cudaFuncSetAttribute(hx_owned<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FL_CUDA_TRY(cudaFuncSetAttribute(hx_owned<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    hx_fill<<<hx_grid(nelem, 256), 256, 0, s>>>(el, nelem, w.cnt, w.cursor, w.list);
    const unsigned gv = (unsigned)((nvert + warps - 1) / warps);
    hx_owned<false><<<gv, 32 * warps, smem, s>>>(el, nvert, cap, warps, P, w);
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
    hx_owned<true><<<gv, 32 * warps, smem, s>>>(el, nvert, cap, warps, P, w);
    const unsigned gn = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nelem + HX_TILE - 1) / HX_TILE, 152 * 4));
    hx_nodes<<<gn, HX_SLOTS * 32, 0, s>>>(X, el, nelem, P, w, tot[0], tot[1], tot[2], outX, outE);
    return launch_status();
}

}  // namespace fl

extern "C" {

int fl_HexNodeLayout(const double *pattern, int64_t nodeperelem, int64_t *counts) {
    if (!counts) return FL_ERR_ARG;
    fl::HxPattern P;
    const int st = fl::classify_hex_pattern(pattern, nodeperelem, &P);
    if (st != FL_OK) return st;
    counts[0] = P.ne;
    counts[1] = P.nf;
    counts[2] = P.ni;
    return FL_OK;
}

size_t fl_RaiseHexOrder_workspace_size(int64_t nelem, int64_t nvert) {
    return fl::hx_layout(nelem, nvert, nullptr, nullptr);
}

int fl_RaiseHexOrder(const double *points, int64_t nvert, const int64_t *elements, int64_t nelem,
                     const double *pattern, int64_t nodeperelem, double *out_points, int64_t points_capacity,
                     int64_t *nnode, int64_t *out_elements, void *workspace, size_t workspace_bytes,
                     fl_stream_t stream) {
    return fl::raise_hex_order(points, nvert, elements, nelem, pattern, nodeperelem, out_points, points_capacity,
                               nnode, out_elements, workspace, workspace_bytes, (cudaStream_t)stream);
}

}  // extern "C"
