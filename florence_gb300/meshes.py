"""Synthetic mesh builders for benchmarks and tests (host numpy, seeded).

Florence builds high-order meshes with its own generators (Mesh.Cube/Parallelepiped +
GetHighOrderMesh, Florence/MeshGeneration/Mesh.py:1339-1410, :5843-5921). The assembly kernels
only need the element's local node layout to match the function-space tables (Jm) they are
given, so these builders take that layout from one reference element (``local_pattern``) and
replicate it over larger meshes:

* ``structured_hex``: nx x ny x nz grid of hexes of order p on a box;
* ``jittered_tet_beam``: seeded jittered lattice split by scipy's Delaunay, reoriented to
  positive volume, raised to order p with the pattern's barycentric node positions.

Global node numbering differs from Florence's; the assembled operator is the same up to that
permutation.
"""
import numpy as np


def local_pattern(points, elements, e=0, element_type="hex"):
    """Reference coordinates of the local nodes of element e.
    hex: [npe,3] in [-1,1]^3 from the element's bounding box (axis-aligned elements only);
    tet: [npe,4] barycentric coordinates with respect to the first four (vertex) nodes."""
    X = np.asarray(points)[np.asarray(elements)[e].astype(np.int64)]
    if element_type == "hex":
        lo, hi = X.min(0), X.max(0)
        return 2.0 * (X - lo) / (hi - lo) - 1.0
    V = X[:4]
    A = np.vstack([V.T, np.ones(4)])
    rhs = np.vstack([X.T, np.ones(len(X))])
    return np.linalg.solve(A, rhs).T


def structured_hex(n, L, pattern):
    """Hex mesh of n = (nx, ny, nz) elements on [0,L0]x[0,L1]x[0,L2] with the node layout `pattern`."""
    nx, ny, nz = n
    pat = np.asarray(pattern)
    u = [np.unique(np.round(pat[:, d], 12)) for d in range(3)]
    p = len(u[0]) - 1
    k = np.stack([np.searchsorted(u[d], np.round(pat[:, d], 12)) for d in range(3)], 1)  # [npe,3] 1-D index
    G = [n_ * p + 1 for n_ in (nx, ny, nz)]
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei, ej, ek = ei.ravel(), ej.ravel(), ek.ravel()
    gx = ei[:, None] * p + k[None, :, 0]
    gy = ej[:, None] * p + k[None, :, 1]
    gz = ek[:, None] * p + k[None, :, 2]
    elements = (gx * G[1] + gy) * G[2] + gz
    # 1-D node coordinates: element offset + scaled reference position
    coords = []
    for d, nn in enumerate((nx, ny, nz)):
        c = np.zeros(nn * p + 1)
        for i in range(nn):
            c[i * p:(i + 1) * p + 1] = (i + (u[d] + 1.0) / 2.0) * (L[d] / nn)
        coords.append(c)
    X, Y, Z = np.meshgrid(*coords, indexing="ij")
    points = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    return points, elements.astype(np.int64)


def jittered_tet_beam(n, L, seed, pattern, jitter=0.15):
    """Tets from a seeded jittered lattice (interior points moved by U(-jitter, jitter) h per
    axis), Delaunay-split, reoriented positive, raised to the order of the barycentric `pattern`."""
    from scipy.spatial import Delaunay
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    xs = [np.linspace(0, L[i], m + 1) for i, m in enumerate((nx, ny, nz))]
    P = np.stack(np.meshgrid(*xs, indexing="ij"), -1).reshape(-1, 3)
    h = np.array([L[0] / nx, L[1] / ny, L[2] / nz])
    interior = np.all((P > 1e-12) & (P < np.array(L) - 1e-12), axis=1)
    P[interior] += rng.uniform(-jitter, jitter, size=(interior.sum(), 3)) * h
    el = Delaunay(P).simplices.astype(np.int64)
    v = P[el]
    vol = np.einsum("ij,ij->i", np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), v[:, 3] - v[:, 0])
    keep = np.abs(vol) > 1e-12 * np.prod(h)
    el, vol = el[keep], vol[keep]
    neg = vol < 0
    el[neg, 1], el[neg, 2] = el[neg, 2].copy(), el[neg, 1].copy()
    return raise_tet_order(P, el, pattern)


def raise_tet_order(P, el, pattern):
    """High-order tet mesh from linear tets P/el and the barycentric node layout `pattern` [npe,4]."""
    lam = np.asarray(pattern)
    E, npe = el.shape[0], lam.shape[0]
    nzmask = np.abs(lam) > 1e-10
    nnz = nzmask.sum(1)
    q = np.round(lam * 1e6).astype(np.int64)
    keys = np.zeros((E, npe, 7), np.int64)
    for a in range(npe):
        idx = np.nonzero(nzmask[a])[0]
        g = el[:, idx]                        # global vertex ids of the nonzero barycentrics
        order = np.argsort(g, axis=1)
        gs = np.take_along_axis(g, order, 1)
        qs = q[a, idx][order]                 # their weights in the same (sorted) order
        keys[:, a, 0] = nnz[a]
        if nnz[a] == 4:                       # element interior: unique per element
            keys[:, a, 1] = np.arange(E)
            keys[:, a, 2] = a
        else:
            keys[:, a, 1:1 + nnz[a]] = gs
            keys[:, a, 4:4 + nnz[a] - 1] = qs[:, :nnz[a] - 1]
    flat = keys.reshape(-1, 7)
    uniq, first, inv = np.unique(flat, axis=0, return_index=True, return_inverse=True)
    elements = inv.reshape(E, npe).astype(np.int64)
    pos = np.einsum("ak,ekd->ead", lam, P[el]).reshape(-1, 3)
    points = pos[first]
    return points, elements
