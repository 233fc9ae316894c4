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
permutation. ``raise_tet_order_device`` / ``raise_hex_order_device`` are the GPU forms of
``raise_tet_order`` / ``raise_hex_order`` (``fl_RaiseTetOrder`` / ``fl_RaiseHexOrder``): the same
node numbering and the same weighted sums for the positions, for meshes too large to raise on the
host.
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


def tet_node_layout(pattern):
    """(nodes inside one edge, inside one face, inside the element) of the barycentric layout
    `pattern` [npe,4], as the device mesher classifies it; ValueError for a layout it rejects."""
    import ctypes
    from . import _native as N
    lam = np.ascontiguousarray(pattern, dtype=np.float64)
    counts = (ctypes.c_int64 * 3)()
    st = N.lib().fl_TetNodeLayout(lam.ctypes.data, lam.shape[0], ctypes.cast(counts, ctypes.c_void_p))
    if st != N.FL_OK:
        raise ValueError("node layout rejected: " + N.lib().fl_status_string(st).decode())
    return tuple(int(c) for c in counts)


def raise_tet_order_device(points, elements, pattern, device="cuda", out_points=None, out_elements=None):
    """High-order tet mesh built on the GPU from linear tets (``fl_RaiseTetOrder``): node numbers
    identical to ``raise_tet_order``, positions the same weighted vertex sums. points [nvert,3],
    elements [E,4] (numpy or tensors); returns (points [nnode,3] float64, elements [E,npe] int64)
    as device tensors on the current stream. Optional preallocated outputs (out_points [cap,3]
    float64, out_elements [E,npe] int64) save the counting call when cap is large enough."""
    import ctypes
    import torch
    from . import _native as N
    L = N.lib()
    dev = torch.device(device)
    lam = np.ascontiguousarray(pattern, dtype=np.float64)
    X = torch.as_tensor(points, dtype=torch.float64).to(dev).contiguous()
    el = torch.as_tensor(np.asarray(elements).astype(np.int64) if not isinstance(elements, torch.Tensor)
                         else elements, dtype=torch.int64).to(dev).contiguous()
    nvert, nelem, npe = X.shape[0], el.shape[0], lam.shape[0]
    ws_bytes = L.fl_RaiseTetOrder_workspace_size(nelem, nvert)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    out_el = out_elements if out_elements is not None else torch.empty((nelem, npe), dtype=torch.int64, device=dev)
    if out_el.shape != (nelem, npe) or out_el.dtype != torch.int64 or not out_el.is_contiguous():
        raise ValueError("out_elements must be a contiguous int64 tensor of shape (nelem, npe)")
    if out_points is not None and (out_points.dtype != torch.float64 or out_points.dim() != 2
                                   or out_points.shape[1] != 3 or not out_points.is_contiguous()):
        raise ValueError("out_points must be a contiguous float64 tensor of shape (capacity, 3)")
    nnode = ctypes.c_int64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def call(out_pts):
        return L.fl_RaiseTetOrder(ctypes.c_void_p(X.data_ptr()), nvert, ctypes.c_void_p(el.data_ptr()), nelem,
                                  lam.ctypes.data, npe,
                                  ctypes.c_void_p(out_pts.data_ptr()) if out_pts is not None else None,
                                  out_pts.shape[0] if out_pts is not None else 0, ctypes.byref(nnode),
                                  ctypes.c_void_p(out_el.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws_bytes, stream)

    out_pts = out_points
    st = call(out_pts)  # without a large enough buffer: counts the nodes only
    if st == N.FL_ERR_CAPACITY:
        out_pts = torch.empty((max(nnode.value, 1), 3), dtype=torch.float64, device=dev)
        st = call(out_pts)
    if st == N.FL_ERR_MESH:
        raise ValueError("an element repeats a vertex")
    N.check(st, "fl_RaiseTetOrder")
    return out_pts[:nnode.value], out_el


def hex_weights(pattern):
    """Trilinear weights [npe, 8] of the local nodes (reference coordinates `pattern` [npe, 3],
    the first 8 nodes the vertices) at the 8 vertices, zeroed below 1e-10, as the device mesher
    forms them."""
    xi = np.asarray(pattern, np.float64)
    sg = np.where(xi[:8] > 0, 1.0, -1.0)
    w = np.ones((xi.shape[0], 8))
    for d in range(3):
        w = w * (0.5 * (1.0 + sg[None, :, d] * xi[:, None, d]))
    w[np.abs(w) <= 1e-10] = 0.0
    return w


def raise_hex_order(P, el, pattern):
    """High-order hex mesh from linear hexes P/el [E,8] and the reference-coordinate node layout
    `pattern` [npe,3] (first 8 nodes the vertices). Numbering: the lexicographic order of (entity
    size, global vertices ascending, weights in that order), as fl_RaiseHexOrder numbers them;
    positions the weighted vertex sums in vertex order."""
    el = np.asarray(el, np.int64)
    w = hex_weights(pattern)
    E, npe = el.shape[0], w.shape[0]
    q = np.rint(w * 1e6).astype(np.int64)
    nz = w != 0.0
    keys = np.zeros((E, npe, 9), np.int64)
    for a in range(npe):
        idx = np.nonzero(nz[a])[0]
        k = len(idx)
        keys[:, a, 0] = k
        if k == 8:                            # element interior: unique per element
            keys[:, a, 1] = np.arange(E)
            keys[:, a, 2] = a
            continue
        g = el[:, idx]
        order = np.argsort(g, axis=1)
        keys[:, a, 1:1 + k] = np.take_along_axis(g, order, 1)
        if k > 1:
            keys[:, a, 5:5 + k] = q[a, idx][order]
    uniq, first, inv = np.unique(keys.reshape(-1, 9), axis=0, return_index=True, return_inverse=True)
    elements = inv.reshape(E, npe).astype(np.int64)
    X = np.asarray(P, np.float64)[el]       # [E, 8, 3]
    pos = w[None, :, 0, None] * X[:, None, 0, :]
    for k in range(1, 8):
        pos = pos + w[None, :, k, None] * X[:, None, k, :]
    points = pos.reshape(-1, 3)[first]
    return points, elements


def hex_node_layout(pattern):
    """(nodes inside one edge, inside one face, inside the element) of the hex layout `pattern`
    [npe,3], as the device mesher classifies it; ValueError for a layout it rejects."""
    import ctypes
    from . import _native as N
    xi = np.ascontiguousarray(pattern, dtype=np.float64)
    counts = (ctypes.c_int64 * 3)()
    st = N.lib().fl_HexNodeLayout(xi.ctypes.data, xi.shape[0], ctypes.cast(counts, ctypes.c_void_p))
    if st != N.FL_OK:
        raise ValueError("node layout rejected: " + N.lib().fl_status_string(st).decode())
    return tuple(int(c) for c in counts)


def raise_hex_order_device(points, elements, pattern, device="cuda"):
    """High-order hex mesh built on the GPU from linear hexes (``fl_RaiseHexOrder``): node numbers
    identical to ``raise_hex_order``, positions the same weighted vertex sums. Returns (points
    [nnode,3] float64, elements [E,npe] int64) as device tensors on the current stream."""
    import ctypes
    import torch
    from . import _native as N
    L = N.lib()
    dev = torch.device(device)
    xi = np.ascontiguousarray(pattern, dtype=np.float64)
    X = torch.as_tensor(points, dtype=torch.float64).to(dev).contiguous()
    el = torch.as_tensor(np.asarray(elements).astype(np.int64) if not isinstance(elements, torch.Tensor)
                         else elements, dtype=torch.int64).to(dev).contiguous()
    nvert, nelem, npe = X.shape[0], el.shape[0], xi.shape[0]
    ws_bytes = L.fl_RaiseHexOrder_workspace_size(nelem, nvert)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    out_el = torch.empty((nelem, npe), dtype=torch.int64, device=dev)
    nnode = ctypes.c_int64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def call(out_pts):
        return L.fl_RaiseHexOrder(ctypes.c_void_p(X.data_ptr()), nvert, ctypes.c_void_p(el.data_ptr()), nelem,
                                  xi.ctypes.data, npe,
                                  ctypes.c_void_p(out_pts.data_ptr()) if out_pts is not None else None,
                                  out_pts.shape[0] if out_pts is not None else 0, ctypes.byref(nnode),
                                  ctypes.c_void_p(out_el.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws_bytes, stream)

    st = call(None)  # counts the nodes
    out_pts = None
    if st == N.FL_ERR_CAPACITY:
        out_pts = torch.empty((max(nnode.value, 1), 3), dtype=torch.float64, device=dev)
        st = call(out_pts)
    if st == N.FL_ERR_MESH:
        raise ValueError("an element repeats a vertex")
    N.check(st, "fl_RaiseHexOrder")
    return out_pts[:nnode.value], out_el


def kuhn_tet_box(n, L=(1.0, 1.0, 1.0)):
    """Linear tets of an nx x ny x nz box of cubes, each cube split into the six tets around its
    main diagonal (the Kuhn split, conforming across cubes), all positively oriented."""
    nx, ny, nz = n
    xs = [np.linspace(0, L[i], m + 1) for i, m in enumerate((nx, ny, nz))]
    P = np.stack(np.meshgrid(*xs, indexing="ij"), -1).reshape(-1, 3)
    ci, cj, ck = [c.ravel() for c in np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")]

    def vid(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k

    tets = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        c = [ci.copy(), cj.copy(), ck.copy()]
        t = [vid(*c)]
        for axis in perm:
            c[axis] = c[axis] + 1
            t.append(vid(*c))
        t = np.stack(t, 1)
        if perm in ((0, 2, 1), (1, 0, 2), (2, 1, 0)):  # odd permutations: negative volume as walked
            t[:, [1, 2]] = t[:, [2, 1]]
        tets.append(t)
    el = np.stack(tets, 1).reshape(-1, 4).astype(np.int64)
    return P, el
