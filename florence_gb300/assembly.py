"""Host side of the GB300 assembly engine: Florence's low-level assembly interface on the device.

Two layers:

* ``DeviceAssembler`` keeps a mesh, its function-space tables and its sparsity pattern resident
  in GPU memory (torch tensors used as plain device buffers) and assembles from device-resident
  current coordinates: the form a Newton or explicit time loop uses.
* Drop-in callables with the names, arguments, return values and errors of the reference's
  Cython wrappers, so that Florence's own dispatcher finds and calls them:

  - ``_LowLevelAssemblyDF__NeoHookean_``, ``_LowLevelAssemblyDF__MooneyRivlin_``
    (Florence/FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDF_.pyx:53-160, names made by
    AOT_Assembler.py:36-118, looked up by _LowLevelAssembly_.py:45-83);
  - ``_LowLevelAssemblyExplicit_DF_DPF_`` (_LowLevelAssemblyExplicit_DF_DPF_.pyx:44-152);
  - ``ComputeSparsityPattern`` (_Assembly_/ComputeSparsityPattern.pyx:44-112);
  - ``__TotalConstantMassIntegrand__`` for lumped and consistent mass (VariationalPrinciple/_Mass_/_MassIntegrand_.pyx:192-348).

  ``install(Florence)`` registers them in Florence's module namespaces.

Every call goes through the CUDA library; there is no CPU path.
"""
import contextlib
import ctypes
import threading
import warnings
import weakref

import numpy as np
import torch

from . import _native as N

__all__ = ["DeviceAssembler", "ComputeSparsityPattern", "_LowLevelAssemblyDF__NeoHookean_",
           "AssembleExternalTractionForces", "AssembleBodyForces",
           "_LowLevelAssemblyDF__AnisotropicMooneyRivlin_1_",
           "_LowLevelAssemblyDF__MooneyRivlin_", "_LowLevelAssemblyExplicit_DF_DPF_",
           "__TotalConstantMassIntegrand__", "install", "material_params", "fp64_peak_gflops",
           "release_host_buffers", "release_device_meshes"]

MATERIALS = {"NeoHookean": N.FL_MATERIAL_NEOHOOKEAN, "MooneyRivlin": N.FL_MATERIAL_MOONEYRIVLIN,
             "NearlyIncompressibleMooneyRivlin": N.FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN,
             "LinearElastic": N.FL_MATERIAL_LINEARELASTIC,
             "AnisotropicMooneyRivlin_1": N.FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1}
# the reference's explicit dispatcher has no transversely isotropic material
# (_LowLevelAssemblyExplicit_DF_DPF_.pyx:72-109)
EXPLICIT_MATERIALS = {k: v for k, v in MATERIALS.items() if k != "AnisotropicMooneyRivlin_1"}
_DF_ENTRY = {N.FL_MATERIAL_NEOHOOKEAN: "fl_GlobalAssemblyDF__NeoHookean_",
             N.FL_MATERIAL_MOONEYRIVLIN: "fl_GlobalAssemblyDF__MooneyRivlin_",
             N.FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN: "fl_GlobalAssemblyDF__NearlyIncompressibleMooneyRivlin_",
             N.FL_MATERIAL_LINEARELASTIC: "fl_GlobalAssemblyDF__LinearElastic_",
             N.FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1: "fl_GlobalAssemblyDF__AnisotropicMooneyRivlin_1_"}


def _abi_params(mat_id, params):
    """(mu, mu1, mu2, lamb, mu3) of the reference's argument list for kernel parameters
    (p0, p1, p2[, p3]): neo-Hookean and linear elastic (mu, lamb); Mooney-Rivlin (mu1, mu2, lamb);
    nearly incompressible Mooney-Rivlin (alpha, beta, kappa) passed as (mu1, mu2, lamb); the
    transversely isotropic Mooney-Rivlin (mu1, mu2, lamb, mu3)."""
    p0, p1, p2 = params[:3]
    p3 = params[3] if len(params) > 3 else 0.0
    if mat_id in (N.FL_MATERIAL_NEOHOOKEAN, N.FL_MATERIAL_LINEARELASTIC):
        return p0, 0.0, 0.0, p1, 0.0
    return 0.0, p0, p1, p2, p3


def rt_supported(npe, nq):
    """Element types the reference-tensor contraction takes (fl_reftensor.cu): 4-, 8-, 10- and
    20-node elements with at most 15 Gauss points."""
    return npe in (4, 8, 10, 20) and 1 <= nq <= 15


class NonPositiveJacobianWarning(RuntimeWarning):
    """det F <= 0 at some Gauss point (the reference propagates such values silently)."""


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _HostPool:
    """Host buffers for the drop-ins' outputs, reused once the caller has dropped the array a
    buffer was last returned as (tracked by a weak reference; a live view or a matrix built on the
    array keeps it alive). Fresh host memory costs a page fault per page on its first write, which
    made the device-to-host copy of a 761 MB tangent run at 27 GB/s; into memory written before,
    the same copy runs at ~190 GB/s over the Grace-GPU link. Buffers for device results are
    page-locked (pinned), which lets the copy engine write them directly. At most `keep` idle
    buffers per size are held; ``release_host_buffers()`` frees them."""

    def __init__(self, keep=2):
        self.keep = keep
        self.slots = []  # [tensor, weakref to the array last handed out]
        self.lock = threading.Lock()

    def take(self, shape, dtype, pinned=False):
        n = int(np.prod(shape))
        with self.lock:
            same = [sl for sl in self.slots if sl[0].numel() == n and sl[0].dtype == dtype
                    and sl[0].is_pinned() == pinned]
            idle = [sl for sl in same if sl[1]() is None]
            if idle:
                slot = idle.pop(0)
            else:
                slot = [torch.empty(n, dtype=dtype, pin_memory=pinned), None]
                self.slots.append(slot)
            drop = {id(sl) for sl in idle[self.keep:]}
            self.slots = [sl for sl in self.slots if id(sl) not in drop]
            # the weak reference is to the array that every view of the returned one has as its
            # base (numpy collapses view chains onto it), so it dies only with the last view
            base = slot[0].numpy()
            slot[1] = weakref.ref(base)
            return slot[0], base.reshape(shape)

    def to_host(self, dev):
        """Copy of a device tensor into a pooled host array (synchronous)."""
        t, arr = self.take(tuple(dev.shape), dev.dtype, pinned=dev.is_cuda)
        t.copy_(dev.reshape(-1))
        return arr

    def release(self):
        with self.lock:
            self.slots = [sl for sl in self.slots if sl[1]() is not None]


_HOST = _HostPool()


def release_host_buffers():
    """Frees the idle host buffers of the drop-ins' outputs (arrays still held are unaffected)."""
    _HOST.release()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _to_dev(a, dtype, device):
    """Host array -> contiguous device tensor. uint64 node ids travel as int64 bits."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    a = np.asarray(a)
    if a.dtype == np.uint64:
        a = a.view(np.int64)
    return torch.from_numpy(np.ascontiguousarray(a, dtype=torch.empty(0, dtype=dtype).numpy().dtype)).to(device)


def material_params(material, name=None, explicit=False):
    """(material id, (p0, p1, p2)) for the kernels, read from a Florence material object as the
    reference's implicit (or, explicit=True, explicit) low-level wrapper reads it."""
    name = name or type(material).__name__
    if explicit and name == "NearlyIncompressibleMooneyRivlin":  # _LowLevelAssemblyExplicit_DF_DPF_.pyx:82-84
        return (N.FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN,
                (float(material.alpha), float(material.beta), float(material.kappa)))
    if name == "NeoHookean":
        return N.FL_MATERIAL_NEOHOOKEAN, (float(material.mu), float(material.lamb), 0.0)
    if name == "MooneyRivlin":
        return N.FL_MATERIAL_MOONEYRIVLIN, (float(material.mu1), float(material.mu2), float(material.lamb))
    if name == "LinearElastic":
        return N.FL_MATERIAL_LINEARELASTIC, (float(material.mu), float(material.lamb), 0.0)
    if name == "NearlyIncompressibleMooneyRivlin":
        # the low-level path constructs the material from (mu1, mu2, lamb) (AOT_Assembler.py:68-69, 110-111)
        return (N.FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN,
                (float(material.mu1), float(material.mu2), float(material.lamb)))
    if name == "AnisotropicMooneyRivlin_1" and not explicit:  # AOT_Assembler.py:72-75, 113-114
        return (N.FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1,
                (float(material.mu1), float(material.mu2), float(material.lamb), float(material.mu3)))
    raise NotImplementedError("Turning optimise option on for {} material is not supported yet. "
                              "Consider 'optimise=False' for now".format(name))


def _check_flags(flags, what):
    f = int(flags.item())
    if f & N.FL_FLAG_BAD_INDEX:
        raise N.FlorenceGB300Error(N.FL_ERR_ARG, what + " (element node id or index map out of range)")
    if f & N.FL_FLAG_TIMEOUT:
        raise N.FlorenceGB300Error(N.FL_ERR_CUDA, what + " (a bounded wait in a tensor-core kernel gave up)")
    if f & N.FL_FLAG_PAIR_RANGE:
        raise N.FlorenceGB300Error(N.FL_ERR_UNSUPPORTED, what + " (the pulled-back tangent left the float-pair "
                                   "exponent range [2^-78, 2^120]: assemble with set_arithmetic('fp64'))")
    if f & N.FL_FLAG_NONPOSITIVE_J:
        warnings.warn("det F <= 0 at some Gauss point in " + what, NonPositiveJacobianWarning, stacklevel=3)


def device_sparsity(elements, nnode, nvar=3, maps=True, stream=None):
    """Sparsity pattern on the device. elements: int64 device tensor [nelem, npe].
    Returns (indices, indptr, data_local, data_global) device int32 tensors (maps None if not maps)."""
    L = N.lib()
    nelem, npe = elements.shape
    dev = elements.device
    ws_bytes = L.fl_ComputeSparsityPattern_workspace_size(nelem, npe, nnode)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    indptr = torch.empty(nnode * nvar + 1, dtype=torch.int32, device=dev)
    cap = (npe * nvar) ** 2 * nelem
    dl = torch.empty(cap, dtype=torch.int32, device=dev) if maps else None
    dg = torch.empty(cap, dtype=torch.int32, device=dev) if maps else None
    nnz = ctypes.c_int64(0)
    # the first call only counts (no indices buffer yet), the second fills
    indices = None
    st = L.fl_ComputeSparsityPattern(_ptr(elements), nelem, npe, nnode, nvar, _ptr(indptr), None, 0,
                                     ctypes.byref(nnz), _ptr(dl), _ptr(dg), _ptr(ws), ws_bytes, stream or _stream())
    if st == N.FL_ERR_CAPACITY:
        indices = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
        st = L.fl_ComputeSparsityPattern(_ptr(elements), nelem, npe, nnode, nvar, _ptr(indptr), _ptr(indices),
                                         indices.numel(), ctypes.byref(nnz), _ptr(dl), _ptr(dg), _ptr(ws), ws_bytes,
                                         stream or _stream())
    if st == N.FL_ERR_MESH:
        raise ValueError("every node must belong to at least one element")
    N.check(st, "fl_ComputeSparsityPattern")
    return indices[:nnz.value], indptr, dl, dg


class DeviceAssembler:
    """Mesh + function space + material resident on the GPU; assembles from device coordinates.

    points [N,3] f64, elements [E,npe] (any integer dtype), Jm [3,npe,nq], AllGauss [nq] or [nq,1],
    material: 'NeoHookean' (mu, lamb), 'MooneyRivlin' (mu1, mu2, lamb), 'LinearElastic' (mu, lamb),
    'NearlyIncompressibleMooneyRivlin' (alpha, beta, kappa) or 'AnisotropicMooneyRivlin_1'
    (mu1, mu2, lamb, mu3, with `orientations` [E,3], one fibre direction per element).
    mode: 'csr' (the reference's element-to-nonzero maps), 'squeeze' (binary search in each row)
    or 'triplet' (I, J, V per element entry).
    deterministic: CSR outputs bit-identical from run to run (the atomic adds of the scatter
    otherwise land in an order that varies): the elements are coloured so that no two elements of
    a colour share a node, and the colours are assembled one after another, so that every CSR entry
    and residual entry receives its contributions in colour order, one per colour.
    """

    def __init__(self, points, elements, Jm, AllGauss, material, params, mode="csr", device="cuda",
                 requires_geometry_update=1, Bases=None, sparsity=None, orientations=None, deterministic=False):
        self.device = torch.device(device)
        self.points = _to_dev(points, torch.float64, self.device)
        self.elements = _to_dev(elements, torch.int64, self.device)
        self.Jm = _to_dev(Jm, torch.float64, self.device)
        self.w = _to_dev(np.ravel(AllGauss) if not isinstance(AllGauss, torch.Tensor) else AllGauss.reshape(-1),
                         torch.float64, self.device)
        self.Bases = _to_dev(Bases, torch.float64, self.device) if Bases is not None else None
        self.nnode = self.points.shape[0]
        self.nelem, self.npe = self.elements.shape
        self.nq = self.w.shape[0]
        self.ndof = 3 * self.npe
        self.material = material
        self.mat_id = MATERIALS[material]
        self.orient = None
        if self.mat_id == N.FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1:
            if orientations is None:
                raise ValueError("AnisotropicMooneyRivlin_1 needs the fibre direction of every element (orientations)")
            self.orient = _to_dev(np.asarray(orientations, np.float64).reshape(-1, 3)
                                  if not isinstance(orientations, torch.Tensor) else orientations.reshape(-1, 3),
                                  torch.float64, self.device)
            if self.orient.shape[0] != self.elements.shape[0]:
                raise ValueError("orientations must hold one direction per element")
        self.params = tuple(float(p) for p in params) + (0.0,) * (3 - len(params))
        self.mode = mode
        self.update = int(requires_geometry_update)
        self.flags = torch.zeros(1, dtype=torch.int32, device=self.device)
        if mode in ("csr", "squeeze"):
            if sparsity is None:
                sparsity = device_sparsity(self.elements, self.nnode, 3, maps=(mode == "csr"))
            ind, ptr, dl, dg = sparsity
            self.indices = _to_dev(ind, torch.int32, self.device)
            self.indptr = _to_dev(ptr, torch.int32, self.device)
            self.data_local = _to_dev(dl, torch.int32, self.device) if mode == "csr" else None
            self.data_global = _to_dev(dg, torch.int32, self.device) if mode == "csr" else None
            self.nnz = self.indices.shape[0]
        elif mode != "triplet":
            raise ValueError("mode must be 'csr', 'squeeze' or 'triplet'")
        self.deterministic = bool(deterministic)
        self._colour = None
        if self.deterministic:
            if mode == "triplet":
                raise ValueError("deterministic assembly takes the CSR modes (triplets have no additions)")
            self._colour = self._colour_elements()

    def _colour_elements(self):
        """Greedy node-disjoint colouring (host, once per mesh): each element takes the smallest
        colour none of its nodes' elements has so far. Returns the colour-sorted element order's
        pieces per colour: (elements, orientations, block offsets, reference geometry)."""
        el = self.elements.cpu().numpy()
        used = np.zeros(self.nnode, np.uint64)          # per node: bitmask of the colours around it
        colour = np.empty(self.nelem, np.int64)
        extra = {}                                      # beyond 64 colours: node -> set of colours
        for e in range(self.nelem):
            nodes = el[e]
            m = np.bitwise_or.reduce(used[nodes])
            if m != np.uint64(0xFFFFFFFFFFFFFFFF):
                c = int((~int(m) & (int(m) + 1)).bit_length() - 1)
            else:
                taken = set().union(*(extra.get(int(n), set()) for n in nodes))
                c = 64
                while c in taken:
                    c += 1
            colour[e] = c
            if c < 64:
                used[nodes] |= np.uint64(1) << np.uint64(c)
            else:
                for n in nodes:
                    extra.setdefault(int(n), set()).add(c)
        order = np.argsort(colour, kind="stable")
        counts = np.bincount(colour)
        pieces = []
        start = 0
        for c, k in enumerate(counts):
            if k == 0:
                continue
            idx = torch.from_numpy(order[start:start + k]).to(self.device)
            sub = self.elements[idx].contiguous()
            orient = self.orient[idx].contiguous() if self.orient is not None else None
            pieces.append(dict(elements=sub, orient=orient, count=int(k)))
            start += k
        return pieces

    # -- implicit tangent + residual ------------------------------------------------------------
    def assemble(self, Eulerx, V=None, T=None, I=None, J=None, stream=None):
        """Tangent and residual at device coordinates Eulerx [N,3] f64. Accumulates into V/T when
        given (zeroed tensors otherwise). Returns (V, T) or, in triplet mode, (I, J, V, T)."""
        L = N.lib()
        x = Eulerx if Eulerx.is_contiguous() else Eulerx.contiguous()
        cap = self.nelem * self.ndof * self.ndof
        if T is None:
            T = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        if self.mode == "triplet":
            I = torch.empty(cap, dtype=torch.int32, device=self.device) if I is None else I
            J = torch.empty(cap, dtype=torch.int32, device=self.device) if J is None else J
            V = torch.empty(cap, dtype=torch.float64, device=self.device) if V is None else V
            Ip, Jp, dl, dg = I, J, None, None
        else:
            V = torch.zeros(self.nnz, dtype=torch.float64, device=self.device) if V is None else V
            Ip, Jp, dl, dg = self.indptr, self.indices, self.data_local, self.data_global
        mu, mu1, mu2, lamb, mu3 = _abi_params(self.mat_id, self.params)
        if self.deterministic:
            self._assemble_by_colour(x, V, T, mu, mu1, mu2, lamb, mu3, stream)
            return V, T
        args = (_ptr(self.points), _ptr(self.elements), _ptr(x), None, None, _ptr(self.Jm), _ptr(self.w),
                3, 3, self.nq, self.nelem, self.npe, self.nnode, 6, self.update, None, None,
                _ptr(Ip), _ptr(Jp), _ptr(V), _ptr(T), 1 if self.mode == "triplet" else 0,
                1 if self.mode == "squeeze" else 0, _ptr(dl), _ptr(dg), None, None,
                1.0, mu, mu1, mu2, mu3, 0.0, lamb, 0.0, 0.0, 0.0, 0.0, _ptr(self.orient), _ptr(self.flags),
                stream or _stream())
        boff = self.block_offsets(stream) if self.mode != "triplet" and \
            N.lib().fl_GetAssemblyArithmetic() == N.FL_ARITH_REFERENCE_TENSOR and rt_supported(self.npe, self.nq) \
            else None
        st = L.fl_GlobalAssemblyDF_Blocks(self.mat_id, _ptr(boff), _ptr(self.reference_geometry(stream)), *args)
        N.check(st, "fl_GlobalAssemblyDF")
        if self.mode == "triplet":
            return I, J, V, T
        return V, T

    def _assemble_by_colour(self, x, V, T, mu, mu1, mu2, lamb, mu3, stream):
        """One call per colour on that colour's elements (their block offsets and reference
        geometry built on first use); the CSR positions by block offsets (reference tensor) or row
        search, never the element-to-nonzero maps (which follow the original element order)."""
        L = N.lib()
        rt = N.lib().fl_GetAssemblyArithmetic() == N.FL_ARITH_REFERENCE_TENSOR and rt_supported(self.npe, self.nq)
        st_ = stream or _stream()
        for pc in self._colour:
            el = pc["elements"]
            if "geo" not in pc:
                geo = torch.empty((10, max(1, pc["count"] * self.nq)), dtype=torch.float64, device=self.device)
                N.check(L.fl_ReferenceGeometry(_ptr(self.points), _ptr(el), _ptr(self.Jm), pc["count"], self.npe,
                                               self.nq, self.nnode, _ptr(geo), _ptr(self.flags), st_),
                        "fl_ReferenceGeometry")
                pc["geo"] = geo
            boff = None
            if rt:
                if "boff" not in pc:
                    b = torch.empty((pc["count"], self.npe, self.npe), dtype=torch.int32, device=self.device)
                    N.check(L.fl_ElementBlockOffsets(_ptr(el), pc["count"], self.npe, self.nnode, _ptr(self.indptr),
                                                     _ptr(self.indices), _ptr(b), _ptr(self.flags), st_),
                            "fl_ElementBlockOffsets")
                    pc["boff"] = b
                boff = pc["boff"]
            args = (_ptr(self.points), _ptr(el), _ptr(x), None, None, _ptr(self.Jm), _ptr(self.w),
                    3, 3, self.nq, pc["count"], self.npe, self.nnode, 6, self.update, None, None,
                    _ptr(self.indptr), _ptr(self.indices), _ptr(V), _ptr(T), 0, 1, None, None, None, None,
                    1.0, mu, mu1, mu2, mu3, 0.0, lamb, 0.0, 0.0, 0.0, 0.0, _ptr(pc["orient"]), _ptr(self.flags), st_)
            N.check(L.fl_GlobalAssemblyDF_Blocks(self.mat_id, _ptr(boff), _ptr(pc["geo"]), *args),
                    "fl_GlobalAssemblyDF (colour)")

    # -- pipelined assembly into host buffers (the drop-in's squeeze path) ---------------------------
    def _pipeline_plan(self, pieces):
        """Elements sorted by their smallest node id and split into `pieces` groups. A CSR row is
        final once the last group holding its node is assembled: after group g the rows of the
        nodes whose last group is g (as runs of consecutive nodes, gaps below 4 MB of values
        merged) can go to the host while the later groups are assembled. Built once per mesh."""
        el = self.elements.cpu().numpy()
        order = np.argsort(el.min(1), kind="stable")
        bounds = np.linspace(0, self.nelem, pieces + 1).astype(np.int64)
        group = np.empty(self.nelem, np.int64)
        for g in range(pieces):
            group[order[bounds[g]:bounds[g + 1]]] = g
        last = np.full(self.nnode, -1, np.int64)
        np.maximum.at(last, el.ravel(), np.repeat(group, self.npe))
        ptr = self.indptr.cpu().numpy().astype(np.int64)
        gap = (4 << 20) // 8
        plan = []
        for g in range(pieces):
            idx = order[bounds[g]:bounds[g + 1]]
            nodes = np.nonzero(last == g)[0]
            runs = []
            if nodes.size:
                cut = np.nonzero(np.diff(nodes) != 1)[0]
                starts = np.concatenate([[nodes[0]], nodes[cut + 1]])
                ends = np.concatenate([nodes[cut] + 1, [nodes[-1] + 1]])
                for a, b in zip(starts, ends):
                    if runs and ptr[3 * a] - ptr[3 * runs[-1][1]] < gap:
                        runs[-1][1] = b            # merge: the rows between are copied again later
                    else:
                        runs.append([a, b])
            sub = torch.from_numpy(el[idx]).to(self.device)
            plan.append(dict(elements=sub.contiguous(), count=int(idx.size),
                             orient=self.orient[torch.from_numpy(idx).to(self.device)].contiguous()
                             if self.orient is not None else None,
                             rows=[(int(ptr[3 * a]), int(ptr[3 * b]), 3 * int(a), 3 * int(b)) for a, b in runs]))
        return plan

    def assemble_to_host(self, Eulerx, V_host, T_host, pieces=8):
        """Tangent (squeeze or csr mode) and residual into the pinned host tensors V_host [nnz] and
        T_host [3N], the assembly in `pieces` groups of elements on the current stream and the
        finished CSR rows copied out on a second stream meanwhile (the copy, ~190 GB/s over the
        Grace-GPU link, is longer than the assembly). Returns when both host tensors are complete.
        Flags as for assemble (check_flags)."""
        if self.mode == "triplet":
            raise ValueError("the pipelined assembly writes the CSR tangent")
        if getattr(self, "_pipe", None) is None or len(self._pipe) != pieces:
            self._pipe = self._pipeline_plan(pieces)
        L = N.lib()
        x = Eulerx if Eulerx.is_contiguous() else Eulerx.contiguous()
        V = torch.zeros(self.nnz, dtype=torch.float64, device=self.device)
        T = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        mu, mu1, mu2, lamb, mu3 = _abi_params(self.mat_id, self.params)
        rt = L.fl_GetAssemblyArithmetic() == N.FL_ARITH_REFERENCE_TENSOR and rt_supported(self.npe, self.nq)
        comp = torch.cuda.current_stream(self.device)
        copy = getattr(self, "_copy_stream", None)
        if copy is None:
            copy = self._copy_stream = torch.cuda.Stream(device=self.device)
        st_ = ctypes.c_void_p(comp.cuda_stream)
        for pc in self._pipe:
            if pc["count"] == 0:
                continue
            if "geo" not in pc:
                geo = torch.empty((10, pc["count"] * self.nq), dtype=torch.float64, device=self.device)
                N.check(L.fl_ReferenceGeometry(_ptr(self.points), _ptr(pc["elements"]), _ptr(self.Jm), pc["count"],
                                               self.npe, self.nq, self.nnode, _ptr(geo), _ptr(self.flags), st_),
                        "fl_ReferenceGeometry")
                pc["geo"] = geo
            if rt and "boff" not in pc:
                b = torch.empty((pc["count"], self.npe, self.npe), dtype=torch.int32, device=self.device)
                N.check(L.fl_ElementBlockOffsets(_ptr(pc["elements"]), pc["count"], self.npe, self.nnode,
                                                 _ptr(self.indptr), _ptr(self.indices), _ptr(b), _ptr(self.flags),
                                                 st_), "fl_ElementBlockOffsets")
                pc["boff"] = b
            args = (_ptr(self.points), _ptr(pc["elements"]), _ptr(x), None, None, _ptr(self.Jm), _ptr(self.w),
                    3, 3, self.nq, pc["count"], self.npe, self.nnode, 6, self.update, None, None,
                    _ptr(self.indptr), _ptr(self.indices), _ptr(V), _ptr(T), 0, 1, None, None, None, None,
                    1.0, mu, mu1, mu2, mu3, 0.0, lamb, 0.0, 0.0, 0.0, 0.0, _ptr(pc["orient"]), _ptr(self.flags), st_)
            N.check(L.fl_GlobalAssemblyDF_Blocks(self.mat_id, _ptr(pc["boff"] if rt else None), _ptr(pc["geo"]),
                                                 *args), "fl_GlobalAssemblyDF (pipelined)")
            done = torch.cuda.Event()
            done.record(comp)
            copy.wait_event(done)
            with torch.cuda.stream(copy):
                for v0, v1, t0, t1 in pc["rows"]:
                    V_host[v0:v1].copy_(V[v0:v1], non_blocking=True)
                    T_host[t0:t1].copy_(T[t0:t1], non_blocking=True)
        V.record_stream(copy)
        T.record_stream(copy)
        copy.synchronize()
        return V_host, T_host

    def reference_geometry(self, stream=None):
        """(dX/dxi)^-1 and det(dX/dxi) per element and Gauss point (fl_ReferenceGeometry), computed
        on first use and kept: [10, nelem * nq] float64. The assembly then forms only the current
        configuration's part of the kinematics."""
        if getattr(self, "_geo", None) is None:
            geo = torch.empty((10, max(1, self.nelem * self.nq)), dtype=torch.float64, device=self.device)
            N.check(N.lib().fl_ReferenceGeometry(_ptr(self.points), _ptr(self.elements), _ptr(self.Jm), self.nelem,
                                                 self.npe, self.nq, self.nnode, _ptr(geo), _ptr(self.flags),
                                                 stream or _stream()), "fl_ReferenceGeometry")
            self._geo = geo
        return self._geo

    def block_offsets(self, stream=None):
        """The pattern's per-element node-block offsets (fl_ElementBlockOffsets), built on first
        use and kept: [nelem, npe, npe] int32, -1 where an entry must be searched."""
        if getattr(self, "_boff", None) is None:
            boff = torch.empty((self.nelem, self.npe, self.npe), dtype=torch.int32, device=self.device)
            st = N.lib().fl_ElementBlockOffsets(_ptr(self.elements), self.nelem, self.npe, self.nnode, _ptr(self.indptr),
                                               _ptr(self.indices), _ptr(boff), _ptr(self.flags), stream or _stream())
            N.check(st, "fl_ElementBlockOffsets")
            self._boff = boff
        return self._boff

    def assemble_mixed(self, Eulerx, V32=None, T=None, stream=None):
        """Inexact-Newton Jacobian: FP32 CSR values from the split-BF16 tensor-core contraction and
        the FP64 residual (csr or squeeze mode). Accumulates into V32/T when given."""
        if self.mode not in ("csr", "squeeze"):
            raise ValueError("the mixed tangent is assembled into the CSR pattern (csr or squeeze mode)")
        L = N.lib()
        x = Eulerx if Eulerx.is_contiguous() else Eulerx.contiguous()
        if V32 is None:
            V32 = torch.zeros(self.nnz, dtype=torch.float32, device=self.device)
        if T is None:
            T = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        mu, mu1, mu2, lamb, mu3 = _abi_params(self.mat_id, self.params)
        st = L.fl_GlobalAssemblyDF_Mixed(self.mat_id, _ptr(self.points), _ptr(self.elements), _ptr(x), _ptr(self.Jm),
                                         _ptr(self.w), self.nq, self.nelem, self.npe, self.nnode, self.update,
                                         _ptr(self.indptr), _ptr(self.indices), _ptr(self.data_local),
                                         _ptr(self.data_global), _ptr(V32), _ptr(T), mu, mu1, mu2, lamb, mu3,
                                         _ptr(self.orient), None, _ptr(self.flags), stream or _stream())
        N.check(st, "fl_GlobalAssemblyDF_Mixed")
        return V32, T

    # -- explicit internal force ----------------------------------------------------------------
    def internal_force(self, Eulerx, T=None, stream=None):
        L = N.lib()
        x = Eulerx if Eulerx.is_contiguous() else Eulerx.contiguous()
        if T is None:
            T = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        if self.mat_id not in EXPLICIT_MATERIALS.values():
            raise NotImplementedError("the explicit internal force has no transversely isotropic material "
                                      "(as in the reference's explicit dispatcher)")
        mu, mu1, mu2, lamb, _ = _abi_params(self.mat_id, self.params)
        # the explicit entry takes the nearly incompressible material's (alpha, beta, kappa) as
        # (mu1, mu2, mu3) (_LowLevelAssemblyExplicit_DF_DPF_.pyx:82-84)
        mu3 = self.params[2] if self.mat_id == N.FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN else 0.0
        st = L.fl_GlobalAssemblyExplicit_DF_DPF_(
            _ptr(self.points), _ptr(self.elements), _ptr(x), None, None, _ptr(self.Jm), _ptr(self.w), 3, 3, self.nq,
            self.nelem, self.npe, self.nnode, 6, 1, _ptr(T), 1.0, mu, mu1, mu2, mu3, 0.0, lamb, 0.0, 0.0, 0.0, 0.0,
            None, self.mat_id, 0, _ptr(self.flags), stream or _stream())
        N.check(st, "fl_GlobalAssemblyExplicit_DF_DPF_")
        return T

    # -- lumped mass ----------------------------------------------------------------------------
    def lumped_mass(self, rho, Bases=None, M=None, stream=None):
        L = N.lib()
        B = self.Bases if Bases is None else _to_dev(Bases, torch.float64, self.device)
        if B is None:
            raise ValueError("lumped mass needs the basis values (Bases [npe, nq])")
        if M is None:
            M = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        st = L.fl_LumpedMass(_ptr(self.points), _ptr(self.elements), _ptr(B), _ptr(self.Jm), _ptr(self.w), 3, 3,
                             self.nq, self.nelem, self.npe, self.nnode, float(rho), _ptr(M), _ptr(self.flags),
                             stream or _stream())
        N.check(st, "fl_LumpedMass")
        return M

    # -- consistent mass -------------------------------------------------------------------------
    def consistent_mass(self, rho, Bases=None, V=None, I=None, J=None, stream=None):
        """Consistent mass sum_g rho N_a N_b w |det dX/dxi| on the nvar diagonal, in the
        assembler's scatter mode: CSR values [nnz] (accumulated into V when given), or in triplet
        mode (I, J, V) in element-local order."""
        L = N.lib()
        B = self.Bases if Bases is None else _to_dev(Bases, torch.float64, self.device)
        if B is None:
            raise ValueError("the mass needs the basis values (Bases [npe, nq])")
        cap = self.nelem * self.ndof * self.ndof
        if self.mode == "triplet":
            I = torch.empty(cap, dtype=torch.int32, device=self.device) if I is None else I
            J = torch.empty(cap, dtype=torch.int32, device=self.device) if J is None else J
            V = torch.empty(cap, dtype=torch.float64, device=self.device) if V is None else V
            ptr, ind, nnz = None, None, cap
        else:
            V = torch.zeros(self.nnz, dtype=torch.float64, device=self.device) if V is None else V
            ptr, ind, nnz = self.indptr, self.indices, self.nnz
        st = L.fl_ConsistentMass(_ptr(self.points), _ptr(self.elements), _ptr(B), _ptr(self.Jm), _ptr(self.w), 3, 3,
                                 self.nq, self.nelem, self.npe, self.nnode, float(rho),
                                 1 if self.mode == "triplet" else 0, 1 if self.mode == "squeeze" else 0, _ptr(ptr),
                                 _ptr(ind), nnz, _ptr(self.data_local if self.mode == "csr" else None),
                                 _ptr(self.data_global if self.mode == "csr" else None), _ptr(I), _ptr(J), _ptr(V),
                                 _ptr(self.flags), stream or _stream())
        N.check(st, "fl_ConsistentMass")
        if self.mode == "triplet":
            return I, J, V
        return V

    def check_flags(self, what="assembly"):
        _check_flags(self.flags, what)
        self.flags.zero_()


# ------------------------------------------------------------------------------------------------
# Drop-in callables (host numpy in, host numpy out, like the reference's Cython wrappers)
# ------------------------------------------------------------------------------------------------

def ComputeSparsityPattern(mesh, nvar, squeeze_sparsity_pattern=False):
    """Device twin of ComputeSparsityPattern.pyx:44-112: returns (indices, indptr) when squeezed,
    else (indices, indptr, data_local_indices, data_global_indices), int32 numpy arrays."""
    nnode = mesh.points.shape[0]
    el = _to_dev(mesh.elements, torch.int64, "cuda")
    ind, ptr, dl, dg = device_sparsity(el, nnode, nvar, maps=not squeeze_sparsity_pattern)
    torch.cuda.current_stream().synchronize()
    if squeeze_sparsity_pattern:
        return ind.cpu().numpy(), ptr.cpu().numpy()
    return ind.cpu().numpy(), ptr.cpu().numpy(), dl.cpu().numpy(), dg.cpu().numpy()


def _check_formulation(formulation, material):
    if formulation.ndim != 3 or formulation.nvar != 3 or material.H_VoigtSize != 6:
        raise NotImplementedError("the GB300 assembly covers three-dimensional mechanics (ndim = nvar = 3)")


def _fingerprint(a, samples=2048):
    """(shape, dtype, hash of an evenly spaced sample of the entries) of a host array: cheap enough
    for every call (microseconds), and it changes when an array is replaced or resized, or its
    sampled entries are rewritten."""
    a = np.asarray(a)
    flat = a.reshape(-1)
    n = flat.shape[0]
    idx = np.linspace(0, n - 1, min(n, samples)).astype(np.int64) if n else np.zeros(0, np.int64)
    return a.shape, a.dtype.str, hash(np.ascontiguousarray(flat[idx]).tobytes())


class _DeviceMeshCache:
    """Device-resident meshes of the drop-in callables. Florence calls the low-level assembly once
    per Newton iteration with the same mesh, function space and sparsity pattern and a new Eulerx
    (FEMSolver.py:973): the first call uploads the mesh, its tables and its CSR pattern, later
    calls with the same arrays upload only Eulerx. An entry is reused when every input array is
    the same object (held by a weak reference, so a freed and reallocated array never matches) with
    the same shape, dtype and sampled entries, and the material and flags are equal. Arrays
    rewritten in place between calls outside the sample go unnoticed: call
    ``release_device_meshes()`` after modifying a mesh in place. At most `keep` meshes are held."""

    def __init__(self, keep=2):
        self.keep = keep
        self.entries = []   # (refs, fingerprints, scalars, DeviceAssembler), most recent first
        self.lock = threading.Lock()

    @staticmethod
    def _refs(arrays):
        refs = []
        for a in arrays:
            if a is None:
                refs.append(None)
                continue
            try:
                refs.append(weakref.ref(a))
            except TypeError:   # not weak-referenceable (a list, a scalar): never cached
                return None
        return refs

    def get(self, arrays, scalars, build):
        refs = self._refs(arrays)
        if refs is None:
            return build()
        fps = [None if a is None else _fingerprint(a) for a in arrays]
        with self.lock:
            for k, (r, f, sc, asm) in enumerate(self.entries):
                same = all((ri is None and a is None) or (ri is not None and ri() is a) for ri, a in zip(r, arrays))
                if same and f == fps and sc == scalars:
                    self.entries.insert(0, self.entries.pop(k))
                    return asm
        asm = build()
        with self.lock:
            self.entries.insert(0, (refs, fps, scalars, asm))
            del self.entries[self.keep:]
        return asm

    def clear(self):
        with self.lock:
            self.entries = []


_MESHES = _DeviceMeshCache()


def release_device_meshes():
    """Drops the device-resident meshes the drop-in callables keep between calls."""
    _MESHES.clear()


PIPELINE_MIN_ELEMENTS = 20000  # the drop-in's pipelined assembly-and-copy from this mesh size on


def _low_level_df(name, fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    _check_formulation(formulation, material)
    mat_id, params = material_params(material, name)
    recompute = bool(fem_solver.recompute_sparsity_pattern)
    # CSR output with or without the reference's element-to-nonzero maps: the device scatter
    # finds every entry's position in the pattern itself (one row search per node pair), which
    # lands each value where the maps would and spares uploading the two E*ndof^2 maps
    mode = "triplet" if recompute else "squeeze"
    sparsity = None
    if not recompute:
        sparsity = (fem_solver.indices, fem_solver.indptr, None, None)
    orient = getattr(material, "anisotropic_orientations", None) if mat_id == N.FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1 \
        else None
    update = int(fem_solver.requires_geometry_update)
    arrays = [mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss, orient] + \
        ([fem_solver.indices, fem_solver.indptr] if not recompute else [None, None])
    asm = _MESHES.get(arrays, (name, tuple(params), mode, update, torch.cuda.current_device()),
                      lambda: DeviceAssembler(mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss,
                                              name, params, mode=mode, requires_geometry_update=update,
                                              sparsity=sparsity, orientations=orient))
    x = _to_dev(Eulerx, torch.float64, asm.device)
    if mode == "squeeze" and asm.nelem >= PIPELINE_MIN_ELEMENTS:
        # large meshes: the assembly in groups of elements, the finished rows copied to the host
        # while the later groups are assembled
        Vt, Va = _HOST.take((asm.nnz,), torch.float64, pinned=True)
        Tt, Ta = _HOST.take((asm.nnode * 3,), torch.float64, pinned=True)
        asm.assemble_to_host(x, Vt, Tt)
        if int(asm.flags.item()) & N.FL_FLAG_PAIR_RANGE:
            asm.flags.zero_()
            with arithmetic("fp64"):
                asm.assemble_to_host(x, Vt, Tt)
        asm.check_flags("_LowLevelAssemblyDF_" + name)
        return Va, Ta
    out = asm.assemble(x)
    if int(asm.flags.item()) & N.FL_FLAG_PAIR_RANGE:
        # values too small or too large for the float pairs of the default arithmetics (units far
        # from O(1)): the same call in FP64
        asm.flags.zero_()
        with arithmetic("fp64"):
            out = asm.assemble(x)
    host = [_HOST.to_host(t) for t in out]
    asm.check_flags("_LowLevelAssemblyDF_" + name)
    return tuple(host)


def _LowLevelAssemblyDF__NeoHookean_(fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDF_.pyx:53-160."""
    return _low_level_df("NeoHookean", fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp)


def _LowLevelAssemblyDF__MooneyRivlin_(fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDF_.pyx:53-160."""
    return _low_level_df("MooneyRivlin", fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp)


def _LowLevelAssemblyDF__NearlyIncompressibleMooneyRivlin_(fem_solver, function_space, formulation, mesh, material,
                                                            Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDF_.pyx:53-160."""
    return _low_level_df("NearlyIncompressibleMooneyRivlin", fem_solver, function_space, formulation, mesh, material,
                         Eulerx, Eulerp)


def _LowLevelAssemblyDF__LinearElastic_(fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDF_.pyx:53-160."""
    return _low_level_df("LinearElastic", fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp)


def _LowLevelAssemblyDF__AnisotropicMooneyRivlin_1_(fem_solver, function_space, formulation, mesh, material, Eulerx,
                                                     Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDF_.pyx:53-160 as
    AOT_Assembler.py builds it for _AnisotropicMooneyRivlin_1_ (mu1, mu2, mu3, lamb and the
    material's anisotropic_orientations, one fibre direction per element)."""
    return _low_level_df("AnisotropicMooneyRivlin_1", fem_solver, function_space, formulation, mesh, material, Eulerx,
                         Eulerp)


def AssembleExternalTractionForces(boundary_condition, mesh, material, function_space, physical_faces=False):
    """F [nnode*nvar, 1] -- Assembly.py:451-514 on the device: for every face with
    boundary_condition.neumann_flags set, F[(a, i)] += applied_neumann[face, i] sum_g N_a(g) w_g
    with the face function space's parent weights, as the reference integrates it. With
    physical_faces=True the weights carry |dX/dxi x dX/deta| of the face (no reference
    counterpart)."""
    if material.ndim != 3 or material.nvar != 3:
        raise NotImplementedError("the GB300 force assembly covers three-dimensional mechanics")
    dev = torch.device("cuda")
    faces = _to_dev(mesh.faces, torch.int64, dev)
    nnode = mesh.points.shape[0]
    F = torch.zeros(nnode * 3, dtype=torch.float64, device=dev)
    flags_dev = torch.zeros(1, dtype=torch.int32, device=dev)
    nf = _to_dev(np.asarray(boundary_condition.neumann_flags).astype(np.uint8).ravel(), torch.uint8, dev)
    tr = _to_dev(np.nan_to_num(np.asarray(boundary_condition.applied_neumann, np.float64).reshape(faces.shape[0], -1)
                               [:, :3]), torch.float64, dev)
    B = _to_dev(function_space.Bases, torch.float64, dev)
    w = _to_dev(np.ravel(function_space.AllGauss), torch.float64, dev)
    P = _to_dev(mesh.points, torch.float64, dev) if physical_faces else None
    Jf = _to_dev(function_space.Jm, torch.float64, dev) if physical_faces else None
    st = N.lib().fl_AssembleExternalTractionForces(_ptr(faces), faces.shape[0], faces.shape[1], _ptr(nf), _ptr(tr),
                                                   _ptr(B), _ptr(w), w.shape[0], _ptr(P), _ptr(Jf), nnode, _ptr(F),
                                                   _ptr(flags_dev), _stream())
    N.check(st, "fl_AssembleExternalTractionForces")
    _check_flags(flags_dev, "AssembleExternalTractionForces")
    return F.cpu().numpy()[:, None]


def AssembleBodyForces(boundary_condition, mesh, material, function_space):
    """F [nnode*nvar, 1] -- Assembly.py:516-560 on the device: the body force -rho in z,
    F[(a, z)] -= rho sum_g N_a(g) w_g for every element, with the parent weights as the reference
    integrates it."""
    if material.ndim != 3 or material.nvar != 3:
        raise NotImplementedError("the GB300 force assembly covers three-dimensional mechanics")
    dev = torch.device("cuda")
    el = _to_dev(mesh.elements, torch.int64, dev)
    nnode = mesh.points.shape[0]
    F = torch.zeros(nnode * 3, dtype=torch.float64, device=dev)
    flags_dev = torch.zeros(1, dtype=torch.int32, device=dev)
    B = _to_dev(function_space.Bases, torch.float64, dev)
    w = _to_dev(np.ravel(function_space.AllGauss), torch.float64, dev)
    st = N.lib().fl_AssembleBodyForces(_ptr(el), el.shape[0], el.shape[1], _ptr(B), _ptr(w), w.shape[0],
                                       float(material.rho), nnode, _ptr(F), _ptr(flags_dev), _stream())
    N.check(st, "fl_AssembleBodyForces")
    _check_flags(flags_dev, "AssembleBodyForces")
    return F.cpu().numpy()[:, None]


def _LowLevelAssemblyExplicit_DF_DPF_(function_space, formulation, mesh, material, Eulerx, Eulerp):
    """Internal force T [nnode*nvar] -- _LowLevelAssemblyExplicit_DF_DPF_.pyx:44-152 (mechanics)."""
    if formulation.fields != "mechanics":
        raise NotImplementedError("the GB300 explicit assembly covers the displacement formulation")
    _check_formulation(formulation, material)
    name = getattr(material, "mtype", type(material).__name__)
    if name not in EXPLICIT_MATERIALS:
        raise NotImplementedError("Low level assembly for material {} not available for explicit analysis."
                                  " Consider 'optimise=False' for now".format(name))
    _, params = material_params(material, name, explicit=True)
    asm = DeviceAssembler(mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss, name, params,
                          mode="triplet")
    T = asm.internal_force(_to_dev(Eulerx, torch.float64, asm.device))
    out = _HOST.to_host(T)
    asm.check_flags("_LowLevelAssemblyExplicit_DF_DPF_")
    return out


def __TotalConstantMassIntegrand__(mesh, function_space, formulation, mass_type="lumped",
                                   recompute_sparsity_pattern=True, squeeze_sparsity_pattern=False,
                                   indices=None, indptr=None, data_global_indices=None, data_local_indices=None):
    """_MassIntegrand_.pyx:192-348 on the device. Lumped: (mass [nvar*N,1], I, J, V) or (mass, V)
    with the 1-element placeholder I/J/V the reference returns. Consistent: (mass placeholder
    [1,1], I_mass, J_mass, V_mass) triplets in element-local order when
    recompute_sparsity_pattern, else (mass placeholder, V_mass) on the given CSR pattern (through
    the element-to-nonzero maps, or by row search when squeeze_sparsity_pattern)."""
    if mass_type not in ("lumped", "consistent"):
        raise ValueError("mass_type must be 'lumped' or 'consistent'")
    if formulation.nvar != 3 or mesh.points.shape[1] != 3:
        raise NotImplementedError("the GB300 mass assembly covers three-dimensional mechanics")
    # constant_mass_integrand[g] = rho N N^T (x) I3 (VariationalPrinciple.py:269-290): its entries sum
    # to 3 rho (sum_a N_a)^2 at every Gauss point, which recovers rho
    cmi = np.asarray(formulation.constant_mass_integrand)
    nsum = float(np.asarray(function_space.Bases)[:, 0].sum())
    rho = float(cmi[0].sum()) / (3.0 * nsum * nsum)
    if mass_type == "consistent":
        if recompute_sparsity_pattern:
            asm = DeviceAssembler(mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss,
                                  "NeoHookean", (1.0, 1.0), mode="triplet", Bases=function_space.Bases)
            I, J, V = asm.consistent_mass(rho)
            asm.check_flags("__TotalConstantMassIntegrand__")
            return np.zeros((1, 1)), I.cpu().numpy(), J.cpu().numpy(), V.cpu().numpy()
        squeeze = bool(squeeze_sparsity_pattern)
        if indices is None or indptr is None or (not squeeze and (data_global_indices is None
                                                                  or data_local_indices is None)):
            raise ValueError("the CSR consistent mass needs indices, indptr and (unless squeezed) the maps")
        sparsity = (indices, indptr, None if squeeze else data_local_indices,
                    None if squeeze else data_global_indices)
        asm = DeviceAssembler(mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss, "NeoHookean",
                              (1.0, 1.0), mode="squeeze" if squeeze else "csr", Bases=function_space.Bases,
                              sparsity=sparsity)
        V = asm.consistent_mass(rho)
        asm.check_flags("__TotalConstantMassIntegrand__")
        return np.zeros((1, 1)), V.cpu().numpy()
    asm = DeviceAssembler(mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss, "NeoHookean",
                          (1.0, 1.0), mode="triplet", Bases=function_space.Bases)
    M = asm.lumped_mass(rho).cpu().numpy()[:, None]
    asm.check_flags("__TotalConstantMassIntegrand__")
    z_i, z_v = np.zeros(1, np.int32), np.zeros(1, np.float64)
    if recompute_sparsity_pattern:
        return M, z_i, z_i.copy(), z_v
    return M, z_v


def install(florence):
    """Registers the GB300 callables in the reference's module namespaces, so that
    FEMSolver(optimise=True) / Assemble / AssembleExplicit dispatch to them."""
    import importlib
    ll = importlib.import_module(florence.__name__ + ".FiniteElements.Assembly._LowLevelAssembly_")
    ll._LowLevelAssemblyDF__NeoHookean_ = _LowLevelAssemblyDF__NeoHookean_
    ll._LowLevelAssemblyDF__MooneyRivlin_ = _LowLevelAssemblyDF__MooneyRivlin_
    ll._LowLevelAssemblyDF__NearlyIncompressibleMooneyRivlin_ = _LowLevelAssemblyDF__NearlyIncompressibleMooneyRivlin_
    ll._LowLevelAssemblyDF__LinearElastic_ = _LowLevelAssemblyDF__LinearElastic_
    ll._LowLevelAssemblyDF__AnisotropicMooneyRivlin_1_ = _LowLevelAssemblyDF__AnisotropicMooneyRivlin_1_
    ll._LowLevelAssemblyExplicit_DF_DPF_ = _LowLevelAssemblyExplicit_DF_DPF_
    from . import electromechanics as em
    for em_name in em.MATERIALS:  # the dispatcher's "_LowLevelAssemblyDPF__" + material name + "_"
        name = "_LowLevelAssemblyDPF__" + em_name + "_"
        setattr(ll, name, getattr(em, name))
    ll.has_low_level_dispatcher = True
    asm_mod = importlib.import_module(florence.__name__ + ".FiniteElements.Assembly.Assembly")
    asm_mod.AssembleExternalTractionForces = AssembleExternalTractionForces
    asm_mod.AssembleBodyForces = AssembleBodyForces
    try:
        sp = importlib.import_module(florence.__name__ + ".FiniteElements.Assembly.ComputeSparsityPattern")
    except ImportError:
        import sys
        import types
        sp = types.ModuleType(florence.__name__ + ".FiniteElements.Assembly.ComputeSparsityPattern")
        sys.modules[sp.__name__] = sp
    sp.ComputeSparsityPattern = ComputeSparsityPattern
    return ll


def fp64_peak_gflops():
    """Measured FP64 FMA throughput of this GPU (GFLOP/s)."""
    g = ctypes.c_double(0.0)
    N.check(N.lib().fl_measure_fp64_peak(ctypes.byref(g), _stream()), "fl_measure_fp64_peak")
    return g.value


def fp32_peak_gflops():
    """Measured FP32 FMA throughput of this GPU (GFLOP/s)."""
    g = ctypes.c_double(0.0)
    N.check(N.lib().fl_measure_fp32_peak(ctypes.byref(g), _stream()), "fl_measure_fp32_peak")
    return g.value


ARITHMETIC = {"fp64": N.FL_ARITH_FP64, "float_pair": N.FL_ARITH_FLOAT_PAIR, "tensor": N.FL_ARITH_TENSOR,
              "reference_tensor": N.FL_ARITH_REFERENCE_TENSOR}


def set_arithmetic(name):
    """Arithmetic of the stiffness contraction for every later FP64 assembly in the process:
    'reference_tensor' (the default: each tile of 14 elements as one tensor-core GEMM of the
    pulled-back tangents against the element type's constant reference tensor, seven BF16 digit
    planes per operand, exact FP64 recombination, ~1e-14; CSR outputs of 4-, 8-, 10- and 20-node
    elements with at most 15 Gauss points, else float pairs), 'float_pair' (hi + lo float pairs on
    the FP32 pipe, ~1e-14 relative to FP64), 'fp64' (FP64 multiply-adds) or 'tensor' (tensor cores
    on the per-element operand U split into six exact BF16 digits, ~1e-13). The material law is
    FP64 in all."""
    N.check(N.lib().fl_SetAssemblyArithmetic(ARITHMETIC[name]), "fl_SetAssemblyArithmetic")


def get_arithmetic():
    code = N.lib().fl_GetAssemblyArithmetic()
    return next(k for k, v in ARITHMETIC.items() if v == code)


@contextlib.contextmanager
def arithmetic(name):
    old = get_arithmetic()
    set_arithmetic(name)
    try:
        yield
    finally:
        set_arithmetic(old)


def set_tensor_core_tiling(tile_group=0, reduction_chunk=0):
    """Tiling of the split-BF16 tensor-core tangent for every later mixed assembly in the process:
    128-row tiles per work item and (Gauss point, direction) columns per tensor-core round
    (a multiple of 16 up to 96); 0 = chosen from the element type's shared-memory needs."""
    N.check(N.lib().fl_SetTensorCoreTiling(int(tile_group), int(reduction_chunk)), "fl_SetTensorCoreTiling")
