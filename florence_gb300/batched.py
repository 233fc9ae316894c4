"""Batched assembly of many independent meshes of uneven size and order.

Instances of one element type are concatenated into one mesh with disjoint node ranges: its CSR
tangent is the direct sum of the instances' tangents, so one pattern build and one pair of
kernel launches (per 64 MB scratch chunk) assemble all of them, each element with its own
material parameters (fl_GlobalAssemblyDF_Batched / fl_GlobalAssemblyDF_Mixed). Instances of
different element orders go to separate launches (the kernels are compiled per element size).
Large batches drop the per-element maps and scatter by binary search in the CSR rows.

The autotuner times the contraction kernel's Gauss-point chunk for each (nodes per element,
Gauss points) on the batch itself and installs the fastest (fl_SetAssemblyTuning).
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .assembly import MATERIALS, _ptr, _stream, _to_dev, device_sparsity


class BatchedAssembler:
    """instances: list of dicts with points [N_k,3], elements [E_k,npe] (one npe for all), Eulerx
    [N_k,3] and params (p0, p1[, p2]). Jm/AllGauss: the element type's tables."""

    def __init__(self, instances, Jm, AllGauss, material, device="cuda", maps=False):
        self.device = torch.device(device)
        self.material = material
        self.mat_id = MATERIALS[material]
        npes = {np.asarray(i["elements"]).shape[1] for i in instances}
        if len(npes) != 1:
            raise ValueError("one element type per batch")
        self.npe = npes.pop()
        node_off = np.cumsum([0] + [np.asarray(i["points"]).shape[0] for i in instances])
        elem_off = np.cumsum([0] + [np.asarray(i["elements"]).shape[0] for i in instances])
        self.node_off, self.elem_off = node_off, elem_off
        P = np.concatenate([np.asarray(i["points"], np.float64) for i in instances])
        X = np.concatenate([np.asarray(i["Eulerx"], np.float64) for i in instances])
        el = np.concatenate([np.asarray(i["elements"], np.int64) + node_off[k] for k, i in enumerate(instances)])
        prm = np.concatenate([np.tile(np.pad(np.asarray(i["params"], np.float64), (0, 3 - len(i["params"]))),
                                      (np.asarray(i["elements"]).shape[0], 1)) for i in instances])
        self.nnode, self.nelem = P.shape[0], el.shape[0]
        self.points = _to_dev(P, torch.float64, self.device)
        self.x = _to_dev(X, torch.float64, self.device)
        self.elements = _to_dev(el, torch.int64, self.device)
        self.eparams = _to_dev(prm, torch.float64, self.device)
        self.Jm = _to_dev(Jm, torch.float64, self.device)
        self.w = _to_dev(np.ravel(AllGauss), torch.float64, self.device)
        self.nq = self.w.shape[0]
        ind, ptr, dl, dg = device_sparsity(self.elements, self.nnode, 3, maps=maps)
        self.indices, self.indptr, self.dl, self.dg = ind, ptr, dl, dg
        self.nnz = ind.shape[0]
        self.flags = torch.zeros(1, dtype=torch.int32, device=self.device)

    def assemble(self, V=None, T=None, mixed=False, stream=None):
        """All instances at once. FP64 CSR values (mixed=False) or FP32 split-BF16 values."""
        L = N.lib()
        if T is None:
            T = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        if mixed:
            V = torch.zeros(self.nnz, dtype=torch.float32, device=self.device) if V is None else V
            st = L.fl_GlobalAssemblyDF_Mixed(self.mat_id, _ptr(self.points), _ptr(self.elements), _ptr(self.x),
                                             _ptr(self.Jm), _ptr(self.w), self.nq, self.nelem, self.npe, self.nnode, 1,
                                             _ptr(self.indptr), _ptr(self.indices), _ptr(self.dl), _ptr(self.dg),
                                             _ptr(V), _ptr(T), 0.0, 0.0, 0.0, 0.0, 0.0, None, _ptr(self.eparams),
                                             _ptr(self.flags), stream or _stream())
            N.check(st, "fl_GlobalAssemblyDF_Mixed")
        else:
            V = torch.zeros(self.nnz, dtype=torch.float64, device=self.device) if V is None else V
            st = L.fl_GlobalAssemblyDF_Batched(self.mat_id, _ptr(self.points), _ptr(self.elements), _ptr(self.x),
                                               _ptr(self.Jm), _ptr(self.w), self.nq, self.nelem, self.npe, self.nnode,
                                               1, _ptr(self.eparams), _ptr(self.indptr), _ptr(self.indices),
                                               _ptr(self.dl), _ptr(self.dg), _ptr(V), _ptr(T), _ptr(self.flags),
                                               stream or _stream())
            N.check(st, "fl_GlobalAssemblyDF_Batched")
        return V, T

    def instance_csr(self, k, V):
        """(indptr, indices, data) of instance k, in its own node numbering (host arrays)."""
        r0, r1 = 3 * int(self.node_off[k]), 3 * int(self.node_off[k + 1])
        ptr = self.indptr[r0:r1 + 1].cpu().numpy().astype(np.int64)
        a, b = ptr[0], ptr[-1]
        ind = self.indices[a:b].cpu().numpy() - r0
        return (ptr - a).astype(np.int32), ind.astype(np.int32), V[a:b].cpu().numpy()

    def autotune(self, candidates=None, reps=2):
        """Times the FP64 assembly for each Gauss-point chunk candidate; installs the fastest."""
        L = N.lib()
        if candidates is None:
            candidates = sorted({c for c in (1, 2, 3, 4, 6, 8, 12, 16) if c <= self.nq})
        best = None
        V = torch.zeros(self.nnz, dtype=torch.float64, device=self.device)
        T = torch.zeros(self.nnode * 3, dtype=torch.float64, device=self.device)
        for qc in candidates:
            N.check(L.fl_SetAssemblyTuning(self.npe, self.nq, int(qc)), "fl_SetAssemblyTuning")
            try:
                self.assemble(V, T)
            except N.FlorenceGB300Error:
                continue  # the chunk does not fit in shared memory
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                self.assemble(V, T)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            if best is None or ms < best[1]:
                best = (qc, ms)
        N.check(L.fl_SetAssemblyTuning(self.npe, self.nq, int(best[0])), "fl_SetAssemblyTuning")
        return dict(npe=self.npe, nq=self.nq, gauss_chunk=best[0], ms=best[1])


def config4_instances(n_instances=512, seed=2):
    """The batched configuration: per instance a cube of n^3 hexes, n ~ U{2..12}, order
    p ~ U{1..4}, neo-Hookean mu ~ U(0.5, 2), lambda ~ U(5, 50), displacement U(-0.01, 0.01)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_instances):
        n = int(rng.integers(2, 13))
        p = int(rng.integers(1, 5))
        mu = float(rng.uniform(0.5, 2.0))
        lamb = float(rng.uniform(5.0, 50.0))
        out.append(dict(k=k, n=n, p=p, mu=mu, lamb=lamb, seed=int(rng.integers(0, 2 ** 31))))
    return out


def hex_tables(p):
    """(pattern, Jm, AllGauss) of the reference's hex of order p with its default quadrature,
    taken from the golden fixtures."""
    import os
    from . import meshes
    here = os.path.dirname(os.path.abspath(__file__))
    name = {1: "hex_p1_nh", 2: "box_hex_p2_nh_big", 3: "hex_p3_nh", 4: "hex_p4_nh"}[p]
    d = np.load(os.path.join(here, "..", "tests", "golden", name + ".npz"))
    return meshes.local_pattern(d["points"], d["elements"], 0, "hex"), d["Jm"], d["AllGauss"]


def build_instance(spec, pattern):
    from . import meshes
    P, el = meshes.structured_hex((spec["n"],) * 3, (1.0, 1.0, 1.0), pattern)
    x = P + np.random.default_rng(spec["seed"]).uniform(-0.01, 0.01, P.shape)
    return dict(points=P, elements=el, Eulerx=x, params=(spec["mu"], spec["lamb"]))
