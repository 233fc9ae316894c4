"""Displacement-potential (electromechanics) assembly on the GPU: three displacements and the
electric potential per node (nvar 4, global dof 4 n + v), IsotropicElectroMechanics_108, _106, _105,
_101, _0, SteinmannModel and Piezoelectric_100 (one fibre direction per element).

* ``DPFAssembler`` keeps the mesh, function-space tables and the nvar=4 CSR pattern on the device
  and assembles the tangent and residual from device coordinates and potentials
  (``fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_``).
* ``_LowLevelAssemblyDPF__IsotropicElectroMechanics_<108|106|105|101|0>_``,
  ``_LowLevelAssemblyDPF__SteinmannModel_`` and ``_LowLevelAssemblyDPF__Piezoelectric_100_`` are the
  drop-ins for the reference's
  Cython wrapper (Florence/FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDPF_.pyx:53-160):
  the reference's dispatcher (_LowLevelAssembly_.py:45-83) finds it by name when
  ``formulation.fields == "electro_mechanics"``; ``florence_gb300.install`` registers them.

There is no CPU path: a missing library raises.
"""
import numpy as np
import torch

from . import _native as N
from .assembly import _HOST, _check_flags, _ptr, _stream, _to_dev, device_sparsity

NVAR = 4
# material -> (entry point, parameter names in the reference's order, AOT_Assembler.py:153-168)
MATERIALS = {"IsotropicElectroMechanics_108": ("fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_",
                                               ("mu1", "mu2", "lamb", "eps_2")),
             "IsotropicElectroMechanics_101": ("fl_GlobalAssemblyDPF__IsotropicElectroMechanics_101_",
                                               ("mu", "lamb", "eps_1")),
             "IsotropicElectroMechanics_0": ("fl_GlobalAssemblyDPF__IsotropicElectroMechanics_0_",
                                             ("mu", "lamb", "eps_1")),
             "IsotropicElectroMechanics_106": ("fl_GlobalAssemblyDPF__IsotropicElectroMechanics_106_",
                                               ("mu1", "mu2", "lamb", "eps_1", "eps_2")),
             "IsotropicElectroMechanics_105": ("fl_GlobalAssemblyDPF__IsotropicElectroMechanics_105_",
                                               ("mu1", "mu2", "lamb", "eps_1", "eps_2")),
             "SteinmannModel": ("fl_GlobalAssemblyDPF__SteinmannModel_", ("mu", "lamb", "c1", "c2", "eps_1")),
             "Piezoelectric_100": ("fl_GlobalAssemblyDPF__Piezoelectric_100_",
                                   ("mu1", "mu2", "mu3", "lamb", "eps_1", "eps_2", "eps_3"))}
# transversely isotropic: one fibre direction per element (material.anisotropic_orientations)
ORIENTED = {"Piezoelectric_100"}
# material attributes passed in other scalar slots of the reference's argument list
# (_LowLevelAssemblyDPF_.pyx as AOT_Assembler.py:202-203 rewrites it for the Steinmann model)
_ABI_SLOT = {"c1": "eps_3", "c2": "eps_2"}
_ABI_SCALARS = ("rho", "mu", "mu1", "mu2", "mu3", "mue", "lamb", "eps_1", "eps_2", "eps_3", "eps_e")


class DPFAssembler:
    """points [N,3], elements [E,npe], Jm [3,npe,nq], AllGauss [nq]; params (mu1, mu2, lamb, eps_2)
    for IsotropicElectroMechanics_108, (mu1, mu2, lamb, eps_1, eps_2) for _106 and _105, (mu, lamb, eps_1)
    for _101 and _0, (mu, lamb, c1, c2, eps_1) for SteinmannModel, (mu1, mu2, mu3, lamb, eps_1, eps_2,
    eps_3) with `orientations` [E,3] for Piezoelectric_100; mode 'csr' (element-to-nonzero
    maps), 'squeeze' (row search) or 'triplet'."""

    def __init__(self, points, elements, Jm, AllGauss, params, material="IsotropicElectroMechanics_108",
                 mode="csr", device="cuda", requires_geometry_update=1, sparsity=None, orientations=None):
        if material not in MATERIALS:
            raise NotImplementedError("the GB300 DPF assembly provides " + ", ".join(MATERIALS))
        self.device = torch.device(device)
        self.points = _to_dev(points, torch.float64, self.device)
        self.elements = _to_dev(elements, torch.int64, self.device)
        self.Jm = _to_dev(Jm, torch.float64, self.device)
        self.w = _to_dev(np.ravel(AllGauss) if not isinstance(AllGauss, torch.Tensor) else AllGauss.reshape(-1),
                         torch.float64, self.device)
        self.nnode = self.points.shape[0]
        self.nelem, self.npe = self.elements.shape
        self.nq = self.w.shape[0]
        self.ndof = NVAR * self.npe
        self.entry, names = MATERIALS[material]
        self.params = tuple(float(p) for p in params)
        if len(self.params) != len(names):
            raise ValueError("%s takes (%s)" % (material, ", ".join(names)))
        given = {_ABI_SLOT.get(k, k): v for k, v in zip(names, self.params)}
        self.scalars = tuple(given.get(k, 1.0 if k == "rho" else 0.0) for k in _ABI_SCALARS)
        self.orient = None
        if material in ORIENTED:
            if orientations is None:
                raise ValueError(material + " needs one fibre direction per element (orientations)")
            self.orient = _to_dev(np.asarray(orientations, np.float64).reshape(-1, 3)
                                  if not isinstance(orientations, torch.Tensor) else orientations.reshape(-1, 3),
                                  torch.float64, self.device)
            if self.orient.shape[0] != self.nelem:
                raise ValueError("orientations must hold one direction per element")
        self.mode = mode
        self.update = int(requires_geometry_update)
        self.flags = torch.zeros(1, dtype=torch.int32, device=self.device)
        if mode in ("csr", "squeeze"):
            if sparsity is None:
                sparsity = device_sparsity(self.elements, self.nnode, NVAR, maps=(mode == "csr"))
            ind, ptr, dl, dg = sparsity
            self.indices = _to_dev(ind, torch.int32, self.device)
            self.indptr = _to_dev(ptr, torch.int32, self.device)
            self.data_local = _to_dev(dl, torch.int32, self.device) if mode == "csr" else None
            self.data_global = _to_dev(dg, torch.int32, self.device) if mode == "csr" else None
            self.nnz = self.indices.shape[0]
        elif mode != "triplet":
            raise ValueError("mode must be 'csr', 'squeeze' or 'triplet'")

    def assemble(self, Eulerx, Eulerp, V=None, T=None, stream=None):
        """Tangent and residual at device coordinates Eulerx [N,3] and potentials Eulerp [N].
        Returns (V, T), or (I, J, V, T) in triplet mode; accumulates into V/T when given."""
        L = N.lib()
        x = Eulerx.contiguous()
        p = Eulerp.reshape(-1).contiguous()
        if T is None:
            T = torch.zeros(self.nnode * NVAR, dtype=torch.float64, device=self.device)
        if self.mode == "triplet":
            cap = self.nelem * self.ndof * self.ndof
            I = torch.empty(cap, dtype=torch.int32, device=self.device)
            J = torch.empty(cap, dtype=torch.int32, device=self.device)
            V = torch.empty(cap, dtype=torch.float64, device=self.device) if V is None else V
            Ip, Jp, dl, dg = I, J, None, None
        else:
            V = torch.zeros(self.nnz, dtype=torch.float64, device=self.device) if V is None else V
            Ip, Jp, dl, dg = self.indptr, self.indices, self.data_local, self.data_global
        st = getattr(L, self.entry)(
            _ptr(self.points), _ptr(self.elements), _ptr(x), _ptr(p), None, _ptr(self.Jm), _ptr(self.w), 3, NVAR,
            self.nq, self.nelem, self.npe, self.nnode, 9, self.update, None, None, _ptr(Ip), _ptr(Jp), _ptr(V),
            _ptr(T), 1 if self.mode == "triplet" else 0, 1 if self.mode == "squeeze" else 0, _ptr(dl), _ptr(dg),
            None, None, *self.scalars, _ptr(self.orient), _ptr(self.flags), stream or _stream())
        N.check(st, self.entry)
        if self.mode == "triplet":
            return I, J, V, T
        return V, T

    def check_flags(self, what="DPF assembly"):
        _check_flags(self.flags, what)
        self.flags.zero_()


def _low_level_dpf(name, fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    if formulation.ndim != 3 or formulation.nvar != NVAR:
        raise NotImplementedError("the GB300 DPF assembly covers three-dimensional electromechanics (nvar 4)")
    params = tuple(float(getattr(material, k)) for k in MATERIALS[name][1])
    recompute = bool(fem_solver.recompute_sparsity_pattern)
    # CSR output without uploading the two E*ndof^2 maps: each entry's position is found by row
    # search, which lands it where the maps would
    mode = "triplet" if recompute else "squeeze"
    sparsity = None if recompute else (fem_solver.indices, fem_solver.indptr, None, None)
    orient = getattr(material, "anisotropic_orientations", None) if name in ORIENTED else None
    asm = DPFAssembler(mesh.points, mesh.elements, function_space.Jm, function_space.AllGauss, params,
                       material=name, mode=mode, requires_geometry_update=fem_solver.requires_geometry_update,
                       sparsity=sparsity, orientations=orient)
    x = _to_dev(Eulerx, torch.float64, asm.device)
    p = _to_dev(np.ravel(Eulerp), torch.float64, asm.device)
    out = asm.assemble(x, p)
    host = [_HOST.to_host(t) for t in out]
    asm.check_flags("_LowLevelAssemblyDPF__" + name + "_")
    return tuple(host)


def _LowLevelAssemblyDPF__IsotropicElectroMechanics_108_(fem_solver, function_space, formulation, mesh, material,
                                                         Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _IsotropicElectroMechanics_108_ (mu1, mu2, lamb, eps_2)."""
    return _low_level_dpf("IsotropicElectroMechanics_108", fem_solver, function_space, formulation, mesh, material,
                          Eulerx, Eulerp)


def _LowLevelAssemblyDPF__IsotropicElectroMechanics_101_(fem_solver, function_space, formulation, mesh, material,
                                                         Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _IsotropicElectroMechanics_101_ (mu, lamb, eps_1)."""
    return _low_level_dpf("IsotropicElectroMechanics_101", fem_solver, function_space, formulation, mesh, material,
                          Eulerx, Eulerp)


def _LowLevelAssemblyDPF__IsotropicElectroMechanics_0_(fem_solver, function_space, formulation, mesh, material,
                                                       Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _IsotropicElectroMechanics_0_ (mu, lamb, eps_1)."""
    return _low_level_dpf("IsotropicElectroMechanics_0", fem_solver, function_space, formulation, mesh, material,
                          Eulerx, Eulerp)


def _LowLevelAssemblyDPF__IsotropicElectroMechanics_106_(fem_solver, function_space, formulation, mesh, material,
                                                         Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _IsotropicElectroMechanics_106_ (mu1, mu2, lamb, eps_1, eps_2)."""
    return _low_level_dpf("IsotropicElectroMechanics_106", fem_solver, function_space, formulation, mesh, material,
                          Eulerx, Eulerp)


def _LowLevelAssemblyDPF__IsotropicElectroMechanics_105_(fem_solver, function_space, formulation, mesh, material,
                                                         Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _IsotropicElectroMechanics_105_ (mu1, mu2, lamb, eps_1, eps_2)."""
    return _low_level_dpf("IsotropicElectroMechanics_105", fem_solver, function_space, formulation, mesh, material,
                          Eulerx, Eulerp)


def _LowLevelAssemblyDPF__SteinmannModel_(fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _SteinmannModel_ (mu, lamb, c1, c2, eps_1)."""
    return _low_level_dpf("SteinmannModel", fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp)


def _LowLevelAssemblyDPF__Piezoelectric_100_(fem_solver, function_space, formulation, mesh, material, Eulerx, Eulerp):
    """(I, J, V, T) if fem_solver.recompute_sparsity_pattern else (V, T) -- _LowLevelAssemblyDPF_.pyx:53-160
    as AOT_Assembler.py builds it for _Piezoelectric_100_ (mu1, mu2, mu3, lamb, eps_1, eps_2, eps_3 and the
    material's anisotropic_orientations, one fibre direction per element)."""
    return _low_level_dpf("Piezoelectric_100", fem_solver, function_space, formulation, mesh, material, Eulerx,
                          Eulerp)
