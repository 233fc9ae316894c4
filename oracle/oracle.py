"""ctypes front-end of the CPU oracle (florence_oracle.c).

TEST INFRASTRUCTURE ONLY. Imported by tests/, by ``__graft_entry__.smoke()`` and by
``bench.py``'s CPU-baseline leg, always as the checker or the timed CPU reference,
never as part of the product path. It restates the reference's assembly
(Florence/FiniteElements/Assembly/_Assembly_/_LowLevelAssemblyDF_.h:8-176 and
the files cited in florence_oracle.c) and is pinned against golden vectors made by
the reference's own code (tests/golden/make_golden.py, tests/test_oracle.py).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
FAST_PATH = os.path.join(HERE, "liboracle_fast.so")
MATERIALS = {"NeoHookean": 1, "MooneyRivlin": 2, "NearlyIncompressibleMooneyRivlin": 3, "LinearElastic": 10,
             "AnisotropicMooneyRivlin_1": 11}

_libs = {}


def build(force=False):
    """Compile liboracle.so (checker) and liboracle_fast.so (timed baseline) from florence_oracle.c."""
    src = os.path.join(HERE, "florence_oracle.c")
    for path in (LIB_PATH, FAST_PATH):
        if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            subprocess.check_call(["make", "-s", "-C", HERE, "-B", os.path.basename(path)])
    return LIB_PATH


def lib(fast=False):
    """The checker build, or with fast=True the build with the reference's optimisation flags."""
    key = "fast" if fast else "ieee"
    if key not in _libs:
        build()
        L = ctypes.CDLL(FAST_PATH if fast else LIB_PATH)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_assemble_df.argtypes = [ctypes.c_int, P, P, P, P, P, P, i64, i64, i64, ctypes.c_int, ctypes.c_int,
                                      P, P, P, P, P, P, P, P, ctypes.c_int]
        L.orc_element_matrices.argtypes = [ctypes.c_int, P, P, P, P, P, P, i64, i64, ctypes.c_int, P, i64, P, P]
        L.orc_internal_force.argtypes = [ctypes.c_int, P, P, P, P, P, P, i64, i64, i64, P, ctypes.c_int]
        L.orc_lumped_mass.argtypes = [ctypes.c_double, P, P, P, P, P, i64, i64, i64, P]
        L.orc_sparsity_nnz.argtypes = [P, i64, i64, i64, i64]
        L.orc_sparsity_nnz.restype = i64
        L.orc_sparsity.argtypes = [P, i64, i64, i64, i64, P, P, P, P]
        L.orc_set_orientations.argtypes = [P]
        _libs[key] = L
    return _libs[key]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class _orientations:
    """Per-element fibre directions [nelem][3] (AnisotropicMooneyRivlin_1) for the calls made
    within the block; the array is kept alive and the pointer cleared afterwards."""

    def __init__(self, L, orientations):
        self.L = L
        self.a = None if orientations is None else _c(orientations, np.float64)

    def __enter__(self):
        self.L.orc_set_orientations(_p(self.a))

    def __exit__(self, *exc):
        self.L.orc_set_orientations(None)


def max_threads():
    return int(lib().orc_max_threads())


def sparsity(elements, nnode, nvar=3, maps=True):
    """Returns (indices, indptr, data_local, data_global) like the reference's ComputeSparsityPattern."""
    el = _c(elements, np.int64)
    nelem, npe = el.shape
    nnz = lib().orc_sparsity_nnz(_p(el), nelem, npe, nnode, nvar)
    if nnz < 0:
        raise ValueError("every node must belong to at least one element")
    indptr = np.zeros(nnode * nvar + 1, np.int32)
    indices = np.zeros(nnz, np.int32)
    cap = (npe * nvar) ** 2 * nelem
    dl = np.zeros(cap, np.int32) if maps else None
    dg = np.zeros(cap, np.int32) if maps else None
    lib().orc_sparsity(_p(el), nelem, npe, nnode, nvar, _p(indptr), _p(indices), _p(dl), _p(dg))
    return indices, indptr, dl, dg


def assemble_df(material, params, points, elements, Eulerx, Jm, AllGauss, mode="csr", sparsity_arrays=None,
                requires_geometry_update=1, nthreads=1, fast=False, orientations=None):
    """Global tangent and residual. mode: 'triplet' -> (I, J, V, T); 'csr'/'squeeze' -> (V, T)."""
    mat = MATERIALS[material]
    prm = _c(params, np.float64)
    X = _c(points, np.float64)
    el = _c(elements, np.int64)
    x = _c(Eulerx, np.float64)
    jm = _c(Jm, np.float64)
    w = _c(np.ravel(AllGauss), np.float64)
    nelem, npe = el.shape
    nq = w.shape[0]
    ndof = 3 * npe
    T = np.zeros(X.shape[0] * 3)
    if mode == "triplet":
        I = np.zeros(nelem * ndof * ndof, np.int32)
        J = np.zeros_like(I)
        V = np.zeros(nelem * ndof * ndof)
        with _orientations(lib(fast), orientations):
            lib(fast).orc_assemble_df(mat, _p(prm), _p(X), _p(el), _p(x), _p(jm), _p(w), nelem, npe, nq,
                                      requires_geometry_update, 0, _p(I), _p(J), _p(V), _p(T), None, None, None, None,
                                      nthreads)
        return I, J, V, T
    indices, indptr, dl, dg = sparsity_arrays
    indices = _c(indices, np.int32)
    indptr = _c(indptr, np.int32)
    V = np.zeros(indices.shape[0])
    m = 1 if mode == "csr" else 2
    with _orientations(lib(fast), orientations):
        lib(fast).orc_assemble_df(mat, _p(prm), _p(X), _p(el), _p(x), _p(jm), _p(w), nelem, npe, nq,
                                  requires_geometry_update, m, None, None, _p(V), _p(T), _p(indptr), _p(indices),
                                  _p(_c(dl, np.int32) if m == 1 else None), _p(_c(dg, np.int32) if m == 1 else None),
                                  nthreads)
    return V, T


def element_matrices(material, params, points, elements, Eulerx, Jm, AllGauss, elem_ids, requires_geometry_update=1,
                     orientations=None):
    mat = MATERIALS[material]
    el = _c(elements, np.int64)
    npe = el.shape[1]
    w = _c(np.ravel(AllGauss), np.float64)
    ids = _c(elem_ids, np.int64)
    ndof = 3 * npe
    Ke = np.zeros((ids.shape[0], ndof, ndof))
    te = np.zeros((ids.shape[0], ndof))
    with _orientations(lib(), orientations):
        lib().orc_element_matrices(mat, _p(_c(params, np.float64)), _p(_c(points, np.float64)), _p(el),
                                   _p(_c(Eulerx, np.float64)), _p(_c(Jm, np.float64)), _p(w), npe, w.shape[0],
                                   requires_geometry_update, _p(ids), ids.shape[0], _p(Ke), _p(te))
    return Ke, te


def internal_force(material, params, points, elements, Eulerx, Jm, AllGauss, nthreads=1, orientations=None):
    mat = MATERIALS[material]
    el = _c(elements, np.int64)
    w = _c(np.ravel(AllGauss), np.float64)
    T = np.zeros(np.shape(points)[0] * 3)
    with _orientations(lib(), orientations):
        lib().orc_internal_force(mat, _p(_c(params, np.float64)), _p(_c(points, np.float64)), _p(el),
                                 _p(_c(Eulerx, np.float64)), _p(_c(Jm, np.float64)), _p(w), el.shape[0], el.shape[1],
                                 w.shape[0], _p(T), nthreads)
    return T


def lumped_mass(rho, points, elements, Jm, AllGauss, Bases):
    el = _c(elements, np.int64)
    w = _c(np.ravel(AllGauss), np.float64)
    M = np.zeros(np.shape(points)[0] * 3)
    lib().orc_lumped_mass(float(rho), _p(_c(points, np.float64)), _p(el), _p(_c(Jm, np.float64)), _p(w),
                          _p(_c(Bases, np.float64)), el.shape[0], el.shape[1], w.shape[0], _p(M))
    return M


def consistent_mass(rho, points, elements, Jm, AllGauss, Bases, nvar=3):
    """Dense [nvar*N, nvar*N] consistent mass (mass_type 1 of _GenericConstantMassIntegrand_,
    VariationalPrinciple/_Mass_/_MassIntegrand_.h:249-400, with the constant integrand
    rho N N^T of VariationalPrinciple.py:255-290): per element sum_g rho N_a N_b w_g |det dX/dxi|
    on the nvar diagonal of every node pair. numpy, for small meshes."""
    P = np.asarray(points, np.float64)
    el = np.asarray(elements, np.int64)
    Jm = np.asarray(Jm, np.float64)                     # [3, npe, nq]
    w = np.ravel(AllGauss).astype(np.float64)
    B = np.asarray(Bases, np.float64)                   # [npe, nq]
    n = P.shape[0] * nvar
    M = np.zeros((n, n))
    for e in range(el.shape[0]):
        X = P[el[e]]                                    # [npe, 3]
        G = np.einsum("dag,ak->gdk", Jm, X)             # dX/dxi per Gauss point
        wdet = w * np.abs(np.linalg.det(G))
        m = np.einsum("ag,bg,g->ab", B, B, wdet) * rho
        for i in range(nvar):
            M[np.ix_(nvar * el[e] + i, nvar * el[e] + i)] += m
    return M


def external_traction(faces, neumann_flags, applied_neumann, Bases, AllGauss, nnode):
    """F [nnode*3] of AssembleExternalTractionForces (Assembly.py:451-514): every flagged face adds
    applied_neumann[face, i] * sum_g Bases[a, g] w_g to its node a, component i (parent weights)."""
    faces = np.asarray(faces, np.int64)
    s = np.asarray(Bases, np.float64) @ np.ravel(AllGauss).astype(np.float64)  # sum_g N_a(g) w_g
    F = np.zeros(nnode * 3)
    for f in np.nonzero(np.ravel(neumann_flags))[0]:
        for a, nd in enumerate(faces[f]):
            F[3 * nd:3 * nd + 3] += np.asarray(applied_neumann[f], np.float64)[:3] * s[a]
    return F


def body_forces(elements, Bases, AllGauss, rho, nnode):
    """F [nnode*3] of AssembleBodyForces (Assembly.py:516-560): -rho * sum_g Bases[a, g] w_g on the z
    component of every element node."""
    el = np.asarray(elements, np.int64)
    s = np.asarray(Bases, np.float64) @ np.ravel(AllGauss).astype(np.float64)
    F = np.zeros(nnode * 3)
    np.add.at(F, 3 * el.ravel() + 2, np.tile(-rho * s, el.shape[0]))
    return F
