"""CPU-only checks of the C ABI: the library builds, loads, and exports every symbol the header declares."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "florence_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fl_\w+)\s*\(", text)))


def test_header_lists_expected_entry_points():
    syms = header_symbols()
    for s in ("fl_ComputeSparsityPattern", "fl_GlobalAssemblyDF__NeoHookean_", "fl_GlobalAssemblyDF__MooneyRivlin_",
              "fl_GlobalAssemblyExplicit_DF_DPF_", "fl_LumpedMass"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from florence_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from florence_gb300 import build
        build.build()
    L = _native.lib()
    missing = [s for s in header_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert sorted(_native.EXPORTS) == sorted(header_symbols())
    assert L.fl_status_string(0) == b"ok"


def test_workspace_size_is_pure_host_arithmetic():
    from florence_gb300 import _native
    L = _native.lib()
    a = L.fl_ComputeSparsityPattern_workspace_size(512, 27, 4913)
    b = L.fl_ComputeSparsityPattern_workspace_size(1024, 27, 4913)
    assert 0 < a < b


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from florence_gb300 import _native
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(ImportError):
        _native.lib()


def test_pcg_workspace_sizes():
    """The split mode carries a float-pair copy of the values (8 bytes per nonzero)."""
    from florence_gb300 import _native as N
    L = N.lib()
    base = L.fl_BlockJacobiPCG_workspace_size(3000, 100000, N.FL_PCG_F64)
    assert L.fl_BlockJacobiPCG_workspace_size(3000, 100000, N.FL_PCG_F32) == base
    assert L.fl_BlockJacobiPCG_workspace_size(3000, 100000, N.FL_PCG_F64_SPLIT) >= base + 8 * 100000


def test_host_side_settings_validate_their_arguments():
    """Process-wide settings are host-only calls: the contraction arithmetic (four names, the
    reference-tensor GEMMs by default) and the split-BF16 tiling (ranges checked, 0 = automatic)."""
    import florence_gb300 as fl
    from florence_gb300._native import FlorenceGB300Error
    assert fl.get_arithmetic() == "reference_tensor"
    for name in ("fp64", "tensor", "float_pair", "reference_tensor"):
        fl.set_arithmetic(name)
        assert fl.get_arithmetic() == name
    with fl.arithmetic("tensor"):
        assert fl.get_arithmetic() == "tensor"
    assert fl.get_arithmetic() == "reference_tensor"
    fl.set_tensor_core_tiling(2, 48)
    fl.set_tensor_core_tiling(0, 0)
    for bad in ((-1, 0), (17, 0), (0, -16), (0, 112)):
        with pytest.raises(FlorenceGB300Error):
            fl.set_tensor_core_tiling(*bad)


def test_new_entry_points_reject_bad_arguments_before_any_device_work():
    """The DPF, consistent-mass and mesher entry points validate their arguments on the host and
    return an error status before any CUDA call (dummy, never dereferenced pointers)."""
    import ctypes
    from florence_gb300 import _native
    L = _native.lib()
    dummy = ctypes.c_void_p(16)
    # DPF: nvar must be 4 and H_VoigtSize 9 (checked before anything is read)
    args = [dummy] * 7 + [3, 3, 8, 6, 10, 27, 9, 1, None, None, dummy, dummy, dummy, dummy, 1, 0, None, None, None,
                          None, 1.0, 1.0, 0.5, 0.3, 0.0, 0.0, 10.0, 1.0, 2.0, 0.0, 0.0, None, None, None]
    for name in ("fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_", "fl_GlobalAssemblyDPF__SteinmannModel_"):
        assert getattr(L, name)(*args) == _native.FL_ERR_ARG
    # material 108 without eps_2
    args108 = list(args)
    args108[7], args108[8], args108[35] = 3, 4, 0.0  # ndim, nvar, eps_2
    assert L.fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_(*args108) == _native.FL_ERR_ARG
    # consistent mass: ndim 2 is refused
    assert L.fl_ConsistentMass(dummy, dummy, dummy, dummy, dummy, 2, 3, 8, 6, 10, 27, 1.0, 1, 0, None, None, 0,
                               None, None, dummy, dummy, dummy, None, None) == _native.FL_ERR_ARG
    # mesher: an empty mesh is refused, an oversized layout is unsupported
    nn = ctypes.c_int64(0)
    lam = np.zeros((4, 4))
    np.fill_diagonal(lam, 1.0)
    assert L.fl_RaiseTetOrder(dummy, 10, dummy, 0, lam.ctypes.data, 4, None, 0, ctypes.byref(nn), dummy, dummy,
                              1 << 20, None) == _native.FL_ERR_ARG
    big = np.zeros((36, 4))
    assert L.fl_RaiseTetOrder(dummy, 10, dummy, 1, big.ctypes.data, 36, None, 0, ctypes.byref(nn), dummy, dummy,
                              1 << 20, None) == _native.FL_ERR_UNSUPPORTED
