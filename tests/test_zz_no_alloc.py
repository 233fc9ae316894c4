"""GPU test of the allocation-free assembly entry point (fl_GlobalAssemblyDF_noalloc).

Some callers cannot allocate device memory while they run (an application that reserves all its
device memory at start-up, or a solver loop that must not stall on cudaMalloc/cudaFree, which can
synchronise the device, or fail under memory pressure). For them the library keeps a fixed 32 MiB
device array as the Gauss-point scratch of this one entry point. This test calls it through the C
ABI, twice in a row (the array is reused and keeps the previous call's contents), in each
contraction arithmetic, and compares each result with the regular entry point's, within the parity
tolerance of the other tests. It checks the entry point's defining property through the driver's
high-water mark of the device's stream-ordered memory pool (the regular entry point raises it, this
one must not), and that a mesh too large for the array is rejected. The file name makes pytest
collect it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8  # CUmemPool_attribute (cuda.h)


class _PoolHighWater:
    """High-water mark of the current memory pool of device 0 (the pool cudaMallocAsync draws
    from), through the driver API: reset() zeroes it, value() reads it."""

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int(0)
        assert self.cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetMemPool(ctypes.byref(self.pool), dev) == 0

    def reset(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def value(self):
        v = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(v)) == 0
        return v.value


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _call(L, fn_name, material_number, d, bufs, mode, nelem=None):
    """Calls an assembly entry point with the reference's argument list (device buffers)."""
    mat = str(d["material"])
    prm = tuple(float(p) for p in d["params"])
    if mat == "NeoHookean":
        mu, mu1, mu2, lamb = prm[0], 0.0, 0.0, prm[1]
    else:
        mu, mu1, mu2, lamb = 0.0, prm[0], prm[1], prm[2]
    npe = d["elements"].shape[1]
    nq = d["AllGauss"].shape[0]
    nelem = d["elements"].shape[0] if nelem is None else nelem
    args = [_p(bufs["points"]), _p(bufs["elements"]), _p(bufs["x"]), None, None, _p(bufs["Jm"]), _p(bufs["w"]),
            3, 3, nq, nelem, npe, d["points"].shape[0], 6, 1, None, None,
            _p(bufs["I"]), _p(bufs["J"]), _p(bufs["V"]), _p(bufs["T"]), 1 if mode == "triplet" else 0, 0,
            _p(bufs.get("dl")), _p(bufs.get("dg")), None, None,
            1.0, mu, mu1, mu2, 0.0, 0.0, lamb, 0.0, 0.0, 0.0, 0.0, None, _p(bufs["flags"]),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)]
    fn = getattr(L, fn_name)
    if material_number is not None:
        return fn(material_number, *args)
    return fn(*args)


def _buffers(d, mode):
    dev = torch.device("cuda")
    b = dict(points=torch.from_numpy(d["points"]).to(dev), elements=torch.from_numpy(d["elements"]).to(dev),
             x=torch.from_numpy(d["Eulerx"]).to(dev), Jm=torch.from_numpy(np.ascontiguousarray(d["Jm"])).to(dev),
             w=torch.from_numpy(np.ravel(d["AllGauss"]).copy()).to(dev),
             T=torch.zeros(d["points"].shape[0] * 3, dtype=torch.float64, device=dev),
             flags=torch.zeros(1, dtype=torch.int32, device=dev))
    ndof = 3 * d["elements"].shape[1]
    cap = d["elements"].shape[0] * ndof * ndof
    if mode == "csr":
        b["I"] = torch.from_numpy(d["sp_indptr"]).to(dev)
        b["J"] = torch.from_numpy(d["sp_indices"]).to(dev)
        b["dl"] = torch.from_numpy(d["sp_data_local"]).to(dev)
        b["dg"] = torch.from_numpy(d["sp_data_global"]).to(dev)
        b["V"] = torch.zeros(d["sp_indices"].shape[0], dtype=torch.float64, device=dev)
    else:
        b["I"] = torch.zeros(cap, dtype=torch.int32, device=dev)
        b["J"] = torch.zeros(cap, dtype=torch.int32, device=dev)
        b["V"] = torch.zeros(cap, dtype=torch.float64, device=dev)
    return b


def _zero(b):
    for k in ("V", "T", "flags"):
        b[k].zero_()


@pytest.fixture
def arithmetic():
    """Yields a setter of the contraction arithmetic and restores the library's default after."""
    import florence_gb300 as fl
    old = fl.get_arithmetic()
    yield fl.set_arithmetic
    fl.set_arithmetic(old)


@pytest.mark.parametrize("arith", ["float_pair", "fp64", "tensor", "reference_tensor"])
@pytest.mark.parametrize("case,mode", [("hex_p2_nh_q5", "csr"), ("tet_p3_mr_jitter", "triplet")])
def test_noalloc_matches_regular_entry_point_twice(case, mode, arith, arithmetic):
    from florence_gb300 import _native as N
    L = N.lib()
    arithmetic(arith)
    d = load_golden(case)
    mat = str(d["material"])
    mat_no = N.FL_MATERIAL_NEOHOOKEAN if mat == "NeoHookean" else N.FL_MATERIAL_MOONEYRIVLIN
    b = _buffers(d, mode)
    pool = _PoolHighWater()
    torch.cuda.synchronize()
    pool.reset()
    assert _call(L, "fl_GlobalAssemblyDF__" + mat + "_", None, d, b, mode) == N.FL_OK
    torch.cuda.synchronize()
    assert pool.value() > 0  # the regular entry point draws its scratch from the pool
    V_ref, T_ref = b["V"].cpu().numpy().copy(), b["T"].cpu().numpy().copy()
    I_ref, J_ref = b["I"].cpu().numpy().copy(), b["J"].cpu().numpy().copy()
    assert int(b["flags"].item()) == 0
    for call in range(2):
        _zero(b)
        if mode == "triplet":
            b["I"].zero_()
            b["J"].zero_()
        torch.cuda.synchronize()
        pool.reset()
        assert _call(L, "fl_GlobalAssemblyDF_noalloc", mat_no, d, b, mode) == N.FL_OK, call
        torch.cuda.synchronize()
        assert pool.value() == 0, call  # nothing drawn from the stream-ordered allocator
        assert int(b["flags"].item()) == 0
        assert rel_fro(b["V"].cpu().numpy(), V_ref) < TOL, call
        assert rel_fro(b["T"].cpu().numpy(), T_ref) < TOL, call
        if mode == "triplet":
            assert np.array_equal(b["I"].cpu().numpy(), I_ref) and np.array_equal(b["J"].cpu().numpy(), J_ref)
    # and against the reference's own values
    if mode == "csr":
        assert rel_fro(b["V"].cpu().numpy(), d["K_data"]) < TOL
    assert rel_fro(b["T"].cpu().numpy(), d["T"]) < TOL


def test_noalloc_rejects_mesh_larger_than_its_array():
    """nelem * ngauss * 432 bytes above the fixed array: FL_ERR_CAPACITY, nothing launched
    (the check precedes every device access)."""
    from florence_gb300 import _native as N
    L = N.lib()
    d = load_golden("hex_p2_nh_q5")
    b = _buffers(d, "csr")
    too_many = N.FL_NOALLOC_SCRATCH_BYTES // (432 * d["AllGauss"].shape[0]) + 1
    st = _call(L, "fl_GlobalAssemblyDF_noalloc", N.FL_MATERIAL_NEOHOOKEAN, d, b, "csr", nelem=too_many)
    assert st == N.FL_ERR_CAPACITY
    torch.cuda.synchronize()
    assert float(b["V"].abs().sum()) == 0.0 and float(b["T"].abs().sum()) == 0.0


def test_noalloc_rejects_materials_outside_its_contract():
    """Only neo-Hookean and Mooney-Rivlin: any other material number is FL_ERR_UNSUPPORTED."""
    from florence_gb300 import _native as N
    L = N.lib()
    d = load_golden("hex_p2_nh_q5")
    b = _buffers(d, "csr")
    for mat_no in (N.FL_MATERIAL_LINEARELASTIC, N.FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN,
                   N.FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1, 12345):
        assert _call(L, "fl_GlobalAssemblyDF_noalloc", mat_no, d, b, "csr") == N.FL_ERR_UNSUPPORTED
