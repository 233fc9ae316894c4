"""GPU tests of the reference-tensor contraction (FL_ARITH_REFERENCE_TENSOR, fl_reftensor.cu): the
FP64 element matrices of a tile of 14 elements as one tcgen05 GEMM of the pulled-back tangents
against the element type's constant reference tensor, six BF16 digit planes per operand.

* every golden case the kernel takes (4-, 8-, 10- and 20-node elements, at most 15 Gauss points)
  against the reference's CSR tangent and residual at 1e-12, both CSR scatter modes, through the
  reference-signature entry point (block offsets built in the call) and through the
  device-resident assembler (block offsets built once);
* the block offsets against the pattern (numpy), bit-exact;
* a CSR whose node rows differ (no node blocks): every entry lands in its column through the
  row-search fallback, the extra entries stay zero;
* a mesh of a hundred tiles (several per CTA, a partial last tile) under a finite deformation,
  three materials, against the oracle;
* accumulation (+=) like the reference's outputs.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rt_cases():
    from florence_gb300.assembly import rt_supported
    out = []
    for c in golden_cases():
        d = load_golden(c)
        if rt_supported(d["elements"].shape[1], np.ravel(d["AllGauss"]).shape[0]):
            out.append(c)
    return out


def _asm(fl, d, mode, **kw):
    kw.setdefault("requires_geometry_update", int(d["update"]))
    if "orientations" in d:
        kw.setdefault("orientations", d["orientations"])
    return fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], str(d["material"]),
                              tuple(d["params"]), mode=mode, **kw)


def test_cases_exist():
    assert {"tet_p3_mr_jitter", "tet_p2_mr", "hex_p1_nh"} <= set(_rt_cases())


@pytest.mark.parametrize("case", _rt_cases())
@pytest.mark.parametrize("mode", ["csr", "squeeze"])
def test_reference_tensor_matches_reference(case, mode):
    import florence_gb300 as fl
    d = load_golden(case)
    asm = _asm(fl, d, mode)
    x = torch.from_numpy(d["Eulerx"]).cuda()
    with fl.arithmetic("reference_tensor"):
        V, T = asm.assemble(x)            # device-resident: block offsets built once, kept
        torch.cuda.synchronize()
        asm.check_flags()
        assert asm._boff is not None
        assert rel_fro(V.cpu().numpy(), d["K_data"]) < TOL
        assert rel_fro(T.cpu().numpy(), d["T"]) < TOL
        asm._boff = None                  # the reference-signature entry point builds them itself
        L = fl._native.lib()
        from florence_gb300.assembly import _DF_ENTRY, _abi_params, _ptr, _stream
        mu, mu1, mu2, lamb, mu3 = _abi_params(asm.mat_id, asm.params)
        V2 = torch.zeros_like(V)
        T2 = torch.zeros_like(T)
        st = getattr(L, _DF_ENTRY[asm.mat_id])(
            _ptr(asm.points), _ptr(asm.elements), _ptr(x), None, None, _ptr(asm.Jm), _ptr(asm.w), 3, 3, asm.nq,
            asm.nelem, asm.npe, asm.nnode, 6, asm.update, None, None, _ptr(asm.indptr), _ptr(asm.indices), _ptr(V2),
            _ptr(T2), 0, 1 if mode == "squeeze" else 0, _ptr(asm.data_local), _ptr(asm.data_global), None, None, 1.0,
            mu, mu1, mu2, mu3, 0.0, lamb, 0.0, 0.0, 0.0, 0.0, _ptr(asm.orient), _ptr(asm.flags), _stream())
        assert st == 0
        torch.cuda.synchronize()
        asm.check_flags()
    assert rel_fro(V2.cpu().numpy(), d["K_data"]) < TOL
    assert rel_fro(T2.cpu().numpy(), d["T"]) < TOL


@pytest.mark.parametrize("case", ["tet_p3_mr_jitter", "tet_p2_mr", "hex_p1_nh"])
def test_block_offsets_bit_exact(case):
    import florence_gb300 as fl
    d = load_golden(case)
    asm = _asm(fl, d, "csr")
    boff = asm.block_offsets().cpu().numpy()
    torch.cuda.synchronize()
    asm.check_flags()
    ptr, ind, el = d["K_indptr"], d["K_indices"], d["elements"].astype(np.int64)
    npe = el.shape[1]
    ref = np.empty((el.shape[0], npe, npe), np.int32)
    for e in range(el.shape[0]):
        for a in range(npe):
            row = 3 * el[e, a]
            cols = ind[ptr[row]:ptr[row + 1]]
            for b in range(npe):
                ref[e, a, b] = int(np.searchsorted(cols, 3 * el[e, b]))
    assert np.array_equal(boff, ref)


def _padded_csr(indptr, indices, every=3, phase=1):
    rows, pos, ptr = [], [], [0]
    for r in range(len(indptr) - 1):
        cols = list(indices[indptr[r]:indptr[r + 1]])
        if r % every == phase:
            c = next(c for c in range(len(cols) + 1) if c not in set(cols))
            cols = sorted(cols + [c])
        base = ptr[-1]
        keep = set(indices[indptr[r]:indptr[r + 1]])
        pos += [base + j for j, c in enumerate(cols) if c in keep]
        rows += cols
        ptr.append(len(rows))
    return np.array(ptr, np.int32), np.array(rows, np.int32), np.array(pos)


def test_row_search_without_node_blocks():
    import florence_gb300 as fl
    d = load_golden("tet_p3_mr_jitter")
    ptr, ind, pos = _padded_csr(d["K_indptr"], d["K_indices"])
    asm = _asm(fl, d, "squeeze", sparsity=(ind, ptr, None, None))
    with fl.arithmetic("reference_tensor"):
        V, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
        torch.cuda.synchronize()
        asm.check_flags()
    assert (asm._boff.cpu().numpy() == -1).any()   # some blocks fall back to the row search
    v = V.cpu().numpy()
    assert rel_fro(v[pos], d["K_data"]) < TOL
    extra = np.setdiff1d(np.arange(v.shape[0]), pos)
    assert extra.size > 0 and np.all(v[extra] == 0.0)


@pytest.mark.parametrize("material,params", [("MooneyRivlin", (0.5, 0.5, 20.0)), ("NeoHookean", (1.0, 10.0)),
                                             ("NearlyIncompressibleMooneyRivlin", (0.5, 0.5, 50.0))])
def test_many_tiles_against_oracle(oracle, material, params):
    """A jittered tet p=3 box of ~1 300 elements (a hundred tiles, several per CTA, a partial last
    tile) under a finite deformation: the reference-tensor tangent and residual against the oracle,
    to 1e-12 or twice the spread of two FP64 evaluations of the reference algorithm (the mesh's
    sliver tetrahedra make its assembled values sensitive to FP64 rounding order); the float-pair
    contraction alongside for comparison."""
    import bench
    import florence_gb300 as fl
    from florence_gb300 import meshes
    t = np.load(bench.os.path.join(bench.GOLDEN, "tet_p3_mr_jitter.npz"))
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((12, 4, 4), (3.0, 1.0, 1.0), 5, pat)
    x = P + bench.smooth_displacement(P, seed=9) * 10.0
    asm = fl.DeviceAssembler(P, el, t["Jm"], t["AllGauss"], material, params, mode="csr")
    xd = torch.from_numpy(x).cuda()
    V1, T1 = asm.assemble(xd)
    with fl.arithmetic("reference_tensor"):
        V2, T2 = asm.assemble(xd)
        V3 = V2.clone()
        T3 = T2.clone()
        asm.assemble(xd, V=V3, T=T3)      # accumulates
        torch.cuda.synchronize()
    asm.check_flags()
    assert el.shape[0] > 1000
    spa = (asm.indices.cpu().numpy(), asm.indptr.cpu().numpy(), asm.data_local.cpu().numpy(),
           asm.data_global.cpu().numpy())
    args = (material, params, P, el, x, t["Jm"], t["AllGauss"])
    Vo, To = oracle.assemble_df(*args, mode="csr", sparsity_arrays=spa, nthreads=oracle.max_threads())
    Vf, Tf = oracle.assemble_df(*args, mode="csr", sparsity_arrays=spa, nthreads=oracle.max_threads(), fast=True)
    bar_k, bar_t = max(1e-12, 2 * rel_fro(Vf, Vo)), max(1e-12, 2 * rel_fro(Tf, To))
    assert rel_fro(V1.cpu().numpy(), Vo) < bar_k and rel_fro(T1.cpu().numpy(), To) < bar_t
    assert rel_fro(V2.cpu().numpy(), Vo) < bar_k
    assert rel_fro(T2.cpu().numpy(), To) < bar_t
    assert rel_fro(V3.cpu().numpy(), 2.0 * V2.cpu().numpy()) < 1e-15
    assert rel_fro(T3.cpu().numpy(), 2.0 * T2.cpu().numpy()) < 1e-15
