"""GPU tests of the deterministic assembly mode (DeviceAssembler(..., deterministic=True)): the
elements coloured so that no two of a colour share a node and assembled colour by colour, every
CSR and residual entry gets its contributions in one fixed order. Repeated assemblies are
bit-identical (the default scatter's atomic adds land in a varying order), in both CSR modes and
for the default and the float-pair contractions, and they meet the FP64 bar against the
reference (golden case) and against the oracle (a jittered box of ~1 300 tets)."""
import numpy as np
import pytest

from conftest import load_golden, rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _box():
    import bench
    from florence_gb300 import meshes
    t = np.load(bench.os.path.join(bench.GOLDEN, "tet_p3_mr_jitter.npz"))
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((12, 4, 4), (3.0, 1.0, 1.0), 5, pat)
    x = P + bench.smooth_displacement(P, seed=9) * 10.0
    return P, el, x, t["Jm"], t["AllGauss"]


@pytest.mark.parametrize("arith", ["reference_tensor", "float_pair"])
@pytest.mark.parametrize("mode", ["csr", "squeeze"])
def test_repeated_assemblies_are_bit_identical(oracle, arith, mode):
    import florence_gb300 as fl
    P, el, x, Jm, w = _box()
    asm = fl.DeviceAssembler(P, el, Jm, w, "MooneyRivlin", (0.5, 0.5, 20.0), mode=mode, deterministic=True)
    assert len(asm._colour) > 1
    xd = torch.from_numpy(x).cuda()
    with fl.arithmetic(arith):
        outs = [asm.assemble(xd) for _ in range(3)]
        torch.cuda.synchronize()
    asm.check_flags()
    for V, T in outs[1:]:
        assert torch.equal(V, outs[0][0]) and torch.equal(T, outs[0][1])
    spa = (asm.indices.cpu().numpy(), asm.indptr.cpu().numpy(), None, None)
    args = ("MooneyRivlin", (0.5, 0.5, 20.0), P, el, x, Jm, w)
    Vo, To = oracle.assemble_df(*args, mode="squeeze", sparsity_arrays=spa, nthreads=oracle.max_threads())
    Vf, Tf = oracle.assemble_df(*args, mode="squeeze", sparsity_arrays=spa, nthreads=oracle.max_threads(), fast=True)
    bar_k, bar_t = max(1e-12, 2 * rel_fro(Vf, Vo)), max(1e-12, 2 * rel_fro(Tf, To))
    assert rel_fro(outs[0][0].cpu().numpy(), Vo) < bar_k
    assert rel_fro(outs[0][1].cpu().numpy(), To) < bar_t


def test_colouring_is_node_disjoint_and_golden_case_holds():
    import florence_gb300 as fl
    d = load_golden("tet_p3_mr_jitter")
    asm = fl.DeviceAssembler(d["points"], d["elements"], d["Jm"], d["AllGauss"], "MooneyRivlin",
                             tuple(d["params"]), mode="csr", requires_geometry_update=int(d["update"]),
                             deterministic=True)
    seen = 0
    for pc in asm._colour:
        e = pc["elements"].cpu().numpy()
        assert len(np.unique(e)) == e.size   # no node twice within a colour
        seen += e.shape[0]
    assert seen == d["elements"].shape[0]
    V, T = asm.assemble(torch.from_numpy(d["Eulerx"]).cuda())
    torch.cuda.synchronize()
    asm.check_flags()
    assert rel_fro(V.cpu().numpy(), d["K_data"]) < 1e-12
    assert rel_fro(T.cpu().numpy(), d["T"]) < 1e-12
