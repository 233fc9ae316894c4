"""GPU tests of the batched assembly of independent meshes (uneven sizes, per-instance
materials): each instance's block of the batched CSR equals the single-mesh assembly of that
instance (1e-12 relative), for the FP64 path with and without element-to-nonzero maps, and the
split-BF16 variant is within 5e-6."""
import numpy as np
import pytest

from conftest import rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _instances(p, sizes, seed=0):
    from florence_gb300.batched import build_instance, hex_tables
    pat, Jm, w = hex_tables(p)
    rng = np.random.default_rng(seed)
    specs = [dict(n=n, p=p, mu=float(rng.uniform(0.5, 2)), lamb=float(rng.uniform(5, 50)),
                  seed=int(rng.integers(0, 1000))) for n in sizes]
    return [build_instance(s, pat) for s in specs], Jm, w


@pytest.mark.parametrize("p,maps", [(1, False), (2, True), (2, False), (3, False)])
def test_batched_blocks_equal_single_mesh_assembly(p, maps):
    import florence_gb300 as fl
    from florence_gb300.batched import BatchedAssembler
    sizes = {1: [2, 3, 4], 2: [2, 3, 2], 3: [1, 2, 1]}[p]
    inst, Jm, w = _instances(p, sizes)
    B = BatchedAssembler(inst, Jm, w, "NeoHookean", maps=maps)
    V, T = B.assemble()
    B_flags = int(B.flags.item())
    assert B_flags == 0
    for k, i in enumerate(inst):
        a = fl.DeviceAssembler(i["points"], i["elements"], Jm, w, "NeoHookean", i["params"], mode="csr")
        Vk, Tk = a.assemble(torch.from_numpy(i["Eulerx"]).cuda())
        ptr, ind, data = B.instance_csr(k, V)
        assert np.array_equal(ptr, a.indptr.cpu().numpy()) and np.array_equal(ind, a.indices.cpu().numpy())
        assert rel_fro(data, Vk.cpu().numpy()) < 1e-12
        r0, r1 = 3 * int(B.node_off[k]), 3 * int(B.node_off[k + 1])
        assert rel_fro(T[r0:r1].cpu().numpy(), Tk.cpu().numpy()) < 1e-12


def test_batched_mixed_close_to_fp64():
    from florence_gb300.batched import BatchedAssembler
    inst, Jm, w = _instances(2, [2, 3])
    B = BatchedAssembler(inst, Jm, w, "NeoHookean", maps=False)
    V64, T64 = B.assemble()
    V32, T32 = B.assemble(mixed=True)
    assert rel_fro(V32.double().cpu().numpy(), V64.cpu().numpy()) < 5e-6
    assert rel_fro(T32.cpu().numpy(), T64.cpu().numpy()) < 1e-13


def test_autotuner_installs_a_working_choice():
    from florence_gb300.batched import BatchedAssembler
    inst, Jm, w = _instances(2, [3, 3])
    B = BatchedAssembler(inst, Jm, w, "NeoHookean")
    Vref, _ = B.assemble()
    r = B.autotune(candidates=[1, 4, 27])
    assert r["gauss_chunk"] in (1, 4, 27)
    V, _ = B.assemble()
    assert rel_fro(V.cpu().numpy(), Vref.cpu().numpy()) < 1e-13
