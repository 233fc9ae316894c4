"""Host logic of the drop-in's pipelined assembly (DeviceAssembler._pipeline_plan): the elements
split into groups in order of their smallest node; every node's CSR rows and residual rows are
copied after the last group that holds the node (possibly also earlier, inside a merged run, to be
overwritten then); every element in exactly one group."""
import types

import numpy as np
import torch

from conftest import load_golden


def _plan(elements, indptr, nnode, pieces):
    from florence_gb300.assembly import DeviceAssembler
    el = torch.as_tensor(elements, dtype=torch.int64)
    obj = types.SimpleNamespace(elements=el, nnode=nnode, nelem=el.shape[0], npe=el.shape[1], orient=None,
                                device=torch.device("cpu"), indptr=torch.as_tensor(indptr, dtype=torch.int32))
    return DeviceAssembler._pipeline_plan(obj, pieces)


def test_plan_covers_every_row_after_its_last_group():
    from florence_gb300 import meshes
    from oracle import oracle
    t = load_golden("tet_p3_mr_jitter")
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((12, 4, 4), (3.0, 1.0, 1.0), 5, pat)
    ind, ptr = oracle.sparsity(el, P.shape[0], maps=False)[:2]
    pieces = 8
    plan = _plan(el, ptr, P.shape[0], pieces)
    assert len(plan) == pieces
    # every element in exactly one group
    rows = np.concatenate([pc["elements"].numpy() for pc in plan])
    key = lambda a: a[np.lexsort(a.T[::-1])]  # noqa: E731
    assert np.array_equal(key(rows), key(el))
    # the last group holding each node
    last = np.full(P.shape[0], -1)
    for g, pc in enumerate(plan):
        last[np.unique(pc["elements"].numpy())] = g
    # each node's rows are copied after its last group (copies in other groups, inside merged runs,
    # are overwritten by that one if earlier, or repeat the final values if later)
    copied = np.zeros((pieces, P.shape[0]), bool)
    for g, pc in enumerate(plan):
        for v0, v1, t0, t1 in pc["rows"]:
            n0, n1 = t0 // 3, t1 // 3
            assert v0 == ptr[3 * n0] and v1 == ptr[3 * n1]
            copied[g, n0:n1] = True
    assert (last >= 0).all()
    assert copied[last, np.arange(P.shape[0])].all()
    # few copies per group on a mesh numbered with locality (vertices, then edge, face, interior
    # nodes, each class in vertex order)
    assert sum(len(pc["rows"]) for pc in plan) <= 8 * pieces
