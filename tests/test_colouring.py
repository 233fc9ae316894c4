"""Host logic of the deterministic assembly mode (DeviceAssembler._colour_elements): every element in
exactly one colour, no node twice within a colour, colours in the greedy order, on a jittered
Delaunay tet mesh and on a structured hex mesh (no GPU: the colouring runs on the host)."""
import types

import numpy as np
import torch

from conftest import load_golden


def _colour(elements, nnode):
    from florence_gb300.assembly import DeviceAssembler
    obj = types.SimpleNamespace(elements=torch.as_tensor(elements, dtype=torch.int64), nnode=nnode,
                                nelem=elements.shape[0], device=torch.device("cpu"), orient=None)
    return DeviceAssembler._colour_elements(obj)


def _check(elements, pieces):
    seen = []
    for pc in pieces:
        e = pc["elements"].numpy()
        assert len(np.unique(e)) == e.size
        seen.append(e)
    allel = np.concatenate(seen)
    assert allel.shape == elements.shape
    # the same multiset of element rows
    key = lambda a: a[np.lexsort(a.T[::-1])]  # noqa: E731
    assert np.array_equal(key(allel), key(np.asarray(elements)))


def test_tet_mesh_colouring():
    from florence_gb300 import meshes
    t = load_golden("tet_p3_mr_jitter")
    pat = meshes.local_pattern(t["points"], t["elements"], 0, "tet")
    P, el = meshes.jittered_tet_beam((10, 4, 4), (2.5, 1.0, 1.0), 3, pat)
    pieces = _colour(el, P.shape[0])
    _check(el, pieces)
    assert 20 <= len(pieces) <= 64


def test_hex_mesh_colouring():
    from florence_gb300 import meshes
    d = load_golden("hex_p2_nh_q5")
    xi = meshes.local_pattern(d["points"], d["elements"], 0, "hex")
    P, el = meshes.structured_hex((6, 5, 4), (1.0, 1.0, 1.0), xi)
    pieces = _colour(el, P.shape[0])
    _check(el, pieces)
    assert len(pieces) == 8  # a structured hex box needs the 8 parities
