"""Host logic of the drop-ins' pooled output buffers (no GPU): a buffer is handed out again only
after every array built on it is gone, and the copies land intact."""
import gc

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_buffer_reused_only_after_release():
    from florence_gb300.assembly import _HostPool
    pool = _HostPool(keep=2)
    src = torch.arange(12, dtype=torch.float64)
    a = pool.to_host(src.reshape(3, 4))
    assert a.shape == (3, 4) and np.array_equal(a.ravel(), np.arange(12.0))
    b = pool.to_host(src * 2)          # a is alive: a second buffer
    assert not np.shares_memory(a, b)
    assert np.array_equal(a.ravel(), np.arange(12.0))
    view = a[1:]                        # a view keeps a's buffer alive
    del a
    gc.collect()
    c = pool.to_host(src * 3)
    assert not np.shares_memory(view, c) and not np.shares_memory(b, c)
    assert np.array_equal(view.ravel(), np.arange(4.0, 12.0))
    ptr_b = b.ctypes.data
    del b
    gc.collect()
    d = pool.to_host(src * 4)           # b's buffer is free again
    assert d.ctypes.data == ptr_b and np.array_equal(d, np.arange(12.0) * 4)


def test_idle_buffers_are_bounded_and_released():
    from florence_gb300.assembly import _HostPool
    pool = _HostPool(keep=1)
    src = torch.ones(8, dtype=torch.float64)
    arrs = [pool.to_host(src) for _ in range(4)]
    assert len(pool.slots) == 4
    del arrs
    gc.collect()
    pool.to_host(src)                   # reuses one, keeps at most one more idle
    assert len(pool.slots) <= 2
    pool.release()
    assert len(pool.slots) == 0 or all(sl[1]() is not None for sl in pool.slots)


def test_device_mesh_cache_reuses_only_identical_inputs():
    """The drop-ins' device-mesh cache (host logic, a stand-in builder): the same array objects with
    the same sampled content reuse the entry; a rewritten array, another object or other scalars
    build anew; at most `keep` entries are held."""
    from florence_gb300.assembly import _DeviceMeshCache
    cache = _DeviceMeshCache(keep=2)
    built = []

    def build():
        built.append(object())
        return built[-1]

    P = np.random.default_rng(0).random((1000, 3))
    E = np.arange(4000, dtype=np.uint64).reshape(1000, 4)
    a = cache.get([P, E, None], ("NeoHookean", 1), build)
    assert cache.get([P, E, None], ("NeoHookean", 1), build) is a and len(built) == 1
    assert cache.get([P, E, None], ("NeoHookean", 2), build) is not a          # other scalars
    P2 = P.copy()
    assert cache.get([P2, E, None], ("NeoHookean", 1), build) is not a         # another object
    assert len(cache.entries) == 2
    P[:] += 1.0                                                                # rewritten in place
    n = len(built)
    cache.get([P, E, None], ("NeoHookean", 1), build)
    assert len(built) == n + 1
    assert cache.get([[1.0], E, None], ("NeoHookean", 1), build) is built[-1] and len(built) == n + 2  # not cacheable
    cache.clear()
    assert cache.entries == []
