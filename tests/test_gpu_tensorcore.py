"""GPU test of the tcgen05 tensor-core path: shared-memory descriptors, instruction descriptor,
tensor-memory accumulator and read-back, against an exact host product (small integers in BF16,
FP32 accumulation: every partial sum is exact)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_tcgen05_product_is_exact():
    from florence_gb300 import _native as N
    from florence_gb300.assembly import _ptr, _stream
    rng = np.random.default_rng(7)
    A = rng.integers(-8, 9, (128, 48)).astype(np.float32)
    B = rng.integers(-8, 9, (32, 48)).astype(np.float32)
    Ad = torch.from_numpy(A).cuda().to(torch.bfloat16).contiguous()
    Bd = torch.from_numpy(B).cuda().to(torch.bfloat16).contiguous()
    D = torch.full((128, 32), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(N.lib().fl_TensorCoreSelfTest(_ptr(Ad), _ptr(Bd), _ptr(D), _ptr(status), _stream()),
            "fl_TensorCoreSelfTest")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert np.array_equal(D.cpu().numpy(), A @ B.T)
