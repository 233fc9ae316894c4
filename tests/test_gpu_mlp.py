"""GPU tests of the warm-start network kernels against the numpy oracle (same BF16 rounding of
GEMM operands, FP64 accumulation): forward within 1e-4, gradients within 1e-3 relative (the
kernels accumulate in FP32; a BF16 rounding tie can flip between the two), and Adam training
that fits a smooth map."""
import numpy as np
import pytest

from conftest import rel_fro

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_forward_and_gradients_match_oracle():
    from florence_gb300.warmstart import MLP
    from oracle import mlp_oracle
    net = MLP(seed=3)
    rng = np.random.default_rng(4)
    # small random biases too, so every gradient block is exercised
    p = net.params.cpu().numpy()
    p += rng.normal(0, 0.01, p.shape).astype(np.float32)
    net.params.copy_(torch.from_numpy(p))
    x = rng.normal(0, 1, (96, 3)).astype(np.float32)
    t = rng.normal(0, 1, (96, 64)).astype(np.float32)
    y = net.forward(torch.from_numpy(x)).cpu().numpy()
    g, loss = net.gradients(torch.from_numpy(x), torch.from_numpy(t))
    g_ref, loss_ref, y_ref = mlp_oracle.gradients(p, x.astype(np.float64), t.astype(np.float64))
    assert rel_fro(y, y_ref) < 1e-4
    assert abs(float(loss) - loss_ref) / loss_ref < 1e-4
    g = g.cpu().numpy()
    off = 0
    for s in mlp_oracle.SIZES:
        k = int(np.prod(s))
        assert rel_fro(g[off:off + k], g_ref[off:off + k]) < 1e-3, s
        off += k


def test_training_fits_a_smooth_map():
    from florence_gb300.warmstart import MLP
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (512, 3))
    W = rng.normal(0, 1, (3, 64))
    Y = np.tanh(X @ W) + 0.1 * np.sin(3 * X[:, :1])
    net = MLP(seed=1)
    Xd = torch.from_numpy(X).float().cuda()
    Yd = torch.from_numpy(Y).float().cuda()
    hist = net.train(Xd, Yd, steps=1500, batch=128, lr=2e-3)
    assert hist[-1] < 0.05 * hist[0]
    pred = net.forward(Xd).double().cpu().numpy()
    assert rel_fro(pred, Y) < 0.1
