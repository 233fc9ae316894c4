"""GPU test of the learned warm start on a small plate: training solves, POD, the network
trained by the project's kernels, then held-out solves. The network's guess must save Newton
iterations over the previous-increment guess, and both must reach the same state (1e-8). The
solves stop at |R| <= 1e-11 |F|: two runs that both stop at 1e-10 can differ by the condition
number times 1e-10 (about 1e-8 on this plate), which says nothing about the guess."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_warm_start_saves_newton_iterations(tmp_path):
    from florence_gb300 import warmstart as W
    prob = W.build_plate_problem(12, 6, 2, seed=5)
    solver = W.PlateSolver(prob, n_increments=4, tol=1e-11)
    X, U, stats = W.generate_snapshots(solver, W.sample_parameters(32, seed=3))
    assert not any(s["failed"] for s in stats)
    assert X.shape == (32 * 5, 3) and U.shape == (solver.ndof, 32 * 5)
    ws, hist, sv, proj = W.train_warm_start(X, U, modes=64, steps=6000)
    assert hist[-1] < 0.01 * hist[0]
    assert proj < 1e-3
    rows, tot = W.evaluate_warm_start(solver, ws, W.sample_parameters(4, seed=4))
    assert tot["plain"]["failed"] == 0 and tot["warm"]["failed"] == 0
    assert tot["warm"]["accepted"] > 0
    assert tot["warm"]["newton"] < tot["plain"]["newton"]
    assert tot["warm"]["max_du"] < 1e-8
    # the checkpoint reproduces the predictions
    W.save(ws, tmp_path / "ws.npz")
    ws2 = W.load(tmp_path / "ws.npz")
    x = solver.increment_inputs(W.sample_parameters(1, seed=9)[0], with_zero=True)
    assert torch.allclose(ws.predict(x), ws2.predict(x))
