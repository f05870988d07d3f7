"""The screen proposer's MLP kernels on a GB300 (through the C ABI), against the FP64 oracle.

Tolerances: gradients per parameter tensor within 1e-2 relative L2 norm of the oracle's (the
oracle applies the same bf16 roundings; the rest is float32 vs float64 accumulation and bf16 ties);
loss within 1e-4 relative."""
import numpy as np
import pytest

from auto_gb300 import _lib
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def proposer():
    from auto_gb300 import native
    from auto_gb300.screen import Proposer
    native.build()
    p = Proposer(seed=3, max_batch=4096)
    yield p
    p.close()


SLICES = {"W1": (M.P_W1, M.P_B1), "b1": (M.P_B1, M.P_W2), "W2": (M.P_W2, M.P_B2), "b2": (M.P_B2, M.P_W3),
          "W3": (M.P_W3, M.P_B3), "b3": (M.P_B3, M.NPARAM)}


@pytest.mark.parametrize("batch", [64, 1000, 4096])
def test_gradients_match_fp64_oracle(proposer, batch):
    rng = np.random.default_rng(batch)
    p = proposer.params()
    p[M.P_B1:M.P_W2] = rng.standard_normal(M.HID) * 0.05  # non-zero biases exercise their gradients
    proposer.set_params(p)
    x = rng.random((batch, M.IN)).astype(np.float32)
    y = (rng.random((batch, M.OUT)) < 0.3).astype(np.float32)
    loss, g = proposer.gradients(x, y)
    want_loss, want = M.loss_and_grads(proposer.params(), x, y)
    assert abs(loss - want_loss) <= 1e-4 * abs(want_loss)
    for name, (a, b) in SLICES.items():
        err = np.linalg.norm(g[a:b] - want[a:b]) / max(np.linalg.norm(want[a:b]), 1e-30)
        assert err < 1e-2, (name, err)


def test_predict_matches_oracle(proposer):
    rng = np.random.default_rng(9)
    x = rng.random((5000, M.IN)).astype(np.float32)  # more rows than max_batch: chunked
    got = proposer.predict(x)
    want = M.predict(proposer.params(), x)
    assert np.abs(got - want).max() < 2e-3


def test_training_learns_a_known_rule():
    from auto_gb300.screen import Proposer
    rng = np.random.default_rng(1)
    x = rng.random((8192, M.IN)).astype(np.float32)
    y = np.stack([x[:, 0] > 0.5, x[:, 1] + x[:, 2] > 1.0, x[:, 3] < 0.3], 1).astype(np.float32)
    mlp = Proposer(seed=7, max_batch=1024)
    hist = mlp.fit(x, y, epochs=15, batch=512, lr=3e-3)
    acc = ((mlp.predict(x) > 0.5) == (y > 0.5)).mean(0)
    mlp.close()
    assert hist[-1] < 0.5 * hist[0], hist
    assert (acc > 0.95).all(), acc


def test_learned_screen_beats_uniform_draws():
    """A small screen: the simulator labels 3072 worlds (256^2, 600 steps); the trained MLP ranks
    65536 candidates; the simulator judges the top 384 and 384 uniform draws.  The learned pick
    must hold more surviving worlds than the uniform one."""
    from auto_gb300 import screen
    cfg = screen.ScreenConfig(train_worlds=3072, side=256, steps=600, every=100, window=200, candidates=65536,
                              top=384, epochs=25, seed=11)
    rep = screen.run(cfg, log=lambda *a: None)
    print("screen:", rep["learned"], rep["uniform"], rep["label_rates_train"])
    assert rep["learned"]["survive"] > rep["uniform"]["survive"]
    assert rep["learned"]["nontrivial"] >= rep["uniform"]["nontrivial"]
