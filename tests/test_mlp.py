"""The learned start vector (blqh_mlp_*): the CUDA forward and backward passes
against the NumPy restatement (oracle/mlp_ref.py, BF16 rounding at the same
points), and what training buys: a trained network's start converges the GPU
Lanczos in fewer steps than the reference's random start at a held-out d.

Tolerances: predictions and gradients agree with the oracle to 2e-2 (relative,
BF16 storage of activations and weights; FP32 accumulation order differs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def B():
    import blqh_gb300 as B

    return B


@pytest.mark.parametrize("tc", ["1", "0"])
def test_forward_and_gradient_match_oracle(B, monkeypatch, tc):
    """tc = 1: the forward and dz GEMMs on tcgen05 (TMA, tensor memory); 0: mma.sync throughout."""
    from oracle import mlp_ref as R

    monkeypatch.setenv("BLQH_MLP_TC", tc)

    b = B.Basis(8, 8, 4, 4, 4)  # real sector (K = nphi / 2), dim 79
    net = B.MLP(16, 256, seed=3)
    w = net.params()
    rng = np.random.default_rng(2)
    conds = [(0.0, 0.0), (1.5, 0.05)]
    tg = rng.standard_normal(2 * b.dim)
    loss, g = net.loss_grad(b, conds, tg)
    Lr, gr = R.loss_grad(w, 16, 256, b.id, conds, tg)
    assert abs(loss - Lr) <= 2e-2 * max(1e-3, abs(Lr))
    assert np.linalg.norm(g - gr) <= 2e-2 * np.linalg.norm(gr), np.linalg.norm(g - gr) / np.linalg.norm(gr)
    # forward
    p = net.predict(b, 1.5, 0.05)
    _, _, k0 = R.layout(16, 256)
    out, _ = R.forward(R.unpack(w, 16, 256), R.features(b.id, 16, 1.5, 0.05, k0))
    out /= np.linalg.norm(out)
    assert np.linalg.norm(p - out) <= 2e-2


@pytest.mark.parametrize("sec,width", [((12, 12, 6, 0, 0), 256), ((16, 6, 3, 0, 0), 128)])
def test_tensor_core_paths_agree(B, monkeypatch, sec, width):
    """tcgen05 against mma.sync on 3 points of a sector (rows over many 128-row
    tiles, the last one ragged; 2 nphi + 2 inputs padded to 32 or 64; layers 256 or
    128 wide): predictions to 2e-3 and gradients to 1e-2 (relative norms; BF16
    storage at the same points, FP32 accumulation in a different order), and the
    loss to 1e-3."""
    b = B.Basis(*sec)
    rng = np.random.default_rng(4)
    conds = [(0.5, 0.0), (1.0, 0.05), (1.5, 0.1)]
    tg = rng.standard_normal(3 * b.dim)
    res = {}
    for tc in ("1", "0"):
        monkeypatch.setenv("BLQH_MLP_TC", tc)
        net = B.MLP(2 * sec[0], width, seed=7)
        loss, g = net.loss_grad(b, conds, tg)
        res[tc] = (loss, g, net.predict(b, 1.25, 0.05))
    (l1, g1, p1), (l0, g0, p0) = res["1"], res["0"]
    assert abs(l1 - l0) <= 1e-3 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 1e-2 * np.linalg.norm(g0)
    assert np.linalg.norm(p1 - p0) <= 2e-3 * np.linalg.norm(p0)


def test_params_round_trip(B):
    net = B.MLP(20, 128, seed=5)
    w = net.params()
    w2 = w * 0.5
    net.set_params(w2)
    assert np.array_equal(net.params(), w2)


def test_training_reduces_loss_and_learned_start_saves_steps(B):
    from blqh_gb300 import learned as Lr

    train = [0.0, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0]
    r = Lr.run(nphi=10, nel=10, nup=5, J=0, K=0, train_ds=train, test_ds=[1.25, 2.25], steps=400, lr=2e-3,
               width=256, seed=1)
    assert r["loss_last"] < 0.5 * r["loss_first"]
    for p in r["points"]:
        assert p["used_learned"] and p["overlap_exact"] > 0.5
        assert p["iterations_learned"] < p["iterations_random"], p
