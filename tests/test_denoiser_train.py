"""The denoiser's training loop (stochasticsampling_gb300.denoiser.train) on
the CPU, with a stand-in network: minibatch order, per-epoch records, and
the choice of the parameters of the epoch of lowest validation loss."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from stochasticsampling_gb300.denoiser import train


class FakeNet:
    """A network whose 'parameters' count the minibatches seen and whose
    validation loss follows a given sequence, one value per epoch."""

    def __init__(self, val_losses):
        self.val_losses = list(val_losses)
        self.epoch_val = iter(self.val_losses)
        self.p = np.zeros(3, dtype=np.float32)
        self.batches = []

    def train(self, x, t, lr=1e-3):
        self.batches.append(x.shape[0])
        self.p = self.p + 1.0
        return float(x.mean())

    def loss(self, x, t):
        return next(self.epoch_val)

    @property
    def params(self):
        return self.p.copy()

    @params.setter
    def params(self, v):
        self.p = np.asarray(v, dtype=np.float32).copy()


def test_keeps_the_epoch_of_lowest_validation_loss():
    X = torch.ones(20, 2, 2, 2)
    T = torch.zeros(20, 2, 2, 2)
    net = FakeNet([0.5, 0.2, 0.3, 0.25])
    hist = train(net, X, T, epochs=4, batch=5, lr=1e-3, seed=1, val=(X[:2], T[:2]))
    assert [h["val"] for h in hist] == [0.5, 0.2, 0.3, 0.25]
    assert [bool(h.get("kept")) for h in hist] == [False, True, False, False]
    # 4 minibatches of 5 per epoch: the kept parameters are those after epoch 2
    assert net.batches == [5] * 16
    assert np.array_equal(net.params, np.full(3, 8.0, dtype=np.float32))


def test_without_validation_the_last_parameters_stay():
    X = torch.ones(8, 2, 2, 2)
    net = FakeNet([])
    hist = train(net, X, X, epochs=3, batch=4)
    assert all("val" not in h and "kept" not in h for h in hist)
    assert np.array_equal(net.params, np.full(3, 6.0, dtype=np.float32))
