"""The learned histogram denoiser over the C ABI (``ss_dn_*`` of
include/ssgpu.h): a 3-D CNN on the (x, y, phi) grid whose 32 -> 32
convolutions run on the tensor cores (tcgen05).  Inputs and outputs are CUDA
float tensors of the grid's shape (torch is used only to hold device memory).

    dn = Denoiser((128, 128, 32), seed=0)
    y = dn.forward(x)                   # x: histogram / mean count
    loss = dn.train(x_batch, t_batch, lr=1e-3)

There is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check

_fp = ctypes.POINTER(ctypes.c_float)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Denoiser:
    """The network on the current CUDA device for grids of `shape` = (nx, ny, nphi)."""

    def __init__(self, shape, seed=0, stream=None):
        self.lib = _lib.load()
        self.shape = tuple(int(v) for v in shape)
        h = ctypes.c_void_p()
        check(self.lib.ss_dn_create(*self.shape, int(seed), ctypes.c_void_p(stream) if stream else None,
                                    ctypes.byref(h)))
        self._h = h
        n = ctypes.c_uint64()
        check(self.lib.ss_dn_info(self._h, ctypes.byref(n), None))
        self.nparams = n.value

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self.lib.ss_dn_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check_grid(self, t, batched=False):
        import torch
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise TypeError("expected a contiguous CUDA float32 tensor")
        # the network runs on its own stream: the tensor's producer must be done
        torch.cuda.current_stream().synchronize()
        n = int(np.prod(self.shape))
        if batched:
            if t.numel() % n or t.numel() == 0:
                raise ValueError(f"expected a batch of grids of shape {self.shape}")
            return t.numel() // n
        if t.numel() != n:
            raise ValueError(f"expected a grid of shape {self.shape}")
        return 1

    def set_loss(self, moment_weight=0.0):
        """Training loss: the mean-square error plus moment_weight times the
        squared second angular harmonic of the residual per cell
        (ss_dn_set_loss), the part of the error that reaches the flow."""
        check(self.lib.ss_dn_set_loss(self._h, float(moment_weight)))

    @property
    def params(self):
        out = np.empty(self.nparams, dtype=np.float32)
        check(self.lib.ss_dn_get_params(self._h, out.ctypes.data_as(_fp), self.nparams))
        return out

    @params.setter
    def params(self, values):
        v = np.ascontiguousarray(values, dtype=np.float32).ravel()
        check(self.lib.ss_dn_set_params(self._h, v.ctypes.data_as(_fp), v.size))

    def forward(self, x, out=None):
        import torch
        self._check_grid(x)
        y = torch.empty_like(x) if out is None else out
        self._check_grid(y)
        check(self.lib.ss_dn_forward(self._h, _ptr(x), _ptr(y)))
        return y

    def train(self, x, t, lr=1e-3):
        """One Adam step on a batch (x, t: [batch, *shape]); returns the batch loss."""
        b = self._check_grid(x, True)
        if self._check_grid(t, True) != b:
            raise ValueError("x and t differ in batch size")
        loss = ctypes.c_double()
        check(self.lib.ss_dn_train(self._h, _ptr(x), _ptr(t), b, float(lr), ctypes.byref(loss)))
        return loss.value

    def loss(self, x, t):
        return self.train(x, t, lr=0.0)

    def gradients(self, x, t):
        """(batch-mean gradient as a numpy array, loss) without an update."""
        b = self._check_grid(x, True)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = ctypes.c_double()
        check(self.lib.ss_dn_gradients(self._h, _ptr(x), _ptr(t), b, g.ctypes.data_as(_fp), self.nparams,
                                       ctypes.byref(loss)))
        return g, loss.value

    def save(self, path):
        np.save(path, self.params)

    def load(self, path):
        self.params = np.load(path)


# parameter layout (offsets into the flat FP32 array)
C, TAPS = 32, 27
OFFSETS = {}
_o = 0
for _name, _size in [("w_in", TAPS * C), ("b_in", C), ("w2", TAPS * C * C), ("b2", C), ("w3", TAPS * C * C),
                     ("b3", C), ("w_out", TAPS * C), ("b_out", 1)]:
    OFFSETS[_name] = (_o, _size)
    _o += _size
NPARAMS = _o


def split_params(p):
    """dict of named views (w_in (27, 32), w2 (27, 32, 32), ...) into a flat parameter array."""
    shapes = {"w_in": (TAPS, C), "b_in": (C,), "w2": (TAPS, C, C), "b2": (C,), "w3": (TAPS, C, C), "b3": (C,),
              "w_out": (TAPS, C), "b_out": (1,)}
    return {k: p[o:o + s].reshape(shapes[k]) for k, (o, s) in OFFSETS.items()}


# ---------------------------------------------------------------- training data
def sample_histogram(shape, n, amp, phase, axis, seed, out=None):
    """Normalised histogram (mean 1) of n particles with density
    1 + amp sin(2 pi s + phase) along `axis` (0: x, 1: y), uniform otherwise,
    sampled on the device (ss_dn_sample_histogram); a CUDA float tensor."""
    import torch
    lib = _lib.load()
    h = torch.zeros(shape, device="cuda", dtype=torch.float32) if out is None else out
    check(lib.ss_dn_sample_histogram(*[int(v) for v in shape], int(n), float(amp), float(phase), int(axis),
                                     int(seed), _ptr(h), None))
    return h


def make_pairs(npairs, shape=(128, 128, 32), n_in=1_000_000, n_target=64_000_000, amp_max=0.05, seed=0):
    """Training pairs generated by the method: for each pair an initial
    condition of the production family (perturbation amplitude uniform in
    [0, amp_max], random phase and axis), histogrammed once with n_in and
    once, independently, with n_target particles.  Returns (inputs,
    targets), CUDA float tensors [npairs, *shape], both normalised to mean 1."""
    import torch
    rng = np.random.default_rng(seed)
    X = torch.zeros((npairs, *shape), device="cuda", dtype=torch.float32)
    T = torch.zeros_like(X)
    for i in range(npairs):
        amp, ph, ax = rng.uniform(0.0, amp_max), rng.uniform(0.0, 2 * np.pi), int(rng.integers(2))
        sample_histogram(shape, n_in, amp, ph, ax, (seed << 32) + 2 * i, out=X[i])
        sample_histogram(shape, n_target, amp, ph, ax, (seed << 32) + 2 * i + 1, out=T[i])
    torch.cuda.synchronize()
    return X, T


def train(dn, X, T, epochs=1, batch=8, lr=1e-3, seed=0, val=None):
    """Adam over shuffled minibatches of (X, T); returns the per-epoch mean
    training loss and, when val = (Xv, Tv) is given, the validation loss.
    With a validation set the network ends with the parameters of the epoch
    of lowest validation loss (marked "kept" in its record): the last epoch
    of a short run at a fixed rate can land on a worse point."""
    import torch
    rng = np.random.default_rng(seed)
    hist = []
    best = None
    n = X.shape[0]
    for _ in range(epochs):
        order = rng.permutation(n)
        losses = []
        for k in range(0, n - batch + 1, batch):
            idx = torch.as_tensor(order[k:k + batch], device=X.device)
            losses.append(dn.train(X[idx].contiguous(), T[idx].contiguous(), lr=lr))
        rec = {"train": float(np.mean(losses))}
        if val is not None:
            rec["val"] = dn.loss(val[0], val[1])
            if best is None or rec["val"] < best[0]:
                best = (rec["val"], len(hist), dn.params)
        hist.append(rec)
    if best is not None:
        dn.params = best[2]
        hist[best[1]]["kept"] = True
    return hist


def _main():
    """python -m stochasticsampling_gb300.denoiser [--forwards K] [--train-steps S] [--shape NX NY NP]:
    K forward passes of a freshly initialised network on a random histogram
    of the given grid (default the production grid 128 x 128 x 32), then S
    training steps (batch 1, Adam) on a random pair, each timed with CUDA
    events; the command the convolution's profiles were taken with."""
    import argparse

    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--forwards", type=int, default=3)
    ap.add_argument("--train-steps", type=int, default=0)
    ap.add_argument("--shape", type=int, nargs=3, default=(128, 128, 32))
    args = ap.parse_args()
    dn = Denoiser(tuple(args.shape), seed=0)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = 1.0 + 0.5 * torch.rand(tuple(args.shape), device="cuda", generator=g)
    y = torch.empty_like(x)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    fwd = [timed(lambda: dn.forward(x, out=y)) for _ in range(args.forwards)]
    t = 1.0 + 0.1 * torch.rand(tuple(args.shape), device="cuda", generator=g)
    train = [timed(lambda: dn.train(x[None], t[None], lr=1e-4)) for _ in range(args.train_steps)]
    dn.close()
    print({"shape": list(args.shape), "forward_ms": fwd, "train_step_ms": train})


if __name__ == "__main__":
    _main()
