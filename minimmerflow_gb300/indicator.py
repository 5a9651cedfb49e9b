"""Learned troubled-cell indicator: the MLP (C ABI mmf_mlp_*), its GPU
training, the training data from seeded order-2 runs, and its use in the
solver (cells predicted smooth take central slopes and skip the limiter)."""
import ctypes as C

import numpy as np

from . import capi


class TroubledCellMLP:
    """135 -> 64 -> 64 -> 1 (3D) / 45 -> 64 -> 64 -> 1 (2D) MLP on the GPU."""

    def __init__(self, dim=3, seed=0, device=0):
        self._lib = capi.load()
        self.dim = dim
        self._p = C.c_void_p()
        capi.check(self._lib.mmf_mlp_create(dim, seed, device, C.byref(self._p)))
        self.nparams = self._lib.mmf_mlp_num_params(self._p)
        self.width = self._lib.mmf_mlp_input_width(self._p)

    @property
    def handle(self):
        return self._p

    def close(self):
        if getattr(self, "_p", None) is not None and self._p.value:
            self._lib.mmf_mlp_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        out = np.empty(self.nparams, dtype=np.float32)
        capi.check(self._lib.mmf_mlp_get_params(self._p, capi.ptr(out), self.nparams))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        capi.check(self._lib.mmf_mlp_set_params(self._p, capi.ptr(p), self.nparams))

    def gradients(self, d_X, d_y, batch):
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_float()
        capi.check(self._lib.mmf_mlp_gradients(self._p, capi.ptr(d_X), capi.ptr(d_y), batch, capi.ptr(g), C.byref(loss)))
        return g, loss.value

    def train_batch(self, d_X, d_y, batch, lr):
        loss = C.c_float()
        capi.check(self._lib.mmf_mlp_train_batch(self._p, capi.ptr(d_X), capi.ptr(d_y), batch, lr, C.byref(loss)))
        return loss.value

    def set_wait_limits(self, wait_limit=1 << 22, probe_limit=0):
        """Iteration limits of the inference kernel's barrier waits
        (mmf_mlp_set_wait_limits)."""
        capi.check(self._lib.mmf_mlp_set_wait_limits(self._p, wait_limit, probe_limit))

    def predict(self, d_X, d_prob):
        capi.check(self._lib.mmf_mlp_predict(self._p, capi.ptr(d_X), d_X.shape[0], capi.ptr(d_prob)))

    def fit(self, X, y, epochs=4, batch=1024, lr=2e-3, seed=0, log=None):
        """Adam on device tensors X (bf16 as int16 [n][width]) and y (uint8 [n])."""
        import torch
        n = (X.shape[0] // batch) * batch
        g = torch.Generator(device="cpu").manual_seed(seed)
        losses = []
        for ep in range(epochs):
            perm = torch.randperm(X.shape[0], generator=g)[:n].to(X.device)
            Xs = X[perm].contiguous()
            ys = y[perm].contiguous()
            tot = 0.0
            for i in range(0, n, batch):
                tot += self.train_batch(Xs[i:i + batch], ys[i:i + batch], batch, lr)
            losses.append(tot / (n // batch))
            if log:
                log("epoch %d loss %.5f" % (ep, losses[-1]))
        return losses


def features(solver, out=None):
    """Stencil features of the solver's uploaded state, device bf16 (int16 storage) [n][width]."""
    import torch
    width = 144 if solver.dim == 3 else 48
    if out is None:
        out = torch.empty((solver.ncells, width), dtype=torch.int16, device="cuda")
    capi.check(solver._lib.mmf_features(solver._ctx, capi.ptr(out)))
    return out


def labels(solver, out=None):
    """Order-2 limiter activation of the solver's uploaded state, device uint8 [n] (grid order)."""
    import torch
    if out is None:
        out = torch.empty(solver.ncells, dtype=torch.uint8, device="cuda")
    capi.check(solver._lib.mmf_limiter_labels(solver._ctx, capi.ptr(out)))
    return out


def generate_dataset(cases, snapshots=4, steps_between=6, samples=1_000_000, seed=0, arith="fast"):
    """(features, labels) from seeded order-2 runs of the plain solver: for
    each case, 'snapshots' states 'steps_between' steps apart; every cell of
    every snapshot is a sample, then 'samples' of them are drawn at random."""
    import torch
    Xs, ys = [], []
    for case in cases:
        with case.solver(arith=arith, order=2) as s:
            s.upload(case.initial_state())
            s.time_setup(case.cfl, 0.0, float("inf"), 10 ** 9)
            for k in range(snapshots):
                try:
                    s.advance(steps_between)
                except capi.MMFError as e:
                    # a strong case that the plain order-2 scheme cannot keep
                    # physical at this CFL: keep the snapshots taken so far
                    if e.code != capi.MMF_ERR_STATE:
                        raise
                    break
                Xs.append(features(s))
                ys.append(labels(s))
    X = torch.cat(Xs)
    y = torch.cat(ys)
    if samples and X.shape[0] > samples:
        g = torch.Generator(device="cpu").manual_seed(seed)
        idx = torch.randperm(X.shape[0], generator=g)[:samples].to(X.device)
        X, y = X[idx].contiguous(), y[idx].contiguous()
    return X, y


def use_indicator(solver, mlp, threshold, period=1):
    """Every following step of 'solver' starts with the indicator on U, or
    every second step with its flags dilated by one cell (period 2)."""
    capi.check(solver._lib.mmf_set_indicator(solver._ctx, mlp.handle if mlp is not None else None, threshold))
    if mlp is not None:
        capi.check(solver._lib.mmf_set_indicator_period(solver._ctx, period))


def run_indicator(solver, mlp, threshold):
    """Indicator on the uploaded state: returns (probabilities, flags) in raw order."""
    p = np.empty(solver.ncells, dtype=np.float32)
    f = np.empty(solver.ncells, dtype=np.uint8)
    capi.check(solver._lib.mmf_indicator(solver._ctx, mlp.handle, threshold, capi.ptr(p), capi.ptr(f)))
    return p, f
