"""Training of the troubled-cell indicator on the GPU.

Labels are where the order-2 limiter (every cell limited, reference
arithmetic) changes a slope, on states of seeded radial-Sod and isentropic-
vortex runs of the plain order-2 solver; features are the normalised
primitive stencils of the same states.  1e6 samples are drawn from the
snapshots and the MLP is trained with the project's own forward, backward and
Adam kernels.

    python -m minimmerflow_gb300.train_indicator --dim 3 --out minimmerflow_gb300/data/indicator_3d.npy
"""
import argparse
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def default_weights_path(dim):
    return os.path.join(HERE, "data", "indicator_%dd.npy" % dim)


def training_cases(dim, seed=20261203, ncases=16, cfl=0.4):
    """Seeded Sod (pressure ratio log-U[2,100], density ratio U[2,10]) and vortex
    (beta U[1,8]) runs on a few resolutions, at the CFL the indicator is used with."""
    from . import problem as P
    rng = np.random.default_rng(seed)
    sizes = (32, 40, 48) if dim == 3 else (96, 128, 192, 256)
    cases = []
    for i in range(ncases):
        n = int(sizes[i % len(sizes)])
        if i % 2 == 0:
            pr = float(np.exp(rng.uniform(np.log(2.0), np.log(100.0))))
            rr = float(rng.uniform(2.0, 10.0))
            c = P.radial_sod_ratios(n, pr, rr, dim=dim)
        else:
            c = P.vortex(dim, n, beta=float(rng.uniform(1.0, 8.0)))
        c.cfl = cfl
        cases.append(c)
    return cases


def calibrate_threshold(mlp, X, y, recall=0.999):
    """Largest threshold whose recall of the troubled cells on (X, y) is >= recall."""
    import torch
    prob = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
    mlp.predict(X, prob)
    p = prob[y.bool()].float().cpu().numpy()
    if p.size == 0:
        return 0.5
    return float(np.quantile(p, 1.0 - recall))


def train(dim=3, samples=1_000_000, epochs=8, batch=4096, lr=2e-3, seed=20261203, log=print, holdout=0.1,
          recall=0.999):
    """Returns (mlp, losses, threshold): the threshold keeps 'recall' of the
    troubled cells of a held-out part of the data above it."""
    import torch
    from . import indicator
    t0 = time.time()
    X, y = indicator.generate_dataset(training_cases(dim, seed), snapshots=6, steps_between=8,
                                      samples=int(samples / (1.0 - holdout)), seed=seed)
    nh = int(holdout * X.shape[0])
    Xh, yh, X, y = X[:nh], y[:nh], X[nh:], y[nh:]
    if log:
        log("dataset: %d samples (+%d held out), %.1f%% troubled, %.1f s"
            % (X.shape[0], nh, 100.0 * float(y.float().mean()), time.time() - t0))
    mlp = indicator.TroubledCellMLP(dim=dim, seed=seed)
    losses = mlp.fit(X, y, epochs=epochs, batch=batch, lr=lr, seed=seed, log=log)
    thr = calibrate_threshold(mlp, Xh, yh, recall)
    if log:
        prob = torch.empty(Xh.shape[0], dtype=torch.float32, device=Xh.device)
        mlp.predict(Xh, prob)
        log("threshold %.4f: recall %.4f, cells skipping the limiter %.3f"
            % (thr, float((prob[yh.bool()] > thr).float().mean()), float((prob <= thr).float().mean())))
    return mlp, losses, thr


def load(dim, path=None, device=0):
    """(mlp, threshold) from a weights file, or (None, None) if it is absent.
    The file holds the parameters followed by the calibrated threshold."""
    from . import indicator
    path = path or default_weights_path(dim)
    if not os.path.exists(path):
        return None, None
    mlp = indicator.TroubledCellMLP(dim=dim, device=device)
    data = np.load(path)
    mlp.set_params(data[:mlp.nparams])
    thr = float(data[mlp.nparams]) if data.size > mlp.nparams else 0.1
    return mlp, thr


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--samples", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    mlp, losses, thr = train(args.dim, args.samples, args.epochs)
    out = args.out or default_weights_path(args.dim)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.save(out, np.concatenate([mlp.params(), np.array([thr], dtype=np.float32)]))
    print("saved", out, "final loss %.5f, threshold %.4f" % (losses[-1], thr))


if __name__ == "__main__":
    main()
