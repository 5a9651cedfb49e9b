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


def training_cases(dim, seed=20261203):
    """Seeded Sod (pressure ratio log-U[2,100], density ratio U[2,10]) and vortex (beta U[1,8]) runs."""
    from . import problem as P
    rng = np.random.default_rng(seed)
    n = 40 if dim == 3 else 128
    cases = []
    for i in range(8):
        if i % 2 == 0:
            pr = float(np.exp(rng.uniform(np.log(2.0), np.log(100.0))))
            rr = float(rng.uniform(2.0, 10.0))
            cases.append(P.radial_sod_ratios(n, pr, rr, dim=dim))
        else:
            cases.append(P.vortex(dim, n, beta=float(rng.uniform(1.0, 8.0))))
    return cases


def train(dim=3, samples=1_000_000, epochs=8, batch=4096, lr=2e-3, seed=20261203, log=print):
    from . import indicator
    t0 = time.time()
    X, y = indicator.generate_dataset(training_cases(dim, seed), snapshots=6, steps_between=8, samples=samples,
                                      seed=seed)
    if log:
        log("dataset: %d samples, %.1f%% troubled, %.1f s" % (X.shape[0], 100.0 * float(y.float().mean()),
                                                              time.time() - t0))
    mlp = indicator.TroubledCellMLP(dim=dim, seed=seed)
    losses = mlp.fit(X, y, epochs=epochs, batch=batch, lr=lr, seed=seed, log=log)
    return mlp, losses, (X, y)


def load(dim, path=None, device=0):
    """The trained indicator from a weights file (None if the file is absent)."""
    from . import indicator
    path = path or default_weights_path(dim)
    if not os.path.exists(path):
        return None
    mlp = indicator.TroubledCellMLP(dim=dim, device=device)
    mlp.set_params(np.load(path))
    return mlp


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--samples", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    mlp, losses, _ = train(args.dim, args.samples, args.epochs)
    out = args.out or default_weights_path(args.dim)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.save(out, mlp.params())
    print("saved", out, "final loss %.5f" % losses[-1])


if __name__ == "__main__":
    main()
