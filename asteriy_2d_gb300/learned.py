"""The learned start value of the exact Riemann solver, end to end.

1. record: run the FP64 exact-Godunov solver and record every face that needs
   the iterative p* solve (features, converged log(p*/p_L), step, face id);
2. sample: order the records by (step, face id) so the set is independent of
   the GPU's scheduling, and draw a uniform sample without replacement from
   numpy's Generator(PCG64(seed));
3. train: initialise (ast_mlp_init) and train with the CUDA kernels
   (ast_mlp_train, Adam, mean-squared error);
4. use: Solver.set_mlp(params) on a solver with guess = MLP.
"""
import numpy as np

from . import abi as A
from .solver import Solver, mlp_init, mlp_train


def record_faces(cfg, s0, u0, nsteps, every=1, capacity=1 << 24, min_strength=0.0):
    """Records of the iterative exact-solver faces over nsteps FP64 steps
    (only those with wave strength above min_strength when it is positive)."""
    c = cfg.copy()
    c.precision = A.PREC_FP64
    c.flux = A.FLUX_GODUNOV
    c.guess = A.GUESS_PVRS
    with Solver(c) as S:
        S.set_state(s0, u0)
        S.record_start(capacity, every, min_strength)
        S.step(nsteps)
        rec, offered = S.record_stop()
    key_step = rec[:, 7].view(np.int32).astype(np.int64)
    key_face = rec[:, 8].view(np.int32).astype(np.int64)
    order = np.lexsort((key_face, key_step))
    return rec[order], offered


def sample_indices(n, k, seed=7):
    """Sorted indices of a uniform sample of min(k, n) of n records."""
    if n <= k:
        return np.arange(n)
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.sort(rng.choice(n, size=k, replace=False))


def sample_records(rec, k, seed=7):
    return rec[sample_indices(len(rec), k, seed)]


def train_guess(samples, epochs=20, batch=8192, lr=3e-3, seed=7):
    params = mlp_init(samples, seed)
    params, losses = mlp_train(samples, params, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return params, losses


def strength(rec):
    """Wave strength of recorded faces, max(|ln(p_R/p_L)|, |u_R-u_L|/min(c_L,c_R)),
    from the record's features (the gate the solver applies before using the
    learned start value)."""
    x1, x2, x3 = rec[:, 1].astype(np.float64), rec[:, 2].astype(np.float64), rec[:, 3].astype(np.float64)
    return np.maximum(np.abs(np.log(x1)), np.abs(x2) / np.minimum(1.0, x3))


def strong_records(rec, gate=0.2):
    """The recorded faces above the gate: the ones the learned start value serves."""
    return rec[strength(rec) > gate]
