"""The learned initial guess of the per-kx Poisson problems: collect
(right-hand side, solution) pairs from the solver's own projections, train
the U-Net on the GPU with the library's kernels, and switch the guess on.

The multigrid stays the solver: the guess only replaces the zero starting
iterate of the kx^2 != 0 problems (scaled by the least-squares factor), the
stopping tolerance is unchanged, and a guess that does not help gets a
factor near zero.  Device buffers are torch CUDA tensors (plumbing only:
every arithmetic operation on them runs in the library's kernels; torch
only allocates, shuffles whole images and synchronises).
"""
from __future__ import annotations

import time

import numpy as np

from .duct import DuctSolver, UNet


def layer_specs(cin: int, C: int):
    """(cin, cout) of the 15 convolutions in the library's parameter order."""
    s = [(cin, C)] + [(C, C)] * 7
    for _ in range(3):
        s += [(2 * C, C), (C, C)]
    return s + [(C, 1)]


def he_init(cin: int, C: int, seed: int) -> np.ndarray:
    """He-normal weights (std sqrt(2 / (9 cin))), zero biases, flat FP32."""
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co in layer_specs(cin, C):
        parts.append((rng.standard_normal(co * 9 * ci) * np.sqrt(2.0 / (9 * ci))).astype(np.float32))
        parts.append(np.zeros(co, np.float32))
    return np.concatenate(parts)


class LearnedGuess:
    """One network for one solver's grid (images of the finest multigrid
    grid averaged over factor x factor blocks)."""

    def __init__(self, solver: DuctSolver, factor: int = 4, channels: int = 32, seed: int = 0):
        import torch
        self.torch = torch
        self.solver, self.factor, self.channels = solver, factor, channels
        self.h, self.w, self.hv, self.wv = solver.guess_geometry(factor)
        self.nq = 2 * (solver.p.nx // 3)          # kx^2 != 0 problems per projection
        self.net = UNet(2, channels, max(self.nq, 64), self.h, self.w)
        self.net.set_params(he_init(2, channels, seed))
        self.x = self.t = None
        self.npairs = 0

    def collect(self, nsteps: int, capacity: int | None = None) -> int:
        """Run nsteps RK3 steps of the solver, keeping the (input, target)
        pairs of every projection; returns the number of pairs."""
        torch = self.torch
        cap = capacity or nsteps * 3 * self.nq
        self.x = torch.empty((cap, self.h, self.w, 2), dtype=torch.float32, device="cuda")
        self.t = torch.empty((cap, self.h, self.w), dtype=torch.float32, device="cuda")
        self.solver.set_pair_sink(self.x.data_ptr(), self.t.data_ptr(), cap, self.factor)
        try:
            self.solver.step(nsteps)
        finally:
            self.npairs = self.solver.pair_count()
            self.solver.set_pair_sink(None, None)
        return self.npairs

    def train(self, iters: int, batch: int = 16, lr: float = 1e-3, val_frac: float = 0.1, seed: int = 0) -> dict:
        """Adam on shuffled minibatches of the collected pairs, cosine-decayed
        learning rate; the last val_frac of the pairs (the latest projections)
        are held out."""
        torch = self.torch
        n = self.npairs
        nval = max(1, int(round(n * val_frac)))
        ntr = n - nval
        if ntr < batch:
            raise ValueError(f"{n} pairs: too few to train with batch {batch}")
        g = torch.Generator(device="cpu").manual_seed(seed)
        order = torch.randperm(ntr, generator=g).to("cuda")
        xs = self.x[:ntr].index_select(0, order).contiguous()
        ts = self.t[:ntr].index_select(0, order).contiguous()
        xv, tv = self.x[ntr:n].contiguous(), self.t[ntr:n].contiguous()
        val0 = self.val_loss(xv, tv)
        t0 = time.perf_counter()
        losses = []
        nb = ntr // batch
        for it in range(iters):
            b = it % nb
            if b == 0 and it > 0:
                perm = torch.randperm(ntr, generator=g).to("cuda")
                xs = xs.index_select(0, perm).contiguous()
                ts = ts.index_select(0, perm).contiguous()
            lr_it = lr * 0.5 * (1.0 + np.cos(np.pi * it / iters))
            losses.append(self.net.train_step(xs[b * batch].data_ptr(), ts[b * batch].data_ptr(), batch,
                                              self.hv, self.wv, lr_it))
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        return {"pairs": n, "train_pairs": ntr, "val_pairs": nval, "iters": iters, "batch": batch,
                "first_loss": float(np.mean(losses[:10])), "last_loss": float(np.mean(losses[-10:])),
                "val_loss_before": val0, "val_loss_after": self.val_loss(xv, tv), "train_s": secs}

    def val_loss(self, xv, tv) -> float:
        tot, m = 0.0, 0
        chunk = min(32, self.net.max_batch)
        for s in range(0, xv.shape[0], chunk):
            k = min(chunk, xv.shape[0] - s)
            loss, _ = self.net.gradient(xv[s].data_ptr(), tv[s].data_ptr(), k, self.hv, self.wv)
            tot += loss * k
            m += k
        return tot / max(m, 1)

    def enable(self, on: bool = True):
        self.solver.set_poisson_guess(self.net if on else None, self.factor)
