"""The learned initial guess of the Poisson problems.

CPU: the oracle network's analytic backward against central finite
differences (float64), and its BF16 rounding.  GPU: the library's forward
pass and parameter gradient against the oracle with the same BF16 rounding
points; Adam steps lowering the loss; and the guess in the solver: trained
on the solver's own (rhs, solution) pairs, it never raises the starting
residual or the number of corrections (the gain it brings is printed), every
problem still converges to the same tolerance, and the state matches the run
without it.
"""
import numpy as np
import pytest

from ekcases import rel_l2, small_case
from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL
from oracle.unet_ref import Net, bf16, init_params, layer_specs


def test_oracle_backward_matches_finite_differences():
    cin, C = 2, 8
    rng = np.random.default_rng(1)
    p0 = init_params(cin, C, 0).astype(np.float64)
    p = p0 + 0.05 * rng.standard_normal(p0.size)
    x = rng.standard_normal((2, 32, 32, cin))
    t = rng.standard_normal((2, 32, 32))
    loss_of = lambda q: Net(q, cin, C, bf16_round=False).loss_and_grads(x, t, 29, 27)[0]
    _, _, g = Net(p, cin, C, bf16_round=False).loss_and_grads(x, t, 29, 27)
    assert (g != 0).mean() > 0.5
    for i in rng.choice(p.size, 24, replace=False):
        e = 1e-6
        qp, qm = p.copy(), p.copy()
        qp[i] += e
        qm[i] -= e
        fd = (loss_of(qp) - loss_of(qm)) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 * (abs(g[i]) + 1e-3 * np.abs(g).max()), i


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -3.14159265, np.inf], np.float32)
    r = bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even (down)
    assert r[2] == 1.0 + 4 * 2 ** -8               # tie to even (up)
    assert r[3] == 1.0 and r[5] == np.inf
    assert r[4] == np.float32(-3.140625)


# --------------------------------------------------------------------------- GPU

def unet_pair(C, n=2, h=32, w=32, seed=0):
    import torch
    from ekman_bl_gb300.duct import UNet
    cin = 2
    rng = np.random.default_rng(seed)
    p = init_params(cin, C, seed)
    p = (p + 0.05 * rng.standard_normal(p.size)).astype(np.float32)
    net = UNet(cin, C, n, h, w)
    net.set_params(p)
    x = rng.standard_normal((n, h, w, cin)).astype(np.float32)
    t = rng.standard_normal((n, h, w)).astype(np.float32)
    return net, p, x, t, torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("C", [8, 32])
def test_gpu_gradient_matches_oracle(C):
    import torch
    n, h, w, hv, wv = 2, 32, 32, 29, 27
    net, p, x, t, xd, td = unet_pair(C, n, h, w)
    yd = torch.zeros((n, h, w), device="cuda")
    loss, g = net.gradient(xd.data_ptr(), td.data_ptr(), n, hv, wv, yd.data_ptr())
    y = yd.cpu().numpy()
    rloss, ry, rg = Net(p, 2, C, bf16_round=True).loss_and_grads(x, t, hv, wv)
    # The GPU accumulates in FP32 in another order than the oracle, so a few
    # values land on the other side of a BF16 rounding boundary and the
    # difference grows through the 15 layers; a wrong index or mask would
    # show as an O(1) error.
    errs = []
    off = 0
    for l, (ci, co, *_) in enumerate(layer_specs(2, C)):
        k = co * 9 * ci + co
        a, b = g[off:off + k], rg[off:off + k]
        errs.append(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))
        off += k
    yerr = np.linalg.norm(y - ry) / np.linalg.norm(ry)
    print(f"C={C} loss {loss:.6g} vs {rloss:.6g}, output {yerr:.2e}, layer gradients", np.round(errs, 5))
    assert off == g.size
    assert abs(loss - rloss) <= 2e-3 * rloss
    assert yerr <= 5e-3
    assert max(errs) <= 2e-2, errs
    # the forward-only entry point gives the same output
    y2 = torch.zeros((n, h, w), device="cuda")
    net.forward(xd.data_ptr(), n, y2.data_ptr())
    assert torch.equal(y2, yd)


@pytest.mark.gpu
@pytest.mark.parametrize("C", [16, 32])
def test_tcgen05_forward_matches_mma_sync(C):
    """The forward convolutions with channel counts that are multiples of 16
    on the tcgen05 kernel (TMEM accumulator) against all layers on the
    mma.sync kernel and against the BF16-rounding oracle: both accumulate the
    same BF16 products in FP32 in another order, so only values at a BF16
    rounding boundary differ, and a wrong operand layout would show as an
    O(1) error.  Also a batch whose pixel count is not a multiple of the
    kernel's 128-pixel tile."""
    import torch
    for n, h, w in ((2, 32, 32), (3, 24, 40)):
        net, p, x, t, xd, td = unet_pair(C, n, h, w)
        y_tc = torch.zeros((n, h, w), device="cuda")
        y_ms = torch.zeros((n, h, w), device="cuda")
        net.forward(xd.data_ptr(), n, y_tc.data_ptr())
        net.set_tcgen05(False)
        net.forward(xd.data_ptr(), n, y_ms.data_ptr())
        a, b = y_tc.cpu().numpy(), y_ms.cpu().numpy()
        ry = Net(p, 2, C, bf16_round=True).loss_and_grads(x, t, h, w)[1]
        e_ms, e_or = rel_l2(a, b), rel_l2(a, ry)
        print(f"C={C} {n}x{h}x{w}: tcgen05 vs mma.sync {e_ms:.2e}, vs oracle {e_or:.2e}, mma.sync vs oracle "
              f"{rel_l2(b, ry):.2e}")
        # (against the oracle the BF16 boundary effects reach ~1e-2 on these
        # random weights, for both kernels alike)
        assert e_ms <= 1e-2 and e_or <= 3e-2


@pytest.mark.gpu
def test_gpu_adam_lowers_loss():
    import torch
    n, h, w = 8, 32, 32
    net, p, x, t, xd, td = unet_pair(16, n, h, w, seed=3)
    # a target the network can represent: a smoothed copy of input channel 0
    xs = torch.from_numpy(x[..., 0]).cuda()
    tt = (0.25 * (xs + xs.roll(1, 1) + xs.roll(1, 2) + xs.roll((1, 1), (1, 2)))).contiguous()
    losses = [net.train_step(xd.data_ptr(), tt.data_ptr(), n, h, w, 3e-3) for _ in range(60)]
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.3 * losses[0], losses[::10]


def guess_case():
    p, xp, yp, st = small_case(nx=64, ny2=65, nz2=65, mg_stop=EK_MG_STOP_RESIDUAL)
    p.mg_tol, p.mg_maxcy, p.mg_fast = 1e-8, 40, 1
    return p, xp, yp, st


@pytest.mark.gpu
def test_guess_in_solver():
    from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
    from ekman_bl_gb300.learned import LearnedGuess
    p, xp, yp, st = guess_case()
    m = metrics_from_grid(p, xp, yp)
    a = DuctSolver(p, m)
    a.upload(*st)
    lg = LearnedGuess(a, factor=2, channels=32, seed=0)
    npairs = lg.collect(4)                          # 12 projections
    assert npairs == 12 * 2 * (p.nx // 3)
    rep = lg.train(iters=400, batch=16, lr=2e-3)
    assert rep["val_loss_after"] < 0.5 * rep["val_loss_before"], rep
    # the same state continued with and without the guess
    b = DuctSolver(p, m)
    b.upload(*a.download())
    b.set_time(*a.get_time()[:2])
    lg.enable()
    rho_g, cyc_g, rho_0, cyc_0 = [], [], [], []
    for rk in (1, 2, 3):
        a.rk_duct(rk)
        b.rk_duct(rk)
        r, c = a.last_guess_stats()
        rho_g.append(r)
        cyc_g.append(c)
        r, c = b.last_guess_stats()
        rho_0.append(r)
        cyc_0.append(c)
        # every kx^2 != 0 problem stops on the residual rule before the cap
        # (the kx = 0 pair keeps MUDPACK's capped cycles, guess or not)
        sa, sb = a.mg_stats(), b.mg_stats()
        assert sa["max_cycles"] < p.mg_maxcy and sb["max_cycles"] < p.mg_maxcy, (sa, sb)
        assert sa["n_not_converged"] == sb["n_not_converged"] <= 2
    print("rho with guess", rho_g, "cycles", cyc_g, "without", cyc_0, rep)
    # What the trained network gains: the starting residual |b - A g|/|b|
    # after the least-squares scaling (1 without a guess) and the mean number
    # of corrections.  The multigrid here already cuts the residual ~100x per
    # cycle and the residual is dominated by the high wavenumbers that an
    # averaged-grid guess cannot carry, so the gain is small; what must hold
    # is that the guess never raises the starting residual or the cycle count.
    assert rho_0 == [1.0, 1.0, 1.0]
    assert max(rho_g) <= 1.0 and min(rho_g) < 1.0, rho_g
    assert np.mean(cyc_g) <= np.mean(cyc_0), (cyc_g, cyc_0)
    for x_, y_ in zip(a.download(), b.download()):
        assert rel_l2(x_, y_) < 1e-6
