"""Reverse-mode adjoint of the FP64 step (mpmg_adj_forward_tape /
mpmg_adj_backward / mpmg_adj_gradient) against central finite differences of
the forward step, for g_local_mu2, isolin and g_nonlocal_mu2 (whose gradient
also covers the nonlocal amplitude A).

The loss is the squared distance of the final particle positions to a target
run with perturbed parameters (the adjoint benchmark's loss, on a small
column).  Finite differences use a relative step of 1e-4 on each parameter
(FP64 forward runs).  Criterion: |adjoint - FD| <= 1e-3 |FD| per parameter.
A thin torch.autograd.Function wraps the C-ABI pair here, in the test
harness only.
"""
import numpy as np
import pytest

import mpm2d
import scenes

pytestmark = pytest.mark.gpu

PARAMS = ("mu_s", "mu_2", "I0", "E")


def column(theta=None, material="g_local_mu2"):
    sc = scenes.column(Nx=33, Ny=33, h=1 / 32, width=0.25, height=0.4, material=material, rho=2450.0,
                       props=(1e6, 0.3), dt=1e-4, mp={"grains_d": 5.3e-4}, jitter=1e-3, seed=5)
    sc["gravity"] = -9.81
    if theta is not None:
        mp = dict(sc.get("mp", {}))
        mp.update({"mu_s": theta[0], "mu_2": theta[1], "I0": theta[2]})
        sc["mp"] = mp
        sc["props"] = [theta[3], 0.3]
    return sc


THETA0 = np.array([0.3819, 0.6435, 0.278, 1e6])
STEPS = 120


def final_positions(theta, steps=STEPS, material="g_local_mu2"):
    sim = mpm2d.Simulation(column(theta, material))
    sim.step(steps)
    x, y = sim.get("x"), sim.get("y")
    sim.close()
    return x, y


def loss(theta, target, material="g_local_mu2"):
    x, y = final_positions(theta, material=material)
    return float(np.sum((x - target[0]) ** 2 + (y - target[1]) ** 2))


def adjoint_grad(theta, target, K, material="g_local_mu2"):
    sim = mpm2d.Simulation(column(theta, material))
    sim.adj_forward_tape(STEPS, K)
    x, y = sim.get("x"), sim.get("y")
    g = sim.adj_backward(2 * (x - target[0]), 2 * (y - target[1]))
    return g, sim


@pytest.fixture(scope="module")
def target():
    return final_positions(THETA0 * np.array([1.0 + 0.02 / 0.3819, 1 - 0.03 / 0.6435, 1.0, 1.1]))


def test_adjoint_matches_central_differences(target):
    g, sim = adjoint_grad(THETA0, target, K=32)
    sim.close()
    for k, name in enumerate(PARAMS):
        h = 1e-4 * THETA0[k]
        tp, tm = THETA0.copy(), THETA0.copy()
        tp[k] += h
        tm[k] -= h
        fd = (loss(tp, target) - loss(tm, target)) / (2 * h)
        assert abs(g[k] - fd) <= 1e-3 * abs(fd), (name, g[k], fd)


def test_adjoint_isolin_young_modulus(target):
    theta = THETA0.copy()
    g, sim = adjoint_grad(theta, target, K=40, material="isolin")
    sim.close()
    h = 1e-4 * theta[3]
    tp, tm = theta.copy(), theta.copy()
    tp[3] += h
    tm[3] -= h
    fd = (loss(tp, target, "isolin") - loss(tm, target, "isolin")) / (2 * h)
    assert abs(g[3] - fd) <= 1e-3 * abs(fd), (g[3], fd)
    assert g[0] == 0 and g[1] == 0 and g[2] == 0


def test_checkpoint_interval_does_not_change_the_gradient(target):
    a, sa = adjoint_grad(THETA0, target, K=STEPS)
    b, sb = adjoint_grad(THETA0, target, K=7)
    np.testing.assert_array_equal(a, b)
    for f in ("x", "y", "vx", "sxx"):
        np.testing.assert_array_equal(sa.adj_state(f), sb.adj_state(f))
    # the contexts are left at the run's final state and keep stepping
    ref = mpm2d.Simulation(column(THETA0))
    ref.step(STEPS + 5)
    sa.step(5)
    np.testing.assert_array_equal(sa.get("x"), ref.get("x"))
    for s in (sa, sb, ref):
        s.close()


def test_initial_position_adjoint_matches_central_differences(target):
    # dL/dx0 of a few particles through the whole trajectory
    g, sim = adjoint_grad(THETA0, target, K=32)
    gx0 = sim.adj_state("x")
    sim.close()
    base = column(THETA0)
    rng = np.random.default_rng(0)
    for i in rng.choice(len(base["particles"]["x"]), size=3, replace=False):
        h = 1e-7
        vals = []
        for sgn in (1, -1):
            sc = column(THETA0)
            sc["particles"] = {k: np.array(v, copy=True) for k, v in sc["particles"].items()}
            sc["particles"]["x"][i] += sgn * h
            sim = mpm2d.Simulation(sc)
            sim.step(STEPS)
            x, y = sim.get("x"), sim.get("y")
            sim.close()
            vals.append(float(np.sum((x - target[0]) ** 2 + (y - target[1]) ** 2)))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(gx0[i] - fd) <= 1e-3 * abs(fd) + 1e-9, (i, gx0[i], fd)


def test_torch_autograd_wrapper(target):
    torch = pytest.importorskip("torch")

    class Trajectory(torch.autograd.Function):
        """Final positions as a function of (mu_s, mu_2, I0, E): forward through
        mpmg_adj_forward_tape, backward through mpmg_adj_backward."""

        @staticmethod
        def forward(ctx, theta):
            sim = mpm2d.Simulation(column(theta.detach().cpu().numpy()))
            sim.adj_forward_tape(STEPS, 32)
            ctx.sim = sim
            return (torch.from_numpy(sim.get("x")), torch.from_numpy(sim.get("y")))

        @staticmethod
        def backward(ctx, gx, gy):
            g = ctx.sim.adj_backward(gx.numpy(), gy.numpy())
            ctx.sim.close()
            return torch.from_numpy(g[:4])     # (mu_s, mu_2, I0, E); g[4] is A's

    theta = torch.tensor(THETA0, dtype=torch.float64, requires_grad=True)
    x, y = Trajectory.apply(theta)
    L = ((x - torch.from_numpy(target[0])) ** 2 + (y - torch.from_numpy(target[1])) ** 2).sum()
    L.backward()
    g, sim = adjoint_grad(THETA0, target, K=32)
    sim.close()
    np.testing.assert_allclose(theta.grad.numpy(), g[:4], rtol=1e-12, atol=0)


# g_nonlocal_mu2: the fluidity solve reversed by a solve of the same symmetric
# system for the fluidity's adjoint, so the gradient also reaches the
# nonlocal amplitude A.  A 32^2 silo from a lithostatic stress above yield
# (the fluidity is non-trivial from the first step), outlet open, 40 steps.
NL_THETA0 = np.array([0.3819, 0.6435, 0.278, 1e6, 0.48])
NL_STEPS = 40


def nl_silo(theta):
    mp = {"grains_d": 5.3e-4, "mu_s": theta[0], "mu_2": theta[1], "I0": theta[2], "A": theta[4]}
    return scenes.silo_prestressed(cells=32, dt=1e-4, mp=mp, props=(theta[3], 0.3))


def nl_final(theta):
    sim = mpm2d.Simulation(nl_silo(theta))
    sim.step(NL_STEPS)
    x, y = sim.get("x"), sim.get("y")
    sim.close()
    return x, y


def test_nonlocal_adjoint_matches_central_differences():
    tx, ty = nl_final(NL_THETA0 * np.array([1.05, 0.95, 1.0, 1.1, 1.2]))

    def nl_loss(theta):
        x, y = nl_final(theta)
        return float(np.sum((x - tx) ** 2 + (y - ty) ** 2))

    sim = mpm2d.Simulation(nl_silo(NL_THETA0))
    sim.adj_forward_tape(NL_STEPS, 10)
    x, y = sim.get("x"), sim.get("y")
    g = sim.adj_backward(2 * (x - tx), 2 * (y - ty))
    sim.close()
    for k, name in enumerate(PARAMS + ("A",)):
        h = 1e-4 * NL_THETA0[k]
        tp, tm = NL_THETA0.copy(), NL_THETA0.copy()
        tp[k] += h
        tm[k] -= h
        fd = (nl_loss(tp) - nl_loss(tm)) / (2 * h)
        assert abs(g[k] - fd) <= 1e-3 * abs(fd), (name, g[k], fd)

