"""The multigrid-preconditioned fluidity solve (the default preconditioner).

The reference solves the nonlocal fluidity system by sparse LU
(g_nonlocal_mu2.c:510-519; CXSparse is not vendored); the library solves the
same assembled system by conjugate gradients to a relative residual.  These
tests check that the multigrid V-cycle preconditioner gives the same solution
as the Jacobi one and as the oracle, on every hierarchy shape the solver
builds:

  * the pre-stressed 33^2 silo of the golden fixtures (one block holds every
    level in shared memory), against the reference's trajectory, for both
    preconditioners;
  * a pre-stressed column on a 257 x 65 grid (level 0 spread over 33 blocks,
    coarse levels held by one block, the y direction no longer coarsened
    below 3 rows), one step against the oracle's CG at 1e-12.

The 513^2 silo (spread levels 0-3) is checked against the oracle's direct
solve in test_gpu_full_size.py.
"""
import os

import numpy as np
import pytest

from conftest import field_err, load_golden, rel_err
from oracle import oracle as O
import mpm2d
import scenes

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_multigrid_and_jacobi_agree_on_golden_silo():
    scene, d = load_golden("nonlocal_mu2_prestressed")
    sims = {pc: mpm2d.Simulation(scene, solver_tol=1e-12, solver_maxit=50000, precond=pc)
            for pc in ("multigrid", "jacobi")}
    done = 0
    iters = {pc: [] for pc in sims}
    for c in (int(c) for c in d["checkpoints"]):
        for pc, sim in sims.items():
            sim.step(c - done)
            rc, it, resid = sim.last_solve()
            assert rc == 0 and resid <= 1e-12, (pc, c, rc, resid)
            iters[pc].append(it)
            want = lambda f, c=c: d["s%d_%s" % (c, f)]
            for f in ("sxx", "sxy", "syy", "x", "y", "vx", "vy"):
                assert field_err(sim.get(f), want, f) <= 1e-8, (pc, c, f)
        done = c
        ga, gb = sims["multigrid"].get("node_gf"), sims["jacobi"].get("node_gf")
        assert rel_err(ga, gb) <= 1e-10, (c, rel_err(ga, gb))
    # the V-cycle makes the count independent of the grid
    assert max(iters["multigrid"]) <= 20, iters
    for sim in sims.values():
        sim.close()


def prestressed_column(Nx=257, Ny=65, width=0.6, height=0.3, k0=0.4, surcharge=500.0, rho=2450.0):
    h = 2.0 / (Nx - 1)
    sc = scenes.column(Nx=Nx, Ny=Ny, h=h, width=width, height=height, ppc_1d=2, material="g_nonlocal_mu2",
                       rho=rho, props=(1e6, 0.3), dt=1e-5, gravity=-9.8,
                       mp={"grains_d": 5.3e-4, "A": 0.48})
    p = sc["particles"]
    H = float(np.max(p["y"])) + 0.25 * h
    p["syy"] = -rho * 9.8 * (H - p["y"]) - surcharge
    p["sxx"] = k0 * p["syy"]
    return sc


@pytest.mark.parametrize("precond", ["multigrid", "jacobi"])
def test_rectangular_multiblock_solve_vs_oracle(precond):
    sc = prestressed_column()
    sim = mpm2d.Simulation(sc, store_transients=True, solver_tol=1e-12, solver_maxit=50000, precond=precond)
    orc = O.Oracle(sc, nthreads=THREADS, solver="cg", cg_tol=1e-12)
    for _ in range(2):
        sim.step(1)
        orc.step(1)
        rc, iters, resid = sim.last_solve()
        assert rc == 0 and resid <= 1e-12, (rc, resid)
        assert np.array_equal(sim.get_map()[1], orc.get_map()[1])
        gf = rel_err(sim.get("node_gf"), orc.get("node_gf"))
        assert gf <= 1e-9, gf
        for f in ("sxx", "sxy", "syy", "x", "y", "vx", "vy"):
            err = field_err(sim.get(f), orc.get, f)
            assert err <= 1e-8, (f, err)
    if precond == "multigrid":
        assert iters <= 20, iters
    sim.close()


@pytest.mark.parametrize("precond", ["multigrid", "jacobi"])
def test_iteration_cap_reports_non_convergence(precond):
    """A solve stopped by solver_maxit before the tolerance reports
    MPMG_ERR_SOLVER (the reference's EXIT_ERROR_CS_SOL) at the next
    read-back, and last_solve gives the iterations it ran.  (The silo starts
    above yield everywhere, so the first step's system has a load.)"""
    scene = scenes.silo_prestressed(cells=32, dt=1e-5)
    sim = mpm2d.Simulation(scene, solver_tol=1e-14, solver_maxit=2, precond=precond)
    with pytest.raises(mpm2d.MpmError) as e:
        sim.step(1)
        sim.synchronize()
    assert e.value.status == 2, e.value
    rc, iters, resid = sim.last_solve()
    assert iters == 2 and resid > 1e-14, (rc, iters, resid)
    sim.close()


def test_multigrid_warm_start_agrees_with_cold():
    """With the previous step's fluidity as the start, the solve meets the
    same tolerance in no more iterations, and the trajectory agrees with the
    cold-started one to the solve's tolerance."""
    scene = scenes.silo_prestressed(cells=64, dt=1e-5)
    cold = mpm2d.Simulation(scene, solver_tol=1e-12, solver_maxit=50000)
    warm = mpm2d.Simulation(scene, solver_tol=1e-12, solver_maxit=50000, warm_start=True)
    it_cold, it_warm = [], []
    for _ in range(5):
        cold.step(1)
        warm.step(1)
        rc_c, ic, _ = cold.last_solve()
        rc_w, iw, rw = warm.last_solve()
        assert rc_c == 0 and rc_w == 0 and rw <= 1e-12
        it_cold.append(ic)
        it_warm.append(iw)
    assert sum(it_warm) <= sum(it_cold), (it_warm, it_cold)
    assert rel_err(warm.get("node_gf"), cold.get("node_gf")) <= 1e-9
    for f in ("sxx", "sxy", "syy", "x", "y"):
        assert rel_err(warm.get(f), cold.get(f)) <= 1e-9, f
    cold.close()
    warm.close()
