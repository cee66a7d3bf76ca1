"""The oracle pinned against the reference: golden vectors recorded from the
reference's own compiled code (tests/golden/), and, where the reference tree
is present, the live reference build.  CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, rel_err, state_at
from oracle import build as obuild
from oracle import oracle as O
import scenes

CASES = ["config1", "mu2_column", "mu2_silo", "nonlocal_mu2_silo", "nonlocal_mu2_prestressed",
         "nonlocal_silo", "musl_config1", "musl_mu2_column", "dp_column", "dp_silo",
         "musl_dp_column", "ps_column", "ps_silo", "t2d_column", "t2d_silo",
         "ext_column", "ext_silo", "nonlocal_avg_silo", "rev_column", "rev_silo"]
COMPARE = ["x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy", "exx", "exy", "eyy", "wxy",
           "ax", "ay"]


def test_band_solver_matches_dense():
    rng = np.random.default_rng(3)
    n, w = 60, 7
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - w), i + 1):
            A[i, j] = A[j, i] = rng.normal()
    A = A @ A.T + n * np.eye(n)          # SPD, wider band is fine for the check
    A[np.abs(np.subtract.outer(np.arange(n), np.arange(n))) > w] = 0.0
    A += n * np.eye(n)
    b = rng.normal(size=n)
    import ctypes as C
    lib = C.CDLL(obuild.build_oracle())
    band = np.zeros((n, w + 1))
    for i in range(n):
        for j in range(max(0, i - w), i + 1):
            band[i, j - i + w] = A[i, j]
    x = b.copy()
    dp = C.POINTER(C.c_double)
    lib.oracle_band_ldlt_solve.argtypes = [C.c_long, C.c_long, dp, dp]
    assert lib.oracle_band_ldlt_solve(n, w, band.ctypes.data_as(dp), x.ctypes.data_as(dp)) == 1
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_golden(case):
    scene, d = load_golden(case)
    orc = O.Oracle(scene, nthreads=2)
    done = 0
    for c in d["checkpoints"]:
        orc.step(int(c) - done)
        done = int(c)
        for f in COMPARE + ["state%d" % k for k in range(11)]:
            got, want = orc.get(f), d["s%d_%s" % (c, f)]
            assert rel_err(got, want) <= 1e-12, (case, c, f, rel_err(got, want))
        e, a = orc.get_map()
        np.testing.assert_array_equal(e, d["s%d_in_element" % c])
        np.testing.assert_array_equal(a, d["s%d_active" % c])
        for f in ("node_m", "node_mx", "node_my", "node_fx", "node_fy", "node_vx", "node_vy"):
            assert rel_err(orc.get(f), d["s%d_%s" % (c, f)]) <= 1e-12, (case, c, f)
        assert orc.t == float(d["s%d_t" % c])


def test_oracle_restart_from_checkpoint_matches_next_step():
    """Teacher forcing: restart the oracle from the reference's state after
    step 1 and compare one step with the reference's step 2."""
    scene, d = load_golden("config1")
    sc = dict(scene)
    st = state_at(d, 1, "isolin")
    sc["particles"] = {"m": scene["particles"]["m"], "v": st["v"], "x": st["x"], "y": st["y"],
                       "vx": st["vx"], "vy": st["vy"], "sxx": st["sxx"], "sxy": st["sxy"],
                       "syy": st["syy"]}
    orc = O.Oracle(sc, nthreads=1)
    orc.set("ux", st["ux"])
    orc.set("uy", st["uy"])
    orc.set("v0", scene["particles"]["v"])
    orc.set_map(d["s1_in_element"], d["s1_active"])
    orc.set_time(float(d["s1_t"]), 1)
    # the driver's time_varying_loads after step 1 (loading.c:34-54)
    orc.set("by", np.full(len(st["x"]), -9.8 * ((float(d["s1_t"]) - 0.0) / 0.1)))
    orc.step(1)
    for f in ("x", "y", "vx", "vy", "sxx", "sxy", "syy"):
        np.testing.assert_array_equal(orc.get(f), d["s2_%s" % f])


def _test_material_history(kind, rows, props, dt):
    """tests/test_material.c:36-195 for one particle, through the oracle."""
    scene = {"Nx": 2, "Ny": 2, "h": 1.0, "dt": dt, "material": kind, "props": list(props),
             "bc": "box", "bcf": [0, 0, 1, 1], "bci": [0, 0, 0, 0],
             "particles": {"m": [2450.0], "v": [1.0], "x": [0.5], "y": [0.5], "vx": [0.0],
                           "vy": [0.0], "sxx": [-1.0], "sxy": [0.0], "syy": [-1.0]}}
    orc = O.Oracle(scene)
    t = 0.0
    out = []
    v = 1.0
    for _ in range(len(rows) - 1):
        L = _velocity_gradient(t)
        orc.set("exx", [L[0]])
        orc.set("exy", [0.5 * (L[1] + L[2])])
        orc.set("wxy", [0.5 * (L[1] - L[2])])
        orc.set("eyy", [L[3]])
        orc.material_only()
        v = v * np.exp(dt * (L[0] + L[3]))
        orc.set("v", [v])
        t += dt
        out.append([orc.get("sxx")[0], orc.get("sxy")[0], orc.get("syy")[0], orc.get("state10")[0]])
    return np.array(out)


def _velocity_gradient(t):
    """set_velocity_gradient, tests/test_material.c:36-81."""
    sh = 0.5
    if 0 <= t < 0.25:
        L = [0, sh, 0, 0]
    elif 0.25 <= t < 0.5:
        a = -1 * (0.125 - abs(t - 0.375)) / 0.125
        L = [a, sh, 0, a]
    elif 0.5 <= t < 0.75:
        L = [0, sh, 0, 0]
    elif 0.75 <= t < 1:
        a = 1 * (0.125 - abs(t - 0.875)) / 0.125
        L = [a, sh, 0, a]
    else:
        L = [0, sh, 0, 0]
    return [v * 1e-1 for v in L]


@pytest.mark.parametrize("kind", ["isolin", "g_local_mu2", "dp_ri_mt", "g_local_mu2_plane_strain",
                                  "g_local_mu2_true_2d", "g_local_mu2_reverse"])
def test_oracle_material_known_answers(kind):
    d = np.load(os.path.join(GOLDEN, "kat_%s.npz" % kind))
    rows = d["rows"]
    got = _test_material_history(kind, rows, d["props"], float(d["dt"]))
    np.testing.assert_array_equal(got[:, 0], rows[1:, 5])
    np.testing.assert_array_equal(got[:, 1], rows[1:, 6])
    np.testing.assert_array_equal(got[:, 2], rows[1:, 7])
    np.testing.assert_array_equal(got[:, 3], rows[1:, 9])


needs_ref = pytest.mark.skipif(not obuild.have_reference(), reason="reference tree not present")


@needs_ref
@pytest.mark.parametrize("threads", [1, 3])
def test_oracle_matches_live_reference_threads(threads):
    sc = scenes.config1(seed=5)
    ref = O.RefHarness(sc, nthreads=threads)
    orc = O.Oracle(sc, nthreads=threads)
    ref.step(60)
    orc.step(60)
    p = ref.particles()
    for f in ("x", "y", "vx", "vy", "sxx", "sxy", "syy", "v"):
        np.testing.assert_array_equal(orc.get(f), p[f])
    lo, ll = orc.color_lists()
    lr, lrl = ref.color_lists()
    np.testing.assert_array_equal(ll, lrl)
    np.testing.assert_array_equal(lo, lr)


@needs_ref
def test_oracle_nonlocal_threads_deterministic():
    """With several threads the oracle equals the single-thread reference (the
    reference itself races there)."""
    sc = scenes.silo(cells=16, material="g_nonlocal_mu2", props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                     open_time=0.0, wall_frac=0.5, fill_height=0.6)
    ref = O.RefHarness(sc, nthreads=1)
    ref.step(40)
    for threads in (2, 4):
        orc = O.Oracle(sc, nthreads=threads)
        orc.step(40)
        np.testing.assert_array_equal(orc.get("sxx"), ref.particles()["sxx"])


def test_oracle_pcg_matches_direct():
    scene, _ = load_golden("nonlocal_mu2_silo")
    a = O.Oracle(scene, solver="direct")
    b = O.Oracle(scene, solver="pcg", cg_tol=1e-13)
    a.step(30)
    b.step(30)
    assert rel_err(b.get("state3"), a.get("state3")) < 1e-8
    assert rel_err(b.get("sxx"), a.get("sxx")) < 1e-9


def test_oracle_particles_leave_through_trapdoor():
    sc = scenes.silo(cells=16, material="g_local_mu2", props=(1e6, 0.3), dt=2e-5, hole_radius=0.3,
                     open_time=0.0, wall_frac=0.5, fill_height=0.3, gravity=-200.0)
    orc = O.Oracle(sc, nthreads=2)
    orc.step(800)
    _, act = orc.get_map()
    assert act.sum() < len(act)          # some particles fell out and went inactive
    e, _ = orc.get_map()
    assert np.all(e[act == 0] == -1) or np.all(act[e == -1] == 0)


def test_oracle_empty_scene():
    sc = scenes.config1()
    sc["particles"] = {k: v[:0] for k, v in sc["particles"].items()}
    orc = O.Oracle(sc)
    assert orc.step(3) == 0


def test_nonlocal_round_off_sensitivity():
    """The reference's g_nonlocal_mu2 sets dense from the sign of the trial
    pressure (g_nonlocal_mu2.c:296-301); at the free surface under the first
    gravity increments p ~ 0, so a 1e-15 relative change of the positions
    switches dense flags and changes the stress at 1e-4 within 20 steps.  A
    pre-stressed fill has no p ~ 0 particles and stays at round-off."""
    def spread(scene):
        a = O.Oracle(scene)
        sc2 = dict(scene)
        sc2["particles"] = {k: v.copy() for k, v in scene["particles"].items()}
        sc2["particles"]["x"] = sc2["particles"]["x"] * (1 + 1e-15)
        b = O.Oracle(sc2)
        a.step(19)
        b.step(19)
        return rel_err(b.get("sxx"), a.get("sxx")), int(np.sum(a.get("state0") != b.get("state0")))
    free, _ = load_golden("nonlocal_mu2_silo")
    pre, _ = load_golden("nonlocal_mu2_prestressed")
    e_free, flips = spread(free)
    e_pre, flips_pre = spread(pre)
    assert e_free > 1e-6 and flips > 0
    assert e_pre < 1e-12 and flips_pre == 0


@needs_ref
def test_nonlocal_plugins_that_share_code():
    """g_nonlocal_bicgstab.c is g_nonlocal_avg.c and g_nonlocalxs71.c is
    g_nonlocal.c (the live reference plugins give bit-identical runs), which
    is why the libmpm layer maps them onto MPMG_G_NONLOCAL_AVG and
    MPMG_G_NONLOCAL; the averaged variant does differ from g_nonlocal."""
    scene, _ = load_golden("nonlocal_silo")
    runs = {}
    for mat in ("g_nonlocal", "g_nonlocalxs71", "g_nonlocal_avg", "g_nonlocal_bicgstab"):
        ref = O.RefHarness(dict(scene, material=mat), nthreads=1)
        ref.step(10)
        runs[mat] = ref.particles()
    for a, b in (("g_nonlocal", "g_nonlocalxs71"), ("g_nonlocal_avg", "g_nonlocal_bicgstab")):
        for f in ("x", "y", "sxx", "state3"):
            np.testing.assert_array_equal(runs[a][f], runs[b][f])
    assert not np.array_equal(runs["g_nonlocal"]["state3"], runs["g_nonlocal_avg"]["state3"])



def test_oracle_matches_reference_over_1000_steps():
    """Configuration 1 over the 1000 steps of its benchmark configuration:
    the oracle equals the reference's own threaded run bit for bit
    (tests/golden/long_config1.npz)."""
    d = np.load(os.path.join(GOLDEN, "long_config1.npz"))
    sc = scenes.config1(seed=0)
    orc = O.Oracle(sc, nthreads=4)
    done = 0
    for c in (int(c) for c in d["checkpoints"]):
        orc.step(c - done)
        done = c
        for f in ("x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy", "node_m", "node_mx", "node_my"):
            np.testing.assert_array_equal(orc.get(f), d["s%d_%s" % (c, f)], err_msg="%d %s" % (c, f))
        e, a = orc.get_map()
        np.testing.assert_array_equal(e, d["s%d_in_element" % c])
        np.testing.assert_array_equal(a, d["s%d_active" % c])
        assert orc.t == float(d["s%d_t" % c])
