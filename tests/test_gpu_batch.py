"""Batched ensembles (mpmg_batch_create): several independent mixed-precision
simulations of uneven sizes, grids, material parameters, boundaries and time
steps advanced by one set of kernel launches per step.

Each member of a batch must reproduce, bit for bit, the same simulation run on
its own: the batch concatenates the members' particles, elements and nodes,
and every per-particle, per-element and per-node operation and its order are
those of the single run (the members' storage orders differ only by a
constant offset).  A single simulation sums P2G and grid update in one
tiled kernel (mx_p2g_grid_kernel) while a batch runs them as two kernels, so
the equality also checks the fused kernel against the unfused pair.
"""
import numpy as np
import pytest

import mpm2d
import scenes

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "m", "v", "sxx", "sxy", "syy", "ux", "uy", "Tzz", "state9", "state10")


def small_ensemble(count=5, seed=7):
    ens = scenes.ensemble(count=count, seed=seed, cells_range=(24, 72), particles_range=(1500, 9000))
    # uneven time steps and one member with a constant body force
    for k, sc in enumerate(ens):
        sc["dt"] = [5e-6, 1e-5, 4e-6, 8e-6, 6e-6][k % 5]
    ens[1]["gravity"] = -9.81
    return ens


@pytest.mark.parametrize("precision", ["mixed", "mixed_f64node"])
def test_batch_members_equal_single_runs(precision):
    ens = small_ensemble()
    batch = mpm2d.Batch(ens, precision=precision)
    batch.step(60)
    for k, sc in enumerate(ens):
        one = mpm2d.Simulation(sc, precision=precision)
        one.step(60)
        for f in FIELDS:
            np.testing.assert_array_equal(batch.member_get(k, f), one.get(f), err_msg="member %d %s" % (k, f))
        for f in ("node_m", "node_vx", "node_vy", "node_ax", "node_ay"):
            np.testing.assert_array_equal(batch.member_get(k, f), one.get(f), err_msg="member %d %s" % (k, f))
        e1, a1 = one.get_map()
        eb, ab = batch.member_map(k)
        np.testing.assert_array_equal(eb, e1)
        np.testing.assert_array_equal(ab, a1)
        t, s = batch.member_time(k)
        assert s == 60
        assert t == one.t
        one.close()


def test_batch_silo_discharges_and_frame_read():
    ens = small_ensemble(count=4, seed=3)
    batch = mpm2d.Batch(ens)
    m = np.concatenate([sc["particles"]["m"] for sc in ens])
    batch.step(200)
    frame = batch.get_frame(("x", "y", "vx", "vy", "sxx", "node_m"))
    for nm, a in frame.items():
        np.testing.assert_array_equal(a, batch.get(nm))
    # mass is conserved in every member: nodal mass equals the active particles' mass
    e, a = batch.get_map()
    nm = batch.get("node_m")
    for k in range(batch.count):
        sl, nsl = batch.members[k]["particles"], batch.members[k]["nodes"]
        mp = m[sl][a[sl] == 1].sum()
        assert abs(nm[nsl].sum() - mp) <= 1e-5 * mp
        assert np.all(e[sl][a[sl] == 1] < batch.members[k]["elements"].stop - batch.members[k]["elements"].start)


def test_batch_deterministic():
    ens = small_ensemble(count=3, seed=11)
    runs = []
    for _ in range(2):
        b = mpm2d.Batch(ens)
        b.step(40)
        runs.append([b.get(f) for f in ("x", "y", "sxx")])
        b.close()
    for u, v in zip(*runs):
        np.testing.assert_array_equal(u, v)


def test_autotune_keeps_the_trajectory():
    """mpmg_autotune times tiles and launch shapes on the simulation itself;
    no knob changes a result, so a tuned batch (whose trajectory ran through
    every candidate tile and shape) continues bit for bit like an untuned one
    advanced by the same steps."""
    ens = small_ensemble(count=3, seed=9)
    tuned = mpm2d.Batch(ens, precision="mixed")
    plain = mpm2d.Batch(ens, precision="mixed")
    t = tuned.autotune(steps_per_trial=8)
    assert t["candidates"] >= 3 * 2 + 3 and t["graph_steps"] in (4, 8, 16) and t["g2p_blocks_per_sm"] >= 1
    assert t["g2p_tile"] in (128, 256) and (t["p2g_elements"], t["p2g_stage"]) in ((256, 1024), (128, 512),
                                                                                  (512, 1024))
    assert t["ms_per_step"] > 0 and t["ms_per_step"] <= t["default_ms_per_step"]
    plain.step(t["steps_advanced"])
    tuned.step(37)
    plain.step(37)
    for k in range(3):
        for f in FIELDS:
            np.testing.assert_array_equal(tuned.member_get(k, f), plain.member_get(k, f), err_msg="%d %s" % (k, f))


def test_batch_dp_ri_mt_members_equal_single_runs():
    """Batches of the rate-independent Drucker-Prager law (szz in the record's
    Tzz slot, mu_s per member) equal their members run alone."""
    ens = small_ensemble(count=3, seed=4)
    for k, sc in enumerate(ens):
        sc["material"] = "dp_ri_mt"
        sc["props"] = [1e6, 0.3, 0.30 + 0.05 * k]
        sc.pop("mp", None)
    batch = mpm2d.Batch(ens, precision="mixed")
    batch.step(40)
    for k, sc in enumerate(ens):
        one = mpm2d.Simulation(sc, precision="mixed")
        one.step(40)
        for f in ("x", "y", "vx", "vy", "sxx", "sxy", "syy", "state1", "state9", "state10"):
            np.testing.assert_array_equal(batch.member_get(k, f), one.get(f), err_msg="member %d %s" % (k, f))
        one.close()


def crowded_scene():
    """The config-1 block plus two crowded elements.  Element (14, 14) holds
    1500 particles, more than the fused kernel's 1024-particle stage, and lies
    in four 16 x 16 element tiles (column and row 14 are each shared by two
    tiles): its owner orders it into perm, the three others into their own
    scratch orders.  Element (20, 3) gets 300 more particles inside the
    block, so its tile is summed in several stage passes."""
    sc = scenes.config1(gravity=-9.81)
    h = sc["h"]
    p = sc["particles"]
    rng = np.random.default_rng(11)
    add = {k: [v] for k, v in p.items()}
    for ei, ej, cnt in ((14, 14, 1500), (20, 3, 300)):
        x = (ei + rng.uniform(0.05, 0.95, cnt)) * h
        y = (ej + rng.uniform(0.05, 0.95, cnt)) * h
        extra = {"m": np.full(cnt, p["m"][0]), "v": np.full(cnt, p["v"][0]), "x": x, "y": y}
        for k in add:
            add[k].append(extra.get(k, np.zeros(cnt)))
    sc["particles"] = {k: np.concatenate(v) for k, v in add.items()}
    return sc


def test_crowded_elements_fused_equals_unfused():
    sc = crowded_scene()
    other = scenes.config1(seed=3)
    batch = mpm2d.Batch([sc, other], precision="mixed")
    batch.step(20)
    one = mpm2d.Simulation(sc, precision="mixed")
    one.step(20)
    for f in ("x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy"):
        np.testing.assert_array_equal(batch.member_get(0, f), one.get(f), err_msg=f)
    for f in ("node_m", "node_vx", "node_vy", "node_ax", "node_ay"):
        np.testing.assert_array_equal(batch.member_get(0, f), one.get(f), err_msg=f)
    # and the crowded run against the FP64 form (a wrong or missing particle
    # in a sum would show as an O(1) error)
    ref = mpm2d.Simulation(sc, precision="fp64")
    ref.step(20)
    for fs in (("x", "y"), ("vx", "vy")):
        a = np.concatenate([one.get(f) for f in fs])
        b = np.concatenate([ref.get(f) for f in fs])
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), fs
    ref.close()
    one.close()



def test_benchmark_ensemble_sampled_members_vs_oracle():
    """The 256-member benchmark ensemble (silo and heap runs, grids 64^2 to
    384^2 elements, 5k-200k particles, outlet 0.02-0.12 m, mu_s 0.30-0.45)
    stepped as one batch in the mixed form: eight members drawn with a fixed
    seed against the oracle (the FP64 CPU restatement) run on each member
    alone, relative L2 error per field <= 1e-4 after 200 steps (a field of
    a physical group scaled by the group's largest norm)."""
    import os
    from oracle import oracle as O
    ens = scenes.ensemble(count=256, seed=1)
    batch = mpm2d.Batch(ens)
    steps = 200
    batch.step(steps)
    groups = {"x": ("x", "y"), "y": ("x", "y"), "vx": ("vx", "vy"), "vy": ("vx", "vy"),
              "sxx": ("sxx", "sxy", "syy"), "sxy": ("sxx", "sxy", "syy"), "syy": ("sxx", "sxy", "syy"),
              "v": ("v",)}
    rng = np.random.default_rng(11)
    worst = 0.0
    for k in sorted(rng.choice(len(ens), size=8, replace=False)):
        orc = O.Oracle(ens[k], nthreads=os.cpu_count() or 1)
        orc.step(steps)
        want = {f: orc.get(f) for f in groups}
        for f, grp in groups.items():
            scale = max(np.linalg.norm(want[g]) for g in grp)
            err = np.linalg.norm(batch.member_get(int(k), f) - want[f]) / scale
            worst = max(worst, err)
            assert err <= 1e-4, (int(k), f, err)
        eb, ab = batch.member_map(int(k))
        oe, oa = orc.get_map()
        # particles that left through an outlet, or crossed an element edge,
        # within FP32 round-off of the FP64 run: at most a few
        assert np.count_nonzero(ab != oa) <= max(2, len(oa) // 10000), int(k)
    print("ensemble members vs oracle: largest relative L2 error %.3e" % worst)
    batch.close()
