"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run here, where the reference tree exists:  python tests/golden/gen_golden.py
It builds oracle/_ref/ (the reference's libmpm, plugins and test_material
compiled from its sources, see oracle/build.py) and records:

  kat_<material>.npz     tests/test_material.c's 1252-row %a histories for
                         isolin and g_local_mu2 (columns t, L11, L12, L21, L22,
                         sxx, sxy, syy, mu, gammadotp), parsed exactly
  step_<case>.npz        particle and node state of the reference's threaded
                         step (explicit_mpm_step_usl_threaded + the driver's
                         time_varying_loads) at a few step counts, with the
                         inputs that produced them
  lists_config1.npz      find_filled_elements' per-element particle order
                         after 100 steps of config 1 (one thread, so one list
                         per colour)
  step_musl_<case>.npz   the same for explicit_mpm_step_musl_threaded
                         (python tests/golden/gen_golden.py musl records only
                         these)
  long_config1.npz       config 1 run to the 1000 steps of its benchmark
                         configuration: particle state, element map and nodal
                         mass and momentum at steps 500 and 1000
                         (python tests/golden/gen_golden.py long)
  writer_<case>.npz      the reference's own src/writer.c output for a
                         recorded state: write_frame, write_element_frame and
                         write_state text (python tests/golden/gen_golden.py
                         writer)

The nonlocal cases run the reference with one thread: with more, its
g_nonlocal_mu2 solve reads particles other threads are still updating
(libmpm/process_usl.c:576-589 has no barrier before the material call), and
the results change from run to run.  The g_nonlocal plugin has no
calculate_stress_threaded; the harness calls its calculate_stress from task 0.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mpm-2d_gb300"))

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402
import scenes  # noqa: E402

PARTICLE_KEYS = ["x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy", "exx", "exy", "eyy",
                 "wxy", "ax", "ay", "Tzz"] + ["state%d" % k for k in range(11)]
NODE_KEYS = ["node_m", "node_mx", "node_my", "node_fx", "node_fy", "node_vx", "node_vy"]


def scene_arrays(sc):
    out = {"in_" + k: np.asarray(v, dtype=np.float64) for k, v in sc["particles"].items()}
    meta = {k: sc[k] for k in ("Nx", "Ny", "h", "dt") if k in sc}
    out["meta_grid"] = np.array([meta["Nx"], meta["Ny"]], dtype=np.int64)
    out["meta_h_dt"] = np.array([meta["h"], meta["dt"]])
    out["meta_props"] = np.asarray(sc.get("props", [1e6, 0.3]), dtype=np.float64)
    out["meta_bcf"] = np.asarray(sc.get("bcf", []), dtype=np.float64)
    out["meta_bci"] = np.asarray(sc.get("bci", []), dtype=np.int64)
    out["meta_material"] = np.array(sc["material"])
    out["meta_bc"] = np.array(sc["bc"])
    out["meta_scheme"] = np.array(sc.get("scheme", "usl"))
    return out


def record_steps(name, sc, checkpoints, nthreads):
    ref = O.RefHarness(sc, nthreads=nthreads)
    data = scene_arrays(sc)
    data["checkpoints"] = np.asarray(checkpoints, dtype=np.int64)
    done = 0
    for c in checkpoints:
        ref.step(c - done)
        done = c
        p = ref.particles()
        n = ref.nodes()
        for k in PARTICLE_KEYS:
            key = {"Tzz": "Tzz"}.get(k, k)
            data["s%d_%s" % (c, k)] = p[key]
        data["s%d_in_element" % c] = p["in_element"]
        data["s%d_active" % c] = p["active"]
        data["s%d_t" % c] = np.array(ref.t)
        for k in NODE_KEYS:
            data["s%d_%s" % (c, k)] = n[k]
    path = os.path.join(HERE, "step_%s.npz" % name)
    np.savez_compressed(path, **data)
    return ref, path


def parse_hex_csv(path):
    rows = []
    with open(path) as f:
        for line in f:
            rows.append([float.fromhex(v) for v in line.strip().split(",")])
    return np.array(rows)


def kat(material, props=(1e6, 0.3)):
    """The reference's tests/test_material.c run with the properties of
    tests/<material>.cfg (isolin, g_local_mu2: E, nu; dp_ri_mt: E, nu, mu_s)."""
    exe = os.path.join(obuild.REF_OUT, "material_" + material)
    with tempfile.TemporaryDirectory() as d:
        hexf = os.path.join(d, "out.csv")
        decf = os.path.join(d, "out_dec.csv")
        cfg = os.path.join(d, "test.cfg")
        with open(cfg, "w") as f:
            f.write("%s\n%s\n" % (hexf, decf) + "".join("%r\n" % p for p in props))
        subprocess.run([exe, cfg], check=True, capture_output=True, cwd=d)
        rows = parse_hex_csv(hexf)
    path = os.path.join(HERE, "kat_%s.npz" % material)
    np.savez_compressed(path, rows=rows, props=np.array(props, dtype=np.float64), dt=np.array(1e-3))
    return path


def dp_cases():
    # dp_ri_mt (materialsrc/dp_ri_mt.c): known answers and two trajectories
    print(kat("dp_ri_mt", props=(1e6, 0.3, 0.3819)))
    sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="dp_ri_mt",
                       rho=2450.0, props=(1e6, 0.3, 0.3819), dt=1e-5, jitter=5e-4, seed=1)
    print(record_steps("dp_column", sc, [1, 50, 300], nthreads=4)[1])
    sc = scenes.silo(cells=32, material="dp_ri_mt", props=(1e6, 0.3, 0.3819), dt=1e-5, hole_radius=0.1,
                     open_time=0.001, wall_frac=0.5, fill_height=0.6)
    print(record_steps("dp_silo", sc, [1, 50, 400], nthreads=4)[1])
    sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="dp_ri_mt",
                       rho=2450.0, props=(1e6, 0.3, 0.3819), dt=1e-5, jitter=5e-4, seed=1)
    sc["scheme"] = "musl"
    print(record_steps("musl_dp_column", sc, [1, 50, 300], nthreads=4)[1])


def plane_cases():
    # g_local_mu2_plane_strain and g_local_mu2_true_2d (E, nu from the
    # configuration; the mu(I) constants are compile-time in the plugins)
    for mat, tag in (("g_local_mu2_plane_strain", "ps"), ("g_local_mu2_true_2d", "t2d")):
        print(kat(mat))
        sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material=mat,
                           rho=2450.0, props=(1e6, 0.3), dt=1e-5, jitter=5e-4, seed=1)
        print(record_steps("%s_column" % tag, sc, [1, 50, 300], nthreads=4)[1])
        sc = scenes.silo(cells=32, material=mat, props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                         open_time=0.001, wall_frac=0.5, fill_height=0.6)
        print(record_steps("%s_silo" % tag, sc, [1, 50, 400], nthreads=4)[1])


def reverse_cases():
    # g_local_mu2_reverse: known answers, a column and a silo
    print(kat("g_local_mu2_reverse"))
    sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="g_local_mu2_reverse",
                       rho=2450.0, props=(1e6, 0.3), dt=1e-5, jitter=5e-4, seed=1)
    print(record_steps("rev_column", sc, [1, 50, 300], nthreads=4)[1])
    sc = scenes.silo(cells=32, material="g_local_mu2_reverse", props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                     open_time=0.001, wall_frac=0.5, fill_height=0.6)
    print(record_steps("rev_silo", sc, [1, 50, 400], nthreads=4)[1])


def nonlocal_avg_cases():
    # g_nonlocal_avg (the element average of the nodal fluidity at the
    # particles), the sheared silo of nonlocal_silo
    sc = scenes.silo(cells=16, material="g_nonlocal_avg", props=(1e8, 0.3), dt=1e-6, hole_radius=0.1,
                     open_time=0.0, wall_frac=0.5, fill_height=0.6)
    n = len(sc["particles"]["x"])
    sc["particles"]["sxx"] = np.full(n, -1000.0)
    sc["particles"]["syy"] = np.full(n, -2000.0)
    sc["particles"]["sxy"] = np.full(n, 600.0)
    print(record_steps("nonlocal_avg_silo", sc, [1, 10, 60], nthreads=1)[1])


def ext_cases():
    # g_local_mu2_ext: the nodal Laplacian of the local fluidity (threaded,
    # with the team's element lists and barriers)
    sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="g_local_mu2_ext",
                       rho=2450.0, props=(1e6, 0.3), dt=1e-5, jitter=5e-4, seed=1)
    print(record_steps("ext_column", sc, [1, 50, 300], nthreads=4)[1])
    sc = scenes.silo(cells=32, material="g_local_mu2_ext", props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                     open_time=0.001, wall_frac=0.5, fill_height=0.6)
    print(record_steps("ext_silo", sc, [1, 50, 400], nthreads=4)[1])


def musl_cases():
    # explicit_mpm_step_musl_threaded (process_usl.c:284-462), threaded
    sc = scenes.config1(seed=0)
    sc["scheme"] = "musl"
    print(record_steps("musl_config1", sc, [1, 2, 100], nthreads=4)[1])
    sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="g_local_mu2",
                       rho=2450.0, props=(1e6, 0.3), dt=1e-5, jitter=5e-4, seed=1)
    sc["scheme"] = "musl"
    print(record_steps("musl_mu2_column", sc, [1, 50, 300], nthreads=4)[1])


LONG_PARTICLE_KEYS = ["x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy"]
LONG_NODE_KEYS = ["node_m", "node_mx", "node_my"]


def long_cases():
    # config 1 over its full 1000 steps (threaded)
    sc = scenes.config1(seed=0)
    ref = O.RefHarness(sc, nthreads=4)
    data = scene_arrays(sc)
    checkpoints = [500, 1000]
    data["checkpoints"] = np.asarray(checkpoints, dtype=np.int64)
    done = 0
    for c in checkpoints:
        ref.step(c - done)
        done = c
        p = ref.particles()
        n = ref.nodes()
        for k in LONG_PARTICLE_KEYS:
            data["s%d_%s" % (c, k)] = p[k]
        data["s%d_in_element" % c] = p["in_element"]
        data["s%d_active" % c] = p["active"]
        data["s%d_t" % c] = np.array(ref.t)
        for k in LONG_NODE_KEYS:
            data["s%d_%s" % (c, k)] = n[k]
    path = os.path.join(HERE, "long_config1.npz")
    np.savez_compressed(path, **data)
    print(path)


def writer_cases():
    # the reference's writer on recorded states: config 1 after 100 steps
    # (isolin) and the g_local_mu2 column after 300 (nonzero plastic state)
    cases = [("config1", scenes.config1(seed=0), 100, 4),
             ("mu2_column", scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="g_local_mu2",
                                          rho=2450.0, props=(1e6, 0.3), dt=1e-5, jitter=5e-4, seed=1), 300, 4)]
    for name, sc, steps, threads in cases:
        ref = O.RefHarness(sc, nthreads=threads)
        ref.step(steps)
        out = {"step": np.array(steps), "t": np.array(ref.t), "frame_number": np.array(3)}
        with tempfile.TemporaryDirectory() as d:
            for what in ("frame", "element_frame", "state"):
                path = os.path.join(d, what + ".txt")
                ref.write(path, what, frame=3, time=ref.t)
                with open(path, "rb") as f:
                    out[what] = np.frombuffer(f.read(), dtype=np.uint8)
        path = os.path.join(HERE, "writer_%s.npz" % name)
        np.savez_compressed(path, **out)
        print(path)


def main():
    if obuild.build_ref(verbose=False) is None:
        raise SystemExit("reference tree not found; fixtures can only be generated where it exists")
    if sys.argv[1:] == ["musl"]:
        musl_cases()
        return
    if sys.argv[1:] == ["dp"]:
        dp_cases()
        return
    if sys.argv[1:] == ["plane"]:
        plane_cases()
        return
    if sys.argv[1:] == ["ext"]:
        ext_cases()
        return
    if sys.argv[1:] == ["nlavg"]:
        nonlocal_avg_cases()
        return
    if sys.argv[1:] == ["reverse"]:
        reverse_cases()
        return
    if sys.argv[1:] == ["long"]:
        long_cases()
        return
    if sys.argv[1:] == ["writer"]:
        writer_cases()
        return
    print(kat("isolin"))
    print(kat("g_local_mu2"))

    # config 1: isolin block in a box (4096 particles, 65^2 nodes), threaded
    sc = scenes.config1(seed=0)
    ref, path = record_steps("config1", sc, [1, 2, 100], nthreads=4)
    print(path)
    # element lists built in step 101 from the positions after step 100
    ref1 = O.RefHarness(sc, nthreads=1)
    ref1.step(100)
    before = ref1.particles()
    ref1.step(1)
    lists, lens = ref1.color_lists()
    p = ref1.particles()
    np.savez_compressed(os.path.join(HERE, "lists_config1.npz"), lists=lists.astype(np.int64),
                        lengths=lens.astype(np.int64), in_element=p["in_element"], active=p["active"],
                        x=before["x"], y=before["y"])

    # g_local_mu2 column collapse on the unit square (2048 particles)
    sc = scenes.column(Nx=65, Ny=65, h=1 / 64, width=0.25, height=0.5, material="g_local_mu2",
                       rho=2450.0, props=(1e6, 0.3), dt=1e-5, jitter=5e-4, seed=1)
    print(record_steps("mu2_column", sc, [1, 50, 300], nthreads=4)[1])

    # g_local_mu2 in the square silo with the trapdoor opening at t = 1 ms
    sc = scenes.silo(cells=32, material="g_local_mu2", props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                     open_time=0.001, wall_frac=0.5, fill_height=0.6)
    print(record_steps("mu2_silo", sc, [1, 50, 400], nthreads=4)[1])

    # g_nonlocal_mu2 silo (one thread, see the module docstring)
    sc = scenes.silo(cells=32, material="g_nonlocal_mu2", props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                     open_time=0.001, wall_frac=0.5, fill_height=0.6)
    print(record_steps("nonlocal_mu2_silo", sc, [1, 20, 120], nthreads=1)[1])

    # the same silo pre-stressed (lithostatic syy, sxx = syy / 2, plus 500 Pa)
    # so that no particle sits at p = 0, where the dense flag switches: from
    # the unstressed fill a 1e-15 relative perturbation of x changes ~200
    # dense flags within 20 steps, which makes whole trajectories
    # incomparable at round-off level.
    sc = scenes.silo(cells=32, material="g_nonlocal_mu2", props=(1e6, 0.3), dt=1e-5, hole_radius=0.1,
                     open_time=0.001, wall_frac=0.5, fill_height=0.6)
    y = sc["particles"]["y"]
    sc["particles"]["syy"] = -2450 * 9.8 * (0.6 - y) - 500.0
    sc["particles"]["sxx"] = 0.5 * sc["particles"]["syy"]
    print(record_steps("nonlocal_mu2_prestressed", sc, [1, 20, 120], nthreads=1)[1])

    # g_nonlocal (operator variant) with a sheared initial stress so that
    # its bulk fluidity is nonzero from the first step
    sc = scenes.silo(cells=16, material="g_nonlocal", props=(1e8, 0.3), dt=1e-6, hole_radius=0.1,
                     open_time=0.0, wall_frac=0.5, fill_height=0.6)
    n = len(sc["particles"]["x"])
    sc["particles"]["sxx"] = np.full(n, -1000.0)
    sc["particles"]["syy"] = np.full(n, -2000.0)
    sc["particles"]["sxy"] = np.full(n, 600.0)
    print(record_steps("nonlocal_silo", sc, [1, 10, 60], nthreads=1)[1])
    musl_cases()
    dp_cases()
    plane_cases()
    ext_cases()
    nonlocal_avg_cases()
    reverse_cases()
    long_cases()
    writer_cases()


if __name__ == "__main__":
    main()
