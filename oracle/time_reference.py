"""Times the reference's own pthreaded CPU step against the oracle port
(test infrastructure: the qualification of the CPU baseline, not the product).

The reference's libmpm, its g_local_mu2 (or isolin) plugin and box plugin are
compiled with the reference's release flags (CMakeLists.txt:4, -O3
-march=native) into oracle/_ref/perf/ and driven by oracle/ref/ref_harness.c,
the driver set-up of src/main.c:747-835: its pthread team runs
explicit_mpm_step_usl_threaded (libmpm/process_usl.c:465-592) and the serial
tail time_varying_loads.  The oracle port (oracle/mpm_oracle.c) runs the same
workload with the same thread count.  Each leg runs in a process of its own.

It needs the reference tree, so it runs only where that tree is (the GPU
host has none; there bench.py times the port and quotes the ratio this
recipe measured).  Usage:

    python -m oracle.time_reference [--cells 512] [--steps 20] [--threads 1,8]

prints one JSON object: particle-steps/s of both legs per thread count and
port_over_reference = port / reference.
"""
import argparse
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _scene(cells, material):
    sys.path.insert(0, os.path.join(ROOT, "mpm-2d_gb300"))
    import scenes
    return scenes.box_fill(cells=cells, ppc_1d=2, material=material, rho=2450.0, props=(1e6, 0.3), dt=2e-6)


def _leg(kind, cells, material, steps, threads, warmup):
    sys.path.insert(0, ROOT)
    from oracle import build as B
    from oracle import oracle as O
    sc = _scene(cells, material)
    n = len(sc["particles"]["x"])
    if kind == "reference":
        sim = O.RefHarness(sc, nthreads=threads, lib_dir=B.PERF_OUT)
    else:
        sim = O.Oracle(sc, nthreads=threads)
    sim.step(warmup)
    t0 = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t0
    return {"particle_steps_per_s": n * steps / dt, "seconds": dt, "steps": steps, "particles": n}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=512)
    ap.add_argument("--material", default="g_local_mu2")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--threads", default="1,%d" % (os.cpu_count() or 1))
    ap.add_argument("--leg", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--t", type=int, default=1, help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.leg:
        print(json.dumps(_leg(a.leg, a.cells, a.material, a.steps, a.t, a.warmup)))
        return 0
    sys.path.insert(0, ROOT)
    from oracle import build as B
    if B.build_ref_perf(materials=(a.material,)) is None:
        print(json.dumps({"unavailable": "reference tree absent"}))
        return 0
    B.build_oracle()
    out = {"workload": "box_fill %d^2 elements, 2x2 per element, %s, box" % (a.cells, a.material),
           "reference_flags": " ".join(B.PERF_CFLAGS), "host_cores": os.cpu_count(), "legs": {}}
    for t in [int(s) for s in a.threads.split(",")]:
        legs = {}
        for kind in ("reference", "port"):
            r = subprocess.run([sys.executable, "-m", "oracle.time_reference", "--leg", kind, "--t", str(t),
                                "--cells", str(a.cells), "--material", a.material, "--steps", str(a.steps),
                                "--warmup", str(a.warmup)], cwd=ROOT, capture_output=True, text=True, check=True)
            legs[kind] = json.loads(r.stdout.strip().splitlines()[-1])
        legs["port_over_reference"] = (legs["port"]["particle_steps_per_s"]
                                       / legs["reference"]["particle_steps_per_s"])
        out["legs"]["threads_%d" % t] = legs
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
