"""Benchmark of the mpm-2d explicit USL step on GB300 (one JSON line).

Workload (N=1): 1 048 576 particles filling the unit square at 2x2 per
element on a 513x513-node grid (512^2 elements), g_local_mu2 granular rheology
(rho 2450, E 1e6, nu 0.3, reference constants), box walls, synthetic seeded
inputs in the reference generator's lattice layout.  A step is one
explicit_mpm_step_usl_threaded + time_varying_loads over all particles.  The
headline runs the plain FP64 form, the reference's own arithmetic, so that it
compares like for like with the reference's FP64 CPU step; the mixed forms
(FP32 particle state and arithmetic with FP64 nodal sums, "mixed_f64node",
the chosen form, and with float-float nodal sums, "mixed") are measured
beside it.  Particle state and per-step scratch exceed the 129 MB L2 (~300 MB
FP64, ~170 MB mixed), so no flush is needed between steps.

  value     particle-steps/s of the FP64 form with the state resident in HBM
            (CUDA events on the library's stream over CUDA-graph steps, max
            over ranks)
  e2e       the same metric through the public C ABI with host buffers over
            a 500-step run: the timed region includes creating the context
            from host arrays (H2D of the particle state), a D2H read of each
            step's result (time, step count, status) after every step, and
            one output frame of the driver's particle fields at the end
  roofline  the dominant kernel (the FP64 G2P + material update): its
            algorithmic bytes per launch over its CUDA-event duration against
            the measured HBM copy peak, and, since it is bound by the FP64
            pipe, its FP64 operations per launch against the measured FP64
            FMA rate
  cpu_baseline  the oracle (the CPU restatement of the reference's pthreaded
            step) on this host's cores over a bounded sample of steps, at all
            cores and at one; the compiled reference is slower than the port
            by the factor oracle/time_reference.py measured

--impl reference times the reference's CPU step (the oracle port on hosts
without the reference build) on all host cores, same metric and config.
Multi-GPU: independent replicas (the step has no cross-rank exchange).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# the particle fields of the driver's output frame (write_frame, src/writer.c)
FRAME_FIELDS = ("m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy", "ux", "uy", "state9", "state10")
PKG = os.path.join(ROOT, "mpm-2d_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-steps/s at 1M pts, mixed vs FP64 GPU; %HBM peak; adjoint/forward time"
UNIT = "particle-steps/s"
WORKLOAD = "box_fill_1M_g_local_mu2"

# Algorithmic bytes per unit of work of each phase (each array read or written
# once per use; node gathers counted once per node), as (per particle, per
# element, per node).
#
# FP64 form, g_local_mu2: keys read x y active (20 B) and write element,
# active, key (12 B) per particle; the sort's scatter reads the key and writes
# slot + sorted key, the P2G's ordering reads the slot and writes perm (20 B
# per particle; bins read, cursor and offsets written, 16 B per element); the
# P2G reads perm and 9 particle doubles and writes 4 corners x 5 sums; the
# grid update reads them back and writes 5 doubles per node; the G2P reads
# element + 13 doubles and writes 13 doubles per particle and gathers 4
# doubles per node.
FP64_BYTES = {
    "keys": (32, 0, 0),
    "sort": (20, 16, 0),
    "p2g": (4 + 9 * 8, 160, 0),
    "grid": (0, 160, 40),
    "g2p": (13 * 8 + 8 + 13 * 8, 0, 32),
}
# The compulsory bytes of the FP64 step (each persistent field read
# and written once, sort scratch and transients excluded): 216 B per
# particle-step for g_local_mu2 and 80 B per node-step.
FP64_STEP_SURVEY_BYTES = (216, 0, 80)

# Mixed form, g_local_mu2 (the builder's accounting of what the kernels move):
#   sort  count fused into the previous G2P; scatter reads the key (4 B) and
#         writes slot + sorted key (8 B); the P2G's ordering reads the slot and
#         writes perm (8 B): 20 B per particle; scan: bins read + cursor,
#         cell_start written, bins zeroed (16 B per element)
#   p2g   P2G and grid update in one kernel (the corner sums stay in shared
#         memory): perm 4 + xl yl m vx vy v sxx sxy syy 36 = 40 B per
#         particle; nodal mass + float4 node = 24 B (float-float) or 32 B
#         (FP64 nodal sums) per node
#   g2p   perm 4 + sorted key 4 + 13 floats 52 + pid 4 read, 14 floats 56 +
#         element 4 + pid 4 written = 128 B per particle; float4 node 16 B per
#         node read
MIXED_BYTES = {
    "sort": (20, 16, 0),
    "p2g": (40, 0, 24),
    "g2p": (128, 0, 16),
}
# The compulsory bytes of the mixed step, which exclude perm, key and
# particle index (index and sort scratch): 112 B per particle-step for
# g_local_mu2, 64 B per node-step; of those the G2P moves the particle state
# (13 floats read, 13 written = 104 B) and the node gathers (16 B per node).
MIXED_STEP_SURVEY_BYTES = (112, 0, 64)
# A batch runs P2G and grid update as two kernels, so the element corner sums
# (5 floats x 4 corners) are written and read back: 80 B per element each.
BATCH_BYTES = {
    "sort": (20, 16, 0),
    "p2g": (40, 80, 0),
    "grid": (0, 80, 24),
    "g2p": (128, 0, 16),
}
MIXED_G2P_SURVEY_BYTES = (104, 0, 16)

# FP64 work per particle of the FP64 G2P + g_local_mu2 after the warm-up
# steps, from one ncu capture of g2p_kernel<1,0> (the same fill at 256^2
# elements, 262 144 particles, step 27; per-particle counts do not depend on
# the size): operations (DADD + DMUL + 2 DFMA: 48.4 + 48.4 + 2 x 54.6) and
# FP64 pipe instructions (pipe-active cycles x 2 per SM, compares and
# conversions included).
G2P64_FLOPS_PER_PARTICLE = 206.0
G2P64_PIPE_INSTR_PER_PARTICLE = 210.8

# DRAM bytes (read + write) of one mx_g2p_kernel launch on this workload from
# one ncu capture: 80.8 MB read + 17.0 MB written; writes still in L2 at the
# kernel's end are not in the figure.
G2P_TRAFFIC_BYTES = 97.8e6
# dram__bytes_read.sum + dram__bytes_write.sum of one g2p_kernel<1,0> launch
# on the 1 048 576-particle workload (126.1 + 49.1 MB, the FP64 step's ncu
# capture)
G2P64_TRAFFIC_BYTES = 175.2e6

# The compiled reference against the oracle port on this workload, same host
# and thread count (oracle/time_reference.py, 8-core x86-64 development host,
# the reference built with its release flags -O3 -march=native): the port
# runs 2.19x the reference's particle-steps/s on 1 thread and 1.64x on 8.  The
# CPU figures below time the port, so they overstate the reference's speed.
PORT_OVER_REFERENCE = {"threads_1": 2.19, "threads_8": 1.64,
                       "how": "oracle/time_reference.py on an 8-core x86-64 host (the GPU host has no "
                              "reference tree to build): reference with -O3 -march=native vs the port, "
                              "10 steps of this workload, each leg in its own process"}


def phase_bytes(table, phase, n, ne, nn):
    a, b, c = table.get(phase, (0, 0, 0))
    return a * n + b * ne + c * nn


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_ranks(torch):
    """One process per GPU under torchrun: NCCL where there are GPUs, gloo on
    CPU hosts."""
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def barrier(torch, dev=None):
    """Device work done, then every rank here."""
    if dev is not None and torch.cuda.is_available():
        torch.cuda.synchronize(dev)
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(torch, t):
    """The largest of the ranks' values of t (a time: the job ends with its
    slowest rank)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return t
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_value(units_per_rank, world, seconds):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    return units_per_rank * world / seconds


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.tmp is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.tmp.flush()
        with open(self.tmp.name) as f:
            rows = [r.strip().split(", ") for r in f if r.strip()]
        os.unlink(self.tmp.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_scene():
    import scenes
    return scenes.box_fill(cells=512, ppc_1d=2, material="g_local_mu2", rho=2450.0,
                           props=(1e6, 0.3), dt=2e-6)


def bench_config(scene, world):
    """The workload both arms print (identical keys and values)."""
    return {"workload": WORKLOAD, "particles": len(scene["particles"]["x"]),
            "grid_nodes": [scene["Nx"], scene["Ny"]], "material": scene["material"], "bc": scene["bc"],
            "dt": scene["dt"], "gravity": "reference ramp (loading.c)",
            "arithmetic": "IEEE FP64 (the reference's)",
            "l2_policy": "state and step scratch exceed the 129 MB L2 between steps",
            "parallelism": "replicas" if world > 1 else "single"}


def cpu_baseline(scene, steps, threads, warmup=1):
    """The oracle (CPU restatement of the reference's pthreaded step) on host
    cores over `steps` steps of the full workload."""
    from oracle import oracle as O
    orc = O.Oracle(scene, nthreads=threads)
    orc.step(warmup)                            # first-touch of arrays, the gravity ramp's first steps
    t0 = time.perf_counter()
    orc.step(steps)
    dt = time.perf_counter() - t0
    n = len(scene["particles"]["x"])
    return n * steps / dt, dt


def cpu_nonlocal_baseline(scene, steps, threads):
    """The nonlocal silo on host cores through the oracle, whose fluidity solve
    here is Jacobi-preconditioned CG to the same 1e-10 (its banded direct
    solve, the stand-in for the reference's CXSparse LU, takes about 40 s a
    step on this silo and is recorded in the baseline notes instead)."""
    from oracle import oracle as O
    orc = O.Oracle(scene, nthreads=threads, solver="cg", cg_tol=1e-10)
    orc.step(1)
    t0 = time.perf_counter()
    orc.step(steps)
    dt = time.perf_counter() - t0
    st, iters, res = orc.last_solve()
    return dt / steps, iters


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    scene = make_scene()
    threads = os.cpu_count() or 1
    steps = max(1, args.steps)
    value, dt = cpu_baseline(scene, steps, threads, warmup=args.warmup)
    n = len(scene["particles"]["x"])
    # the reference's own objects are built from its sources, which only the
    # development host has; here the oracle (the CPU restatement) is timed
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(scene, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d steps of the full %d-particle workload after %d warm-up steps"
                                   % (steps, n, args.warmup),
                         "port_over_reference": PORT_OVER_REFERENCE},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def time_steps(sim, steps, stream, torch):
    """CUDA-event time of `steps` steps on the library's stream (ms)."""
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.step(steps)
    ev1.record(stream)
    sim.synchronize()
    return ev0.elapsed_time(ev1)


def phase_profile(sim, steps, table, n, ne, nn):
    """Per-phase CUDA-event times (eager launches, events around each phase)
    and the achieved algorithmic bandwidth of each phase."""
    sim.enable_phase_timing(True)
    sim.step(steps)
    ph = sim.phase_times()
    sim.enable_phase_timing(False)
    out = {}
    for k, (ms, cnt) in ph.items():
        if cnt == 0:
            continue
        avg_s = ms / cnt / 1e3
        b = phase_bytes(table, k, n, ne, nn)
        out[k] = {"ms": ms / cnt, "alg_bytes": b, "gbs": (b / avg_s / 1e9) if b else None}
    return out


ACC_FIELDS = ("x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy")
ACC_GROUPS = {"sxy": ("sxx", "syy"), "vx": ("vx", "vy"), "vy": ("vx", "vy"), "ux": ("ux", "uy"),
              "uy": ("ux", "uy")}


def accuracy_report(mpm2d, scenes, scene, dev):
    """The mixed form against the FP64 form: relative L2 error per field after
    100 steps of the benchmark workload (a field of a physical group, such as
    sxy, scaled by the group's largest norm), and the silo discharge rate and
    column runout of the mixed-form tests (3000 steps each)."""
    out = {}
    sims = {p: mpm2d.Simulation(scene, device=dev, precision=p) for p in ("mixed", "fp64")}
    for s_ in sims.values():
        s_.step(100)
    ref = {f: sims["fp64"].get(f) for f in ACC_FIELDS}
    err = {}
    for f in ACC_FIELDS:
        a, b = sims["mixed"].get(f), ref[f]
        scale = max(np.linalg.norm(ref[g]) for g in ACC_GROUPS[f]) if f in ACC_GROUPS else np.linalg.norm(b)
        err[f] = float(np.linalg.norm(a - b) / scale) if scale > 0 else float(np.linalg.norm(a - b))
    for s_ in sims.values():
        s_.close()
    out["rel_l2_after_100_steps"] = err

    def active_mass_rate(sim, m, steps, every):
        hist = []
        for _ in range(steps // every):
            sim.step(every)
            _, act = sim.get_map()
            hist.append((sim.t, float(m[act == 1].sum())))
        h = np.array(hist)
        t, mass = h[:, 0], h[:, 1]
        flowing = mass < mass[0] * (1 - 1e-9)
        t, mass = t[flowing], mass[flowing]
        return float(-np.polyfit(t, mass, 1)[0]) if t.size >= 2 else 0.0

    silo = scenes.silo(cells=48, material="g_local_mu2", props=(1e6, 0.3), dt=1e-4, hole_radius=0.12,
                       open_time=0.05, wall_frac=0.5, fill_height=0.5, mp={"grains_d": 5.3e-4})
    q = {}
    for p in ("mixed", "fp64"):
        s_ = mpm2d.Simulation(silo, device=dev, precision=p)
        q[p] = active_mass_rate(s_, silo["particles"]["m"], 3000, 50)
        s_.close()
    out["silo_discharge_rate"] = {"mixed": q["mixed"], "fp64": q["fp64"],
                                  "rel_diff": abs(q["mixed"] - q["fp64"]) / q["fp64"] if q["fp64"] else None,
                                  "scene": "g_local_mu2 silo, 48^2 elements, 3000 steps (kg/s per unit depth)"}
    col = scenes.column(Nx=129, Ny=129, h=1 / 128, width=0.25, height=0.4, material="g_local_mu2", rho=2450.0,
                        props=(1e6, 0.3), dt=1e-5, mp={"grains_d": 5.3e-4}, jitter=1e-3, seed=4)
    r, at100 = {}, {}
    for p in ("mixed", "fp64"):
        s_ = mpm2d.Simulation(col, device=dev, precision=p)
        s_.step(100)
        at100[p] = {f: s_.get(f) for f in ACC_FIELDS}
        s_.step(2900)
        r[p] = float(s_.get("x")[s_.get_map()[1] == 1].max())
        s_.close()
    cerr = {}
    for f in ACC_FIELDS:
        a, b = at100["mixed"][f], at100["fp64"][f]
        scale = (max(np.linalg.norm(at100["fp64"][g]) for g in ACC_GROUPS[f]) if f in ACC_GROUPS
                 else np.linalg.norm(b))
        cerr[f] = float(np.linalg.norm(a - b) / scale) if scale > 0 else float(np.linalg.norm(a - b))
    out["column_rel_l2_after_100_steps"] = cerr
    out["column_runout"] = {"mixed": r["mixed"], "fp64": r["fp64"], "rel_diff": abs(r["mixed"] - r["fp64"]) / r["fp64"],
                            "scene": "g_local_mu2 column, 128^2 elements, 3000 steps (largest active x, m)"}
    return out


def run_gpu(args):
    import torch

    rank, world, local = init_ranks(torch)
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    import mpm2d
    import scenes

    scene = make_scene()
    n = len(scene["particles"]["x"])
    nn = scene["Nx"] * scene["Ny"]
    ne = (scene["Nx"] - 1) * (scene["Ny"] - 1)
    peak, peak_kind = measured_peaks()

    def sync_all():
        barrier(torch, dev)

    def slowest(t):
        return max_over_ranks(torch, t)

    # --- plain FP64 form (headline) -------------------------------------------
    sim64 = mpm2d.Simulation(scene, device=dev, precision="fp64")
    stream64 = torch.cuda.ExternalStream(sim64.stream(), device=dev)
    sim64.step(args.warmup)
    sim64.synchronize()
    launches0 = sim64.launch_count()
    sync_all()
    with ClockSampler(dev) as clocks:
        ms64 = time_steps(sim64, args.steps, stream64, torch)
        sync_all()
    launches = sim64.launch_count() - launches0
    clk = clocks.summary()
    t64 = slowest(ms64 / 1e3)
    value = job_value(n * args.steps, world, t64)
    phases64 = phase_profile(sim64, max(3, min(args.steps, 10)), FP64_BYTES, n, ne, nn)
    sim64.close()
    g2p64 = phases64["g2p"]
    fp64_peak = mpm2d.fp64_rate(dev)
    step64_survey = phase_bytes({"s": FP64_STEP_SURVEY_BYTES}, "s", n, ne, nn)
    roofline = {"bound": "hbm", "kernel": "g2p (FP64 G2P + g_local_mu2, g2p_kernel<1,0>)",
                "achieved": g2p64["gbs"], "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": g2p64["gbs"] / peak,
                "traffic": G2P64_TRAFFIC_BYTES if n == 1048576 else None,
                "compute_bound": {
                    "pipe": "fp64", "unit": "FLOP/s", "peak": fp64_peak,
                    "peak_kind": "measured (mpmg_measure_fp64_rate: independent FMA chains, this GPU)"},
                "top_phase": max(phases64.items(), key=lambda kv: kv[1]["ms"])[0],
                "step_survey_bytes": step64_survey,
                "step_survey_frac": step64_survey / (ms64 / args.steps / 1e3) / 1e9 / peak,
                "phases": phases64}
    if G2P64_FLOPS_PER_PARTICLE:
        g2p_s = g2p64["ms"] / 1e3
        fl = G2P64_FLOPS_PER_PARTICLE * n / g2p_s
        # the pipe issues one FP64 instruction (an FMA is two FLOP) per slot
        inst = G2P64_PIPE_INSTR_PER_PARTICLE * n / g2p_s
        roofline["compute_bound"].update({"achieved": fl, "frac": fl / fp64_peak,
                                          "flops_per_particle": G2P64_FLOPS_PER_PARTICLE,
                                          "pipe_instr_per_particle": G2P64_PIPE_INSTR_PER_PARTICLE,
                                          "pipe_instr_per_s": inst, "pipe_frac": inst / (fp64_peak / 2)})

    # --- end to end through the C ABI with host buffers (FP64) ------------------
    # The user's run: create the simulation from host arrays (H2D of the
    # particle state), step in CUDA graphs of 8 steps with every step writing
    # its result (the step record: time, step count, device status) into a
    # ring in mapped pinned host memory (mpmg_record_ring), read each step's
    # record on the host one chunk behind (mpmg_record_ring_wait), and write
    # the output frame at the end (mpmg_get_fields of the driver's
    # write_frame fields into pinned host buffers).
    def e2e_run(precision, e2e_steps):
        host = {f: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for f in FRAME_FIELDS}
        sync_all()
        t0 = time.perf_counter()
        sim2 = mpm2d.Simulation(scene, device=dev, precision=precision)
        sim2.record_ring(32)
        t1 = time.perf_counter()
        last = None
        pending = []
        k = 0
        while k < e2e_steps:
            c = min(8, e2e_steps - k)
            sim2.step(c)
            for s_ in pending:
                last = sim2.record_ring_wait(s_)
            pending = list(range(k + 1, k + c + 1))
            k += c
        for s_ in pending:
            last = sim2.record_ring_wait(s_)
        t2 = time.perf_counter()
        assert last[1] == e2e_steps
        sim2.get_frame(FRAME_FIELDS, out=host)
        t3 = time.perf_counter()
        sync_all()
        e2e_t = slowest(t3 - t0)
        sim2.close()
        h2d_total = 9 * 8 * n                      # m v x y vx vy sxx sxy syy
        d2h_frame = len(FRAME_FIELDS) * 8 * n      # the frame's FP64 fields in particle order
        step_record = 80                           # ring slot: step number + step record + status word
        return {"value": n * e2e_steps * world / e2e_t, "unit": UNIT,
                "h2d_bytes_per_step": h2d_total / e2e_steps,
                "d2h_bytes_per_step": step_record + d2h_frame / e2e_steps, "steps": e2e_steps,
                "create_s": t1 - t0, "steps_s": t2 - t1, "frame_s": t3 - t2,
                "path": "mpmg_create from host arrays, mpmg_step in CUDA graphs of 8 steps, every step's "
                        "record written by the step into mapped pinned host memory and read on the host "
                        "(mpmg_record_ring / mpmg_record_ring_wait, one chunk behind), "
                        "one output frame (mpmg_get_fields of %d fields)" % len(FRAME_FIELDS)}

    e2e = e2e_run("fp64", args.e2e_steps)

    # --- mixed forms (FP32 particles), same workload ------------------------------
    def mixed_run(precision):
        sim = mpm2d.Simulation(scene, device=dev, precision=precision)
        stream = torch.cuda.ExternalStream(sim.stream(), device=dev)
        sim.step(args.warmup)
        sim.synchronize()
        msteps = max(args.steps, 50)
        sync_all()
        ms = time_steps(sim, msteps, stream, torch)
        sync_all()
        t = slowest(ms / 1e3)
        phases = phase_profile(sim, max(3, min(args.steps, 10)), MIXED_BYTES, n, ne, nn)
        sim.close()
        step_ms = ms / msteps
        builder = sum(phase_bytes(MIXED_BYTES, k, n, ne, nn) for k in MIXED_BYTES)
        survey = phase_bytes({"s": MIXED_STEP_SURVEY_BYTES}, "s", n, ne, nn)
        g2p_survey = phase_bytes({"s": MIXED_G2P_SURVEY_BYTES}, "s", n, ne, nn)
        g2p_s = phases["g2p"]["ms"] / 1e3
        return {"value": job_value(n * msteps, world, t), "unit": UNIT, "steps": msteps, "ms_per_step": step_ms,
                "dtype": "f32 particles",
                "roofline": {"bound": "hbm", "kernel": "g2p (mx_g2p_kernel)", "unit": "GB/s", "peak": peak,
                             "g2p_achieved_builder_bytes": phases["g2p"]["gbs"],
                             "g2p_frac_builder_bytes": phases["g2p"]["gbs"] / peak,
                             "g2p_achieved_survey_bytes": g2p_survey / g2p_s / 1e9,
                             "g2p_frac_survey_bytes": g2p_survey / g2p_s / 1e9 / peak,
                             "traffic": G2P_TRAFFIC_BYTES if n == 1048576 else None,
                             "step_builder_bytes": builder,
                             "step_frac_builder_bytes": builder / (step_ms / 1e3) / 1e9 / peak,
                             "step_survey_bytes": survey,
                             "step_frac_survey_bytes": survey / (step_ms / 1e3) / 1e9 / peak,
                             "phases": phases}}

    mixed_f64node = mixed_run("mixed_f64node")
    mixed_f64node["note"] = ("the chosen form: FP32 particle state, P2G/G2P and material law; FP64 nodal mass "
                             "and momentum sums and the division by nodal mass")
    mixed = mixed_run("mixed")
    mixed["note"] = ("float-float (48-bit) nodal mass and momentum sums and division on the FP32 pipe in place "
                     "of FP64: a deviation from the chosen form, kept because GB300 runs FP64 at 1/64 of the "
                     "FP32 rate")


    # --- accuracy of the mixed form against the FP64 form ------------------------
    accuracy_line = accuracy_report(mpm2d, scenes, scene, dev) if not args.no_accuracy else None

    # --- batched ensemble: 256 independent silo / heap runs in one context ------
    batch_line = None
    if not args.no_batch:
        ens = scenes.ensemble(count=256, seed=1)
        nb = sum(len(sc["particles"]["x"]) for sc in ens)
        bsim = mpm2d.Batch(ens)
        bstream = torch.cuda.ExternalStream(bsim.stream(), device=dev)
        bsim.step(args.warmup)
        bsim.synchronize()
        # launch shape tuned on the batch itself (mpmg_autotune; results unchanged)
        tuning = bsim.autotune(steps_per_trial=16)
        bsim.synchronize()
        bsteps = args.batch_steps
        sync_all()
        msb = time_steps(bsim, bsteps, bstream, torch)
        sync_all()
        bsim.close()
        value_b = nb * bsteps * world / slowest(msb / 1e3)
        # algorithmic bytes of a batched step: the builder's accounting of the
        # unfused kernels a batch runs, and the compulsory bytes
        bn = nb
        be = int(sum((sc["Nx"] - 1) * (sc["Ny"] - 1) for sc in ens))
        bnn = int(sum(sc["Nx"] * sc["Ny"] for sc in ens))
        b_builder = sum(phase_bytes(BATCH_BYTES, k, bn, be, bnn) for k in BATCH_BYTES)
        b_survey = phase_bytes({"s": MIXED_STEP_SURVEY_BYTES}, "s", bn, be, bnn)
        b_step_s = msb / bsteps / 1e3
        # the same members one at a time (each its own context and step graphs)
        seq_ms = 0.0
        for sc in ens:
            one = mpm2d.Simulation(sc, device=dev, precision="mixed")
            ostream = torch.cuda.ExternalStream(one.stream(), device=dev)
            one.step(3)
            one.synchronize()
            seq_ms += time_steps(one, 5, ostream, torch) / 5
            one.close()
        value_seq = nb / (seq_ms / 1e3)
        batch_line = {"value": value_b, "unit": UNIT, "members": len(ens), "particles": nb,
                      "elements": int(sum((sc["Nx"] - 1) * (sc["Ny"] - 1) for sc in ens)),
                      "steps": bsteps, "ms_per_step": msb / bsteps,
                      "sequential_value": value_seq, "batch_over_sequential": value_b / value_seq,
                      "autotune": tuning,
                      "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak,
                                   "step_builder_bytes": b_builder,
                                   "step_frac_builder_bytes": b_builder / b_step_s / 1e9 / peak,
                                   "step_survey_bytes": b_survey,
                                   "step_frac_survey_bytes": b_survey / b_step_s / 1e9 / peak},
                      "workload": "ensemble of 256 g_local_mu2 runs (silo / heap), grids 64^2-384^2 "
                                  "elements, 5k-200k particles log-uniform, outlet 0.02-0.12, mu_s 0.30-0.45 "
                                  "(seed 1), mixed precision"}

    # --- nonlocal silo (g_nonlocal_mu2, FP64, fluidity PCG every step) -------------
    nonlocal_line = None
    if not args.no_nonlocal:
        nsc = scenes.silo_prestressed(cells=512)
        nnl = len(nsc["particles"]["x"])
        nsim = mpm2d.Simulation(nsc, device=dev)
        nstream = torch.cuda.ExternalStream(nsim.stream(), device=dev)
        nsim.step(args.warmup)
        nsim.synchronize()
        nsteps_nl = max(3, min(args.steps, 10))
        sync_all()
        msn = time_steps(nsim, nsteps_nl, nstream, torch)
        sync_all()
        iters = []
        nsim.enable_phase_timing(True)
        for _ in range(3):
            nsim.step(1)
            nsim.synchronize()
            rc_s, it, res = nsim.last_solve()
            iters.append(it)
        pt = nsim.phase_times()
        nsim.enable_phase_timing(False)
        e_map, a_map = nsim.get_map()
        filled = int(np.unique(e_map[a_map == 1]).size)
        nsim.close()
        # the same silo in the mixed form (FP32 step, FP64 fluidity solve)
        msim = mpm2d.Simulation(nsc, device=dev, precision="mixed")
        mstream = torch.cuda.ExternalStream(msim.stream(), device=dev)
        msim.step(args.warmup)
        msim.synchronize()
        sync_all()
        msm = time_steps(msim, nsteps_nl, mstream, torch)
        sync_all()
        msim.close()
        solve_ms = pt["fluidity"][0] / max(pt["fluidity"][1], 1)
        it_mean = float(np.mean(iters))
        dofs = nsc["Nx"] * nsc["Ny"]

        # the same steps with the Jacobi preconditioner, and both later in the
        # run (step 60), where the flow near the outlet has developed and
        # Jacobi-PCG needs hundreds of iterations a step
        def timed_run(precond, start, steps):
            sim_ = mpm2d.Simulation(nsc, device=dev, precond=precond)
            st_ = torch.cuda.ExternalStream(sim_.stream(), device=dev)
            sim_.step(start)
            sim_.synchronize()
            ms_ = time_steps(sim_, steps, st_, torch)
            its_ = []
            for _ in range(2):
                sim_.step(1)
                sim_.synchronize()
                its_.append(sim_.last_solve()[1])
            sim_.close()
            return ms_ / steps, float(np.mean(its_))

        jac_ms, jac_it = timed_run("jacobi", args.warmup, nsteps_nl)
        late_mg_ms, late_mg_it = timed_run("multigrid", 60, 5)
        late_jac_ms, late_jac_it = timed_run("jacobi", 60, 3)
        nonlocal_line = {
            "workload": "g_nonlocal_mu2 square silo, 835 996 particles, 513x513 nodes, outlet radius 0.06, "
                        "lithostatic start, CG to relative residual 1e-10 every step",
            "dtype": "f64", "value": nnl * nsteps_nl / (msn / 1e3), "unit": UNIT,
            "ms_per_step": msn / nsteps_nl, "precond": "multigrid",
            "iterations_per_step": it_mean,
            "mixed_value": nnl * nsteps_nl / (msm / 1e3), "mixed_ms_per_step": msm / nsteps_nl,
            "fluidity_ms_per_step": solve_ms,
            "jacobi": {"ms_per_step": jac_ms, "iterations_per_step": jac_it},
            "step_60": {"multigrid": {"ms_per_step": late_mg_ms, "iterations_per_step": late_mg_it},
                        "jacobi": {"ms_per_step": late_jac_ms, "iterations_per_step": late_jac_it}},
            "dofs": dofs, "filled_elements": filled,
            "cpu_baseline": None,
            "note": "steps %d-%d of the run; fluidity phase = bulk fluidity, element assembly, "
                    "multigrid-preconditioned CG (one cooperative kernel), stress update"
                    % (args.warmup + 1, args.warmup + nsteps_nl)}
        if rank == 0 and not args.no_cpu_baseline:
            cpu_threads = os.cpu_count() or 1
            cpu_s, cpu_it = cpu_nonlocal_baseline(nsc, 2, cpu_threads)
            nonlocal_line["cpu_baseline"] = {
                "value": nnl / cpu_s, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                "ms_per_step": 1e3 * cpu_s, "iterations_per_step": cpu_it,
                "sample": "steps 2-3 of the same silo through the oracle with Jacobi-CG to 1e-10"}

    # --- adjoint: gradient of a trajectory loss w.r.t. (mu_s, mu_2, I0, E) -----
    adjoint_line = None
    if not args.no_adjoint:
        adj_steps, adj_k = 2000, 100
        theta0 = np.array([0.3819, 0.6435, 0.278, 1e6])
        theta_t = theta0 + np.array([0.02, -0.03, 0.0, 0.0])
        theta_t[3] *= 1.1

        def final_xy(theta):
            s_ = mpm2d.Simulation(scenes.adjoint_column(theta), device=dev)
            s_.step(adj_steps)
            xy = (s_.get("x"), s_.get("y"))
            s_.close()
            return xy

        xt, yt = final_xy(theta_t)
        s_ = mpm2d.Simulation(scenes.adjoint_column(theta0), device=dev)
        s_.step(3)
        s_.synchronize()
        t0 = time.perf_counter()
        s_.step(adj_steps)
        s_.synchronize()
        t_fwd = time.perf_counter() - t0
        s_.close()
        s_ = mpm2d.Simulation(scenes.adjoint_column(theta0), device=dev)
        t0 = time.perf_counter()
        s_.adj_forward_tape(adj_steps, adj_k)
        t_tape = time.perf_counter() - t0
        xa, ya = s_.get("x"), s_.get("y")
        t0 = time.perf_counter()
        grad = s_.adj_backward(2 * (xa - xt), 2 * (ya - yt))
        t_bwd = time.perf_counter() - t0
        s_.close()
        fd = []
        for k in range(4):
            hk = 1e-4 * theta0[k]
            tp, tm = theta0.copy(), theta0.copy()
            tp[k] += hk
            tm[k] -= hk
            (xp, yp), (xm, ym) = final_xy(tp), final_xy(tm)
            fd.append((np.sum((xp - xt) ** 2 + (yp - yt) ** 2) - np.sum((xm - xt) ** 2 + (ym - yt) ** 2))
                      / (2 * hk))
        names = ("mu_s", "mu_2", "I0", "E")
        adjoint_line = {
            "workload": "g_local_mu2 column, 65 536 particles, 256x128 elements, dt 2e-6, 2000 steps, "
                        "loss = sum |x(T) - x_target(T)|^2 against mu_s+0.02, mu_2-0.03, E*1.1",
            "dtype": "f64", "steps": adj_steps, "checkpoint_every": adj_k,
            "forward_s": t_fwd, "tape_forward_s": t_tape, "backward_s": t_bwd,
            "adjoint_over_forward": t_bwd / t_fwd,
            "grad": dict(zip(names, map(float, grad))), "fd_central_1e-4": dict(zip(names, map(float, fd))),
            "max_rel_err_vs_fd": float(max(abs(g - f) / abs(f) for g, f in zip(grad, fd) if f != 0))}

        # the nonlocal step (g_nonlocal_mu2: the fluidity solve reversed by an
        # adjoint solve), whose gradient also reaches the nonlocal amplitude A
        # 50 steps: over longer horizons the nonlocal silo's loss turns rough
        # (finite differences stop agreeing across step sizes)
        nl_steps, nl_k = 50, 25
        nl0 = np.array([0.3819, 0.6435, 0.278, 1e6, 0.48])

        def nl_scene(th):
            mp = {"grains_d": 5.3e-4, "mu_s": th[0], "mu_2": th[1], "I0": th[2], "A": th[4]}
            return scenes.silo_prestressed(cells=128, dt=2e-5, mp=mp, props=(th[3], 0.3))

        def nl_xy(th):
            s_ = mpm2d.Simulation(nl_scene(th), device=dev)
            s_.step(nl_steps)
            xy = (s_.get("x"), s_.get("y"))
            s_.close()
            return xy

        nxt, nyt = nl_xy(nl0 * np.array([1.05, 0.95, 1.0, 1.1, 1.2]))
        s_ = mpm2d.Simulation(nl_scene(nl0), device=dev)
        nl_n = s_.n
        s_.synchronize()
        t0 = time.perf_counter()
        s_.step(nl_steps)
        s_.synchronize()
        nl_fwd = time.perf_counter() - t0
        s_.close()
        s_ = mpm2d.Simulation(nl_scene(nl0), device=dev)
        t0 = time.perf_counter()
        s_.adj_forward_tape(nl_steps, nl_k)
        nl_tape = time.perf_counter() - t0
        xa, ya = s_.get("x"), s_.get("y")
        t0 = time.perf_counter()
        nl_grad = s_.adj_backward(2 * (xa - nxt), 2 * (ya - nyt))
        nl_bwd = time.perf_counter() - t0
        s_.close()
        hA = 1e-4 * nl0[4]
        tp, tm = nl0.copy(), nl0.copy()
        tp[4] += hA
        tm[4] -= hA
        (xp, yp), (xm, ym) = nl_xy(tp), nl_xy(tm)
        fdA = (np.sum((xp - nxt) ** 2 + (yp - nyt) ** 2) - np.sum((xm - nxt) ** 2 + (ym - nyt) ** 2)) / (2 * hA)
        adjoint_line["nonlocal"] = {
            "workload": "g_nonlocal_mu2 square silo from a lithostatic stress, %d particles, 128^2 elements, "
                        "dt 2e-5, %d steps, loss against mu_s*1.05, mu_2*0.95, E*1.1, A*1.2" % (nl_n, nl_steps),
            "checkpoint_every": nl_k, "forward_s": nl_fwd, "tape_forward_s": nl_tape, "backward_s": nl_bwd,
            "adjoint_over_forward": nl_bwd / nl_fwd,
            "grad": dict(zip(names + ("A",), map(float, nl_grad))), "fd_central_1e-4_A": float(fdA),
            "rel_err_A_vs_fd": float(abs(nl_grad[4] - fdA) / abs(fdA)) if fdA != 0 else None}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms64 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(scene, world),
        "step_launch": "CUDA graphs of 8 steps",
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roofline,
        "e2e": e2e,
        "mixed_f64node": mixed_f64node,
        "mixed": mixed,
        "mixed_f64node_over_fp64": mixed_f64node["value"] / value,
        "mixed_over_fp64": mixed["value"] / value,
        "batch": batch_line,
        "accuracy": accuracy_line,
        "adjoint": adjoint_line,
        "nonlocal_silo": nonlocal_line,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cb, cb_t = cpu_baseline(scene, args.cpu_steps, threads)
        cb1, cb1_t = cpu_baseline(scene, args.cpu_steps_1, 1)
        line["cpu_baseline"] = {
            "value": cb, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d steps of the full %d-particle workload (%.1f s)" % (args.cpu_steps, n, cb_t),
            "threads_all": {"value": cb, "cores": threads, "steps": args.cpu_steps, "seconds": cb_t},
            "threads_1": {"value": cb1, "cores": 1, "steps": args.cpu_steps_1, "seconds": cb1_t},
            "port_over_reference": PORT_OVER_REFERENCE}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=60, help="CPU-baseline steps on all host cores")
    ap.add_argument("--cpu-steps-1", type=int, default=8, help="CPU-baseline steps on one core")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--batch-steps", type=int, default=2000, help="timed steps of the batched ensemble")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    ap.add_argument("--no-nonlocal", action="store_true", help="skip the nonlocal silo measurement")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the mixed-vs-FP64 accuracy report")
    ap.add_argument("--e2e-steps", type=int, default=500,
                    help="steps of the end-to-end run (one output frame at its end)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3         # at least three untimed warm-up steps
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
