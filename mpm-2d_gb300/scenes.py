"""Seeded synthetic inputs in the layouts the reference's generators use.

The reference ships particle generators (generate_block_particles.py:26-51,
examples/silo/generate_silo_particles.py): material points on a regular
lattice of spacing s at (k + 1/2) s from the block's lower-left corner,
ordered x-major, with mass rho s^2 and volume s^2.  The reference publishes no
benchmark inputs, so every workload here is synthetic with those layouts.

Workloads (sizes follow the configurations the benchmark plan names):
  config1        isolin block in a box: 65x65 nodes on the unit square, block
                 [0.25, 0.75] x [0, 0.5] at 2x2 particles per element (4096),
                 jittered +-1e-3 (seeded), rho 1500, E 1e6, nu 0.3, dt 1e-5
  box_fill       1 048 576 particles: 513x513 nodes, the whole unit square at
                 2x2 per element, box walls (the "1 M particles" workload)
  column         granular column collapse (g_local_mu2 constants of the
                 benchmark: rho 2450, d 5.3e-4) on an Nx x Ny grid
  silo           square-silo discharge fill (x < wall fraction, 2x2 per element)
"""
import numpy as np


def block_particles(x0, y0, width, height, spacing, rho, jitter=0.0, seed=0, reflect_y=True):
    """Lattice block in x-major order (generate_block_particles.py:26-51)."""
    nx = int(np.floor(width / spacing + 1e-9))
    ny = int(np.floor(height / spacing + 1e-9))
    sx = (0.5 + np.arange(nx)) * spacing + x0
    sy = (0.5 + np.arange(ny)) * spacing + y0
    X, Y = np.meshgrid(sx, sy, indexing="ij")     # x-major: y varies fastest
    x = X.ravel().copy()
    y = Y.ravel().copy()
    if jitter > 0:
        rng = np.random.default_rng(seed)
        x += rng.uniform(-jitter, jitter, size=x.shape)
        y += rng.uniform(-jitter, jitter, size=y.shape)
        if reflect_y:
            y = np.abs(y)
    n = x.size
    return {
        "m": np.full(n, rho * spacing * spacing),
        "v": np.full(n, spacing * spacing),
        "x": x, "y": y,
        "vx": np.zeros(n), "vy": np.zeros(n),
        "sxx": np.zeros(n), "sxy": np.zeros(n), "syy": np.zeros(n),
    }


def config1(seed=0, gravity=None):
    """Plain FP64 USL, isolin block in the box BC (4096 particles, 65^2 nodes)."""
    N = 65
    h = 1.0 / (N - 1)
    p = block_particles(0.25, 0.0, 0.5, 0.5, h / 2, 1500.0, jitter=1e-3, seed=seed)
    return {"Nx": N, "Ny": N, "h": h, "dt": 1e-5, "material": "isolin", "props": [1e6, 0.3],
            "bc": "box", "bcf": [0.0, 0.0, 1.0, 1.0], "bci": [1, 3, 1, 0], "gravity": gravity,
            "particles": p, "steps": 1000}


def box_fill(cells=512, ppc_1d=2, material="g_local_mu2", rho=2450.0, props=(1e6, 0.3), dt=2e-6,
             gravity=None, mp=None):
    """The whole unit square filled at ppc_1d^2 particles per element."""
    N = cells + 1
    h = 1.0 / cells
    p = block_particles(0.0, 0.0, 1.0, 1.0, h / ppc_1d, rho)
    scene = {"Nx": N, "Ny": N, "h": h, "dt": dt, "material": material, "props": list(props),
             "bc": "box", "bcf": [0.0, 0.0, 1.0, 1.0], "bci": [1, 3, 1, 0], "gravity": gravity,
             "particles": p}
    if mp:
        scene["mp"] = dict(mp)
    return scene


def column(Nx=65, Ny=65, h=1.0 / 64, width=0.25, height=0.5, ppc_1d=2, material="g_local_mu2",
           rho=2450.0, props=(1e6, 0.3), dt=1e-5, gravity=None, mp=None, jitter=0.0, seed=0):
    """Granular column at the left wall of an Nx x Ny grid (box walls)."""
    p = block_particles(0.0, 0.0, width, height, h / ppc_1d, rho, jitter=jitter, seed=seed)
    scene = {"Nx": Nx, "Ny": Ny, "h": h, "xmax": (Nx - 1) * h if Nx != Ny else 1.0,
             "ymax": (Ny - 1) * h if Nx != Ny else 1.0, "dt": dt, "material": material,
             "props": list(props), "bc": "box", "bcf": [0.0, 0.0, 1.0, 1.0], "bci": [1, 3, 1, 0],
             "gravity": gravity, "particles": p}
    if mp:
        scene["mp"] = dict(mp)
    return scene


def silo(cells=512, ppc_1d=2, hole_radius=0.06, open_time=0.1, wall_frac=0.8,
         material="g_nonlocal_mu2", rho=2450.0, props=(1e6, 0.3), dt=1e-6, fill_height=None,
         gravity=None, mp=None):
    """Silo fill left of the wall column (square_silo.c:44), 2x2 per element."""
    N = cells + 1
    h = 1.0 / cells
    wall_col = int((N - 1) * wall_frac)
    width = wall_col * h
    height = (cells - 1) * h if fill_height is None else fill_height
    p = block_particles(0.0, 0.0, width, height, h / ppc_1d, rho)
    scene = {"Nx": N, "Ny": N, "h": h, "dt": dt, "material": material, "props": list(props),
             "bc": "square_silo", "bcf": [hole_radius, open_time, wall_frac], "bci": [],
             "gravity": gravity, "particles": p}
    if mp:
        scene["mp"] = dict(mp)
    return scene


def with_particles(scene, idx):
    """A copy of scene keeping only particles idx (for bounded samples)."""
    out = dict(scene)
    out["particles"] = {k: np.ascontiguousarray(v[idx]) for k, v in scene["particles"].items()}
    return out


def ensemble(count=256, seed=1, ppc_1d=2, cells_range=(64, 384), particles_range=(5e3, 2e5),
             outlet_range=(0.02, 0.12), mu_s_range=(0.30, 0.45), dt=5e-6, rho=2450.0, props=(1e6, 0.3),
             grains_d=5.3e-4):
    """Independent silo and heap runs of uneven sizes for a batch: per member a
    grid of n x n elements (n uniform in cells_range), a target particle count
    log-uniform in particles_range (a silo fill left of the wall or a column
    on the floor of a box, 2x2 per element, clipped to the domain), a silo
    outlet (hole radius) uniform in outlet_range and mu_s uniform in
    mu_s_range; g_local_mu2 with the benchmark's grain size."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(cells_range[0], cells_range[1] + 1))
        target = float(np.exp(rng.uniform(np.log(particles_range[0]), np.log(particles_range[1]))))
        outlet = float(rng.uniform(*outlet_range))
        mu_s = float(rng.uniform(*mu_s_range))
        h = 1.0 / n
        s = h / ppc_1d
        mp = {"mu_s": mu_s, "grains_d": grains_d}
        if k % 2 == 0:
            wall_frac = 0.8
            width = int(n * wall_frac) * h
            cols = int(width / s)
            rows = max(1, min(int(round(target / cols)), int((1.0 - 2 * h) / s)))
            p = block_particles(0.0, 0.0, width, rows * s, s, rho)
            sc = {"Nx": n + 1, "Ny": n + 1, "h": h, "dt": dt, "material": "g_local_mu2", "props": list(props),
                  "bc": "square_silo", "bcf": [outlet, 0.0, wall_frac], "bci": [], "gravity": None,
                  "particles": p, "mp": mp}
        else:
            width = float(rng.uniform(0.2, 0.5))
            cols = int(width / s)
            rows = max(1, min(int(round(target / cols)), int((1.0 - 2 * h) / s)))
            p = block_particles(0.0, 0.0, width, rows * s, s, rho)
            sc = {"Nx": n + 1, "Ny": n + 1, "h": h, "dt": dt, "material": "g_local_mu2", "props": list(props),
                  "bc": "box", "bcf": [0.0, 0.0, 1.0, 1.0], "bci": [1, 3, 1, 0], "gravity": None,
                  "particles": p, "mp": mp}
        out.append(sc)
    return out


def column_2x05(fine=False, gravity=-9.81):
    """The rectangular column-collapse workload: a 0.4 x 0.3 m g_local_mu2
    column (mu(I) constants of the reference, grain size 5.3e-4 m) at 2 x 2
    particles per element in a 2 x 0.5 m box, dt 2e-6.  fine=False: 512 x 128
    elements (h = 1/256, 31 212 particles); fine=True: 1024 x 256 elements
    (h = 1/512, 125 563 particles).  Constant gravity by default (the
    reference's ramp reaches only a tenth of g in the 5000 steps the workload
    runs)."""
    n = 1024 if fine else 512
    h = 2.0 / n
    return column(Nx=n + 1, Ny=n // 4 + 1, h=h, width=0.4, height=0.3, ppc_1d=2, material="g_local_mu2",
                  rho=2450.0, props=(1e6, 0.3), dt=2e-6, gravity=gravity, mp={"grains_d": 5.3e-4})


def adjoint_column(theta=(0.3819, 0.6435, 0.278, 1e6), seed=2):
    """The adjoint benchmark: a 0.25 x 0.25 m g_local_mu2 column (64 x 64
    elements at 4 x 4 particles each: 65 536 particles) in a 1 x 0.5 m box of
    256 x 128 elements, dt 2e-6; theta = (mu_s, mu_2, I0, E)."""
    return column(Nx=257, Ny=129, h=1.0 / 256, width=0.25, height=0.25, ppc_1d=4, material="g_local_mu2",
                  rho=2450.0, props=(theta[3], 0.3), dt=2e-6,
                  mp={"grains_d": 5.3e-4, "mu_s": theta[0], "mu_2": theta[1], "I0": theta[2]},
                  jitter=1e-4, seed=seed)


def silo_prestressed(cells=512, material="g_nonlocal_mu2", hole_radius=0.06, open_time=0.0, wall_frac=0.8,
                     dt=1e-6, rho=2450.0, props=(1e6, 0.3), mp=None, surcharge=500.0, k0=0.4):
    """The nonlocal silo benchmark (513^2 nodes, 835 996 particles at 2x2 per
    element left of the wall column) starting from a lithostatic stress
    (syy = -rho g (H - y) - surcharge, sxx = k0 syy) under constant gravity,
    with the outlet open.  With k0 = 0.4 the stress ratio tau / p = 0.43
    exceeds mu_s everywhere, so the fluidity solve is non-trivial from the
    first step."""
    sc = silo(cells=cells, material=material, hole_radius=hole_radius, open_time=open_time,
              wall_frac=wall_frac, rho=rho, props=props, dt=dt, gravity=-9.8,
              mp=mp if mp is not None else {"grains_d": 5.3e-4, "A": 0.48})
    p = sc["particles"]
    H = float(np.max(p["y"])) + 0.5 / cells
    p["syy"] = -rho * 9.8 * (H - p["y"]) - surcharge
    p["sxx"] = k0 * p["syy"]
    return sc

