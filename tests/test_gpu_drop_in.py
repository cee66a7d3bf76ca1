"""The libmpm-compatible entry points (include/mpm_libmpm.h) driven by a C
host that uses them as the reference's driver uses libmpm: a pthread team
calling explicit_mpm_step_usl_threaded, the serial tail with the frame check
and time_varying_loads (tests/drop_in/driver_test.c).  Results are compared
with the oracle run with the same number of threads."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT, field_err
from oracle import oracle as O
import mpmg_build
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = mpmg_build.build()
    out = str(tmp_path_factory.mktemp("drop_in") / "driver_test")
    cmd = ["gcc", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "drop_in", "driver_test.c"),
           "-L", os.path.dirname(lib), "-lmpm_gb300", "-lpthread",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True)
    return out


def run_driver(driver, tmp_path, scene, threads, steps, sample_rate, musl=False):
    p = scene["particles"]
    n = len(p["x"])
    mprops = scene.get("props", [1e6, 0.3])
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(struct.pack("6i", scene["Nx"], threads, steps, len(mprops), len(scene["bcf"]),
                            len(scene["bci"])))
        f.write(struct.pack("3d", scene["h"], scene["dt"], sample_rate))
        f.write(scene["material"].encode().ljust(64, b"\0"))
        f.write(scene["bc"].encode().ljust(64, b"\0"))
        f.write(np.asarray(mprops, dtype=np.float64).tobytes())
        f.write(np.asarray(scene["bcf"], dtype=np.float64).tobytes())
        f.write(np.asarray(scene["bci"], dtype=np.int32).tobytes())
        f.write(struct.pack("q", n))
        f.write(np.stack([np.asarray(p[k], dtype=np.float64) for k in
                          ("m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy")], axis=1).tobytes())
    subprocess.run([driver, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")] + (["musl"] if musl else []),
                   check=True, capture_output=True, timeout=600)
    raw = open(tmp_path / "out.bin", "rb").read()
    n_out, t, frames = struct.unpack_from("qdq", raw, 0)
    rec = np.dtype([("d", "<f8", 12), ("i", "<i4", 2)])
    arr = np.frombuffer(raw, dtype=rec, offset=24, count=n_out)
    names = ["x", "y", "vx", "vy", "sxx", "sxy", "syy", "v", "ux", "uy", "state9", "state10"]
    out = {k: arr["d"][:, j].copy() for j, k in enumerate(names)}
    out["in_element"] = arr["i"][:, 0].copy()
    out["active"] = arr["i"][:, 1].copy()
    return t, frames, out


@pytest.mark.parametrize("case", ["isolin_box", "mu2_silo", "dp_silo", "t2d_silo", "ext_silo"])
def test_drop_in_driver_matches_oracle(driver, tmp_path, case):
    if case == "isolin_box":
        scene, steps = scenes.config1(seed=2), 200
    else:
        material, props = {"mu2_silo": ("g_local_mu2", (1e6, 0.3)),
                           "dp_silo": ("dp_ri_mt", (1e6, 0.3, 0.3819)),
                           "t2d_silo": ("g_local_mu2_true_2d", (1e6, 0.3)),
                           "ext_silo": ("g_local_mu2_ext", (1e6, 0.3))}[case]
        scene = scenes.silo(cells=32, material=material, props=props, dt=1e-5, hole_radius=0.1,
                            open_time=0.001, wall_frac=0.5, fill_height=0.6)
        steps = 300
    threads = 3
    t, frames, got = run_driver(driver, tmp_path, scene, threads, steps, sample_rate=5000.0)
    orc = O.Oracle(scene, nthreads=threads)
    orc.step(steps)
    assert t == orc.t
    # one frame per 0.2 ms (20 steps), from t = 0 (src/main.c:955)
    assert frames == sum(1 for k in range(1000) if orc.t >= k / 5000.0)
    for f in ("x", "y", "vx", "vy", "sxx", "sxy", "syy", "v", "ux", "uy"):
        assert field_err(got[f], orc.get, f) <= 1e-9, (case, f, field_err(got[f], orc.get, f))
    e, a = orc.get_map()
    np.testing.assert_array_equal(got["active"], a)
    np.testing.assert_array_equal(got["in_element"][a == 1], e[a == 1])
    if scene["material"] != "isolin":
        for f in ("state9", "state10"):
            assert field_err(got[f], orc.get, f) <= 1e-8, (case, f)


@pytest.mark.parametrize("case", ["isolin_box", "dp_silo"])
def test_drop_in_musl_entry_point_matches_oracle(driver, tmp_path, case):
    """explicit_mpm_step_musl_threaded through the libmpm layer, against the
    oracle's MUSL step with the same number of threads."""
    if case == "isolin_box":
        scene, steps = scenes.config1(seed=2), 200
    else:
        scene = scenes.silo(cells=32, material="dp_ri_mt", props=(1e6, 0.3, 0.3819), dt=1e-5, hole_radius=0.1,
                            open_time=0.001, wall_frac=0.5, fill_height=0.6)
        steps = 300
    threads = 3
    t, frames, got = run_driver(driver, tmp_path, scene, threads, steps, sample_rate=5000.0, musl=True)
    orc = O.Oracle(dict(scene, scheme="musl"), nthreads=threads)
    orc.step(steps)
    assert t == orc.t
    for f in ("x", "y", "vx", "vy", "sxx", "sxy", "syy", "v", "ux", "uy"):
        assert field_err(got[f], orc.get, f) <= 1e-9, (case, f, field_err(got[f], orc.get, f))
    e, a = orc.get_map()
    np.testing.assert_array_equal(got["active"], a)

