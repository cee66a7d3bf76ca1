import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mpm-2d_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


# Fields of the particle state that fully determine the next step.
STATE_FIELDS = ["x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "ux", "uy"]


def load_golden(name):
    """Scene and recorded reference data of tests/golden/step_<name>.npz."""
    d = np.load(os.path.join(GOLDEN, "step_%s.npz" % name))
    Nx, Ny = (int(v) for v in d["meta_grid"])
    h, dt = (float(v) for v in d["meta_h_dt"])
    scene = {
        "Nx": Nx, "Ny": Ny, "h": h, "dt": dt,
        "material": str(d["meta_material"]), "bc": str(d["meta_bc"]),
        "props": [float(v) for v in d["meta_props"]],
        "bcf": [float(v) for v in d["meta_bcf"]],
        "bci": [int(v) for v in d["meta_bci"]],
        "gravity": None,
        "particles": {k[3:]: d[k] for k in d.files if k.startswith("in_")},
    }
    if "meta_scheme" in d.files:
        scene["scheme"] = str(d["meta_scheme"])
    return scene, d


def state_at(d, step, material):
    """Per-particle fields needed to restart the reference at a checkpoint."""
    fields = {k: d["s%d_%s" % (step, k)] for k in STATE_FIELDS}
    if material == "g_local_mu2":
        fields["Tzz"] = d["s%d_Tzz" % step]
        for k in (9, 10):
            fields["state%d" % k] = d["s%d_state%d" % (step, k)]
    elif material == "g_nonlocal_mu2":
        for k in (0, 3, 4, 5, 6, 9, 10):
            fields["state%d" % k] = d["s%d_state%d" % (step, k)]
    elif material == "g_nonlocal":
        for k in (3, 4, 5, 9, 10):
            fields["state%d" % k] = d["s%d_state%d" % (step, k)]
    return fields


def rel_err(a, b, scale=None):
    """Max abs difference over a field divided by a magnitude: `scale` when
    given, else the field's own max magnitude (0 for equal fields)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if not a.size:
        return 0.0
    if scale is None:
        scale = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / max(scale, 1e-300))


# Fields compared against the magnitude of their physical group, so that a
# component that is zero up to round-off (sxy of a symmetric block) is judged
# against the stress scale rather than against its own noise.
FIELD_GROUPS = {
    "x": ("x", "y"), "y": ("x", "y"),
    "vx": ("vx", "vy"), "vy": ("vx", "vy"),
    "ax": ("ax", "ay"), "ay": ("ax", "ay"),
    "ux": ("ux", "uy"), "uy": ("ux", "uy"),
    "sxx": ("sxx", "sxy", "syy"), "sxy": ("sxx", "sxy", "syy"), "syy": ("sxx", "sxy", "syy"),
    "Tzz": ("sxx", "syy", "Tzz"),
    "exx": ("exx", "exy", "eyy", "wxy"), "exy": ("exx", "exy", "eyy", "wxy"),
    "eyy": ("exx", "exy", "eyy", "wxy"), "wxy": ("exx", "exy", "eyy", "wxy"),
    "node_mx": ("node_mx", "node_my"), "node_my": ("node_mx", "node_my"),
    "node_fx": ("node_fx", "node_fy"), "node_fy": ("node_fx", "node_fy"),
    "node_vx": ("node_vx", "node_vy"), "node_vy": ("node_vx", "node_vy"),
    # szz of the 3D-trial materials; beta = -p / (K dt) (tensile branch, zero
    # up to round-off at a free surface) against the plastic-rate scale
    "state1": ("sxx", "syy", "state1"),
    "state5": ("state5", "state10"),
}


def group_scale(get, field):
    """Magnitude of a field's group; get(name) returns the reference array."""
    names = FIELD_GROUPS.get(field, (field,))
    return max(float(np.max(np.abs(get(n)))) if np.size(get(n)) else 0.0 for n in names)


def field_err(got, want_get, field):
    """rel_err of one field against its group's magnitude."""
    return rel_err(got, want_get(field), group_scale(want_get, field))


@pytest.fixture(scope="session")
def golden():
    return load_golden
