"""Python binding of the mpm_gb300 C ABI (include/mpm_gb300.h) over ctypes.

``Simulation`` holds one device-resident mpm-2d simulation: the reference's
explicit USL step (libmpm/process_usl.c:465-592) with one of its material
plugins (isolin, g_local_mu2, g_nonlocal_mu2, g_nonlocal) and boundary
plugins (box, square_silo), run as sm_103a kernels.  There is no CPU path:
loading fails loudly when the shared library or a GPU is missing.

A scene is a dict:
  Nx, Ny, h           grid nodes per row / column and element size
  xmax, ymax          element-map inside bounds (default 1.0 as the reference)
  dt                  time step
  material            "isolin" | "g_local_mu2" | "g_nonlocal_mu2" | "g_nonlocal"
  props               [E, nu] (the configuration file's material properties)
  mp                  {slot: value} overrides of the material constants
  bc                  "box" | "square_silo"
  bcf, bci            boundary properties / integer properties
  gravity             None for the reference ramp, else a constant body force
  particles           dict of arrays m, v, x, y, vx, vy, sxx, sxy, syy
"""
import ctypes as C
import os

import numpy as np

import mpmg_build as _build

MATERIALS = {"isolin": 0, "g_local_mu2": 1, "g_nonlocal_mu2": 2, "g_nonlocal": 3, "dp_ri_mt": 4,
             "g_local_mu2_plane_strain": 5, "g_local_mu2_true_2d": 6,
             "g_local_mu2_ext": 7, "g_nonlocal_avg": 8, "g_local_mu2_reverse": 9,
             # plugins whose code is one of the above: g_nonlocal_bicgstab.c is g_nonlocal_avg.c,
             # g_nonlocalxs71.c is g_nonlocal.c
             "g_nonlocal_bicgstab": 8, "g_nonlocalxs71": 3}
BCS = {"box": 0, "square_silo": 1}
MP_COUNT = 16
MP = {"E": 0, "nu": 1, "mu_s": 2, "mu_2": 3, "I0": 4, "grains_rho": 5, "grains_d": 6, "A": 7,
      "rho_critical": 8, "B": 9, "cohesion": 10}
STATUS_SOLVER = 2


class MpmError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("mpm_gb300 status %d: %s" % (status, message))
        self.status = status


class Config(C.Structure):
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("h", C.c_double), ("xmax", C.c_double),
                ("ymax", C.c_double), ("dt", C.c_double), ("material", C.c_int),
                ("mp", C.c_double * MP_COUNT), ("bc", C.c_int), ("bcf", C.c_double * 4),
                ("bci", C.c_int * 4), ("gravity_mode", C.c_int), ("gravity", C.c_double),
                ("store_transients", C.c_int), ("solver_tol", C.c_double),
                ("solver_maxit", C.c_int), ("device", C.c_int), ("solver_warm_start", C.c_int),
                ("precision", C.c_int), ("scheme", C.c_int), ("solver_precond", C.c_int)]


_lib = None


class Tuning(C.Structure):
    _fields_ = [("g2p_blocks_per_sm", C.c_int), ("graph_steps", C.c_int), ("ms_per_step", C.c_double),
                ("default_ms_per_step", C.c_double), ("candidates", C.c_int), ("steps_advanced", C.c_int),
                ("p2g_elements", C.c_int), ("p2g_stage", C.c_int), ("g2p_tile", C.c_int)]


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Loads libmpm_gb300.so (building it first when missing or stale)."""
    global _lib
    if _lib is None:
        path = _build.build() if build_if_missing else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError("libmpm_gb300.so not built")
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        vp = C.c_void_p
        L.mpmg_default_params.argtypes = [C.c_int, dp]
        L.mpmg_config_init.argtypes = [C.POINTER(Config)]
        L.mpmg_create.argtypes = [C.POINTER(Config), C.c_size_t] + [dp] * 9 + [C.POINTER(vp)]
        L.mpmg_destroy.argtypes = [vp]
        L.mpmg_step.argtypes = [vp, C.c_int]
        L.mpmg_synchronize.argtypes = [vp]
        L.mpmg_get_field.argtypes = [vp, C.c_char_p, dp]
        L.mpmg_set_field.argtypes = [vp, C.c_char_p, dp]
        L.mpmg_get_fields.argtypes = [vp, C.c_int, C.POINTER(C.c_char_p), C.POINTER(dp)]
        L.mpmg_batch_create.argtypes = ([C.c_int, C.POINTER(Config), C.POINTER(C.c_size_t)] + [dp] * 9
                                        + [C.POINTER(vp)])
        L.mpmg_batch_count.argtypes = [vp, ip]
        L.mpmg_batch_member.argtypes = [vp, C.c_int] + [C.POINTER(C.c_size_t)] * 6
        L.mpmg_batch_get_time.argtypes = [vp, C.c_int, dp, ip]
        L.mpmg_write_frame.argtypes = [vp, vp, C.c_size_t, C.c_double]
        L.mpmg_write_state.argtypes = [vp, vp, C.c_double]
        L.mpmg_write_element_frame.argtypes = [vp, vp, C.c_size_t, C.c_double]
        L.mpmg_read_state.argtypes = [vp, C.POINTER(Config), C.POINTER(vp)]
        L.mpmg_adj_forward_tape.argtypes = [vp, C.c_int, C.c_int]
        L.mpmg_adj_backward.argtypes = [vp, dp, dp, dp]
        L.mpmg_autotune.argtypes = [vp, C.c_int, C.POINTER(Tuning)]
        L.mpmg_record_async.argtypes = [vp, C.c_int]
        L.mpmg_record_wait.argtypes = [vp, C.c_int, dp, ip]
        L.mpmg_adj_state.argtypes = [vp, C.c_char_p, dp]
        L.mpmg_adj_gradient.argtypes = [vp, C.c_int, dp]
        L.mpmg_record_ring.argtypes = [vp, C.c_int]
        L.mpmg_record_ring_wait.argtypes = [vp, C.c_longlong, dp, ip]
        L.mpmg_get_map.argtypes = [vp, ip, ip]
        L.mpmg_set_map.argtypes = [vp, ip, ip]
        L.mpmg_get_sort.argtypes = [vp, ip, ip, ip]
        L.mpmg_get_time.argtypes = [vp, dp, ip]
        L.mpmg_set_time.argtypes = [vp, C.c_double, C.c_int]
        L.mpmg_sizes.argtypes = [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        L.mpmg_material_only.argtypes = [vp]
        L.mpmg_get_stream.argtypes = [vp, C.POINTER(vp)]
        L.mpmg_enable_phase_timing.argtypes = [vp, C.c_int]
        L.mpmg_phase_count.argtypes = []
        L.mpmg_phase_name.argtypes = [C.c_int]
        L.mpmg_phase_name.restype = C.c_char_p
        L.mpmg_phase_times.argtypes = [vp, dp, C.POINTER(C.c_long)]
        L.mpmg_last_solve.argtypes = [vp, ip, dp]
        L.mpmg_launch_count.argtypes = [vp, C.POINTER(C.c_long), C.c_int]
        L.mpmg_status_string.argtypes = [C.c_int]
        L.mpmg_status_string.restype = C.c_char_p
        L.mpmg_last_error.argtypes = []
        L.mpmg_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        L = lib()
        raise MpmError(rc, "%s (%s)" % (L.mpmg_status_string(rc).decode(), L.mpmg_last_error().decode()))


def _libc():
    c = C.CDLL(None)
    c.fopen.restype = C.c_void_p
    c.fopen.argtypes = [C.c_char_p, C.c_char_p]
    c.fclose.argtypes = [C.c_void_p]
    return c


class _File:
    """A C FILE* for the frame and state entry points."""

    def __init__(self, path, mode):
        self.libc = _libc()
        self.fp = self.libc.fopen(str(path).encode(), mode.encode())
        if not self.fp:
            raise OSError("cannot open %s" % path)

    def __enter__(self):
        return self.fp

    def __exit__(self, *exc):
        self.libc.fclose(self.fp)


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def default_params(material):
    mp = np.zeros(MP_COUNT)
    _check(lib().mpmg_default_params(MATERIALS[material], _dptr(mp)))
    return mp


def fp64_rate(device=0):
    """Measured FP64 FMA throughput of the device in FLOP/s
    (mpmg_measure_fp64_rate)."""
    L = lib()
    L.mpmg_measure_fp64_rate.argtypes = [C.c_int, C.POINTER(C.c_double)]
    out = C.c_double()
    _check(L.mpmg_measure_fp64_rate(device, C.byref(out)))
    return out.value


PRECISIONS = {"fp64": 0, "mixed": 1, "mixed_f64node": 2}
SCHEMES = {"usl": 0, "musl": 1}
PRECONDS = {"multigrid": 0, "jacobi": 1}


def make_config(scene, store_transients=False, solver_tol=1e-10, solver_maxit=20000, device=0,
                warm_start=False, precision="fp64", precond="multigrid"):
    cfg = Config()
    _check(lib().mpmg_config_init(C.byref(cfg)))
    cfg.Nx, cfg.Ny, cfg.h = scene["Nx"], scene["Ny"], scene["h"]
    cfg.xmax, cfg.ymax = scene.get("xmax", 1.0), scene.get("ymax", 1.0)
    cfg.dt = scene["dt"]
    cfg.material = MATERIALS[scene["material"]]
    mp = default_params(scene["material"])
    props = scene.get("props")
    if props is not None:
        mp[0], mp[1] = props[0], props[1]
        if scene["material"] == "dp_ri_mt" and len(props) > 2:
            mp[MP["mu_s"]] = props[2]   # dp_ri_mt.c:73 fp64_props[2] = mu_s
    for k, val in scene.get("mp", {}).items():
        mp[MP[k] if isinstance(k, str) else k] = val
    for k in range(MP_COUNT):
        cfg.mp[k] = mp[k]
    cfg.bc = BCS[scene["bc"]]
    for k, val in enumerate(scene.get("bcf", [])):
        cfg.bcf[k] = val
    for k, val in enumerate(scene.get("bci", [])):
        cfg.bci[k] = val
    cfg.gravity_mode = 1 if scene.get("gravity") is not None else 0
    cfg.gravity = scene.get("gravity") or 0.0
    cfg.store_transients = 1 if store_transients else 0
    cfg.solver_tol = solver_tol
    cfg.solver_maxit = solver_maxit
    cfg.device = device
    cfg.solver_warm_start = 1 if warm_start else 0
    cfg.precision = PRECISIONS[precision]
    cfg.scheme = SCHEMES[scene.get("scheme", "usl")]
    cfg.solver_precond = PRECONDS[precond]
    return cfg


class Simulation:
    """One simulation resident on the GPU."""

    def __init__(self, scene, store_transients=False, solver_tol=1e-10, solver_maxit=20000, device=0,
                 warm_start=False, precision="fp64", precond="multigrid"):
        L = lib()
        cfg = make_config(scene, store_transients, solver_tol, solver_maxit, device, warm_start, precision,
                          precond)
        self.precision = precision
        p = scene["particles"]
        self.n = len(p["x"])
        arrs = [np.ascontiguousarray(p[k], dtype=np.float64)
                for k in ("m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy")]
        h = C.c_void_p()
        _check(L.mpmg_create(C.byref(cfg), self.n, *[_dptr(a) for a in arrs], C.byref(h)))
        self._h = h
        npart, nn, ne = C.c_size_t(), C.c_size_t(), C.c_size_t()
        _check(L.mpmg_sizes(self._h, C.byref(npart), C.byref(nn), C.byref(ne)))
        self.nn, self.ne = nn.value, ne.value
        self.scene = scene

    def close(self):
        if getattr(self, "_h", None):
            lib().mpmg_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def step(self, n=1):
        _check(lib().mpmg_step(self._h, n))

    def record_ring(self, slots):
        """Have every step write its record into a ring of `slots` entries in
        mapped pinned host memory (0: off); see record_ring_wait."""
        _check(lib().mpmg_record_ring(self._h, slots))

    def record_ring_wait(self, step_number):
        """(t, step_count) of step step_number's record from the ring."""
        t = C.c_double()
        k = C.c_int()
        _check(lib().mpmg_record_ring_wait(self._h, step_number, C.byref(t), C.byref(k)))
        return t.value, k.value

    def record_async(self, slot):
        """Enqueue the read-back of the step record into ring slot 0-3 (mpmg_record_async)."""
        _check(lib().mpmg_record_async(self._h, slot))

    def record_wait(self, slot):
        """(t, step count) of the record enqueued in slot (mpmg_record_wait)."""
        t = C.c_double()
        k = C.c_int()
        _check(lib().mpmg_record_wait(self._h, slot, C.byref(t), C.byref(k)))
        return t.value, k.value

    def autotune(self, steps_per_trial=16):
        """Online tuning of the mixed step's launch shape (mpmg_autotune):
        advances the simulation by the returned steps_advanced."""
        t = Tuning()
        _check(lib().mpmg_autotune(self._h, steps_per_trial, C.byref(t)))
        return {f: getattr(t, f) for f, _ in Tuning._fields_}

    def synchronize(self):
        _check(lib().mpmg_synchronize(self._h))

    def get(self, name):
        n = self.nn if name.startswith("node_") else self.n
        out = np.empty(n)
        _check(lib().mpmg_get_field(self._h, name.encode(), _dptr(out)))
        return out

    def write_frame(self, path, frame, t=None, mode="w"):
        """Append one write_frame block (the driver's particle output) to path."""
        if t is None:
            t = self.t
        with _File(path, mode) as fp:
            _check(lib().mpmg_write_frame(self._h, fp, frame, t))

    def write_element_frame(self, path, frame, t, mode="w"):
        """The driver's element frame (write_element_frame) appended or written to path."""
        with _File(path, mode) as fp:
            _check(lib().mpmg_write_element_frame(self._h, fp, frame, t))

    def write_state(self, path, t_stop=0.0):
        """The driver's state (restart) file, exact to FP64."""
        with _File(path, "w") as fp:
            _check(lib().mpmg_write_state(self._h, fp, t_stop))

    @classmethod
    def read_state(cls, path, scene, precision="fp64", device=0, store_transients=False):
        """A simulation restarted from a state file; material and boundary
        conditions come from scene (its grid and dt come from the file)."""
        cfg = make_config(scene, store_transients, device=device, precision=precision)
        h = C.c_void_p()
        with _File(path, "r") as fp:
            _check(lib().mpmg_read_state(fp, C.byref(cfg), C.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        self.precision = precision
        self.scene = scene
        npart, nn, ne = C.c_size_t(), C.c_size_t(), C.c_size_t()
        _check(lib().mpmg_sizes(self._h, C.byref(npart), C.byref(nn), C.byref(ne)))
        self.n, self.nn, self.ne = npart.value, nn.value, ne.value
        return self

    def adj_forward_tape(self, nsteps, checkpoint_every=100):
        """Advance nsteps FP64 steps keeping checkpoints for mpmg_adj_backward."""
        _check(lib().mpmg_adj_forward_tape(self._h, nsteps, checkpoint_every))

    def adj_backward(self, dl_dx, dl_dy):
        """Gradient of a loss on the taped run's final positions with respect to
        (mu_s, mu_2, I0, E, A), given dL/dx and dL/dy per particle; A is
        g_nonlocal_mu2's nonlocal amplitude (zero for the local materials)."""
        gx = np.ascontiguousarray(dl_dx, dtype=np.float64)
        gy = np.ascontiguousarray(dl_dy, dtype=np.float64)
        out = np.zeros(5)
        _check(lib().mpmg_adj_backward(self._h, _dptr(gx), _dptr(gy), _dptr(out)))
        a = C.c_double()
        _check(lib().mpmg_adj_gradient(self._h, 4, C.byref(a)))
        out[4] = a.value
        return out

    def adj_state(self, name):
        """Adjoint of one field of the taped run's initial state."""
        out = np.empty(self.n)
        _check(lib().mpmg_adj_state(self._h, name.encode(), _dptr(out)))
        return out

    def get_frame(self, names, out=None):
        """Several fields in one read-back (mpmg_get_fields): a dict name -> array.
        `out` may map names to preallocated float64 arrays (e.g. pinned host
        buffers) to fill instead."""
        names = list(names)
        arrays = {}
        for nm in names:
            if out is not None and nm in out:
                arrays[nm] = out[nm]
            else:
                arrays[nm] = np.empty(self.nn if nm.startswith("node_") else self.n)
        cnames = (C.c_char_p * len(names))(*[nm.encode() for nm in names])
        ptrs = (C.POINTER(C.c_double) * len(names))(*[_dptr(arrays[nm]) for nm in names])
        _check(lib().mpmg_get_fields(self._h, len(names), cnames, ptrs))
        return arrays

    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().mpmg_set_field(self._h, name.encode(), _dptr(a)))

    def get_map(self):
        e = np.empty(self.n, dtype=np.int32)
        a = np.empty(self.n, dtype=np.int32)
        _check(lib().mpmg_get_map(self._h, _iptr(e), _iptr(a)))
        return e, a

    def set_map(self, in_element, active):
        e = np.ascontiguousarray(in_element, dtype=np.int32)
        a = np.ascontiguousarray(active, dtype=np.int32)
        _check(lib().mpmg_set_map(self._h, _iptr(e), _iptr(a)))

    def get_sort(self):
        k = np.empty(self.n, dtype=np.int32)
        p = np.empty(self.n, dtype=np.int32)
        c = np.empty(self.ne + 1, dtype=np.int32)
        _check(lib().mpmg_get_sort(self._h, _iptr(k), _iptr(p), _iptr(c)))
        return k, p, c

    @property
    def t(self):
        t = C.c_double()
        s = C.c_int()
        _check(lib().mpmg_get_time(self._h, C.byref(t), C.byref(s)))
        return t.value

    @property
    def step_count(self):
        t = C.c_double()
        s = C.c_int()
        _check(lib().mpmg_get_time(self._h, C.byref(t), C.byref(s)))
        return s.value

    def set_time(self, t, step_number):
        _check(lib().mpmg_set_time(self._h, t, step_number))

    def material_only(self):
        _check(lib().mpmg_material_only(self._h))

    def stream(self):
        s = C.c_void_p()
        _check(lib().mpmg_get_stream(self._h, C.byref(s)))
        return s.value

    def enable_phase_timing(self, on=True):
        _check(lib().mpmg_enable_phase_timing(self._h, 1 if on else 0))

    def phase_times(self):
        L = lib()
        n = L.mpmg_phase_count()
        ms = np.zeros(n)
        cnt = (C.c_long * n)()
        _check(L.mpmg_phase_times(self._h, _dptr(ms), cnt))
        return {L.mpmg_phase_name(k).decode(): (ms[k], cnt[k]) for k in range(n)}

    def last_solve(self):
        it = C.c_int()
        r = C.c_double()
        rc = lib().mpmg_last_solve(self._h, C.byref(it), C.byref(r))
        return rc, it.value, r.value

    def launch_count(self, reset=False):
        n = C.c_long()
        _check(lib().mpmg_launch_count(self._h, C.byref(n), 1 if reset else 0))
        return n.value


class Batch(Simulation):
    """Several independent simulations in one context (mpmg_batch_create):
    one set of kernel launches steps them all.  Fields read back concatenated
    in member order; `member(k)` gives member k's slices."""

    def __init__(self, scenes, precision="mixed", device=0, store_transients=False):
        L = lib()
        count = len(scenes)
        cfgs = (Config * count)(*[make_config(sc, store_transients, device=device, precision=precision)
                                  for sc in scenes])
        counts = (C.c_size_t * count)(*[len(sc["particles"]["x"]) for sc in scenes])
        arrs = [np.ascontiguousarray(np.concatenate([np.asarray(sc["particles"][k], dtype=np.float64)
                                                     for sc in scenes]))
                for k in ("m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy")]
        h = C.c_void_p()
        _check(L.mpmg_batch_create(count, cfgs, counts, *[_dptr(a) for a in arrs], C.byref(h)))
        self._h = h
        self.precision = precision
        self.count = count
        self.scenes = list(scenes)
        self.scene = scenes[0]
        npart, nn, ne = C.c_size_t(), C.c_size_t(), C.c_size_t()
        _check(L.mpmg_sizes(self._h, C.byref(npart), C.byref(nn), C.byref(ne)))
        self.n, self.nn, self.ne = npart.value, nn.value, ne.value
        self.members = []
        for k in range(count):
            v = [C.c_size_t() for _ in range(6)]
            _check(L.mpmg_batch_member(self._h, k, *[C.byref(x) for x in v]))
            p0, np_, n0, nn_, e0, ne_ = [x.value for x in v]
            self.members.append({"particles": slice(p0, p0 + np_), "nodes": slice(n0, n0 + nn_),
                                 "elements": slice(e0, e0 + ne_)})

    def member_get(self, k, name):
        a = self.get(name)
        return a[self.members[k]["nodes" if name.startswith("node_") else "particles"]]

    def member_map(self, k):
        e, a = self.get_map()
        sl = self.members[k]["particles"]
        return e[sl], a[sl]

    def member_time(self, k):
        t = C.c_double()
        s = C.c_int()
        _check(lib().mpmg_batch_get_time(self._h, k, C.byref(t), C.byref(s)))
        return t.value, s.value

