"""ctypes access to the oracle (test infrastructure, not the product).

``Oracle`` wraps oracle/_build/liboracle.so, the CPU restatement of the
reference's USL step.  ``RefHarness`` wraps oracle/_ref/libref_harness.so,
which drives the reference's own compiled libmpm and plugins; it exists only
where the reference tree was available to build it.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

MATERIALS = {"isolin": 0, "g_local_mu2": 1, "g_nonlocal_mu2": 2, "g_nonlocal": 3, "dp_ri_mt": 4,
             "g_local_mu2_plane_strain": 5, "g_local_mu2_true_2d": 6,
             "g_local_mu2_ext": 7, "g_nonlocal_avg": 8, "g_local_mu2_reverse": 9,
             # plugins whose code is one of the above: g_nonlocal_bicgstab.c is g_nonlocal_avg.c,
             # g_nonlocalxs71.c is g_nonlocal.c
             "g_nonlocal_bicgstab": 8, "g_nonlocalxs71": 3}
BCS = {"box": 0, "square_silo": 1}
# material parameter slots by name (enum orc_mparam)
MP = {"E": 0, "nu": 1, "mu_s": 2, "mu_2": 3, "I0": 4, "grains_rho": 5, "grains_d": 6, "A": 7,
      "rho_critical": 8, "B": 9, "cohesion": 10}
MP_COUNT = 16
PARTICLE_FIELDS = ["x", "y", "xl", "yl", "v", "v0", "m", "vx", "vy", "ax", "ay", "bx", "by",
                   "sxx", "sxy", "syy", "ux", "uy", "exx", "exy", "eyy", "wxy",
                   "Txx", "Txy", "Tyx", "Tyy", "Tzz"] + ["state%d" % k for k in range(11)]
NODE_FIELDS = ["node_m", "node_mx", "node_my", "node_fx", "node_fy", "node_vx", "node_vy",
               "node_ax", "node_ay", "node_gf"]


class OrcConfig(C.Structure):
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("h", C.c_double), ("xmax", C.c_double),
                ("ymax", C.c_double), ("dt", C.c_double), ("material", C.c_int),
                ("mp", C.c_double * MP_COUNT), ("bc", C.c_int), ("bcf", C.c_double * 4),
                ("bci", C.c_int * 4), ("gravity_mode", C.c_int), ("gravity", C.c_double),
                ("nthreads", C.c_int), ("solver", C.c_int), ("cg_tol", C.c_double),
                ("cg_maxit", C.c_int), ("scheme", C.c_int)]

SCHEMES = {"usl": 0, "musl": 1}


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.orc_default_params.argtypes = [C.c_int, dp]
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcConfig), C.c_size_t] + [dp] * 9
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_step.restype = C.c_int
        L.orc_material_only.argtypes = [C.c_void_p]
        L.orc_material_only.restype = C.c_int
        L.orc_get_field.argtypes = [C.c_void_p, C.c_char_p, dp]
        L.orc_get_field.restype = C.c_long
        L.orc_set_field.argtypes = [C.c_void_p, C.c_char_p, dp]
        L.orc_set_field.restype = C.c_long
        ip = C.POINTER(C.c_int)
        L.orc_get_map.argtypes = [C.c_void_p, ip, ip]
        L.orc_set_map.argtypes = [C.c_void_p, ip, ip]
        L.orc_time.argtypes = [C.c_void_p]
        L.orc_time.restype = C.c_double
        L.orc_set_time.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.orc_num_particles.argtypes = [C.c_void_p]
        L.orc_num_particles.restype = C.c_size_t
        L.orc_num_nodes.argtypes = [C.c_void_p]
        L.orc_num_nodes.restype = C.c_size_t
        sp = C.POINTER(C.c_size_t)
        L.orc_get_color_lists.argtypes = [C.c_void_p, sp, sp]
        L.orc_get_elements.argtypes = [C.c_void_p, ip, ip, dp]
        L.orc_last_solve.argtypes = [C.c_void_p, ip, dp]
        L.orc_last_solve.restype = C.c_int
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def default_params(material):
    mp = np.zeros(MP_COUNT)
    lib().orc_default_params(MATERIALS[material], _dptr(mp))
    return mp


class Oracle:
    """One simulation in the CPU restatement."""

    def __init__(self, scene, nthreads=1, solver="direct", cg_tol=1e-10, cg_maxit=100000):
        L = lib()
        cfg = OrcConfig()
        cfg.Nx, cfg.Ny, cfg.h = scene["Nx"], scene["Ny"], scene["h"]
        cfg.xmax, cfg.ymax = scene.get("xmax", 1.0), scene.get("ymax", 1.0)
        cfg.dt = scene["dt"]
        cfg.material = MATERIALS[scene["material"]]
        mp = default_params(scene["material"])
        props = scene.get("props")
        if props is not None:
            mp[0], mp[1] = props[0], props[1]
            if scene["material"] == "dp_ri_mt" and len(props) > 2:
                mp[2] = props[2]   # dp_ri_mt.c:73 fp64_props[2] = mu_s
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
        cfg.nthreads = nthreads
        cfg.solver = 0 if solver == "direct" else 1
        cfg.cg_tol = cg_tol
        cfg.cg_maxit = cg_maxit
        cfg.scheme = SCHEMES[scene.get("scheme", "usl")]
        p = scene["particles"]
        self.n = len(p["x"])
        arrs = [np.ascontiguousarray(p[k], dtype=np.float64)
                for k in ("m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy")]
        self._h = L.orc_create(C.byref(cfg), self.n, *[_dptr(a) for a in arrs])
        if not self._h:
            raise ValueError("orc_create rejected the configuration")
        self.nn = L.orc_num_nodes(self._h)
        self.ne = (cfg.Nx - 1) * (cfg.Ny - 1)
        self.nthreads = nthreads

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_destroy(h)
            self._h = None

    def step(self, n=1):
        return lib().orc_step(self._h, n)

    def material_only(self):
        return lib().orc_material_only(self._h)

    @property
    def t(self):
        return lib().orc_time(self._h)

    def set_time(self, t, step_number=0):
        lib().orc_set_time(self._h, t, step_number)

    def get(self, name):
        n = self.nn if name.startswith("node_") else self.n
        out = np.empty(n)
        if lib().orc_get_field(self._h, name.encode(), _dptr(out)) < 0:
            raise KeyError(name)
        return out

    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        if lib().orc_set_field(self._h, name.encode(), _dptr(a)) < 0:
            raise KeyError(name)

    def get_map(self):
        e = np.empty(self.n, dtype=np.int32)
        a = np.empty(self.n, dtype=np.int32)
        lib().orc_get_map(self._h, _iptr(e), _iptr(a))
        return e, a

    def set_map(self, in_element, active):
        e = np.ascontiguousarray(in_element, dtype=np.int32)
        a = np.ascontiguousarray(active, dtype=np.int32)
        lib().orc_set_map(self._h, _iptr(e), _iptr(a))

    def color_lists(self):
        out = np.empty(max(self.n, 1), dtype=np.uint64)
        lens = np.empty(self.nthreads * 4, dtype=np.uint64)
        lib().orc_get_color_lists(self._h, out.ctypes.data_as(C.POINTER(C.c_size_t)),
                                  lens.ctypes.data_as(C.POINTER(C.c_size_t)))
        return out, lens

    def elements(self):
        f = np.empty(self.ne, dtype=np.int32)
        c = np.empty(self.ne, dtype=np.int32)
        m = np.empty(self.ne)
        lib().orc_get_elements(self._h, _iptr(f), _iptr(c), _dptr(m))
        return f, c, m

    def last_solve(self):
        it = C.c_int()
        r = C.c_double()
        st = lib().orc_last_solve(self._h, C.byref(it), C.byref(r))
        return st, it.value, r.value


REFH_FIELDS = ["x", "y", "xl", "yl", "v", "m", "vx", "vy", "ax", "ay", "bx", "by",
               "sxx", "sxy", "syy", "ux", "uy", "exx", "exy", "eyy", "wxy",
               "Txx", "Txy", "Tyx", "Tyy", "Tzz"] + ["state%d" % k for k in range(11)]
REFH_NODE_FIELDS = ["node_m", "node_mx", "node_my", "node_fx", "node_fy", "node_vx",
                    "node_vy", "node_ax", "node_ay"]

_ref = {}


def ref_available():
    return os.path.isfile(os.path.join(_build.REF_OUT, "libref_harness.so")) or _build.have_reference()


def ref_lib(lib_dir=None):
    """The harness library of the reference build in lib_dir (default the
    bit-exact build in oracle/_ref; oracle/_ref/perf holds the build with the
    reference's release flags, loaded in a process of its own)."""
    lib_dir = lib_dir or _build.REF_OUT
    if lib_dir not in _ref:
        path = os.path.join(lib_dir, "libref_harness.so")
        if not os.path.isfile(path):
            if _build.build_ref() is None:
                raise RuntimeError("reference build unavailable")
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.refh_create.restype = C.c_void_p
        L.refh_create.argtypes = [C.c_int, C.c_double, C.c_size_t, dp, C.c_char_p, dp,
                                  C.c_size_t, C.c_char_p, dp, C.c_size_t, ip, C.c_size_t,
                                  C.c_double, C.c_int]
        L.refh_step.argtypes = [C.c_void_p, C.c_int]
        L.refh_set_scheme.argtypes = [C.c_void_p, C.c_int]
        L.refh_time.argtypes = [C.c_void_p]
        L.refh_time.restype = C.c_double
        L.refh_get_particles.argtypes = [C.c_void_p, dp, ip, ip]
        L.refh_get_nodes.argtypes = [C.c_void_p, dp]
        L.refh_get_elements.argtypes = [C.c_void_p, ip, ip, dp]
        sp = C.POINTER(C.c_size_t)
        L.refh_get_color_lists.argtypes = [C.c_void_p, sp, sp]
        L.refh_destroy.argtypes = [C.c_void_p]
        L.refh_write.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_size_t, C.c_double]
        L.refh_write.restype = C.c_int
        _ref[lib_dir] = L
    return _ref[lib_dir]


class RefHarness:
    """One simulation in the reference's own compiled code (square N x N grid,
    unit-square element map, compile-time material constants, reference
    gravity ramp)."""

    def __init__(self, scene, nthreads=1, lib_dir=None):
        self._lib_dir = lib_dir or _build.REF_OUT
        L = ref_lib(self._lib_dir)
        assert scene["Nx"] == scene["Ny"], "the reference grid is N x N"
        assert scene.get("gravity") is None, "the reference ramps gravity"
        p = scene["particles"]
        self.n = len(p["x"])
        pin = np.ascontiguousarray(np.stack(
            [np.asarray(p[k], dtype=np.float64) for k in
             ("m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy")], axis=1))
        mprops = np.ascontiguousarray(scene.get("props", [1e6, 0.3]), dtype=np.float64)
        bprops = np.ascontiguousarray(scene.get("bcf", []), dtype=np.float64)
        biprops = np.ascontiguousarray(scene.get("bci", []), dtype=np.int32)
        mat_so = os.path.join(self._lib_dir, scene["material"] + ".so").encode()
        bc_so = os.path.join(self._lib_dir, scene["bc"] + ".so").encode()
        self._keep = (pin, mprops, bprops, biprops, mat_so, bc_so)
        self._h = L.refh_create(scene["Nx"], scene["h"], self.n, _dptr(pin), mat_so,
                                _dptr(mprops), len(mprops), bc_so, _dptr(bprops), len(bprops),
                                _iptr(biprops), len(biprops), scene["dt"], nthreads)
        if self._h:
            L.refh_set_scheme(self._h, SCHEMES[scene.get("scheme", "usl")])
        if not self._h:
            raise RuntimeError("refh_create failed")
        self.N = scene["Nx"]
        self.nthreads = nthreads

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            ref_lib(self._lib_dir).refh_destroy(h)
            self._h = None

    def step(self, n=1):
        ref_lib(self._lib_dir).refh_step(self._h, n)

    def write(self, path, what, frame=0, time=0.0):
        """The reference's writer on the job: what = "frame" (write_frame),
        "element_frame" (write_element_frame) or "state" (write_state)."""
        code = {"frame": 0, "element_frame": 1, "state": 2}[what]
        if ref_lib(self._lib_dir).refh_write(self._h, path.encode(), code, frame, time) != 0:
            raise RuntimeError("refh_write could not open %s" % path)

    @property
    def t(self):
        return ref_lib(self._lib_dir).refh_time(self._h)

    def particles(self):
        out = np.empty((self.n, len(REFH_FIELDS)))
        e = np.empty(self.n, dtype=np.int32)
        a = np.empty(self.n, dtype=np.int32)
        ref_lib(self._lib_dir).refh_get_particles(self._h, _dptr(out), _iptr(e), _iptr(a))
        d = {k: out[:, i].copy() for i, k in enumerate(REFH_FIELDS)}
        d["in_element"] = e
        d["active"] = a
        return d

    def nodes(self):
        nn = self.N * self.N
        out = np.empty((nn, len(REFH_NODE_FIELDS)))
        ref_lib(self._lib_dir).refh_get_nodes(self._h, _dptr(out))
        return {k: out[:, i].copy() for i, k in enumerate(REFH_NODE_FIELDS)}

    def elements(self):
        ne = (self.N - 1) ** 2
        f = np.empty(ne, dtype=np.int32)
        c = np.empty(ne, dtype=np.int32)
        m = np.empty(ne)
        ref_lib(self._lib_dir).refh_get_elements(self._h, _iptr(f), _iptr(c), _dptr(m))
        return f, c, m

    def color_lists(self):
        out = np.empty(max(self.n, 1), dtype=np.uint64)
        lens = np.empty(self.nthreads * 4, dtype=np.uint64)
        ref_lib(self._lib_dir).refh_get_color_lists(self._h, out.ctypes.data_as(C.POINTER(C.c_size_t)),
                                       lens.ctypes.data_as(C.POINTER(C.c_size_t)))
        return out, lens
