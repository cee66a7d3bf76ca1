"""The exported phase functions of the threaded step (libmpm/process_usl.h:15-22).

Each phase runs on the GPU over the job's host arrays.  The test builds a job
through the library's own mpm_init (the config-1 block, 65^2 nodes), fills
random particle and node state (a few inactive particles, a few massless
nodes), calls each phase over sub-ranges, and compares the host arrays with
a numpy restatement of the reference's lines: bit for bit, except the
volume update's exp (1 ulp).
"""
import ctypes as C

import numpy as np
import pytest

import mpm2d
import scenes

D, I, Z, P = C.c_double, C.c_int, C.c_size_t, C.c_void_p


class Particle(C.Structure):
    _fields_ = [("x", D), ("y", D), ("xl", D), ("yl", D), ("v", D), ("v0", D), ("s", D * 4), ("m", D),
                ("x_t", D), ("y_t", D), ("x_tt", D), ("y_tt", D), ("bx", D), ("by", D), ("sxx", D),
                ("sxy", D), ("syy", D), ("T", D * 9), ("exx_t", D), ("exy_t", D), ("eyy_t", D),
                ("wxy_t", D), ("L", D * 9), ("Fxx", D), ("Fxy", D), ("Fyx", D), ("Fyy", D), ("ux", D),
                ("uy", D), ("color", D), ("state", D * 11), ("material", I), ("grad_s", D * 8),
                ("element", I), ("real_sxx", D), ("real_sxy", D), ("real_syy", D), ("real_state", D * 11),
                ("r1_initial", D * 2), ("r2_initial", D * 2), ("r1", D * 2), ("r2", D * 2),
                ("corners", D * 8), ("cornersl", D * 8), ("sc", D * 16), ("grad_sc", D * 32),
                ("corner_elements", I * 4), ("material_data", P), ("id", Z)]


class Node(C.Structure):
    _fields_ = [("num_filled_element_neighbors", I), ("mass_filled_element_neighbors", D), ("m", D),
                ("x", D), ("y", D), ("ux", D), ("uy", D), ("x_t", D), ("y_t", D), ("x_tt", D), ("y_tt", D),
                ("mx_t", D), ("my_t", D), ("mx_tt", D), ("my_tt", D), ("fx", D), ("fy", D), ("rho", D),
                ("velocity_update_flag", I)]


class Element(C.Structure):
    _fields_ = [("color", I), ("color_idx", I), ("nodes", I * 4), ("n", I), ("m", D), ("filled", I),
                ("neighbors", I * 8), ("grad_x", D), ("grad_y", D), ("grad_mag", D), ("n_x", D), ("n_y", D),
                ("n_theta", D), ("v", D), ("p_index", I), ("p_dist", D), ("sxx", D), ("sxy", D), ("syy", D),
                ("exx_t", D), ("exy_t", D), ("eyy_t", D), ("wxy_t", D), ("p", D), ("tau", D),
                ("kku_element", D * 144), ("f_element", D * 12), ("jacobian", D * 4)]


class TimestepControl(C.Structure):
    _fields_ = [("dt_max", D), ("dt_min", D), ("dt", D), ("automatic_dt", I), ("allow_dt_increase", I),
                ("stable_dt_threshold", I)]


class ImplicitControl(C.Structure):
    _fields_ = [("du_norm_ratio", D), ("q_norm_ratio", D), ("du_norm_converged", D),
                ("unstable_iteration_count", I), ("stable_step_count", I)]


class OutputControl(C.Structure):
    _fields_ = [(k, P) for k in ("directory", "user", "particle_filename", "element_filename", "state_filename",
                                 "log_filename", "particle_filename_fullpath", "element_filename_fullpath",
                                 "state_filename_fullpath", "log_filename_fullpath", "particle_fd",
                                 "element_fd", "state_fd", "log_fd", "info_fd", "job_name",
                                 "job_description")] + \
               [("job_id", I), ("date", P), ("override_directory_with_id", I), ("prepend_date", I),
                ("modified_directory", I), ("sample_rate_hz", D)]


class MaterialControl(C.Structure):
    _fields_ = [("material_filename", P), ("use_builtin", I), ("material_init", P), ("calculate_stress", P),
                ("calculate_stress_threaded", P), ("fp64_props", P), ("int_props", P),
                ("num_fp64_props", Z), ("num_int_props", Z)]


class BoundaryControl(C.Structure):
    _fields_ = [("bc_filename", P), ("use_builtin", I), ("bc_init", P), ("bc_validate", P),
                ("bc_time_varying", P), ("bc_momentum", P), ("bc_force", P), ("fp64_props", P),
                ("int_props", P), ("num_fp64_props", Z), ("num_int_props", Z)]


class Job(C.Structure):
    _fields_ = [("t", D), ("dt", D), ("t_stop", D), ("frame", Z), ("stepcount", I), ("num_particles", Z),
                ("num_nodes", Z), ("num_elements", Z), ("num_colors", Z), ("color_indices", P),
                ("particle_by_element_color_lengths", C.POINTER(Z)),
                ("particle_by_element_color_lists", C.POINTER(C.POINTER(Z))), ("N", Z), ("h", D),
                ("use_cpdi", I), ("tic", C.c_long * 2), ("toc", C.c_long * 2), ("nodes", C.POINTER(Node)),
                ("particles", C.POINTER(Particle)), ("elements", C.POINTER(Element)),
                ("in_element", C.POINTER(I)), ("active", C.POINTER(I))] + \
               [(k, C.POINTER(D)) for k in ("h1", "h2", "h3", "h4", "b11", "b12", "b13", "b14",
                                            "b21", "b22", "b23", "b24")] + \
               [("node_u_map", P), ("inv_node_u_map", P), ("u_dirichlet", P), ("u_dirichlet_mask", P),
                ("node_number_override", P), ("vec_len", I), ("solver", I), ("timestep", TimestepControl),
                ("implicit", ImplicitControl), ("output", OutputControl), ("material", MaterialControl),
                ("boundary", BoundaryControl), ("step_number", I), ("step_start_time", D),
                ("step_barrier", P), ("serialize_barrier", P), ("num_threads", Z),
                ("update_elementlists", C.POINTER(I)), ("update_elementlists_flag", P)]


class Task(C.Structure):
    _fields_ = [("id", Z), ("num_threads", Z), ("gidx_min", Z), ("gidx_max", Z), ("offset", Z), ("blocksize", Z),
                ("n_offset", Z), ("n_blocksize", Z), ("e_offset", Z), ("e_blocksize", Z), ("stride", Z),
                ("job", C.POINTER(Job))]


SF = ("h1", "h2", "h3", "h4", "b11", "b12", "b13", "b14", "b21", "b22", "b23", "b24")


def test_layouts_match_the_header():
    assert C.sizeof(Particle) == 1280 and C.sizeof(Node) == 152 and C.sizeof(Element) == 1504
    assert C.sizeof(Job) == 800 and C.sizeof(Task) == 96
    assert Job.in_element.offset == 176 and Job.h1.offset == 192
    assert Job.material.offset == 584 and Job.boundary.offset == 656
    assert Particle.T.offset == 160 and Particle.state.offset == 392


@pytest.fixture(scope="module")
def job():
    L = mpm2d.lib()
    L.mpm_init.restype = C.POINTER(Job)
    L.mpm_init.argtypes = [I, D, C.POINTER(Particle), Z, D]
    for name in ("move_grid_split", "calculate_shapefunctions_split", "calculate_strainrate_split",
                 "move_particles_explicit_usl_split", "update_particle_densities_split"):
        getattr(L, name).argtypes = [C.POINTER(Job), Z, Z]
    L.map_to_grid_explicit_split.argtypes = [C.POINTER(Job), Z]
    L.create_particle_to_element_map_threaded.argtypes = [C.POINTER(Task)]
    L.find_filled_elements.argtypes = [C.POINTER(Job)]
    L.mpm_cleanup.argtypes = [C.POINTER(Job)]
    sc = scenes.config1(seed=0)
    p = sc["particles"]
    n = len(p["x"])
    rng = np.random.default_rng(7)
    arr = (Particle * n)()
    for i in range(n):
        q = arr[i]
        q.x, q.y, q.m, q.v = p["x"][i], p["y"][i], p["m"][i], p["v"][i]
        q.x_t, q.y_t, q.x_tt, q.y_tt = rng.normal(size=4)
        q.bx, q.by = rng.normal(size=2)
        q.sxx, q.sxy, q.syy = rng.normal(size=3) * 1e3
        q.ux, q.uy = rng.normal(size=2) * 1e-3
        q.exx_t, q.exy_t, q.eyy_t = rng.normal(size=3) * 10
    J = L.mpm_init(65, 1.0 / 64, arr, n, 0.0)
    j = J.contents
    j.dt = 1e-5
    T = 2
    j.num_threads = T
    lengths = (Z * (4 * T))()
    lists = (C.POINTER(Z) * (4 * T))()
    keep = []
    for k in range(4 * T):
        buf = (Z * (n + 1))()
        keep.append(buf)
        lists[k] = C.cast(buf, C.POINTER(Z))
    j.particle_by_element_color_lengths = C.cast(lengths, C.POINTER(Z))
    j.particle_by_element_color_lists = C.cast(lists, C.POINTER(C.POINTER(Z)))
    upd = (I * T)()
    j.update_elementlists = C.cast(upd, C.POINTER(I))
    for i in rng.choice(n, 20, replace=False):
        j.active[int(i)] = 0
    L.find_filled_elements(J)
    nn = j.num_nodes
    for k in range(nn):
        d = j.nodes[k]
        d.m = abs(rng.normal()) + 0.01
        d.fx, d.fy, d.mx_t, d.my_t, d.x_t, d.y_t, d.mx_tt, d.my_tt = rng.normal(size=8)
        d.ux, d.uy = rng.normal(size=2)
    yield L, J, n, rng, keep, lengths, lists, upd, arr
    L.mpm_cleanup(J)


def particles(j, n, *fields):
    return [np.array([getattr(j.particles[i], f) for i in range(n)]) for f in fields]


def nodes(j, *fields):
    return [np.array([getattr(j.nodes[k], f) for k in range(j.num_nodes)]) for f in fields]


def shape_arrays(j, n):
    return {k: np.ctypeslib.as_array(getattr(j, k), shape=(n,)).copy() for k in SF}


def elem_nodes(j, n):
    ie = np.ctypeslib.as_array(j.in_element, shape=(n,))
    return np.array([list(j.elements[e].nodes) if e >= 0 else [0, 0, 0, 0] for e in ie])


def active(j, n):
    return np.ctypeslib.as_array(j.active, shape=(n,)).copy() != 0


@pytest.mark.gpu
def test_shapefunctions(job):
    L, J, n, *_ = job
    j = J.contents
    before = shape_arrays(j, n)
    L.calculate_shapefunctions_split(J, 0, n // 3)
    L.calculate_shapefunctions_split(J, n // 3, n)
    act = active(j, n)
    x, y, xl_got, yl_got = particles(j, n, "x", "y", "xl", "yl")
    en = elem_nodes(j, n)
    xn = np.array([j.nodes[int(k)].x for k in en[:, 0]])
    yn = np.array([j.nodes[int(k)].y for k in en[:, 0]])
    h = j.h

    def local(v, r):     # particle.c:14-30
        l = (v - r) / h
        sg = np.copysign(1.0, l)
        snap = (sg * l > 1.0) & ((sg * l - 1.0) < 1e-10)
        return np.where(snap, sg, l)

    xl, yl = local(x, xn), local(y, yn)
    ox, oy = 1 - xl, 1 - yl
    d = 1.0 / h
    want = {"h1": ox * oy, "h2": xl * oy, "h3": xl * yl, "h4": ox * yl,
            "b11": -oy * d, "b12": oy * d, "b13": yl * d, "b14": -yl * d,
            "b21": -ox * d, "b22": -xl * d, "b23": xl * d, "b24": ox * d}
    got = shape_arrays(j, n)
    for k in SF:
        np.testing.assert_array_equal(got[k][act], want[k][act], err_msg=k)
        np.testing.assert_array_equal(got[k][~act], before[k][~act], err_msg=k)
    np.testing.assert_array_equal(xl_got[act], xl[act])
    np.testing.assert_array_equal(yl_got[act], yl[act])


@pytest.mark.gpu
def test_strainrate(job):
    L, J, n, *_ = job
    j = J.contents
    L.calculate_shapefunctions_split(J, 0, n)
    old = particles(j, n, "exx_t", "exy_t", "eyy_t", "wxy_t")
    L.calculate_strainrate_split(J, 0, 1000)
    L.calculate_strainrate_split(J, 1000, n)
    act = active(j, n)
    sf = shape_arrays(j, n)
    en = elem_nodes(j, n)
    xt = np.array([[j.nodes[int(k)].x_t for k in row] for row in en])
    yt = np.array([[j.nodes[int(k)].y_t for k in row] for row in en])

    def smear(a, v):      # process_usl.c:53-58, left to right
        return ((a[0] * v[:, 0] + a[1] * v[:, 1]) + a[2] * v[:, 2]) + a[3] * v[:, 3]

    b1 = [sf["b11"], sf["b12"], sf["b13"], sf["b14"]]
    b2 = [sf["b21"], sf["b22"], sf["b23"], sf["b24"]]
    dxtdy, dytdx = smear(b2, xt), smear(b1, yt)
    want = [smear(b1, xt), 0.5 * (dxtdy + dytdx), smear(b2, yt), 0.5 * (dxtdy - dytdx)]
    got = particles(j, n, "exx_t", "exy_t", "eyy_t", "wxy_t")
    for g, w, o in zip(got, want, old):
        np.testing.assert_array_equal(g[act], w[act])
        np.testing.assert_array_equal(g[~act], o[~act])


@pytest.mark.gpu
def test_map_to_grid_in_the_references_order(job):
    L, J, n, *_ = job
    j = J.contents
    L.calculate_shapefunctions_split(J, 0, n)
    fields = ("m", "mx_t", "my_t", "mx_tt", "my_tt", "fx", "fy")
    want = {f: a.copy() for f, a in zip(fields, nodes(j, *fields))}
    sf = shape_arrays(j, n)
    pf = dict(zip(("m", "x_t", "y_t", "x_tt", "y_tt", "bx", "by", "sxx", "sxy", "syy", "v"),
                  particles(j, n, "m", "x_t", "y_t", "x_tt", "y_tt", "bx", "by", "sxx", "sxy", "syy", "v")))
    T, Cn = j.num_threads, j.num_colors
    ie = np.ctypeslib.as_array(j.in_element, shape=(n,))
    for c in range(Cn):                      # process_usl.c:849-906: colour, thread, list order
        for t in range(T):
            tc = t * Cn + c
            for q in range(j.particle_by_element_color_lengths[tc]):
                p = j.particle_by_element_color_lists[tc][q]
                nl = list(j.elements[int(ie[p])].nodes)
                m = pf["m"][p]
                pdata = [m, pf["x_t"][p] * m, pf["y_t"][p] * m, pf["x_tt"][p] * m, pf["y_tt"][p] * m,
                         pf["bx"][p] * m, pf["by"][p] * m]
                s = [sf["h1"][p], sf["h2"][p], sf["h3"][p], sf["h4"][p]]
                for k in range(4):             # map.c:85-104, list47
                    for f, v in zip(fields, pdata):
                        want[f][nl[k]] += s[k] * v
                sd = [-pf["sxx"][p] * pf["v"][p], -pf["sxy"][p] * pf["v"][p], -pf["syy"][p] * pf["v"][p]]
                for off, b in ((0, ("b11", "b12", "b13", "b14")), (1, ("b21", "b22", "b23", "b24"))):
                    for k in range(4):         # list42 with &stressdata[off]
                        want["fx"][nl[k]] += sf[b[k]][p] * sd[off]
                        want["fy"][nl[k]] += sf[b[k]][p] * sd[off + 1]
    L.map_to_grid_explicit_split(J, 0)
    for f, g in zip(fields, nodes(j, *fields)):
        np.testing.assert_array_equal(g, want[f], err_msg=f)


@pytest.mark.gpu
def set_masses(j, rng):
    """Some massless nodes and some at exactly the threshold (TOL = 1e-10):
    move_grid_split treats those as massless, move_particles_explicit_usl_split
    does not (process_usl.c:604, :925)."""
    nn = j.num_nodes
    for k in rng.choice(nn, 40, replace=False):
        j.nodes[int(k)].m = 0.0
    for k in rng.choice(nn, 10, replace=False):
        j.nodes[int(k)].m = 1e-10


@pytest.mark.gpu
def test_move_grid(job):
    L, J, n, rng, *_ = job
    j = J.contents
    nn = j.num_nodes
    set_masses(j, rng)
    m, fx, fy, mx, my, ux, uy, xt, yt, xtt, ytt = nodes(j, "m", "fx", "fy", "mx_t", "my_t", "ux", "uy", "x_t",
                                                      "y_t", "x_tt", "y_tt")
    L.move_grid_split(J, 0, nn // 2)
    L.move_grid_split(J, nn // 2, nn)
    dt = j.dt
    on = m > 1e-10
    mx2 = np.where(on, mx + dt * fx, mx)
    my2 = np.where(on, my + dt * fy, my)
    with np.errstate(divide="ignore", invalid="ignore"):
        want = {"x_tt": np.where(on, fx / m, 0.0), "y_tt": np.where(on, fy / m, 0.0), "mx_t": mx2, "my_t": my2,
                "x_t": np.where(on, mx2 / m, 0.0), "y_t": np.where(on, my2 / m, 0.0)}
    want["ux"] = np.where(on, dt * want["x_t"], ux)
    want["uy"] = np.where(on, dt * want["y_t"], uy)
    for f, g in zip(want, nodes(j, *want)):
        np.testing.assert_array_equal(g, want[f], err_msg=f)


@pytest.mark.gpu
def test_move_particles(job):
    L, J, n, rng, *_ = job
    j = J.contents
    set_masses(j, rng)
    L.calculate_shapefunctions_split(J, 0, n)
    act = active(j, n)
    sf = shape_arrays(j, n)
    en = elem_nodes(j, n)
    nf = {f: a for f, a in zip(("m", "fx", "fy", "mx_t", "my_t"), nodes(j, "m", "fx", "fy", "mx_t", "my_t"))}
    xt, yt, x, y, ux, uy = particles(j, n, "x_t", "y_t", "x", "y", "ux", "uy")
    L.move_particles_explicit_usl_split(J, 0, 2048)
    L.move_particles_explicit_usl_split(J, 2048, n)
    dt = j.dt
    s = [sf["h1"], sf["h2"], sf["h3"], sf["h4"]]
    xtt = np.zeros(n)
    ytt = np.zeros(n)
    dux = np.zeros(n)
    duy = np.zeros(n)
    for k in range(4):                        # process_usl.c:923-944
        m = nf["m"][en[:, k]]
        use = m >= 1e-10
        with np.errstate(divide="ignore", invalid="ignore"):
            xtt = np.where(use, xtt + (s[k] * nf["fx"][en[:, k]]) / m, xtt)
            ytt = np.where(use, ytt + (s[k] * nf["fy"][en[:, k]]) / m, ytt)
    for k in range(4):
        m = nf["m"][en[:, k]]
        use = m >= 1e-10
        with np.errstate(divide="ignore", invalid="ignore"):
            dux = np.where(use, dux + (s[k] * nf["mx_t"][en[:, k]]) / m, dux)
            duy = np.where(use, duy + (s[k] * nf["my_t"][en[:, k]]) / m, duy)
    dux, duy = dux * dt, duy * dt
    want = [xtt, ytt, xt + dt * xtt, yt + dt * ytt, x + dux, y + duy, ux + dux, uy + duy]
    old = [None, None, xt, yt, x, y, ux, uy]
    got = particles(j, n, "x_tt", "y_tt", "x_t", "y_t", "x", "y", "ux", "uy")
    for g, w, o in zip(got, want, old):
        np.testing.assert_array_equal(g[act], w[act])
        if o is not None:
            np.testing.assert_array_equal(g[~act], o[~act])


@pytest.mark.gpu
def test_densities(job):
    L, J, n, *_ = job
    j = J.contents
    act = active(j, n)
    v, exx, eyy = particles(j, n, "v", "exx_t", "eyy_t")
    L.update_particle_densities_split(J, 0, n)
    want = v * np.exp(j.dt * (exx + eyy))     # process_usl.c:961-970
    got = particles(j, n, "v")[0]
    np.testing.assert_allclose(got[act], want[act], rtol=2.3e-16, atol=0)
    np.testing.assert_array_equal(got[~act], v[~act])


@pytest.mark.gpu
def test_element_map(job):
    L, J, n, rng, keep, lengths, lists, upd, arr = job
    j = J.contents
    moved = rng.choice(n, 50, replace=False)
    for i in moved[:40]:
        j.particles[int(i)].x = float(rng.uniform(0, 1))
    for i in moved[40:]:
        j.particles[int(i)].y = 1.5          # outside the grid
    ie0 = np.ctypeslib.as_array(j.in_element, shape=(n,)).copy()
    act0 = active(j, n)
    x, y = particles(j, n, "x", "y")
    h, N = j.h, j.N
    inside = (x < 1.0) & (x >= 0.0) & (y < 1.0) & (y >= 0.0)
    want = np.where(inside, (np.floor(x / h) + np.floor(y / h) * (N - 1)), -1).astype(np.int64)
    T = 2
    for t in range(T):
        task = Task()
        task.id, task.num_threads = t, T
        task.offset = t * (n // T)
        task.blocksize = n // T if t < T - 1 else n - t * (n // T)
        task.job = J
        L.create_particle_to_element_map_threaded(C.byref(task))
        lo, hi = task.offset, task.offset + task.blocksize
        ch = np.any((want[lo:hi] != ie0[lo:hi]) & act0[lo:hi])
        assert upd[t] == int(ch)
    ie = np.ctypeslib.as_array(j.in_element, shape=(n,))
    np.testing.assert_array_equal(ie[act0], want[act0])
    np.testing.assert_array_equal(ie[~act0], ie0[~act0])
    np.testing.assert_array_equal(active(j, n), act0 & (want != -1))
