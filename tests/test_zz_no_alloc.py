"""The allocation-free cell sort, mpmg_sort_cells_noalloc, for callers that
cannot call cudaMalloc (hosts whose device memory belongs to their own pool
allocator, the reference's dlopen'd plugins, which own no device memory).

It is checked through the C ABI against the sort every mpmg_step runs with
its own allocated scratch: the same sorted keys, permutation and element
offsets, exactly (integers), on two calls in a row over different particle
distributions, and with no change in free device memory across a call.  The
radix sort behind it runs one pass for up to 10 key bits, two up to 20 and
three beyond; each pass count is compared with numpy's stable argsort, with
keys outside [0, num_elements] (which count as outside the grid) mixed in.
This file is collected last so that a run stopping at the first failure has
run every other test already; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import mpm2d
import scenes

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 20     # MPMG_NOALLOC_MAX_PARTICLES
INVALID = 16                # MPMG_ERR_INVALID
SCRATCH_LIMIT = 22          # MPMG_ERR_SCRATCH_LIMIT


def _entry():
    fn = mpm2d.lib().mpmg_sort_cells_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _call(torch, fn, keys, ne):
    """One call on device copies of keys; returns (sorted keys, perm, starts)."""
    n = keys.size
    d_keys = torch.from_numpy(keys.astype(np.int32)).cuda()
    out_keys = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    out_perm = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    out_start = torch.full((ne + 1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = fn(d_keys.data_ptr(), n, ne, out_keys.data_ptr(), out_perm.data_ptr(), out_start.data_ptr(),
            stream.cuda_stream)
    assert rc == 0, mpm2d.lib().mpmg_last_error().decode()
    torch.cuda.synchronize()
    return out_keys.cpu().numpy()[:n], out_perm.cpu().numpy()[:n], out_start.cpu().numpy()


def _expected(keys, ne):
    k = np.where((keys < 0) | (keys > ne), ne, keys).astype(np.int64)
    perm = np.argsort(k, kind="stable")
    starts = np.searchsorted(k[perm], np.arange(ne + 1), side="left")
    return k[perm].astype(np.int32), perm.astype(np.int32), starts.astype(np.int32)


def test_noalloc_sort_matches_step_sort_on_two_calls():
    torch = pytest.importorskip("torch")
    fn = _entry()
    sc = scenes.column(Nx=129, Ny=129, h=1 / 128, width=0.3, height=0.6, material="g_local_mu2",
                       jitter=2e-3, seed=11)
    sim = mpm2d.Simulation(sc)
    n, ne = sim.n, sim.ne
    stream = torch.cuda.current_stream()
    free_between = []
    for steps in (1, 60):
        sim.step(steps)
        e, a = sim.get_map()
        want_keys, want_perm, want_start = sim.get_sort()
        keys = np.where(a == 1, e, ne).astype(np.int32)
        d_keys = torch.from_numpy(keys).cuda()
        out_keys = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        out_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        out_start = torch.full((ne + 1,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = fn(d_keys.data_ptr(), n, ne, out_keys.data_ptr(), out_perm.data_ptr(),
                out_start.data_ptr(), stream.cuda_stream)
        assert rc == 0, mpm2d.lib().mpmg_last_error().decode()
        torch.cuda.synchronize()
        free_between.append((free_before, torch.cuda.mem_get_info()[0]))
        np.testing.assert_array_equal(out_keys.cpu().numpy(), want_keys)
        np.testing.assert_array_equal(out_perm.cpu().numpy(), want_perm)
        np.testing.assert_array_equal(out_start.cpu().numpy(), want_start)
    # the second call (scratch address already set up) changes no device memory
    assert free_between[1][0] == free_between[1][1]
    sim.close()


@pytest.mark.parametrize("ne,n", [(900, 20000),            # 10 key bits: one radix pass
                                  (262144, 300000),        # 19 bits: two passes
                                  (1200000, MAX_PARTICLES)])  # 21 bits: three passes
def test_noalloc_sort_every_pass_count_against_stable_argsort(ne, n):
    torch = pytest.importorskip("torch")
    fn = _entry()
    rng = np.random.default_rng(ne)
    for call in range(2):
        keys = rng.integers(0, ne, size=n).astype(np.int64)
        # runs of equal keys, as binned particles have, and keys that mark a
        # particle outside the grid: the marker itself, the reference's -1,
        # other negatives and keys beyond the marker
        keys[: n // 4] = np.sort(keys[: n // 4])
        odd = rng.choice(n, size=max(n // 50, 1), replace=False)
        keys[odd] = rng.choice(np.array([ne, -1, -12345, ne + 1, 2**31 - 1]), size=odd.size)
        got = _call(torch, fn, keys.astype(np.int32), ne)
        want = _expected(keys, ne)
        for g, w, name in zip(got, want, ("sorted keys", "perm", "cell start")):
            np.testing.assert_array_equal(g, w, err_msg="%s, call %d" % (name, call))


def test_noalloc_sort_in_place_keys():
    """d_sorted_keys may be d_keys itself: the sort reads its own clamped copy."""
    torch = pytest.importorskip("torch")
    fn = _entry()
    ne, n = 5000, 70000
    keys = np.random.default_rng(3).integers(-2, ne + 3, size=n).astype(np.int32)
    d = torch.from_numpy(keys).cuda()
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    start = torch.empty(ne + 1, dtype=torch.int32, device="cuda")
    rc = fn(d.data_ptr(), n, ne, d.data_ptr(), perm.data_ptr(), start.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    assert rc == 0, mpm2d.lib().mpmg_last_error().decode()
    torch.cuda.synchronize()
    want = _expected(keys, ne)
    np.testing.assert_array_equal(d.cpu().numpy(), want[0])
    np.testing.assert_array_equal(perm.cpu().numpy(), want[1])
    np.testing.assert_array_equal(start.cpu().numpy(), want[2])


def test_noalloc_sort_captured_in_a_cuda_graph():
    """A call captured into a CUDA graph, after one warm-up call outside
    capture (which looks the scratch address up), and replayed twice over
    new keys in the same input buffer: each replay equals numpy's stable
    argsort.  Only kernel launches go into the graph."""
    torch = pytest.importorskip("torch")
    fn = _entry()
    rng = np.random.default_rng(5)
    ne, n = 5000, 60000
    d_keys = torch.empty(n, dtype=torch.int32, device="cuda")
    out_keys = torch.empty(n, dtype=torch.int32, device="cuda")
    out_perm = torch.empty(n, dtype=torch.int32, device="cuda")
    out_start = torch.empty(ne + 1, dtype=torch.int32, device="cuda")
    args = lambda s: (d_keys.data_ptr(), n, ne, out_keys.data_ptr(), out_perm.data_ptr(),
                      out_start.data_ptr(), s)
    d_keys.copy_(torch.from_numpy(rng.integers(0, ne, size=n).astype(np.int32)))
    assert fn(*args(torch.cuda.current_stream().cuda_stream)) == 0, mpm2d.lib().mpmg_last_error().decode()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rc = fn(*args(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, mpm2d.lib().mpmg_last_error().decode()
    for replay in range(2):
        keys = rng.integers(-2, ne + 3, size=n).astype(np.int32)
        keys[: n // 3] = np.sort(keys[: n // 3])
        d_keys.copy_(torch.from_numpy(keys))
        for t in (out_keys, out_perm, out_start):
            t.fill_(-7)
        graph.replay()
        torch.cuda.synchronize()
        want = _expected(keys, ne)
        for g, w, name in zip((out_keys, out_perm, out_start), want, ("sorted keys", "perm", "cell start")):
            np.testing.assert_array_equal(g.cpu().numpy(), w, err_msg="%s, replay %d" % (name, replay))


def test_noalloc_sort_rejects_bad_sizes():
    torch = pytest.importorskip("torch")
    fn = _entry()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = buf.data_ptr()
    rc = fn(p, MAX_PARTICLES + 1, 4, p, p, p, None)
    assert rc == SCRATCH_LIMIT
    assert b"scratch" in mpm2d.lib().mpmg_last_error()
    assert fn(p, 4, 1 << 30, p, p, p, None) == INVALID
    assert fn(p, 4, 0, p, p, p, None) == INVALID
