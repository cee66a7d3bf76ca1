"""The allocation-free cell sort, mpmg_sort_cells_noalloc, for callers that
cannot call cudaMalloc (code inside a CUDA stream capture, hosts whose device
memory belongs to their own pool allocator, the reference's dlopen'd plugins).

It is checked through the C ABI against the sort every mpmg_step runs with
its own allocated scratch: the same sorted keys, permutation and element
offsets, exactly (integers), on two calls in a row over different particle
distributions, and with no change in free device memory across a call.
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
SCRATCH_LIMIT = 22          # MPMG_ERR_SCRATCH_LIMIT


def _entry():
    fn = mpm2d.lib().mpmg_sort_cells_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


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


def test_noalloc_sort_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    fn = _entry()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = buf.data_ptr()
    rc = fn(p, MAX_PARTICLES + 1, 4, p, p, p, None)
    assert rc == SCRATCH_LIMIT
    assert b"scratch" in mpm2d.lib().mpmg_last_error()
