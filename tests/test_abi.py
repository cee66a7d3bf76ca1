"""The C ABI library without a GPU: it builds, loads, exports every entry
point its headers declare, and fails loudly (no CPU fallback) when no CUDA
device is present."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT
import mpm2d
import mpmg_build
import scenes

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"MPMG_API\s+[\w\s\*]+?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert {"mpmg_create", "mpmg_step", "mpmg_destroy", "mpmg_get_field"} <= names


def test_library_exports_every_declared_symbol():
    path = mpmg_build.build()
    lib = C.CDLL(path)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_default_params_are_the_reference_constants():
    mp = mpm2d.default_params("g_local_mu2")
    assert mp[mpm2d.MP["mu_s"]] == 0.3819 and mp[mpm2d.MP["mu_2"]] == 0.6435
    assert mp[mpm2d.MP["I0"]] == 0.278 and mp[mpm2d.MP["grains_d"]] == 0.005
    assert mp[mpm2d.MP["rho_critical"]] == 1485.0
    mp = mpm2d.default_params("dp_ri_mt")
    assert mp[mpm2d.MP["mu_s"]] == 0.3819 and mp[mpm2d.MP["rho_critical"]] == 1485.0
    mp = mpm2d.default_params("g_nonlocal")
    assert mp[mpm2d.MP["E"]] == 1e8 and mp[mpm2d.MP["B"]] == 0.9377 * 20
    assert mp[mpm2d.MP["grains_d"]] == 0.05


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_have_gpu(), reason="checks the no-GPU failure path")
def test_create_without_gpu_fails_loudly():
    with pytest.raises(mpm2d.MpmError) as e:
        mpm2d.Simulation(scenes.config1())
    assert e.value.status == 17          # MPMG_ERR_CUDA


def test_invalid_configuration_is_rejected():
    sc = scenes.config1()
    sc["Nx"] = 1
    with pytest.raises(mpm2d.MpmError) as e:
        mpm2d.Simulation(sc)
    assert e.value.status == 16          # MPMG_ERR_INVALID
    sc = scenes.config1()
    sc["bcf"] = [0.5, 0.0, 0.9, 1.0]      # box.c:88-91: box outside the unit fractions
    with pytest.raises(mpm2d.MpmError) as e:
        mpm2d.Simulation(sc)
    assert e.value.status == 16
    cfg = mpm2d.make_config(scenes.config1())
    cfg.material = 10                      # not an mpmg_material
    h = mpm2d.C.c_void_p()
    z = mpm2d.np.zeros(1)
    rc = mpm2d.lib().mpmg_create(mpm2d.C.byref(cfg), 1, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h))
    assert rc == 20 and not h.value
    cfg = mpm2d.make_config(scenes.config1())
    cfg.precision = 7                      # not an mpmg_precision
    h = mpm2d.C.c_void_p()
    z = mpm2d.np.zeros(1)
    rc = mpm2d.lib().mpmg_create(mpm2d.C.byref(cfg), 1, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h))
    assert rc == 16 and not h.value
    cfg = mpm2d.make_config(scenes.config1())
    cfg.scheme = 1
    cfg.precision = 1                      # MUSL runs in the FP64 form
    rc = mpm2d.lib().mpmg_create(mpm2d.C.byref(cfg), 1, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h))
    assert rc == 20 and not h.value


def test_batch_configuration_is_rejected():
    ens = scenes.ensemble(count=2, seed=1, cells_range=(16, 16), particles_range=(100, 200))
    cfgs = (mpm2d.Config * 2)(*[mpm2d.make_config(sc, precision="mixed") for sc in ens])
    counts = (mpm2d.C.c_size_t * 2)(*[len(sc["particles"]["x"]) for sc in ens])
    z = mpm2d.np.zeros(sum(counts))
    h = mpm2d.C.c_void_p()
    L = mpm2d.lib()
    cfgs[1].precision = 0                  # the FP64 form does not batch
    assert L.mpmg_batch_create(2, cfgs, counts, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h)) == 20
    cfgs[1].precision = 2                  # members must share the precision
    assert L.mpmg_batch_create(2, cfgs, counts, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h)) == 16
    cfgs[1].precision = 1
    cfgs[1].material = 0                   # and the material kind
    assert L.mpmg_batch_create(2, cfgs, counts, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h)) == 16
    assert L.mpmg_batch_create(0, cfgs, counts, *([mpm2d._dptr(z)] * 9), mpm2d.C.byref(h)) == 16
    assert not h.value


def test_frame_read_entry_point_is_exported():
    L = mpm2d.lib()
    assert hasattr(L, "mpmg_get_fields")
    assert mpm2d.PRECISIONS == {"fp64": 0, "mixed": 1, "mixed_f64node": 2}


def test_record_ring_and_adjoint_gradient_reject_bad_arguments():
    """The per-step record ring and the adjoint's parameter gradient check
    their arguments before touching the device."""
    L = mpm2d.lib()
    out = C.c_double()
    k = C.c_int()
    assert L.mpmg_record_ring(None, 8) == 16                  # MPMG_ERR_INVALID: no context
    assert L.mpmg_record_ring_wait(None, 1, C.byref(out), C.byref(k)) == 16
    assert L.mpmg_adj_gradient(None, 4, C.byref(out)) == 16


COPY_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_size_t)


def _ring_reader():
    fn = mpm2d.lib().mpmg_ring_read_slot
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_longlong, C.c_void_p, C.c_double, COPY_FN]
    fn.restype = C.c_int
    return fn


def _fake_slot(seq, body):
    import numpy as np
    slot = np.zeros(2 + body.size, dtype=np.int64)      # 16-byte header, then the body
    slot[0] = seq
    slot[2:] = body
    return slot


def test_ring_reader_returns_a_consistent_slot():
    import numpy as np
    fn = _ring_reader()
    body = np.arange(10, dtype=np.int64) * 7
    slot = _fake_slot(5, body)
    out = np.zeros_like(body)
    assert fn(slot.ctypes.data, body.nbytes, 5, out.ctypes.data, 1.0, COPY_FN(0)) == 0
    np.testing.assert_array_equal(out, body)


def test_ring_reader_detects_a_lap_during_the_copy():
    """A later step that starts rewriting the slot while the host copies it
    (the sequence word turns -1, then the later step number) must not be
    returned as this step's record."""
    import numpy as np
    fn = _ring_reader()
    body = np.arange(10, dtype=np.int64)
    out = np.zeros_like(body)
    for lapped_to in (-1, 5 + 32):
        slot = _fake_slot(5, body)

        def copy_then_lap(dst, src, n, slot=slot, lapped_to=lapped_to):
            C.memmove(dst, src, n)
            slot[0] = lapped_to            # the GPU reached the slot mid-copy

        cb = COPY_FN(copy_then_lap)
        assert fn(slot.ctypes.data, body.nbytes, 5, out.ctypes.data, 1.0, cb) == 16
        assert b"while it was read" in mpm2d.lib().mpmg_last_error()


def test_ring_reader_detects_an_overwritten_slot_and_times_out():
    import numpy as np
    fn = _ring_reader()
    body = np.arange(4, dtype=np.int64)
    out = np.zeros_like(body)
    slot = _fake_slot(9 + 8, body)            # already holds a later step
    assert fn(slot.ctypes.data, body.nbytes, 9, out.ctypes.data, 1.0, COPY_FN(0)) == 16
    assert b"before it was read" in mpm2d.lib().mpmg_last_error()
    slot = _fake_slot(-1, body)               # a body being written that never completes
    assert fn(slot.ctypes.data, body.nbytes, 9, out.ctypes.data, 0.05, COPY_FN(0)) == 21   # MPMG_ERR_DEVICE
    slot = _fake_slot(8, body)                # this step has not arrived
    assert fn(slot.ctypes.data, body.nbytes, 9, out.ctypes.data, 0.05, COPY_FN(0)) == 21
    assert fn(None, 8, 1, out.ctypes.data, 0.05, COPY_FN(0)) == 16
