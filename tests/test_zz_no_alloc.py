"""tfv_hydro_step_static: the step for callers that cannot allocate.

Some hosts own every byte of GPU memory through a pool of their own, or run
the step where the device synchronisation of cudaMalloc is not acceptable.
For them the library keeps the step's scratch in a fixed 1 MiB array of its
own device memory.  These tests call that entry point through the C ABI, two
times in a row with different inputs and then in a chain of grids of other
sizes and dimensions, and require exactly the output of tfv_hydro_step with a
caller-provided workspace (the double-precision path is bit-exact throughout
this suite, so the tolerance here is zero as well).  They also check that
repeated calls leave the device's free memory unchanged.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from torch_gb300 import _lib  # noqa: E402
from torch_gb300.session import make_config  # noqa: E402


def rough_state(seed, shape):
    rng = np.random.default_rng(seed)
    p = np.empty((len(shape) + 2,) + shape)
    p[0] = 0.5 + rng.random(shape)
    p[1:-1] = 0.6 * (rng.random((len(shape),) + shape) - 0.5)
    p[-1] = 0.5 + rng.random(shape)
    s = p.copy()
    s[1:-1] *= p[0]
    s[-1] = p[-1] / 0.4 + 0.5 * p[0] * np.sum(p[1:-1] ** 2, axis=0)
    return s


def config_for(shape, bcs, limiter):
    dim = len(shape)
    counts = list(shape[::-1])
    return make_config(dim, counts, [1.0] * dim, bcs, t_end=1.0, cfl=0.4, gamma=1.4,
                       limiter=limiter, max_steps=1)


def face_buffers(u, dim, fluxes=True):
    out = []
    for k in range(dim if fluxes else 0):
        shape = list(u.shape)
        shape[dim - k] += 1
        out.append(torch.empty(shape, dtype=u.dtype, device=u.device))
    return out + [None] * (3 - len(out))


def step_with_workspace(cfg, u, dt, stream, fluxes=True):
    lib = _lib.load()
    ws = C.c_size_t()
    _lib.check(lib.tfv_step_workspace_size(C.byref(cfg), _lib.TFV_FP64, C.byref(ws)))
    work = torch.empty(ws.value + 256, dtype=torch.uint8, device=u.device)
    wp = work.data_ptr() + ((-work.data_ptr()) % 256)
    out = torch.empty_like(u)
    fl = face_buffers(u, cfg.dim, fluxes)
    used = C.c_int32()
    _lib.check(lib.tfv_hydro_step(C.byref(cfg), _lib.TFV_FP64, _lib.ptr(u), _lib.ptr(out), None,
                                  dt, *[_lib.ptr(f) for f in fl], C.c_void_p(wp), C.byref(used),
                                  _lib.stream_ptr(stream)))
    return out, fl, used.value


def stable_dt(shape):
    """A dt well inside the CFL limit of rough_state on a unit box (wave
    speeds below 2.5)."""
    return 0.05 / max(shape)


def static_call(cfg, u, out, fl, stream):
    """One call of the entry point into buffers the caller already holds."""
    lib = _lib.load()
    used = C.c_int32()
    _lib.check(lib.tfv_hydro_step_static(C.byref(cfg), _lib.TFV_FP64, _lib.ptr(u),
                                         _lib.ptr(out), None, stable_dt(u.shape[1:]),
                                         *[_lib.ptr(f) for f in fl], C.byref(used),
                                         _lib.stream_ptr(stream)))
    return used.value


def step_static(cfg, u, dt, stream, fluxes=True):
    lib = _lib.load()
    out = torch.empty_like(u)
    fl = face_buffers(u, cfg.dim, fluxes)
    used = C.c_int32()
    _lib.check(lib.tfv_hydro_step_static(C.byref(cfg), _lib.TFV_FP64, _lib.ptr(u),
                                         _lib.ptr(out), None, dt, *[_lib.ptr(f) for f in fl],
                                         C.byref(used), _lib.stream_ptr(stream)))
    return out, fl, used.value


# Calls of different sizes and dimensions through the one shared array, the
# largest first: a call must never read what a differently laid out earlier
# call left there (tile table, per-tile sums, tensor maps, the 1D tube's
# per-cell interface data).
CHAIN = [((40, 36, 33), ("Open", "Reflective", "Periodic"), "Superbee", 11, True),
         ((12, 20, 33), ("Periodic", "Open", "Reflective"), "VanLeer", 12, True),
         ((96, 80), ("Reflective", "Open"), "MINBEE", 13, True),
         ((3001,), ("Open",), "VanLeer", 14, False),
         ((12, 20, 33), ("Open", "Open", "Open"), "Albada", 15, True)]


def test_static_scratch_step_matches_workspace_step_twice_in_a_row():
    stream = torch.cuda.Stream()
    cases = [((12, 20, 33), ("Open", "Reflective", "Periodic"), "Superbee", 11),
             ((12, 20, 33), ("Periodic", "Open", "Reflective"), "VanLeer", 12)]
    for shape, bcs, limiter, seed in cases:
        u = torch.as_tensor(rough_state(seed, shape), device="cuda")
        cfg = config_for(shape, bcs, limiter)
        dt = 2e-3
        got, got_f, got_fb = step_static(cfg, u, dt, stream)
        want, want_f, want_fb = step_with_workspace(cfg, u, dt, stream)
        stream.synchronize()
        assert got_fb == want_fb
        assert torch.equal(got, want)
        for a, b in zip(got_f, want_f):
            if a is not None:
                assert torch.equal(a, b)


def test_static_scratch_calls_of_other_layouts_in_a_chain():
    stream = torch.cuda.Stream()
    for shape, bcs, limiter, seed, fluxes in CHAIN:
        u = torch.as_tensor(rough_state(seed, shape), device="cuda")
        cfg = config_for(shape, bcs, limiter)
        dt = stable_dt(shape)
        got, got_f, got_fb = step_static(cfg, u, dt, stream, fluxes)
        want, want_f, want_fb = step_with_workspace(cfg, u, dt, stream, fluxes)
        stream.synchronize()
        assert got_fb == want_fb, shape
        assert torch.equal(got, want), shape
        for a, b in zip(got_f, want_f):
            if a is not None:
                assert torch.equal(a, b), shape


def test_static_scratch_calls_take_no_device_memory():
    """After one round of warm-up calls (which load the kernels), further
    calls leave the device's free memory exactly where it was."""
    stream = torch.cuda.Stream()
    held = []
    for shape, bcs, limiter, seed, fluxes in CHAIN:
        u = torch.as_tensor(rough_state(seed, shape), device="cuda")
        held.append((config_for(shape, bcs, limiter), u, torch.empty_like(u),
                     face_buffers(u, len(shape), fluxes)))
    for cfg, u, out, fl in held:
        static_call(cfg, u, out, fl, stream)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for cfg, u, out, fl in held:
            static_call(cfg, u, out, fl, stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_static_scratch_rejects_grids_beyond_its_limit():
    lib = _lib.load()
    cfg = config_for((1024, 1024, 1024), ("Open",) * 3, "MINBEE")
    code = lib.tfv_hydro_step_static(C.byref(cfg), _lib.TFV_FP64, C.c_void_p(16), C.c_void_p(16),
                                     None, 1e-3, None, None, None, None, None)
    assert code == _lib.TFV_EINVAL
    assert "scratch" in _lib.last_error()
