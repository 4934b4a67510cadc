"""The allocation-free 1D ADER step (gpr_ader_stepper_1d_noalloc).

It exists for callers that cannot allocate device memory (an application
owning the device through its own fixed pool, or a loop where an allocation
would synchronise the device): its scratch is a fixed array inside the
library.  Called through the C ABI, it must give the same result as the
allocating entry point gpr_ader_stepper on two calls in a row (the second
call on a different grid and material, so contents left in the shared array
by the first call cannot leak into it), and it must reject grids beyond its
fixed size with GPR_E_TOO_LARGE.  This file is collected last so that a run
stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _case(nx, mu, steps):
    from oracle import Oracle
    from phd_gb300 import problems
    O = Oracle()
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=nx, mu=mu)
    u, _, _ = O.run(u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=steps)
    dt = O.timestep(u, dX, 0.8, 0.0, 1e9, steps, MP)
    ub = O.boundaries(u, [nx], [0, 0])
    return u.ravel().copy(), ub, MP, dt, dX[0]


def _run_both(lib, nx, u, ub, MP, dt, dx):
    dev = "cuda"
    V = 17
    par = MP.to_ctypes()
    pp = ctypes.cast(ctypes.pointer(par), ctypes.c_void_p)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ub_d = torch.tensor(ub, dtype=torch.float64, device=dev)
    # allocating entry point with caller scratch
    u_ref = torch.tensor(u, dtype=torch.float64, device=dev)
    nX = np.array([nx], np.int32)
    dX = np.array([dx], np.float64)
    nscr = lib.gpr_ader_scratch_doubles(nX.ctypes.data_as(ctypes.c_void_p), 1, V)
    scr = torch.empty(nscr, dtype=torch.float64, device=dev)
    rc = lib.gpr_ader_stepper(ctypes.c_void_p(u_ref.data_ptr()), ctypes.c_void_p(ub_d.data_ptr()),
                              nX.ctypes.data_as(ctypes.c_void_p), 1, dt,
                              dX.ctypes.data_as(ctypes.c_void_p), 0, 0, pp, None,
                              ctypes.c_void_p(scr.data_ptr()), None, V, stream)
    assert rc == 0
    # allocation-free entry point
    u_na = torch.tensor(u, dtype=torch.float64, device=dev)
    rc = lib.gpr_ader_stepper_1d_noalloc(ctypes.c_void_p(u_na.data_ptr()),
                                         ctypes.c_void_p(ub_d.data_ptr()), nx, dt, dx, 0, 0,
                                         pp, None, None, V, stream)
    assert rc == 0
    torch.cuda.synchronize()
    return u_na.cpu().numpy(), u_ref.cpu().numpy()


def test_noalloc_matches_allocating_step_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300 import _lib
    lib = _lib.load()
    # first call: 200-cell tube; second call: a smaller grid, other material
    for nx, mu, steps in ((200, 1e-2, 20), (96, 3e-3, 7)):
        u, ub, MP, dt, dx = _case(nx, mu, steps)
        got, ref = _run_both(lib, nx, u, ub, MP, dt, dx)
        assert np.isfinite(got).all()
        assert rel_err(got, ref) < 1e-13, (nx, rel_err(got, ref))
        assert rel_err(got, u) > 0.0  # the step did change the state


def test_noalloc_rejects_grids_beyond_its_fixed_size():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300 import _lib
    from phd_gb300.params import material_params
    lib = _lib.load()
    MP = material_params("sg", 1.0, cv=2.5, gamma=1.4, b0=1.0, calpha=1.0, mu=1e-2, Pr=2 / 3)
    par = MP.to_ctypes()
    pp = ctypes.cast(ctypes.pointer(par), ctypes.c_void_p)
    u = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.gpr_ader_stepper_1d_noalloc(ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(u.data_ptr()),
                                         4097, 1e-3, 1e-3, 0, 0, pp, None, None, 17,
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -4  # GPR_E_TOO_LARGE, checked on the host before any launch
