"""The allocation-free 1D ADER step (gpr_ader_stepper_1d_noalloc).

It exists for callers that cannot allocate device memory (an application
owning the device through its own fixed pool, or a loop where an allocation
would synchronise the device): its scratch is a fixed array inside the
library.  Called through the C ABI, it must give the same result as the
allocating entry point gpr_ader_stepper on calls in a row (each later call on
another grid, material, flux or layout, so contents left in the shared array
by an earlier call cannot leak into it): at the largest grid it accepts
(GPR_NOALLOC_MAX_CELLS cells), with the status output and the stiff Newton
predictor, with the Osher flux, and for the V = 15 (level set) layout.  It
must reject grids beyond its fixed size with GPR_E_TOO_LARGE.  This file is
collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

MAX_CELLS = 4096  # GPR_NOALLOC_MAX_CELLS in include/gpr_gb300.h


def _case(nx, mu, steps, cs=1.0):
    from oracle import Oracle
    from phd_gb300 import problems
    O = Oracle()
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=nx, mu=mu, cs=cs)
    u, _, _ = O.run(u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=steps)
    dt = O.timestep(u, dX, 0.8, 0.0, 1e9, steps, MP)
    ub = O.boundaries(u, [nx], [0, 0])
    return u.ravel().copy(), ub.ravel().copy(), MP, dt, dX[0], 17


def _case15(nx):
    """A V = 15 state (viscous, level set): the 1D helium-bubble layout; the
    ghost cells come from the library's own boundary fill."""
    from phd_gb300 import _lib, problems
    lib = _lib.load()
    u0, MPs, tf, dX, bcs = problems.helium_bubble_1d(nx=nx, shear=0.2)
    ub = torch.empty((nx + 4) * 15, dtype=torch.float64, device="cuda")
    u = torch.tensor(u0.ravel(), dtype=torch.float64, device="cuda")
    nX = np.array([nx], np.int32)
    bc = np.array([0, 0], np.int32)
    assert lib.gpr_boundaries(ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(ub.data_ptr()),
                              nX.ctypes.data_as(ctypes.c_void_p), 1,
                              bc.ctypes.data_as(ctypes.c_void_p), 15,
                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    torch.cuda.synchronize()
    return u0.ravel().copy(), ub.cpu().numpy(), MPs[0], 2e-4, dX[0], 15


def _run_both(lib, nx, u, ub, MP, dt, dx, V, flux=0, stiff=0):
    dev = "cuda"
    par = MP.to_ctypes()
    pp = ctypes.cast(ctypes.pointer(par), ctypes.c_void_p)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ub_d = torch.tensor(ub, dtype=torch.float64, device=dev)
    ncb = nx + 2
    # allocating entry point with caller scratch
    u_ref = torch.tensor(u, dtype=torch.float64, device=dev)
    st_ref = torch.full((ncb,), -7, dtype=torch.int32, device=dev)
    nX = np.array([nx], np.int32)
    dX = np.array([dx], np.float64)
    nscr = lib.gpr_ader_scratch_doubles(nX.ctypes.data_as(ctypes.c_void_p), 1, V)
    scr = torch.empty(nscr, dtype=torch.float64, device=dev)
    rc = lib.gpr_ader_stepper(ctypes.c_void_p(u_ref.data_ptr()), ctypes.c_void_p(ub_d.data_ptr()),
                              nX.ctypes.data_as(ctypes.c_void_p), 1, dt,
                              dX.ctypes.data_as(ctypes.c_void_p), stiff, flux, pp, None,
                              ctypes.c_void_p(scr.data_ptr()), ctypes.c_void_p(st_ref.data_ptr()),
                              V, stream)
    assert rc == 0
    # allocation-free entry point
    u_na = torch.tensor(u, dtype=torch.float64, device=dev)
    st_na = torch.full((ncb,), -7, dtype=torch.int32, device=dev)
    rc = lib.gpr_ader_stepper_1d_noalloc(ctypes.c_void_p(u_na.data_ptr()),
                                         ctypes.c_void_p(ub_d.data_ptr()), nx, dt, dx, stiff,
                                         flux, pp, None, ctypes.c_void_p(st_na.data_ptr()), V,
                                         stream)
    assert rc == 0
    torch.cuda.synchronize()
    return (u_na.cpu().numpy(), u_ref.cpu().numpy(), st_na.cpu().numpy(),
            st_ref.cpu().numpy())


def test_noalloc_matches_allocating_step_in_a_row():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300 import _lib
    lib = _lib.load()
    cases = [
        # (label, case builder, flux, stiff)
        ("200 cells", lambda: _case(200, 1e-2, 20), 0, 0),
        ("96 cells, other material", lambda: _case(96, 3e-3, 7), 0, 0),
        ("largest grid", lambda: _case(MAX_CELLS, 1e-2, 3), 0, 0),
        ("stiff Newton predictor", lambda: _case(64, 1e-4, 3, cs=5.0), 0, 1),
        ("Osher flux", lambda: _case(80, 1e-2, 10), 2, 0),
        ("V = 15 layout", lambda: _case15(120), 0, 0),
    ]
    for label, make, flux, stiff in cases:
        u, ub, MP, dt, dx, V = make()
        nx = u.size // V
        got, ref, st, st_ref = _run_both(lib, nx, u, ub, MP, dt, dx, V, flux=flux, stiff=stiff)
        assert np.isfinite(got).all(), label
        assert rel_err(got, ref) < 1e-13, (label, rel_err(got, ref))
        assert rel_err(got, u) > 0.0, label  # the step did change the state
        # the status output is forwarded: every predictor cell written, alike
        assert (st != -7).all() and (st == st_ref).all(), label
        if stiff:
            assert ((st & 0xff) == 1).all(), label  # Newton finished every cell


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
                                         MAX_CELLS + 1, 1e-3, 1e-3, 0, 0, pp, None, None, 17,
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -4  # GPR_E_TOO_LARGE, checked on the host before any launch
