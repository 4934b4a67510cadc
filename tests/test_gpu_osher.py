"""Osher-Solomon and Roe dissipation on the GPU (solvers/fv/fluxes.cpp:22-64)
against the golden vectors of the reference's own C++ and against the
oracle: pointwise D_OSH / D_ROE along x, y and z, the 1D and 2D FV stages and
steps with FLUX = 2, shock-tube runs with FLUX = 1 and 2, and 2D steps with
FLUX = 1 and 2."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from phd_gb300.params import Par

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def G():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import phd_gb300
    return phd_gb300


def T(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=DEV)


def H(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def test_pointwise_osher_roe(G):
    """Same bar as the oracle against the reference (1e-10): the 17x17
    eigen-decomposition of the system matrix carries the reference's own
    conditioning at the 9-fold advection eigenvalue."""
    g = golden("pointwise_v17.npz")
    for m in range(g["Q"].shape[0]):
        MP = Par.from_array(g["mp_arrays"][m])
        Q, Q2 = T(g["Q"][m]), T(g["Q2"][m])
        assert rel_err(H(G.solvers.fv.D_OSH(Q, Q2, 0, MP)), g["D_OSH"][m, :, 0]) < 1e-10, m
        assert rel_err(H(G.solvers.fv.D_ROE(Q, Q2, 0, MP)), g["D_ROE"][m, :, 0]) < 1e-10, m


def test_pointwise_osher_roe_other_directions(G):
    """D_OSH / D_ROE along y and z (the x form on states with the axes
    exchanged) against the reference's own d = 1, 2 evaluations."""
    g = golden("pointwise_v17.npz")
    for m in range(g["Q"].shape[0]):
        MP = Par.from_array(g["mp_arrays"][m])
        Q, Q2 = T(g["Q"][m]), T(g["Q2"][m])
        for d in (1, 2):
            assert rel_err(H(G.solvers.fv.D_OSH(Q, Q2, d, MP)), g["D_OSH"][m, :, d]) < 1e-10
            assert rel_err(H(G.solvers.fv.D_ROE(Q, Q2, d, MP)), g["D_ROE"][m, :, d]) < 1e-10


def test_stages_osher_2d(G):
    """The reference's 2D FV stage and ADER step with FLUX = 2 (Taylor-Green
    tile, stages2d_osh_v17.npz)."""
    g = golden("stages2d_osh_v17.npz")
    assert int(g["flux"]) == 2
    MP = Par.from_array(g["mp"])
    nX = g["nX"].astype(np.int32)
    dX = list(g["dX"])
    mask = torch.ones(int(np.prod(nX + 2)), dtype=torch.bool, device=DEV)
    dt = float(g["dt"])
    G.api.set_grid(nX)
    u = T(g["u"])
    G.solvers.fv.fv_launcher(u, T(g["qh"]), nX, dt, dX, True, True, 2, MP, mask)
    assert rel_err(H(u), g["u_fv"]) < 1e-12
    u = T(g["u"])
    G.solvers.fv.interfs2(u, T(g["qh"]), int(nX[0]), int(nX[1]), dt, dX[0], dX[1], True, 2,
                          MP, mask)
    assert rel_err(H(u), g["u_interfs"]) < 1e-12
    u = T(g["u"])
    G.solvers.ader_stepper(u, T(g["ub"]), nX, dt, dX, False, 2, MP, mask)
    G.solvers.renorm_distortion(u, [MP])
    assert rel_err(H(u), g["u_step"]) < 1e-12


@pytest.mark.parametrize("flux", [1, 2])
def test_2d_osher_roe_steps_against_oracle(G, flux):
    """Three steps of the 12 x 10 Taylor-Green tile with FLUX = 1, 2 through
    the device-resident iterator against the oracle."""
    import ctypes
    from oracle import Oracle
    from phd_gb300 import _lib, problems
    u0, MP, tf, dX, bcs = problems.taylor_green(n=12, ny=10, cs=10.0, mu=1.0)
    O = Oracle()
    ref, _, _ = O.run(u0, MP, 1e9, dX, 1, cfl=0.4, flux=flux, max_steps=3)
    lib = _lib.load()
    nx = np.array([12, 10], np.int32)
    dxa = np.array(dX, np.float64)
    bca = np.array([1, 1, 1, 1], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles(nx.ctypes.data_as(ctypes.c_void_p), 2, 17),
                      dtype=torch.float64, device=DEV)
    ut = T(u0.ravel())
    clk = torch.tensor([0.0, 0.0, 1e9, 0.4, 0.0], dtype=torch.float64, device=DEV)
    _lib.check(lib.gpr_iterate(
        ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 2,
        dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p), flux,
        ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None, ctypes.c_void_p(clk.data_ptr()),
        3, ctypes.c_void_p(scr.data_ptr()), None, float("inf"), 17,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "iterate")
    assert rel_err(H(ut).reshape(ref.shape), ref) < 1e-10


def test_stages_osher_1d(G):
    g = golden("stages1d_osh_v17.npz")
    assert int(g["flux"]) == 2
    MP = Par.from_array(g["mp"])
    nX = g["nX"].astype(np.int32)
    dX = list(g["dX"])
    ncb = int(nX[0] + 2)
    mask = torch.ones(ncb, dtype=torch.bool, device=DEV)
    dt = float(g["dt"])
    G.api.set_grid(nX)
    u = T(g["u"])
    G.solvers.fv.fv_launcher(u, T(g["qh"]), nX, dt, dX, True, True, 2, MP, mask)
    assert rel_err(H(u), g["u_fv"]) < 1e-12
    u = T(g["u"])
    G.solvers.fv.interfs1(u, T(g["qh"]), int(nX[0]), dt, dX[0], True, 2, MP, mask)
    assert rel_err(H(u), g["u_interfs"]) < 1e-12
    u = T(g["u"])
    G.solvers.ader_stepper(u, T(g["ub"]), nX, dt, dX, False, 2, MP, mask)
    G.solvers.renorm_distortion(u, [MP])
    assert rel_err(H(u), g["u_step"]) < 1e-12


@pytest.mark.parametrize("flux,steps", [(2, 40), (1, 20)])
def test_shock_tube_osher_roe_against_oracle(G, flux, steps):
    """Config 1 with FLUX = 2 (and Roe) through the shock: per-step bar
    1e-8 through shocks; compared after `steps` steps of the iterator."""
    from oracle import Oracle
    from phd_gb300 import problems
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=200)
    ref, n, t = Oracle().run(u0, MP, tf, dX, 0, cfl=0.8, flux=flux, max_steps=steps)
    u = T(u0).view(-1)
    ret = G.solvers.iterator(u, tf, [200], dX, 0.8, [0, 0], False, True, False, flux, [MP],
                             max_steps=steps)
    got = H(ret[99]).reshape(ref.shape)
    assert rel_err(got, ref) < 1e-8, rel_err(got, ref)
