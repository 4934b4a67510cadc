"""The contortion check and reset (solvers/utils.cpp:44-85, applied by the
reference's time loop after every step, iterator.cpp:150-151) on the GPU:
gpr_reset_contorted against the oracle and the reference's golden vectors,
and the time loops with a tolerance that triggers a reset against the
reference's own loop."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from oracle import Oracle
from phd_gb300.params import Par

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def G(cuda_ok):
    import phd_gb300
    return phd_gb300


def T(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=DEV)


def test_reset_against_golden(G):
    g = golden("contortion_v17.npz")
    MP = Par.from_array(g["mp"])
    for tol, hit in zip(g["contorted_tol"], g["contorted"]):
        q = T(g["Q"])
        assert G.solvers.contorted(q, float(tol)) == bool(hit)
        flag = G.solvers.reset_contorted(q, float(tol), [MP])
        assert int(flag.item()) == int(hit)
        ref = g["reset"] if hit else g["Q"]
        assert rel_err(q.cpu().numpy(), ref) < 1e-14
    g = golden("contortion_v15.npz")
    MPs = [Par.from_array(a) for a in g["mp"]]
    q = T(g["Q"])
    assert int(G.solvers.reset_contorted(q, 0.0, MPs).item()) == 1
    assert rel_err(q.cpu().numpy(), g["reset"]) < 1e-14


def test_loops_reset_like_the_reference(G):
    """Sheared shock tube, contorted_tol 0.02: the reference's loop resets;
    the Python driver (per-step entry points) and the device-resident
    gpr_iterate both follow it."""
    import ctypes
    from phd_gb300 import _lib
    g = golden("contortion_v17.npz")
    MP = Par.from_array(g["mp"])
    tf, tol, dX = float(g["run_tf"]), float(g["run_tol"]), list(g["run_dX"])
    ret = G.solvers.iterator(T(g["run_u0"]), tf, [200], dX, 0.8, [0, 0], False, True, False, 0,
                             MP, tol)
    assert rel_err(ret[99].cpu().numpy().reshape(g["run_u_end"].shape), g["run_u_end"]) < 1e-10
    lib = _lib.load()
    nx = np.array([200], np.int32)
    dxa = np.array(dX, np.float64)
    bca = np.array([0, 0], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles(nx.ctypes.data_as(ctypes.c_void_p), 1, 17),
                      dtype=torch.float64, device=DEV)
    ut = T(g["run_u0"].ravel())
    clk = torch.tensor([0.0, 0.0, tf, 0.8, 0.0], dtype=torch.float64, device=DEV)
    _lib.check(lib.gpr_iterate(
        ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 1,
        dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p), 0,
        ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None, ctypes.c_void_p(clk.data_ptr()),
        100, ctypes.c_void_p(scr.data_ptr()), None, tol, 17,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "iterate")
    torch.cuda.synchronize()
    assert rel_err(ut.cpu().numpy().reshape(g["run_u_end"].shape), g["run_u_end"]) < 1e-10
    # without the reset the result differs: the tolerance matters
    O = Oracle()
    u_nr, _, _ = O.run(g["run_u0"], MP, tf, dX, 0, cfl=0.8)
    assert rel_err(u_nr, g["run_u_end"]) > 1e-3


def test_two_material_loop_applies_the_reset(G):
    """The ghost-fluid loop with a tolerance that triggers on a sheared
    bubble, against one oracle step.  (After the reset every distortion is
    isotropic, where the interface Riemann states are conditioned by
    rounding, so later steps are not compared at this bar.)"""
    from phd_gb300 import problems
    from phd_gb300.ghost import MultiIterator
    O = Oracle(N=2, thermal=False, lset=1)
    u0, MPs, tf, dX, bcs = problems.shock_bubble(nx=40, ny=20, mu=1e-2, shear=0.3)
    nX = np.array(u0.shape[:2], np.int32)
    it = MultiIterator(nX, dX, 0, MPs, 0.8, 1e9, device=DEV, contorted_tol=0.02)
    ut = T(u0.ravel())
    prev, dt_prev, t = u0.copy(), 0.0, 0.0
    for s in range(1):
        it.run(ut, 1)
        t1, dt, _, _, _ = it.clock.tolist()
        ref = prev.copy()
        O.step_multi(ref, dt_prev, t, 1e9, s, MPs, dX, 0, dt=dt, contorted_tol=0.02)
        got = ut.cpu().numpy().reshape(u0.shape)
        assert rel_err(got, ref) < 1e-8, s
        prev, dt_prev, t = got, dt, t1
    A = prev[..., 5:14].reshape(-1, 3, 3)
    assert np.abs(A[:, 0, 1]).max() < 1e-2  # the shear was reset
