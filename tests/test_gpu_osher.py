"""Osher-Solomon and Roe dissipation on the GPU (solvers/fv/fluxes.cpp:22-64)
against the golden vectors of the reference's own C++ and against the
oracle: pointwise D_OSH / D_ROE, the 1D FV stage and step with FLUX = 2,
and shock-tube runs with FLUX = 1 and 2."""
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


def test_osher_unsupported_directions_raise(G):
    g = golden("pointwise_v17.npz")
    MP = Par.from_array(g["mp_arrays"][0])
    Q = T(g["Q"][0])
    with pytest.raises(RuntimeError):
        G.solvers.fv.D_OSH(Q, Q, 1, MP)


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
