"""The CUDA path against the oracle at the sizes the benchmark measures, not
only at test sizes: one step of the 512 x 512 Taylor-Green vortex (cs = 10,
mu = 1e-2, CFL 0.4, the headline workload) from a state a few oracle steps
in, and the device CFL time step of that state.  The bar is the smooth-data
per-step bar, max |a-b| / (1 + |b|) <= 1e-10."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import Oracle

pytestmark = pytest.mark.gpu

DEV = "cuda"


@pytest.fixture(scope="module")
def G():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import phd_gb300
    phd_gb300.load()
    return phd_gb300


def T(a, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device=DEV)


@pytest.fixture(scope="module")
def tgv512():
    """The 512 x 512 TGV (cs = 10, mu = 1e-2) after three oracle steps at
    CFL 0.4."""
    from phd_gb300 import problems
    O = Oracle()
    n = 512
    u0, MP, tf, dX, bcs = problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    u_np, steps, _ = O.run(u0, MP, 1e9, dX, [1] * 4, cfl=0.4, max_steps=3)
    assert steps == 3
    return u_np, MP, dX


def test_tgv512_step_against_oracle(G, tgv512):
    O = Oracle()
    n, cfl = 512, 0.4
    u_np, MP, dX = tgv512
    nX = np.array([n, n], np.int32)
    dt = O.timestep(u_np, dX, cfl, 0.0, 1e9, 10, MP)
    # the device time step of the same state
    u = T(u_np).view(-1)
    dt_dev = G.api.timestep_device(u, dX, cfl, 0.0, 1e9, 10, MP)
    assert abs(float(dt_dev.item()) - dt) <= 1e-14 * dt
    ub = O.boundaries(u_np, nX, [1] * 4)
    ref = u_np.reshape(-1).copy()
    O.ader_stepper(ref, ub, nX, dt, dX, MP)
    O.renorm_distortion(ref, MP)
    ubt = torch.empty(ub.size, dtype=torch.float64, device=DEV)
    G.boundaries(u, ubt, nX, [1] * 4)
    status = torch.full(((n + 2) ** 2,), -1, dtype=torch.int32, device=DEV)
    G.solvers.ader_stepper(u, ubt, nX, dt, dX, False, 0, MP, None, status=status)
    G.solvers.renorm_distortion(u, [MP])
    got = u.cpu().numpy()
    st = status.cpu().numpy()
    assert ((st & 0xff) == 0).all(), "every cell converges by Picard at CFL 0.4"
    assert rel_err(got, ref) < 1e-10, rel_err(got, ref)
    assert rel_err(got, u_np.reshape(-1)) > 1e-6  # the step moved the state


def test_tgv512_cfl08_step_against_oracle(G, tgv512):
    """The production CFL 0.8 step of the same workload: the reference's
    Picard iteration fails in most predictor cells (relaxation time 6e-4
    against dt 3.5e-4), the device Newton pass finishes them, the oracle's
    Newton fallback solves the same fixed point; the same cells take the
    stiff path and the step agrees to 1e-10."""
    O = Oracle()
    n, cfl = 512, 0.8
    u_np, MP, dX = tgv512
    nX = np.array([n, n], np.int32)
    dt = O.timestep(u_np, dX, cfl, 0.0, 1e9, 10, MP)
    ub = O.boundaries(u_np, nX, [1] * 4)
    ref = u_np.reshape(-1).copy()
    _, st_ref = O.ader_stepper(ref, ub, nX, dt, dX, MP, newton_fallback=1)
    O.renorm_distortion(ref, MP)
    newton_ref = st_ref < -1000
    assert newton_ref.mean() > 0.5, "the case must exercise the stiff path"
    assert not ((st_ref == -1) | (st_ref == -2)).any()
    u = T(u_np).view(-1)
    ubt = torch.empty(ub.size, dtype=torch.float64, device=DEV)
    G.boundaries(u, ubt, nX, [1] * 4)
    status = torch.full(((n + 2) ** 2,), -1, dtype=torch.int32, device=DEV)
    G.solvers.ader_stepper(u, ubt, nX, dt, dX, False, 0, MP, None, status=status)
    G.solvers.renorm_distortion(u, [MP])
    got = u.cpu().numpy()
    st = status.cpu().numpy()
    assert ((st & 0xff) != 2).all(), "no cell may be left unconverged"
    assert (((st & 0xff) == 1) == newton_ref).all(), "same cells take the stiff path"
    assert rel_err(got, ref) < 1e-10, rel_err(got, ref)
