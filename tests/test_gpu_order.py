"""The 1D and 2D step at N = 3 Gauss nodes (the reference's third-order
scheme) through the C ABI, against the reference's golden N = 3 stages and
the N = 3 oracle, and the same kernels at N = 2 against the N = 2 library.

Bars (max |a-b| / (1+|b|)): stages 1e-13, except the WENO reconstruction,
which at N = 3 adds the central stencil with weight 1e5 and epsilon 1e-14:
on the nearly constant states of a shock tube the reference itself moves by
~1e-8 under a one-ulp change of its input, so the reconstruction (and a step
or run through it) is held at 1e-7."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from oracle import Oracle
from phd_gb300.params import Par

pytestmark = pytest.mark.gpu

DEV = "cuda"


@pytest.fixture(scope="module")
def G3():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300.order import for_order
    return for_order(3)


def T(a, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device=DEV)


def H(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def test_n3_stages_against_golden(G3):
    g = golden("stages1d_rus_v17n3.npz")
    MP = Par.from_array(g["mp"])
    nX, dX = [int(g["nX"][0])], list(g["dX"])
    nx = nX[0]
    dt = float(g["dt"])
    u = T(g["u"])
    ub = torch.full((g["ub"].size,), np.nan, dtype=torch.float64, device=DEV)
    G3.boundaries(u, ub, nX, [int(g["bcs"])] * 2)
    assert rel_err(H(ub), g["ub"]) == 0.0
    wh = torch.full((g["wh"].size,), np.nan, dtype=torch.float64, device=DEV)
    G3.solvers.weno.weno_launcher(wh, T(g["ub"]), nX)
    assert rel_err(H(wh), g["wh"]) < 1e-7
    qh = torch.full((g["qh"].size,), np.nan, dtype=torch.float64, device=DEV)
    mask = torch.ones(nx + 2, dtype=torch.bool, device=DEV)
    status = torch.full((nx + 2,), -1, dtype=torch.int32, device=DEV)
    G3.solvers.dg.predictor(qh, T(g["wh"]), dt, dX, False, False, MP, mask, status=status)
    assert ((H(status) & 0xff) == 0).all()
    assert rel_err(H(qh), g["qh"]) < 1e-13
    ufv = T(g["u"])
    G3.solvers.fv.fv_launcher(ufv, T(g["qh"]), nX, dt, dX, True, True, 0, MP, mask)
    assert rel_err(H(ufv), g["u_fv"]) < 1e-14
    ust = T(g["u"])
    G3.solvers.ader_stepper(ust, T(g["ub"]), nX, dt, dX, False, 0, MP, mask)
    import phd_gb300
    phd_gb300.solvers.renorm_distortion(ust, [MP])
    assert rel_err(H(ust), g["u_step"]) < 1e-7


def test_n3_stages_against_oracle(G3):
    """On a state with structure everywhere (a shock tube after 30 oracle
    steps): WENO to the conditioning bar, predictor, FV update and one full
    step from the oracle's inputs to 1e-13."""
    from phd_gb300 import problems
    O = Oracle(N=3)
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=128)
    u_np, _, _ = O.run(u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=30)
    nX = np.array([128], np.int32)
    dt = O.timestep(u_np, dX, 0.8, 0.0, 1e9, 30, MP)
    ub = O.boundaries(u_np, nX, [0, 0])
    wh = O.weno_launcher(ub, nX)
    wh_d = torch.empty(wh.size, dtype=torch.float64, device=DEV)
    G3.solvers.weno.weno_launcher(wh_d, T(ub), nX)
    assert rel_err(H(wh_d), wh) < 1e-7
    qh, st = O.predictor(wh, dt, dX, nX, MP, newton_fallback=0)
    assert (st > 0).all()
    qh_d = torch.empty(qh.size, dtype=torch.float64, device=DEV)
    status = torch.full((130,), -1, dtype=torch.int32, device=DEV)
    G3.solvers.dg.predictor(qh_d, T(wh), dt, dX, False, False, MP, None, status=status, nX=nX)
    assert rel_err(H(qh_d), qh) < 1e-13
    assert ((H(status) >> 8) == st).all(), "the same Picard iteration counts"
    ref = u_np.ravel().copy()
    O.fv_launcher(ref, qh, nX, dt, dX, MP)
    u = T(u_np).view(-1)
    G3.solvers.fv.fv_launcher(u, T(qh), nX, dt, dX, True, True, 0, MP, None)
    assert rel_err(H(u), ref) < 1e-13


def test_n3_shock_tube_run_against_oracle(G3):
    """60 steps of the 200-cell shock tube at N = 3 through the device loop
    (CFL time step, boundaries, step, renorm, contortion check on the
    device clock) against the oracle's loop.  The bar is the reference
    scheme's own rounding sensitivity on this run, measured here: the oracle
    rerun from the initial state times (1 + 1e-16 xi) moves by ~5e-7 after
    60 steps (the central WENO stencil on the tube's nearly constant states);
    the device run must stay within 10x that."""
    from phd_gb300 import problems
    O = Oracle(N=3)
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=200)
    ref, n, t = O.run(u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=60, contorted_tol=1.0)
    rng = np.random.default_rng(1)
    resp = 0.0
    for _ in range(2):
        up = u0 * (1 + 1e-16 * rng.standard_normal(u0.shape))
        r2, _, _ = O.run(up, MP, 1e9, dX, 0, cfl=0.8, max_steps=60, contorted_tol=1.0)
        resp = max(resp, rel_err(r2, ref))
    assert 1e-9 < resp < 1e-5, resp
    u = T(u0).view(-1)
    clock = torch.tensor([0.0, 0.0, 1e9, 0.8, 0.0], dtype=torch.float64, device=DEV)
    G3.iterate(u, [200], dX, [0, 0], MP, clock, 60, contorted_tol=1.0)
    c = H(clock)
    assert int(c[4]) == 60
    # the clock sums the CFL steps of states held to the WENO bar
    assert abs(c[0] - t) <= 1e-7 * t
    got = H(u).reshape(ref.shape)
    assert np.isfinite(got).all()
    assert rel_err(got, ref) < 10 * resp, (rel_err(got, ref), resp)


def test_generic_kernels_at_n2_match_the_n2_library():
    """The node-per-thread kernels at N = 2 against the shuffle-based N = 2
    kernels: one full step of a 300-cell tube (the two formulations round in
    different orders)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import phd_gb300 as G
    from phd_gb300 import problems
    from phd_gb300.order import for_order
    G2 = for_order(2)
    O = Oracle()
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=300)
    u_np, _, _ = O.run(u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=25)
    nX = np.array([300], np.int32)
    dt = O.timestep(u_np, dX, 0.8, 0.0, 1e9, 25, MP)
    ub = T(O.boundaries(u_np, nX, [0, 0]))
    a = T(u_np).view(-1)
    b = T(u_np).view(-1)
    G.solvers.ader_stepper(a, ub, nX, dt, dX, False, 0, MP, None)
    G2.solvers.ader_stepper(b, ub, nX, dt, dX, False, 0, MP, None)
    assert rel_err(H(b), H(a)) < 1e-13
    assert rel_err(H(b), u_np.ravel()) > 1e-6


def test_order_arguments_are_checked(G3):
    from phd_gb300 import _lib, problems
    lib = _lib.load()
    assert lib.gpr_order_supported(3, 1, 17) == 1
    assert lib.gpr_order_supported(3, 2, 17) == 1
    assert lib.gpr_order_supported(3, 3, 17) == 0
    assert lib.gpr_order_supported(4, 1, 17) == 0
    u0, MP, tf, dX, bcs = problems.shock_tube(nx=16)
    u = T(u0).view(-1)
    ub = torch.zeros((16 + 6) * 17, dtype=torch.float64, device=DEV)
    with pytest.raises(RuntimeError):  # unknown flux code
        G3.solvers.ader_stepper(u, ub, [16], 1e-3, dX, False, 5, MP, None)
    with pytest.raises(RuntimeError):  # unknown boundary code
        G3.boundaries(u, ub, [16], [0, 9])


@pytest.mark.parametrize("case", ["tgv16_cfl08", "tube_stiff", "forced_stiff"])
def test_n3_stiff_predictor_against_oracle(G3, case):
    """The stiff-source Newton pass at N = 3: cells where the reference's
    Picard iteration does not converge (all of them on the 16 x 16 vortex at
    CFL 0.8, 6 of 66 on the stiff tube), or every cell with STIFF, are
    finished by the Newton iteration on the (27 x 27 and 9 x 9 per spatial
    node) correction systems; the same cells as the oracle's, whose Newton
    solve (dg_stiff at N = 3) converges to 1e-11 and agrees with its dense
    finite-difference Newton solve of the same fixed point; then one ADER
    step with that predictor against the oracle's."""
    from phd_gb300 import problems
    O = Oracle(N=3)
    stiff = False
    if case == "tgv16_cfl08":
        u0, MP, tf, dX, bcs = problems.taylor_green(n=16, cs=10.0, mu=1e-2)
        nX, bc, cfl = np.array([16, 16], np.int32), [1] * 4, 0.8
    elif case == "tube_stiff":
        u0, MP, tf, dX, bcs = problems.shock_tube(nx=64, mu=1e-4, cs=5.0)
        nX, bc, cfl = np.array([64], np.int32), [0, 0], 0.8
    else:  # STIFF = True on a non-stiff tube: Newton from the start
        u0, MP, tf, dX, bcs = problems.shock_tube(nx=48)
        nX, bc, cfl, stiff = np.array([48], np.int32), [0, 0], 0.8, True
    u, _, _ = O.run(u0, MP, 1e9, dX, bc[0], cfl=0.4, max_steps=3)
    dt = O.timestep(u, dX, cfl, 0.0, 1e9, 10, MP)
    ub = O.boundaries(u, nX, bc)
    wh = O.weno_launcher(ub, nX)
    ref, st_ref = O.predictor(wh, dt, dX, nX, MP, stiff=stiff, newton_fallback=1)
    fd, st_fd = O.predictor(wh, dt, dX, nX, MP, stiff=stiff, newton_fallback=2)
    assert (st_ref < -1000).sum() > 0, "case must exercise the stiff path"
    assert not ((st_ref == -1) | (st_ref == -2)).any()
    ncb = int(np.prod(nX + 2))
    qh = torch.full((ref.size,), np.nan, dtype=torch.float64, device=DEV)
    status = torch.full((ncb,), -1, dtype=torch.int32, device=DEV)
    G3.solvers.dg.predictor(qh, T(wh), dt, dX, stiff, False, MP, None, status=status, nX=nX)
    got, st = H(qh), H(status)
    assert np.isfinite(got).all()
    newton = (st & 0xff) == 1
    assert (newton == (st_ref < -1000)).all(), "same cells take the stiff path"
    assert ((st & 0xff) != 2).all(), "no cell may be left unconverged"
    pic = st_ref > 0
    assert ((st[pic] >> 8) == st_ref[pic]).all(), "the same Picard iteration counts"
    assert rel_err(got, ref) < 1e-10, rel_err(got, ref)
    assert rel_err(got, fd) < 1e-9, rel_err(got, fd)
    # one ADER step with the stiff predictor.  Both Newton passes stop at
    # relative updates of 1e-11, so their predictors differ at that level,
    # and the step's stiff volume source multiplies a difference in the
    # distortion by about dt / tau (the stiffness that makes Picard fail
    # here): 1e-9 for the step (1.3e-10 measured on the vortex, where every
    # cell takes the Newton pass)
    ref_u = u.ravel().copy()
    O.ader_stepper(ref_u, ub, nX, dt, dX, MP, stiff=stiff, newton_fallback=1)
    ud = T(u).view(-1)
    G3.solvers.ader_stepper(ud, T(ub), nX, dt, dX, stiff, 0, MP, None)
    assert rel_err(H(ud), ref_u) < 1e-9, rel_err(H(ud), ref_u)


@pytest.mark.parametrize("flux", [1, 2])
@pytest.mark.parametrize("dim", [1, 2])
def test_n3_roe_osher_against_oracle(G3, dim, flux):
    """Roe (1) and Osher (2) at N = 3: the eigen dissipation at every face
    point with the scheme's three path nodes (Osher: three 17 x 17
    eigen-decompositions per point, Roe: one of the path-averaged matrix),
    x and y faces in 2D; the FV update from the oracle's predictor within
    1e-12 of the oracle's; one ADER step within 1e-10 in 1D and, in 2D,
    within 10x the oracle's own response to 1e-16 relative noise on its input
    (the central WENO stencil's conditioning on the vortex's near-constant
    fields, as for the Rusanov step)."""
    from phd_gb300 import problems
    O = Oracle(N=3)
    if dim == 1:
        u0, MP, tf, dX, bcs = problems.shock_tube(nx=64)
        nX, bc = np.array([64], np.int32), [0, 0]
        u, _, _ = O.run(u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=20)
    else:
        # mu = 1: Picard converges in every cell (the stiff pass is tested
        # above)
        u0, MP, tf, dX, bcs = problems.taylor_green(n=12, ny=10, cs=10.0, mu=1.0)
        nX, bc = np.array([12, 10], np.int32), [1] * 4
        u, _, _ = O.run(u0, MP, 1e9, dX, 1, cfl=0.4, max_steps=2)
    dt = O.timestep(u, dX, 0.4, 0.0, 1e9, 10, MP)
    ub = O.boundaries(u, nX, bc)
    wh = O.weno_launcher(ub, nX)
    qh, st = O.predictor(wh, dt, dX, nX, MP)
    assert (st > 0).all()
    ref = u.ravel().copy()
    O.fv_launcher(ref, qh, nX, dt, dX, MP, flux=flux)
    assert np.isfinite(ref).all()
    ud = T(u).view(-1)
    G3.solvers.fv.fv_launcher(ud, T(qh), nX, dt, dX, True, True, flux, MP, None)
    assert rel_err(H(ud), ref) < 1e-12, rel_err(H(ud), ref)
    ref_u = u.ravel().copy()
    O.ader_stepper(ref_u, ub, nX, dt, dX, MP, flux=flux)
    bar = 1e-10
    if dim == 2:
        rng = np.random.default_rng(3)
        resp = 0.0
        for _ in range(2):
            up = u * (1 + 1e-16 * rng.standard_normal(u.shape))
            r2 = up.ravel().copy()
            O.ader_stepper(r2, O.boundaries(up, nX, bc), nX, dt, dX, MP, flux=flux)
            resp = max(resp, rel_err(r2, ref_u))
        assert resp < 1e-6, resp
        bar = max(bar, 10 * resp)
    ud = T(u).view(-1)
    G3.solvers.ader_stepper(ud, T(ub), nX, dt, dX, False, flux, MP, None)
    assert rel_err(H(ud), ref_u) < bar, (rel_err(H(ud), ref_u), bar)


def test_n3_2d_stages_against_golden(G3):
    """The 12 x 10 Taylor-Green vortex (periodic) at N = 3: the reference's
    own stages.  The reconstruction's bar is the conditioning bar (the
    vortex's constant fields make the central stencil's weight a ratio of
    rounding-level indicators; the oracle differs from the reference by
    3e-8 there)."""
    g = golden("stages2d_rus_v17n3.npz")
    MP = Par.from_array(g["mp"])
    nX, dX = [int(x) for x in g["nX"]], list(g["dX"])
    ncb = (nX[0] + 2) * (nX[1] + 2)
    dt = float(g["dt"])
    u = T(g["u"])
    ub = torch.full((g["ub"].size,), np.nan, dtype=torch.float64, device=DEV)
    G3.boundaries(u, ub, nX, [int(g["bcs"])] * 4)
    assert rel_err(H(ub), g["ub"]) == 0.0
    wh = torch.full((g["wh"].size,), np.nan, dtype=torch.float64, device=DEV)
    G3.solvers.weno.weno_launcher(wh, T(g["ub"]), nX)
    assert rel_err(H(wh), g["wh"]) < 1e-7
    qh = torch.full((g["qh"].size,), np.nan, dtype=torch.float64, device=DEV)
    mask = torch.ones(ncb, dtype=torch.bool, device=DEV)
    status = torch.full((ncb,), -1, dtype=torch.int32, device=DEV)
    G3.solvers.dg.predictor(qh, T(g["wh"]), dt, dX, False, False, MP, mask, status=status)
    assert ((H(status) & 0xff) == 0).all()
    assert rel_err(H(qh), g["qh"]) < 1e-13
    ufv = T(g["u"])
    G3.solvers.fv.fv_launcher(ufv, T(g["qh"]), nX, dt, dX, True, True, 0, MP, mask)
    assert rel_err(H(ufv), g["u_fv"]) < 1e-14
    ust = T(g["u"])
    G3.solvers.ader_stepper(ust, T(g["ub"]), nX, dt, dX, False, 0, MP, mask)
    import phd_gb300
    phd_gb300.solvers.renorm_distortion(ust, [MP])
    assert rel_err(H(ust), g["u_step"]) < 1e-7


def _vortex(n=24, ny=20, steps=3):
    from phd_gb300 import problems
    O = Oracle(N=3)
    u0, MP, tf, dX, bcs = problems.taylor_green(n=n, ny=ny, cs=10.0, mu=0.1)
    u_np, k, _ = O.run(u0, MP, 1e9, dX, [1] * 4, cfl=0.4, max_steps=steps)
    assert k == steps
    return O, u_np.ravel(), MP, dX, np.array([n, ny], np.int32)


def test_n3_2d_boundaries_every_code(G3):
    """Ghost cells of a 2D state with a different boundary code on each
    side, every code once on an x side and once on a y side: bit-equal to
    the oracle, corners included (the y transform of the x transform)."""
    O, u_np, MP, dX, nX = _vortex(steps=1)
    rng = np.random.default_rng(3)
    u_np = u_np * (1 + 0.1 * rng.standard_normal(u_np.shape))  # no symmetry to hide behind
    u = T(u_np)
    nub = int(np.prod(nX + 6))
    for bcs in ([2, 3, 4, 5], [5, 4, 3, 2], [0, 1, 2, 3], [4, 5, 0, 1], [1, 1, 0, 0], [0, 0, 1, 1]):
        ref = O.boundaries(u_np, nX, bcs)
        ub = torch.full((nub * 17,), np.nan, dtype=torch.float64, device=DEV)
        G3.boundaries(u, ub, nX, bcs)
        assert np.array_equal(H(ub), ref), bcs


def test_n3_2d_stages_against_oracle(G3):
    """A 24 x 20 vortex after three N = 3 oracle steps, with a mask that
    leaves out a block of cells: predictor (the same Picard iteration
    counts) and FV update from the oracle's inputs to 1e-13, the WENO
    reconstruction to the conditioning bar."""
    O, u_np, MP, dX, nX = _vortex()
    ncb = int(np.prod(nX + 2))
    dt = O.timestep(u_np, dX, 0.4, 0.0, 1e9, 3, MP)
    mask = np.ones((nX[0] + 2, nX[1] + 2), np.uint8)
    mask[7:11, 5:12] = 0
    mask = mask.ravel()
    ub = O.boundaries(u_np, nX, [1] * 4)
    wh = O.weno_launcher(ub, nX)
    wh_d = torch.empty(wh.size, dtype=torch.float64, device=DEV)
    G3.solvers.weno.weno_launcher(wh_d, T(ub), nX)
    assert rel_err(H(wh_d), wh) < 1e-7
    qh, st = O.predictor(wh, dt, dX, nX, MP, mask=mask, newton_fallback=0)
    assert (st[mask == 1] > 0).all()
    qh_d = torch.zeros(qh.size, dtype=torch.float64, device=DEV)
    status = torch.full((ncb,), -1, dtype=torch.int32, device=DEV)
    md = T(mask, torch.uint8)
    G3.solvers.dg.predictor(qh_d, T(wh), dt, dX, False, False, MP, md, status=status, nX=nX)
    got = H(qh_d).reshape(ncb, -1)
    on = mask == 1
    assert rel_err(got[on], qh.reshape(ncb, -1)[on]) < 1e-13
    assert ((H(status)[on] >> 8) == st[on]).all(), "the same Picard iteration counts"
    qh = np.where(on[:, None], qh.reshape(ncb, -1), 0.0).ravel()
    ref = u_np.copy()
    O.fv_launcher(ref, qh, nX, dt, dX, MP, mask=mask)
    u = T(u_np)
    G3.solvers.fv.fv_launcher(u, T(qh), nX, dt, dX, True, True, 0, MP, md)
    assert rel_err(H(u), ref) < 1e-13
    assert rel_err(H(u), u_np) > 1e-6


def test_n3_2d_run_against_oracle(G3):
    """Ten steps of the 32 x 32 vortex (mu = 0.1: at this resolution and
    mu = 1e-2 the time step exceeds the relaxation time and the reference's
    Picard iteration diverges) at N = 3 through the device loop
    against the oracle's loop, held to 10x the oracle's own response to
    1e-16 relative noise on its initial state (the central WENO stencil's
    conditioning on the vortex's constant fields)."""
    from phd_gb300 import problems
    O = Oracle(N=3)
    u0, MP, tf, dX, bcs = problems.taylor_green(n=32, cs=10.0, mu=0.1)
    ref, n, t = O.run(u0, MP, 1e9, dX, [1] * 4, cfl=0.4, max_steps=10, contorted_tol=1.0)
    rng = np.random.default_rng(2)
    resp = 0.0
    for _ in range(2):
        up = u0 * (1 + 1e-16 * rng.standard_normal(u0.shape))
        r2, _, _ = O.run(up, MP, 1e9, dX, [1] * 4, cfl=0.4, max_steps=10, contorted_tol=1.0)
        resp = max(resp, rel_err(r2, ref))
    assert resp < 1e-5, resp
    u = T(u0).view(-1)
    clock = torch.tensor([0.0, 0.0, 1e9, 0.4, 0.0], dtype=torch.float64, device=DEV)
    status = torch.full((34 * 34,), -1, dtype=torch.int32, device=DEV)
    G3.iterate(u, [32, 32], dX, [1] * 4, MP, clock, 10, status=status, contorted_tol=1.0)
    assert ((H(status) & 0xff) == 0).all(), "Picard converges in every cell"
    c = H(clock)
    assert int(c[4]) == 10
    assert abs(c[0] - t) <= 1e-7 * t
    got = H(u).reshape(ref.shape)
    assert np.isfinite(got).all()
    assert rel_err(got, ref) < max(1e-12, 10 * resp), (rel_err(got, ref), resp)
    assert rel_err(got, u0) > 1e-6


def test_generic_kernels_at_n2_match_the_n2_library_2d():
    """The node-per-thread kernels at N = 2 on a 2D grid against the N = 2
    library's 2D step: one step of a 40 x 36 vortex with slip walls in x."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import phd_gb300 as G
    from phd_gb300 import problems
    from phd_gb300.order import for_order
    G2 = for_order(2)
    O = Oracle()
    u0, MP, tf, dX, bcs = problems.taylor_green(n=40, ny=36, cs=10.0, mu=0.1)
    u_np, _, _ = O.run(u0, MP, 1e9, dX, [2, 2, 1, 1], cfl=0.4, max_steps=3)
    nX = np.array([40, 36], np.int32)
    dt = O.timestep(u_np, dX, 0.4, 0.0, 1e9, 3, MP)
    ub_ref = O.boundaries(u_np, nX, [2, 2, 1, 1])
    ub = torch.empty(ub_ref.size, dtype=torch.float64, device=DEV)
    G2.boundaries(T(u_np).view(-1), ub, nX, [2, 2, 1, 1])
    assert np.array_equal(H(ub), ub_ref)
    a = T(u_np).view(-1)
    b = T(u_np).view(-1)
    G.solvers.ader_stepper(a, ub, nX, dt, dX, False, 0, MP, None)
    G2.solvers.ader_stepper(b, ub, nX, dt, dX, False, 0, MP, None)
    assert rel_err(H(b), H(a)) < 1e-13
    assert rel_err(H(b), u_np.ravel()) > 1e-6
