"""Adjoint of the 1D step: pointwise Jacobians against finite differences of
the device physics, one-step dot-product tests, whole-run gradients of the
first-Stokes-problem misfit against central finite differences (h = 1e-6)
of the GPU forward and of the tight-tolerance oracle, and the batched form.

The gradient bar is 1e-6 relative.  Central differences use h = 1e-6;
where the WENO weights make their truncation error visible (state
directions on varying data) one Richardson step is taken."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MU, CS, CALPHA = 1e-2, 1.0, 1.0     # true parameters of the Stokes problem
THETA = np.array([1.2e-2, 0.9, 1.1])  # where gradients are taken


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def make_par(theta, gamma=1.4):
    """theta = (mu, cs, calpha[, gamma])."""
    from phd_gb300.params import material_params
    mu, cs, calpha = theta[0], theta[1], theta[2]
    if len(theta) > 3:
        gamma = theta[3]
    return material_params("sg", 1.0, cv=1.0, gamma=gamma, b0=cs, calpha=calpha, mu=mu,
                           Pr=0.75)


def _stokes(nx=400, tf=1.0):
    from phd_gb300 import problems
    u, MP, tf_, dX, bc = problems.stokes(nx=nx, mu=MU, cs=CS, calpha=CALPHA, tf=tf)
    return u, dX[0], bc


def _problem(nx, dx, ninst=1, tf=1.0, frozen=False, K=32):
    from phd_gb300.adjoint import Problem
    return Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf,
                   frozen_dt=frozen, checkpoint_every=K)


def test_point_jacobians_match_finite_differences():
    _cuda()
    from phd_gb300 import _lib, api
    from phd_gb300.adjoint import FIELDS
    lib = _lib.load()
    rng = np.random.default_rng(5)
    u, dx, _ = _stokes(nx=16)
    Q = u[:8].copy()
    Q += 0.05 * rng.standard_normal(Q.shape) * (np.abs(Q) + 0.1)
    Q[:, 0] = np.abs(Q[:, 0]) + 0.5
    MP = make_par(THETA)
    V, K, n = Q.shape[1], Q.shape[1] + len(FIELDS), Q.shape[0]
    Qd = torch.tensor(Q, device="cuda")
    JF = torch.zeros(n * K * V, dtype=torch.float64, device="cuda")
    JS = torch.zeros_like(JF)
    dl = torch.zeros(n * K, dtype=torch.float64, device="cuda")
    c = MP.to_ctypes()
    rc = lib.gpr_adj_point_jacobians(ctypes.c_void_p(Qd.data_ptr()), n,
                                     ctypes.cast(ctypes.pointer(c), ctypes.c_void_p),
                                     ctypes.c_void_p(JF.data_ptr()),
                                     ctypes.c_void_p(JS.data_ptr()),
                                     ctypes.c_void_p(dl.data_ptr()), V, None)
    assert rc == 0
    torch.cuda.synchronize()
    JF = JF.cpu().numpy().reshape(n, K, V)
    JS = JS.cpu().numpy().reshape(n, K, V)
    dl = dl.cpu().numpy().reshape(n, K)

    def evals(Qx, MPx):
        q = torch.tensor(Qx, device="cuda")
        F = api.flux(q, 0, MPx).cpu().numpy()
        S = api.source(q, MPx).cpu().numpy()
        lam = api.max_abs_eigs(q, 0, MPx).cpu().numpy()
        return F, S, lam

    # lambda is evaluated to a few ulps: its finite differences carry
    # ~1e-15 / h noise, so it is compared on the scale of its whole gradient
    lam_scale = np.abs(dl[:, :V]).max()
    for k in range(V):
        h = 1e-6 * np.maximum(1.0, np.abs(Q[:, k]))
        Qp, Qm = Q.copy(), Q.copy()
        Qp[:, k] += h
        Qm[:, k] -= h
        Fp, Sp, lp = evals(Qp, MP)
        Fm, Sm, lm = evals(Qm, MP)
        for a, fp, fm in ((JF[:, k], Fp, Fm), (JS[:, k], Sp, Sm)):
            fd = (fp - fm) / (2 * h[:, None])
            scale = np.abs(fd).max() + np.abs(a).max() + 1e-12
            assert np.abs(a - fd).max() < 1e-6 * scale, (k, np.abs(a - fd).max(), scale)
        fd = (lp - lm) / (2 * h)
        assert np.abs(dl[:, k] - fd).max() < 1e-6 * lam_scale, (k, np.abs(dl[:, k] - fd).max())
    # material fields: perturb Par members that move one device field each
    # (gamma also moves 1/(gamma - 1))
    def perturbed(field, s):
        p = MP.copy()
        setattr(p, field, getattr(p, field) + s)
        return p
    checks = {"b02": ("b02", [2]), "calpha2": ("calpha2", [4]),
              "kappa": ("kappa", [5]), "mu": ("mu", [3]), "gamma": ("gamma", [0, 1])}
    for name, (field, cols) in checks.items():
        x = getattr(MP, field)
        h = 1e-6 * abs(x)
        Fp, Sp, lp = evals(Q, perturbed(field, h))
        Fm, Sm, lm = evals(Q, perturbed(field, -h))
        # chain factor d(field col)/d(member)
        if name == "kappa":
            fac = {5: -1.0 / x ** 2}
        elif name == "mu":
            fac = {3: -MP.rho0 / (2 * x * x)}
        elif name == "gamma":
            fac = {0: 1.0, 1: -1.0 / (x - 1) ** 2}
        else:
            fac = {cols[0]: 1.0}
        for a, fp, fm in ((JF, Fp, Fm), (JS, Sp, Sm)):
            ad = sum(f * a[:, V + col] for col, f in fac.items())
            fd = (fp - fm) / (2 * h)
            # gamma moves two fields whose effects on T cancel exactly:
            # compare on the scale of the terms combined
            terms = sum(abs(f) * np.abs(a[:, V + col]).max() for col, f in fac.items())
            scale = np.abs(fd).max() + terms + 1e-12
            assert np.abs(ad - fd).max() < 1e-6 * scale, (name, np.abs(ad - fd).max(), scale)
        ad = sum(f * dl[:, V + col] for col, f in fac.items())
        fd = (lp - lm) / (2 * h)
        assert np.abs(ad - fd).max() < 1e-6 * (np.abs(fd).max() + lam_scale * x), name


def richardson(cd, h):
    """Central differences at h with one Richardson step (h, 2h).  Across
    the WENO weights the h^2 truncation error of plain central differences
    reaches 1e-5 .. 1e-4 relative at h = 1e-6 on varying data; the
    extrapolation (4 cd(h) - cd(2h)) / 3 removes it."""
    return (4.0 * cd(h) - cd(2.0 * h)) / 3.0


def _misfit_setup(nx, tf, ninst=1):
    """Target v_y from the true parameters; the loss at THETA."""
    from phd_gb300.adjoint import Problem
    u0, dx, _ = _stokes(nx=nx, tf=tf)
    u0p = np.tile(u0, (ninst, 1))
    prob_t = Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf)
    uT = prob_t.forward(torch.tensor(u0p, device="cuda"),
                        [make_par(np.array([MU, CS, CALPHA]))] * ninst)
    target = (uT[:, 3] / uT[:, 0]).clone()
    return u0p, dx, target


def _loss(uN, target):
    vy = uN[:, 3] / uN[:, 0]
    return 0.5 * torch.sum((vy - target) ** 2)


def _noisy_state(nx, rng):
    """A Stokes state with every variable varying from cell to cell.

    Finite differences of the WENO step are only meaningful where the data
    vary: on exactly constant data the smoothness indicator sits at its
    epsilon (1e-14) and the weights move on a perturbation scale of
    sqrt(1e-14) = 1e-7, below a step of h = 1e-6 (the derivative there is
    still exact; central differences just cannot resolve it)."""
    u0, dx, _ = _stokes(nx=nx, tf=1.0)
    u0 = u0 * (1.0 + 1e-2 * rng.standard_normal(u0.shape))
    u0[:, 2] = u0[:, 0] * (0.05 + 0.01 * rng.standard_normal(nx))
    u0[:, 4] = u0[:, 0] * (0.02 + 0.01 * rng.standard_normal(nx))
    u0[:, 5:14] += 1e-2 * rng.standard_normal((nx, 9))
    u0[:, 14:17] = 0.01 * rng.standard_normal((nx, 3))
    return u0, dx


@pytest.mark.parametrize("nvar", [17, 14])
def test_point_vjp_matches_dual_jacobians(nvar):
    """The reverse-mode products the backward step uses equal the dual-number
    Jacobians contracted with the same cotangents."""
    _cuda()
    from phd_gb300 import _lib
    from phd_gb300.adjoint import FIELDS
    lib = _lib.load()
    rng = np.random.default_rng(11)
    u, dx, _ = _stokes(nx=64)
    Q = u[:48, :nvar].copy()
    Q += 0.1 * rng.standard_normal(Q.shape) * (np.abs(Q) + 0.1)
    Q[:, 0] = np.abs(Q[:, 0]) + 0.5
    MP = make_par(THETA)
    V, K, n = nvar, nvar + len(FIELDS), Q.shape[0]
    Fb = rng.standard_normal((n, V))
    Sb = rng.standard_normal((n, V))
    lb = rng.standard_normal(n)
    c = MP.to_ctypes()
    pc = ctypes.cast(ctypes.pointer(c), ctypes.c_void_p)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    Qd = dev(Q)
    JF = torch.zeros(n * K * V, dtype=torch.float64, device="cuda")
    JS = torch.zeros_like(JF)
    dl = torch.zeros(n * K, dtype=torch.float64, device="cuda")
    assert lib.gpr_adj_point_jacobians(ptr(Qd), n, pc, ptr(JF), ptr(JS), ptr(dl), V, None) == 0
    Fd, Sd, ld = dev(Fb), dev(Sb), dev(lb)
    qb = torch.zeros(n * V, dtype=torch.float64, device="cuda")
    thb = torch.zeros(n * len(FIELDS), dtype=torch.float64, device="cuda")
    assert lib.gpr_adj_point_vjp(ptr(Qd), n, pc, ptr(Fd), ptr(Sd), ptr(ld), ptr(qb), ptr(thb),
                                 V, None) == 0
    torch.cuda.synchronize()
    JF = JF.cpu().numpy().reshape(n, K, V)
    JS = JS.cpu().numpy().reshape(n, K, V)
    dl = dl.cpu().numpy().reshape(n, K)
    want = (np.einsum("nkj,nj->nk", JF, Fb) + np.einsum("nkj,nj->nk", JS, Sb)
            + dl * lb[:, None])
    got = np.concatenate([qb.cpu().numpy().reshape(n, V),
                          thb.cpu().numpy().reshape(n, len(FIELDS))], axis=1)
    scale = (np.abs(JF).max(axis=2) * np.abs(Fb).max(axis=1)[:, None]
             + np.abs(JS).max(axis=2) * np.abs(Sb).max(axis=1)[:, None]
             + np.abs(dl * lb[:, None]) + 1e-300)
    err = np.abs(got - want) / scale
    assert err.max() < 1e-12, (np.unravel_index(err.argmax(), err.shape), err.max())


def test_one_step_jacobian_matches_finite_differences():
    """The full Jacobian of one step (6 cells x 17 variables, held dt) from
    the backward step, row by row, against central differences column by
    column.  dt / tau1 = 0.34 here, so cells take the dense transposed
    solve as well as the iteration."""
    _cuda()
    from phd_gb300.adjoint import Problem
    rng = np.random.default_rng(7)
    nx, V = 6, 17
    u0, dx = _noisy_state(nx, rng)
    MP = make_par(THETA)
    n = nx * V
    P = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=1.0, frozen_dt=True,
                checkpoint_every=1)
    P.forward(torch.tensor(u0, device="cuda"), [MP], max_steps=1)
    sched = list(P.schedule)
    JA = np.zeros((n, n))
    for o in range(n):
        ub = np.zeros(n)
        ub[o] = 1.0
        P.forward(torch.tensor(u0, device="cuda"), [MP], max_steps=1)
        g, _ = P.backward(torch.tensor(ub.reshape(nx, V), device="cuda"))
        JA[o] = g.cpu().numpy().ravel()
    Q = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=1.0)
    uf = u0.ravel()
    JF = np.zeros((n, n))
    for i in range(n):
        h = 1e-6 * max(1.0, abs(uf[i]))
        up, um = uf.copy(), uf.copy()
        up[i] += h
        um[i] -= h
        a = Q.forward(torch.tensor(up.reshape(nx, V), device="cuda"), [MP], schedule=sched,
                      max_steps=1).cpu().numpy().ravel()
        b = Q.forward(torch.tensor(um.reshape(nx, V), device="cuda"), [MP], schedule=sched,
                      max_steps=1).cpu().numpy().ravel()
        JF[:, i] = (a - b) / (2 * h)
    assert np.abs(JA - JF).max() < 1e-6 * np.abs(JF).max(), np.abs(JA - JF).max()


def test_dot_product_through_cfl_steps():
    """<ubar_N, J du> by central differences equals <J^T ubar_N, du> over 1
    and 7 steps with dt differentiated through the CFL rule (the noisy state
    has a unique CFL maximum) and with dt held."""
    _cuda()
    from phd_gb300.adjoint import Problem
    rng = np.random.default_rng(11)
    nx = 64
    u0, dx = _noisy_state(nx, rng)
    MP = make_par(THETA)
    ub = rng.standard_normal(u0.shape)
    du = rng.standard_normal(u0.shape) * (np.abs(u0) + 1e-2)
    for frozen in (True, False):
        for nsteps in (1, 7):
            P = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=1.0, frozen_dt=frozen,
                        checkpoint_every=4)
            P.forward(torch.tensor(u0, device="cuda"), [MP], max_steps=nsteps)
            sched = list(P.schedule) if frozen else None
            g0, fb = P.backward(torch.tensor(ub, device="cuda"))
            ad = float(np.sum(g0.cpu().numpy() * du))
            Q = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=1.0)

            def cd(h):
                up = Q.forward(torch.tensor(u0 + h * du, device="cuda"), [MP], schedule=sched,
                               max_steps=nsteps).cpu().numpy()
                um = Q.forward(torch.tensor(u0 - h * du, device="cuda"), [MP], schedule=sched,
                               max_steps=nsteps).cpu().numpy()
                return float(np.sum(ub * (up - um))) / (2 * h)

            fd = richardson(cd, 1e-6)
            assert abs(ad - fd) <= 1e-6 * abs(fd), (frozen, nsteps, ad, fd)


def test_stokes_parameter_gradient_matches_finite_differences():
    """Config: 400 cells on [-1, 1], t_end = 1.0 (385 steps at CFL 0.8),
    checkpoints every 32 steps; gradient of the v_y misfit with respect to
    (mu, cs, calpha) through the CFL time steps."""
    _cuda()
    from phd_gb300.adjoint import Problem, solve
    nx, tf = 400, 1.0
    u0p, dx, target = _misfit_setup(nx, tf)
    prob = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf, checkpoint_every=32)
    u0 = torch.tensor(u0p, device="cuda", requires_grad=True)
    th = torch.tensor(THETA[None, :], dtype=torch.float64, requires_grad=True)
    L = _loss(solve(u0, th, prob), target)
    L.backward()
    assert prob.nsteps > 300
    g = th.grad.numpy()[0]
    for j in range(3):
        h = 1e-6 * THETA[j]
        Lpm = []
        for s in (1, -1):
            t2 = THETA.copy()
            t2[j] += s * h
            P2 = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf)
            Lpm.append(float(_loss(P2.forward(torch.tensor(u0p, device="cuda"),
                                              [make_par(t2)]), target)))
        fd = (Lpm[0] - Lpm[1]) / (2 * h)
        assert abs(g[j] - fd) <= 1e-6 * abs(fd), (j, g[j], fd)


def test_stokes_gamma_gradient_matches_finite_differences():
    """The same misfit with the ratio of specific heats among the parameters,
    theta = (mu, cs, calpha, gamma) at (1.2e-2, 0.9, 1.1, 1.45): gamma enters
    the device fields gamma, 1/(gamma - 1) and 1/kappa (kappa = mu gamma cv /
    Pr); every component against central differences (h = 1e-6 theta_j)."""
    _cuda()
    from phd_gb300.adjoint import Problem, solve
    nx, tf = 400, 1.0
    theta = np.array([1.2e-2, 0.9, 1.1, 1.45])
    u0p, dx, target = _misfit_setup(nx, tf)
    prob = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf, checkpoint_every=32)
    u0 = torch.tensor(u0p, device="cuda", requires_grad=True)
    th = torch.tensor(theta[None, :], dtype=torch.float64, requires_grad=True)
    L = _loss(solve(u0, th, prob), target)
    L.backward()
    g = th.grad.numpy()[0]
    assert g[3] != 0.0
    for j in range(4):
        h = 1e-6 * theta[j]
        Lpm = []
        for s in (1, -1):
            t2 = theta.copy()
            t2[j] += s * h
            P2 = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf)
            Lpm.append(float(_loss(P2.forward(torch.tensor(u0p, device="cuda"),
                                              [make_par(t2)]), target)))
        fd = (Lpm[0] - Lpm[1]) / (2 * h)
        assert abs(g[j] - fd) <= 1e-6 * abs(fd), (j, g[j], fd)


def _smooth_field(rng, x, scale, modes=3):
    d = np.zeros((x.size, scale.size))
    for k in range(scale.size):
        a = rng.standard_normal(modes)
        ph = rng.uniform(0, 2 * np.pi, modes)
        d[:, k] = scale[k] * sum(a[m] * np.sin((m + 1) * np.pi * x + ph[m]) for m in range(modes))
    return d


def _state_gradient_check(nsteps, ndir, bound):
    from phd_gb300.adjoint import Problem, solve
    nx, tf = 400, 1.0
    u0p, dx, target = _misfit_setup(nx, tf)
    x = (np.arange(nx) + 0.5) / nx
    rng0 = np.random.default_rng(17)
    # a background x-velocity keeps |v_x| in the Rusanov speed away from its
    # kink at v_x = 0 (the Stokes state has v_x = 0 everywhere)
    u0p[:, 2] += 0.05 * u0p[:, 0]
    u0p = u0p + 1e-2 * _smooth_field(rng0, x, np.abs(u0p).max(axis=0) + 1e-2, modes=16)
    prob = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf, frozen_dt=True)
    u0 = torch.tensor(u0p, device="cuda", requires_grad=True)
    th = torch.tensor(THETA[None, :], dtype=torch.float64, requires_grad=True)
    if nsteps is not None:
        uN = prob.forward(u0, [make_par(THETA)], max_steps=nsteps).clone().requires_grad_(True)
        L = _loss(uN, target)
        L.backward()
        g, _ = prob.backward(uN.grad)
        g = g.cpu().numpy()
    else:
        _loss(solve(u0, th, prob), target).backward()
        g = u0.grad.cpu().numpy()
    sched = list(prob.schedule)
    rng = np.random.default_rng(3)
    MP = make_par(THETA)
    scale = np.abs(u0p).max(axis=0) + 1e-2
    P2 = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf)
    worst = 0.0
    for _ in range(ndir):
        d = _smooth_field(rng, x, scale)

        def cd(h):
            Lpm = [float(_loss(P2.forward(torch.tensor(u0p + sg * h * d, device="cuda"),
                                          [MP], schedule=sched), target)) for sg in (1, -1)]
            return (Lpm[0] - Lpm[1]) / (2 * h)

        fd = richardson(cd, 1e-6)
        ad = float(np.sum(g * d))
        worst = max(worst, abs(ad - fd) / abs(fd))
    assert worst <= bound, worst


def test_stokes_state_gradient_matches_finite_differences():
    """Initial-state gradient (400 x 17) along 16 random smooth directions
    (a few Fourier modes per variable) over 64 steps (two checkpoint
    segments), with the step schedule held fixed (the CFL maximum is tied
    across the uniform far field, where dt is not differentiable in the
    state).

    The gradient is taken at the Stokes state plus a background x-velocity
    of 0.05 (|v_x| in the Rusanov speed has a kink at v_x = 0, where the
    Stokes state sits) and a smooth perturbation of 1e-2 of each variable's
    scale.  The WENO weights go as (eps + t)^-8 with t ~ (cell-to-cell
    difference)^2, so central differences are linear only while the step's
    own cell-to-cell change stays far below 1/16 of the data's: on the
    exact Stokes data (constant away from x = 0, t at eps = 1e-14) a step of
    h = 1e-6 is far outside that range and cannot resolve the (exact)
    derivative."""
    _cuda()
    _state_gradient_check(64, 16, 1e-6)


def test_stokes_state_gradient_full_run():
    """The same over the whole run (385 steps) to a looser bound: on smooth
    data many faces have lambda_L close to lambda_R, and over 1.5e5 face
    evaluations the finite-difference step crosses some of the switches of
    the Rusanov speed max(lambda_L, lambda_R), where the discrete map is
    only piecewise smooth; the differences then scatter by ~1e-4 while
    converging to the adjoint value as h shrinks (1e-6 .. 1e-8 relative at
    h = 6e-8)."""
    _cuda()
    _state_gradient_check(None, 8, 3e-4)


def test_stokes_gradient_matches_oracle_finite_differences():
    """Reference gradient: central differences of the CPU oracle run at the
    same tight predictor tolerance (a shorter run to keep the CPU time
    small)."""
    _cuda()
    from oracle import Oracle
    from phd_gb300.adjoint import Problem, solve
    nx, tf = 200, 0.25
    u0p, dx, target = _misfit_setup(nx, tf)
    prob = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf)
    u0 = torch.tensor(u0p, device="cuda", requires_grad=True)
    th = torch.tensor(THETA[None, :], dtype=torch.float64, requires_grad=True)
    _loss(solve(u0, th, prob), target).backward()
    g = th.grad.numpy()[0]
    O = Oracle(dg_tol=1e-13, dg_it=300)
    tg = target.cpu().numpy()

    def L_or(theta):
        u, n, t = O.run(u0p, make_par(theta), tf, [dx], 0, cfl=0.8)
        return 0.5 * np.sum((u[:, 3] / u[:, 0] - tg) ** 2)

    for j in range(3):
        h = 1e-6 * THETA[j]
        tp, tm = THETA.copy(), THETA.copy()
        tp[j] += h
        tm[j] -= h
        fd = (L_or(tp) - L_or(tm)) / (2 * h)
        assert abs(g[j] - fd) <= 1e-6 * abs(fd), (j, g[j], fd)


def test_batched_gradients_equal_single_instance():
    """64 Stokes instances with parameters perturbed by up to 10%: the
    batched adjoint gives each instance the gradient its own run gives."""
    _cuda()
    from phd_gb300.adjoint import Problem, solve
    nx, tf, ninst = 400, 1.0, 64
    u0p, dx, target = _misfit_setup(nx, tf, ninst=ninst)
    rng = np.random.default_rng(20261203)
    theta = THETA[None, :] * (1.0 + 0.1 * rng.uniform(-1, 1, (ninst, 3)))
    prob = Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf)
    u0 = torch.tensor(u0p, device="cuda", requires_grad=True)
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    _loss(solve(u0, th, prob), target).backward()
    G = th.grad.numpy()
    G0 = u0.grad.cpu().numpy()
    for k in (0, 17, 63):
        P1 = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf)
        u1 = torch.tensor(u0p[k * nx:(k + 1) * nx], device="cuda", requires_grad=True)
        t1 = torch.tensor(theta[k:k + 1], dtype=torch.float64, requires_grad=True)
        _loss(solve(u1, t1, P1), target[k * nx:(k + 1) * nx]).backward()
        assert np.allclose(t1.grad.numpy()[0], G[k], rtol=1e-12, atol=0), k
        assert np.allclose(u1.grad.cpu().numpy(), G0[k * nx:(k + 1) * nx], rtol=1e-12,
                           atol=1e-300), k


def test_taped_forward_gives_the_checkpointed_gradient():
    """A forward pass that keeps its segments' tapes (tape_budget_bytes) lets
    the backward pass skip the recompute; the tapes are the ones the
    recompute would write, so the gradients are identical, also when only
    the first segments fit the budget."""
    _cuda()
    from phd_gb300.adjoint import Problem
    nx, tf = 400, 1.0
    u0p, dx, target = _misfit_setup(nx, tf)
    pars = [make_par(THETA)]
    out = []
    for budget in (0, 1 << 34, None):
        prob = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf, checkpoint_every=32)
        if budget is None:  # two segments' worth: the rest is recomputed
            budget = 2 * 32 * prob.tape_len * 8
        prob.tape_budget = budget
        uN = prob.forward(torch.tensor(u0p, device="cuda"), pars, max_steps=100)
        uN = uN.clone().requires_grad_(True)
        _loss(uN, target).backward()
        ub0, fb = prob.backward(uN.grad)
        out.append((ub0.cpu().numpy(), fb.cpu().numpy(), prob.recomputed_steps))
    assert out[0][2] == 100 and out[1][2] == 0 and out[2][2] == 100 - 64
    for k in (1, 2):
        assert np.array_equal(out[k][0], out[0][0])
        assert np.array_equal(out[k][1], out[0][1])
