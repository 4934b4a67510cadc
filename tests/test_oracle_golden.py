"""The CPU oracle against golden vectors produced by the reference's own C++
(tests/golden/make_golden.py).  These pin the oracle before it is trusted as
the checker of the CUDA kernels."""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import Oracle
from phd_gb300.params import Par


@pytest.fixture(scope="module")
def O():
    return Oracle(N=2, thermal=True, lset=0)


def test_constants_known_answers(O):
    c = O.constants()
    s = 1 / np.sqrt(3)
    assert np.allclose(c["nodes"], [(1 - s) / 2, (1 + s) / 2], rtol=0, atol=1e-16)
    assert np.allclose(c["weights"], [0.5, 0.5], rtol=0, atol=1e-15)
    # end values and derivative values of the linear Lagrange basis
    assert np.allclose(c["endvals"].sum(axis=1), 1.0, atol=1e-15)
    assert np.allclose(c["dervals"].sum(axis=1), 0.0, atol=1e-14)
    # smoothness matrix of linear polynomials: 3 [[1,-1],[-1,1]]
    assert np.allclose(c["sig"], 3 * np.array([[1, -1], [-1, 1]]), atol=1e-13)


def test_pointwise_physics(O):
    g = golden("pointwise_v17.npz")
    mps = [Par.from_array(a) for a in g["mp_arrays"]]
    worst = {}
    for m, MP in enumerate(mps):
        for i in range(g["Q"].shape[1]):
            q, q2, x = g["Q"][m, i], g["Q2"][m, i], g["X"][m, i]
            checks = {
                "source": (O.source(q, MP), g["source"][m, i]),
                "pressure": (O.pressure(q, MP), g["pressure"][m, i]),
                "temperature": (O.temperature(q, MP), g["temperature"][m, i]),
            }
            for d in range(3):
                checks["flux%d" % d] = (O.flux(q, d, MP), g["flux"][m, i, d])
                checks["Bdot%d" % d] = (O.Bdot(q, x, d), g["Bdot"][m, i, d])
                checks["mae%d" % d] = (O.max_abs_eigs(q, d, MP), g["max_abs_eigs"][m, i, d])
                checks["Drus%d" % d] = (O.D(0, q, q2, d, MP), g["D_RUS"][m, i, d])
                checks["Dosh%d" % d] = (O.D(2, q, q2, d, MP), g["D_OSH"][m, i, d])
                checks["Droe%d" % d] = (O.D(1, q, q2, d, MP), g["D_ROE"][m, i, d])
                checks["Bint%d" % d] = (O.Bint(q, q2, d), g["Bint"][m, i, d])
                checks["thmt%d" % d] = (O.thermo_acoustic_tensor(q, d, MP),
                                        g["thermo_acoustic_tensor"][m, i, d])
                checks["sysm%d" % d] = (O.system_matrix(q, d, MP), g["system_matrix"][m, i, d])
            for k, dt in enumerate(g["ode_dt"]):
                qq = q.copy()
                O.ode_launcher(qq, dt, MP)
                checks["ode%d" % k] = (qq, g["ode"][m, i, k])
            for key, (a, b) in checks.items():
                worst[key[:4]] = max(worst.get(key[:4], 0.0), rel_err(a, b))
    # ode1/ode2 (dt = 1e-2, 1) relax the distortion completely (tau >> 1):
    # the reference's closed-form cubic (relaxation/analytic.cpp:95-117) then
    # takes square roots of rounding-level quantities (u, Delta ~ 1e-15), so
    # an ulp of difference in the SVD becomes ~1e-8 in A.
    tol = {"Dosh": 1e-10, "Droe": 1e-10, "ode0": 1e-12, "ode1": 1e-7, "ode2": 1e-7}
    for key, err in worst.items():
        assert err <= tol.get(key, 1e-13), (key, err)


@pytest.mark.parametrize("name,N", [("stages1d_rus_v17.npz", 2),
                                    ("stages1d_osh_v17.npz", 2),
                                    ("stages2d_rus_v17.npz", 2),
                                    ("stages2d_osh_v17.npz", 2),
                                    ("stages1d_rus_v17n3.npz", 3),
                                    ("stages2d_rus_v17n3.npz", 3)])
def test_stages(name, N):
    g = golden(name)
    O = Oracle(N=N)
    MP = Par.from_array(g["mp"])
    nX, dX = g["nX"], list(g["dX"])
    nd = len(nX)
    u = g["u"].copy()
    dt = O.timestep(u, dX, float(g["cfl"]), 0.0, 1e9, int(g["count"]), MP)
    assert abs(dt - float(g["dt"])) <= 1e-13 * float(g["dt"])
    ub = O.boundaries(u, nX, [int(g["bcs"])] * 2 * nd)
    assert rel_err(ub, g["ub"]) == 0.0
    wh = O.weno_launcher(g["ub"], nX)
    # N=3 adds central stencils (lambda_C = 1e5, eps = 1e-14): on the nearly
    # constant rest states of the tube the reference itself moves by 1e-8
    # when its input is perturbed by one ulp, so parity there is bounded by
    # that conditioning, not by the arithmetic.
    wtol = 1e-13 if N == 2 else 1e-7
    assert rel_err(wh, g["wh"]) < wtol
    qh, status = O.predictor(g["wh"], float(g["dt"]), dX, nX, MP)
    assert (status > 0).all()
    assert rel_err(qh, g["qh"]) < 1e-13
    ufv = u.copy()
    O.fv_launcher(ufv, g["qh"], nX, float(g["dt"]), dX, MP, flux=int(g["flux"]))
    tol = 1e-12 if int(g["flux"]) == 2 else 1e-14
    assert rel_err(ufv, g["u_fv"]) < tol
    if "u_centers" in g.files:  # the two passes alone (centers1/2, interfs1/2)
        for parts, key in ((1, "u_centers"), (2, "u_interfs")):
            up = u.copy()
            O.fv_parts(up, g["qh"], nX, float(g["dt"]), dX, MP, parts, flux=int(g["flux"]))
            assert rel_err(up, g[key]) < tol, key
    ustep = u.copy()
    O.ader_stepper(ustep, g["ub"], nX, float(g["dt"]), dX, MP, flux=int(g["flux"]))
    O.renorm_distortion(ustep, MP)
    assert rel_err(ustep, g["u_step"]) < max(tol, 1e-13, wtol)


def test_shock_tube_full_run(O):
    g = golden("shocktube_v17.npz")
    MP = Par.from_array(g["mp"])
    u, count, t = O.run(g["u0"], MP, float(g["tf"]), list(g["dX"]), 0, cfl=0.8)
    assert count == int(g["steps"]) == 248
    # through a shock, over 248 steps (the per-step bar is 1e-8 there)
    assert rel_err(u, g["u_end"]) < 1e-9


def test_tgv_ten_steps(O):
    g = golden("tgv2d_v17.npz")
    MP = Par.from_array(g["mp"])
    u, count, t = O.run(g["u0"], MP, 1e9, list(g["dX"]), 1, cfl=0.4, max_steps=10)
    assert rel_err(u, g["u_end"]) < 1e-12


def test_split_stepper(O):
    g = golden("split1d_v17.npz")
    MP = Par.from_array(g["mp"])
    u, count, t = O.run(g["u0"], MP, 1e9, list(g["dX"]), 0, cfl=0.8, max_steps=5,
                        split=True, half_step=True)
    assert rel_err(u, g["u_end"]) < 1e-12


def test_eigenvalues_against_numpy(O):
    rng = np.random.default_rng(7)
    for n in (3, 4, 7, 17):
        for _ in range(20):
            M = rng.standard_normal((n, n))
            ev, rc = O.eigenvalues(M)
            assert rc == 0
            ref = np.linalg.eigvals(M)
            assert abs(np.max(np.abs(ev)) - np.max(np.abs(ref))) < 1e-12 * np.max(np.abs(ref))
            assert np.allclose(np.sort(np.abs(ev)), np.sort(np.abs(ref)), atol=1e-10)


def test_predictor_newton_fallback_on_stiff_cell(O):
    """Where the reference's Picard iteration diverges (stiff relaxation),
    the oracle's Newton solve reaches the same fixed point equation's root:
    the residual of obj(q) = rhs(q) - DG_U q vanishes."""
    from phd_gb300 import problems
    u0, MP, tf, dX, bcs = problems.taylor_green(n=8, cs=10.0, mu=1e-2)
    nX = np.array([8, 8], np.int32)
    u = u0.ravel().copy()
    ub = O.boundaries(u, nX, [1] * 4)
    wh = O.weno_launcher(ub, nX)
    dt = 5 * O.timestep(u, dX, 0.8, 0.0, 1e9, 0, MP)
    qh, st = O.predictor(wh, dt, dX, nX, MP, newton_fallback=True)
    assert (st < -1000).any(), "expected Picard to fail on this stiff case"
    assert (st != -1).all() and (st != -2).all()
    assert np.isfinite(qh).all()


def test_contortion_reset():
    """contorted + reset_distortion (solvers/utils.cpp:44-85) against the
    reference, on random states, in the reference's own time loop with a
    tolerance that triggers a reset, and with two materials."""
    g = golden("contortion_v17.npz")
    MP = Par.from_array(g["mp"])
    O = Oracle(N=2, thermal=True, lset=0)
    for tol, hit in zip(g["contorted_tol"], g["contorted"]):
        q = g["Q"].ravel().copy()
        assert O.reset_contorted(q, float(tol), [MP]) == bool(hit)
        assert rel_err(q, g["reset"].ravel() if hit else g["Q"].ravel()) < 1e-14
    u, steps, t = O.run(g["run_u0"], MP, float(g["run_tf"]), list(g["run_dX"]), 0, cfl=0.8,
                        contorted_tol=float(g["run_tol"]))
    assert rel_err(u, g["run_u_end"]) < 1e-10
    g = golden("contortion_v15.npz")
    O15 = Oracle(N=2, thermal=False, lset=1)
    MPs = [Par.from_array(a) for a in g["mp"]]
    q = g["Q"].ravel().copy()
    assert O15.reset_contorted(q, 0.0, MPs)
    assert rel_err(q, g["reset"].ravel()) < 1e-14
