"""Generate the golden fixtures under tests/golden/ from the compiled
reference solver (oracle/_ref, built by `python oracle/build_ref.py v17
v17n3 v14`).

Every array in the fixtures is an output of the reference's own C++ code
(haranjackson/phd, code/cpp/src) on seeded inputs; inputs are stored beside
the outputs.  The fixtures pin the CPU oracle (tests/test_oracle_golden.py)
and, through it, the CUDA kernels.  Run here, where the reference sources
exist:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)

import refdrive as rd  # noqa: E402
from phd_gb300 import problems  # noqa: E402
from phd_gb300.params import material_params  # noqa: E402

SEED = 20261203


def pointwise(R, name, thermal=True):
    V = R.NV()
    rng = np.random.default_rng(SEED)
    MPs = [material_params("sg", 1.0, cv=2.5, gamma=1.4, b0=1.0, calpha=1.0,
                           mu=1e-2, Pr=2 / 3),
           material_params("sg", 1.3, cv=1.7, gamma=1.67, pINF=0.3, b0=2.0,
                           calpha=0.7, mu=3e-3, Pr=0.75)]
    if not thermal:
        MPs = [material_params("sg", 1.0, cv=1.0, gamma=1.4, b0=10.0, mu=1e-2)]
    out = {}
    cnt = 24
    Q = np.zeros((len(MPs), cnt, V))
    Q2 = np.zeros_like(Q)
    X = rng.standard_normal((len(MPs), cnt, V))
    flux = np.zeros((len(MPs), cnt, 3, V))
    bdot = np.zeros_like(flux)
    mae = np.zeros((len(MPs), cnt, 3))
    src = np.zeros((len(MPs), cnt, V))
    drus = np.zeros((len(MPs), cnt, 3, V))
    dosh = np.zeros_like(drus)
    droe = np.zeros_like(drus)
    bint = np.zeros_like(drus)
    ode = np.zeros((len(MPs), cnt, 3, V))
    pres = np.zeros((len(MPs), cnt))
    temp = np.zeros((len(MPs), cnt))
    for m, MP in enumerate(MPs):
        P = rd.to_ref_par(R, MP)
        for i in range(cnt):
            q = rd.random_state(rng, MP, V=V)
            q2 = rd.random_state(rng, MP, V=V)
            Q[m, i], Q2[m, i] = q, q2
            src[m, i] = R.source(q, P)
            pres[m, i] = R.pressure(q, P)
            temp[m, i] = R.temperature(q, P) if thermal else 0.0
            for d in range(3):
                flux[m, i, d] = R.flux(q, d, P)
                bdot[m, i, d] = R.Bdot(q, X[m, i], d, P)
                mae[m, i, d] = R.max_abs_eigs(q, d, P)
                drus[m, i, d] = R.D(0, q, q2, d, P)
                dosh[m, i, d] = R.D(2, q, q2, d, P)
                droe[m, i, d] = R.D(1, q, q2, d, P)
                bint[m, i, d] = R.Bint(q, q2, d, P)
            for k, dt in enumerate((1e-4, 1e-2, 1.0)):
                ode[m, i, k] = R.ode_cell(q, dt, P)
    out.update(Q=Q, Q2=Q2, X=X, flux=flux, Bdot=bdot, max_abs_eigs=mae,
               source=src, D_RUS=drus, D_OSH=dosh, D_ROE=droe, Bint=bint,
               ode=ode, ode_dt=np.array([1e-4, 1e-2, 1.0]), pressure=pres,
               temperature=temp)
    out["mp_" + "arrays"] = np.stack([MP.to_array() for MP in MPs])
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def stages(R, u0, MP, dX, bcs, cfl, presteps, flux=0):
    """Reference stage outputs for one step taken after `presteps` steps."""
    u, _, _ = rd.run_ref(R, u0, MP, 1e9, dX, bcs, cfl=cfl, flux=flux,
                         max_steps=presteps) if presteps else (u0.copy(), 0, 0)
    P = rd.to_ref_par(R, MP)
    nX = np.array(u0.shape[:-1], np.int32)
    nd = len(nX)
    V = u0.shape[-1]
    N = R.N()
    uf = np.ascontiguousarray(u, dtype=np.float64).ravel()
    dXa = np.asarray(dX, dtype=np.float64)
    dt = R.timestep_single(uf, dXa, cfl, 0.0, 1e9, presteps, P)
    ub = np.zeros(int(np.prod(nX + 2 * N)) * V)
    R.boundaries(uf, ub, nX, np.array([bcs] * 2 * nd, np.int32))
    wh = np.zeros(int(np.prod(nX + 2)) * N ** nd * V)
    R.weno_launcher(wh, ub, nX, P)
    qh = np.full(int(np.prod(nX + 2)) * N ** (nd + 1) * V, np.nan)
    mask = np.ones(int(np.prod(nX + 2)), bool)
    R.predictor(qh, wh, dt, dXa, False, False, P, mask)
    assert not np.isnan(qh).any(), "reference Picard did not converge"
    ufv = uf.copy()
    R.fv_launcher(ufv, qh, nX, dt, dXa, True, True, flux, P, mask)
    ustep = uf.copy()
    R.ader_stepper(ustep, ub, nX, dt, dXa, False, flux, P, mask)
    R.renorm_single(ustep, P)
    return dict(u=uf, dt=np.array(dt), ub=ub, wh=wh, qh=qh, u_fv=ufv,
                u_step=ustep, nX=nX, dX=dXa, bcs=np.array(bcs), cfl=np.array(cfl),
                count=np.array(presteps), flux=np.array(flux),
                mp=MP.to_array())


def sheared(u0, MP, shear=0.3):
    """Same tube with A = rho^1/3 [[1, shear, 0], [0, 1, 0], [0, 0, 1]]
    (det A unchanged) and the energy adjusted for the extra E_2A."""
    from phd_gb300.params import Cvec
    u = u0.copy()
    for i in range(u.shape[0]):
        rho = u[i, 0]
        v = u[i, 2:5] / rho
        A = u[i, 5:14].reshape(3, 3)
        p_old = None
        # recover p from the isotropic state, then rebuild with sheared A
        from oracle import Oracle
        p_old = Oracle().pressure(u[i], MP)
        A2 = A @ np.array([[1, shear, 0], [0, 1, 0], [0, 0, 1.0]])
        u[i] = Cvec(rho, p_old, v, MP, A2, u[i, 14:17] / rho)
    return u


def main():
    R = rd.load("v17")
    if R is None:
        print("oracle/_ref/GPRref_v17 not built; run oracle/build_ref.py v17")
        return 1
    pointwise(R, "pointwise_v17.npz")

    # 1D shock tube (200 cells): stages after 20 steps, Rusanov and Osher
    u0, MP, tf, dX, bcs = problems.shock_tube()
    np.savez_compressed(os.path.join(HERE, "stages1d_rus_v17.npz"),
                        **stages(R, u0, MP, dX, 0, 0.8, 20, flux=0))
    np.savez_compressed(os.path.join(HERE, "stages1d_osh_v17.npz"),
                        **stages(R, u0, MP, dX, 0, 0.8, 20, flux=2))
    # full run to t_end = 0.2
    uend, count, t = rd.run_ref(R, u0, MP, tf, dX, 0, cfl=0.8)
    np.savez_compressed(os.path.join(HERE, "shocktube_v17.npz"), u0=u0,
                        u_end=uend, steps=np.array(count), t=np.array(t),
                        mp=MP.to_array(), dX=np.array(dX), tf=np.array(tf))
    print("shock tube steps", count)

    # 2D Taylor-Green (non-square, non-stiff enough for the reference Picard)
    u0, MP, tf, dX, bcs = problems.taylor_green(n=12, ny=10, cs=10.0, mu=0.1)
    np.savez_compressed(os.path.join(HERE, "stages2d_rus_v17.npz"),
                        **stages(R, u0, MP, dX, 1, 0.4, 2, flux=0))
    np.savez_compressed(os.path.join(HERE, "stages2d_osh_v17.npz"),
                        **stages(R, u0, MP, dX, 1, 0.4, 1, flux=2))
    # 10 steps need a less stiff relaxation (mu = 1) for the reference Picard
    # iteration to converge once the first-five-steps dt reduction ends
    u0, MP, tf, dX, bcs = problems.taylor_green(n=12, ny=10, cs=10.0, mu=1.0)
    uend, count, t = rd.run_ref(R, u0, MP, 1e9, dX, 1, cfl=0.4, max_steps=10)
    np.savez_compressed(os.path.join(HERE, "tgv2d_v17.npz"), u0=u0, u_end=uend,
                        steps=np.array(count), mp=MP.to_array(), dX=np.array(dX))

    # split stepper (ODE half steps + WENO + midstepper + FV), 1D, 5 steps.
    # The isotropic tube (A = rho^1/3 I) sits on the reference's u0 >= 1e-12
    # branch switch of the distortion ODE (relaxation/analytic.cpp:89), where
    # one ulp of input moves the reference's own result by 1e-3; a sheared
    # distortion keeps the ODE step well conditioned.
    u0, MP, tf, dX, bcs = problems.shock_tube()
    u0 = sheared(u0, MP)
    uend, count, t = rd.run_ref(R, u0, MP, 1e9, dX, 0, cfl=0.8, max_steps=5,
                                split=True, half_step=True)
    np.savez_compressed(os.path.join(HERE, "split1d_v17.npz"), u0=u0, u_end=uend,
                        steps=np.array(count), mp=MP.to_array(), dX=np.array(dX))

    R3 = rd.load("v17n3")
    if R3 is not None:
        u0, MP, tf, dX, bcs = problems.shock_tube(nx=64)
        np.savez_compressed(os.path.join(HERE, "stages1d_rus_v17n3.npz"),
                            **stages(R3, u0, MP, dX, 0, 0.8, 10, flux=0))
    return 0


if __name__ == "__main__":
    sys.exit(main())
