"""Generate the golden fixtures under tests/golden/ from the compiled
reference solver (oracle/_ref, built by `python oracle/build_ref.py v17
v17n3 v15`), one reference variant per process (`make_golden.py v17n3`
writes the N = 3 fixtures alone, `make_golden.py distance` the
re-distancing fixture alone).

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
    sysm = np.zeros((len(MPs), cnt, 3, V, V))
    mt = 4 if thermal else 3
    thermo = np.zeros((len(MPs), cnt, 3, mt, mt))
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
                sysm[m, i, d] = R.system_matrix(q, d, P)
                thermo[m, i, d] = R.thermo_acoustic_tensor(q, d, P)
            for k, dt in enumerate((1e-4, 1e-2, 1.0)):
                ode[m, i, k] = R.ode_cell(q, dt, P)
    out.update(Q=Q, Q2=Q2, X=X, flux=flux, Bdot=bdot, max_abs_eigs=mae,
               source=src, D_RUS=drus, D_OSH=dosh, D_ROE=droe, Bint=bint,
               ode=ode, ode_dt=np.array([1e-4, 1e-2, 1.0]), pressure=pres,
               temperature=temp, system_matrix=sysm, thermo_acoustic_tensor=thermo)
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
    # the two passes of fv_launcher on their own (fv.cpp:11-279)
    ucen, uint = uf.copy(), uf.copy()
    if nd == 1:
        R.centers1(ucen, qh, int(nX[0]), dt, float(dXa[0]), True, True, P, mask)
        R.interfs1(uint, qh, int(nX[0]), dt, float(dXa[0]), True, flux, P, mask)
    else:
        R.centers2(ucen, qh, int(nX[0]), int(nX[1]), dt, float(dXa[0]), float(dXa[1]),
                   True, True, P, mask)
        R.interfs2(uint, qh, int(nX[0]), int(nX[1]), dt, float(dXa[0]), float(dXa[1]),
                   True, flux, P, mask)
    ustep = uf.copy()
    R.ader_stepper(ustep, ub, nX, dt, dXa, False, flux, P, mask)
    R.renorm_single(ustep, P)
    return dict(u=uf, dt=np.array(dt), ub=ub, wh=wh, qh=qh, u_fv=ufv,
                u_centers=ucen, u_interfs=uint, u_step=ustep, nX=nX, dX=dXa, bcs=np.array(bcs), cfl=np.array(cfl),
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


def multi(R, name):
    """Level-set ghost fluid (V = 15: viscous, one level set), two sg gases.

    * distance / finite_difference / find_interface_cells on a perturbed
      circular level set (80 x 40);
    * left_star_state on random moving, sheared state pairs;
    * fill_ghost_cells on a 48 x 24 sheared shock-bubble state after a few
      reference steps;
    * full reference time loops (solvers/iterator.cpp:85-170 with the ghost
      fill): 40 x 20 and 1D helium-bubble runs.
    Distortions are sheared: at an isotropic distortion the two shear
    eigenvalues of the acoustic tensor coincide and the reference's
    eigenvector matrix in riemann_constraints (riemann.cpp:136-141) is only
    conditioned by rounding."""
    out = {}
    rng = np.random.default_rng(SEED)
    bc2 = np.zeros(4, np.int32)
    u, MPs, tf, dX, bcs = problems.shock_bubble(nx=80, ny=40, mu=1e-2, shear=0.3)
    nX = np.array(u.shape[:2], np.int32)
    phi = u[..., -1].ravel() * (1 + 0.3 * np.sin(3 * np.arange(u[..., -1].size)))
    d = np.asarray(R.distance(phi, np.array(dX), nX))
    out.update(ls_phi=phi, ls_nX=nX, ls_dX=np.array(dX), ls_dist=d,
               ls_fd=np.asarray(R.finite_difference(d, np.array(dX), nX)),
               ls_intmask=np.asarray(R.find_interface_cells(d, nX)))
    RM = [rd.to_ref_par(R, m) for m in MPs]
    cnt = 24
    QL = np.zeros((cnt, 15))
    QR = np.zeros((cnt, 15))
    nn = np.zeros((cnt, 2))
    dts = np.zeros(cnt)
    star = np.zeros((cnt, 15))
    sens = np.zeros(cnt)
    for k in range(cnt):
        QL[k] = rd.random_state(rng, MPs[0], V=14, vscale=0.2, lset=1)
        QR[k] = rd.random_state(rng, MPs[1], V=14, vscale=0.2, lset=1)
        QL[k, -1], QR[k, -1] = -0.5, 0.5
        a = rng.uniform(0, 2 * np.pi)
        nn[k] = np.cos(a), np.sin(a)
        dts[k] = (0.0, 1e-3, 1e-2)[k % 3]
        star[k] = R.left_star_state(QL[k], QR[k], RM[0], RM[1], dts[k], nn[k])
        # the reference's own movement under 1e-15 relative input noise
        for j in range(3):
            ql = QL[k] * (1 + 1e-15 * rng.standard_normal(15))
            qr = QR[k] * (1 + 1e-15 * rng.standard_normal(15))
            sp = R.left_star_state(ql, qr, RM[0], RM[1], dts[k], nn[k])
            sens[k] = max(sens[k], np.max(np.abs(sp - star[k]) / (1 + np.abs(star[k]))))
    out.update(star_QL=QL, star_QR=QR, star_n=nn, star_dt=dts, star_out=star,
               star_sens=sens)

    u, MPs, tf, dX, bcs = problems.shock_bubble(nx=48, ny=24, mu=1e-2, shear=0.3)
    nX = np.array(u.shape[:2], np.int32)
    RM = [rd.to_ref_par(R, m) for m in MPs]
    ret = R.iterator_multi(u.ravel().copy(), 0.01, nX, np.array(dX), 0.8, bc2, False,
                           False, False, 0, RM, 1e9)
    uf = np.asarray(ret[99]).copy()
    ur = uf.copy()
    g, m = R.fill_ghost_cells(ur, nX, np.array(dX), 2e-3, RM)
    out.update(fill_u=uf, fill_nX=nX, fill_dX=np.array(dX), fill_dt=np.array(2e-3),
               fill_u_out=ur, fill_grids=np.stack([np.asarray(x) for x in g]),
               fill_masks=np.stack([np.asarray(x) != 0 for x in m]))

    u, MPs, tf, dX, bcs = problems.shock_bubble(nx=40, ny=20, mu=1e-2, shear=0.3)
    nX = np.array(u.shape[:2], np.int32)
    RM = [rd.to_ref_par(R, m) for m in MPs]
    ret = R.iterator_multi(u.ravel().copy(), 0.004, nX, np.array(dX), 0.8, bc2, False,
                           False, False, 0, RM, 1e9)
    out.update(run2d_u0=u, run2d_tf=np.array(0.004), run2d_dX=np.array(dX),
               run2d_u_end=np.asarray(ret[99]).reshape(u.shape))
    u, MPs, tf, dX, bcs = problems.helium_bubble_1d(nx=200, shear=0.3)
    ret = R.iterator_multi(u.ravel().copy(), 0.05, np.array([200], np.int32),
                           np.array(dX), 0.8, np.zeros(2, np.int32), False, False,
                           False, 0, RM, 1e9)
    out.update(run1d_u0=u, run1d_tf=np.array(0.05), run1d_dX=np.array(dX),
               run1d_u_end=np.asarray(ret[99]).reshape(u.shape))
    out["mp_arrays"] = np.stack([MP.to_array() for MP in MPs])
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def multi_schemes(R, name):
    """The two-material loop (solvers/iterator.cpp:85-170, LSET = 1) with
    the reference driver's own scheme, SPLIT = True and FLUX = 1 (Roe,
    code/python/main.py:19-22), and with the other schemes and fluxes, on
    the 1D helium bubble (200 cells) and a 40 x 20 shock bubble, both with
    sheared distortions.  For the longer 1D split run (52 steps) the
    reference's own response to 1e-15 relative noise on u0 is stored beside
    it: the split scheme's analytic distortion step is ill-conditioned at
    near-isotropic distortions, so rounding grows along that run."""
    out = {}
    rng = np.random.default_rng(SEED + 11)
    cases = [  # (label, problem, tf, SPLIT, HALF_STEP, FLUX)
        ("h_split_roe", "1d", 0.01, True, True, 1),
        ("h_split_rus_nohalf", "1d", 0.01, True, False, 0),
        ("h_ader_osh", "1d", 0.01, False, True, 2),
        ("h_ader_roe_long", "1d", 0.05, False, True, 1),
        ("h_split_roe_long", "1d", 0.05, True, True, 1),
        ("b_split_roe", "2d", 0.004, True, True, 1),
        ("b_ader_osh", "2d", 0.004, False, True, 2),
    ]
    for label, kind, tf, split, half, flux in cases:
        if kind == "1d":
            u, MPs, _, dX, _ = problems.helium_bubble_1d(nx=200, shear=0.3)
        else:
            u, MPs, _, dX, _ = problems.shock_bubble(nx=40, ny=20, mu=1e-2, shear=0.3)
        nX = np.array(u.shape[:-1], np.int32)
        RM = [rd.to_ref_par(R, m) for m in MPs]
        bc = np.zeros(2 * nX.size, np.int32)

        def run(u0):
            ret = R.iterator_multi(u0.ravel().copy(), tf, nX, np.array(dX), 0.8, bc, split,
                                   half, False, flux, RM, 1e9)
            return np.asarray(ret[99]).reshape(u.shape)

        end = run(u)
        sens = np.zeros(u.shape[:-1])
        if label.endswith("_long"):
            for _ in range(3):
                un = u * (1 + 1e-15 * rng.standard_normal(u.shape))
                e = np.max(np.abs(run(un) - end) / (1 + np.abs(end)), axis=-1)
                sens = np.maximum(sens, e)
        out.update({label + "_u0": u, label + "_u_end": end, label + "_dX": np.array(dX),
                    label + "_opts": np.array([tf, split, half, flux], np.float64),
                    label + "_sens": sens,
                    label + "_mp": np.stack([MP.to_array() for MP in MPs])})
    out["labels"] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def contortion(R, name):
    """contorted + reset_distortion (solvers/utils.cpp:44-85): random
    distorted states, and the reference's own time loop (iterator.cpp:85-170
    with contorted_tol) on a sheared shock tube whose normalised distortion
    exceeds the tolerance, so that it resets."""
    rng = np.random.default_rng(SEED + 7)
    out = {}
    u, MP, tf, dX, bcs = problems.shock_tube()
    P = rd.to_ref_par(R, MP)
    Q = np.stack([rd.random_state(rng, MP, V=17) for _ in range(40)])
    m0 = []
    for q in Q:
        A = q[5:14].reshape(3, 3)
        sv = np.linalg.svd(A, compute_uv=False)
        m0.append(np.mean(sv ** 2) / np.prod(sv) ** (2 / 3))
    out["m0"] = np.array(m0)
    out["Q"] = Q
    out["contorted_tol"] = np.array([0.05, 0.2, 10.0])
    out["contorted"] = np.array([bool(R.contorted(Q.ravel().copy(), t))
                                 for t in out["contorted_tol"]])
    qr = Q.ravel().copy()
    R.reset_single(qr, P)
    out["reset"] = qr.reshape(Q.shape)
    out["mp"] = MP.to_array()
    u0 = sheared(u, MP)
    ret = R.iterator_single(u0.ravel().copy(), 0.02, np.array([200], np.int32),
                            np.array(dX), 0.8, np.zeros(2, np.int32), False, False, False, 0,
                            P, 0.02)
    out.update(run_u0=u0, run_tf=np.array(0.02), run_tol=np.array(0.02),
               run_dX=np.array(dX), run_u_end=np.asarray(ret[99]).reshape(u0.shape))
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def contortion_multi(R15, name):
    """reset_distortion with two materials (the material of each cell from
    its level set) on random distortions."""
    rng = np.random.default_rng(SEED + 8)
    u2, MPs, tf2, dX2, bcs2 = problems.shock_bubble(nx=12, ny=6, mu=1e-2)
    Q2 = u2.reshape(-1, 15).copy()
    for k in range(Q2.shape[0]):
        while True:
            A = np.eye(3) + 0.3 * rng.standard_normal((3, 3))
            if np.linalg.det(A) > 0.2:
                break
        Q2[k, 5:14] = A.ravel()
    q2 = Q2.ravel().copy()
    R15.reset_multi(q2, [rd.to_ref_par(R15, m) for m in MPs])
    np.savez_compressed(os.path.join(HERE, name), Q=Q2, reset=q2.reshape(Q2.shape),
                        mp=np.stack([m.to_array() for m in MPs]))
    print("wrote", name)


def distance_cases():
    """Level sets for the re-distancing fixture: circles with unequal
    spacings, a field with many exact zeros, a noisy field with isolated
    cells, two bubbles, 1D slabs (one with exact zeros)."""
    out = []
    nx, ny = 61, 37
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny * 2.0
    X, Y = np.meshgrid(x, y, indexing="ij")
    phi = np.sqrt((X - 0.4) ** 2 + (Y - 1.1) ** 2) - 0.3
    out.append((phi.ravel(), [1.0 / nx, 2.0 / ny], [nx, ny]))
    out.append((np.round(phi * 8).ravel() / 8, [1.0 / nx, 2.0 / ny], [nx, ny]))
    rng = np.random.default_rng(SEED)
    out.append(((rng.uniform(-1, 1, (40, 30)) + 0.6).ravel(), [0.05, 0.05], [40, 30]))
    nx, ny = 160, 80
    x = (np.arange(nx) + 0.5) * 2.0 / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y, indexing="ij")
    phi = np.minimum(np.hypot(X - 0.5, Y - 0.5) - 0.2, np.hypot(X - 1.3, Y - 0.45) - 0.15)
    out.append((phi.ravel(), [2.0 / nx, 1.0 / ny], [nx, ny]))
    out.append((np.where((np.arange(200) >= 80) & (np.arange(200) < 120), 1.0, -1.0),
                [0.005], [200]))
    out.append((np.sin(np.arange(3000) * 0.01) + 0.2, [0.001], [3000]))
    out.append((np.round(np.sin(np.arange(500) * 0.03) * 4) / 4, [0.01], [500]))
    return out


def distances(R, name):
    """distance (multi/pfmm.cpp:4-26, the vendored scikit-fmm marcher) of
    the reference build on distance_cases()."""
    arrs = {}
    cases = distance_cases()
    for k, (phi, dX, nX) in enumerate(cases):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        nXa = np.array(nX, np.int32)
        arrs["phi%d" % k] = phi
        arrs["dX%d" % k] = np.array(dX, np.float64)
        arrs["nX%d" % k] = nXa
        arrs["dist%d" % k] = np.asarray(R.distance(phi, np.array(dX, np.float64), nXa))
    arrs["count"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, name), **arrs)


def main():
    # one reference variant per process: the variants' Par types collide in
    # pybind11's registry
    variant = sys.argv[1] if len(sys.argv) > 1 else None
    if variant is None:
        import subprocess
        for v in ("v15", "v17"):
            subprocess.run([sys.executable, os.path.abspath(__file__), v], check=True)
        return 0
    if variant == "v17n3":  # the N = 3 fixtures alone (this variant only)
        R3 = rd.load("v17n3")
        if R3 is None:
            print("oracle/_ref/GPRref_v17n3 not built; run oracle/build_ref.py v17n3")
            return 1
        u0, MP, tf, dX, bcs = problems.shock_tube(nx=64)
        np.savez_compressed(os.path.join(HERE, "stages1d_rus_v17n3.npz"),
                            **stages(R3, u0, MP, dX, 0, 0.8, 10, flux=0))
        u0, MP, tf, dX, bcs = problems.taylor_green(n=12, ny=10, cs=10.0, mu=0.1)
        np.savez_compressed(os.path.join(HERE, "stages2d_rus_v17n3.npz"),
                            **stages(R3, u0, MP, dX, 1, 0.4, 2, flux=0))
        return 0
    if variant == "distance":  # the re-distancing fixture alone
        R = rd.load("v17")
        if R is None:
            print("oracle/_ref/GPRref_v17 not built; run oracle/build_ref.py v17")
            return 1
        distances(R, "distance_v17.npz")
        return 0
    if variant == "v15":
        R15 = rd.load("v15")
        multi(R15, "multi_v15.npz")
        contortion_multi(R15, "contortion_v15.npz")
        multi_schemes(R15, "multi_schemes_v15.npz")
        return 0
    if variant == "v15schemes":  # the two-material scheme fixtures alone
        R15 = rd.load("v15")
        if R15 is None:
            print("oracle/_ref/GPRref_v15 not built; run oracle/build_ref.py v15")
            return 1
        multi_schemes(R15, "multi_schemes_v15.npz")
        return 0
    R = rd.load("v17")
    if R is None:
        print("oracle/_ref/GPRref_v17 not built; run oracle/build_ref.py v17")
        return 1
    contortion(R, "contortion_v17.npz")
    pointwise(R, "pointwise_v17.npz")
    distances(R, "distance_v17.npz")

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
