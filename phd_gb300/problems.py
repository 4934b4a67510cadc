"""Synthetic GPR problems with the shapes of the workloads this library is
measured on.  Every factory returns ``(u, MP, tf, dX, bcs)`` like the
reference's problem library (code/python/tests/*), where ``u`` has shape
``(nx, V)`` or ``(nx, ny, V)`` in the reference's conserved, cell-major
layout.

* shock_tube      - 1D viscous, heat-conducting ideal-gas Riemann problem
                    (primitive_IC of code/python/tests/common.py:28-46).
* taylor_green    - 2D periodic Taylor-Green vortex (upscaled
                    code/python/tests/fluid/newtonian2.py:161-189, with
                    heat conduction so that V=17).
* stokes          - 1D first problem of Stokes on [-1, 1]
                    (code/python/tests/fluid/newtonian1.py:45-72, 400 cells).
* batched_shock_tubes - many independent shock tubes with seeded random
                    sizes, states and materials.
* shock_bubble    - 2D two-material ghost-fluid shock-bubble interaction
                    (V = 15: viscous, one level set; the material layout of
                    helium_bubble, code/python/tests/multi/material.py:43-96).
* helium_bubble_1d - 1D two-material ghost-fluid problem with the layout of
                    helium_bubble (code/python/tests/multi/material.py:43-96):
                    shocked air, air, a helium slab, air; level set +-1.
"""
import numpy as np

from .params import Cvec, material_params

BC_CODES = {"transitive": 0, "periodic": 1, "slip": 2, "stick": 3,
            "moving": 4, "symmetric": 5}


def riemann_ic(nx, dx, QL, QR, x0):
    u = np.zeros((nx, len(QL)))
    for i in range(nx):
        u[i] = QL if i * dx < x0 else QR
    return u


def shock_tube(nx=200, mu=1e-2, cs=1.0, gamma=1.4, cv=2.5, calpha=1.0,
               Pr=2.0 / 3.0, rhoL=1.0, pL=1.0, rhoR=0.125, pR=0.1,
               vL=(0, 0, 0), vR=(0, 0, 0), tf=0.2):
    MP = material_params("sg", 1.0, cv=cv, gamma=gamma, b0=cs, calpha=calpha,
                         mu=mu, Pr=Pr)
    dx = 1.0 / nx
    AL = (rhoL / MP.rho0) ** (1 / 3) * np.eye(3)
    AR = (rhoR / MP.rho0) ** (1 / 3) * np.eye(3)
    QL = Cvec(rhoL, pL, np.array(vL, float), MP, AL, np.zeros(3))
    QR = Cvec(rhoR, pR, np.array(vR, float), MP, AR, np.zeros(3))
    return riemann_ic(nx, dx, QL, QR, 0.5), MP, tf, [dx], "transitive"


def taylor_green(n=512, cs=10.0, mu=1e-2, gamma=1.4, cv=2.5, calpha=1.0,
                 Pr=2.0 / 3.0, tf=1.0, ny=None):
    ny = n if ny is None else ny
    L = 2 * np.pi
    MP = material_params("sg", 1.0, cv=cv, gamma=gamma, b0=cs, calpha=calpha,
                         mu=mu, Pr=Pr)
    dX = [L / n, L / ny]
    x = (np.arange(n) + 0.5) * dX[0]
    y = (np.arange(ny) + 0.5) * dX[1]
    X, Y = np.meshgrid(x, y, indexing="ij")
    rho = 1.0
    p = 100 / gamma + (np.cos(2 * X) + np.cos(2 * Y)) / 4
    v0 = np.sin(X) * np.cos(Y)
    v1 = -np.cos(X) * np.sin(Y)
    # E = E_1 + E_3 with A = I (E_2A = 0) and J = 0, vectorised form of Cvec
    e1 = (p - (-MP.pINF)) / (rho * (gamma - 1)) + MP.pINF / rho
    u = np.zeros((n, ny, 17))
    u[..., 0] = rho
    u[..., 1] = rho * (e1 + 0.5 * (v0 * v0 + v1 * v1))
    u[..., 2] = rho * v0
    u[..., 3] = rho * v1
    u[..., 5] = 1.0
    u[..., 9] = 1.0
    u[..., 13] = 1.0
    return u, MP, tf, dX, "periodic"


def stokes(nx=400, mu=1e-2, cs=1.0, gamma=1.4, cv=1.0, calpha=1.0, Pr=0.75,
           tf=1.0):
    MP = material_params("sg", 1.0, cv=cv, gamma=gamma, b0=cs, calpha=calpha,
                         mu=mu, Pr=Pr)
    dx = 2.0 / nx
    A = np.eye(3)
    QL = Cvec(1.0, 1 / gamma, np.array([0, 0.1, 0.0]), MP, A, np.zeros(3))
    QR = Cvec(1.0, 1 / gamma, np.array([0, -0.1, 0.0]), MP, A, np.zeros(3))
    return riemann_ic(nx, dx, QL, QR, 1.0), MP, tf, [dx], "transitive"


def batched_shock_tubes(count=512, nmin=128, nmax=2048, seed=20261203, tf=0.2):
    """Independent 1D shock tubes with cell counts ~U{nmin..nmax},
    rho ~ U[0.1, 2], p ~ logU[0.1, 10], v ~ U[-0.5, 0.5],
    mu ~ logU[1e-4, 1e-1], cs ~ U[0.5, 5], gamma ~ U[1.2, 1.67]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx = int(rng.integers(nmin, nmax + 1))
        rhoL, rhoR = rng.uniform(0.1, 2.0, 2)
        pL, pR = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 2))
        vL, vR = rng.uniform(-0.5, 0.5, 2)
        mu = float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-1))))
        cs = float(rng.uniform(0.5, 5.0))
        gamma = float(rng.uniform(1.2, 1.67))
        out.append(shock_tube(nx=nx, mu=mu, cs=cs, gamma=gamma, rhoL=rhoL,
                              pL=pL, rhoR=rhoR, pR=pR, vL=(vL, 0, 0),
                              vR=(vR, 0, 0), tf=tf))
    return out


def _shear(s):
    return np.array([[1.0, s, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def shock_bubble(nx=800, ny=400, mu=1e-4, cs=1.0, mach=1.22, x_shock=0.2,
                 radius=0.2, centre=(0.6, 0.5), rho_b=0.138, gamma_b=1.67, tf=0.8,
                 shear=0.0):
    """A Mach `mach` planar shock in an ideal gas (gamma 1.4, rho 1, p 1)
    travelling right into a circular bubble of a second gas (gamma_b, rho_b,
    p 1) on [0, 2] x [0, 1].  Both materials are viscous GPR fluids with shear
    sound speed cs and viscosity mu, without heat conduction, so V = 15:
    [rho, rho E, rho v, A, phi] with the level set phi = radius - |x - centre|
    (positive inside the bubble: material 1, as in the reference's
    helium_bubble where the second material carries phi = +1).  `shear`
    multiplies every distortion by [[1, shear, 0], [0, 1, 0], [0, 0, 1]]
    (det unchanged, energy adjusted): a parity variant whose interface
    Riemann problems are well conditioned (at an isotropic distortion the
    shear eigenvalues of the acoustic tensor coincide).  Returns
    (u[nx, ny, 15], [MP_gas, MP_bubble], tf, dX, bcs)."""
    g = 1.4
    gas = material_params("sg", 1.0, cv=2.5, gamma=g, b0=cs, mu=mu)
    bub = material_params("sg", rho_b, cv=2.5, gamma=gamma_b, b0=cs, mu=mu)
    # Rankine-Hugoniot post-shock state for a shock of Mach `mach` into (1, 1)
    M2 = mach * mach
    p2 = 1.0 + 2 * g / (g + 1) * (M2 - 1)
    r2 = (g + 1) * M2 / ((g - 1) * M2 + 2)
    s = mach * np.sqrt(g)
    v2 = s * (1 - 1 / r2)
    dX = [2.0 / nx, 1.0 / ny]
    x = (np.arange(nx) + 0.5) * dX[0]
    y = (np.arange(ny) + 0.5) * dX[1]
    X, Y = np.meshgrid(x, y, indexing="ij")
    phi = radius - np.sqrt((X - centre[0]) ** 2 + (Y - centre[1]) ** 2)

    def Q(rho, p, v, MP):
        A = (rho / MP.rho0) ** (1 / 3) * _shear(shear)
        return np.concatenate([Cvec(rho, p, np.array([v, 0.0, 0.0]), MP, A), [0.0]])

    Qpost, Qpre, Qbub = Q(r2, p2, v2, gas), Q(1.0, 1.0, 0.0, gas), Q(rho_b, 1.0, 0.0, bub)
    u = np.where((X < x_shock)[..., None], Qpost, Qpre)
    u = np.where((phi >= 0)[..., None], Qbub, u)
    u[..., -1] = phi
    return np.ascontiguousarray(u), [gas, bub], tf, dX, "transitive"


def helium_bubble_1d(nx=200, mu=1e-2, cs=1.0, mach=1.22, rho_b=0.138, gamma_b=1.67,
                     tf=0.3, shear=0.0):
    """1D counterpart of shock_bubble with the layout of the reference's
    helium_bubble: a Mach `mach` shock in air (gamma 1.4, rho 1, p 1) at
    x < 0.05 moving right, air up to 0.4, a slab of the second gas on
    [0.4, 0.6), air beyond; level set -1 in air, +1 in the slab (it is
    re-distanced every step).  V = 15.  Returns (u[nx, 15], MPs, tf, dX,
    bcs)."""
    g = 1.4
    gas = material_params("sg", 1.0, cv=2.5, gamma=g, b0=cs, mu=mu)
    bub = material_params("sg", rho_b, cv=2.5, gamma=gamma_b, b0=cs, mu=mu)
    M2 = mach * mach
    p2 = 1.0 + 2 * g / (g + 1) * (M2 - 1)
    r2 = (g + 1) * M2 / ((g - 1) * M2 + 2)
    v2 = mach * np.sqrt(g) * (1 - 1 / r2)
    dx = 1.0 / nx

    def Q(rho, p, v, MP, phi):
        A = (rho / MP.rho0) ** (1 / 3) * _shear(shear)
        return np.concatenate([Cvec(rho, p, np.array([v, 0.0, 0.0]), MP, A), [phi]])

    u = np.zeros((nx, 15))
    for i in range(nx):
        x = i * dx
        if x < 0.05:
            u[i] = Q(r2, p2, v2, gas, -1.0)
        elif 0.4 <= x < 0.6:
            u[i] = Q(rho_b, 1.0, 0.0, bub, 1.0)
        else:
            u[i] = Q(1.0, 1.0, 0.0, gas, -1.0)
    return u, [gas, bub], tf, [dx], "transitive"
