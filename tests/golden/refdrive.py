"""Helpers that drive the compiled reference solver (oracle/_ref, built by
oracle/build_ref.py from the reference sources).  Only make_golden.py and
tests that are skipped when oracle/_ref is absent import this module; it
never runs on a GPU host."""
import importlib
import os
import sys

# One OpenMP thread, set before the reference module (and its OpenMP
# runtime) loads: the reference's 2D boundary fill is an OpenMP loop whose
# iterations read cells that other iterations write (multi/fill.cpp:220-233),
# so with several threads its result depends on the schedule (8e-4 on a
# 40 x 20 shock bubble after 4 steps).  One thread gives the loop's
# sequential (i, j) order, the order the oracle and the device fill follow.
os.environ["OMP_NUM_THREADS"] = "1"

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "..", "..", "oracle", "_ref")


def load(variant="v17"):
    """Import GPRref_<variant>; returns None when it has not been built."""
    path = os.path.abspath(REF_DIR)
    if not os.path.isdir(path):
        return None
    if path not in sys.path:
        sys.path.insert(0, path)
    try:
        return importlib.import_module("GPRref_%s" % variant)
    except ImportError:
        return None


def to_ref_par(R, MP):
    """phd_gb300.params.Par -> the reference's Par."""
    P = R.Par()
    for k in ("EOS", "rho0", "Tref", "cv", "pINF", "Gamma0", "c02", "s",
              "alpha", "beta", "gamma", "A", "B", "R1", "R2", "b02", "mu",
              "tau0", "sigmaY", "n", "calpha2", "kappa"):
        setattr(P, k, getattr(MP, k))
    P.SOLID = bool(MP.SOLID)
    P.POWER_LAW = bool(MP.POWER_LAW)
    P.BINGHAM = bool(MP.BINGHAM)
    P.MULTI = False
    P.dp = np.asarray(MP.dp, dtype=np.float64)
    P.REACTION = -1
    return P


def random_state(rng, MP, V=17, vscale=1.0, jscale=1.0, lset=0):
    """Random admissible conserved state in the spirit of the reference's
    generate_vector (code/cpp/bindings/bindings_tests/test_functions.py:9-17):
    random A with det A > 0, rho = det(A) rho0, random p, v, J."""
    from phd_gb300.params import Cvec
    while True:
        A = np.eye(3) + 0.25 * rng.standard_normal((3, 3))
        if np.linalg.det(A) > 0.2:
            break
    rho = np.linalg.det(A) * MP.rho0
    p = rng.uniform(0.2, 2.0)
    v = vscale * rng.uniform(-1, 1, 3)
    J = jscale * rng.uniform(-1, 1, 3) if V >= 17 else None
    Q = Cvec(rho, p, v, MP, A, J)
    if lset:
        Q = np.concatenate([Q, rng.uniform(-1, 1, lset)])
    return Q


def run_ref(R, u0, MP, tf, dX, bcs, cfl=0.8, flux=0, max_steps=None,
            split=False, half_step=True, stiff=False):
    """Reference time loop for one material: solvers/iterator.cpp:109-167
    restricted to boundaries -> timestep -> stepper -> renorm (no level set,
    no contortion reset)."""
    P = to_ref_par(R, MP)
    shape = u0.shape
    nX = np.array(shape[:-1], dtype=np.int32)
    nd = len(nX)
    V = shape[-1]
    N = R.N()
    u = np.ascontiguousarray(u0, dtype=np.float64).ravel().copy()
    ub = np.zeros(int(np.prod(nX + 2 * N)) * V)
    mask = np.ones(int(np.prod(nX + 2)), dtype=bool)
    bc = np.array([bcs] * 2 * nd, dtype=np.int32)
    dXa = np.asarray(dX, dtype=np.float64)
    t, count = 0.0, 0
    while t < tf:
        dt = R.timestep_single(u, dXa, cfl, t, tf, count, P)
        R.boundaries(u, ub, nX, bc)
        if split:
            R.split_stepper(u, ub, nX, dt, dXa, half_step, flux, P, mask)
        else:
            R.ader_stepper(u, ub, nX, dt, dXa, stiff, flux, P, mask)
        R.renorm_single(u, P)
        t += dt
        count += 1
        if max_steps is not None and count >= max_steps:
            break
    return u.reshape(shape), count, t
