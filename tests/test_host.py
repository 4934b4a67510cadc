"""Host-side checks that need no GPU: the C-ABI library builds, loads and
exports every entry point include/gpr_gb300.h declares; the parameter
builder matches the reference's defaults; problem factories have the
configured shapes."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "gpr_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gpr_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from phd_gb300 import _lib
    path = _lib.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding table covers them
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_library_reports_version_without_gpu():
    from phd_gb300 import _lib
    lib = _lib.load()
    assert lib.gpr_version() >= 100
    buf = (ctypes.c_int32 * 8)()
    n = lib.gpr_supported_nvars(ctypes.cast(buf, ctypes.c_void_p), 8)
    assert 17 in list(buf)[:n]


# The names the reference's GPRpy module binds (bindings/bindings.cpp:69-265),
# split into those this package mirrors and those it leaves out: the EOS /
# Jacobian scalars and the inner steps of bound functions (computed inside
# the kernels), the reactive and multi-phase hooks, the SciPy ports (replaced
# by the device Newton pass), the polynomial objects and forward stencil
# matrices, and rotate_distortion (off in options.h:16).
BOUND = """options.N options.NV options.VISCOUS options.THERMAL options.MULTI options.LSET
classes.Params classes.Par boundaries extend_mask
multi.renormalize_levelsets multi.finite_difference multi.find_interface_cells
multi.fill_boundary_cells multi.fill_neighbor_cells multi.fill_ghost_cells
multi.material_indicator system.flux system.source system.Bdot system.system_matrix
system.max_abs_eigs system.thermo_acoustic_tensor system.multi.left_star_state
system.multi.distance solvers.common.scaled_nodes solvers.common.scaled_weights
solvers.common.end_values solvers.common.derivative_values solvers.extended_dimensions
solvers.ader_stepper solvers.ader_stepper_para solvers.split_stepper
solvers.split_stepper_para solvers.iterator solvers.make_u solvers.contorted
solvers.timestep solvers.renorm_distortion solvers.weno.oscillation_indicator
solvers.weno.weno_launcher solvers.split.midstepper solvers.split.ode_launcher
solvers.fv.Bint solvers.fv.D_RUS solvers.fv.D_ROE solvers.fv.D_OSH solvers.fv.centers1
solvers.fv.centers2 solvers.fv.interfs1 solvers.fv.interfs2 solvers.fv.fv_launcher""".split()
NOT_BOUND = """classes.poly scipy.lgmres_wrapper scipy.newton_krylov system.block
system.reaction_rate system.ode_stepper_numerical system.dFdP system.dPdQ
system.multi.eigen system.multi.riemann_constraints system.multi.star_stepper
solvers.common.basis_polys solvers.rotate_distortion solvers.weno.coefficient_matrices
solvers.split.analyticSolver_distortion solvers.split.analyticSolver_thermal
solvers.split.stiff_ode_solve solvers.split.runge_kutta_launcher
solvers.split.ode_stepper_numerical system.variables.pressure
system.variables.temperature system.variables.dEdρ system.variables.reaction_rate
system.variables.solve_multi system.variables.temperature_mg""".split()


def _lookup(mod, name):
    for part in name.split("."):
        mod = getattr(mod, part)
    return mod


def test_python_mirror_binds_the_reference_names():
    import phd_gb300 as G
    assert len(BOUND) + len(NOT_BOUND) == 77 and not set(BOUND) & set(NOT_BOUND)
    missing = [n for n in BOUND if not callable(_lookup(G, n))]
    assert not missing, missing
    for n in NOT_BOUND:
        with pytest.raises(AttributeError):
            _lookup(G, n)


def test_scratch_queries_and_argument_errors_without_gpu():
    from phd_gb300 import _lib
    lib = _lib.load()
    nX = (ctypes.c_int32 * 2)(512, 512)
    p = ctypes.cast(nX, ctypes.c_void_p)
    assert lib.gpr_ader_scratch_doubles(p, 2, 17) > 514 * 514 * 8 * 17
    assert lib.gpr_ader_scratch_doubles(p, 2, 16) == -3  # unsupported V
    assert lib.gpr_ader_scratch_doubles(p, 3, 17) == -1  # bad ndim
    bad = (ctypes.c_int32 * 1)(0)
    assert lib.gpr_weno_scratch_doubles(ctypes.cast(bad, ctypes.c_void_p), 1, 17) == -1


def test_material_params_defaults():
    from phd_gb300.params import material_params, Par
    MP = material_params("sg", 1.0, cv=2.5, gamma=1.4, b0=1.0, calpha=1.0, mu=1e-2, Pr=2 / 3)
    assert MP.EOS == 0 and MP.n == 1 and not MP.POWER_LAW and not MP.SOLID
    assert MP.b02 == 1.0 and MP.calpha2 == 1.0 and MP.pINF == 0 and MP.Tref == 0
    assert abs(MP.kappa - 0.0525) < 1e-15
    back = Par.from_array(MP.to_array())
    for k in ("rho0", "cv", "gamma", "b02", "mu", "n", "calpha2", "kappa"):
        assert getattr(back, k) == getattr(MP, k)
    elastic = material_params("sg", 1.0, gamma=1.4, b0=1.0)
    assert elastic.SOLID and not elastic.POWER_LAW


def test_problem_shapes():
    from phd_gb300 import problems
    u, MP, tf, dX, bcs = problems.shock_tube()
    assert u.shape == (200, 17) and tf == 0.2 and bcs == "transitive"
    assert np.all(u[:100, 0] == 1.0) and np.all(u[100:, 0] == 0.125)
    u, MP, tf, dX, bcs = problems.taylor_green(n=8)
    assert u.shape == (8, 8, 17) and bcs == "periodic"
    u, MP, tf, dX, bcs = problems.stokes()
    assert u.shape == (400, 17)
    insts = problems.batched_shock_tubes(count=4)
    assert len(insts) == 4 and all(128 <= i[0].shape[0] <= 2048 for i in insts)


def test_cvec_matches_reference_energy():
    """Cvec reproduces the reference's conserved energy on the golden states."""
    from conftest import golden
    from phd_gb300.params import Par
    from oracle import Oracle
    g = golden("pointwise_v17.npz")
    O = Oracle()
    for m in range(g["Q"].shape[0]):
        MP = Par.from_array(g["mp_arrays"][m])
        for Q in g["Q"][m][:6]:
            p = O.pressure(Q, MP)
            from phd_gb300.params import Cvec
            Q2 = Cvec(Q[0], p, Q[2:5] / Q[0], MP, Q[5:14].reshape(3, 3), Q[14:17] / Q[0])
            assert np.allclose(Q2, Q, rtol=1e-13, atol=1e-13)


def test_snapshot_files_in_the_reference_format(tmp_path):
    """store.py:7-14 / main.py:47-52: leading set snapshots, saved as one
    array under <problem>_<N>_<cfl>_<SPLIT>_<FLUX>_<time>.npy."""
    import numpy as np
    from phd_gb300 import store
    shape = (5, 3)
    sol = [np.full(15, float(k)) for k in range(4)] + [None] * 95 + [np.full(15, 9.0)]
    ul = store.snapshots(sol, shape)
    assert len(ul) == 4 and ul[3].shape == shape and ul[2][0, 0] == 2.0

    def shock_tube():
        pass
    path = store.save_results(ul, shock_tube, 2, 0.8, True, 1, directory=str(tmp_path),
                              stamp=1700000000)
    assert os.path.basename(path) == "shock_tube_2_0.8_True_1_1700000000.npy"
    back = np.load(path)
    assert back.shape == (4,) + shape and back[1, 0, 0] == 1.0


def test_adjoint_field_jacobian_matches_finite_differences():
    """The chain rule from user parameters (mu, cs, calpha, gamma) to the six
    device fields the backward step differentiates, by complex steps, against
    central differences of the same material builder."""
    from phd_gb300.adjoint import FIELDS, dev_fields, field_jacobian
    from phd_gb300.params import material_params

    def make_par(th):
        return material_params("sg", 1.0, cv=1.0, gamma=th[3], b0=th[1], calpha=th[2],
                               mu=th[0], Pr=0.75)

    theta = np.array([1.2e-2, 0.9, 1.1, 1.4])
    J = field_jacobian(make_par, theta)
    assert J.shape == (len(FIELDS), theta.size)
    for j in range(theta.size):
        h = 1e-6 * theta[j]
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        fd = (np.array(dev_fields(make_par(tp))) - np.array(dev_fields(make_par(tm)))) / (2 * h)
        scale = np.abs(fd) + np.abs(J[:, j]) + 1e-12
        assert (np.abs(J[:, j] - fd) / scale).max() < 1e-7, (j, J[:, j], fd)


def test_scheme_constants_without_gpu():
    """solvers.common.* and solvers.weno.oscillation_indicator: the constants
    the kernels use, from the library on the host, against the oracle's
    (pinned by the golden stage tests) and the closed forms."""
    import phd_gb300 as G
    from oracle import Oracle
    c = Oracle().constants()
    s3 = 1 / np.sqrt(3)
    nodes = G.solvers.common.scaled_nodes()
    assert np.allclose(nodes, [(1 - s3) / 2, (1 + s3) / 2], rtol=0, atol=1e-16)
    assert np.allclose(nodes, c["nodes"], rtol=0, atol=1e-16)
    assert np.allclose(G.solvers.common.scaled_weights(), c["weights"], rtol=0, atol=1e-15)
    assert np.allclose(G.solvers.common.end_values(), c["endvals"], rtol=0, atol=1e-15)
    assert np.allclose(G.solvers.common.derivative_values(), c["dervals"], rtol=0, atol=1e-14)
    assert np.allclose(G.solvers.weno.oscillation_indicator(), c["sig"], rtol=0, atol=1e-13)


def test_scheme_constants_at_three_nodes_without_gpu():
    """The N = 3 constants the node kernels use, from the library on the host,
    against the N = 3 oracle's (pinned by the golden N = 3 stages) and the
    closed forms of three-point Gauss-Legendre on [0, 1]."""
    from oracle import Oracle
    from phd_gb300.order import for_order
    c = Oracle(N=3).constants()
    k = for_order(3).scheme_constants()
    s = np.sqrt(0.6)
    assert np.allclose(k["nodes"], [(1 - s) / 2, 0.5, (1 + s) / 2], rtol=0, atol=1e-16)
    assert np.allclose(k["weights"], [5 / 18, 8 / 18, 5 / 18], rtol=0, atol=1e-15)
    for key in ("nodes", "weights", "endvals", "dervals"):
        assert np.allclose(k[key], c[key], rtol=0, atol=1e-13), key
    assert np.allclose(k["sig"], c["sig"], rtol=1e-13, atol=1e-12)
