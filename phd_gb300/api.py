"""GPRpy-compatible entry points over the CUDA library.

Each function keeps the name, argument order and in-place semantics of the
reference's pybind11 module `GPRpy` (code/cpp/bindings/bindings.cpp:59-265):
arrays are float64 (grid data, in place), int32 (nX, boundary codes) and bool
(masks).  Grid data must be contiguous float64 CUDA tensors; nX, dX and the
boundary codes may be host sequences.  Work is enqueued on torch's current
CUDA stream and errors are raised as RuntimeError.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .params import Par

N = 2


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(t, name, dtype=torch.float64):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != dtype:
        raise TypeError("%s must be %s, got %s" % (name, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return ctypes.c_void_p(t.data_ptr())


def _mask_ptr(mask, n):
    if mask is None:
        return None, None
    if mask.dtype == torch.bool:
        mask = mask.view(torch.uint8)
    if mask.numel() != n:
        raise ValueError("mask has %d entries, expected %d" % (mask.numel(), n))
    return _dev(mask, "mask", torch.uint8), mask


def _i32(a):
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
    return arr, arr.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return arr, arr.ctypes.data_as(ctypes.c_void_p)


def _par(MP):
    c = MP.to_ctypes()
    return c, ctypes.cast(ctypes.pointer(c), ctypes.c_void_p)


def _nvar(t, ncell):
    v = t.numel() // ncell
    if v * ncell != t.numel():
        raise ValueError("tensor size %d is not a multiple of %d cells" % (t.numel(), ncell))
    return v


def _scratch(ndoubles, like):
    return torch.empty(max(int(ndoubles), 1), dtype=torch.float64, device=like.device)


# ---------------------------------------------------------------------------
# grid helpers

def boundaries(u, ub, nX, boundaryTypes):
    """GPRpy.boundaries (etc/grid.h:6)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    bca, pb = _i32(boundaryTypes)
    nd = nXa.size
    if bca.size != 2 * nd:
        raise ValueError("expected %d boundary codes" % (2 * nd))
    V = _nvar(u, int(np.prod(nXa)))
    if ub.numel() != int(np.prod(nXa + 2 * N)) * V:
        raise ValueError("ub has the wrong size")
    _lib.check(lib.gpr_boundaries(_dev(u, "u"), _dev(ub, "ub"), pn, nd, pb, V, _stream()),
               "boundaries")
    return ub


def extend_mask(mask, maskb, nX):
    """GPRpy.extend_mask (etc/grid.h:10)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    pm, _ = _mask_ptr(mask, int(np.prod(nXa)))
    pmb, _ = _mask_ptr(maskb, int(np.prod(nXa + 2)))
    _lib.check(lib.gpr_extend_mask(pm, pmb, pn, nXa.size, _stream()), "extend_mask")
    return maskb


def extended_dimensions(nX, ext):
    return int(np.prod(np.asarray(nX) + 2 * ext))


# ---------------------------------------------------------------------------
# stages

def weno_launcher(wh, ub, nX, MP=None):
    """GPRpy.solvers.weno.weno_launcher (solvers/weno/weno.h:6)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    nd = nXa.size
    V = _nvar(ub, int(np.prod(nXa + 2 * N)))
    scr = _scratch(lib.gpr_weno_scratch_doubles(pn, nd, V), ub)
    _lib.check(lib.gpr_weno_launcher(_dev(wh, "wh"), _dev(ub, "ub"), pn, nd, _dev(scr, "s"),
                                     V, _stream()), "weno_launcher")
    return wh


def predictor(qh, wh, dt, dX, STIFF, STIFF_IG, MP, mask, status=None):
    """GPRpy.solvers.dg.predictor (solvers/dg/dg.h:7).  `status` (optional
    int32 CUDA tensor, one entry per predictor cell) receives the per-cell
    solver status and Picard iteration count."""
    lib = _lib.load()
    dXa, pd = _f64(dX)
    nd = dXa.size
    ncb = mask.numel()
    V = _nvar(wh, ncb * N ** nd)
    nX = _grid_from_mask(mask, nd, qh, wh)
    nXa, pn = _i32(nX)
    pm, _ = _mask_ptr(mask, ncb)
    c, pp = _par(MP)
    ps = _dev(status, "status", torch.int32) if status is not None else None
    _lib.check(lib.gpr_predictor(_dev(qh, "qh"), _dev(wh, "wh"), float(dt), pd, nd, pn,
                                 int(bool(STIFF)), pp, pm, ps, V, _stream()), "predictor")
    return qh


_GRID = {}


def set_grid(nX):
    """Registers the interior grid size for the stage calls that, as in the
    reference, do not take nX (predictor): the last grid passed to any call
    with nX is used."""
    _GRID["nX"] = tuple(int(x) for x in nX)


def _grid_from_mask(mask, nd, *tensors):
    nX = _GRID.get("nX")
    if nX is None or len(nX) != nd or int(np.prod(np.asarray(nX) + 2)) != mask.numel():
        if nd == 1:
            return (mask.numel() - 2,)
        raise ValueError("call set_grid(nX) (or a stage taking nX) before predictor in 2D")
    return nX


def fv_launcher(u, rec, nX, dt, dX, SOURCES, TIME, FLUX, MP, mask):
    """GPRpy.solvers.fv.fv_launcher (solvers/fv/fv.h:17)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    set_grid(nXa)
    dXa, pd = _f64(dX)
    nd = nXa.size
    V = _nvar(u, int(np.prod(nXa)))
    pm, _ = _mask_ptr(mask, int(np.prod(nXa + 2)))
    c, pp = _par(MP)
    scr = _scratch(lib.gpr_fv_scratch_doubles(pn, nd, V), u)
    _lib.check(lib.gpr_fv_launcher(_dev(u, "u"), _dev(rec, "rec"), pn, float(dt), pd, nd,
                                   int(bool(SOURCES)), int(bool(TIME)), int(FLUX), pp, pm,
                                   _dev(scr, "s"), V, _stream()), "fv_launcher")
    return u


def _fv_part(u, rec, nX, dt, dX, SOURCES, TIME, FLUX, MP, mask, part):
    lib = _lib.load()
    nXa, pn = _i32(nX)
    set_grid(nXa)
    dXa, pd = _f64(dX)
    nd = nXa.size
    V = _nvar(u, int(np.prod(nXa)))
    pm, _ = _mask_ptr(mask, int(np.prod(nXa + 2)))
    c, pp = _par(MP)
    if part == "centers":
        _lib.check(lib.gpr_fv_centers(_dev(u, "u"), _dev(rec, "rec"), pn, float(dt), pd, nd,
                                      int(bool(SOURCES)), int(bool(TIME)), pp, pm, V,
                                      _stream()), "centers")
    else:
        scr = _scratch(lib.gpr_fv_scratch_doubles(pn, nd, V), u)
        _lib.check(lib.gpr_fv_interfs(_dev(u, "u"), _dev(rec, "rec"), pn, float(dt), pd, nd,
                                      int(bool(TIME)), int(FLUX), pp, pm, _dev(scr, "s"), V,
                                      _stream()), "interfs")
    return u


def centers1(u, rec, nx, dt, dx, SOURCES, TIME, MP, mask):
    """GPRpy.solvers.fv.centers1 (solvers/fv/fv.h:7): the volume term of the
    FV update (sources and non-conservative products), in place on u."""
    return _fv_part(u, rec, [nx], dt, [dx], SOURCES, TIME, 0, MP, mask, "centers")


def centers2(u, rec, nx, ny, dt, dx, dy, SOURCES, TIME, MP, mask):
    """GPRpy.solvers.fv.centers2 (solvers/fv/fv.h:9)."""
    return _fv_part(u, rec, [nx, ny], dt, [dx, dy], SOURCES, TIME, 0, MP, mask, "centers")


def interfs1(u, rec, nx, dt, dx, TIME, FLUX, MP, mask):
    """GPRpy.solvers.fv.interfs1 (solvers/fv/fv.h:12): the interface terms
    of the FV update (fluxes and path integrals), in place on u."""
    return _fv_part(u, rec, [nx], dt, [dx], False, TIME, FLUX, MP, mask, "interfs")


def interfs2(u, rec, nx, ny, dt, dx, dy, TIME, FLUX, MP, mask):
    """GPRpy.solvers.fv.interfs2 (solvers/fv/fv.h:14)."""
    return _fv_part(u, rec, [nx, ny], dt, [dx, dy], False, TIME, FLUX, MP, mask, "interfs")


def ader_stepper(u, ub, nX, dt, dX, STIFF, FLUX, MP, mask, status=None):
    """GPRpy.solvers.ader_stepper (solvers/steppers.cpp:10-22)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    set_grid(nXa)
    dXa, pd = _f64(dX)
    nd = nXa.size
    V = _nvar(u, int(np.prod(nXa)))
    pm, _ = _mask_ptr(mask, int(np.prod(nXa + 2)))
    c, pp = _par(MP)
    scr = _scratch(lib.gpr_ader_scratch_doubles(pn, nd, V), u)
    ps = _dev(status, "status", torch.int32) if status is not None else None
    _lib.check(lib.gpr_ader_stepper(_dev(u, "u"), _dev(ub, "ub"), pn, nd, float(dt), pd,
                                    int(bool(STIFF)), int(FLUX), pp, pm, _dev(scr, "s"), ps,
                                    V, _stream()), "ader_stepper")
    return u


ader_stepper_para = ader_stepper


def midstepper(wh, dt, dX, MP, mask, nX=None):
    """GPRpy.solvers.split.midstepper (split/homogeneous.h:7): half step of
    the homogeneous system at the WENO nodes, in place."""
    lib = _lib.load()
    dXa, pd = _f64(dX)
    nd = dXa.size
    nXa = np.asarray(_grid_from_mask(mask, nd) if nX is None else nX, dtype=np.int32)
    nXa, pn = _i32(nXa)
    V = _nvar(wh, int(np.prod(nXa + 2)) * 2 ** nd)
    pm, _ = _mask_ptr(mask, int(np.prod(nXa + 2)))
    c, pp = _par(MP)
    _lib.check(lib.gpr_midstepper(_dev(wh, "wh"), float(dt), pd, nd, pn, pp, pm, V, _stream()),
               "midstepper")
    return wh


def split_stepper(u, ub, nX, dt, dX, HALF_STEP, FLUX, MP, mask):
    """GPRpy.solvers.split_stepper (solvers/steppers.cpp:50-66); ub is
    modified (ODE half step)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    set_grid(nXa)
    dXa, pd = _f64(dX)
    nd = nXa.size
    V = _nvar(u, int(np.prod(nXa)))
    pm, _ = _mask_ptr(mask, int(np.prod(nXa + 2)))
    c, pp = _par(MP)
    scr = _scratch(lib.gpr_split_scratch_doubles(pn, nd, V), u)
    _lib.check(lib.gpr_split_stepper(_dev(u, "u"), _dev(ub, "ub"), pn, nd, float(dt), pd,
                                     int(bool(HALF_STEP)), int(FLUX), pp, pm, _dev(scr, "s"),
                                     V, _stream()), "split_stepper")
    return u


split_stepper_para = split_stepper


def timestep_device(u, dX, CFL, t, tf, count, MP, out=None):
    """Device form of solvers.timestep: returns a 1-element CUDA tensor."""
    lib = _lib.load()
    dXa, pd = _f64(dX)
    nd = dXa.size
    ncell = u.numel() // _guess_nvar(u)
    V = u.numel() // ncell
    c, pp = _par(MP)
    if out is None:
        out = torch.empty(1, dtype=torch.float64, device=u.device)
    scr = _scratch(lib.gpr_timestep_scratch_doubles(ncell), u)
    _lib.check(lib.gpr_timestep(_dev(u, "u"), ncell, pd, nd, float(CFL), float(t), float(tf),
                                int(count), pp, _dev(out, "dt"), _dev(scr, "s"), V, _stream()),
               "timestep")
    return out


_NVAR = {}


def set_nvar(V):
    _NVAR["V"] = int(V)


def _guess_nvar(u):
    if "V" in _NVAR:
        return _NVAR["V"]
    if u.dim() >= 2:
        return u.shape[-1]
    return 17


def timestep(grids, masks, dX, CFL, t, tf, count, MPs, nmat=1):
    """solvers.timestep (solvers/iterator.cpp:54-83) for the first
    material's grid; returns a host float."""
    u = grids[0] if isinstance(grids, (list, tuple)) else grids
    MP = MPs[0] if isinstance(MPs, (list, tuple)) else MPs
    return float(timestep_device(u, dX, CFL, t, tf, count, MP).item())


def renorm_distortion(u, MPs):
    """solvers.renorm_distortion (solvers/utils.cpp:6-23), one material."""
    lib = _lib.load()
    MP = MPs[0] if isinstance(MPs, (list, tuple)) else MPs
    V = _guess_nvar(u)
    c, pp = _par(MP)
    _lib.check(lib.gpr_renorm_distortion(_dev(u, "u"), u.numel() // V, pp, V, _stream()),
               "renorm_distortion")
    return u


def contorted(u, contorted_tol):
    """GPRpy.solvers.contorted (solvers/utils.cpp:65-85): True if any cell's
    normalised distortion m0 = |A|_F^2 / (3 |det A|^(2/3)) has m0 - 1 >
    contorted_tol.  Returns a Python bool (synchronises, as the reference's
    bool return does)."""
    lib = _lib.load()
    V = _guess_nvar(u) if u.dim() == 1 else u.shape[-1]
    flag = torch.zeros(1, dtype=torch.int32, device=u.device)
    _lib.check(lib.gpr_contorted(_dev(u, "u"), u.numel() // V, float(contorted_tol),
                                 _dev(flag, "flag", torch.int32), V, _stream()), "contorted")
    return bool(flag.item())


def reset_contorted(u, contorted_tol, MPs, flag=None):
    """solvers/utils.cpp:44-85: contorted(u, tol) and, if so,
    reset_distortion(u, MPs), in place (two materials: by level set).
    Returns the device flag (int32, 1 if it reset); no synchronisation."""
    lib = _lib.load()
    MPs = MPs if isinstance(MPs, (list, tuple)) else [MPs]
    V = _guess_nvar(u) if u.dim() == 1 else u.shape[-1]
    if flag is None:
        flag = torch.zeros(1, dtype=torch.int32, device=u.device)
    import ctypes
    from .params import GprParC
    arr = (GprParC * len(MPs))(*[MP.to_ctypes() for MP in MPs])
    _lib.check(lib.gpr_reset_contorted(_dev(u, "u"), u.numel() // V, float(contorted_tol),
                                       ctypes.cast(arr, ctypes.c_void_p), len(MPs),
                                       _dev(flag, "flag", torch.int32), V, _stream()),
               "reset_contorted")
    return flag


def ode_launcher(u, dt, MP):
    """solvers.split.ode_launcher (solvers/split/ode.cpp:5-11)."""
    lib = _lib.load()
    V = _guess_nvar(u)
    c, pp = _par(MP)
    _lib.check(lib.gpr_ode_launcher(_dev(u, "u"), u.numel() // V, float(dt), pp, V,
                                    _stream()), "ode_launcher")
    return u


# ---------------------------------------------------------------------------
# pointwise physics (GPRpy.system.*), batched over the leading dimension

def _pointwise(fn, Q, MP, *extra):
    lib = _lib.load()
    Q = Q.contiguous()
    V = Q.shape[-1]
    count = Q.numel() // V
    c, pp = _par(MP)
    return lib, Q, V, count, pp


def flux(Q, d, MP, out=None):
    lib, Q, V, count, pp = _pointwise(None, Q, MP)
    out = torch.zeros_like(Q) if out is None else out
    _lib.check(lib.gpr_flux(_dev(Q, "Q"), _dev(out, "out"), count, int(d), pp, V, _stream()),
               "flux")
    return out


def source(Q, MP):
    lib, Q, V, count, pp = _pointwise(None, Q, MP)
    out = torch.empty_like(Q)
    _lib.check(lib.gpr_source(_dev(Q, "Q"), _dev(out, "out"), count, pp, V, _stream()),
               "source")
    return out


def Bdot(Q, x, d, MP):
    lib, Q, V, count, pp = _pointwise(None, Q, MP)
    x = x.contiguous()
    out = torch.empty_like(Q)
    _lib.check(lib.gpr_Bdot(_dev(Q, "Q"), _dev(x, "x"), _dev(out, "out"), count, int(d), pp,
                            V, _stream()), "Bdot")
    return out


def max_abs_eigs(Q, d, MP):
    lib, Q, V, count, pp = _pointwise(None, Q, MP)
    out = torch.empty(Q.shape[:-1] if Q.dim() > 1 else (1,), dtype=torch.float64,
                      device=Q.device)
    _lib.check(lib.gpr_max_abs_eigs(_dev(Q, "Q"), _dev(out, "out"), count, int(d), pp, V,
                                    _stream()), "max_abs_eigs")
    return out


def _scheme_constants():
    lib = _lib.load()
    out = np.zeros(16, dtype=np.float64)
    _lib.check(lib.gpr_scheme_constants(out.ctypes.data_as(ctypes.c_void_p), out.size),
               "scheme_constants")
    return out


def scaled_nodes():
    """GPRpy.solvers.common.scaled_nodes (poly/basis.cpp): the N Gauss-Legendre
    nodes on [0, 1] the kernels use."""
    return _scheme_constants()[0:2].copy()


def scaled_weights():
    """GPRpy.solvers.common.scaled_weights: the Gauss-Legendre weights on [0, 1]."""
    return _scheme_constants()[2:4].copy()


def end_values(basis=None):
    """GPRpy.solvers.common.end_values: [psi_j(0); psi_j(1)] of the nodal
    Lagrange basis (2 x N).  The basis argument of the reference is accepted
    and ignored: the basis is the one on the Gauss nodes."""
    return _scheme_constants()[4:8].reshape(2, 2).copy()


def derivative_values(basis=None, nodes=None):
    """GPRpy.solvers.common.derivative_values: psi_j'(x_i) (N x N) at the Gauss
    nodes (arguments accepted and ignored, as in end_values)."""
    return _scheme_constants()[8:12].reshape(2, 2).copy()


def oscillation_indicator(basis=None):
    """GPRpy.solvers.weno.oscillation_indicator (weno_matrices.cpp:31-42): the
    WENO smoothness matrix sum_a int psi_i^(a) psi_j^(a) (N x N)."""
    return _scheme_constants()[12:16].reshape(2, 2).copy()


def system_matrix(Q, d, MP):
    """GPRpy.system.system_matrix (system/equations.cpp:169-176): dF_d/dQ +
    B_d, [..., V, V] with rows the equations."""
    lib, Q, V, count, pp = _pointwise(None, Q, MP)
    out = torch.empty(Q.shape[:-1] + (V, V), dtype=torch.float64, device=Q.device)
    _lib.check(lib.gpr_system_matrix(_dev(Q, "Q"), _dev(out, "out"), count, int(d), pp, V,
                                     _stream()), "system_matrix")
    return out


def thermo_acoustic_tensor(Q, d, MP):
    """GPRpy.system.thermo_acoustic_tensor (system/eig.cpp:55-64): Xi1 Xi2
    along d, [..., m, m] with m = 4 for V = 17 (heat conduction), else 3."""
    lib, Q, V, count, pp = _pointwise(None, Q, MP)
    m = 4 if V == 17 else 3
    out = torch.empty(Q.shape[:-1] + (m, m), dtype=torch.float64, device=Q.device)
    _lib.check(lib.gpr_thermo_acoustic_tensor(_dev(Q, "Q"), _dev(out, "out"), count, int(d),
                                              pp, V, _stream()), "thermo_acoustic_tensor")
    return out


def interface_terms(qL, qR, d, FLUX, MP):
    """(D_FLUX(qL, qR), Bint(qL, qR)) of solvers/fv/fluxes.cpp:9-75."""
    lib, qL, V, count, pp = _pointwise(None, qL, MP)
    qR = qR.contiguous()
    out = torch.empty_like(qL)
    bout = torch.empty_like(qL)
    _lib.check(lib.gpr_interface_terms(_dev(qL, "qL"), _dev(qR, "qR"), _dev(out, "o"),
                                       _dev(bout, "b"), count, int(d), int(FLUX), pp, V,
                                       _stream()), "interface_terms")
    return out, bout


def D_RUS(qL, qR, d, MP):
    return interface_terms(qL, qR, d, 0, MP)[0]


def D_ROE(qL, qR, d, MP):
    """Roe dissipation plus F(qL) + F(qR) (fluxes.cpp:46-64); d = 0."""
    return interface_terms(qL, qR, d, 1, MP)[0]


def D_OSH(qL, qR, d, MP):
    """Osher-Solomon dissipation plus F(qL) + F(qR) (fluxes.cpp:22-44); d = 0."""
    return interface_terms(qL, qR, d, 2, MP)[0]


def Bint(qL, qR, d, MP):
    return interface_terms(qL, qR, d, 0, MP)[1]
