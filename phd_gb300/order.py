"""The step at another number of Gauss nodes N (the reference's compile-time
N, code/cpp/src/options.h:15): N = 3 is its third-order scheme.

The reference builds one N per compiled module; here the N = 2 entry points
live in the package root (`phd_gb300.solvers` ...), and `for_order(N)`
returns the same GPRpy names for N (1D and 2D grids; Rusanov, Roe and Osher
fluxes; the stiff Newton pass):

    G3 = phd_gb300.order.for_order(3)
    G3.boundaries(u, ub, nX, bcs)
    G3.solvers.ader_stepper(u, ub, nX, dt, dX, False, 0, MP, mask)

Buffers are torch float64 CUDA tensors in the reference's layouts with N =
order and n_s = N^d space nodes per cell (x-major): ub [nx + 2N]([ny + 2N])
[V], wh [nx + 2]([ny + 2])[n_s][V], qh [nx + 2]([ny + 2])[N][n_s][V].  Calls
enqueue on the current stream through the C ABI (gpr_*_n in
include/gpr_gb300.h); a missing library raises.
"""
from types import SimpleNamespace

import numpy as np
import torch

from . import _lib
from .api import _dev, _f64, _i32, _mask_ptr, _par, _stream


def _nvar(t, ncell):
    V = t.numel() // ncell
    if V * ncell != t.numel():
        raise ValueError("tensor size is not a multiple of the cell count")
    return V


def _cells(nXa, pad=0):
    return int(np.prod(nXa.astype(np.int64) + pad))


def for_order(N):
    """The GPRpy-named entry points at N Gauss nodes."""
    lib = _lib.load()
    N = int(N)
    grid = {}

    def check_supported(nd, V):
        if not lib.gpr_order_supported(N, nd, V):
            raise RuntimeError("N = %d in %dD with %d variables is not compiled in" % (N, nd, V))

    def remember(nXa):
        grid["nX"] = tuple(int(x) for x in nXa)

    def boundaries(u, ub, nX, boundaryTypes):
        nXa, pn = _i32(nX)
        bca, pb = _i32(boundaryTypes)
        nd = nXa.size
        if bca.size < 2 * nd:
            raise ValueError("boundaryTypes needs %d entries" % (2 * nd))
        V = _nvar(u, _cells(nXa))
        check_supported(nd, V)
        remember(nXa)
        if ub.numel() != _cells(nXa, 2 * N) * V:
            raise ValueError("ub has the wrong size")
        _lib.check(lib.gpr_boundaries_n(_dev(u, "u"), _dev(ub, "ub"), pn, nd, pb, V, N,
                                        _stream()), "boundaries")
        return ub

    def weno_launcher(wh, ub, nX):
        nXa, pn = _i32(nX)
        nd = nXa.size
        V = _nvar(ub, _cells(nXa, 2 * N))
        check_supported(nd, V)
        remember(nXa)
        n = lib.gpr_weno_scratch_doubles_n(pn, nd, V, N)
        _lib.check(n, "weno_launcher")
        scr = torch.empty(max(n, 1), dtype=torch.float64, device=ub.device)
        _lib.check(lib.gpr_weno_launcher_n(_dev(wh, "wh"), _dev(ub, "ub"), pn, nd,
                                           _dev(scr, "s"), V, N, _stream()), "weno_launcher")
        return wh

    def predictor(qh, wh, dt, dX, STIFF, STIFF_IG, MP, mask, status=None, nX=None):
        """As the reference, the call takes no grid size: in 1D it comes
        from the mask (nx + 2 predictor cells); in 2D from nX, else from the
        last grid given to a call of this namespace that takes nX.  STIFF
        sends every cell to the stiff-source Newton pass (STIFF_IG, the
        reference's option of a stiff initial guess, is not used: the Newton
        pass starts from the standard initial guess)."""
        dXa, pd = _f64(dX)
        nd = dXa.size
        if nX is not None:
            nXa = np.asarray(nX, dtype=np.int32).ravel()
        elif nd == 1 and mask is not None:
            nXa = np.array([mask.numel() - 2], dtype=np.int32)
        elif grid.get("nX") is not None and len(grid["nX"]) == nd:
            nXa = np.array(grid["nX"], dtype=np.int32)
        else:
            raise ValueError("pass nX (or the mask, in 1D)")
        nXa, pn = _i32(nXa)
        ncb = _cells(nXa, 2)
        if mask is not None and mask.numel() != ncb:
            raise ValueError("mask has %d entries, expected %d" % (mask.numel(), ncb))
        V = _nvar(wh, ncb * N ** nd)
        check_supported(nd, V)
        pm, _ = _mask_ptr(mask, ncb)
        c, pp = _par(MP)
        ps = _dev(status, "status", torch.int32) if status is not None else None
        _lib.check(lib.gpr_predictor_n(_dev(qh, "qh"), _dev(wh, "wh"), float(dt), pd, nd, pn,
                                       int(bool(STIFF)), pp, pm, ps, V, N, _stream()),
                   "predictor")
        return qh

    def fv_launcher(u, qh, nX, dt, dX, SOURCES, TIME, FLUX, MP, mask):
        if not (SOURCES and TIME):
            raise RuntimeError("N = %d: the ADER update (sources and time integration) only" % N)
        nXa, pn = _i32(nX)
        dXa, pd = _f64(dX)
        nd = nXa.size
        V = _nvar(u, _cells(nXa))
        check_supported(nd, V)
        remember(nXa)
        pm, _ = _mask_ptr(mask, _cells(nXa, 2))
        c, pp = _par(MP)
        scr = torch.empty(lib.gpr_fv_scratch_doubles_n(pn, nd, V, N), dtype=torch.float64,
                          device=u.device)
        _lib.check(lib.gpr_fv_launcher_n(_dev(u, "u"), _dev(qh, "qh"), pn, float(dt), pd, nd,
                                         int(FLUX), pp, pm, _dev(scr, "s"), V, N, _stream()),
                   "fv_launcher")
        return u

    def ader_stepper(u, ub, nX, dt, dX, STIFF, FLUX, MP, mask, status=None):
        nXa, pn = _i32(nX)
        dXa, pd = _f64(dX)
        nd = nXa.size
        V = _nvar(u, _cells(nXa))
        check_supported(nd, V)
        remember(nXa)
        pm, _ = _mask_ptr(mask, _cells(nXa, 2))
        c, pp = _par(MP)
        scr = torch.empty(lib.gpr_ader_scratch_doubles_n(pn, nd, V, N), dtype=torch.float64,
                          device=u.device)
        ps = _dev(status, "status", torch.int32) if status is not None else None
        _lib.check(lib.gpr_ader_stepper_n(_dev(u, "u"), _dev(ub, "ub"), pn, nd, float(dt), pd,
                                          int(bool(STIFF)), int(FLUX), pp, pm, _dev(scr, "s"),
                                          ps, V, N, _stream()), "ader_stepper")
        return u

    def iterate(u, nX, dX, bcs, MP, clock, nsteps, FLUX=0, mask=None, status=None,
                contorted_tol=1.0):
        """nsteps steps of the reference iterator's loop body (CFL time step,
        boundaries, ADER step, renormalisation, contortion reset) with the
        device clock {t, dt, tf, cfl, count} in `clock`."""
        nXa, pn = _i32(nX)
        dXa, pd = _f64(dX)
        bca, pb = _i32(bcs)
        nd = nXa.size
        if bca.size < 2 * nd:
            raise ValueError("bcs needs %d entries" % (2 * nd))
        V = _nvar(u, _cells(nXa))
        check_supported(nd, V)
        pm, _ = _mask_ptr(mask, _cells(nXa, 2))
        c, pp = _par(MP)
        scr = torch.empty(lib.gpr_iterate_scratch_doubles_n(pn, nd, V, N), dtype=torch.float64,
                          device=u.device)
        ps = _dev(status, "status", torch.int32) if status is not None else None
        _lib.check(lib.gpr_iterate_n(_dev(u, "u"), pn, nd, pd, pb, int(FLUX), pp, pm,
                                     _dev(clock, "clock"), int(nsteps), _dev(scr, "s"), ps,
                                     float(contorted_tol), V, N, _stream()), "iterate")
        return u

    def scheme_constants():
        out = np.zeros(4 * N + 2 * N * N)
        n = lib.gpr_scheme_constants_n(out.ctypes.data_as(_lib.ctypes.c_void_p), out.size, N)
        _lib.check(n, "scheme_constants")
        return dict(nodes=out[:N], weights=out[N:2 * N],
                    endvals=out[2 * N:4 * N].reshape(2, N),
                    dervals=out[4 * N:4 * N + N * N].reshape(N, N),
                    sig=out[4 * N + N * N:].reshape(N, N))

    return SimpleNamespace(
        N=N, boundaries=boundaries, iterate=iterate, scheme_constants=scheme_constants,
        solvers=SimpleNamespace(
            weno=SimpleNamespace(weno_launcher=weno_launcher),
            dg=SimpleNamespace(predictor=predictor),
            fv=SimpleNamespace(fv_launcher=fv_launcher),
            ader_stepper=ader_stepper))
