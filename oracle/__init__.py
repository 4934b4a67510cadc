"""CPU oracle for the GPR ADER-WENO step (test infrastructure).

`liboracle_gpr.so` is built from oracle/gpr_oracle.c (a plain-C restatement
of the reference's hot path) by `build()`.  Only the tests, the smoke check
and bench.py's CPU-baseline leg use this module, as the checker; the CUDA
library never calls it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle_gpr.so")
SRC = os.path.join(HERE, "gpr_oracle.c")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def build(force=False):
    """Compile the oracle with gcc (portable flags: x86 and aarch64)."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None
_cfg = None


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        from phd_gb300.params import GprParC  # noqa: F401 (struct layout)
        P = ctypes.c_void_p
        sig = {
            "or_configure": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_int]),
            "or_nvar": (ctypes.c_int, []),
            "or_set_stiff": (None, [ctypes.c_double, ctypes.c_int]),
            "or_constants": (None, [_dp]),
            "or_pressure": (ctypes.c_double, [_dp, P]),
            "or_temperature": (ctypes.c_double, [_dp, P]),
            "or_flux": (None, [_dp, ctypes.c_int, P, _dp]),
            "or_source": (None, [_dp, P, _dp]),
            "or_Bdot": (None, [_dp, _dp, ctypes.c_int, _dp]),
            "or_eigenvalues": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp]),
            "or_thermo_acoustic_tensor": (None, [_dp, ctypes.c_int, P, _dp]),
            "or_max_abs_eigs": (ctypes.c_double, [_dp, ctypes.c_int, P]),
            "or_system_matrix": (None, [_dp, ctypes.c_int, P, _dp]),
            "or_Bint": (None, [_dp, _dp, ctypes.c_int, _dp]),
            "or_D_RUS": (None, [_dp, _dp, ctypes.c_int, P, _dp]),
            "or_D_OSH": (None, [_dp, _dp, ctypes.c_int, P, _dp]),
            "or_D_ROE": (None, [_dp, _dp, ctypes.c_int, P, _dp]),
            "or_boundaries": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_int, _ip]),
            "or_extend_mask": (ctypes.c_int, [_u8p, _u8p, _ip, ctypes.c_int]),
            "or_weno_launcher": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_int]),
            "or_predictor": (ctypes.c_int, [_dp, _dp, ctypes.c_double, _dp,
                                            ctypes.c_int, _ip, ctypes.c_int, P,
                                            _u8p, _ip, ctypes.c_int]),
            "or_fv_launcher": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_double, _dp,
                                              ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, P, _u8p]),
            "or_fv_parts": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_double, _dp, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, P, _u8p,
                                           ctypes.c_int]),
            "or_timestep": (ctypes.c_double, [_dp, ctypes.c_long, _dp, ctypes.c_int,
                                              ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int, P]),
            "or_renorm_distortion": (None, [_dp, ctypes.c_long, P]),
            "or_ode_cell": (None, [_dp, ctypes.c_double, P]),
            "or_ode_launcher": (None, [_dp, ctypes.c_long, ctypes.c_double, P]),
            "or_ader_stepper": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_int,
                                               ctypes.c_double, _dp, ctypes.c_int,
                                               ctypes.c_int, P, _u8p, _ip,
                                               ctypes.c_int]),
            "or_midstepper": (ctypes.c_int, [_dp, ctypes.c_double, _dp, ctypes.c_int,
                                             P, _u8p, ctypes.c_long]),
            "or_split_stepper": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_int,
                                                ctypes.c_double, _dp, ctypes.c_int,
                                                ctypes.c_int, P, _u8p]),
            "or_distance": (ctypes.c_int, [_dp, _dp, _ip, ctypes.c_int, _dp]),
            "or_finite_difference": (None, [_dp, _dp, _ip, ctypes.c_int, _dp]),
            "or_find_interface_cells": (None, [_dp, _ip, ctypes.c_int, _ip]),
            "or_left_star_state": (ctypes.c_int, [_dp, _dp, P, P, ctypes.c_double, _dp,
                                                  ctypes.c_int, _dp]),
            "or_fill_ghost_cells": (ctypes.c_int, [_dp, _u8p, _dp, _ip, ctypes.c_int, _dp,
                                                   ctypes.c_double, P, ctypes.c_int, _ip]),
            "or_make_u": (None, [_dp, _dp, _u8p, ctypes.c_long, P, ctypes.c_int]),
            "or_fill_boundary_cells": (ctypes.c_int, [_dp, _ip, ctypes.c_int, _dp, _dp, _dp,
                                                      P, ctypes.c_double, _ip, ctypes.c_int]),
            "or_fill_neighbor_cells": (ctypes.c_int, [_dp, _ip, _dp, _dp, _ip, ctypes.c_int]),
            "or_timestep_multi": (ctypes.c_double, [_dp, _u8p, ctypes.c_long, _dp,
                                                    ctypes.c_int, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_int, P, ctypes.c_int]),
            "or_renorm_multi": (None, [_dp, ctypes.c_long, P]),
            "or_reset_contorted": (ctypes.c_int, [_dp, ctypes.c_long, ctypes.c_double, P,
                                                  ctypes.c_int]),
            "or_num_threads": (ctypes.c_int, []),
            "or_set_num_threads": (None, [ctypes.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def _u8(a):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(_u8p)


class Oracle:
    """CPU restatement of the reference solver for one variant
    (N Gauss nodes, THERMAL on/off, LSET 0/1)."""

    def __init__(self, N=2, thermal=True, lset=0, dg_tol=6e-6, dg_it=50):
        self.N = N
        self.thermal = bool(thermal)
        self.lset = lset
        self.dg_tol = dg_tol
        self.dg_it = dg_it
        self.V = 14 + 3 * self.thermal + lset
        self.lib = _load()

    def _cfg(self):
        global _cfg
        key = (self.N, self.thermal, self.lset, self.dg_tol, self.dg_it)
        if _cfg != key:
            self.lib.or_configure(self.N, int(self.thermal), self.lset,
                                  self.dg_tol, self.dg_it)
            _cfg = key
        return self.lib

    @staticmethod
    def _par(MP):
        c = MP.to_ctypes()
        return c, ctypes.cast(ctypes.pointer(c), ctypes.c_void_p)

    # -- constants ---------------------------------------------------------
    def constants(self):
        lib = self._cfg()
        out = np.zeros(4 + 4 + 8 + 16 * 4)
        lib.or_constants(_d(out))
        N = self.N
        return dict(nodes=out[:N], weights=out[4:4 + N],
                    endvals=out[8:16].reshape(2, 4)[:, :N],
                    dervals=out[16:32].reshape(4, 4)[:N, :N],
                    dg_der=out[32:48].reshape(4, 4)[:N, :N],
                    dg_mat=out[48:64].reshape(4, 4)[:N, :N],
                    sig=out[64:80].reshape(4, 4)[:N, :N])

    # -- pointwise physics -------------------------------------------------
    def pressure(self, Q, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        c, p = self._par(MP)
        return lib.or_pressure(_d(Q), p)

    def temperature(self, Q, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        c, p = self._par(MP)
        return lib.or_temperature(_d(Q), p)

    def flux(self, Q, d, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = np.zeros(self.V)
        c, p = self._par(MP)
        lib.or_flux(_d(Q), d, p, _d(out))
        return out

    def source(self, Q, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = np.zeros(self.V)
        c, p = self._par(MP)
        lib.or_source(_d(Q), p, _d(out))
        return out

    def Bdot(self, Q, x, d, MP=None):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(self.V)
        lib.or_Bdot(_d(Q), _d(x), d, _d(out))
        return out

    def eigenvalues(self, M):
        lib = self._cfg()
        M = np.ascontiguousarray(M, dtype=np.float64)
        n = M.shape[0]
        wr = np.zeros(n)
        wi = np.zeros(n)
        rc = lib.or_eigenvalues(n, _d(M), _d(wr), _d(wi))
        return wr + 1j * wi, rc

    def thermo_acoustic_tensor(self, Q, d, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        m = 4 if self.thermal else 3
        out = np.zeros(m * m)
        c, p = self._par(MP)
        lib.or_thermo_acoustic_tensor(_d(Q), d, p, _d(out))
        return out.reshape(m, m)

    def max_abs_eigs(self, Q, d, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        c, p = self._par(MP)
        return lib.or_max_abs_eigs(_d(Q), d, p)

    def system_matrix(self, Q, d, MP):
        lib = self._cfg()
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = np.zeros(self.V * self.V)
        c, p = self._par(MP)
        lib.or_system_matrix(_d(Q), d, p, _d(out))
        return out.reshape(self.V, self.V)

    def Bint(self, qL, qR, d, MP=None):
        lib = self._cfg()
        qL = np.ascontiguousarray(qL, dtype=np.float64)
        qR = np.ascontiguousarray(qR, dtype=np.float64)
        out = np.zeros(self.V)
        lib.or_Bint(_d(qL), _d(qR), d, _d(out))
        return out

    def D(self, which, qL, qR, d, MP):
        lib = self._cfg()
        qL = np.ascontiguousarray(qL, dtype=np.float64)
        qR = np.ascontiguousarray(qR, dtype=np.float64)
        out = np.zeros(self.V)
        c, p = self._par(MP)
        fn = {0: lib.or_D_RUS, 1: lib.or_D_ROE, 2: lib.or_D_OSH}[which]
        fn(_d(qL), _d(qR), d, p, _d(out))
        return out

    # -- grid stages ---------------------------------------------------------
    def boundaries(self, u, nX, bcs):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        ub = np.zeros(int(np.prod(nX + 2 * self.N)) * self.V)
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        lib.or_boundaries(_d(u), _d(ub), _i(nX), nd,
                          _i(np.asarray(bcs, dtype=np.int32)))
        return ub

    def extend_mask(self, mask, nX):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        maskb = np.zeros(int(np.prod(nX + 2)), dtype=np.uint8)
        mask = np.ascontiguousarray(mask, dtype=np.uint8).ravel()
        lib.or_extend_mask(_u8(mask), _u8(maskb), _i(nX), len(nX))
        return maskb

    def weno_launcher(self, ub, nX):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        wh = np.zeros(int(np.prod(nX + 2)) * self.N ** nd * self.V)
        lib.or_weno_launcher(_d(wh), _d(np.ascontiguousarray(ub)), _i(nX), nd)
        return wh

    def predictor(self, wh, dt, dX, nX, MP, mask=None, stiff=False,
                  newton_fallback=True, qh=None):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        ncb = int(np.prod(nX + 2))
        if mask is None:
            mask = np.ones(ncb, dtype=np.uint8)
        if qh is None:
            qh = np.full(ncb * self.N ** (nd + 1) * self.V, np.nan)
        status = np.zeros(ncb, dtype=np.int32)
        c, p = self._par(MP)
        lib.or_predictor(_d(qh), _d(np.ascontiguousarray(wh)), dt,
                         _d(np.asarray(dX, dtype=np.float64)), nd, _i(nX),
                         int(stiff), p, _u8(np.ascontiguousarray(mask, dtype=np.uint8)),
                         _i(status), int(newton_fallback))
        return qh, status

    def fv_launcher(self, u, qh, nX, dt, dX, MP, mask=None, sources=True,
                    time=True, flux=0):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        if mask is None:
            mask = np.ones(int(np.prod(nX + 2)), dtype=np.uint8)
        c, p = self._par(MP)
        lib.or_fv_launcher(_d(u), _d(np.ascontiguousarray(qh)), _i(nX), dt,
                           _d(np.asarray(dX, dtype=np.float64)), nd, int(sources),
                           int(time), int(flux), p,
                           _u8(np.ascontiguousarray(mask, dtype=np.uint8)))
        return u

    def fv_parts(self, u, qh, nX, dt, dX, MP, parts, mask=None, sources=True, time=True,
                 flux=0):
        """One or both passes of fv_launcher: parts 1 = centers1/2 (volume
        term), 2 = interfs1/2 (interface terms), 3 = both."""
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        if mask is None:
            mask = np.ones(int(np.prod(nX + 2)), dtype=np.uint8)
        c, p = self._par(MP)
        lib.or_fv_parts(_d(u), _d(np.ascontiguousarray(qh)), _i(nX), dt,
                        _d(np.asarray(dX, dtype=np.float64)), nd, int(sources), int(time),
                        int(flux), p, _u8(np.ascontiguousarray(mask, dtype=np.uint8)),
                        int(parts))
        return u

    def timestep(self, u, dX, cfl, t, tf, count, MP):
        lib = self._cfg()
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        c, p = self._par(MP)
        return lib.or_timestep(_d(u), u.size // self.V,
                               _d(np.asarray(dX, dtype=np.float64)), len(dX),
                               cfl, t, tf, count, p)

    def renorm_distortion(self, u, MP):
        lib = self._cfg()
        c, p = self._par(MP)
        lib.or_renorm_distortion(_d(u), u.size // self.V, p)
        return u

    def ode_launcher(self, u, dt, MP):
        lib = self._cfg()
        c, p = self._par(MP)
        lib.or_ode_launcher(_d(u), u.size // self.V, dt, p)
        return u

    def ader_stepper(self, u, ub, nX, dt, dX, MP, mask=None, flux=0,
                     stiff=False, newton_fallback=True):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        ncb = int(np.prod(nX + 2))
        if mask is None:
            mask = np.ones(ncb, dtype=np.uint8)
        status = np.zeros(ncb, dtype=np.int32)
        c, p = self._par(MP)
        lib.or_ader_stepper(_d(u), _d(np.ascontiguousarray(ub)), _i(nX), nd, dt,
                            _d(np.asarray(dX, dtype=np.float64)), int(stiff),
                            int(flux), p,
                            _u8(np.ascontiguousarray(mask, dtype=np.uint8)),
                            _i(status), int(newton_fallback))
        return u, status

    def midstepper(self, wh, dt, dX, nX, MP, mask=None):
        """split/homogeneous.cpp:5-67 on a copy of wh (returned)."""
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        ncb = int(np.prod(nX + 2))
        if mask is None:
            mask = np.ones(ncb, dtype=np.uint8)
        w = np.ascontiguousarray(wh, dtype=np.float64).ravel().copy()
        c, p = self._par(MP)
        lib.or_midstepper(_d(w), dt, _d(np.asarray(dX, dtype=np.float64)), len(nX), p,
                          _u8(np.ascontiguousarray(mask, dtype=np.uint8)), ncb)
        return w

    def split_stepper(self, u, ub, nX, dt, dX, MP, mask=None, flux=0,
                      half_step=True):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        nd = len(nX)
        if mask is None:
            mask = np.ones(int(np.prod(nX + 2)), dtype=np.uint8)
        c, p = self._par(MP)
        lib.or_split_stepper(_d(u), _d(ub), _i(nX), nd, dt,
                             _d(np.asarray(dX, dtype=np.float64)), int(half_step),
                             int(flux), p,
                             _u8(np.ascontiguousarray(mask, dtype=np.uint8)))
        return u

    # -- level-set ghost fluid (LSET = 1, non-thermal) ----------------------
    @staticmethod
    def _pars(MPs):
        from phd_gb300.params import GprParC
        arr = (GprParC * len(MPs))(*[MP.to_ctypes() for MP in MPs])
        return arr, ctypes.cast(arr, ctypes.c_void_p)

    def distance(self, phi, dX, nX):
        """multi/pfmm.cpp:4-26 (first-order fast marching)."""
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        phi = np.ascontiguousarray(phi, dtype=np.float64).ravel()
        out = np.zeros_like(phi)
        lib.or_distance(_d(phi), _d(np.asarray(dX, dtype=np.float64)), _i(nX), len(nX),
                        _d(out))
        return out

    def finite_difference(self, phi, dX, nX):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        phi = np.ascontiguousarray(phi, dtype=np.float64).ravel()
        out = np.zeros((phi.size, len(nX)))
        lib.or_finite_difference(_d(phi), _d(np.asarray(dX, dtype=np.float64)), _i(nX),
                                 len(nX), _d(out))
        return out

    def find_interface_cells(self, phi, nX):
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        phi = np.ascontiguousarray(phi, dtype=np.float64).ravel()
        out = np.zeros(phi.size, dtype=np.int32)
        lib.or_find_interface_cells(_d(phi), _i(nX), len(nX), _i(out))
        return out

    def left_star_state(self, QL, QR, MPL, MPR, dt, n):
        lib = self._cfg()
        out = np.zeros(self.V)
        n = np.ascontiguousarray(n, dtype=np.float64)
        cl, pl = self._par(MPL)
        cr, pr = self._par(MPR)
        lib.or_left_star_state(_d(np.ascontiguousarray(QL, dtype=np.float64)),
                               _d(np.ascontiguousarray(QR, dtype=np.float64)), pl, pr, dt,
                               _d(n), n.size, _d(out))
        return out

    def fill_ghost_cells(self, u, nX, dX, dt, MPs):
        """multi/fill.cpp:330-370 on a copy of u.  Returns (u with its level
        set re-distanced, grids [nmat, ncell, V], masks [nmat, ncell] bool,
        intMask [nmat, ncell], cells whose fill would read off the grid)."""
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        u = np.ascontiguousarray(u, dtype=np.float64).ravel().copy()
        ncell = u.size // self.V
        nmat = len(MPs)
        grids = np.zeros((nmat, ncell, self.V))
        masks = np.zeros((nmat, ncell), dtype=np.uint8)
        im = np.zeros((nmat, ncell), dtype=np.int32)
        arr, p = self._pars(MPs)
        bad = lib.or_fill_ghost_cells(_d(grids), _u8(masks), _d(u), _i(nX), len(nX),
                                      _d(np.asarray(dX, dtype=np.float64)), dt, p, nmat,
                                      _i(im))
        if bad < 0:
            raise RuntimeError("oracle fill_ghost_cells: unsupported variant")
        return u, grids, masks.astype(bool), im, bad

    def fill_boundary_cells(self, grid, mask, mat, phi, dphi, dX, MPs, dt, nX):
        """multi/fill.cpp:200-235 in the reference's (i, j) order, in place on
        grid; returns the number of cells whose fill would read off the grid."""
        lib = self._cfg()
        arr, p = self._pars(MPs)
        nX = np.asarray(nX, dtype=np.int32)
        return lib.or_fill_boundary_cells(
            _d(grid), _i(np.ascontiguousarray(mask, dtype=np.int32)), int(mat),
            _d(np.ascontiguousarray(phi, dtype=np.float64)),
            _d(np.ascontiguousarray(dphi, dtype=np.float64)),
            _d(np.asarray(dX, dtype=np.float64)), p, float(dt), _i(nX), len(nX))

    def fill_neighbor_cells(self, grid, mask, dphi, dX, nX):
        """multi/fill.cpp:255-328, in place on grid and mask (int32)."""
        lib = self._cfg()
        nX = np.asarray(nX, dtype=np.int32)
        return lib.or_fill_neighbor_cells(_d(grid), _i(mask),
                                          _d(np.ascontiguousarray(dphi, dtype=np.float64)),
                                          _d(np.asarray(dX, dtype=np.float64)), _i(nX),
                                          len(nX))

    def make_u(self, u, grids, masks, MPs):
        lib = self._cfg()
        arr, p = self._pars(MPs)
        g = np.ascontiguousarray(grids, dtype=np.float64)
        m = np.ascontiguousarray(masks, dtype=np.uint8)
        lib.or_make_u(_d(u), _d(g), _u8(m), u.size // self.V, p, len(MPs))
        return u

    def timestep_multi(self, grids, masks, dX, cfl, t, tf, count, MPs):
        lib = self._cfg()
        arr, p = self._pars(MPs)
        g = np.ascontiguousarray(grids, dtype=np.float64)
        m = np.ascontiguousarray(masks, dtype=np.uint8)
        return lib.or_timestep_multi(_d(g), _u8(m), m.shape[1],
                                     _d(np.asarray(dX, dtype=np.float64)), len(dX), cfl, t,
                                     tf, count, p, len(MPs))

    def renorm_multi(self, u, MPs):
        lib = self._cfg()
        arr, p = self._pars(MPs)
        lib.or_renorm_multi(_d(u), u.size // self.V, p)
        return u

    def step_multi(self, u, dt_prev, t, tf, count, MPs, dX, bcs, cfl=0.8, dt=None,
                   contorted_tol=None, split=False, half_step=True, stiff=False, flux=0):
        """One step of the time loop of solvers/iterator.cpp:85-151 with the
        ghost-fluid fill (LSET = 1): fill (with the previous step's dt) ->
        timestep -> per material boundaries + the ADER step (or the split
        step, iterator.cpp:123-129) on its masked cells -> make_u -> renorm.
        u (flat or shaped, cell-major) is updated in place; `dt` overrides
        the CFL step.  Returns dt."""
        nd = len(dX)
        ncell = u.size // self.V
        nX = np.asarray(u.shape[:-1] if u.ndim > 1 else [ncell], dtype=np.int32)
        if nX.size != nd:
            raise ValueError("pass u shaped (nx[, ny], V)")
        uf = u.reshape(-1)
        nmat = len(MPs)
        bc = (np.array([bcs] * 2 * nd, dtype=np.int32) if np.isscalar(bcs)
              else np.asarray(bcs, np.int32))
        uf[:], grids, masks, _, _ = self.fill_ghost_cells(uf, nX, dX, dt_prev, MPs)
        if dt is None:
            dt = self.timestep_multi(grids, masks, dX, cfl, t, tf, count, MPs)
        for mat in range(nmat):
            if MPs[mat].EOS <= -1:
                continue
            g = np.ascontiguousarray(grids[mat]).ravel()
            ub = self.boundaries(g, nX, bc)
            maskb = self.extend_mask(masks[mat].astype(np.uint8), nX)
            if split:
                self.split_stepper(g, ub, nX, dt, dX, MPs[mat], mask=maskb, flux=flux,
                                   half_step=half_step)
            else:
                self.ader_stepper(g, ub, nX, dt, dX, MPs[mat], mask=maskb, flux=flux,
                                  stiff=stiff)
            grids[mat] = g.reshape(ncell, self.V)
        self.make_u(uf, grids, masks, MPs)
        self.renorm_multi(uf, MPs)
        if contorted_tol is not None:
            self.reset_contorted(uf, contorted_tol, MPs)
        return dt

    def run_multi(self, u0, MPs, tf, dX, bcs, cfl=0.8, max_steps=None, contorted_tol=None,
                  split=False, half_step=True, stiff=False, flux=0):
        """The two-material time loop (step_multi until tf).  Returns
        (u, steps, t)."""
        u = np.ascontiguousarray(u0, dtype=np.float64).copy()
        t, count, dt = 0.0, 0, 0.0
        while t < tf:
            dt = self.step_multi(u, dt, t, tf, count, MPs, dX, bcs, cfl,
                                 contorted_tol=contorted_tol, split=split,
                                 half_step=half_step, stiff=stiff, flux=flux)
            t += dt
            count += 1
            if max_steps is not None and count >= max_steps:
                break
        return u, count, t

    def reset_contorted(self, u, tol, MPs):
        """contorted + reset_distortion (solvers/utils.cpp:44-85) in place;
        returns True if the distortion was reset."""
        lib = self._cfg()
        MPs = MPs if isinstance(MPs, (list, tuple)) else [MPs]
        arr, p = self._pars(MPs)
        return bool(lib.or_reset_contorted(_d(u), u.size // self.V, float(tol), p, len(MPs)))

    def num_threads(self):
        return self.lib.or_num_threads()

    def set_num_threads(self, n):
        self.lib.or_set_num_threads(int(n))

    # -- a full run ------------------------------------------------------------
    def run(self, u0, MP, tf, dX, bcs, cfl=0.8, flux=0, max_steps=None,
            split=False, half_step=True, contorted_tol=None):
        """Time loop of solvers/iterator.cpp:85-170 for one material
        (boundaries -> timestep -> stepper -> renorm [-> contortion reset if
        contorted_tol is given]), returning the final state and the number
        of steps."""
        shape = u0.shape
        nX = np.array(shape[:-1], dtype=np.int32)
        u = np.ascontiguousarray(u0, dtype=np.float64).ravel().copy()
        t, count = 0.0, 0
        bc = np.array([bcs] * 2 * len(nX), dtype=np.int32) if np.isscalar(bcs) else np.asarray(bcs, np.int32)
        while t < tf:
            dt = self.timestep(u, dX, cfl, t, tf, count, MP)
            ub = self.boundaries(u, nX, bc)
            if split:
                self.split_stepper(u, ub, nX, dt, dX, MP, flux=flux,
                                   half_step=half_step)
            else:
                self.ader_stepper(u, ub, nX, dt, dX, MP, flux=flux)
            self.renorm_distortion(u, MP)
            if contorted_tol is not None:
                self.reset_contorted(u, contorted_tol, [MP])
            t += dt
            count += 1
            if max_steps is not None and count >= max_steps:
                break
        return u.reshape(shape), count, t
