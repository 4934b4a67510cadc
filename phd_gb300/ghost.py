"""GPRpy-compatible level-set ghost fluid over the CUDA library.

Mirrors the reference's `GPRpy.multi` module, `GPRpy.system.multi` and the
two-material forms of `GPRpy.solvers.{make_u, renorm_distortion, timestep,
iterator}` (code/cpp/bindings/bindings.cpp:180-232) for the V = 15 layout
(viscous, one level set, no heat conduction) and two materials: material 0
occupies phi < 0, material 1 phi >= 0.  Arrays are CUDA tensors
(float64 grid data, int32 interface masks, bool/uint8 update masks) and are
updated in place like the reference's Eigen::Ref arguments.

Every fill call accumulates its error counts in a status tensor (int32[4],
device): [0] the re-distancing did not converge within its round budget,
[1] boundary cells whose fill would read outside the grid in the reference,
[2] extrapolation cells whose copy source would lie outside the grid.
Pass `status=` to collect them; `check_status(status)` raises on any.
"""
import numpy as np
import torch

from . import _lib
from .api import _dev, _f64, _i32, _par, _scratch, _stream
from .params import GprParC

V = 15


def _pars(MPs):
    if len(MPs) != 2:
        raise ValueError("the ghost fill takes exactly two materials")
    arr = (GprParC * 2)(*[MP.to_ctypes() for MP in MPs])
    import ctypes
    return arr, ctypes.cast(arr, ctypes.c_void_p)


def _status(status, like):
    if status is None:
        status = torch.zeros(4, dtype=torch.int32, device=like.device)
    return status


def check_status(status):
    """Raise if a fill recorded an error (synchronises)."""
    s = status.cpu().numpy()
    if s[0]:
        raise RuntimeError("re-distancing did not converge")
    if s[1] or s[2]:
        raise RuntimeError("ghost fill read outside the grid (%d boundary, %d layer cells)"
                           % (s[1], s[2]))


def _u8(mask):
    return mask.view(torch.uint8) if mask.dtype == torch.bool else mask


# ---------------------------------------------------------------------------
# multi/pfmm.cpp, multi/functions.cpp

def distance(phi, dX, nX, status=None):
    """GPRpy.system.multi.distance (multi/pfmm.cpp:4-26): first-order signed
    distance to the zero level of phi (a new tensor); zeros when phi has no
    zero crossing."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    dXa, pd = _f64(dX)
    phi = phi.contiguous()
    out = torch.empty_like(phi)
    status = _status(status, phi)
    scr = _scratch(lib.gpr_distance_scratch_doubles(pn, nXa.size), phi)
    _lib.check(lib.gpr_distance(_dev(phi, "phi"), _dev(out, "out"), pn, nXa.size, pd,
                                _dev(scr, "s"), _dev(status, "status", torch.int32),
                                _stream()), "distance")
    return out


def renormalize_levelsets(u, dX, nX, status=None):
    """GPRpy.multi.renormalize_levelsets (multi/functions.cpp:56-64): the
    level set column of u (ncell x V) replaced by its signed distance."""
    col = u.view(-1, V)[:, V - 1].contiguous()
    u.view(-1, V)[:, V - 1] = distance(col, dX, nX, status=status)
    return u


def finite_difference(dphi, phi, dX, nX):
    """GPRpy.multi.finite_difference (multi/functions.cpp:16-54):
    dphi[ncell][ndim]."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    dXa, pd = _f64(dX)
    _lib.check(lib.gpr_finite_difference(_dev(phi, "phi"), _dev(dphi, "dphi"), pn, nXa.size,
                                         pd, _stream()), "finite_difference")
    return dphi


def find_interface_cells(intMask, phi, nX):
    """GPRpy.multi.find_interface_cells (multi/fill.cpp:20-74)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    _lib.check(lib.gpr_find_interface_cells(_dev(phi, "phi"),
                                            _dev(intMask, "intMask", torch.int32), pn,
                                            nXa.size, _stream()), "find_interface_cells")
    return intMask


def material_indicator(phi, u, mat, nmat, dX, nX):
    """GPRpy.multi.material_indicator (multi/functions.cpp:66-81) for two
    materials: phi = u's level set for material 0, its negation for 1."""
    if nmat != 2:
        raise ValueError("two materials only")
    col = u.view(-1, V)[:, V - 1]
    phi.copy_(col if mat == 0 else -col)
    return phi


# ---------------------------------------------------------------------------
# multi/fill.cpp

def fill_boundary_cells(grid, intMask, mat, phi, dphi, dX, MPs, dt, nX, status=None):
    """GPRpy.multi.fill_boundary_cells (multi/fill.cpp:200-235)."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    dXa, pd = _f64(dX)
    arr, pp = _pars(MPs)
    status = _status(status, grid)
    scr = _scratch(lib.gpr_fill_scratch_doubles(pn, nXa.size, V), grid)
    _lib.check(lib.gpr_fill_boundary_cells(
        _dev(grid, "grid"), _dev(intMask, "intMask", torch.int32), int(mat), _dev(phi, "phi"),
        _dev(dphi, "dphi"), pd, pp, 2, float(dt), pn, nXa.size, _dev(scr, "s"),
        _dev(status, "status", torch.int32), V, _stream()), "fill_boundary_cells")
    return grid


def fill_neighbor_cells(grid, intMask, dphi, dX, nX, status=None):
    """GPRpy.multi.fill_neighbor_cells (multi/fill.cpp:255-328); intMask is
    updated in place."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    dXa, pd = _f64(dX)
    status = _status(status, grid)
    scr = _scratch(lib.gpr_fill_scratch_doubles(pn, nXa.size, V), grid)
    _lib.check(lib.gpr_fill_neighbor_cells(
        _dev(grid, "grid"), _dev(intMask, "intMask", torch.int32), _dev(dphi, "dphi"), pd, pn,
        nXa.size, _dev(scr, "s"), _dev(status, "status", torch.int32), V, _stream()),
        "fill_neighbor_cells")
    return grid


def _stack(x, shape, dtype):
    if isinstance(x, (list, tuple)):
        return torch.stack([t.reshape(shape) for t in x]).to(dtype), True
    return x, False


def fill_ghost_cells(grids, masks, u, nX, dX, dt, MPs, status=None):
    """GPRpy.multi.fill_ghost_cells (multi/fill.cpp:330-370): re-distances
    u's level set in place and fills both material grids and their update
    masks.  grids: [2][ncell*V] tensor (or a list of two), masks: [2][ncell]
    bool/uint8 (or a list of two).  Returns the status tensor."""
    lib = _lib.load()
    nXa, pn = _i32(nX)
    dXa, pd = _f64(dX)
    ncell = int(np.prod(nXa))
    arr, pp = _pars(MPs)
    g, gl = _stack(grids, (-1,), torch.float64)
    m, ml = _stack(masks, (-1,), torch.uint8)
    if g.numel() != 2 * ncell * V or m.numel() != 2 * ncell:
        raise ValueError("grids / masks have the wrong size")
    status = _status(status, u)
    scr = _scratch(lib.gpr_fill_scratch_doubles(pn, nXa.size, V), u)
    _lib.check(lib.gpr_fill_ghost_cells(
        _dev(g, "grids"), _dev(_u8(m), "masks", torch.uint8), _dev(u, "u"), pn, nXa.size, pd,
        float(dt), pp, 2, _dev(scr, "s"), _dev(status, "status", torch.int32), V, _stream()),
        "fill_ghost_cells")
    if gl:
        for k in range(2):
            grids[k].view(-1).copy_(g[k].view(-1))
    if ml:
        for k in range(2):
            masks[k].view(-1).copy_(m[k].view(-1).to(masks[k].dtype))
    return status


# ---------------------------------------------------------------------------
# system/multi/riemann.cpp

def left_star_state(QL, QR, MPL, MPR, dt, n):
    """GPRpy.system.multi.left_star_state (riemann.cpp:203-233), batched over
    the leading dimension: QL, QR [..., V], n [..., ndim]."""
    lib = _lib.load()
    QL = QL.contiguous()
    QR = QR.contiguous()
    n = n.contiguous().to(torch.float64)
    count = QL.numel() // V
    nd = n.numel() // max(count, 1)
    out = torch.empty_like(QL)
    cl, pl = _par(MPL)
    cr, pr = _par(MPR)
    _lib.check(lib.gpr_left_star_state(_dev(QL, "QL"), _dev(QR, "QR"), _dev(n, "n"),
                                       _dev(out, "out"), count, nd, float(dt), pl, pr, V,
                                       _stream()), "left_star_state")
    return out


# ---------------------------------------------------------------------------
# solvers/iterator.cpp, solvers/utils.cpp

def make_u(u, grids, masks, MPs):
    """GPRpy.solvers.make_u (solvers/iterator.cpp:12-42)."""
    lib = _lib.load()
    ncell = u.numel() // V
    arr, pp = _pars(MPs)
    g, _ = _stack(grids, (-1,), torch.float64)
    m, _ = _stack(masks, (-1,), torch.uint8)
    _lib.check(lib.gpr_make_u(_dev(u, "u"), _dev(g.contiguous(), "grids"),
                              _dev(_u8(m).contiguous(), "masks", torch.uint8), ncell, pp, 2,
                              V, _stream()), "make_u")
    return u


def renorm_distortion(u, MPs):
    """GPRpy.solvers.renorm_distortion (solvers/utils.cpp:6-23), each cell
    with the material of its level set."""
    lib = _lib.load()
    arr, pp = _pars(MPs)
    _lib.check(lib.gpr_renorm_multi(_dev(u, "u"), u.numel() // V, pp, 2, V, _stream()),
               "renorm_distortion")
    return u


def timestep_device(grids, masks, dX, CFL, t, tf, count, MPs, out=None):
    """solvers/iterator.cpp:54-83 over the masked cells of both grids;
    returns a 1-element CUDA tensor."""
    lib = _lib.load()
    dXa, pd = _f64(dX)
    arr, pp = _pars(MPs)
    g, _ = _stack(grids, (-1,), torch.float64)
    m, _ = _stack(masks, (-1,), torch.uint8)
    ncell = m.numel() // 2
    if out is None:
        out = torch.empty(1, dtype=torch.float64, device=g.device)
    scr = _scratch(1, g)
    _lib.check(lib.gpr_timestep_multi(_dev(g.contiguous(), "grids"),
                                      _dev(_u8(m).contiguous(), "masks", torch.uint8), ncell,
                                      pd, dXa.size, float(CFL), float(t), float(tf), int(count),
                                      pp, 2, _dev(out, "dt"), _dev(scr, "s"), V, _stream()),
               "timestep")
    return out


class MultiIterator:
    """Device buffers of the two-material time loop (gpr_iterate_multi)."""

    def __init__(self, nX, dX, bcs, MPs, cfl, tf, device="cuda", contorted_tol=1.0,
                 split=False, half_step=True, stiff=False, flux=0):
        self.lib = _lib.load()
        self.split, self.half_step = int(bool(split)), int(bool(half_step))
        self.stiff, self.flux = int(bool(stiff)), int(flux)
        self.nX, self.pn = _i32(nX)
        self.dX, self.pd = _f64(dX)
        self.nd = self.nX.size
        self.bcs, self.pb = _i32(bcs if not np.isscalar(bcs) else [bcs] * 2 * self.nd)
        self.arr, self.pp = _pars(MPs)
        self.scr = torch.empty(max(int(self.lib.gpr_iterate_multi_scratch_doubles(
            self.pn, self.nd, V)), 1), dtype=torch.float64, device=device)
        self.clock = torch.tensor([0.0, 0.0, float(tf), float(cfl), 0.0], dtype=torch.float64,
                                  device=device)
        self.status = torch.zeros(4, dtype=torch.int32, device=device)
        self.contorted_tol = float(contorted_tol)

    def run(self, u, nsteps):
        """Enqueue nsteps steps on u (in place); no host synchronisation."""
        _lib.check(self.lib.gpr_iterate_multi_scheme(
            _dev(u, "u"), self.pn, self.nd, self.pd, self.pb, self.split, self.half_step,
            self.stiff, self.flux, self.pp, 2, _dev(self.clock, "clock"), int(nsteps),
            _dev(self.scr, "s"), _dev(self.status, "status", torch.int32), self.contorted_tol,
            V, _stream()), "iterate_multi")
        return u


def iterate(u, tf, nX, dX, CFL, boundaryTypes, MPs, max_steps=None, contorted_tol=1.0,
            SPLIT=False, HALF_STEP=True, STIFF=False, FLUX=0):
    """GPRpy.solvers.iterator (solvers/iterator.cpp:85-170) with the ghost
    fill: the ADER scheme (STIFF: predictor straight to the Newton pass) or
    the split scheme (SPLIT, HALF_STEP), flux FLUX (0 Rusanov, 1 Roe,
    2 Osher); the reference's 100-snapshot list, with the NaN early exit and
    the contortion reset."""
    it = MultiIterator(nX, dX, boundaryTypes, MPs, CFL, tf, device=u.device,
                       contorted_tol=contorted_tol, split=SPLIT, half_step=HALF_STEP,
                       stiff=STIFF, flux=FLUX)
    uf = u.view(-1)
    ret = [None] * 100
    push, count = 0, 0
    while True:
        uprev = uf.clone()
        it.run(uf, 1)
        t, dt, _, _, cnt = it.clock.tolist()
        if dt == 0.0:
            break
        count += 1
        if t >= (push + 1) / 100.0 * tf:
            ret[push] = uf.clone()
            push += 1
        if torch.isnan(uf).any():
            ret[push] = uprev
            if push + 1 < 100:
                ret[push + 1] = uf.clone()
            return ret
        if t >= tf or (max_steps is not None and count >= max_steps):
            break
    ret[99] = uf.clone()
    check_status(it.status)
    return ret
