"""Time loop of the reference's `solvers.iterator` (code/cpp/src/solvers/
iterator.cpp:85-170) for one material, on the GPU: CFL time step ->
boundaries -> ADER step (or the split scheme, SPLIT = True) -> distortion
renormalisation -> contortion reset (solvers/utils.cpp:44-85), with the
reference's 100-snapshot return convention and NaN early exit."""
import numpy as np
import torch

from . import api

N = api.N


class Stepper:
    """Device buffers for repeated steps of one grid (no per-step allocation)."""

    def __init__(self, nX, V, device="cuda"):
        from . import _lib
        self.lib = _lib.load()
        self.nX = np.asarray(nX, dtype=np.int32)
        self.nd = self.nX.size
        self.V = V
        ncb = int(np.prod(self.nX + 2))
        self.ub = torch.empty(int(np.prod(self.nX + 2 * N)) * V, dtype=torch.float64,
                              device=device)
        self.mask = torch.ones(ncb, dtype=torch.uint8, device=device)
        self.status = torch.zeros(ncb, dtype=torch.int32, device=device)
        self.dt = torch.empty(1, dtype=torch.float64, device=device)
        self.flag = torch.zeros(1, dtype=torch.int32, device=device)

    def step(self, u, dt, dX, bcs, MP, flux=0, stiff=False, split=False, half_step=True,
             contorted_tol=None):
        api.boundaries(u, self.ub, self.nX, bcs)
        if split:
            api.split_stepper(u, self.ub, self.nX, dt, dX, half_step, flux, MP, self.mask)
        else:
            api.ader_stepper(u, self.ub, self.nX, dt, dX, stiff, flux, MP, self.mask,
                             status=self.status)
        api.renorm_distortion(u, [MP])
        if contorted_tol is not None:
            api.reset_contorted(u, contorted_tol, [MP], flag=self.flag)
        return u


def iterate(u, tf, nX, dX, CFL, boundaryTypes, SPLIT=False, HALF_STEP=True, STIFF=False,
            FLUX=0, MPs=None, max_steps=None, contorted_tol=1.0):
    MP = MPs[0] if isinstance(MPs, (list, tuple)) else MPs
    nXa = np.asarray(nX, dtype=np.int32)
    V = u.numel() // int(np.prod(nXa))
    api.set_nvar(V)
    st = Stepper(nXa, V, device=u.device)
    uf = u.view(-1)
    ret = [None] * 100
    t, count, push = 0.0, 0, 0
    while t < tf:
        uprev = uf.clone()
        dt = float(api.timestep_device(uf, dX, CFL, t, tf, count, MP, out=st.dt).item())
        st.step(uf, dt, dX, boundaryTypes, MP, flux=FLUX, stiff=STIFF, split=SPLIT,
                half_step=HALF_STEP, contorted_tol=contorted_tol)
        t += dt
        count += 1
        if t >= (push + 1) / 100.0 * tf:
            ret[push] = uf.clone()
            push += 1
        if torch.isnan(uf).any():
            ret[push] = uprev
            if push + 1 < 100:
                ret[push + 1] = uf.clone()
            return ret
        if max_steps is not None and count >= max_steps:
            break
    ret[99] = uf.clone()
    return ret
