"""Differentiation form: gradients of a misfit of the final states of many 1D
GPR runs with respect to their initial states and material parameters.

The forward pass is the batched time loop (phd_gb300.batch; the reference's
solvers.iterator, code/cpp/src/solvers/iterator.cpp:85-170, per instance)
with the predictor converged to a tight tolerance, so that its result is the
fixed point the adjoint differentiates.  It keeps a checkpoint of the states
and clocks every `checkpoint_every` steps.  The backward pass walks the
segments in reverse: it restores a checkpoint, recomputes the segment while
recording a tape per step, and runs the hand-written backward step of the
CUDA library over the tape (include/gpr_gb300.h, "Adjoint").

Material parameters enter through six device fields per instance
(FIELDS); `make_par(theta)` builds a Par from a user parameter vector, and
the chain rule d(fields)/d(theta) is taken by complex-step differentiation
of the same builder (exact to rounding for the analytic maps involved).

`solve(u0, theta, problem)` is a torch.autograd.Function: `uN = solve(...)`
then `loss(uN).backward()` fills `u0.grad` and `theta.grad`.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .batch import BC
from .params import GprParC

FIELDS = ("gamma", "iG", "b02", "th1c", "calpha2", "ikappa")


def dev_fields(MP):
    """The six differentiable device fields of a stiffened-gas Par (complex
    attributes allowed): gamma, 1/(gamma-1), b0^2, rho0/(2 mu^(1/n)),
    calpha^2, 1/kappa."""
    n = MP.n if MP.n else 1.0
    return [MP.gamma, 1.0 / (MP.gamma - 1.0), MP.b02, MP.rho0 / (2.0 * MP.mu ** (1.0 / n)),
            MP.calpha2, 1.0 / MP.kappa]


def field_jacobian(make_par, theta, h=1e-30):
    """d(dev_fields)/d(theta), 6 x len(theta), by complex steps."""
    theta = np.asarray(theta, dtype=np.float64)
    J = np.zeros((len(FIELDS), theta.size))
    for j in range(theta.size):
        th = theta.astype(np.complex128)
        th[j] += 1j * h
        J[:, j] = np.imag(np.array(dev_fields(make_par(th)), dtype=np.complex128)) / h
    return J


class Problem:
    """A batch of 1D instances for the differentiable loop.

    nx: cells per instance; dx: cell widths; bcs: boundary name or code per
    instance; cfl, tf: as the reference's iterator; make_par(theta) -> Par.
    frozen_dt: differentiate with each step's dt held fixed (False: through
    the CFL rule).  dg_tol / dg_it: predictor stopping rule of the forward.
    checkpoint_every: steps per segment; the backward pass restores each
    segment's checkpoint and recomputes its steps with a tape.
    tape_budget_bytes: device memory the forward pass may spend on keeping
    the tapes of whole segments as it runs (0: none, the classic
    checkpointing); a segment taped in the forward needs no recompute in the
    backward.  The first segments that fit are kept.
    """

    def __init__(self, nx, dx, bcs, make_par, cfl=0.8, tf=1.0, nvar=17, frozen_dt=False,
                 dg_tol=1e-13, dg_it=300, checkpoint_every=32, tape_budget_bytes=0,
                 device="cuda"):
        self.lib = _lib.load()
        self.nx = np.ascontiguousarray(np.asarray(nx, dtype=np.int32))
        self.ninst = self.nx.size
        self.dx = np.ascontiguousarray(np.asarray(dx, dtype=np.float64).reshape(self.ninst))
        codes = []
        for b in (bcs if isinstance(bcs, (list, tuple)) else [bcs] * self.ninst):
            c = BC[b] if isinstance(b, str) else int(b)
            codes += [c, c]
        self.bcs = np.ascontiguousarray(np.array(codes, dtype=np.int32))
        self.make_par = make_par
        self.cfl, self.tf, self.V = float(cfl), float(tf), int(nvar)
        self.frozen_dt = bool(frozen_dt)
        self.dg_tol, self.dg_it = float(dg_tol), int(dg_it)
        self.K = int(checkpoint_every)
        self.device = torch.device(device)
        self.nu = int(self.nx.sum())
        self.nb = int((self.nx + 2).sum())
        self.off = np.concatenate([[0], np.cumsum(self.nx)]).astype(np.int64)
        n = self.lib.gpr_batch_scratch_doubles(self.ninst, self._p(self.nx), self.V)
        self.scratch = torch.empty(_lib.check(n, "batch_scratch_doubles"), dtype=torch.float64,
                                   device=self.device)
        n = self.lib.gpr_adj_tape_doubles(self.ninst, self._p(self.nx), self.V)
        self.tape_len = _lib.check(n, "adj_tape_doubles")
        n = self.lib.gpr_adj_scratch_doubles(self.ninst, self._p(self.nx), self.V)
        self.ascratch = torch.empty(_lib.check(n, "adj_scratch_doubles"), dtype=torch.float64,
                                    device=self.device)
        self.tapes = None
        self.tape_budget = int(tape_budget_bytes)
        self.seg_tapes = {}  # segment start step -> [K, tape_len] tapes kept by the forward
        self.clock = torch.zeros(5 * self.ninst, dtype=torch.float64, device=self.device)
        self.status = torch.zeros(self.nb, dtype=torch.int32, device=self.device)
        self.info = torch.zeros(self.nb, dtype=torch.int32, device=self.device)
        self.schedule = []   # per-step dt [ninst] (device)
        self.checkpoints = []
        self.nsteps = 0
        self.pars = None

    # -- plumbing -----------------------------------------------------------
    @staticmethod
    def _p(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    @staticmethod
    def _t(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None

    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _init(self, pars):
        cp = (GprParC * self.ninst)()
        for k, MP in enumerate(pars):
            cp[k] = MP.to_ctypes()
        rc = self.lib.gpr_adj_supported(self.ninst, ctypes.cast(cp, ctypes.c_void_p),
                                        self._p(self.bcs), self.V)
        if rc != 0:
            raise RuntimeError("the adjoint supports the stiffened-gas EOS, Newtonian "
                               "viscosity, beta = 0, Tref = 0 and non-moving boundaries")
        _lib.check(self.lib.gpr_batch_init(
            self._t(self.clock), self.ninst, self._p(self.nx), self._p(self.dx),
            self._p(self.bcs), ctypes.cast(cp, ctypes.c_void_p), self.cfl, self.tf,
            self._t(self.scratch), self.V, self._stream()), "batch_init")
        self._cpars = cp

    def _step(self, u, tape, step, replay):
        """One forward step; replay=True reads dt from the recorded schedule."""
        if replay:
            dt_io, mode = self.schedule[step], 1
        else:
            if step == len(self.schedule):
                self.schedule.append(torch.zeros(self.ninst, dtype=torch.float64,
                                                 device=self.device))
            dt_io, mode = self.schedule[step], 0
        _lib.check(self.lib.gpr_adj_forward_step(
            self._t(u), self._t(self.clock), self.ninst, self._p(self.nx),
            self._t(self.scratch), self._t(tape), self._t(dt_io), mode, self.dg_tol,
            self.dg_it, self._t(self.status), self.V, self._stream()), "adj_forward_step")

    def _done(self):
        c = self.clock.view(-1, 5).cpu().numpy()
        return bool(np.all(c[:, 0] >= c[:, 2]))

    # -- forward / backward ---------------------------------------------------
    def forward(self, u0, pars, schedule=None, max_steps=None):
        """Run every instance to tf from the packed states u0 [nu, V]
        (or flat).  schedule: a list of per-step dt tensors to replay (a
        fixed-step forward, e.g. for finite differences of the frozen-dt
        adjoint).  Returns the packed final states."""
        self.pars = list(pars)
        self._init(self.pars)
        u = u0.detach().to(self.device, torch.float64).reshape(-1).clone()
        if schedule is not None:
            self.schedule = list(schedule)
        else:
            self.schedule = []
        replay = schedule is not None
        self.checkpoints = []
        self.seg_tapes = {}
        seg_bytes = self.K * self.tape_len * 8
        kept = 0
        tape = None
        step = 0
        # the clocks are checked once per segment; steps taken after an
        # instance reached tf have dt = 0 and change nothing
        while True:
            if replay and step >= len(self.schedule):
                break
            if max_steps is not None and step >= max_steps:
                break
            if step % self.K == 0:
                if not replay and self._done():
                    break
                self.checkpoints.append((step, u.clone(), self.clock.clone()))
                tape = None
                if kept + seg_bytes <= self.tape_budget:
                    tape = torch.empty(self.K, self.tape_len, dtype=torch.float64,
                                       device=self.device)
                    self.seg_tapes[step] = tape
                    kept += seg_bytes
            self._step(u, tape[step % self.K] if tape is not None else None, step, replay)
            step += 1
        self.nsteps = step
        self.replayed = replay
        return u.view(-1, self.V)

    def backward(self, ubar_final):
        """Cotangents of the initial states [nu, V] and of the six device
        fields [ninst, 6], given the cotangent of the final states."""
        if self.tapes is None:
            self.tapes = [torch.empty(self.tape_len, dtype=torch.float64, device=self.device)
                          for _ in range(self.K)]
        ubar = ubar_final.detach().to(self.device, torch.float64).reshape(-1).clone()
        thbar = torch.zeros(self.ninst * 6, dtype=torch.float64, device=self.device)
        tbar = torch.zeros(self.ninst, dtype=torch.float64, device=self.device)
        self.info.zero_()
        self.recomputed_steps = 0
        for (s0, u_ck, clk_ck) in reversed(self.checkpoints):
            n = min(self.K, self.nsteps - s0)
            tapes = self.seg_tapes.get(s0)
            if tapes is None:  # recompute the segment from its checkpoint
                tapes = self.tapes
                u = u_ck.clone()
                self.clock.copy_(clk_ck)
                for j in range(n):
                    self._step(u, tapes[j], s0 + j, self.replayed)
                self.recomputed_steps += n
            else:  # the forward's own tape; the backward step needs the clock
                self.clock.copy_(clk_ck)
            for j in reversed(range(n)):
                _lib.check(self.lib.gpr_adj_backward_step(
                    self._t(ubar), self._t(thbar), self._t(tbar), int(self.frozen_dt),
                    self.ninst, self._p(self.nx), self._t(self.scratch), self._t(tapes[j]),
                    self._t(self.ascratch), self._t(self.info), self.V, self._stream()),
                    "adj_backward_step")
        bad = (self.info & 0xff) != 0
        if bool(bad.any().item()):
            raise RuntimeError("transposed predictor iteration did not converge in %d cells"
                               % int(bad.sum().item()))
        # mean transposed-iteration count per predictor cell and step
        self.adj_iterations = float((self.info >> 8).sum().item()) / max(
            1, self.nb * self.nsteps)
        return ubar.view(-1, self.V), thbar.view(self.ninst, 6)

    def theta_grad(self, fieldbar, theta):
        """Chain rule from the six device fields to the user parameters."""
        fb = fieldbar.detach().cpu().numpy()
        theta = np.asarray(theta, dtype=np.float64).reshape(self.ninst, -1)
        out = np.zeros_like(theta)
        for k in range(self.ninst):
            out[k] = fb[k] @ field_jacobian(self.make_par, theta[k])
        return out


class _Solve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, theta, problem):
        th = theta.detach().cpu().numpy().reshape(problem.ninst, -1)
        pars = [problem.make_par(th[k]) for k in range(problem.ninst)]
        uN = problem.forward(u0, pars)
        ctx.problem = problem
        ctx.theta = th
        ctx.theta_meta = (theta.dtype, theta.device, theta.shape)
        return uN.clone().view(u0.shape)

    @staticmethod
    def backward(ctx, gN):
        prob = ctx.problem
        ub0, fb = prob.backward(gN.contiguous())
        g = prob.theta_grad(fb, ctx.theta)
        dtype, device, shape = ctx.theta_meta
        gth = torch.tensor(g, dtype=dtype, device=device).view(shape)
        return ub0.view(gN.shape), gth, None


def solve(u0, theta, problem):
    """Final states of every instance; differentiable in u0 and theta."""
    return _Solve.apply(u0, theta, problem)
