"""Batched form: many independent 1D GPR grids advanced together.

Each instance has its own cell count, material, boundary codes and CFL
clock (the reference runs one grid per `solvers.iterator` call,
code/cpp/src/solvers/iterator.cpp:85-170).  All instances are packed into
one device buffer and every stage of the step is one kernel launch for all of
them; the step loop needs no host synchronisation and can be captured in a
CUDA graph (`capture`).  The launch shapes of the stages (threads per block,
the face pass's lane layout) are chosen per batch by the library's autotuner
(`autotune`, run by the constructor unless autotune=False).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .params import GprParC

BC = {"transitive": 0, "transmissive": 0, "periodic": 1, "slip": 2, "stick": 3,
      "moving": 4, "symmetric": 5}


class Batch:
    """instances: list of (u0 [nx, V] array, Par, dx, bcs) tuples."""

    SHAPE_NAMES = ("weno_block", "first_block", "picard_block", "faces_four_lanes",
                   "faces_block", "cells_block")

    def __init__(self, instances, cfl=0.8, tf=0.2, device="cuda", autotune=True):
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.V = int(instances[0][0].shape[-1])
        self.ninst = len(instances)
        self.nx = np.array([inst[0].shape[0] for inst in instances], dtype=np.int32)
        self.off = np.concatenate([[0], np.cumsum(self.nx)]).astype(np.int64)
        dx = np.array([float(inst[2][0] if np.ndim(inst[2]) else inst[2]) for inst in instances])
        bcs = []
        for inst in instances:
            b = inst[3]
            code = BC[b] if isinstance(b, str) else int(b)
            bcs += [code, code]
        self.dx = np.ascontiguousarray(dx)
        self.bcs = np.ascontiguousarray(np.array(bcs, dtype=np.int32))
        pars = (GprParC * self.ninst)()
        for k, inst in enumerate(instances):
            pars[k] = inst[1].to_ctypes()
        self._pars = pars
        u = np.concatenate([np.asarray(inst[0], dtype=np.float64).reshape(-1, self.V)
                            for inst in instances])
        self.u = torch.tensor(u.reshape(-1), dtype=torch.float64, device=self.device)
        self.clock = torch.zeros(5 * self.ninst, dtype=torch.float64, device=self.device)
        nscr = self.lib.gpr_batch_scratch_doubles(self.ninst, self._p(self.nx), self.V)
        _lib.check(nscr, "batch_scratch_doubles")
        self.scratch = torch.empty(nscr, dtype=torch.float64, device=self.device)
        self.status = torch.zeros(int((self.nx + 2).sum()), dtype=torch.int32,
                                  device=self.device)
        self.updates = torch.zeros(1, dtype=torch.int64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.gpr_batch_init(
                self._t(self.clock), self.ninst, self._p(self.nx), self._p(self.dx),
                self._p(self.bcs), ctypes.cast(pars, ctypes.c_void_p), float(cfl), float(tf),
                self._t(self.scratch), self.V, self._stream()), "batch_init")
        self.tuning = None
        if autotune:
            self.autotune()

    def autotune(self):
        """Time the candidate launch shapes on the current state and keep the
        fastest (gpr_batch_autotune); returns {name: value} of the choice
        and keeps the per-candidate times in self.tuning."""
        shapes = np.zeros(6, np.int32)
        times = np.zeros(22, np.float32)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.gpr_batch_autotune(
                self._t(self.u), self._t(self.clock), self.ninst, self._p(self.nx),
                self._t(self.scratch), self._p(shapes), self._p(times), self.V,
                self._stream()), "batch_autotune")
        self.tuning = {"shapes": dict(zip(self.SHAPE_NAMES, shapes.tolist())),
                       "candidate_ms": times.tolist()}
        return self.tuning["shapes"]

    def shapes(self):
        """The launch shapes gpr_batch_iterate uses for this batch."""
        out = np.zeros(6, np.int32)
        _lib.check(self.lib.gpr_batch_get_shapes(self._t(self.scratch), self._p(out)),
                   "batch_get_shapes")
        return dict(zip(self.SHAPE_NAMES, out.tolist()))

    def set_shapes(self, shapes):
        """Launch with the given shapes ({name: value} or a sequence of 6)."""
        vals = [shapes[k] for k in self.SHAPE_NAMES] if isinstance(shapes, dict) else shapes
        a = np.ascontiguousarray(np.asarray(vals, dtype=np.int32))
        _lib.check(self.lib.gpr_batch_set_shapes(self._t(self.scratch), self._p(a)),
                   "batch_set_shapes")

    @staticmethod
    def _p(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    @staticmethod
    def _t(t):
        return ctypes.c_void_p(t.data_ptr())

    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def step(self, nsteps=1):
        """Enqueue nsteps steps of every instance on the current stream."""
        _lib.check(self.lib.gpr_batch_iterate(
            self._t(self.u), self._t(self.clock), self.ninst, self._p(self.nx), int(nsteps),
            self._t(self.scratch), self._t(self.status), self._t(self.updates), self.V,
            self._stream()), "batch_iterate")

    def capture(self, nsteps=1):
        """A CUDA graph of nsteps steps (replay with graph.replay())."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.step(nsteps)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g

    def state(self, k):
        """Instance k's state as a [nx, V] tensor view."""
        a, b = int(self.off[k]), int(self.off[k + 1])
        return self.u.view(-1, self.V)[a:b]

    def times(self):
        c = self.clock.view(-1, 5).cpu().numpy()
        return c[:, 0], c[:, 4].astype(int)

    def done(self):
        t, _ = self.times()
        return bool(np.all(t >= self.clock.view(-1, 5)[:, 2].cpu().numpy()))
