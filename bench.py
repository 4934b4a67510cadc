"""Benchmark of the GB300 GPR ADER-WENO step.

Workload: 2D Taylor-Green vortex, 512 x 512 cells on [0, 2pi]^2, V = 17
(viscous + heat conduction), FP64, N = 2, Rusanov flux, periodic boundaries,
cs = 10, mu = 1e-2.  A step is one full time step of the reference's
iterator for one material: CFL time step -> boundaries -> WENO -> space-time
predictor -> FV update -> distortion renormalisation, device resident (dt
never leaves the GPU).  Metric: cell-updates per second (one interior cell
advanced one time step), whole job.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU oracle (a C restatement of the reference
solver; the reference's own C++ cannot be built on the GPU host) on the host
cores, on the same 512 x 512 problem for the requested steps, and prints its
own JSON line.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# The headline metric; "value" is its first part (plain path, TGV 512^2
# step), the batched form and adjoint / forward ratio are the "batched" and
# "adjoint" objects of the same line.
METRIC = "FP64 Mcell-updates/s plain vs batched; adjoint\u00f7forward time at 1e-6 grad err"
UNIT = "Mcell-updates/s"

# Algorithmic FP64 operation counts per unit of work of the algorithm the
# kernels implement (add/sub/mul/div/sqrt = 1 flop, transcendental call = 1;
# the FP32 start of the wave-speed root iteration is not counted), counted by
# oracle/opcount_device.cpp on the device physics compiled for the host.  The
# reference's own formulation needs ~2x more (oracle/opcount.cpp: it
# recomputes the pressure per call and runs a QR eigen-solve per wave
# speed); the roofline uses the work this implementation has to do.
# The reference driver's contortion tolerance (code/python/main.py:21): a
# step resets every distortion when one cell's normalised distortion exceeds
# 1 + CONTORTED_TOL.
CONTORTED_TOL = 1.0

# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# the TGV 512^2 kernels, from an earlier ncu capture of each (not measured by
# this script; the line labels it so).
TRAFFIC = {
    # one in-place face pass (x faces of even index): every predictor
    # cell's qh read (each cell has a face of each parity) and u updated
    "k_faces2d": 323.219456e6 + 159.500544e6,
    "k_predictor_picard": 143.945728e6 + 229.694720e6,
}

OPS = {
    "predictor_per_cell_iter": 4904.0,    # per predictor cell and Picard iteration
    "face_quadrature_point": 1427.0,      # D_RUS + Bint + extrapolation, per point
    "cells_per_cell": 2293.0,             # volume term (both time nodes), per cell
    "weno_point": 48.0,                   # per (cell, variable, sweep)
    "cfl_per_cell": 848.0,                # per cell (two max_abs_eigs)
}
# the same for the 1D kernels (the batched form)
OPS_1D = {
    "predictor_per_cell_iter": 1840.0,    # per predictor cell and Picard iteration
    "face_point": 1423.0,                 # per (face, time node)
    "cells_per_cell": 963.0,              # volume term, per cell
    "weno_per_cell": 816.0,               # per predictor cell (17 points)
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--cfl", type=float, default=0.4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-issue", action="store_true",
                    help="print the FP64 issue-rate probe (cycles per warp instruction) and exit")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-shock-bubble", action="store_true")
    ap.add_argument("--profile-shock-bubble", type=int, default=0, metavar="NX",
                    help="run --profile-steps steps of the NX x NX/2 shock bubble only "
                         "(for ncu captures)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="run only this many steps (for ncu captures), no JSON")
    ap.add_argument("--profile-flux", type=int, default=0,
                    help="with --profile-steps: the TGV steps' flux (0 Rusanov, 1 Roe, 2 Osher)")
    ap.add_argument("--profile-shock-tube", type=int, default=-1, metavar="FLUX",
                    help="with --profile-steps K: K steps of the 200-cell shock tube with "
                         "flux FLUX (0 Rusanov, 1 Roe, 2 Osher) through gpr_iterate, no JSON")
    ap.add_argument("--split", action="store_true",
                    help="with --profile-shock-tube: the split scheme (gpr_iterate_split)")
    ap.add_argument("--profile-batched", action="store_true",
                    help="with --profile-steps K: K steps of the 512 batched shock tubes with "
                         "the default launch shapes or --shapes, no JSON")
    ap.add_argument("--shapes", default="",
                    help="six comma-separated launch shapes for --profile-batched")
    ap.add_argument("--profile-n3", type=int, default=0, metavar="N",
                    help="with --profile-steps K: K steps of the N x N Taylor-Green vortex at "
                         "third order (N = 3 Gauss nodes), no JSON")
    ap.add_argument("--profile-adjoint", type=int, default=0, metavar="NINST",
                    help="with --profile-steps K: K steps of the Stokes differentiation "
                         "problem for NINST instances, forward then backward (for ncu "
                         "captures), no JSON")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replicas_result(ms, ncell, steps, world, device):
    """N independent replicas (one per rank, no collective in the step): the
    timed region's duration is the maximum over ranks, and the whole job
    advanced every rank's ncell cells for `steps` steps.  Returns (ms, value
    in Mcell-updates/s)."""
    import torch
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    return ms, ncell * world * steps / (ms * 1e-3) / 1e6


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline / reference arm

def cpu_baseline(steps, warmup, n=512, cfl=0.4, flux=0):
    """Oracle (C restatement of the reference solver) on all host cores,
    `steps` timed steps of the full n x n TGV (after `warmup` untimed ones):
    timestep -> boundaries -> ADER step -> renorm, the reference iterator's
    loop body (solvers/iterator.cpp:109-151)."""
    from oracle import Oracle
    from phd_gb300 import problems
    O = Oracle()
    threads = O.num_threads()
    u0, MP, tf, dX, bcs = problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    u = np.ascontiguousarray(u0).copy()
    nX = np.array([n, n], np.int32)
    ncell = n * n
    count = 0

    def one():
        nonlocal count
        dt = O.timestep(u, dX, cfl, 0, 1e9, count, MP)
        ub = O.boundaries(u, nX, [1] * 4)
        O.ader_stepper(u.reshape(-1), ub, nX, dt, dX, MP, flux=flux)
        O.renorm_distortion(u.reshape(-1), MP)
        count += 1
    for _ in range(warmup):
        one()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    el = time.perf_counter() - t0
    value = ncell * steps / el / 1e6
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "TGV %dx%d (the full grid), %d timed steps after %d warm-up, "
                      "oracle/gpr_oracle.c with %d OpenMP threads" % (n, n, steps, warmup,
                                                                      threads),
            "seconds": el, "ms_per_step": el * 1e3 / max(steps, 1)}


def step_vs_oracle(torch, u_dev, MP, nX, dX, bcs, cfl, flux=0, count=10, V=17):
    """One step of the GPU path and one oracle step from the same state
    (u_dev, left unchanged): CFL time step (taken by the oracle and given to
    both), boundaries, ADER step, renormalisation.  Returns (max |a-b| /
    (1 + |b|), oracle seconds for the step)."""
    import phd_gb300 as G
    from oracle import Oracle
    O = Oracle()
    nX = np.array(nX, np.int32)
    u_np = u_dev.detach().cpu().numpy().reshape(tuple(int(k) for k in nX) + (V,)).copy()
    t0 = time.perf_counter()
    dt = O.timestep(u_np, dX, cfl, 0.0, 1e9, count, MP)
    ub = O.boundaries(u_np, nX, bcs)
    ref = u_np.reshape(-1).copy()
    O.ader_stepper(ref, ub, nX, dt, dX, MP, flux=flux)
    O.renorm_distortion(ref, MP)
    cpu_s = time.perf_counter() - t0
    u = u_dev.detach().clone().reshape(-1)
    ubt = torch.empty(int(np.prod(nX + 4)) * V, dtype=torch.float64, device=u.device)
    G.boundaries(u, ubt, nX, bcs)
    G.solvers.ader_stepper(u, ubt, nX, dt, dX, False, flux, MP, None)
    G.solvers.renorm_distortion(u, [MP])
    got = u.cpu().numpy()
    return float(np.max(np.abs(got - ref) / (1.0 + np.abs(ref)))), cpu_s


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    cb = cpu_baseline(args.steps, args.warmup, n=args.n, cfl=args.cfl)
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "tgv2d_512x512_v17_rusanov_cfl%.2g" % args.cfl,
                       "grid": [args.n, args.n], "nvar": 17, "order_N": 2,
                       "parallelism": "cpu"},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# FP64 peak microbenchmark (own kernel): independent DFMA chains

FP64_PEAK_SRC = r"""
#include <cuda_runtime.h>
// 16 independent DFMA chains per thread; the result is consumed so nothing
// is dead code.
__global__ void dfma_peak(double *out, int iters) {
  double a[16];
#pragma unroll
  for (int k = 0; k < 16; k++)
    a[k] = threadIdx.x * 1e-9 + k;
  const double b = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
#pragma unroll
      for (int k = 0; k < 16; k++)
        a[k] = fma(a[k], b, c);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 16; k++)
    s += a[k];
  if (s == 12345.678) out[0] = s;
}
extern "C" int dfma_peak_launch(double *out, int iters, int grid, int block, void *stream) {
  dfma_peak<<<grid, block, 0, (cudaStream_t)stream>>>(out, iters);
  return (int)cudaGetLastError();
}
"""


# FP64 tensor-core throughput (DMMA: mma.sync m8n8k4 f64, 512 flops per warp
# instruction) measured the same way, to decide DMMA against DFMA for the
# small FP64 contractions of the path: 8 independent accumulator chains per
# warp, operands in registers, one guarded store so nothing is dead code.
DMMA_PEAK_SRC = r"""
#include <cuda_runtime.h>
__global__ void dmma_peak(double *out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-9, b = 0.999999999;
  double c[8][2];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    c[k][0] = k * 1e-3;
    c[k][1] = k * 2e-3;
  }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, "
                   "{%0, %1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++)
    s += c[k][0] + c[k][1];
  if (s == 12345.678) out[0] = s;
}
extern "C" int dmma_peak_launch(double *out, int iters, int grid, int block, void *stream) {
  dmma_peak<<<grid, block, 0, (cudaStream_t)stream>>>(out, iters);
  return (int)cudaGetLastError();
}
"""


# FP64 issue rate of one warp and of one SM (own kernel): each thread of one
# block runs `iters` dependent DFMAs (or four independent chains) if its lane
# is below `active`; clock64 around the loop.  Cycles per warp instruction
# against active lanes and warps per block show what bounds a kernel whose
# few warps each run a long FP64 chain (the small 1D grids).
FP64_ISSUE_SRC = r"""
#include <cuda_runtime.h>
__global__ void fp64_issue(double *out, long long *cyc, int active, int iters, int ilp) {
  const int lane = threadIdx.x & 31;
  double a = 1.0 + threadIdx.x * 1e-9, a2 = a + 1e-3, a3 = a + 2e-3, a4 = a + 3e-3;
  const double b = 0.999999, c = 1e-7;
  __syncwarp();
  const long long t0 = clock64();
  if (lane < active) {
    if (ilp == 1) {
      for (int i = 0; i < iters; i++)
        a = fma(a, b, c);
    } else {
      for (int i = 0; i < iters; i++) {
        a = fma(a, b, c);
        a2 = fma(a2, b, c);
        a3 = fma(a3, b, c);
        a4 = fma(a4, b, c);
      }
    }
  }
  __syncwarp();
  const long long t1 = clock64();
  out[threadIdx.x] = a + a2 + a3 + a4;
  if (threadIdx.x == 0)
    cyc[0] = t1 - t0;
}
extern "C" int fp64_issue_launch(double *out, long long *cyc, int active, int iters, int ilp,
                                 int block, void *stream) {
  fp64_issue<<<1, block, 0, (cudaStream_t)stream>>>(out, cyc, active, iters, ilp);
  return (int)cudaGetLastError();
}
"""


def fp64_issue_probe(torch):
    """Cycles per FP64 warp instruction of one block on one SM, for 1 / 4 / 8
    warps, 1 and 32 active lanes, dependent and four-way independent chains:
    one JSON line."""
    from phd_gb300 import _lib
    bdir = os.path.join(ROOT, "phd_gb300", "_build")
    so = os.path.join(bdir, "fp64issue.so")
    src = os.path.join(bdir, "fp64issue.cu")
    os.makedirs(bdir, exist_ok=True)
    if not os.path.exists(so) or not os.path.exists(src) or open(src).read() != FP64_ISSUE_SRC:
        open(src, "w").write(FP64_ISSUE_SRC)
        subprocess.run(["nvcc"] + _lib.ARCH + ["-O3", "-shared", "-Xcompiler", "-fPIC", "-o",
                                               so, src], check=True)
    lib = ctypes.CDLL(so)
    lib.fp64_issue_launch.restype = ctypes.c_int
    lib.fp64_issue_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 4 + [
        ctypes.c_void_p]
    out = torch.zeros(256, dtype=torch.float64, device="cuda")
    cyc = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    iters = 4096
    rows = []
    for ilp in (1, 4):
        for block in (32, 128, 256):
            for active in (1, 32):
                for _ in range(2):  # the second launch is the one kept
                    assert lib.fp64_issue_launch(ctypes.c_void_p(out.data_ptr()),
                                                 ctypes.c_void_p(cyc.data_ptr()), active, iters,
                                                 ilp, block, stream) == 0
                torch.cuda.synchronize()
                per = float(cyc.item()) / (iters * ilp)
                rows.append({"independent_chains": ilp, "warps_per_sm": block // 32,
                             "active_lanes": active,
                             "cycles_per_warp_fp64_instruction": round(per, 1)})
    print(json.dumps({"fp64_issue": rows, "iters": iters}), flush=True)
    return 0


def dmma_peak_tflops(torch):
    """Measured FP64 tensor-core (DMMA) throughput of this GPU in TFLOP/s."""
    from phd_gb300 import _lib
    bdir = os.path.join(ROOT, "phd_gb300", "_build")
    so = os.path.join(bdir, "dmmapeak.so")
    src = os.path.join(bdir, "dmmapeak.cu")
    os.makedirs(bdir, exist_ok=True)
    if not os.path.exists(so) or not os.path.exists(src) or open(src).read() != DMMA_PEAK_SRC:
        open(src, "w").write(DMMA_PEAK_SRC)
        subprocess.run(["nvcc"] + _lib.ARCH + ["-O3", "-shared", "-Xcompiler", "-fPIC", "-o",
                                               so, src], check=True)
    lib = ctypes.CDLL(so)
    lib.dmma_peak_launch.restype = ctypes.c_int
    lib.dmma_peak_launch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_void_p]
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    iters = 1024
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    grid, block = sms * 4, 256
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    po = ctypes.c_void_p(out.data_ptr())
    assert lib.dmma_peak_launch(po, iters, grid, block, stream) == 0
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        e0.record()
        lib.dmma_peak_launch(po, iters, grid, block, stream)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        flops = 512.0 * 8 * iters * grid * (block // 32)
        best = max(best, flops / (ms * 1e-3) / 1e12)
    return best


def fp64_peak_tflops(torch):
    """Measured FP64 FMA throughput of this GPU (TFLOP/s, 2 flops per DFMA),
    from an own kernel of independent DFMA chains."""
    from phd_gb300 import _lib
    bdir = os.path.join(ROOT, "phd_gb300", "_build")
    so = os.path.join(bdir, "fp64peak.so")
    src = os.path.join(bdir, "fp64peak.cu")
    os.makedirs(bdir, exist_ok=True)
    if not os.path.exists(so) or not os.path.exists(src) or open(src).read() != FP64_PEAK_SRC:
        open(src, "w").write(FP64_PEAK_SRC)
        subprocess.run(["nvcc"] + _lib.ARCH + ["-O3", "-shared", "-Xcompiler", "-fPIC", "-o",
                                               so, src], check=True)
    lib = ctypes.CDLL(so)
    lib.dfma_peak_launch.restype = ctypes.c_int
    lib.dfma_peak_launch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_void_p]
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    iters = 1024
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    grid, block = sms * 4, 256
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    po = ctypes.c_void_p(out.data_ptr())
    assert lib.dfma_peak_launch(po, iters, grid, block, stream) == 0
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        e0.record()
        lib.dfma_peak_launch(po, iters, grid, block, stream)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        flops = 2.0 * 16 * 8 * iters * grid * block
        best = max(best, flops / (ms * 1e-3) / 1e12)
    return best


# ---------------------------------------------------------------------------
# GB300 arm

def run_gb300(args):
    import torch
    import phd_gb300 as G
    from phd_gb300 import _lib, api

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    lib = _lib.load()

    n = args.n
    u0, MP, tf, dX, bcs = G.problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    V = 17
    nX = np.array([n, n], np.int32)
    ncell = n * n
    pn = nX.ctypes.data_as(ctypes.c_void_p)
    dXa = np.array(dX, dtype=np.float64)
    pd = dXa.ctypes.data_as(ctypes.c_void_p)
    bc = np.array([1, 1, 1, 1], np.int32)
    pb = bc.ctypes.data_as(ctypes.c_void_p)
    cpar = MP.to_ctypes()
    pp = ctypes.cast(ctypes.pointer(cpar), ctypes.c_void_p)

    u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device=dev)
    nscr = lib.gpr_iterate_scratch_doubles(pn, 2, V)
    scratch = torch.empty(nscr, dtype=torch.float64, device=dev)
    status = torch.zeros((n + 2) * (n + 2), dtype=torch.int32, device=dev)
    clock = torch.tensor([0.0, 0.0, 1e9, args.cfl, 0.0], dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    flux = args.profile_flux if args.profile_steps else 0

    def step(k=1, uu=None):
        uu = u if uu is None else uu
        _lib.check(lib.gpr_iterate(ctypes.c_void_p(uu.data_ptr()), pn, 2, pd, pb, flux, pp, None,
                                   ctypes.c_void_p(clock.data_ptr()), k,
                                   ctypes.c_void_p(scratch.data_ptr()),
                                   ctypes.c_void_p(status.data_ptr()), CONTORTED_TOL, V, sp),
                   "iterate")

    if args.profile_steps:
        for _ in range(args.profile_steps):
            step()
        torch.cuda.synchronize()
        return 0

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as cs:
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms, value = replicas_result(e0.elapsed_time(e1), ncell, args.steps, world, dev)
    ms_per_step = ms / args.steps
    st = status.cpu().numpy()
    iters = (st >> 8)
    kind = st & 0xff
    picard_ok = kind == 0
    newton = kind == 1
    hist = np.bincount(iters[picard_ok], minlength=1).tolist()
    nhist = np.bincount(iters[newton], minlength=1).tolist() if newton.any() else []
    mean_iters = float(iters[picard_ok].mean()) if picard_ok.any() else 0.0
    mean_newton = float(iters[newton].mean()) if newton.any() else 0.0
    failed = int((kind == 2).sum())
    clk = clock.cpu().numpy()

    # stage timing (CUDA events on the launching stream) for the roofline
    stage_ms = stage_times(lib, torch, u, MP, nX, dXa, bc, args.cfl, V, dev, sp, stream)

    # end-to-end through the C ABI with host buffers: H2D of the state,
    # one step, D2H of the state, every step
    host = torch.empty(ncell * V, dtype=torch.float64, pin_memory=True)
    host.copy_(u.cpu())
    ue = torch.empty_like(u)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    f0.record(stream)
    for _ in range(args.steps):
        ue.copy_(host, non_blocking=True)
        step(uu=ue)
        host.copy_(ue, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = f0.elapsed_time(f1)
    e2e_value = ncell * world * args.steps / (e2e_ms * 1e-3) / 1e6

    peak = None
    try:
        peak = fp64_peak_tflops(torch)
    except Exception as ex:  # report, do not hide
        peak_err = str(ex)
    else:
        peak_err = None

    roof = roofline(stage_ms, ncell, n, mean_iters, peak)
    try:
        roof["dmma_peak_tflops"] = dmma_peak_tflops(torch)
        roof["dmma_note"] = ("FP64 tensor-core (mma.sync m8n8k4 f64) throughput measured "
                             "beside the DFMA peak; the path's contractions stay on DFMA "
                             "unless this is higher")
    except Exception as ex:  # reported, not fatal to the line
        roof["dmma_error"] = str(ex)
    batched = None
    if rank == 0 and not args.no_batched:
        try:
            batched = batched_bench(torch)
        except Exception as ex:
            batched = {"error": str(ex)}
    shock = None
    if rank == 0 and not args.no_batched:
        try:
            shock = shock_tube_bench(torch)
        except Exception as ex:  # reported, not fatal to the main line
            shock = {"error": str(ex)}
    flux2d = None
    if rank == 0 and not args.no_shock_bubble:
        try:
            flux2d = flux2d_bench(torch, cpu=not args.no_cpu_baseline)
        except Exception as ex:  # reported, not fatal to the main line
            flux2d = {"error": str(ex)}
    cfl08 = None
    if rank == 0 and not args.no_shock_bubble:
        try:
            cfl08 = tgv_cfl08_bench(torch, cpu=not args.no_cpu_baseline)
        except Exception as ex:  # reported, not fatal to the main line
            cfl08 = {"error": str(ex)}
    third = None
    if rank == 0 and not args.no_shock_bubble:
        try:
            third = tgv_n3_bench(torch, cpu=not args.no_cpu_baseline)
        except Exception as ex:  # reported, not fatal to the main line
            third = {"error": str(ex)}
        try:
            third["roe_osher"] = tgv_n3_flux_bench(torch, cpu=not args.no_cpu_baseline)
        except Exception as ex:
            third["roe_osher"] = {"error": str(ex)}
    bubble = None
    if rank == 0 and not args.no_shock_bubble:
        try:
            bubble = shock_bubble_bench(torch, cpu_steps=0 if args.no_cpu_baseline else 2)
        except Exception as ex:  # reported, not fatal to the main line
            bubble = {"error": str(ex)}
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        try:
            adjoint = adjoint_bench(torch)
        except Exception as ex:  # reported, not fatal to the main line
            adjoint = {"error": str(ex)}
    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "tgv2d_512x512_v17_rusanov_cfl%.2g" % args.cfl,
                       "grid": [n, n], "nvar": 17, "order_N": 2, "flux": "rusanov",
                       "cfl": args.cfl, "material": "sg gamma=1.4 cv=2.5 cs=10 mu=1e-2 "
                                                    "calpha=1 Pr=2/3",
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "per-step working set (u, ub, wh, qh: ~0.5 GB) exceeds the "
                             "129 MB L2; no flush needed"},
            "predictor": {"picard_iteration_histogram": hist,
                          "mean_picard_iterations": mean_iters,
                          "newton_cells": int(newton.sum()),
                          "newton_iteration_histogram": nhist,
                          "mean_newton_iterations": mean_newton,
                          "unconverged_cells": failed},
            "sim_time": float(clk[0]), "sim_steps": int(clk[4]),
            "stage_ms": stage_ms,
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": ncell * V * 8,
                    "d2h_bytes_per_step": ncell * V * 8},
            "batched": batched,
            "shock_tube": shock,
            "tgv_roe_osher": flux2d,
            "tgv_cfl08": cfl08,
            "tgv_third_order": third,
            "shock_bubble": bubble,
            "adjoint": adjoint,
            # kernels of one 2D gpr_iterate step: k_cfl_max, k_clock_finalize,
            # k_fill_interior, k_ghosts x2, k_weno2d, k_predictor_first,
            # k_predictor_picard, k_predictor_stiff, k_cells, k_faces2d x4,
            # k_renorm, k_contorted, k_reset_distortion, k_clock_advance
            "gpu_launches": 18 * args.steps,
            "clocks": cs.summary()}
    if peak_err:
        line["roofline"]["peak_error"] = peak_err
    if not args.no_cpu_baseline:
        cb = cpu_baseline(3, 1, n=n, cfl=args.cfl)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        # one step of the timed workload against one oracle step from the
        # same state (the state the timed steps left)
        line["max_rel_diff_vs_oracle"] = step_vs_oracle(torch, u, MP, nX, dX, [1] * 4,
                                                        args.cfl)[0]
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def shock_tube_bench(torch):
    """The reference's CPU-runnable case: 1D shock tube, 200 cells, CFL 0.8,
    t_end = 0.2 (248 steps), Rusanov (FLUX 0) and Osher (FLUX 2) ADER steps,
    and the reference driver's default split scheme (SPLIT, HALF_STEP).  The whole
    run is one gpr_iterate call (dt on the device, no host synchronisation),
    captured once in a CUDA graph and timed as one replay with CUDA events
    (`gpu_ms_stream_launches`: the same call's launches on the stream); the
    oracle (C restatement of the reference) runs the same problem on the host
    cores."""
    import phd_gb300 as G
    from phd_gb300 import _lib
    from oracle import Oracle
    lib = _lib.load()
    u0, MP, tf, dX, bcs = G.problems.shock_tube(nx=200)
    nx = np.array([200], np.int32)
    dxa = np.array(dX, np.float64)
    bca = np.array([0, 0], np.int32)
    cp = MP.to_ctypes()
    V = 17
    scr = torch.empty(lib.gpr_iterate_scratch_doubles(nx.ctypes.data_as(ctypes.c_void_p), 1, V),
                      dtype=torch.float64, device="cuda")
    O = Oracle()
    out = {"workload": "shock tube 200 cells, V=17, CFL 0.8, t_end 0.2"}
    ut = torch.empty(200 * V, dtype=torch.float64, device="cuda")
    clk = torch.empty(5, dtype=torch.float64, device="cuda")
    u0d = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
    clk0 = torch.tensor([0.0, 0.0, tf, 0.8, 0.0], dtype=torch.float64, device="cuda")
    for flux, split, name in ((0, 0, "rusanov"), (2, 0, "osher"), (0, 1, "split_rusanov")):
        def run():
            # the whole run (260 >= 248 steps; steps past tf change nothing)
            # on the current stream, inputs already on the device
            ut.copy_(u0d)
            clk.copy_(clk0)
            sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            if split:  # the reference driver's default (SPLIT, HALF_STEP)
                rc = lib.gpr_iterate_split(
                    ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 1,
                    dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p),
                    flux, 1, ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
                    ctypes.c_void_p(clk.data_ptr()), 260, ctypes.c_void_p(scr.data_ptr()),
                    CONTORTED_TOL, V, sp)
            else:
                rc = lib.gpr_iterate(
                    ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 1,
                    dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p),
                    flux, ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
                    ctypes.c_void_p(clk.data_ptr()), 260, ctypes.c_void_p(scr.data_ptr()), None,
                    CONTORTED_TOL, V, sp)
            _lib.check(rc, "iterate")
        run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        torch.cuda.synchronize()
        ms_stream = e0.elapsed_time(e1)
        # the same run captured once in a CUDA graph and replayed (the loop
        # needs no host synchronisation); the run's own launches are
        # latency-bound at this size, so the replay removes launch gaps
        g = torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream()
        cs.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(cs):
            with torch.cuda.graph(g, stream=cs):
                run()
        torch.cuda.current_stream().wait_stream(cs)
        g.replay()
        torch.cuda.synchronize()
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        steps = int(clk[4].item())
        t0 = time.perf_counter()
        ref, n, _ = O.run(u0, MP, tf, dX, 0, cfl=0.8, flux=flux, split=bool(split),
                          half_step=True)
        cpu_s = time.perf_counter() - t0
        got = ut.cpu().numpy().reshape(ref.shape)
        out[name] = {"steps": steps, "gpu_ms": ms, "gpu_ms_stream_launches": ms_stream,
                     "gpu_value": 200 * steps / (ms * 1e-3) / 1e6,
                     "cpu_value": 200 * n / cpu_s / 1e6, "cpu_cores": O.num_threads(),
                     "unit": UNIT, "max_rel_diff_vs_oracle":
                         float(np.max(np.abs(got - ref) / (1.0 + np.abs(ref))))}
    return out


def flux2d_bench(torch, n=512, steps=3, warmup=1, cfl=0.4, cpu=True):
    """The 512 x 512 Taylor-Green step with the Roe (FLUX = 1, the reference
    driver's default, code/python/main.py) and Osher (FLUX = 2) dissipation:
    a V x V eigen-decomposition of the system matrix per face point (and
    path node), through gpr_iterate; the oracle runs one step of the same
    grid on the host cores from the state the timed steps left, and the GPU
    step from that state is compared with it."""
    import phd_gb300 as G
    from phd_gb300 import _lib
    lib = _lib.load()
    u0, MP, tf, dX, bcs = G.problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    V = 17
    nX = np.array([n, n], np.int32)
    pn = nX.ctypes.data_as(ctypes.c_void_p)
    dXa = np.array(dX, np.float64)
    bc = np.array([1, 1, 1, 1], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles(pn, 2, V), dtype=torch.float64,
                      device="cuda")
    out = {"workload": "tgv2d_%dx%d_v17_cfl%.2g" % (n, n, cfl)}
    for flux, name in ((1, "roe"), (2, "osher")):
        u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
        clk = torch.tensor([0.0, 0.0, 1e9, cfl, 0.0], dtype=torch.float64, device="cuda")
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def run(k):
            _lib.check(lib.gpr_iterate(
                ctypes.c_void_p(u.data_ptr()), pn, 2, dXa.ctypes.data_as(ctypes.c_void_p),
                bc.ctypes.data_as(ctypes.c_void_p), flux,
                ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
                ctypes.c_void_p(clk.data_ptr()), k, ctypes.c_void_p(scr.data_ptr()), None,
                CONTORTED_TOL, V, sp), "iterate")
        run(warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run(steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        r = {"steps": steps, "ms_per_step": ms / steps,
             "value": n * n * steps / (ms * 1e-3) / 1e6, "unit": UNIT,
             "finite": bool(torch.isfinite(u).all().item())}
        if cpu:
            # one GPU step and one oracle step from the state the timed steps
            # left: the difference, and the oracle's time for the full grid
            from oracle import Oracle
            err, cpu_s = step_vs_oracle(torch, u, MP, nX, dX, [1] * 4, cfl, flux=flux)
            r["max_rel_diff_vs_oracle"] = err
            r["cpu_baseline"] = {"value": n * n / cpu_s / 1e6, "unit": UNIT,
                                 "cores": Oracle().num_threads(), "kind": "port",
                                 "sample": "one step of the full %dx%d grid, "
                                           "oracle/gpr_oracle.c" % (n, n)}
        out[name] = r
    return out


def tgv_cfl08_bench(torch, n=512, steps=10, warmup=8, cfl=0.8, cpu=True):
    """The 512 x 512 Taylor-Green step at the production CFL 0.8 (Rusanov):
    dt ~ 3.5e-4 against the distortion relaxation time 6e-4, where the
    reference's Picard iteration fails in most predictor cells and the device
    Newton pass finishes them.  Through gpr_iterate after `warmup` steps (past
    the reduced first five); the predictor status of the last timed step
    gives the Picard and Newton iteration histograms; one GPU step and one
    oracle step (Newton fallback) from the state the timed steps left."""
    import phd_gb300 as G
    from phd_gb300 import _lib
    lib = _lib.load()
    u0, MP, tf, dX, bcs = G.problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    V = 17
    nX = np.array([n, n], np.int32)
    pn = nX.ctypes.data_as(ctypes.c_void_p)
    dXa = np.array(dX, np.float64)
    bc = np.array([1, 1, 1, 1], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles(pn, 2, V), dtype=torch.float64,
                      device="cuda")
    status = torch.zeros((n + 2) ** 2, dtype=torch.int32, device="cuda")
    u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
    clk = torch.tensor([0.0, 0.0, 1e9, cfl, 0.0], dtype=torch.float64, device="cuda")
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run(k):
        _lib.check(lib.gpr_iterate(
            ctypes.c_void_p(u.data_ptr()), pn, 2, dXa.ctypes.data_as(ctypes.c_void_p),
            bc.ctypes.data_as(ctypes.c_void_p), 0,
            ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
            ctypes.c_void_p(clk.data_ptr()), k, ctypes.c_void_p(scr.data_ptr()),
            ctypes.c_void_p(status.data_ptr()), CONTORTED_TOL, V, sp), "iterate")
    run(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run(steps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = status.cpu().numpy()
    iters, kind = st >> 8, st & 0xff
    pic, newt = kind == 0, kind == 1
    c = clk.cpu().numpy()
    r = {"workload": "tgv2d_%dx%d_v17_rusanov_cfl%.2g" % (n, n, cfl), "steps": steps,
         "warmup": warmup, "ms_per_step": ms / steps,
         "value": n * n * steps / (ms * 1e-3) / 1e6, "unit": UNIT, "dt": float(c[1]),
         "predictor": {"cells": int(st.size), "picard_cells": int(pic.sum()),
                       "newton_cells": int(newt.sum()),
                       "unconverged_cells": int((kind == 2).sum()),
                       "picard_iteration_histogram": np.bincount(iters[pic]).tolist()
                       if pic.any() else [],
                       "newton_iteration_histogram": np.bincount(iters[newt]).tolist()
                       if newt.any() else [],
                       "mean_newton_iterations": float(iters[newt].mean()) if newt.any()
                       else 0.0}}
    if cpu:
        from oracle import Oracle
        err, cpu_s = step_vs_oracle(torch, u, MP, nX, dX, [1] * 4, cfl)
        r["max_rel_diff_vs_oracle"] = err
        r["cpu_baseline"] = {"value": n * n / cpu_s / 1e6, "unit": UNIT,
                             "cores": Oracle().num_threads(), "kind": "port",
                             "sample": "one step of the full %dx%d grid with the oracle's "
                                       "Newton fallback, oracle/gpr_oracle.c" % (n, n)}
    return r


def tgv_n3_bench(torch, n=512, steps=10, warmup=8, cfl=0.4, cpu=True, profile_steps=0):
    """The 512 x 512 Taylor-Green step at N = 3 Gauss nodes (the reference's
    third-order scheme: 27 space-time nodes per cell) through
    gpr_iterate_n, after `warmup` steps (past the reduced first five); one
    GPU step and one N = 3 oracle step from the state the timed steps left.
    With profile_steps: that many steps and nothing else (ncu captures)."""
    import phd_gb300 as G
    from phd_gb300 import _lib
    lib = _lib.load()
    u0, MP, tf, dX, bcs = G.problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    V, N = 17, 3
    nX = np.array([n, n], np.int32)
    pn = nX.ctypes.data_as(ctypes.c_void_p)
    dXa = np.array(dX, np.float64)
    bc = np.array([1, 1, 1, 1], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles_n(pn, 2, V, N), dtype=torch.float64,
                      device="cuda")
    status = torch.zeros((n + 2) ** 2, dtype=torch.int32, device="cuda")
    u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
    clk = torch.tensor([0.0, 0.0, 1e9, cfl, 0.0], dtype=torch.float64, device="cuda")
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run(k):
        _lib.check(lib.gpr_iterate_n(
            ctypes.c_void_p(u.data_ptr()), pn, 2, dXa.ctypes.data_as(ctypes.c_void_p),
            bc.ctypes.data_as(ctypes.c_void_p), 0,
            ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
            ctypes.c_void_p(clk.data_ptr()), k, ctypes.c_void_p(scr.data_ptr()),
            ctypes.c_void_p(status.data_ptr()), CONTORTED_TOL, V, N, sp), "iterate_n")
    if profile_steps:
        run(profile_steps)
        torch.cuda.synchronize()
        return None
    run(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run(steps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = status.cpu().numpy()
    iters, kind = st >> 8, st & 0xff
    pic = kind == 0
    c = clk.cpu().numpy()
    r = {"workload": "tgv2d_%dx%d_v17_rusanov_cfl%.2g_N3" % (n, n, cfl), "order_N": N,
         "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
         "value": n * n * steps / (ms * 1e-3) / 1e6, "unit": UNIT, "dt": float(c[1]),
         "predictor": {"cells": int(st.size), "picard_cells": int(pic.sum()),
                       "newton_cells": int((kind == 1).sum()),
                       "unconverged_cells": int((kind == 2).sum()),
                       "picard_iteration_histogram": np.bincount(iters[pic]).tolist()
                       if pic.any() else []},
         # per step: k_cfl_max, k_clock_finalize, k_boundaries_n, k_weno2d_x_n,
         # k_weno2d_y_n, k_predictor_n, k_predictor_stiff_n, k_faces_n x2,
         # k_cells_n, k_renorm, k_contorted, k_reset_distortion, k_clock_advance
         "gpu_launches": 14 * steps}
    if cpu:
        from oracle import Oracle
        O = Oracle(N=N)
        u_np = u.detach().cpu().numpy().reshape(n, n, V).copy()
        t0 = time.perf_counter()
        dt = O.timestep(u_np, dX, cfl, 0.0, 1e9, 10, MP)
        ub = O.boundaries(u_np, nX, [1] * 4)
        ref = u_np.reshape(-1).copy()
        O.ader_stepper(ref, ub, nX, dt, dX, MP, newton_fallback=0)
        O.renorm_distortion(ref, MP)
        cpu_s = time.perf_counter() - t0
        from phd_gb300.order import for_order
        G3 = for_order(N)
        ud = u.detach().clone()
        ubt = torch.empty(ub.size, dtype=torch.float64, device="cuda")
        G3.boundaries(ud, ubt, nX, [1] * 4)
        G3.solvers.ader_stepper(ud, ubt, nX, dt, dX, False, 0, MP, None)
        G.solvers.renorm_distortion(ud, [MP])
        got = ud.cpu().numpy()
        r["max_rel_diff_vs_oracle"] = float(np.max(np.abs(got - ref) / (1.0 + np.abs(ref))))
        r["cpu_baseline"] = {"value": n * n / cpu_s / 1e6, "unit": UNIT,
                             "cores": O.num_threads(), "kind": "port",
                             "sample": "one step of the full %dx%d grid at N = 3, "
                                       "oracle/gpr_oracle.c" % (n, n)}
    return r


def tgv_n3_flux_bench(torch, n=256, steps=2, warmup=1, cfl=0.4, cpu=True):
    """The Taylor-Green step at N = 3 with the Roe (1) and Osher (2)
    dissipation through gpr_iterate_n (the eigen dissipation at each of the
    9 points of a face with three path nodes), 256 x 256 (a 512 x 512 step
    takes seconds); one GPU step and one N = 3 oracle step from the state the
    timed steps left."""
    import phd_gb300 as G
    from phd_gb300 import _lib
    lib = _lib.load()
    u0, MP, tf, dX, bcs = G.problems.taylor_green(n=n, cs=10.0, mu=1e-2)
    V, N = 17, 3
    nX = np.array([n, n], np.int32)
    pn = nX.ctypes.data_as(ctypes.c_void_p)
    dXa = np.array(dX, np.float64)
    bc = np.array([1, 1, 1, 1], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles_n(pn, 2, V, N), dtype=torch.float64,
                      device="cuda")
    status = torch.zeros((n + 2) ** 2, dtype=torch.int32, device="cuda")
    out = {"workload": "tgv2d_%dx%d_v17_cfl%.2g_N3" % (n, n, cfl)}
    for flux, name in ((1, "roe"), (2, "osher")):
        u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
        clk = torch.tensor([0.0, 0.0, 1e9, cfl, 0.0], dtype=torch.float64, device="cuda")
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def run(k):
            _lib.check(lib.gpr_iterate_n(
                ctypes.c_void_p(u.data_ptr()), pn, 2, dXa.ctypes.data_as(ctypes.c_void_p),
                bc.ctypes.data_as(ctypes.c_void_p), flux,
                ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
                ctypes.c_void_p(clk.data_ptr()), k, ctypes.c_void_p(scr.data_ptr()),
                ctypes.c_void_p(status.data_ptr()), CONTORTED_TOL, V, N, sp), "iterate_n")
        run(warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run(steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        kind = status.cpu().numpy() & 0xff
        r = {"steps": steps, "ms_per_step": ms / steps,
             "value": n * n * steps / (ms * 1e-3) / 1e6, "unit": UNIT,
             "finite": bool(torch.isfinite(u).all().item()),
             "newton_cells": int((kind == 1).sum())}
        if cpu:
            from oracle import Oracle
            from phd_gb300.order import for_order
            O = Oracle(N=N)
            G3 = for_order(N)
            u_np = u.detach().cpu().numpy().reshape(n, n, V).copy()
            t0 = time.perf_counter()
            dt = O.timestep(u_np, dX, cfl, 0.0, 1e9, 10, MP)
            ub = O.boundaries(u_np, nX, [1] * 4)
            ref = u_np.reshape(-1).copy()
            O.ader_stepper(ref, ub, nX, dt, dX, MP, flux=flux)
            O.renorm_distortion(ref, MP)
            cpu_s = time.perf_counter() - t0
            ud = u.detach().clone()
            ubt = torch.empty(ub.size, dtype=torch.float64, device="cuda")
            G3.boundaries(ud, ubt, nX, [1] * 4)
            G3.solvers.ader_stepper(ud, ubt, nX, dt, dX, False, flux, MP, None)
            G.solvers.renorm_distortion(ud, [MP])
            got = ud.cpu().numpy()
            r["max_rel_diff_vs_oracle"] = float(np.max(np.abs(got - ref) / (1.0 + np.abs(ref))))
            r["cpu_baseline"] = {"value": n * n / cpu_s / 1e6, "unit": UNIT,
                                 "cores": O.num_threads(), "kind": "port",
                                 "sample": "one step of the full %dx%d grid at N = 3, "
                                           "oracle/gpr_oracle.c" % (n, n)}
        out[name] = r
    return out


def shock_bubble_bench(torch, steps=10, warmup=3, nx=800, cpu_steps=2):
    """2D two-material ghost-fluid shock-bubble: 800 x 400 cells on [0, 2] x
    [0, 1], V = 15 (viscous, one level set), ideal gas gamma 1.4 (rho 1, p
    1) around a circular bubble of radius 0.2 at (0.6, 0.5) of gamma 1.67,
    rho 0.138, p 1; a Mach 1.22 shock from the left; cs = 1, mu = 1e-4;
    Rusanov flux, CFL 0.8, transmissive boundaries.  A step is one step of the
    reference's two-material iterator: ghost fill (re-distancing, interface
    Riemann states, extrapolation layers, for both materials) -> CFL over
    both masked grids -> masked ADER step of each material -> make_u ->
    renorm, device resident (gpr_iterate_multi).  The ghost fill is also
    timed alone; the oracle runs `cpu_steps` steps of the same grid on the
    host cores."""
    from phd_gb300 import ghost, problems
    from oracle import Oracle
    ny = nx // 2
    u0, MPs, tf, dX, bcs = problems.shock_bubble(nx=nx, ny=ny)
    nX = np.array([nx, ny], np.int32)
    ncell = nx * ny
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device=dev)
    it = ghost.MultiIterator(nX, dX, 0, MPs, 0.8, tf, device=dev)
    it.run(u, warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    it.run(u, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = it.clock.cpu().numpy()
    status = it.status.cpu().numpy().tolist()
    # the ghost fill alone, on the current state
    grids = torch.empty(2, ncell * 15, dtype=torch.float64, device=dev)
    masks = torch.empty(2, ncell, dtype=torch.bool, device=dev)
    uf = u.clone()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ghost.fill_ghost_cells(grids, masks, uf, nX, dX, float(clk[1]), MPs)
    torch.cuda.synchronize()
    f0.record(stream)
    for _ in range(3):
        ghost.fill_ghost_cells(grids, masks, uf, nX, dX, float(clk[1]), MPs)
    f1.record(stream)
    torch.cuda.synchronize()
    fill_ms = f0.elapsed_time(f1) / 3
    # the re-distancing alone (FP64 sweeps), on the current level set, and
    # its largest difference from the oracle's marcher there
    col = u.view(-1, 15)[:, 14].contiguous()
    dst = torch.zeros(4, dtype=torch.int32, device=dev)
    dd = ghost.distance(col, dX, nX, status=dst)
    torch.cuda.synchronize()
    redist_sweeps = int(dst[3].item())
    f0.record(stream)
    for _ in range(3):
        dd = ghost.distance(col, dX, nX)
    f1.record(stream)
    torch.cuda.synchronize()
    redist_ms = f0.elapsed_time(f1) / 3
    redist_diff = float(np.max(np.abs(
        dd.cpu().numpy() - Oracle(N=2, thermal=False, lset=1).distance(
            col.cpu().numpy(), dX, np.asarray(nX, np.int32)))))
    # end to end with host buffers: H2D of the state, one step, D2H, per step
    host = torch.empty(ncell * 15, dtype=torch.float64, pin_memory=True)
    host.copy_(u.cpu())
    ue = torch.empty_like(u)
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(steps):
        ue.copy_(host, non_blocking=True)
        it.run(ue, 1)
        host.copy_(ue, non_blocking=True)
    g1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = g0.elapsed_time(g1)
    out = {"workload": "shock bubble %dx%d, V=15, two materials, mu=1e-4, CFL 0.8, Rusanov"
                       % (nx, ny),
           "steps": steps, "ms_per_step": ms / steps,
           "value": ncell * steps / (ms * 1e-3) / 1e6, "unit": UNIT,
           "fill_ms": fill_ms, "fill_share": fill_ms / (ms / steps),
           "redistance_ms": redist_ms, "redistance_share": redist_ms / (ms / steps),
           "redistance_sweeps": redist_sweeps,
           "redistance_us_per_sweep": 1e3 * redist_ms / max(redist_sweeps, 1),
           "redistance_max_abs_diff_vs_oracle": redist_diff,
           "e2e": {"value": ncell * steps / (e2e_ms * 1e-3) / 1e6, "unit": UNIT,
                   "h2d_bytes_per_step": ncell * 15 * 8, "d2h_bytes_per_step": ncell * 15 * 8},
           "sim_time": float(clk[0]), "sim_steps": int(clk[4]), "fill_status": status}
    # one step of the device loop and one oracle step (the reference's loop
    # body with the ghost fill, solvers/iterator.cpp:109-151) from the same
    # state and clock: the state the steps above left
    clk = it.clock.cpu().numpy()
    O = Oracle(N=2, thermal=False, lset=1)
    uc = ue.cpu().numpy().reshape(nx, ny, 15).copy()
    O.step_multi(uc, float(clk[1]), float(clk[0]), tf, int(clk[4]), MPs, dX, 0, cfl=0.8,
                 contorted_tol=CONTORTED_TOL)
    it.run(ue, 1)
    got = ue.cpu().numpy().reshape(nx, ny, 15)
    cell_err = np.max(np.abs(got - uc) / (1.0 + np.abs(uc)), axis=-1)
    out["max_rel_diff_vs_oracle"] = float(cell_err.max())
    out["cells_within_1e-10_of_oracle"] = float((cell_err <= 1e-10).mean())
    if cpu_steps:
        uc = u0.copy()
        t0 = time.perf_counter()
        dt, t = 0.0, 0.0
        for s in range(cpu_steps):
            dt = O.step_multi(uc, dt, t, tf, s, MPs, dX, 0)
            t += dt
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": ncell * cpu_steps / cpu_s / 1e6, "unit": UNIT,
                               "cores": O.num_threads(), "kind": "port",
                               "sample": "first %d steps of the %dx%d grid" % (cpu_steps, nx, ny)}
    return out


def profile_shock_bubble(nx, steps):
    """`steps` steps of the nx x nx/2 shock bubble (for ncu captures)."""
    import torch
    from phd_gb300 import ghost, problems
    u0, MPs, tf, dX, bcs = problems.shock_bubble(nx=nx, ny=nx // 2)
    u = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
    it = ghost.MultiIterator(np.array([nx, nx // 2], np.int32), dX, 0, MPs, 0.8, tf)
    it.run(u, steps)
    torch.cuda.synchronize()
    ghost.check_status(it.status)
    return 0


def adjoint_bench(torch, fd_check=True):
    """Differentiation form on the first Stokes problem (400 cells on
    [-1, 1], t_end = 1.0, CFL 0.8, checkpoints every 32 steps): misfit of
    v_y against the run at the true parameters (mu, cs, calpha) =
    (1e-2, 1, 1), gradient at (1.2e-2, 0.9, 1.1) with respect to the
    parameters (mu, cs, calpha, gamma) and the 400 x 17 initial state.  Times the forward pass and
    the backward pass (segment recompute + backward steps) with CUDA events,
    reports their ratio per step, and the largest relative error of the
    parameter gradient against central differences (h = 1e-6) of the same
    forward.  The same for 64 instances with parameters perturbed by up to
    10%, in one batched loop."""
    import phd_gb300 as G
    from phd_gb300.adjoint import Problem, solve
    from phd_gb300.params import material_params

    def make_par(th):  # th = (mu, cs, calpha, gamma)
        return material_params("sg", 1.0, cv=1.0, gamma=th[3], b0=th[1], calpha=th[2],
                               mu=th[0], Pr=0.75)

    nx, tf = 400, 1.0
    u0, _, _, dX, _ = G.problems.stokes(nx=nx, mu=1e-2, cs=1.0, calpha=1.0, tf=tf)
    dx = dX[0]
    theta = np.array([1.2e-2, 0.9, 1.1, 1.45])
    npar = theta.size
    out = {}
    for ninst in (1, 64):
        rng = np.random.default_rng(20261203)
        th = theta[None, :] * (1.0 + (0.1 * rng.uniform(-1, 1, (ninst, npar)) if ninst > 1
                                      else 0.0))
        u0p = np.tile(u0, (ninst, 1))
        Pt = Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf)
        uT = Pt.forward(torch.tensor(u0p, device="cuda"),
                        [make_par(np.array([1e-2, 1.0, 1.0, 1.4]))] * ninst)
        target = (uT[:, 3] / uT[:, 0]).clone()

        def loss(uN):
            return 0.5 * torch.sum((uN[:, 3] / uN[:, 0] - target) ** 2)

        prob = Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf)
        pars = [make_par(th[k]) for k in range(ninst)]
        # warm-up (builds, allocates the tapes)
        uN = prob.forward(torch.tensor(u0p, device="cuda"), pars).clone().requires_grad_(True)
        loss(uN).backward()
        prob.backward(uN.grad)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record()
        uN = prob.forward(torch.tensor(u0p, device="cuda"), pars)
        e[1].record()
        uN = uN.clone().requires_grad_(True)
        loss(uN).backward()
        ub0, fb = prob.backward(uN.grad)
        e[2].record()
        torch.cuda.synchronize()
        fwd, bwd = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
        nsteps = prob.nsteps
        # the plain forward (reference stopping rule 6e-6) for comparison
        plain = Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf,
                        dg_tol=6e-6, dg_it=50)
        plain.forward(torch.tensor(u0p, device="cuda"), pars)
        torch.cuda.synchronize()
        e[0].record()
        plain.forward(torch.tensor(u0p, device="cuda"), pars)
        e[1].record()
        torch.cuda.synchronize()
        fwd_plain = e[0].elapsed_time(e[1])
        # the same gradient with the forward keeping its segments' tapes (the
        # whole run fits in device memory): the backward recomputes nothing
        tp = Problem([nx] * ninst, [dx] * ninst, "transitive", make_par, cfl=0.8, tf=tf,
                     tape_budget_bytes=32 << 30)
        uN = tp.forward(torch.tensor(u0p, device="cuda"), pars).clone().requires_grad_(True)
        loss(uN).backward()
        tp.backward(uN.grad)
        torch.cuda.synchronize()
        e[0].record()
        uN = tp.forward(torch.tensor(u0p, device="cuda"), pars)
        e[1].record()
        uN = uN.clone().requires_grad_(True)
        loss(uN).backward()
        ub1, fb1 = tp.backward(uN.grad)
        e[2].record()
        torch.cuda.synchronize()
        fwd_t, bwd_t = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
        same = float(torch.max(torch.abs(fb1 - fb) / (1 + torch.abs(fb))).item())
        r = {"instances": ninst, "cells": nx * ninst, "steps": nsteps,
             "forward_ms_per_step": fwd / nsteps, "backward_ms_per_step": bwd / nsteps,
             "adjoint_over_forward": bwd / fwd,
             "plain_forward_ms_per_step": fwd_plain / plain.nsteps,
             "adjoint_over_plain_forward": (bwd / nsteps) / (fwd_plain / plain.nsteps),
             "checkpoint_every": prob.K,
             "taped_forward": {"forward_ms_per_step": fwd_t / tp.nsteps,
                               "backward_ms_per_step": bwd_t / tp.nsteps,
                               "recomputed_steps": tp.recomputed_steps,
                               "tape_gb": len(tp.seg_tapes) * tp.K * tp.tape_len * 8 / 1e9,
                               "adjoint_over_plain_forward": (bwd_t / tp.nsteps) /
                                                             (fwd_plain / plain.nsteps),
                               "field_gradient_rel_diff_vs_checkpointed": same},
             "cell_updates_per_s_forward": nx * ninst * nsteps / (fwd * 1e-3),
             "transposed_iterations_mean": prob.adj_iterations}
        if fd_check and ninst == 1:
            g = prob.theta_grad(fb, th)[0]
            errs = []
            for j in range(npar):
                h = 1e-6 * theta[j]
                Ls = []
                for s in (1, -1):
                    t2 = theta.copy()
                    t2[j] += s * h
                    P2 = Problem([nx], [dx], "transitive", make_par, cfl=0.8, tf=tf)
                    Ls.append(float(loss(P2.forward(torch.tensor(u0p, device="cuda"),
                                                    [make_par(t2)]))))
                fd = (Ls[0] - Ls[1]) / (2 * h)
                errs.append(abs(g[j] - fd) / abs(fd))
            r["grad_wrt_mu_cs_calpha_gamma"] = [float(x) for x in g]
            r["grad_rel_err_vs_fd_h1e-6"] = max(errs)
        out["stokes_%d" % ninst] = r
    return out


def batched_bench(torch, steps=10, plain_steps=2, count=512):
    """512 independent 1D shock tubes (cell counts ~U{128..2048}, random
    states and materials) advanced by the batched form (one launch per stage
    for all instances, the step captured in a CUDA graph), against looping the
    plain path (gpr_iterate, one instance at a time) over the same instances.
    Both count cell-updates actually performed."""
    import phd_gb300 as G
    from phd_gb300 import _lib
    from phd_gb300.batch import Batch
    lib = _lib.load()
    insts = [(u, MP, dX, bcs) for (u, MP, tf, dX, bcs) in G.problems.batched_shock_tubes(count)]
    B = Batch(insts, cfl=0.8, tf=0.2)
    for _ in range(3):  # warm-up
        B.step(1)
    g = B.capture(1)
    torch.cuda.synchronize()
    u0 = int(B.updates.item())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1)
    upd_b = int(B.updates.item()) - u0
    st = B.status.cpu().numpy()
    # plain path: one gpr_iterate call per instance and step
    V = 17
    bufs = []
    for (u, MP, dX, bc) in insts:
        nx = np.array([u.shape[0]], np.int32)
        ut = torch.tensor(u.reshape(-1), dtype=torch.float64, device="cuda")
        scr = torch.empty(lib.gpr_iterate_scratch_doubles(nx.ctypes.data_as(ctypes.c_void_p), 1, V),
                          dtype=torch.float64, device="cuda")
        clk = torch.tensor([0.0, 0.0, 0.2, 0.8, 0.0], dtype=torch.float64, device="cuda")
        dxa = np.array(dX, np.float64)
        bca = np.array([0, 0], np.int32)
        cp = MP.to_ctypes()
        bufs.append((nx, ut, scr, clk, dxa, bca, cp))
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def plain_step():
        for (nx, ut, scr, clk, dxa, bca, cp) in bufs:
            lib.gpr_iterate(ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 1,
                            dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p),
                            0, ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
                            ctypes.c_void_p(clk.data_ptr()), 1, ctypes.c_void_p(scr.data_ptr()),
                            None, float("inf"), V, sp)  # as the batched form: no reset
    for _ in range(3):
        plain_step()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(plain_steps):
        plain_step()
    e1.record()
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1)
    cells = int(B.nx.sum())
    vb = upd_b / (ms_b * 1e-3) / 1e6
    vp = cells * plain_steps / (ms_p * 1e-3) / 1e6
    # per-stage times at the current state: the autotuner's timings of the
    # shapes it keeps (CUDA events per launch), and the predictor status of
    # one step from that state for the Picard iteration count
    shapes = B.autotune()
    tm = np.array(B.tuning["candidate_ms"])
    u_before = B.u.cpu().numpy().copy()
    B.step(1)
    st2 = B.status.cpu().numpy()
    # that step of every running instance against one oracle step from the
    # same state and with the same dt (the Newton fallback where Picard fails)
    from oracle import Oracle
    O = Oracle()
    clk = B.clock.view(-1, 5).cpu().numpy()
    u_after = B.u.cpu().numpy()
    worst, ninst_checked = 0.0, 0
    errs, above = [], []
    boff = np.concatenate([[0], np.cumsum(B.nx + 2)]).astype(np.int64)
    for k, (u_, MP, dX, bc) in enumerate(insts):
        dtk = float(clk[k, 1])
        if dtk == 0.0:
            continue
        a, b = int(B.off[k]) * V, int(B.off[k + 1]) * V
        st_k = u_before[a:b].reshape(-1, V)
        nxk = np.array([st_k.shape[0]], np.int32)
        code = 1 if bc == "periodic" else 0
        ref = st_k.ravel().copy()
        _, sto = O.ader_stepper(ref, O.boundaries(st_k, nxk, [code, code]), nxk, dtk, dX, MP)
        O.renorm_distortion(ref, MP)
        e = float(np.max(np.abs(u_after[a:b] - ref) / (1.0 + np.abs(ref))))
        errs.append(e)
        worst = max(worst, e)
        ninst_checked += 1
        if e > 1e-10:
            # the device status of this instance: Picard count << 8 | kind
            sg = st2[boff[k]:boff[k + 1]]
            pic_g, pic_o = (sg & 0xff) == 0, sto > 0
            flips = int(np.sum(pic_g & pic_o & ((sg >> 8) != sto)))
            path = int(np.sum(pic_g != pic_o))
            above.append({"instance": k, "max_rel_diff": e, "cells": int(nxk[0]),
                          "picard_count_differs_in_cells": flips,
                          "picard_vs_newton_differs_in_cells": path})
    iters, kind = st2 >> 8, st2 & 0xff
    mean_it = float(iters[kind == 0].mean())
    bs3 = [32, 64, 128]
    nb = int((B.nx + 2).sum())
    nf = int((B.nx + 1).sum())
    stage = {
        "k_b_weno": (tm[[64, 128, 256, 512].index(shapes["weno_block"])],
                     OPS_1D["weno_per_cell"] * nb),
        "k_predictor_first+k_predictor_picard": (
            tm[4 + 3 * bs3.index(shapes["first_block"]) + bs3.index(shapes["picard_block"])],
            OPS_1D["predictor_per_cell_iter"] * nb * (mean_it - 0.5)),
        "k_faces1d" + ("_split" if shapes["faces_four_lanes"] else ""): (
            tm[13 + 3 * shapes["faces_four_lanes"] + bs3.index(shapes["faces_block"])],
            OPS_1D["face_point"] * nf * 2),
        "k_cells": (tm[19 + bs3.index(shapes["cells_block"])], OPS_1D["cells_per_cell"] * cells),
    }
    peak = None
    try:
        peak = fp64_peak_tflops(torch)
    except Exception:
        pass
    per = {}
    for k, (ms, fl) in stage.items():
        ach = fl / (ms * 1e-3) / 1e12
        per[k] = {"ms_per_launch": float(ms), "algorithmic_flops_per_launch": float(fl),
                  "achieved": ach, "frac": ach / peak if peak else None}
    dom = max(per, key=lambda k: per[k]["ms_per_launch"])
    roof = {"bound": "fp64", "kernel": dom, "unit": "TFLOP/s", "peak": peak,
            "peak_source": "measured: FP64 DFMA microbenchmark in bench.py on this GPU",
            "achieved": per[dom]["achieved"], "frac": per[dom]["frac"],
            "algorithmic_flops_per_launch": per[dom]["algorithmic_flops_per_launch"],
            "mean_picard_iterations": mean_it, "per_kernel": per, "traffic": None}
    return {"workload": "%d 1D shock tubes, nx ~ U{128..2048} (%d cells), random states and "
                        "materials (mu ~ logU[1e-4,1e-1], cs ~ U[0.5,5], gamma ~ U[1.2,1.67]), "
                        "own CFL-0.8 clocks" % (count, cells),
            "batched_value": vb, "plain_loop_value": vp, "unit": UNIT,
            "speedup": vb / vp, "batched_ms_per_step": ms_b / steps,
            "plain_loop_ms_per_step": ms_p / plain_steps,
            "newton_cells_last_step": int(((st & 0xff) == 1).sum()),
            "batched_steps": steps, "plain_steps": plain_steps,
            "autotuned_shapes": shapes, "roofline": roof,
            "max_rel_diff_vs_oracle": worst, "instances_checked_against_oracle": ninst_checked,
            "instances_within_1e-10": int(np.sum(np.array(errs) <= 1e-10)),
            # the reference's Picard stopping rule |dq| <= 6e-6 (1 + |q|) is
            # discontinuous in its input: a cell at the threshold that stops
            # one iteration earlier or later moves the step by ~1e-8
            "instances_above_1e-10": above}


def stage_times(lib, torch, u, MP, nX, dXa, bc, cfl, V, dev, sp, stream, reps=3):
    """Average device time of each stage of a step, CUDA events on the
    launching stream."""
    from phd_gb300 import _lib
    pn = nX.ctypes.data_as(ctypes.c_void_p)
    pd = dXa.ctypes.data_as(ctypes.c_void_p)
    pb = bc.ctypes.data_as(ctypes.c_void_p)
    cpar = MP.to_ctypes()
    pp = ctypes.cast(ctypes.pointer(cpar), ctypes.c_void_p)
    n0, n1 = int(nX[0]), int(nX[1])
    ncell = n0 * n1
    ncb = (n0 + 2) * (n1 + 2)
    uu = u.clone()
    ub = torch.empty((n0 + 4) * (n1 + 4) * V, dtype=torch.float64, device=dev)
    wh = torch.empty(ncb * 4 * V, dtype=torch.float64, device=dev)
    qh = torch.empty(ncb * 8 * V, dtype=torch.float64, device=dev)
    ws = torch.empty(max(lib.gpr_weno_scratch_doubles(pn, 2, V),
                         lib.gpr_fv_scratch_doubles(pn, 2, V)), dtype=torch.float64, device=dev)
    dtd = torch.empty(1, dtype=torch.float64, device=dev)
    tsc = torch.empty(1, dtype=torch.float64, device=dev)
    st = torch.zeros(ncb, dtype=torch.int32, device=dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    names = ["cfl", "boundaries", "weno", "predictor", "fv", "renorm"]
    acc = {k: 0.0 for k in names}
    acc["faces"] = 0.0
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
    fe0, fe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for r in range(reps + 1):
        ev[0].record(stream)
        _lib.check(lib.gpr_timestep(P(uu), ncell, pd, 2, cfl, 0.0, 1e9, 10, pp, P(dtd), P(tsc),
                                    V, sp), "timestep")
        ev[1].record(stream)
        dt = float(dtd.item())
        ev[1].record(stream)
        _lib.check(lib.gpr_boundaries(P(uu), P(ub), pn, 2, pb, V, sp), "bc")
        ev[2].record(stream)
        _lib.check(lib.gpr_weno_launcher(P(wh), P(ub), pn, 2, P(ws), V, sp), "weno")
        ev[3].record(stream)
        _lib.check(lib.gpr_predictor(P(qh), P(wh), dt, pd, 2, pn, 0, pp, None, P(st), V, sp),
                   "pred")
        ev[4].record(stream)
        _lib.check(lib.gpr_fv_launcher(P(uu), P(qh), pn, dt, pd, 2, 1, 1, 0, pp, None, P(ws),
                                       V, sp), "fv")
        ev[5].record(stream)
        _lib.check(lib.gpr_renorm_distortion(P(uu), ncell, pp, V, sp), "renorm")
        ev[6].record(stream)
        torch.cuda.synchronize()
        if r == 0:
            continue
        for i, k in enumerate(names):
            if k == "cfl":
                continue
            acc[k] += ev[i].elapsed_time(ev[i + 1]) / reps

    # the CFL stage alone (its events straddle a host read above)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        lib.gpr_timestep(P(uu), ncell, pd, 2, cfl, 0.0, 1e9, 10, pp, P(dtd), P(tsc), V, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    acc["cfl"] = e0.elapsed_time(e1) / reps
    # the two parts of the fv stage alone: the face terms (four in-place
    # k_faces2d passes) and the volume term (k_cells)
    fe0.record(stream)
    for _ in range(reps):
        _lib.check(lib.gpr_fv_interfs(P(uu), P(qh), pn, dt, pd, 2, 1, 0, pp, None, P(ws), V,
                                      sp), "faces")
    fe1.record(stream)
    torch.cuda.synchronize()
    acc["faces"] = fe0.elapsed_time(fe1) / reps
    fe0.record(stream)
    for _ in range(reps):
        _lib.check(lib.gpr_fv_centers(P(uu), P(qh), pn, dt, pd, 2, 1, 1, pp, None, V, sp),
                   "centers")
    fe1.record(stream)
    torch.cuda.synchronize()
    acc["centers"] = fe0.elapsed_time(fe1) / reps
    acc["_mean_picard_iterations_stage_run"] = float((st.cpu().numpy() >> 8).mean())
    return acc


def roofline(stage_ms, ncell, n, mean_iters, peak):
    """Roofline of the dominant kernel against the measured FP64 peak.
    Per-launch time: the stage's CUDA-event time divided by its launches."""
    ncb = (n + 2) ** 2
    nf = (n + 1) ** 2  # faces per direction
    # kernel: (time per launch ms, algorithmic flops per launch)
    kern = {
        # four in-place passes (x / y faces, even / odd), half the faces each
        "k_faces2d": (stage_ms["faces"] / 4, OPS["face_quadrature_point"] * 4 * nf / 2),
        # the first iteration runs at one thread per spatial node
        # (k_predictor_first): half the per-iteration work
        "k_predictor_picard": (stage_ms["predictor"],
                               OPS["predictor_per_cell_iter"] * ncb * (mean_iters - 0.5)),
        "k_cells": (stage_ms["centers"], OPS["cells_per_cell"] * ncell),
        "k_cfl_max": (stage_ms["cfl"], OPS["cfl_per_cell"] * ncell),
    }
    per_step = {"k_faces2d": 4 * kern["k_faces2d"][0], "k_predictor_picard": kern["k_predictor_picard"][0],
                "k_cells": kern["k_cells"][0], "k_cfl_max": kern["k_cfl_max"][0]}
    dom = max(per_step, key=per_step.get)
    out = {"bound": "fp64", "kernel": dom, "unit": "TFLOP/s", "peak": peak,
           "peak_source": "measured: FP64 DFMA microbenchmark in bench.py on this GPU "
                          "(MEASURED_PEAKS.json has no FP64 figure)",
           "traffic": None, "per_kernel": {}}
    for k, (ms, fl) in kern.items():
        ach = fl / (ms * 1e-3) / 1e12
        out["per_kernel"][k] = {"ms_per_launch": ms, "algorithmic_flops_per_launch": fl,
                                "achieved": ach, "frac": ach / peak if peak else None}
    d = out["per_kernel"][dom]
    out.update(achieved=d["achieved"], frac=d["frac"],
               algorithmic_flops_per_launch=d["algorithmic_flops_per_launch"])
    if dom in TRAFFIC:
        out["traffic"] = TRAFFIC[dom]
        out["traffic_unit"] = "bytes per launch"
        out["traffic_source"] = ("from an earlier ncu capture of %s on the TGV 512^2 step "
                                 "(dram__bytes_read.sum + dram__bytes_write.sum), not "
                                 "measured in this run" % dom)
    return out


def profile_adjoint(ninst, steps):
    """Forward and backward of `steps` steps of the Stokes problem (400 cells
    per instance), twice (the second run is the one to capture)."""
    import torch
    import phd_gb300 as G
    from phd_gb300.adjoint import Problem
    from phd_gb300.params import material_params

    def make_par(th):
        return material_params("sg", 1.0, cv=1.0, gamma=1.4, b0=th[1], calpha=th[2], mu=th[0],
                               Pr=0.75)

    u0, _, _, dX, _ = G.problems.stokes(nx=400, tf=1.0)
    u0p = np.tile(u0, (ninst, 1))
    prob = Problem([400] * ninst, [dX[0]] * ninst, "transitive", make_par, cfl=0.8, tf=1.0)
    pars = [make_par(np.array([1.2e-2, 0.9, 1.1]))] * ninst
    for _ in range(2):
        uN = prob.forward(torch.tensor(u0p, device="cuda"), pars, max_steps=steps)
        prob.backward(torch.ones_like(uN))
    torch.cuda.synchronize()
    return 0


def profile_batched(steps, shapes):
    """`steps` steps of the 512 batched shock tubes (for ncu captures), with
    the given launch shapes (default shapes if empty), no autotuning."""
    import torch
    import phd_gb300 as G
    from phd_gb300.batch import Batch
    insts = [(u, MP, dX, bcs) for (u, MP, tf, dX, bcs) in G.problems.batched_shock_tubes(512)]
    B = Batch(insts, cfl=0.8, tf=0.2, autotune=False)
    if shapes:
        B.set_shapes([int(x) for x in shapes.split(",")])
    B.step(steps)
    torch.cuda.synchronize()
    return 0


def profile_shock_tube(flux, steps, split=False):
    """`steps` steps of the 200-cell shock tube through gpr_iterate, or
    gpr_iterate_split with the half step (for ncu captures)."""
    import torch
    import phd_gb300 as G
    from phd_gb300 import _lib
    lib = _lib.load()
    u0, MP, tf, dX, bcs = G.problems.shock_tube(nx=200)
    nx = np.array([200], np.int32)
    dxa = np.array(dX, np.float64)
    bca = np.array([0, 0], np.int32)
    cp = MP.to_ctypes()
    scr = torch.empty(lib.gpr_iterate_scratch_doubles(nx.ctypes.data_as(ctypes.c_void_p), 1, 17),
                      dtype=torch.float64, device="cuda")
    ut = torch.tensor(u0.reshape(-1), dtype=torch.float64, device="cuda")
    clk = torch.tensor([0.0, 0.0, tf, 0.8, 0.0], dtype=torch.float64, device="cuda")
    if split:
        rc = lib.gpr_iterate_split(
            ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 1,
            dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p), flux, 1,
            ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
            ctypes.c_void_p(clk.data_ptr()), steps, ctypes.c_void_p(scr.data_ptr()),
            CONTORTED_TOL, 17, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    else:
        rc = lib.gpr_iterate(
            ctypes.c_void_p(ut.data_ptr()), nx.ctypes.data_as(ctypes.c_void_p), 1,
            dxa.ctypes.data_as(ctypes.c_void_p), bca.ctypes.data_as(ctypes.c_void_p), flux,
            ctypes.cast(ctypes.pointer(cp), ctypes.c_void_p), None,
            ctypes.c_void_p(clk.data_ptr()), steps, ctypes.c_void_p(scr.data_ptr()), None,
            CONTORTED_TOL, 17, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "iterate")
    torch.cuda.synchronize()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.fp64_issue:
        import torch
        return fp64_issue_probe(torch)
    if args.profile_batched:
        return profile_batched(args.profile_steps or 3, args.shapes)
    if args.profile_n3:
        import torch
        return tgv_n3_bench(torch, n=args.profile_n3, profile_steps=args.profile_steps or 3)
    if args.profile_adjoint:
        return profile_adjoint(args.profile_adjoint, args.profile_steps or 32)
    if args.profile_shock_tube >= 0:
        return profile_shock_tube(args.profile_shock_tube, args.profile_steps or 10, args.split)
    if args.profile_shock_bubble:
        return profile_shock_bubble(args.profile_shock_bubble, args.profile_steps or 4)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
