"""Build and load the CUDA library (libgpr_gb300.so, C ABI in
include/gpr_gb300.h).

The library is compiled in-tree with nvcc for sm_103a only.  There is no
fallback: if the library cannot be loaded, every entry point raises.
"""
import ctypes
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libgpr_gb300.so")
SOURCES = ["gpr_capi.cu", "gpr_adjoint.cu", "gpr_multi.cu", "gpr_order.cu"]
HEADERS = ["gpr_device.cuh", "gpr_kernels.cuh", "gpr_consts.cuh", "gpr_ode.cuh", "gpr_host.cuh",
           "gpr_osher.cuh", "gpr_ops.cuh", "gpr_ops15.h", "gpr_multi.cuh",
           "gpr_adjoint.cuh", "gpr_order.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

_lock = threading.Lock()
_lib = None


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "gpr_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile the CUDA sources into phd_gb300/libgpr_gb300.so."""
    if not force and not _stale():
        return LIB
    nvcc = os.environ.get("NVCC", "nvcc")
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(HERE, "_build", os.path.splitext(src)[0] + ".o")
        os.makedirs(os.path.dirname(obj), exist_ok=True)
        cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                               "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                       stderr=subprocess.STDOUT), cmd))
        objs.append(obj)
    for p, cmd in procs:
        out, _ = p.communicate()
        if p.returncode:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode()[-6000:]))
        if verbose:
            print(out.decode())
    tmp = LIB + ".tmp"
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB)
    return LIB


_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double
_I64 = ctypes.c_int64

SIGNATURES = {
    "gpr_version": (_I, []),
    "gpr_scheme_constants": (_I, [_P, _I]),
    "gpr_supported_nvars": (_I, [_P, _I]),
    "gpr_boundaries": (_I, [_P, _P, _P, _I, _P, _I, _P]),
    "gpr_extend_mask": (_I, [_P, _P, _P, _I, _P]),
    "gpr_weno_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_weno_launcher": (_I, [_P, _P, _P, _I, _P, _I, _P]),
    "gpr_predictor": (_I, [_P, _P, _D, _P, _I, _P, _I, _P, _P, _P, _I, _P]),
    "gpr_fv_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_fv_launcher": (_I, [_P, _P, _P, _D, _P, _I, _I, _I, _I, _P, _P, _P, _I, _P]),
    "gpr_fv_face_fluxes": (_I, [_P, _P, _D, _P, _I, _I, _I, _P, _P, _P, _I, _P]),
    "gpr_fv_centers": (_I, [_P, _P, _P, _D, _P, _I, _I, _I, _P, _P, _I, _P]),
    "gpr_fv_interfs": (_I, [_P, _P, _P, _D, _P, _I, _I, _I, _P, _P, _P, _I, _P]),
    "gpr_timestep_scratch_doubles": (_I, [_I64]),
    "gpr_timestep": (_I, [_P, _I64, _P, _I, _D, _D, _D, _I, _P, _P, _P, _I, _P]),
    "gpr_renorm_distortion": (_I, [_P, _I64, _P, _I, _P]),
    "gpr_ode_launcher": (_I, [_P, _I64, _D, _P, _I, _P]),
    "gpr_ader_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_ader_stepper": (_I, [_P, _P, _P, _I, _D, _P, _I, _I, _P, _P, _P, _P, _I, _P]),
    "gpr_iterate_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_iterate": (_I, [_P, _P, _I, _P, _P, _I, _P, _P, _P, _I, _P, _P, _D, _I, _P]),
    "gpr_reset_contorted": (_I, [_P, _I64, _D, _P, _I, _P, _I, _P]),
    "gpr_contorted": (_I, [_P, _I64, _D, _P, _I, _P]),
    "gpr_ader_stepper_1d_noalloc": (_I, [_P, _P, ctypes.c_int32, _D, _D, _I, _I, _P, _P, _P,
                                         _I, _P]),
    "gpr_midstepper": (_I, [_P, _D, _P, _I, _P, _P, _P, _I, _P]),
    "gpr_split_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_split_stepper": (_I, [_P, _P, _P, _I, _D, _P, _I, _I, _P, _P, _P, _I, _P]),
    "gpr_iterate_split": (_I, [_P, _P, _I, _P, _P, _I, _I, _P, _P, _P, _I, _P, _D, _I, _P]),
    "gpr_batch_scratch_doubles": (_L, [_I, _P, _I]),
    "gpr_batch_init": (_I, [_P, _I, _P, _P, _P, _P, _D, _D, _P, _I, _P]),
    "gpr_batch_iterate": (_I, [_P, _P, _I, _P, _I, _P, _P, _P, _I, _P]),
    "gpr_batch_autotune": (_I, [_P, _P, _I, _P, _P, _P, _P, _I, _P]),
    "gpr_order_supported": (_I, [_I, _I, _I]),
    "gpr_scheme_constants_n": (_I, [_P, _I, _I]),
    "gpr_boundaries_n": (_I, [_P, _P, _P, _I, _P, _I, _I, _P]),
    "gpr_weno_scratch_doubles_n": (_L, [_P, _I, _I, _I]),
    "gpr_weno_launcher_n": (_I, [_P, _P, _P, _I, _P, _I, _I, _P]),
    "gpr_predictor_n": (_I, [_P, _P, _D, _P, _I, _P, _I, _P, _P, _P, _I, _I, _P]),
    "gpr_fv_scratch_doubles_n": (_L, [_P, _I, _I, _I]),
    "gpr_fv_launcher_n": (_I, [_P, _P, _P, _D, _P, _I, _I, _P, _P, _P, _I, _I, _P]),
    "gpr_ader_scratch_doubles_n": (_L, [_P, _I, _I, _I]),
    "gpr_ader_stepper_n": (_I, [_P, _P, _P, _I, _D, _P, _I, _I, _P, _P, _P, _P, _I, _I, _P]),
    "gpr_iterate_scratch_doubles_n": (_L, [_P, _I, _I, _I]),
    "gpr_iterate_n": (_I, [_P, _P, _I, _P, _P, _I, _P, _P, _P, _I, _P, _P, _D, _I, _I, _P]),
    "gpr_batch_get_shapes": (_I, [_P, _P]),
    "gpr_batch_set_shapes": (_I, [_P, _P]),
    "gpr_adj_num_fields": (_I, []),
    "gpr_adj_supported": (_I, [_I, _P, _P, _I]),
    "gpr_adj_tape_doubles": (_L, [_I, _P, _I]),
    "gpr_adj_scratch_doubles": (_L, [_I, _P, _I]),
    "gpr_adj_forward_step": (_I, [_P, _P, _I, _P, _P, _P, _P, _I, _D, _I, _P, _I, _P]),
    "gpr_adj_backward_step": (_I, [_P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _I, _P]),
    "gpr_adj_point_jacobians": (_I, [_P, _I64, _P, _P, _P, _P, _I, _P]),
    "gpr_adj_point_vjp": (_I, [_P, _I64, _P, _P, _P, _P, _P, _P, _I, _P]),
    "gpr_distance_scratch_doubles": (_L, [_P, _I]),
    "gpr_distance": (_I, [_P, _P, _P, _I, _P, _P, _P, _P]),
    "gpr_finite_difference": (_I, [_P, _P, _P, _I, _P, _P]),
    "gpr_find_interface_cells": (_I, [_P, _P, _P, _I, _P]),
    "gpr_left_star_state": (_I, [_P, _P, _P, _P, _I64, _I, _D, _P, _P, _I, _P]),
    "gpr_fill_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_fill_boundary_cells": (_I, [_P, _P, _I, _P, _P, _P, _P, _I, _D, _P, _I, _P, _P, _I,
                                     _P]),
    "gpr_fill_neighbor_cells": (_I, [_P, _P, _P, _P, _P, _I, _P, _P, _I, _P]),
    "gpr_fill_ghost_cells": (_I, [_P, _P, _P, _P, _I, _P, _D, _P, _I, _P, _P, _I, _P]),
    "gpr_make_u": (_I, [_P, _P, _P, _I64, _P, _I, _I, _P]),
    "gpr_renorm_multi": (_I, [_P, _I64, _P, _I, _I, _P]),
    "gpr_timestep_multi": (_I, [_P, _P, _I64, _P, _I, _D, _D, _D, _I, _P, _I, _P, _P, _I, _P]),
    "gpr_iterate_multi_scratch_doubles": (_L, [_P, _I, _I]),
    "gpr_iterate_multi": (_I, [_P, _P, _I, _P, _P, _I, _P, _I, _P, _I, _P, _P, _D, _I, _P]),
    "gpr_iterate_multi_scheme": (_I, [_P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _I, _P, _I, _P,
                                      _P, _D, _I, _P]),
    "gpr_flux": (_I, [_P, _P, _I64, _I, _P, _I, _P]),
    "gpr_source": (_I, [_P, _P, _I64, _P, _I, _P]),
    "gpr_Bdot": (_I, [_P, _P, _P, _I64, _I, _P, _I, _P]),
    "gpr_max_abs_eigs": (_I, [_P, _P, _I64, _I, _P, _I, _P]),
    "gpr_system_matrix": (_I, [_P, _P, _I64, _I, _P, _I, _P]),
    "gpr_thermo_acoustic_tensor": (_I, [_P, _P, _I64, _I, _P, _I, _P]),
    "gpr_interface_terms": (_I, [_P, _P, _P, _P, _I64, _I, _I, _P, _I, _P]),
}


def load():
    """Load the library (building it first if needed) and bind every
    declared entry point."""
    global _lib
    with _lock:
        if _lib is None:
            if _stale():
                build()
            lib = ctypes.CDLL(LIB)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
    return _lib


ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "unsupported variant",
          -4: "size beyond the fixed maximum"}


def check(rc, what):
    if rc < 0:
        raise RuntimeError("%s failed: %s (%d)" % (what, ERRORS.get(rc, "error"), rc))
    return rc
