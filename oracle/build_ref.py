"""Recipe: compile the reference GPR solver (haranjackson/phd, code/cpp) into a
test-only Python module under oracle/_ref/.

This is test infrastructure.  It reads the reference sources from the
reference checkout (read-only; its root is taken from --ref ROOT, else the
environment variable GPR_REFERENCE_ROOT, else /root/reference), copies them
to a scratch directory under /tmp, applies the minimum patch needed for them
to compile and to select a model variant, and links them with oracle/ref_bindings.cpp (own code) into
oracle/_ref/GPRref_<variant>.so.  Reference sources are never copied into the
repository; oracle/_ref/ is git-ignored.

Patches applied to the scratch copy:
  * src/options.h: VISCOUS/THERMAL/MULTI/LSET/N/DG_TOL/DG_IT per variant
    (options.h:5-33 are compile-time constants in the reference);
  * src/solvers/fv/fluxes.cpp: the second, identical definition of D_RUS
    (fluxes.cpp:77-86 duplicates :66-75) is removed, since a duplicate
    definition is a hard compile error.

The build uses g++ directly (no cmake), the vendored Eigen 3.3.4 and
skfmm sources, and the pip pybind11 headers.  It only runs where the
reference checkout exists (the x86 development container); a GPU host never
needs it.

Usage:  python oracle/build_ref.py [--ref ROOT] [variant ...]     (default: v17)
"""
import os
import re
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

REF_ROOT = os.environ.get("GPR_REFERENCE_ROOT", "/root/reference")
if "--ref" in sys.argv:  # python oracle/build_ref.py --ref ROOT [variant ...]
    _k = sys.argv.index("--ref")
    REF_ROOT = sys.argv[_k + 1]
    del sys.argv[_k:_k + 2]
REF = os.path.join(REF_ROOT, "code", "cpp")
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

VARIANTS = {
    # V = 5 + 9 VISCOUS + 3 THERMAL + MULTI + LSET   (options.h:34)
    "v17": dict(VISCOUS="true", THERMAL="true", MULTI="false", LSET=0, N=2),
    "v17n3": dict(VISCOUS="true", THERMAL="true", MULTI="false", LSET=0, N=3),
    "v17tight": dict(VISCOUS="true", THERMAL="true", MULTI="false", LSET=0, N=2,
                     DG_TOL="1e-13", DG_IT=400),
    "v14": dict(VISCOUS="true", THERMAL="false", MULTI="false", LSET=0, N=2),
    "v15": dict(VISCOUS="true", THERMAL="false", MULTI="false", LSET=1, N=2),
    "v18": dict(VISCOUS="true", THERMAL="true", MULTI="false", LSET=1, N=2),
}

SOURCES = """
include/skfmm/base_marcher.cpp include/skfmm/distance_marcher.cpp include/skfmm/heap.cpp
src/etc/debug.cpp src/etc/globals.cpp src/etc/grid.cpp
src/multi/fill.cpp src/multi/functions.cpp src/multi/pfmm.cpp
src/scipy/legendre.cpp src/scipy/lgmres.cpp src/scipy/newton_krylov.cpp src/scipy/poly.cpp
src/solvers/iterator.cpp src/solvers/steppers.cpp src/solvers/utils.cpp
src/solvers/fv/fluxes.cpp src/solvers/fv/fv.cpp
src/solvers/split/homogeneous.cpp src/solvers/split/ode.cpp src/solvers/split/numeric.cpp
src/solvers/split/rk.cpp
src/solvers/dg/dg.cpp src/solvers/dg/dg1.cpp src/solvers/dg/dg2.cpp
src/solvers/dg/dg_matrices.cpp src/solvers/dg/initial_guess.cpp
src/solvers/poly/basis.cpp src/solvers/poly/evaluations.cpp
src/solvers/weno/weno.cpp src/solvers/weno/weno_matrices.cpp
src/system/eig.cpp src/system/equations.cpp src/system/jacobians.cpp
src/system/energy/derivatives.cpp src/system/energy/eos.cpp src/system/energy/mg.cpp
src/system/energy/multi.cpp
src/system/functions/matrices.cpp src/system/functions/vectors.cpp
src/system/multi/conditions.cpp src/system/multi/eigenvecs.cpp src/system/multi/riemann.cpp
src/system/multi/rotations.cpp
src/system/relaxation/analytic.cpp src/system/relaxation/numerical.cpp
src/system/variables/sources.cpp src/system/variables/state.cpp
src/system/waves/shear.cpp src/system/waves/speeds.cpp
""".split()


def _patch_options(path, opts):
    txt = open(path).read()
    for key in ("VISCOUS", "THERMAL", "MULTI"):
        if key in opts:
            txt, n = re.subn(r"const bool %s = \w+;" % key,
                             "const bool %s = %s;" % (key, opts[key]), txt)
            assert n == 1, key
    for key in ("LSET", "N", "DG_IT"):
        if key in opts:
            txt, n = re.subn(r"const int %s = [^;]+;" % key,
                             "const int %s = %s;" % (key, opts[key]), txt)
            assert n == 1, key
    if "DG_TOL" in opts:
        txt, n = re.subn(r"const double DG_TOL = [^;]+;",
                         "const double DG_TOL = %s;" % opts["DG_TOL"], txt)
        assert n == 1
    open(path, "w").write(txt)


def _patch_fluxes(path):
    txt = open(path).read()
    key = "VecV D_RUS(VecVr qL, VecVr qR, int d, Par &MP) {"
    assert txt.count(key) == 2, "expected the duplicated D_RUS definition"
    first = txt.find(key)
    second = txt.find(key, first + 1)
    body1 = txt[first:second].strip()
    body2 = txt[second:].strip()
    assert body1 == body2, "the two D_RUS definitions differ"
    open(path, "w").write(txt[:second])


def build(variant):
    opts = VARIANTS[variant]
    scratch = "/tmp/phd_ref_build/%s" % variant
    if os.path.isdir(scratch):
        shutil.rmtree(scratch)
    os.makedirs(scratch)
    shutil.copytree(os.path.join(REF, "src"), os.path.join(scratch, "src"))
    os.makedirs(os.path.join(scratch, "include"))
    for sub in ("eigen3", "skfmm"):
        shutil.copytree(os.path.join(REF, "include", sub),
                        os.path.join(scratch, "include", sub))
    shim = os.path.join(scratch, "shim")
    os.makedirs(shim)
    os.symlink(os.path.join(scratch, "include", "eigen3"),
               os.path.join(shim, "Eigen"))
    _patch_options(os.path.join(scratch, "src", "options.h"), opts)
    _patch_fluxes(os.path.join(scratch, "src", "solvers", "fv", "fluxes.cpp"))

    import pybind11
    inc = ["-I" + os.path.join(scratch, "src"),
           "-I" + os.path.join(scratch, "include"),
           "-I" + shim, "-I" + pybind11.get_include(),
           "-I" + sysconfig.get_paths()["include"]]
    flags = ["-std=c++17", "-O3", "-march=native", "-fopenmp", "-fPIC", "-w"]
    objdir = os.path.join(scratch, "obj")
    os.makedirs(objdir)
    srcs = [os.path.join(scratch, s) for s in SOURCES]
    srcs.append(os.path.join(HERE, "ref_bindings.cpp"))
    modname = "GPRref_%s" % variant

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = ["g++"] + flags + inc + ["-DMODNAME=%s" % modname, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("compile failed: %s\n%s" % (src, r.stderr[-4000:]))
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    os.makedirs(OUT, exist_ok=True)
    target = os.path.join(OUT, modname + sysconfig.get_config_var("EXT_SUFFIX"))
    cmd = ["g++", "-shared", "-fopenmp", "-o", target] + objs
    subprocess.run(cmd, check=True)
    return target


def main(argv):
    if not os.path.isdir(REF):
        print("reference sources not present; nothing to build")
        return 0
    for v in (argv or ["v17"]):
        print("built", build(v))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
