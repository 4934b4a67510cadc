"""phd_gb300 - GB300-native (sm_103a, FP64) GPR ADER-WENO time step.

A drop-in for the hot path of the reference's pybind11 module `GPRpy`
(haranjackson/phd, code/cpp/bindings/bindings.cpp): the same names and
argument orders, operating in place on torch CUDA tensors, backed by the
hand-written CUDA kernels in phd_gb300/csrc through the C ABI declared in
include/gpr_gb300.h.

    import phd_gb300 as GPRpy
    GPRpy.boundaries(u, ub, nX, bcs)
    GPRpy.solvers.ader_stepper(u, ub, nX, dt, dX, False, 0, MP, mask)
"""
from types import SimpleNamespace

from . import api
from . import ghost as _multi
from ._lib import build, load
from .params import Par, material_params, Cvec
from . import problems

__all__ = ["boundaries", "extend_mask", "options", "classes", "solvers", "system", "multi",
           "build", "load", "Par", "material_params", "Cvec", "problems"]

boundaries = api.boundaries
extend_mask = api.extend_mask

options = SimpleNamespace(N=lambda: 2, NV=lambda: 17, VISCOUS=lambda: True,
                          THERMAL=lambda: True, MULTI=lambda: False, LSET=lambda: 0)

# The reference binds both Params and its subclass Par (system/objects.h:22-60);
# a Par carries every Params field, so one class serves both names.
classes = SimpleNamespace(Par=Par, Params=Par)

system = SimpleNamespace(flux=api.flux, source=api.source, Bdot=api.Bdot,
                         max_abs_eigs=api.max_abs_eigs, system_matrix=api.system_matrix,
                         thermo_acoustic_tensor=api.thermo_acoustic_tensor,
                         multi=SimpleNamespace(left_star_state=_multi.left_star_state,
                                               distance=_multi.distance))

multi = SimpleNamespace(renormalize_levelsets=_multi.renormalize_levelsets,
                        finite_difference=_multi.finite_difference,
                        find_interface_cells=_multi.find_interface_cells,
                        fill_boundary_cells=_multi.fill_boundary_cells,
                        fill_neighbor_cells=_multi.fill_neighbor_cells,
                        fill_ghost_cells=_multi.fill_ghost_cells,
                        material_indicator=_multi.material_indicator)


def _two_materials(u, MPs):
    return isinstance(MPs, (list, tuple)) and len(MPs) == 2 and (
        u.shape[-1] == _multi.V if u.dim() > 1 else api._NVAR.get("V") == _multi.V)


def _iterator(u, tf, nX, dX, CFL, boundaryTypes, SPLIT, HALF_STEP, STIFF, FLUX, MPs,
              contorted_tol=1.0, max_steps=None):
    """solvers.iterator: the two-material ghost-fluid loop for V = 15 and two
    materials, else the one-material loop; both take the reference's SPLIT,
    HALF_STEP, STIFF and FLUX."""
    if _two_materials(u, MPs):
        return _multi.iterate(u, tf, nX, dX, CFL, boundaryTypes, MPs, max_steps=max_steps,
                              contorted_tol=contorted_tol, SPLIT=SPLIT, HALF_STEP=HALF_STEP,
                              STIFF=STIFF, FLUX=FLUX)
    from .driver import iterate
    return iterate(u, tf, nX, dX, CFL, boundaryTypes, SPLIT, HALF_STEP, STIFF, FLUX, MPs,
                   max_steps=max_steps, contorted_tol=contorted_tol)


def _renorm_distortion(u, MPs):
    if _two_materials(u, MPs):
        return _multi.renorm_distortion(u, MPs)
    return api.renorm_distortion(u, MPs)


solvers = SimpleNamespace(
    weno=SimpleNamespace(weno_launcher=api.weno_launcher,
                         oscillation_indicator=api.oscillation_indicator),
    common=SimpleNamespace(scaled_nodes=api.scaled_nodes, scaled_weights=api.scaled_weights,
                           end_values=api.end_values, derivative_values=api.derivative_values),
    dg=SimpleNamespace(predictor=api.predictor),
    fv=SimpleNamespace(fv_launcher=api.fv_launcher, centers1=api.centers1,
                       centers2=api.centers2, interfs1=api.interfs1, interfs2=api.interfs2,
                       D_RUS=api.D_RUS, D_ROE=api.D_ROE, D_OSH=api.D_OSH, Bint=api.Bint),
    split=SimpleNamespace(ode_launcher=api.ode_launcher, midstepper=api.midstepper),
    ader_stepper=api.ader_stepper,
    ader_stepper_para=api.ader_stepper_para,
    split_stepper=api.split_stepper,
    split_stepper_para=api.split_stepper_para,
    timestep=api.timestep,
    renorm_distortion=_renorm_distortion,
    contorted=api.contorted,
    reset_contorted=api.reset_contorted,
    make_u=_multi.make_u,
    extended_dimensions=api.extended_dimensions,
    iterator=_iterator,
)
