// Test-only pybind11 module over the reference GPR solver (haranjackson/phd,
// code/cpp/src).  It is compiled by oracle/build_ref.py against a patched
// scratch copy of the reference sources and is used ONLY to pin the CPU
// oracle (oracle/gpr_oracle.c) and to generate the golden fixtures under
// tests/golden/.  Nothing in the product imports it.
//
// It differs from the reference's own bindings (code/cpp/bindings/bindings.cpp)
// in three ways:
//   * it exports solvers.dg.predictor, which the reference declares
//     (solvers/dg/dg.h:7) but does not bind (bindings.cpp:79);
//   * multi-material containers are replaced by single-material wrappers
//     (timestep_single, renorm_single) so plain numpy arrays can be passed;
//   * small-matrix results are returned as numpy arrays;
//   * the ghost-fluid routines (multi/) take and return plain arrays and
//     lists of arrays.
#include "etc/types.h"
#include "options.h"

#include "pybind11/eigen.h"
#include "pybind11/pybind11.h"
#include "pybind11/stl.h"

#include "etc/globals.h"
#include "etc/grid.h"
#include "multi/fill.h"
#include "multi/functions.h"
#include "multi/pfmm.h"
#include "solvers/dg/dg.h"
#include "solvers/fv/fluxes.h"
#include "solvers/fv/fv.h"
#include "solvers/iterator.h"
#include "solvers/split/homogeneous.h"
#include "solvers/split/ode.h"
#include "solvers/steppers.h"
#include "solvers/utils.h"
#include "solvers/weno/weno.h"
#include "system/eig.h"
#include "system/multi/riemann.h"
#include "system/equations.h"
#include "system/jacobians.h"
#include "system/relaxation/analytic.h"
#include "system/variables/state.h"

#ifndef MODNAME
#define MODNAME GPRref
#endif

namespace py = pybind11;

static double timestep_single(Vecr u, Vecr dX, double CFL, double t, double tf,
                              int count, Par &MP) {
  std::vector<Vec> grids(1);
  grids[0] = u;
  std::vector<bVec> masks(1);
  masks[0] = bVec::Ones(u.size() / V);
  std::vector<Par> MPs(1, MP);
  aVec dXa = dX.array();
  return timestep(grids, masks, dXa, CFL, t, tf, count, MPs, 1);
}

static void renorm_single(Vecr u, Par &MP) {
  std::vector<Par> MPs(1, MP);
  renorm_distortion(u, MPs);
}

static bool vcontorted(Vecr u, double tol) { return contorted(u, tol); }

static void reset_single(Vecr u, Par &MP) {
  std::vector<Par> MPs(1, MP);
  reset_distortion(u, MPs);
}

static void reset_multi(Vecr u, std::vector<Par> MPs) { reset_distortion(u, MPs); }

static py::list iterator_single(Vecr u, double tf, iVecr nX, Vecr dX,
                                double CFL, iVecr bcs, bool SPLIT,
                                bool HALF_STEP, bool STIFF, int FLUX, Par &MP,
                                double contorted_tol) {
  std::vector<Par> MPs(1, MP);
  aVec dXa = dX.array();
  std::vector<Vec> ret = iterator(u, tf, nX, dXa, CFL, bcs, SPLIT, HALF_STEP,
                                  STIFF, FLUX, MPs, contorted_tol);
  py::list out;
  for (auto &r : ret)
    out.append(r);
  return out;
}

static Vec vflux(Vecr Q, int d, Par &MP) {
  VecV ret = VecV::Zero();
  VecV q = Q;
  flux(ret, q, d, MP);
  return ret;
}

static Vec vsource(Vecr Q, Par &MP) {
  VecV ret;
  VecV q = Q;
  source(ret, q, MP);
  return ret;
}

static Vec vBdot(Vecr Q, Vecr x, int d, Par &MP) {
  VecV ret = VecV::Zero();
  VecV q = Q, xx = x;
  Bdot(ret, q, xx, d, MP);
  return ret;
}

static Mat vsystem_matrix(Vecr Q, int d, Par &MP) {
  VecV q = Q;
  MatV_V m = system_matrix(q, d, MP);
  return m;
}

static Mat vthermo(Vecr Q, int d, Par &MP) {
  VecV q = Q;
  return thermo_acoustic_tensor(q, d, MP);
}

static double vmax_abs_eigs(Vecr Q, int d, Par &MP) {
  VecV q = Q;
  return max_abs_eigs(q, d, MP);
}

static double vpressure(Vecr Q, Par &MP) {
  VecV q = Q;
  return pressure(q, MP);
}

static double vtemperature(Vecr Q, Par &MP) {
  VecV q = Q;
  return temperature(q, MP);
}

static Vec vD(int which, Vecr qL, Vecr qR, int d, Par &MP) {
  VecV l = qL, r = qR;
  switch (which) {
  case 0:
    return D_RUS(l, r, d, MP);
  case 1:
    return D_ROE(l, r, d, MP);
  default:
    return D_OSH(l, r, d, MP);
  }
}

static Vec vBint(Vecr qL, Vecr qR, int d, Par &MP) {
  VecV l = qL, r = qR;
  return Bint(l, r, d, MP);
}

static Vec vode_cell(Vecr Q, double dt, Par &MP) {
  VecV q = Q;
  ode_stepper_analytic(q, dt, MP);
  return q;
}

// ---- level-set ghost fluid (LSET > 0 variants) ----
static Vec vdistance(Vecr phi, Vecr dX, iVecr nX) {
  aVec d = dX.array();
  return distance(phi, d, nX);
}

static Mat vfinite_difference(Vecr phi, Vecr dX, iVecr nX) {
  Mat D(phi.size(), nX.size());
  aVec d = dX.array();
  iVec n = nX;
  finite_difference(D, phi, d, n);
  return D;
}

static iVec vfind_interface_cells(Vecr phi, iVecr nX) {
  iVec m(phi.size());
  find_interface_cells(m, phi, nX);
  return m;
}

static Vec vleft_star_state(Vecr QL, Vecr QR, Par &MPL, Par &MPR, double dt,
                            Vecr n) {
  VecV l = QL, r = QR;
  Vec nn = n;
  return left_star_state(l, r, MPL, MPR, dt, nn);
}

// fill_ghost_cells on u (re-distanced in place); returns (grids, masks).
static py::tuple vfill_ghost_cells(Vecr u, iVecr nX, Vecr dX, double dt,
                                   std::vector<Par> MPs) {
  int nmat = MPs.size();
  int ncell = u.size() / V;
  std::vector<Vec> grids(nmat);
  std::vector<bVec> masks(nmat);
  for (int i = 0; i < nmat; i++) {
    grids[i] = u;
    masks[i] = bVec::Ones(ncell);
  }
  aVec dXa = dX.array();
  fill_ghost_cells(grids, masks, u, nX, dXa, dt, MPs);
  py::list g, mk;
  for (int i = 0; i < nmat; i++) {
    g.append(grids[i]);
    Vec mm = masks[i].cast<double>();
    mk.append(mm);
  }
  return py::make_tuple(g, mk);
}

static void vmake_u(Vecr u, std::vector<Vec> grids, std::vector<Vec> masks,
                    std::vector<Par> MPs) {
  std::vector<bVec> bm(masks.size());
  for (size_t i = 0; i < masks.size(); i++)
    bm[i] = masks[i].array() != 0.;
  make_u(u, grids, bm, MPs);
}

static py::list iterator_multi(Vecr u, double tf, iVecr nX, Vecr dX, double CFL,
                               iVecr bcs, bool SPLIT, bool HALF_STEP, bool STIFF,
                               int FLUX, std::vector<Par> MPs,
                               double contorted_tol) {
  aVec dXa = dX.array();
  std::vector<Vec> ret = iterator(u, tf, nX, dXa, CFL, bcs, SPLIT, HALF_STEP,
                                  STIFF, FLUX, MPs, contorted_tol);
  py::list out;
  for (auto &r : ret)
    out.append(r);
  return out;
}

PYBIND11_MODULE(MODNAME, m) {
  m.doc() = "test-only bindings over the reference GPR solver";

  m.def("N", []() { return N; });
  m.def("NV", []() { return V; });
  m.def("THERMAL", []() { return THERMAL; });
  m.def("LSET", []() { return LSET; });
  m.def("DG_TOL", []() { return DG_TOL; });
  m.def("DG_IT", []() { return DG_IT; });

  py::class_<Par>(m, "Par")
      .def(py::init<>())
      .def_readwrite("EOS", &Par::EOS)
      .def_readwrite("SOLID", &Par::SOLID)
      .def_readwrite("POWER_LAW", &Par::POWER_LAW)
      .def_readwrite("BINGHAM", &Par::BINGHAM)
      .def_readwrite("MULTI", &Par::MULTI)
      .def_readwrite("rho0", &Par::ρ0)
      .def_readwrite("T0", &Par::T0)
      .def_readwrite("Tref", &Par::Tref)
      .def_readwrite("cv", &Par::cv)
      .def_readwrite("pINF", &Par::pINF)
      .def_readwrite("Gamma0", &Par::Γ0)
      .def_readwrite("c02", &Par::c02)
      .def_readwrite("s", &Par::s)
      .def_readwrite("alpha", &Par::α)
      .def_readwrite("beta", &Par::β)
      .def_readwrite("gamma", &Par::γ)
      .def_readwrite("A", &Par::A)
      .def_readwrite("B", &Par::B)
      .def_readwrite("R1", &Par::R1)
      .def_readwrite("R2", &Par::R2)
      .def_readwrite("b02", &Par::b02)
      .def_readwrite("mu", &Par::μ)
      .def_readwrite("tau0", &Par::τ0)
      .def_readwrite("sigmaY", &Par::σY)
      .def_readwrite("n", &Par::n)
      .def_readwrite("calpha2", &Par::cα2)
      .def_readwrite("kappa", &Par::κ)
      .def_readwrite("dp", &Par::δp)
      .def_readwrite("REACTION", &Par::REACTION);

  m.def("boundaries", &boundaries);
  m.def("extend_mask", &extend_mask);
  m.def("extended_dimensions", &extended_dimensions);
  m.def("weno_launcher", &weno_launcher);
  m.def("predictor", &predictor);
  m.def("fv_launcher", &fv_launcher);
  m.def("centers1", &centers1);
  m.def("centers2", &centers2);
  m.def("interfs1", &interfs1);
  m.def("interfs2", &interfs2);
  m.def("ader_stepper", &ader_stepper);
  m.def("ader_stepper_para", &ader_stepper_para);
  m.def("split_stepper", &split_stepper);
  m.def("midstepper", &midstepper);
  m.def("ode_launcher", &ode_launcher);
  m.def("timestep_single", &timestep_single);
  m.def("renorm_single", &renorm_single);
  m.def("contorted", &vcontorted);
  m.def("reset_single", &reset_single);
  m.def("reset_multi", &reset_multi);
  m.def("iterator_single", &iterator_single);

  m.def("flux", &vflux);
  m.def("source", &vsource);
  m.def("Bdot", &vBdot);
  m.def("system_matrix", &vsystem_matrix);
  m.def("thermo_acoustic_tensor", &vthermo);
  m.def("max_abs_eigs", &vmax_abs_eigs);
  m.def("pressure", &vpressure);
  m.def("temperature", &vtemperature);
  m.def("D", &vD);
  m.def("Bint", &vBint);
  m.def("ode_cell", &vode_cell);

  m.def("distance", &vdistance);
  m.def("finite_difference", &vfinite_difference);
  m.def("find_interface_cells", &vfind_interface_cells);
  m.def("left_star_state", &vleft_star_state);
  m.def("fill_ghost_cells", &vfill_ghost_cells);
  m.def("make_u", &vmake_u);
  m.def("iterator_multi", &iterator_multi);
}
