// Internal interface between the solver (ldg_capi.cu) and the learned
// closure (ldg_closure.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/ldg.h"
#include "ldg_device.cuh"

namespace ldg {

// What the closure needs to know about a solver.
struct SolverView {
  int N, n, nf, nE, nx, ny, nz, p;
  const DevOps* ops;
  const OpsT<double>* o64;
  cudaStream_t stream;
  int device;
  bool mixed;
  double* Un;  // current state, Gauss basis
  double* Q;   // gradient scratch
};

SolverView solver_view(ldg_solver* s);
int solver_rhs_gauss(ldg_solver* s, const double* U, double* K);
int solver_set_gauss_state(ldg_solver* s, const double* U);

// Closure hooks used by the solver's stage loop.
int closure_check_solver(ldg_closure* c, const SolverView& v);
int closure_correction(ldg_closure* c, const SolverView& v, const double* U, const double* Q, double* Kadd,
                       cudaStream_t st);

}  // namespace ldg
