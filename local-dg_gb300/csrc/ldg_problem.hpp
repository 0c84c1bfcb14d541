// Host-side set-up of one periodic LDG problem, shared by the solver handle
// (ldg_capi.cu) and the batched ensemble (ldg_ensemble.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/ldg.h"
#include "ldg_kernels.cuh"
#include "ldg_ops.hpp"

namespace ldg {

struct Problem {
  ldg_config cfg;
  int N = 0, n = 0, nf = 0, nE = 0;
  double dt = 0, tf = 0;
  long long timesteps = 0;
  DevOps ops;
  Ops1D o1;
  double xi[kMaxN];  // CGL nodes as the reference computes them
  double lo[3], hi[3];
  double p0 = 0, T0 = 0, R = 8.314, rho0 = 1.0, V0 = 1.0;
};

// Validates cfg and fills the problem: physics and CFL time step
// (solver.cpp:30-52), domain and element sizes (mesh.cpp:51-151), operator
// block.  Returns an LDG status; on failure the message is in *err.
int setup_problem(const ldg_config& cfg, Problem* pb, std::string* err);

// Taylor-Green initial condition (plus the configured perturbation) at the
// CGL nodes, reference layout, into `nodal`.
cudaError_t launch_initial_condition(const Problem& pb, double* nodal, cudaStream_t st);

// Nodal <-> Gauss tensor transform (inverse = 1: Gauss -> nodal).
cudaError_t launch_transform_any(int N, const double* in, double* out, int nE, const DevOps& ops, int inverse,
                                 cudaStream_t st);

// FP64 face traces of an FP64 state.
cudaError_t launch_traces_fp64(int N, const double* U, double* Tu, int nE, const OpsT<double>& o,
                               cudaStream_t st);

// One gradient pass and one RHS/RK pass of the solo FP64 kernels (the
// launches ldg_step makes), for callers outside the solver handle.
cudaError_t launch_grad_fp64(int N, const double* U, const double* Tu, double* Q, double* Tq, double* Fm,
                             const DevOps& ops, const OpsT<double>& o, cudaStream_t st);
cudaError_t launch_rhs_fp64(int N, const StageArgs<double>& a, const DevOps& ops, const OpsT<double>& o,
                            cudaStream_t st);

void set_last_error(const std::string& msg);

}  // namespace ldg
