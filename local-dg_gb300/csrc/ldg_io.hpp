// Host-only view of a solver's mesh geometry for the snapshot writer
// (ldg_io.cpp), filled by the solver handle (ldg_capi.cu).
#pragma once
#include <string>

#include "../../include/ldg.h"

namespace ldg {

struct Geometry {
  int N = 0, nx = 0, ny = 0, nz = 0;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  double xi[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // CGL nodes (dgMath.cpp:41)
};

// The element boxes and reference nodes of the solver's mesh.
int solver_geometry(const ldg_solver* s, Geometry* g);

// Writes the X-Y-Z-V CSV of a nodal state in the reference layout
// (dofs, 5, nE) column-major to `path`.  Returns an LDG status.
int write_xyzv_file(const std::string& path, const Geometry& g, const double* u);

void set_last_error(const std::string& msg);

}  // namespace ldg
