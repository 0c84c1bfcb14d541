// ldg_solver.hpp -- the reference's C++ Solver/Mesh interface rebuilt on the
// C ABI in ldg.h, so reference-style host code switches to the GB300 path by
// changing its include and namespace.
//
// Reference interface (Local-DG):
//   Point{x,y,z}                                   mesh.h:13-30
//   Mesh(nx,ny,nz,botLeft,topRight[,mpi])          mesh.h:53-58, mesh.cpp:44-355
//   Solver(p, dtSnaps, tf, L, mesh); Solver()      solver.h:110-111, solver.cpp:4-71
//   void Solver::dgTimeStep()                      solver.h:113, solver.cpp:295-453
// Differences by design: errors throw ldg_gb300::Error instead of exit(-1)
// (mesh.cpp:102-107, solver.cpp:356-380); the Mesh is a value (the
// reference's Mesh copy is a non-owning view, array.h:93-99); the MPI
// decomposition argument is absent (one GPU, periodic wrap on device); the
// CSV snapshots of dgTimeStep (output/xyzu.txt.<k> every dtSnaps steps,
// solver.cpp:366-381) are written only after enableSnapshots().  Extra
// accessors expose the state and the kinetic-energy series that dgTimeStep
// prints (solver.cpp:428-450), and exact checkpoints.
#pragma once
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "ldg.h"

namespace ldg_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& where)
      : std::runtime_error(where + ": " + ldg_error_string(status) + " (" + ldg_last_error_message() + ")"),
        status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* where) {
  if (status != LDG_OK) throw Error(status, where);
}

struct Point {
  double x = 0, y = 0, z = 0;
  Point() = default;
  Point(double x_, double y_, double z_) : x(x_), y(y_), z(z_) {}
};

class Mesh {
 public:
  Mesh() : Mesh(10, 10, 10) {}  // mesh.cpp:44
  Mesh(int nx, int ny, int nz) : Mesh(nx, ny, nz, Point{0, 0, 0}, Point{1, 1, 1}) {}  // mesh.cpp:46
  Mesh(int nx, int ny, int nz, const Point& botLeft, const Point& topRight)
      : nx_(nx), ny_(ny), nz_(nz), lo_(botLeft), hi_(topRight) {
    if (nx < 3 || ny < 3 || nz < 3)  // mesh.cpp:102-107
      throw Error(LDG_ERR_INVALID, "Mesh: each direction needs at least 3 elements");
  }
  int nx() const { return nx_; }
  int ny() const { return ny_; }
  int nz() const { return nz_; }
  int nElements() const { return nx_ * ny_ * nz_; }
  const Point& botLeft() const { return lo_; }
  const Point& topRight() const { return hi_; }
  double minDX() const { return (hi_.x - lo_.x) / nx_; }  // mesh.cpp:149-151
  double minDY() const { return (hi_.y - lo_.y) / ny_; }
  double minDZ() const { return (hi_.z - lo_.z) / nz_; }

 private:
  int nx_, ny_, nz_;
  Point lo_, hi_;
};

class Solver {
 public:
  // Solver() delegates to p=2, dtSnaps=10, tf=1, L=1, Mesh{} (solver.cpp:4).
  Solver() : Solver(2, 10, 1.0, 1.0, Mesh{}) {}

  Solver(int p, int dtSnaps, double tf, double L, const Mesh& mesh, int device = 0) : mesh_(mesh) {
    ldg_config c;
    check(ldg_config_default(&c), "ldg_config_default");
    c.p = p;
    c.dt_snaps = dtSnaps;
    c.tf = tf;
    c.L = L;
    c.nx = mesh.nx();
    c.ny = mesh.ny();
    c.nz = mesh.nz();
    c.use_box = 1;
    c.box_lo[0] = mesh.botLeft().x;
    c.box_lo[1] = mesh.botLeft().y;
    c.box_lo[2] = mesh.botLeft().z;
    c.box_hi[0] = mesh.topRight().x;
    c.box_hi[1] = mesh.topRight().y;
    c.box_hi[2] = mesh.topRight().z;
    c.device = device;
    dtSnaps_ = dtSnaps;
    check(ldg_create(&c, &s_), "Solver");
  }
  ~Solver() { ldg_destroy(s_); }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  // Advances to tf (Solver::dgTimeStep, solver.cpp:295-453).
  void dgTimeStep() { check(ldg_time_step(s_), "dgTimeStep"); }

  // One or more RK4 steps (the loop body of dgTimeStep, solver.cpp:410-440).
  void step(int nsteps = 1) { check(ldg_step(s_, nsteps), "step"); }

  ldg_info info() const {
    ldg_info i;
    check(ldg_get_info(s_, &i), "info");
    return i;
  }
  double dt() const { return info().dt; }
  long long timesteps() const { return info().timesteps; }
  int dofs() const { return info().dofs; }
  const Mesh& mesh() const { return mesh_; }

  // Solver::u (solver.h:44), darray(dofs, 5, nElements) column major.
  std::vector<double> state() const {
    std::vector<double> u((size_t)dofs() * 5 * mesh_.nElements());
    check(ldg_get_state(s_, u.data(), LDG_HOST), "state");
    return u;
  }
  void setState(const std::vector<double>& u) {
    if (u.size() != (size_t)dofs() * 5 * mesh_.nElements()) throw Error(LDG_ERR_INVALID, "setState: wrong size");
    check(ldg_set_state(s_, u.data(), LDG_HOST), "setState");
  }
  // k = rhs(uCurr) (Solver::rk4Rhs, solver.cpp:486-535).
  std::vector<double> rhs(const std::vector<double>& uCurr) {
    std::vector<double> k(uCurr.size());
    check(ldg_rhs(s_, uCurr.data(), k.data(), LDG_HOST), "rhs");
    return k;
  }
  // kes and keDissipation of dgTimeStep (solver.cpp:437-450).
  std::vector<double> kineticEnergy() const {
    int n = 0;
    check(ldg_ke_history(s_, nullptr, 0, &n), "kineticEnergy");
    std::vector<double> ke(n);
    if (n) check(ldg_ke_history(s_, ke.data(), n, &n), "kineticEnergy");
    return ke;
  }
  std::vector<double> keDissipation() const {
    int n = 0;
    check(ldg_ke_dissipation(s_, nullptr, 0, &n), "keDissipation");
    std::vector<double> e(n);
    if (n) check(ldg_ke_dissipation(s_, e.data(), n, &n), "keDissipation");
    return e;
  }
  // The reference's snapshots: dgTimeStep writes <filename>.<k> before step
  // k*dtSnaps (solver.cpp:366-381, format io.cpp:8-72).
  void enableSnapshots(const std::string& filename = "output/xyzu.txt") {
    check(ldg_set_snapshots(s_, filename.c_str(), dtSnaps_), "enableSnapshots");
  }
  void disableSnapshots() { check(ldg_set_snapshots(s_, nullptr, 0), "disableSnapshots"); }
  // One X-Y-Z-V snapshot of the current state (exportToXYZVFile).
  void writeSnapshot(const std::string& filename, int timeseries = -1) {
    check(ldg_write_xyzv(s_, filename.c_str(), timeseries), "writeSnapshot");
  }
  // Exact checkpoint / resume (loading requires the same discretisation).
  void saveCheckpoint(const std::string& path) { check(ldg_save_checkpoint(s_, path.c_str()), "saveCheckpoint"); }
  void loadCheckpoint(const std::string& path) { check(ldg_load_checkpoint(s_, path.c_str()), "loadCheckpoint"); }
  ldg_solver* handle() { return s_; }

 private:
  Mesh mesh_;
  int dtSnaps_ = 0;
  ldg_solver* s_ = nullptr;
};

}  // namespace ldg_gb300
