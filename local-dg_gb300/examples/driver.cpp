// Taylor-Green driver on the GB300 path, written the way the reference's
// driver.cpp:20-47 (commented out there) uses Mesh and Solver:
//   Mesh mesh{nx,nx,nx,botLeft,topRight,mpi}; Solver dgSolver{p,dtSnaps,tf,L,mesh};
//   dgSolver.dgTimeStep();
// Usage: driver <nx> <p> <tf> [snapshot_file]
//   prints dt, steps and the KE series; with snapshot_file, dgTimeStep also
//   writes the reference's CSV snapshots <snapshot_file>.<k> every dtSnaps
//   steps (solver.cpp:366-381).
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "ldg_solver.hpp"

int main(int argc, char** argv) {
  int nx = argc > 1 ? std::atoi(argv[1]) : 10;
  int p = argc > 2 ? std::atoi(argv[2]) : 2;
  double tf = argc > 3 ? std::atof(argv[3]) : 10.0;
  try {
    double L = 1;
    double size = M_PI * L;
    ldg_gb300::Point botLeft{-size, -size, -size};
    ldg_gb300::Point topRight{size, size, size};
    ldg_gb300::Mesh mesh{nx, nx, nx, botLeft, topRight};
    int dtSnaps = 30;
    ldg_gb300::Solver dgSolver{p, dtSnaps, tf, L, mesh};
    if (argc > 4) dgSolver.enableSnapshots(argv[4]);
    std::printf("dt %.17g\nsteps %lld\n", dgSolver.dt(), dgSolver.timesteps());
    dgSolver.dgTimeStep();
    std::vector<double> ke = dgSolver.kineticEnergy();
    for (size_t i = 0; i < ke.size(); ++i) std::printf("ke %zu %.17g\n", i, ke[i]);
    std::vector<double> u = dgSolver.state();
    std::printf("u_0_4_0 %.17g\n", u[4 * dgSolver.dofs()]);
  } catch (const ldg_gb300::Error& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
