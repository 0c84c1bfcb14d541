/*
 * Driver for the unmodified reference sources (test infrastructure: it
 * produces the golden vectors that pin the oracle and the CUDA path; it is
 * never shipped or timed as the product).
 *
 * The reference's own main() is a no-op (driver.cpp:20-48 commented out),
 * and Solver::dgTimeStep() (solver.cpp:295-453) interleaves the RK4 loop
 * with CSV snapshots and per-step prints.  This driver replicates the
 * inner loop of dgTimeStep (solver.cpp:410-440) step by step, without IO,
 * by reaching the private stage functions (rk4UpdateCurr, rk4Rhs,
 * computeKE) through "#define private public".
 *
 * Modes:
 *   step <nx> <p> <steps> <outprefix> [dump_every] [threads] [state_in]
 *        Taylor-Green (or <state_in> if given) -> <steps> RK4 steps.
 *        Writes <outprefix>.ke (steps doubles), <outprefix>.u<step> for
 *        every step that is a multiple of dump_every (and the last), each
 *        (dofs,5,nE) column-major doubles, and <outprefix>.meta (text).
 *   rhs  <nx> <p> <state_in|-> <outprefix> [threads]
 *        One rk4Rhs on the given state (or Taylor-Green), istage 0:
 *        writes <outprefix>.k (dofs,5,nE) and <outprefix>.u0.
 *   series <nx> <p> <steps> <outprefix> <index_file> [threads] [ens_every]
 *        Taylor-Green -> <steps> RK4 steps, recording after every step the
 *        KE (<outprefix>.ke), the sum of squares of each conserved
 *        variable over all nodes and elements (<outprefix>.norms,
 *        steps x 5) and the state entries at the flat column-major
 *        indices listed in <index_file> (int64) (<outprefix>.samples,
 *        steps x count).  For meshes whose full states are too large to
 *        keep for every step.  With ens_every > 0, after every
 *        ens_every-th step also the enstrophy of the state
 *        (<outprefix>.enst: pairs step, value), from the reference's own
 *        LDG gradient Dus of that state (one extra rk4Rhs, whose ks slot
 *        0 is dead once the step is accumulated).
 *   csv  <nx> <p> <steps> <outprefix> [threads]
 *        Taylor-Green -> <steps> RK4 steps, then the reference's own
 *        snapshot writer (initXYZVFile + exportToXYZVFile, io.cpp:8-99)
 *        on the state: <outprefix>.0.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <algorithm>
#include <functional>
#include <numeric>
#include <stdexcept>

#include <mpi.h>
#include <cblas.h>
#include <lapacke.h>

#define private public
#include "solver.h"
#undef private

static void write_doubles(const std::string& path, const double* p, long n) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::fprintf(stderr, "cannot open %s\n", path.c_str()); std::exit(2); }
  if ((long)std::fwrite(p, sizeof(double), n, f) != n) { std::fprintf(stderr, "short write\n"); std::exit(2); }
  std::fclose(f);
}

static void read_doubles(const std::string& path, double* p, long n) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { std::fprintf(stderr, "cannot open %s\n", path.c_str()); std::exit(2); }
  if ((long)std::fread(p, sizeof(double), n, f) != n) { std::fprintf(stderr, "short read %s\n", path.c_str()); std::exit(2); }
  std::fclose(f);
}

/* tf such that the constructor's ceil(tf/dt) (solver.cpp:51) gives exactly
 * `steps` and dt = tf/steps equals the CFL dt up to the last bits. */
static double tf_for_steps(int nx, int p, double L, int steps) {
  double minDX = (M_PI * L - (-M_PI * L)) / nx;
  double dt0 = 0.01 * minDX / (1.0 * (2 * p + 1));
  double tf = steps * dt0;
  while ((long)std::ceil(tf / dt0) > steps) tf = std::nextafter(tf, 0.0);
  return tf;
}

/* Enstrophy of the state whose rk4Rhs just ran: the quadrature over the
 * Gauss points of rho |curl v|^2 / 2, normalised like computeKE
 * (solver.cpp:1007-1034) by rho0 (2 pi L)^3, from the reference's own
 * interpolants uInterp3D = Interp3D u and DuInterp3D = Interp3D Dus
 * (solver.cpp:495-514).  v = m/rho, d_j v_i = (d_j m_i - v_i d_j rho)/rho. */
static double enstrophy(Solver& s, const darray& uI3, const darray& DuI3) {
  darray xQ, wQ;
  int nQ3D = gaussQuad3D(2 * s.order, xQ, wQ);
  double J = s.mesh.minDX / 2.0 * s.mesh.minDY / 2.0 * s.mesh.minDZ / 2.0;
  double total = 0.0;
  for (int iK = 0; iK < s.mesh.nElements; ++iK) {
    double el = 0.0;
    for (int q = 0; q < nQ3D; ++q) {
      double rho = uI3(q, 0, iK), v[3], G[3][3];
      for (int i = 0; i < 3; ++i) v[i] = uI3(q, 1 + i, iK) / rho;
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) G[i][j] = (DuI3(q, 1 + i, iK, j) - DuI3(q, 0, iK, j) * v[i]) / rho;
      double wx = G[2][1] - G[1][2], wy = G[0][2] - G[2][0], wz = G[1][0] - G[0][1];
      el += J * wQ(q) * 0.5 * rho * (wx * wx + wy * wy + wz * wz);
    }
    total += el;
  }
  return total / (s.p.rho0 * std::pow(2 * M_PI * s.p.L, 3.0));
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ldg_ref step|rhs ...\n");
    return 1;
  }
  MPI_Init(&argc, &argv);
  std::string mode = argv[1];
  const double L = 1.0;
  if (mode == "step" || mode == "series" || mode == "csv") {
    const bool series = mode == "series", csv = mode == "csv";
    if (argc < (series ? 7 : 6)) {
      std::fprintf(stderr, "step <nx> <p> <steps> <out> [dump_every] [threads] [state_in]\n"
                           "series <nx> <p> <steps> <out> <index_file> [threads]\n");
      return 1;
    }
    int nx = std::atoi(argv[2]), p = std::atoi(argv[3]), steps = std::atoi(argv[4]);
    // csv with 0 steps writes the initial condition (the solver is built for 1)
    const int run_steps = steps;
    if (csv && steps == 0) steps = 1;
    std::string out = argv[5];
    int dump_every = (!series && !csv && argc > 6) ? std::atoi(argv[6]) : steps;
    int threads = csv ? (argc > 6 ? std::atoi(argv[6]) : 1) : (argc > 7 ? std::atoi(argv[7]) : 1);
    const int ens_every = (series && argc > 8) ? std::atoi(argv[8]) : 0;
    std::vector<double> enst;
    scipy_openblas_set_num_threads(threads);
    MPIUtil mpi{};
    double size = M_PI * L;
    Point botLeft{-size, -size, -size};
    Point topRight{size, size, size};
    Mesh mesh{nx, nx, nx, botLeft, topRight, mpi};
    double tf = tf_for_steps(nx, p, L, steps);
    Solver s{p, 1 << 30, tf, L, mesh};
    if (s.timesteps != steps) { std::fprintf(stderr, "timesteps %d != %d\n", (int)s.timesteps, steps); return 2; }
    long nU = (long)s.dofs * s.nStates * s.mesh.nElements;
    if (!series && !csv && argc > 8 && std::string(argv[8]) != "-") read_doubles(argv[8], s.u.data(), nU);
    std::vector<long long> idx;
    if (series) {
      FILE* f = std::fopen(argv[6], "rb");
      if (!f) { std::fprintf(stderr, "cannot open %s\n", argv[6]); return 2; }
      long long v;
      while (std::fread(&v, sizeof(v), 1, f) == 1) {
        if (v < 0 || v >= nU) { std::fprintf(stderr, "index %lld out of range\n", v); return 2; }
        idx.push_back(v);
      }
      std::fclose(f);
    }
    std::vector<double> norms, samples;

    /* Work arrays exactly as dgTimeStep allocates them (solver.cpp:298-338). */
    int nStages = 4;
    darray b{nStages};
    b(0) = 1 / 6.0; b(1) = 1 / 3.0; b(2) = 1 / 3.0; b(3) = 1 / 6.0;
    darray diagA{nStages - 1};
    diagA(0) = 0.5; diagA(1) = 0.5; diagA(2) = 1.0;
    int nQ2D = s.mesh.nFQNodes;
    int nE = s.mesh.nElements, nG = s.mesh.nGElements, dofs = s.dofs, nS = s.nStates;
    darray uCurr{dofs, nS, nE, 1};
    darray uInterp2D{nQ2D, nS, Mesh::N_FACES, nE + nG, 1};
    darray uInterp3D{s.Interp3D.size(0), nS, nE, 1};
    darray ks{dofs, nS, nE, nStages};
    darray Dus{dofs, nS, nE, Mesh::DIM};
    darray DuInterp2D{nQ2D, nS, Mesh::N_FACES, nE + nG, Mesh::DIM};
    darray DuInterp3D{s.Interp3D.size(0), nS, nE, Mesh::DIM};
    int nBElems = max(s.mesh.mpiNBElems);
    darray toSend{nQ2D, nS, nBElems, Mesh::DIM, MPIUtil::N_FACES};
    darray toRecv{nQ2D, nS, nBElems, Mesh::DIM, MPIUtil::N_FACES};
    MPI_Request rk4Reqs[2 * MPIUtil::N_FACES];
    std::vector<double> kes(steps);

    if (!series && !csv) write_doubles(out + ".u0", s.u.data(), nU);
    double ke0 = s.computeKE(uInterp3D);
    auto t0 = std::chrono::high_resolution_clock::now();
    for (int iStep = 0; iStep < run_steps; ++iStep) {
      for (int istage = 0; istage < nStages; ++istage) {
        s.rk4UpdateCurr(uCurr, diagA, ks, istage);
        s.rk4Rhs(uCurr, uInterp2D, uInterp3D, Dus, DuInterp2D, DuInterp3D, toSend, toRecv, rk4Reqs,
                 ks, istage);
      }
      /* RK accumulate, stage order 0..3 (solver.cpp:422-434), prints dropped. */
      for (int istage = 0; istage < nStages; ++istage)
        for (int iK = 0; iK < nE; ++iK)
          for (int iS = 0; iS < nS; ++iS)
            for (int iN = 0; iN < dofs; ++iN)
              s.u(iN, iS, iK) += s.dt * b(istage) * ks(iN, iS, iK, istage);
      kes[iStep] = s.computeKE(uInterp3D);
      if (series) {
        for (int iS = 0; iS < nS; ++iS) {
          double acc = 0.0;
          for (int iK = 0; iK < nE; ++iK)
            for (int iN = 0; iN < dofs; ++iN) acc += s.u(iN, iS, iK) * s.u(iN, iS, iK);
          norms.push_back(acc);
        }
        for (long long j : idx) samples.push_back(s.u.data()[j]);
        if (ens_every > 0 && (iStep + 1) % ens_every == 0) {
          s.rk4UpdateCurr(uCurr, diagA, ks, 0);  // stage 0: uCurr = u
          s.rk4Rhs(uCurr, uInterp2D, uInterp3D, Dus, DuInterp2D, DuInterp3D, toSend, toRecv, rk4Reqs,
                   ks, 0);
          enst.push_back(iStep + 1);
          enst.push_back(enstrophy(s, uInterp3D, DuInterp3D));
        }
        continue;
      }
      if (csv) continue;
      if ((iStep + 1) % dump_every == 0 || iStep + 1 == steps) {
        std::ostringstream oss;
        oss << out << ".u" << (iStep + 1);
        write_doubles(oss.str(), s.u.data(), nU);
      }
    }
    auto t1 = std::chrono::high_resolution_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    write_doubles(out + ".ke", kes.data(), steps);
    if (csv && !(initXYZVFile(out, 0, "u", nS) && exportToXYZVFile(out, 0, s.mesh.globalCoords, s.u))) {
      std::fprintf(stderr, "snapshot writer failed\n");
      return 2;
    }
    if (series) {
      write_doubles(out + ".norms", norms.data(), (long)norms.size());
      write_doubles(out + ".samples", samples.data(), (long)samples.size());
      if (!enst.empty()) write_doubles(out + ".enst", enst.data(), (long)enst.size());
    }
    std::ofstream meta(out + ".meta");
    meta.precision(17);
    meta << "nx " << nx << "\np " << p << "\nsteps " << steps << "\ndt " << s.dt << "\ntf " << s.tf
         << "\nke0 " << ke0 << "\nseconds " << secs << "\nthreads " << threads
         << "\ndof_stage_per_s " << (double)dofs * nE * 4.0 * steps / secs << "\n";
    std::printf("seconds %.6f dof_stage_per_s %.6e dt %.17g\n", secs, (double)dofs * nE * 4.0 * steps / secs, s.dt);
  } else if (mode == "rhs") {
    if (argc < 6) { std::fprintf(stderr, "rhs <nx> <p> <state_in|-> <out> [threads]\n"); return 1; }
    int nx = std::atoi(argv[2]), p = std::atoi(argv[3]);
    std::string in = argv[4], out = argv[5];
    int threads = argc > 6 ? std::atoi(argv[6]) : 1;
    scipy_openblas_set_num_threads(threads);
    MPIUtil mpi{};
    double size = M_PI * L;
    Point botLeft{-size, -size, -size};
    Point topRight{size, size, size};
    Mesh mesh{nx, nx, nx, botLeft, topRight, mpi};
    Solver s{p, 1 << 30, tf_for_steps(nx, p, L, 1), L, mesh};
    long nU = (long)s.dofs * s.nStates * s.mesh.nElements;
    if (in != "-") read_doubles(in, s.u.data(), nU);
    int nQ2D = s.mesh.nFQNodes;
    int nE = s.mesh.nElements, nG = s.mesh.nGElements, dofs = s.dofs, nS = s.nStates;
    darray diagA{3};
    diagA(0) = 0.5; diagA(1) = 0.5; diagA(2) = 1.0;
    darray uCurr{dofs, nS, nE, 1};
    darray uInterp2D{nQ2D, nS, Mesh::N_FACES, nE + nG, 1};
    darray uInterp3D{s.Interp3D.size(0), nS, nE, 1};
    darray ks{dofs, nS, nE, 4};
    darray Dus{dofs, nS, nE, Mesh::DIM};
    darray DuInterp2D{nQ2D, nS, Mesh::N_FACES, nE + nG, Mesh::DIM};
    darray DuInterp3D{s.Interp3D.size(0), nS, nE, Mesh::DIM};
    int nBElems = max(s.mesh.mpiNBElems);
    darray toSend{nQ2D, nS, nBElems, Mesh::DIM, MPIUtil::N_FACES};
    darray toRecv{nQ2D, nS, nBElems, Mesh::DIM, MPIUtil::N_FACES};
    MPI_Request rk4Reqs[2 * MPIUtil::N_FACES];
    s.rk4UpdateCurr(uCurr, diagA, ks, 0);
    s.rk4Rhs(uCurr, uInterp2D, uInterp3D, Dus, DuInterp2D, DuInterp3D, toSend, toRecv, rk4Reqs, ks, 0);
    write_doubles(out + ".u0", s.u.data(), nU);
    write_doubles(out + ".k", &ks(0, 0, 0, 0), nU);
    write_doubles(out + ".q", Dus.data(), nU * 3);
    std::ofstream meta(out + ".meta");
    meta.precision(17);
    meta << "nx " << nx << "\np " << p << "\ndt " << s.dt << "\n";
  } else {
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 1;
  }
  MPI_Finalize();
  return 0;
}
