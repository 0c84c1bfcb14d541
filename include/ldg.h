/*
 * ldg.h -- C ABI of the GB300 (sm_103a) LDG Navier-Stokes right-hand side.
 *
 * This is the drop-in boundary for the hot path of Local-DG: the RK4
 * time step of the Local Discontinuous Galerkin discretisation of 3-D
 * compressible Navier-Stokes on a periodic uniform hex mesh.  The
 * reference has no FFI; its boundary is the C++ class Solver
 * (solver.h:20-115), whose constructor Solver(p, dtSnaps, tf, L, mesh)
 * (solver.cpp:7-71) and dgTimeStep() (solver.cpp:295-453) drive the
 * internal seam rk4UpdateCurr/rk4Rhs (solver.h:76-79).  Each entry point
 * below names the reference interface it replaces.  include/ldg_solver.hpp
 * rebuilds the Solver/Mesh classes on top of these calls.
 *
 * Conventions
 *  - Every call returns an int status: LDG_OK (0) or a negative LDG_ERR_*.
 *    ldg_error_string() names it; ldg_last_error_message() gives detail.
 *  - State arrays use the reference layout: darray u(dofs, 5, nElements),
 *    column major (solver.cpp:62), i.e. element-major blocks of 5 variables
 *    (rho, rho*u, rho*v, rho*w, rho*E; solver.cpp:217-229), each a block of
 *    dofs = (p+1)^3 nodal values, node = ix + N*iy + N*N*iz, N = p+1.
 *  - Elements are numbered e = ix + nx*(iy + ny*iz) (mesh.cpp:162) on the
 *    periodic cube [-pi L, pi L]^3.
 *  - Pointers are host pointers unless the call takes `where` =
 *    LDG_DEVICE, in which case they are device pointers on the solver's GPU.
 *  - A handle owns its device buffers and one CUDA stream; calls on one
 *    handle are not thread safe (like the reference Solver).  All calls
 *    are stream ordered; calls that return host data synchronise.
 */
#ifndef LDG_H
#define LDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LDG_ABI_VERSION 1

/* status codes */
#define LDG_OK 0
#define LDG_ERR_INVALID -1     /* bad argument or configuration            */
#define LDG_ERR_CUDA -2        /* a CUDA call failed                       */
#define LDG_ERR_NOMEM -3       /* device or host allocation failed         */
#define LDG_ERR_NONFINITE -4   /* NaN/Inf found in the state after a step  */
#define LDG_ERR_UNSUPPORTED -5 /* order or mode not built                  */
#define LDG_ERR_NODEVICE -6    /* no CUDA device visible                   */
#define LDG_ERR_TIMEOUT -7     /* a bounded on-device wait gave up          */
#define LDG_ERR_IO -8          /* a file could not be written or read, or a
                                  checkpoint failed its checks              */

/* where a pointer lives */
#define LDG_HOST 0
#define LDG_DEVICE 1

/* arithmetic of the RHS */
#define LDG_FP64 0        /* every operation in FP64 */
#define LDG_MIXED_F32X2 1 /* RHS in FP32-pair ("double-word") arithmetic on
                             the FP32 pipe; FP64 state, RK4 accumulation,
                             inverse mass and reductions.  Not bitwise the
                             reference; error reported against FP64. */

typedef struct ldg_config {
  int p;            /* polynomial order, 1..7 (Solver ctor _p)           */
  int nx, ny, nz;   /* elements per direction, each >= 3 (mesh.cpp:102) */
  double L;         /* domain [-pi L, pi L]^3 (driver.cpp:26-31)        */
  double tf;        /* final time (Solver ctor _tf)                      */
  int dt_snaps;     /* snapshot cadence (Solver ctor _dtSnaps); 0 = none */
  double Re;        /* Reynolds number (solver.cpp:30), default 1600     */
  double Pr;        /* Prandtl number (solver.cpp:31), default 0.71      */
  double gamma;     /* ratio of specific heats (solver.cpp:32), 1.4      */
  double Ma;        /* Mach number (solver.cpp:33), default 0.1          */
  double cfl;       /* dt = cfl*min(dx)/(V0(2p+1)) (solver.cpp:47), 0.01 */
  int precision;    /* LDG_FP64 or LDG_MIXED_F32X2                       */
  int device;       /* CUDA device ordinal                               */
  int check_finite; /* nonzero: ldg_step scans the state for NaN/Inf     */
  int use_box;      /* 0: domain [-pi L, pi L]^3 (driver.cpp:28-31);
                       1: [box_lo, box_hi] (Mesh botLeft/topRight,
                       mesh.cpp:51-151); periodic either way             */
  double box_lo[3], box_hi[3];
  /* Seeded velocity perturbation added to the Taylor-Green initial
   * condition (no reference counterpart; ensemble inputs):
   *   dv_c = perturb_amp*V0/12 * sum_{k=1..4} sum_{d=x,y,z} sin(k x_d/L + phi)
   * with phases phi = 2 pi U[0,1) from SplitMix64 keyed by (seed, instance,
   * c, k, d).  perturb_amp = 0 gives the reference's initial condition. */
  double perturb_amp;
  unsigned long long seed;
  int instance;
  int reserved[7];
} ldg_config;

typedef struct ldg_info {
  int p, dofs, nf;          /* (p+1)^3 nodes, (p+1)^2 face points       */
  int nx, ny, nz, nelements;
  double dt;                /* time step after the tf adjustment         */
  long long timesteps;      /* ceil(tf/dt) (solver.cpp:51-52)            */
  long long step;           /* RK4 steps taken so far                    */
  double time;              /* step * dt                                 */
  size_t device_bytes;      /* device memory held by the handle          */
  int precision;
} ldg_info;

typedef struct ldg_solver ldg_solver;

/* Fills the reference defaults (solver.cpp:30-52; driver.cpp:26-39). */
int ldg_config_default(ldg_config* cfg);

/* Replaces Solver::Solver(p, dtSnaps, tf, L, mesh) (solver.cpp:7-71):
 * physics, CFL time step, operators, and the Taylor-Green initial
 * condition (solver.cpp:194-236) as the current state. */
int ldg_create(const ldg_config* cfg, ldg_solver** out);

/* Frees the handle and every device buffer it owns. */
int ldg_destroy(ldg_solver* s);

int ldg_get_info(const ldg_solver* s, ldg_info* info);

/* Sets / reads the solver state Solver::u (solver.h:44) in the reference
 * layout; where = LDG_HOST or LDG_DEVICE. */
int ldg_set_state(ldg_solver* s, const double* u, int where);
int ldg_get_state(ldg_solver* s, double* u, int where);
/* Host buffers (in ldg_set_state, ldg_get_state, ldg_rhs) move in `chunks`
 * element ranges (1..64, default 8) on a copy stream, so that the copy of
 * one range overlaps the basis transform of the previous one; 1 copies the
 * whole state before transforming it.  (No reference counterpart.) */
int ldg_set_transfer_chunks(ldg_solver* s, int chunks);
/* ldg_set_state(u_in) + ldg_step(nsteps) + ldg_get_state(u_out) with host
 * buffers, bit for bit, in one call that overlaps the transfers with the
 * step: the upload comes in z-plane chunks and stage 0's gradient pass of a
 * chunk starts as soon as the chunk and its -z neighbour plane are there;
 * the last stage's RHS pass runs chunk by chunk and each chunk of the new
 * state goes back to the host while the next one is computed.  For a
 * caller that keeps the state on the host, as the reference keeps
 * Solver::u (solver.h:44) around dgTimeStep (solver.cpp:295-453).  u_in
 * may equal u_out.  Returns once u_out holds the result.  With a closure
 * attached it runs the three calls in sequence. */
int ldg_advance_host(ldg_solver* s, const double* u_in, double* u_out, int nsteps);

/* Resets the state to the Taylor-Green vortex (solver.cpp:194-236) and the
 * step counter to 0. */
int ldg_set_initial_condition(ldg_solver* s);

/* One right-hand side k = rhs(uCurr), both in the reference layout: the
 * seam Solver::rk4Rhs(uCurr, ..., ks, istage) (solver.h:77-79,
 * solver.cpp:486-535) for one stage.  Does not change the state. */
int ldg_rhs(ldg_solver* s, const double* u_curr, double* k, int where);

/* Advances nsteps classical RK4 steps (the loop body of
 * Solver::dgTimeStep, solver.cpp:410-440: stage combine rk4UpdateCurr
 * solver.cpp:458-480, rk4Rhs, accumulation u += dt*b_s*k_s in stage order)
 * and records computeKE (solver.cpp:1007-1034) after every step. */
int ldg_step(ldg_solver* s, int nsteps);

/* Replaces Solver::dgTimeStep() (solver.cpp:295-453): all remaining steps
 * to tf.  No CSV output (io.cpp is out of scope); the KE series is kept. */
int ldg_time_step(ldg_solver* s);

/* Diagnostics of the current state:
 *   ke_ref    computeKE exactly as the reference (nodal values weighted by
 *             Gauss weights, solver.cpp:1021-1031);
 *   ke        kinetic energy by Gauss quadrature of |m|^2/(2 rho);
 *   enstrophy quadrature of rho |curl v|^2 / 2 from the LDG gradient;
 * each normalised by rho0 (2 pi L)^3.  Any pointer may be NULL. */
int ldg_diagnostics(ldg_solver* s, double* ke_ref, double* ke, double* enstrophy);

/* KE series recorded by ldg_step (computeKE after each step, as
 * dgTimeStep's kes, solver.cpp:437), and the dissipation rate
 * -(KE_n - KE_{n-2})/(2 dt) (solver.cpp:438-440).  *count receives the
 * number of entries available; at most max are copied. */
int ldg_ke_history(ldg_solver* s, double* ke, int max, int* count);
int ldg_ke_dissipation(ldg_solver* s, double* eps, int max, int* count);

/* Waits for all work queued on the handle's stream. */
int ldg_synchronize(ldg_solver* s);

/* ---- Snapshots (solver.cpp:366-381, io.cpp:8-99) and checkpoints. */

/* Writes the current state as the reference's X-Y-Z-V CSV file
 * (initXYZVFile + exportToXYZVFile, io.cpp:8-72): the header line
 * "X, Y, Z, u0, u1, u2, u3, u4", then one line per element and node, in
 * element then node order, holding the node's coordinates (the CGL nodes
 * mapped into the element, mesh.cpp:389-408) and the five conserved
 * variables, each printed the way a C++ stream prints a double by default
 * (printf "%.6g"), separated by ", ".  The file is <filename>.<timeseries>
 * (io.cpp:30-35), or <filename> when timeseries < 0.  Overwrites. */
int ldg_write_xyzv(ldg_solver* s, const char* filename, int timeseries);

/* Snapshot cadence of ldg_time_step: with every > 0 it writes
 * <filename>.<step/every> before each step whose index is a multiple of
 * every, as dgTimeStep writes output/xyzu.txt.<k> (solver.cpp:366-381).
 * filename NULL or every <= 0 turns snapshots off (the default). */
int ldg_set_snapshots(ldg_solver* s, const char* filename, int every);

/* Exact checkpoints.  No reference counterpart: the reference dumps a CSV
 * of u when it reaches its wall-clock limit (solver.cpp:351-360) and has
 * no reader.  The file holds the config, the step count and time step,
 * the internal FP64 Gauss-point state, the face traces of that state and
 * the KE series, with a 64-bit FNV-1a hash of the payload.  A solver
 * created from the stored config (ldg_checkpoint_config) that loads the
 * file continues bit for bit as the saved solver would have.  Loading
 * into a solver whose discretisation (p, mesh, box, physics, precision or
 * dt) differs returns LDG_ERR_INVALID; a truncated, foreign or corrupted
 * file returns LDG_ERR_IO.  Save writes <path>.tmp and renames it. */
int ldg_save_checkpoint(ldg_solver* s, const char* path);
int ldg_checkpoint_config(const char* path, ldg_config* cfg);
int ldg_load_checkpoint(ldg_solver* s, const char* path);

/* The handle's CUDA stream (a cudaStream_t) so callers can order their
 * own work against it. */
void* ldg_stream(ldg_solver* s);

/* Per-kernel device time, for roofline reporting.  enable != 0 brackets
 * every kernel that ldg_step launches with CUDA events on the handle's
 * stream; ldg_kernel_times then returns, per kernel class, the summed
 * milliseconds and launch counts since the last reset (reset != 0 clears
 * them).  Classes: 0 gradient pass, 1 RHS+RK pass, 2 KE reduction.
 * (No reference counterpart: the reference only prints wall-clock,
 * solver.cpp:344-371.) */
#define LDG_KERNEL_CLASSES 3
int ldg_enable_kernel_timing(ldg_solver* s, int enable);
int ldg_kernel_times(ldg_solver* s, double* ms, long long* launches, int max_classes, int reset);

/* Measures the FP64 FMA rate of the device (TFLOP/s, 2 flops per FMA) with
 * a register-resident FMA chain; the roofline denominator for the FP64
 * kernels.  (No reference counterpart.) */
int ldg_probe_fp64_peak(int device, double* tflops);
/* The same probe with two more readings: FP64 FMAs issued per SM per SM
 * clock (from clock64 spans, independent of the clock frequency) and the
 * SM clock the probe ran at, in MHz (cycles over event time).  Either
 * pointer may be NULL.  (No reference counterpart.) */
int ldg_probe_fp64(int device, double* tflops, double* fma_per_sm_clk, double* sm_mhz);
/* Applies the flux kernels' FP64 reciprocal (an FP32 special-function seed
 * and one third-order correction) and reciprocal square root (CUDA's
 * rsqrt) to the n host operands x, writing 1/x to r and 1/sqrt(x) to rs
 * (host buffers).  For checking them against correctly rounded values.
 * (No reference counterpart: the reference divides and calls sqrt,
 * solver.cpp:1291-1372.) */
int ldg_probe_recip(int device, const double* x, double* r, double* rs, long n);
/* The 1-D factors of the element operators for order p (1..7), host only
 * (no device needed): Gauss points x and weights w (N = p+1 each), the weak
 * derivative A[q*N + r] = (w_r/w_q) L_q'(x_r) (N*N), and the face lifts
 * Lp/Lm[q] = L_q(+-1)/w_q (N each), L_q the Lagrange polynomial of Gauss
 * point q.  The step kernels apply them by sum factorisation, and the FP64
 * gradient pass uses their symmetries (A skew-centrosymmetric, Lp the
 * mirror of Lm).  These are the 1-D factors of the reference's Sels, Kels
 * and Kels2D with its mass matrix (solver.cpp:74-192) in the Gauss-point
 * basis. */
int ldg_operators_1d(int p, double* x, double* w, double* A, double* Lp, double* Lm);
/* Measures the gradient pass's volume contraction alone (the product the
 * reference evaluates as a dense DGEMM, solver.cpp:500, here the
 * sum-factorised 1-D products along each direction) on the solver's
 * current state, in one of four arithmetics: mode 0 FP64 FMAs, 1 FP32-pair
 * FMAs, 2 FP32-pair compensated dot products, 3 tensor cores with exact
 * integer slices (p = 4 only).  *ms: mean time of one launch over reps
 * launches; *max_rel_err: largest difference from mode 0 over the first
 * 2048 elements, relative to their largest value.  Overwrites the solver's
 * scratch buffers (gradient, spare traces), not its state.  (No reference
 * counterpart: it decides the arithmetic of the mixed path.) */
int ldg_probe_contraction(ldg_solver* s, int mode, int reps, double* ms, double* max_rel_err);

/* ---- Batched ensemble.  No reference counterpart (the reference runs one
 * problem per MPI job).  Members are independent problems, each an
 * ldg_config (p in 2..4, LDG_FP64, all on one device; mesh size, order, Re
 * and the seeded perturbation may differ).  Every RK4 stage of all members
 * is one persistent kernel launch over a work queue of (member, element
 * block) items; a step (4 launches + KE reductions) is replayed from a CUDA
 * graph.  Each member's state and KE series equal a solo ldg_create/ldg_step
 * run of the same config bit for bit.  The tile shape (threads per CTA) and
 * the persistent grid size are picked by timing at creation. */
typedef struct ldg_ensemble ldg_ensemble;
int ldg_ensemble_create(const ldg_config* cfgs, int count, ldg_ensemble** out);
int ldg_ensemble_destroy(ldg_ensemble* e);
/* nsteps RK4 steps of every member (each with its own dt).  An RHS item
 * waits (bounded) for its member's gradient items; a wait that runs out
 * stops the step at a stage boundary with every member's step-start state
 * intact.  By default the step is then re-run member by member with the
 * solo kernels (the same bits) and the call carries on; with recovery off
 * the call returns LDG_ERR_TIMEOUT and the state is that step's start.
 * (The reference has no batched path; its MPI waits block, MPIUtil.cpp.) */
int ldg_ensemble_step(ldg_ensemble* e, int nsteps);
/* The bounded wait's limit in polls of ~100 ns (default 2^22, about half a
 * second; 0 gives up as soon as a gradient item is still running) and
 * whether a step that gave up is re-run member by member (recover != 0,
 * the default) or reported as LDG_ERR_TIMEOUT. */
int ldg_ensemble_set_wait_limit(ldg_ensemble* e, long long polls, int recover);
/* Steps re-run member by member so far. */
int ldg_ensemble_recovered_steps(const ldg_ensemble* e, long long* steps);
/* Test hook, host-side fault injection: on != 0 raises member's
 * gradient-item target by one, so that its RHS items wait for an item that
 * never comes and their waits run out; on = 0 restores it. */
int ldg_ensemble_inject_stall(ldg_ensemble* e, int member, int on);
/* A member's state in the reference layout (host or device pointer). */
int ldg_ensemble_get_state(ldg_ensemble* e, int member, double* u, int where);
/* A member's computeKE series, one entry per step. */
int ldg_ensemble_ke_history(ldg_ensemble* e, int member, double* ke, int max, int* count);
int ldg_ensemble_member_info(const ldg_ensemble* e, int member, ldg_info* info);
/* The autotuner's choice and its timings: stage_ms[tile*4 + g] for tiles
 * {128, 256 threads} x grids {1, 2, 4, 8} x SM count. */
int ldg_ensemble_tuning(const ldg_ensemble* e, int* threads_per_cta, int* persistent_ctas, float* stage_ms,
                        int max);
void* ldg_ensemble_stream(ldg_ensemble* e);

/* ---- Learned closure.  No reference counterpart.  A per-element MLP
 * (features: the coarse element's 5 conserved variables and 15 gradient
 * components at its (p+1)^3 Gauss points; two hidden GELU layers; output:
 * a 5 x (p+1)^3 RHS correction) trained on the GPU by the library's own
 * BF16 tensor-core kernels (FP32 accumulation, FP32 master weights, Adam)
 * to map a coarse solver's RHS onto the L2 projection of a fine FP64
 * solver's RHS.  Attached to a coarse FP64 solver, every RK stage adds the
 * correction before the update; detached (or for an element whose
 * prediction is not finite) the plain LDG operator is used. */
typedef struct ldg_closure ldg_closure;
int ldg_closure_create(int p_coarse, int hidden, unsigned long long seed, int device, ldg_closure** out);
int ldg_closure_destroy(ldg_closure* c);
/* One training sample per coarse element from the fine solver's current
 * state: the fine state and RHS L2-projected onto the coarse mesh (the fine
 * mesh must refine the coarse one uniformly, same domain), the coarse
 * gradient and RHS of the projected state.  Both solvers FP64. */
int ldg_closure_add_samples(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse);
/* Solver in the loop.  ldg_closure_project_state makes the L2 projection of
 * the fine solver's state the coarse solver's state (no samples).
 * ldg_closure_add_samples_coarse then takes one sample per coarse element
 * with the coarse solver's own current state and gradient as features and
 * P(K_f) - K_c(u_c) as target: after the coarse solver has run on its own
 * from the projection, these are the states it produces itself, which is
 * what an attached closure sees. */
int ldg_closure_project_state(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse);
int ldg_closure_add_samples_coarse(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse);
int ldg_closure_sample_count(const ldg_closure* c, long long* count);
/* Per-channel normalisation statistics from samples [first, first+count). */
int ldg_closure_finalize_data(ldg_closure* c, long long first, long long count);
/* iters Adam steps on random batches from samples [first, first+count);
 * losses[i] (optional) receives the normalised MSE of step i. */
int ldg_closure_train(ldg_closure* c, long long first, long long count, int iters, int batch, float lr,
                      unsigned long long seed, float* losses);
/* Mean squared RHS error (in units of the target's channel deviation) on
 * samples [first, first+count): of the plain coarse operator and with the
 * closure. */
int ldg_closure_evaluate(ldg_closure* c, long long first, long long count, double* err_plain, double* err_closure);
int ldg_closure_param_count(const ldg_closure* c, long long* count);
int ldg_closure_get_params(ldg_closure* c, float* out);
/* Sets the parameters (layout of ldg_closure_get_params) and restarts the
 * optimiser (Adam moments and step count). */
int ldg_closure_set_params(ldg_closure* c, const float* in);
/* mean[20], std[20] of the input channels, mean[5], std[5] of the outputs */
int ldg_closure_get_stats(ldg_closure* c, float* out50);
/* Raw network on normalised host batches: y = MLP(x), and the parameter
 * gradient of sum(y * dy) (layout of ldg_closure_get_params). */
int ldg_closure_mlp_forward(ldg_closure* c, const float* x, float* y, int batch);
int ldg_closure_mlp_backward(ldg_closure* c, const float* x, const float* dy, int batch, float* grad);
/* Raw samples [first, first+count): features (count x 20 (p+1)^3) and
 * targets (count x 5 (p+1)^3) as float; either pointer may be NULL. */
int ldg_closure_get_samples(ldg_closure* c, long long first, long long count, float* X, float* Y);
/* Element-stage corrections dropped so far (features outside the
 * training range, |x| > ood_sigma training standard deviations, or a non-finite
 * prediction: the element keeps the plain LDG operator). */
int ldg_closure_fallbacks(ldg_closure* c, long long* count);
/* The same count, and the element-stage corrections whose kinetic-energy
 * raising component was removed (energy-stable projection). */
int ldg_closure_counters(ldg_closure* c, long long* fallbacks, long long* clipped);
/* Training and inference options.
 *   input_noise  standard deviation of Gaussian noise added to the
 *                normalised features of every training batch (0: none)
 *   energy       what the attached correction may do to an element's
 *                kinetic energy: LDG_CLOSURE_ENERGY_NONE (no constraint),
 *                _DISSIPATIVE (its KE-raising component is removed; the
 *                default), _NEUTRAL (its KE production is removed)
 *   scale        factor on the correction before the projection (1)
 *   ood_sigma    elements with a normalised feature beyond this many
 *                training standard deviations keep the plain LDG RHS (10)
 *   lr_final     cosine decay of the learning rate from lr to
 *                lr * lr_final over a training call (1: constant) */
#define LDG_CLOSURE_ENERGY_NONE 0
#define LDG_CLOSURE_ENERGY_DISSIPATIVE 1
#define LDG_CLOSURE_ENERGY_NEUTRAL 2
typedef struct ldg_closure_options {
  float input_noise;
  int energy;
  float scale;
  float ood_sigma;
  float lr_final;
  int reserved[3];
} ldg_closure_options;
int ldg_closure_get_options(const ldg_closure* c, ldg_closure_options* o);
int ldg_closure_set_options(ldg_closure* c, const ldg_closure_options* o);
/* Attach (c) or detach (NULL) a closure on a coarse FP64 solver: every RK
 * stage of ldg_step, and ldg_rhs, then add the closure's correction. */
int ldg_solver_attach_closure(ldg_solver* s, ldg_closure* c);

/* RHS evaluation without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot let the library allocate
 * device memory -- an application whose memory is owned by its own arena or
 * by another framework's caching allocator, or a real-time loop in which a
 * cudaMalloc (which may synchronise the device and can fail under
 * fragmentation) is not allowed.  Such callers cannot use ldg_create, which
 * allocates the solver's buffers.
 *
 * Computes k = rhs(u) in FP64 like ldg_rhs for the mesh and physics in cfg
 * (cfg->precision must be LDG_FP64: LDG_MIXED_F32X2 returns
 * LDG_ERR_UNSUPPORTED, any other value LDG_ERR_INVALID), with u
 * and k DEVICE pointers in the reference layout (dofs, 5, nElements) on
 * device cfg->device; work is enqueued on `stream` (a cudaStream_t; NULL =
 * the legacy default stream) and the call returns without synchronising.
 * Intermediate buffers live in one fixed file-scope device array of
 * LDG_NOALLOC_SCRATCH_BYTES (64 MiB), which every GPU that loads the
 * library holds until the process exits.  A mesh whose buffers need more
 * (nElements * (20 (p+1)^3 + 90 (p+1)^2) * 8 bytes, i.e. about 1760
 * elements at p=4, 3080 at p=3, 6210 at p=2) is rejected with LDG_ERR_INVALID.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  All calls share the array and it keeps the
 * last call's contents (every part is overwritten before it is read), so
 * calls whose GPU work overlaps race: order them on one stream. */
#define LDG_NOALLOC_SCRATCH_BYTES (64ull << 20)
int ldg_rhs_noalloc(const ldg_config* cfg, const double* u_dev, double* k_dev, void* stream);

const char* ldg_error_string(int status);
const char* ldg_last_error_message(void);
int ldg_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LDG_H */
