// C-ABI implementation (include/ldg.h): solver handle, device buffers,
// stage orchestration of the FP64 LDG right-hand side.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <algorithm>
#include <vector>

#include "../../include/ldg.h"
#include "ldg_kernels.cuh"
#include "ldg_ops.hpp"
#include "ldg_tc.cuh"
#include "ldg_problem.hpp"
#include "ldg_closure.hpp"
#include "ldg_io.hpp"

using namespace ldg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define LDG_CUDA(call)                                                             \
  do {                                                                             \
    cudaError_t err_ = (call);                                                     \
    if (err_ != cudaSuccess)                                                       \
      return fail(LDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_)); \
  } while (0)

// Classical RK4 tableau (solver.cpp:298-315).
const double kRkB[4] = {1 / 6.0, 1 / 3.0, 1 / 3.0, 1 / 6.0};
const double kRkA[3] = {0.5, 0.5, 1.0};

}  // namespace

namespace ldg {
// Lets other translation units of the library report through
// ldg_last_error_message().
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace ldg

struct ldg_solver {
  ldg_config cfg;
  int N = 0, n = 0, nf = 0, nE = 0;
  double dt = 0, tf = 0;
  long long timesteps = 0, step = 0;
  DevOps ops;
  OpsT<double> o64;  // arithmetic constants of the FP64 path
  OpsT<dd> odd;      // ... of the FP32-pair (mixed) path
  bool mixed = false;
  ldg_closure* closure = nullptr;  // learned RHS correction (FP64 path), or none
  double* Kadd = nullptr;          // its per-stage output
  Ops1D o1;
  double xi[kMaxN];  // CGL nodes as the reference computes them
  double lo[3], hi[3];
  double p0 = 0, T0 = 0, R = 8.314, rho0 = 1.0, V0 = 1.0;
  cudaStream_t stream = nullptr;
  // host <-> device state transfers: a copy stream and per-chunk events,
  // made on first use (kMaxXferChunks + 1 events)
  cudaStream_t xfer = nullptr;
  std::vector<cudaEvent_t> xev;
  int xfer_chunks = 8;  // ldg_set_transfer_chunks
  // device buffers
  double *Un = nullptr, *Uacc = nullptr, *Us = nullptr, *Q = nullptr, *Tq = nullptr, *Fm = nullptr;
  double* Tu[2] = {nullptr, nullptr};
  double *nodal = nullptr, *diag = nullptr, *ens = nullptr, *ke_dev = nullptr, *red = nullptr;
  int* flag = nullptr;
  int cur = 0;  // Tu[cur] holds the traces of Un
  long long ke_cap = 0;
  size_t bytes = 0;
  // optional per-kernel event timing
  bool timing = false;
  std::vector<cudaEvent_t> ev;       // event pool, pairs per launch
  std::vector<int> ev_class;         // class per pair
  size_t ev_used = 0;
  double kt_ms[LDG_KERNEL_CLASSES] = {0, 0, 0};
  long long kt_n[LDG_KERNEL_CLASSES] = {0, 0, 0};
  // snapshot cadence of ldg_time_step (ldg_set_snapshots)
  std::string snap_file;
  int snap_every = 0;
};

namespace {

// ---------------------------------------------------------------- kernels
// Taylor-Green vortex at the CGL nodes (solver.cpp:194-236; node
// coordinates mesh.cpp:127-151, 389-408), reference layout.
struct IcArgs {
  double xi[kMaxN];
  double lo[3], hi[3];
  double p0, rho0, V0, R, T0, gamma, L;
  double amp;            // perturbation amplitude * V0 / 12 (0: none)
  double phi[3][4][3];   // phases [component][wavenumber-1][direction]
  int N, nx, ny, nz;
};

__global__ void k_taylor_green(double* __restrict__ u, long total, const __grid_constant__ IcArgs a) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int N = a.N, n = N * N * N;
  const long k = i / n;
  const int v = (int)(i - k * n);
  const int ix = (int)(k % a.nx), iy = (int)((k / a.nx) % a.ny), iz = (int)(k / ((long)a.nx * a.ny));
  const int c0 = v % N, c1 = (v / N) % N, c2 = v / (N * N);
  double x0 = ix * (a.hi[0] - a.lo[0]) / a.nx + a.lo[0], x1 = (ix + 1) * (a.hi[0] - a.lo[0]) / a.nx + a.lo[0];
  double y0 = iy * (a.hi[1] - a.lo[1]) / a.ny + a.lo[1], y1 = (iy + 1) * (a.hi[1] - a.lo[1]) / a.ny + a.lo[1];
  double z0 = iz * (a.hi[2] - a.lo[2]) / a.nz + a.lo[2], z1 = (iz + 1) * (a.hi[2] - a.lo[2]) / a.nz + a.lo[2];
  double x = x0 + .5 * (a.xi[c0] + 1.0) * (x1 - x0);
  double y = y0 + .5 * (a.xi[c1] + 1.0) * (y1 - y0);
  double z = z0 + .5 * (a.xi[c2] + 1.0) * (z1 - z0);
  double L = a.L;
  double pr = a.p0 + (a.rho0 * a.V0 * a.V0 / 16.0) * (cos(2 * x / L) + cos(2 * y / L)) * (cos(2 * z / L) + 2);
  double r = pr / (a.R * a.T0);
  double mx = a.rho0 * a.V0 * sin(x / L) * cos(y / L) * cos(z / L);
  double my = -a.rho0 * a.V0 * cos(x / L) * sin(y / L) * cos(z / L);
  double mz = 0 * a.rho0;
  if (a.amp != 0.0) {
    const double X[3] = {x / L, y / L, z / L};
    double dv[3] = {0, 0, 0};
    for (int cpt = 0; cpt < 3; ++cpt)
      for (int k = 1; k <= 4; ++k)
        for (int d = 0; d < 3; ++d) dv[cpt] += sin(k * X[d] + a.phi[cpt][k - 1][d]);
    mx += a.rho0 * a.amp * dv[0];
    my += a.rho0 * a.amp * dv[1];
    mz += a.rho0 * a.amp * dv[2];
  }
  double* uk = u + k * 5 * n;
  uk[v] = r;
  uk[v + n] = mx;
  uk[v + 2 * n] = my;
  uk[v + 3 * n] = mz;
  uk[v + 4 * n] = pr / (a.gamma - 1) + (mx * mx + my * my + mz * mz) / (2.0 * r);
}

// SplitMix64 (Steele, Lea & Flood, OOPSLA 2014): counter-based stream.
unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Phases of the seeded velocity perturbation, 2 pi U[0,1) per
// (component, wavenumber, direction).
void perturbation_phases(unsigned long long seed, int instance, double phi[3][4][3]) {
  const unsigned long long base = splitmix64(seed ^ splitmix64(0x4C44470000000000ULL + (unsigned)instance));
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) {
        unsigned long long r = splitmix64(base + (unsigned long long)(c * 16 + k * 4 + d));
        phi[c][k][d] = 2.0 * M_PI * (double)(r >> 11) * (1.0 / 9007199254740992.0);
      }
}

// Deterministic single-CTA sum: out[0] = scale * sum_i x[i*stride + off].
// Fixed per-thread order with Neumaier compensation, fixed tree.
__global__ void k_reduce(const double* __restrict__ x, long count, int stride, int off, double scale,
                         double* __restrict__ out) {
  __shared__ double ss[1024];
  __shared__ double sc[1024];
  double s = 0.0, c = 0.0;
  for (long i = threadIdx.x; i < count; i += blockDim.x) {
    double v = x[i * stride + off];
    double t = s + v;
    c += fabs(s) >= fabs(v) ? (s - t) + v : (v - t) + s;
    s = t;
  }
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      double a = ss[threadIdx.x], b = ss[threadIdx.x + h];
      double t = a + b;
      double e = fabs(a) >= fabs(b) ? (a - t) + b : (b - t) + a;
      ss[threadIdx.x] = t;
      sc[threadIdx.x] += sc[threadIdx.x + h] + e;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = scale * (ss[0] + sc[0]);
}

// --------------------------------------------------------------- dispatch
template <int N>
size_t smem_transform(int nv) { return sizeof(double) * 2 * Cfg<N>::EPC * nv * Cfg<N>::n; }
template <int N>
size_t smem_traces() { return sizeof(double) * Cfg<N>::EPC * kNS * Cfg<N>::n; }
template <int N>
size_t smem_grad() {
  return sizeof(double) * Cfg<N>::EPC * grad_smem_values_per_element<N>();
}
template <int N>
size_t smem_rhs() {
  return sizeof(double) * Cfg<N>::EPC * (kNQ * Cfg<N>::n + 6 * kNS * Cfg<N>::nf);
}

template <int N>
size_t smem_ke() { return sizeof(double) * Cfg<N>::EPC * 13 * Cfg<N>::n; }

template <int N>
int grid_for(int nE) {
  return (nE + Cfg<N>::EPC - 1) / Cfg<N>::EPC;
}

template <int N, class T>
cudaError_t set_attrs_t() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_traces<N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_traces<N>())) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_grad<N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_grad<N>())) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(k_rhs<N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rhs<N>());
}

template <int N>
cudaError_t set_attrs() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_transform<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_transform<N>(kNS))) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_ke<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_ke<N>())) != cudaSuccess)
    return e;
  if ((e = set_attrs_t<N, double>()) != cudaSuccess) return e;
  if ((e = set_attrs_t<N, dd>()) != cudaSuccess) return e;
  done = true;
  return cudaSuccess;
}

// Type-erased stage call: pointers to S-typed buffers are void*.
struct StageCall {
  const void* Us = nullptr;
  const void* Q = nullptr;
  const void* Tu = nullptr;
  const void* Tq = nullptr;
  const void* Fm = nullptr;
  const double* Un = nullptr;
  double* Uacc = nullptr;
  void* Unext = nullptr;
  void* Tu_out = nullptr;
  double* Kout = nullptr;
  const double* Kadd = nullptr;
  double* diag = nullptr;
  int* flag = nullptr;
  double cacc = 0, cnext = 0;
  int stage = -1;
};

template <int N>
cudaError_t launch_transform(const double* in, double* out, int nE, const DevOps& ops, int inverse,
                             cudaStream_t st) {
  k_transform<N><<<grid_for<N>(nE), Cfg<N>::T, smem_transform<N>(kNS), st>>>(in, out, nE, kNS, ops, inverse);
  return cudaGetLastError();
}
template <int N, class T>
cudaError_t launch_traces(const double* U, void* Ucopy, void* Tu, int nE, const OpsT<T>& o, cudaStream_t st) {
  using S = typename Real<T>::S;
  k_traces<N, T><<<grid_for<N>(nE), Cfg<N>::T, smem_traces<N>(), st>>>(U, (S*)Ucopy, (S*)Tu, nE, o);
  return cudaGetLastError();
}
template <int N, class T>
cudaError_t launch_grad(const void* U, const void* Tu, void* Q, void* Tq, void* Fm, double* ens,
                        const DevOps& ops, const OpsT<T>& o, cudaStream_t st, int ebase = 0, int eend = -1) {
  using S = typename Real<T>::S;
  if (eend < 0) eend = ops.nE;
  k_grad<N, T><<<grid_for<N>(eend - ebase), Cfg<N>::T, smem_grad<N>(), st>>>(
      (const S*)U, (const S*)Tu, (S*)Q, (S*)Tq, (S*)Fm, ens, ops, o, ebase, eend);
  return cudaGetLastError();
}
template <int N, class T>
cudaError_t launch_rhs(const StageCall& c, const DevOps& ops, const OpsT<T>& o, cudaStream_t st, int ebase = 0,
                       int eend = -1) {
  using S = typename Real<T>::S;
  StageArgs<T> a{};
  a.Us = (const S*)c.Us;
  a.Q = (const S*)c.Q;
  a.Tu = (const S*)c.Tu;
  a.Tq = (const S*)c.Tq;
  a.Fm = (const S*)c.Fm;
  a.Un = c.Un;
  a.Uacc = c.Uacc;
  a.Unext = (S*)c.Unext;
  a.Tu_out = (S*)c.Tu_out;
  a.Kout = c.Kout;
  a.Kadd = c.Kadd;
  a.diag = c.diag;
  a.flag = c.flag;
  a.cacc = c.cacc;
  a.cnext = c.cnext;
  a.stage = c.stage;
  if (eend < 0) eend = ops.nE;
  k_rhs<N, T><<<grid_for<N>(eend - ebase), Cfg<N>::T, smem_rhs<N>(), st>>>(a, ops, o, ebase, eend);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_ke(const double* U, double* diag, const DevOps& ops, cudaStream_t st) {
  k_ke<N><<<grid_for<N>(ops.nE), Cfg<N>::T, smem_ke<N>(), st>>>(U, diag, ops);
  return cudaGetLastError();
}

#define LDG_DISPATCH(Nv, expr)               \
  switch (Nv) {                              \
    case 2: { constexpr int NN = 2; return expr; } \
    case 3: { constexpr int NN = 3; return expr; } \
    case 4: { constexpr int NN = 4; return expr; } \
    case 5: { constexpr int NN = 5; return expr; } \
    case 6: { constexpr int NN = 6; return expr; } \
    case 7: { constexpr int NN = 7; return expr; } \
    default: return cudaErrorInvalidValue;   \
  }

cudaError_t d_attrs(int N) { LDG_DISPATCH(N, set_attrs<NN>()); }
cudaError_t d_transform(int N, const double* in, double* out, int nE, const DevOps& ops, int inv, cudaStream_t st) {
  LDG_DISPATCH(N, launch_transform<NN>(in, out, nE, ops, inv, st));
}
cudaError_t d_ke(int N, const double* U, double* diag, const DevOps& ops, cudaStream_t st) {
  LDG_DISPATCH(N, launch_ke<NN>(U, diag, ops, st));
}

// ---------------------------------------------------------------- helpers
void free_all(ldg_solver* s) {
  double* bufs[] = {s->Un, s->Uacc, s->Us, s->Q, s->Tq, s->Fm, s->Tu[0], s->Tu[1], s->nodal, s->diag, s->ens, s->ke_dev, s->red};
  for (double* b : bufs)
    if (b) cudaFree(b);
  if (s->flag) cudaFree(s->flag);
  if (s->Kadd) cudaFree(s->Kadd);
  for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
  s->ev.clear();
  for (cudaEvent_t e : s->xev) cudaEventDestroy(e);
  s->xev.clear();
  if (s->xfer) cudaStreamDestroy(s->xfer);
  if (s->stream) cudaStreamDestroy(s->stream);
}

int dmalloc(ldg_solver* s, double** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(double));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(LDG_ERR_NOMEM, "cudaMalloc of " + std::to_string(count * sizeof(double)) + " bytes: " +
                                   cudaGetErrorString(e));
  }
  s->bytes += count * sizeof(double);
  return LDG_OK;
}

size_t state_count(const ldg_solver* s) { return (size_t)s->nE * kNS * s->n; }

// Event bracketing of launches (only when timing is enabled).
cudaError_t tic(ldg_solver* s, int cls) {
  if (!s->timing) return cudaSuccess;
  if (s->ev_used + 2 > s->ev.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      cudaError_t err = cudaEventCreate(&e);
      if (err != cudaSuccess) return err;
      s->ev.push_back(e);
    }
  }
  s->ev_class.push_back(cls);
  return cudaEventRecord(s->ev[s->ev_used], s->stream);
}
cudaError_t toc(ldg_solver* s) {
  if (!s->timing) return cudaSuccess;
  cudaError_t e = cudaEventRecord(s->ev[s->ev_used + 1], s->stream);
  s->ev_used += 2;
  return e;
}
cudaError_t harvest_times(ldg_solver* s) {
  if (s->ev_used == 0) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return e;
  for (size_t i = 0; i < s->ev_used / 2; ++i) {
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, s->ev[2 * i], s->ev[2 * i + 1]);
    if (e != cudaSuccess) return e;
    s->kt_ms[s->ev_class[i]] += ms;
    s->kt_n[s->ev_class[i]] += 1;
  }
  s->ev_used = 0;
  s->ev_class.clear();
  return cudaSuccess;
}

// FP64 FMA throughput probe: 16 independent FMA chains per thread (enough
// to cover the FMA latency at full occupancy), the loop unrolled so that
// its counter and branch are a small share of the issue slots.  Thread 0
// of each block records the block's SM cycle count (clock64), which gives
// the FMA rate per SM per clock independently of the clock frequency.
__global__ void __launch_bounds__(256) k_fp64_chain(double* out, long long* cycles, int* smid, int iters) {
  double a[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = threadIdx.x * 1e-9 + k * 1e-9;
  const double m = 0.999999999, c = 1e-12;
  __syncthreads();
  const long long t0 = clock64();
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = fma(a[k], m, c);
  }
  __syncthreads();
  const long long t1 = clock64();
  double r = 0.0;
#pragma unroll
  for (int k = 0; k < 16; ++k) r += a[k];
  if (r == 1234.5) out[0] = r;  // keeps the chains live; never true
  if (threadIdx.x == 0) {
    unsigned sm;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
    cycles[blockIdx.x] = t1 - t0;
    smid[blockIdx.x] = (int)sm;
  }
}

// The flux kernels' FP64 reciprocal and reciprocal square root on n
// operands (ldg_probe_recip).
__global__ void k_recip(const double* __restrict__ x, double* __restrict__ r, double* __restrict__ rs, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    r[i] = rcp(x[i]);
    rs[i] = rsqrt_(x[i]);
  }
}

// Stage kernels in the solver's arithmetic (mixed: FP32 pairs) or FP64.
cudaError_t s_traces(ldg_solver* s, bool mixed, const double* U, void* Ucopy, void* Tu) {
  if (mixed) LDG_DISPATCH(s->N, (launch_traces<NN, dd>(U, Ucopy, Tu, s->nE, s->odd, s->stream)));
  LDG_DISPATCH(s->N, (launch_traces<NN, double>(U, Ucopy, Tu, s->nE, s->o64, s->stream)));
}
// Elements [ebase, eend) (eend < 0: all).
cudaError_t s_grad(ldg_solver* s, bool mixed, const void* U, const void* Tu, double* ens, int ebase = 0,
                   int eend = -1) {
  if (mixed)
    LDG_DISPATCH(s->N, (launch_grad<NN, dd>(U, Tu, s->Q, s->Tq, s->Fm, ens, s->ops, s->odd, s->stream, ebase, eend)));
  LDG_DISPATCH(s->N,
               (launch_grad<NN, double>(U, Tu, s->Q, s->Tq, s->Fm, ens, s->ops, s->o64, s->stream, ebase, eend)));
}
cudaError_t s_rhs(ldg_solver* s, bool mixed, const StageCall& c, int ebase = 0, int eend = -1) {
  if (mixed) LDG_DISPATCH(s->N, (launch_rhs<NN, dd>(c, s->ops, s->odd, s->stream, ebase, eend)));
  LDG_DISPATCH(s->N, (launch_rhs<NN, double>(c, s->ops, s->o64, s->stream, ebase, eend)));
}

// nodal (reference layout, in s->nodal) -> Un and the traces of Un; on the
// mixed path also the FP32-pair copy of Un in Us (the stage-0 input).
// Traces of elements [e0, e0+ne) only (each element's traces depend on its
// own values alone).
cudaError_t s_traces_range(ldg_solver* s, bool mixed, const double* U, void* Ucopy, double* Tu, int e0, int ne) {
  const long per = (long)kNS * s->n, tper = 6L * kNS * s->nf;
  double* uc = Ucopy ? static_cast<double*>(Ucopy) + e0 * per : nullptr;  // 8-byte values either way
  if (mixed) LDG_DISPATCH(s->N, (launch_traces<NN, dd>(U + e0 * per, uc, Tu + e0 * tper, ne, s->odd, s->stream)));
  LDG_DISPATCH(s->N, (launch_traces<NN, double>(U + e0 * per, uc, Tu + e0 * tper, ne, s->o64, s->stream)));
}

// Host <-> device state transfers are cut into s->xfer_chunks element
// ranges: the copy of one chunk (on the copy stream) overlaps the basis
// transform and traces of the previous one (on the solver's stream).
constexpr int kMaxXferChunks = 64;

int ensure_xfer(ldg_solver* s) {
  if (s->xfer) return LDG_OK;
  LDG_CUDA(cudaStreamCreateWithFlags(&s->xfer, cudaStreamNonBlocking));
  s->xev.assign(kMaxXferChunks + 1, nullptr);
  for (auto& e : s->xev) LDG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return LDG_OK;
}

void chunk_range(int nE, int chunks, int c, int* e0, int* e1) {
  *e0 = (int)((long)nE * c / chunks);
  *e1 = (int)((long)nE * (c + 1) / chunks);
}

// A state in the reference layout (host or device) -> its Gauss values in U
// on the solver's stream; with Tu also the traces of U (and, on the mixed
// path, the pair copy Ucopy).  Host sources pass through s->nodal.
int upload_gauss(ldg_solver* s, const double* u, int where, double* U, void* Ucopy, double* Tu, bool mixed) {
  if (!u) return fail(LDG_ERR_INVALID, "null state pointer");
  if (where == LDG_DEVICE) {
    LDG_CUDA(d_transform(s->N, u, U, s->nE, s->ops, 0, s->stream));
    if (Tu) LDG_CUDA(s_traces(s, mixed, U, Ucopy, Tu));
    return LDG_OK;
  }
  int st = ensure_xfer(s);
  if (st) return st;
  const long per = (long)kNS * s->n;
  // the copies start after the work already queued, which may read s->nodal
  LDG_CUDA(cudaEventRecord(s->xev[kMaxXferChunks], s->stream));
  LDG_CUDA(cudaStreamWaitEvent(s->xfer, s->xev[kMaxXferChunks], 0));
  for (int c = 0; c < s->xfer_chunks; ++c) {
    int e0, e1;
    chunk_range(s->nE, s->xfer_chunks, c, &e0, &e1);
    if (e1 == e0) continue;
    LDG_CUDA(cudaMemcpyAsync(s->nodal + e0 * per, u + e0 * per, (size_t)(e1 - e0) * per * sizeof(double),
                             cudaMemcpyHostToDevice, s->xfer));
    LDG_CUDA(cudaEventRecord(s->xev[c], s->xfer));
    LDG_CUDA(cudaStreamWaitEvent(s->stream, s->xev[c], 0));
    LDG_CUDA(d_transform(s->N, s->nodal + e0 * per, U + e0 * per, e1 - e0, s->ops, 0, s->stream));
    if (Tu) LDG_CUDA(s_traces_range(s, mixed, U, Ucopy, Tu, e0, e1 - e0));
  }
  return LDG_OK;
}

// Gauss values U -> the reference layout in u (host or device).  Host
// outputs pass through s->nodal; the call returns once they are on the host.
int download_gauss(ldg_solver* s, const double* U, double* u, int where) {
  if (!u) return fail(LDG_ERR_INVALID, "null output pointer");
  if (where == LDG_DEVICE) {
    LDG_CUDA(d_transform(s->N, U, u, s->nE, s->ops, 1, s->stream));
    return LDG_OK;
  }
  int st = ensure_xfer(s);
  if (st) return st;
  const long per = (long)kNS * s->n;
  for (int c = 0; c < s->xfer_chunks; ++c) {
    int e0, e1;
    chunk_range(s->nE, s->xfer_chunks, c, &e0, &e1);
    if (e1 == e0) continue;
    LDG_CUDA(d_transform(s->N, U + e0 * per, s->nodal + e0 * per, e1 - e0, s->ops, 1, s->stream));
    LDG_CUDA(cudaEventRecord(s->xev[c], s->stream));
    LDG_CUDA(cudaStreamWaitEvent(s->xfer, s->xev[c], 0));
    LDG_CUDA(cudaMemcpyAsync(u + e0 * per, s->nodal + e0 * per, (size_t)(e1 - e0) * per * sizeof(double),
                             cudaMemcpyDeviceToHost, s->xfer));
  }
  LDG_CUDA(cudaStreamSynchronize(s->xfer));
  return LDG_OK;
}

int load_state_from_nodal(ldg_solver* s) {
  LDG_CUDA(d_transform(s->N, s->nodal, s->Un, s->nE, s->ops, 0, s->stream));
  LDG_CUDA(s_traces(s, s->mixed, s->Un, s->mixed ? (void*)s->Us : nullptr, s->Tu[s->cur]));
  return LDG_OK;
}

int ensure_ke_capacity(ldg_solver* s, long long need) {
  if (need <= s->ke_cap) return LDG_OK;
  long long cap = s->ke_cap ? s->ke_cap : 1024;
  while (cap < need) cap *= 2;
  double* nb = nullptr;
  LDG_CUDA(cudaMalloc((void**)&nb, cap * sizeof(double)));
  if (s->ke_dev) {
    LDG_CUDA(cudaMemcpyAsync(nb, s->ke_dev, s->ke_cap * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    LDG_CUDA(cudaStreamSynchronize(s->stream));
    cudaFree(s->ke_dev);
    s->bytes -= s->ke_cap * sizeof(double);
  }
  s->ke_dev = nb;
  s->bytes += cap * sizeof(double);
  s->ke_cap = cap;
  return LDG_OK;
}

}  // namespace

namespace ldg {

int setup_problem(const ldg_config& c, Problem* pb, std::string* err) {
  if (c.p < 1 || c.p > 6) return *err = "order p must be 1..6", LDG_ERR_UNSUPPORTED;
  if (c.nx < 3 || c.ny < 3 || c.nz < 3)  // mesh.cpp:102-107
    return *err = "each direction needs at least 3 elements", LDG_ERR_INVALID;
  if (!(c.tf > 0) || !(c.Re > 0) || !(c.Pr > 0) || !(c.gamma > 1) || !(c.Ma > 0) || !(c.cfl > 0) || !(c.L > 0))
    return *err = "physical parameters must be positive (gamma > 1)", LDG_ERR_INVALID;
  if (c.precision != LDG_FP64 && c.precision != LDG_MIXED_F32X2)
    return *err = "precision mode not built", LDG_ERR_UNSUPPORTED;
  if ((long long)c.nx * c.ny * c.nz > 0x7fffffffLL / 8) return *err = "mesh too large", LDG_ERR_INVALID;
  if (!(c.perturb_amp >= 0)) return *err = "perturbation amplitude must be >= 0", LDG_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return *err = "no CUDA device", LDG_ERR_NODEVICE;
  }
  if (c.device < 0 || c.device >= ndev) return *err = "bad device ordinal", LDG_ERR_INVALID;
  pb->cfg = c;
  pb->N = c.p + 1;
  pb->n = pb->N * pb->N * pb->N;
  pb->nf = pb->N * pb->N;
  pb->nE = c.nx * c.ny * c.nz;
  if (!build_ops1d(c.p, &pb->o1)) return *err = "operator setup failed", LDG_ERR_UNSUPPORTED;
  // Domain (driver.cpp:28-31 / Mesh botLeft, topRight) and element sizes
  // (mesh.cpp:149-151).
  double size = M_PI * c.L;
  for (int l = 0; l < 3; ++l) {
    pb->lo[l] = c.use_box ? c.box_lo[l] : -size;
    pb->hi[l] = c.use_box ? c.box_hi[l] : size;
  }
  const int nd[3] = {c.nx, c.ny, c.nz};
  double mind[3];
  for (int l = 0; l < 3; ++l) {
    mind[l] = (pb->hi[l] - pb->lo[l]) / nd[l];
    if (!(mind[l] > 0)) return *err = "empty box", LDG_ERR_INVALID;
  }
  // Physics and time step (solver.cpp:30-52).
  const double c0 = pb->V0 / c.Ma;
  pb->p0 = pb->rho0 * c0 * c0 / c.gamma;
  pb->T0 = pb->p0 / (pb->R * pb->rho0);
  const double maxVel = pb->V0;
  pb->dt = c.cfl * std::min(std::min(mind[0], mind[1]), mind[2]) / (maxVel * (2 * c.p + 1));
  pb->tf = c.tf;
  pb->timesteps = (long long)std::ceil(c.tf / pb->dt);
  if (pb->timesteps < 1) pb->timesteps = 1;
  pb->dt = c.tf / pb->timesteps;
  for (int i = 0; i < kMaxN; ++i) pb->xi[i] = 0.0;
  for (int i = 0; i <= c.p; ++i) pb->xi[i] = std::cos((c.p - i) * M_PI / c.p);  // dgMath.cpp:41
  // Device operator block.
  DevOps& o = pb->ops;
  std::memset(&o, 0, sizeof(o));
  const int N = pb->N;
  for (int i = 0; i < N * N; ++i) {
    o.A[i] = pb->o1.A[i];
    o.B[i] = pb->o1.B[i];
    o.Bi[i] = pb->o1.Bi[i];
  }
  for (int i = 0; i < N; ++i) {
    o.lp[i] = pb->o1.lp[i];
    o.lm[i] = pb->o1.lm[i];
    o.Lp[i] = pb->o1.Lp[i];
    o.Lm[i] = pb->o1.Lm[i];
    o.w[i] = pb->o1.w[i];
  }
  double alpha[3];
  for (int l = 0; l < 3; ++l) {
    alpha[l] = mind[l] / 2.0;  // solver.cpp:144-148
    o.ia[l] = 1.0 / alpha[l];
  }
  o.J = alpha[0] * alpha[1] * alpha[2];
  o.inv_re = 1.0 / c.Re;
  o.gamma = c.gamma;
  o.g1 = (c.gamma == 1.4) ? 0.4 : c.gamma - 1.0;  // the reference's literal 0.4
  o.kappa = c.gamma * (1.0 / c.Pr);
  o.ke_norm = 1.0 / (pb->rho0 * std::pow(2 * M_PI * c.L, 3.0));  // solver.cpp:1031
  o.nx = c.nx;
  o.ny = c.ny;
  o.nz = c.nz;
  o.nE = pb->nE;
  return LDG_OK;
}

cudaError_t launch_initial_condition(const Problem& pb, double* nodal, cudaStream_t st) {
  IcArgs a;
  std::memset(&a, 0, sizeof(a));
  a.amp = pb.cfg.perturb_amp * pb.V0 / 12.0;
  perturbation_phases(pb.cfg.seed, pb.cfg.instance, a.phi);
  for (int i = 0; i < pb.N; ++i) a.xi[i] = pb.xi[i];
  for (int l = 0; l < 3; ++l) {
    a.lo[l] = pb.lo[l];
    a.hi[l] = pb.hi[l];
  }
  a.p0 = pb.p0;
  a.rho0 = pb.rho0;
  a.V0 = pb.V0;
  a.R = pb.R;
  a.T0 = pb.T0;
  a.gamma = pb.cfg.gamma;
  a.L = pb.cfg.L;
  a.N = pb.N;
  a.nx = pb.cfg.nx;
  a.ny = pb.cfg.ny;
  a.nz = pb.cfg.nz;
  const long total = (long)pb.nE * pb.n;
  k_taylor_green<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(nodal, total, a);
  return cudaGetLastError();
}

cudaError_t launch_transform_any(int N, const double* in, double* out, int nE, const DevOps& ops, int inverse,
                                 cudaStream_t st) {
  cudaError_t e = d_attrs(N);
  if (e != cudaSuccess) return e;
  return d_transform(N, in, out, nE, ops, inverse, st);
}

cudaError_t launch_traces_fp64(int N, const double* U, double* Tu, int nE, const OpsT<double>& o,
                               cudaStream_t st) {
  cudaError_t e = d_attrs(N);
  if (e != cudaSuccess) return e;
  LDG_DISPATCH(N, (launch_traces<NN, double>(U, nullptr, Tu, nE, o, st)));
}

cudaError_t launch_grad_fp64(int N, const double* U, const double* Tu, double* Q, double* Tq, double* Fm,
                             const DevOps& ops, const OpsT<double>& o, cudaStream_t st) {
  cudaError_t e = d_attrs(N);
  if (e != cudaSuccess) return e;
  LDG_DISPATCH(N, (launch_grad<NN, double>(U, Tu, Q, Tq, Fm, nullptr, ops, o, st)));
}

cudaError_t launch_rhs_fp64(int N, const StageArgs<double>& a, const DevOps& ops, const OpsT<double>& o,
                            cudaStream_t st) {
  cudaError_t e = d_attrs(N);
  if (e != cudaSuccess) return e;
  StageCall c;
  c.Us = a.Us;
  c.Q = a.Q;
  c.Tu = a.Tu;
  c.Tq = a.Tq;
  c.Fm = a.Fm;
  c.Un = a.Un;
  c.Uacc = a.Uacc;
  c.Unext = a.Unext;
  c.Tu_out = a.Tu_out;
  c.Kout = a.Kout;
  c.Kadd = a.Kadd;
  c.diag = a.diag;
  c.flag = a.flag;
  c.cacc = a.cacc;
  c.cnext = a.cnext;
  c.stage = a.stage;
  LDG_DISPATCH(N, (launch_rhs<NN, double>(c, ops, o, st)));
}

}  // namespace ldg

namespace ldg {

SolverView solver_view(ldg_solver* s) {
  SolverView v;
  v.N = s->N;
  v.n = s->n;
  v.nf = s->nf;
  v.nE = s->nE;
  v.nx = s->cfg.nx;
  v.ny = s->cfg.ny;
  v.nz = s->cfg.nz;
  v.p = s->cfg.p;
  v.ops = &s->ops;
  v.o64 = &s->o64;
  v.stream = s->stream;
  v.device = s->cfg.device;
  v.mixed = s->mixed;
  v.Un = s->Un;
  v.Q = s->Q;
  return v;
}

// K = rhs(U) in the Gauss basis (FP64), U any Gauss-space state of this
// solver's mesh; the solver's state is not touched.  The gradient of U is
// left in s->Q (valid until the next call on s).  Uses the spare trace
// buffer, Tq and Us as scratch.
int solver_rhs_gauss(ldg_solver* s, const double* U, double* K) {
  if (s->mixed) return fail(LDG_ERR_UNSUPPORTED, "closure data needs FP64 solvers");
  double* Tu = s->Tu[1 - s->cur];
  LDG_CUDA(s_traces(s, false, U, nullptr, Tu));
  LDG_CUDA(s_grad(s, false, U, Tu, nullptr));
  StageCall c;
  c.Us = U;
  c.Q = s->Q;
  c.Tu = Tu;
  c.Tq = s->Tq;
  c.Fm = s->Fm;
  c.Kout = K;
  c.stage = -1;
  LDG_CUDA(s_rhs(s, false, c));
  return LDG_OK;
}

// Makes U (Gauss basis) the solver's state.
int solver_set_gauss_state(ldg_solver* s, const double* U) {
  LDG_CUDA(cudaMemcpyAsync(s->Un, U, state_count(s) * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
  LDG_CUDA(s_traces(s, s->mixed, s->Un, s->mixed ? (void*)s->Us : nullptr, s->Tu[s->cur]));
  return LDG_OK;
}

}  // namespace ldg

// ---------------------------------------------------------------- geometry + checkpoints
namespace ldg {

int solver_geometry(const ldg_solver* s, Geometry* g) {
  static_assert(kMaxN <= 8, "Geometry holds 8 reference nodes");
  g->N = s->N;
  g->nx = s->cfg.nx;
  g->ny = s->cfg.ny;
  g->nz = s->cfg.nz;
  for (int l = 0; l < 3; ++l) {
    g->lo[l] = s->lo[l];
    g->hi[l] = s->hi[l];
  }
  for (int i = 0; i < kMaxN; ++i) g->xi[i] = s->xi[i];
  return LDG_OK;
}

}  // namespace ldg

namespace {

// Checkpoint file: this header, then the FP64 Gauss-point state Un
// [nE][5][n], the face traces of Un [nE][6][5][nf] (FP64 on the FP64 path,
// FP32 pairs on the mixed path: 8 bytes per value either way) and the KE
// series [step].  Native byte order.
struct CkptHeader {
  char magic[8];
  uint32_t version, header_bytes;
  ldg_config cfg;
  int64_t step;
  double dt;
  int32_t N, nE, precision, pad;
  int64_t state_bytes, trace_bytes, ke_count;
  uint64_t payload_hash;
};
const char kCkptMagic[8] = {'L', 'D', 'G', 'C', 'K', 'P', 'T', '1'};
const uint64_t kFnvBasis = 14695981039346656037ull;

// 64-bit FNV-1a (Fowler, Noll, Vo).
uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

size_t trace_count(const ldg_solver* s) { return (size_t)s->nE * 6 * kNS * s->nf; }

int read_header(FILE* f, const char* path, CkptHeader* h) {
  if (std::fread(h, sizeof(*h), 1, f) != 1 || std::memcmp(h->magic, kCkptMagic, 8) != 0 || h->version != 1 ||
      h->header_bytes != sizeof(CkptHeader))
    return fail(LDG_ERR_IO, std::string("not a checkpoint of this library: ") + path);
  return LDG_OK;
}

// Fields that define the discretisation and must agree for a resume.
bool same_problem(const ldg_config& a, const ldg_config& b) {
  bool same = a.p == b.p && a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.L == b.L && a.Re == b.Re &&
              a.Pr == b.Pr && a.gamma == b.gamma && a.Ma == b.Ma && a.precision == b.precision &&
              a.use_box == b.use_box;
  if (same && a.use_box)
    for (int l = 0; l < 3; ++l) same = same && a.box_lo[l] == b.box_lo[l] && a.box_hi[l] == b.box_hi[l];
  return same;
}

}  // namespace

extern "C" {

int ldg_solver_attach_closure(ldg_solver* s, ldg_closure* c) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  if (!c) {  // detach: the plain LDG operator
    s->closure = nullptr;
    return LDG_OK;
  }
  if (s->mixed) return fail(LDG_ERR_UNSUPPORTED, "the closure corrects FP64 solvers");
  int st = closure_check_solver(c, solver_view(s));
  if (st) return st;
  if (!s->Kadd) {
    double* p = nullptr;
    if ((st = dmalloc(s, &p, state_count(s)))) return st;
    s->Kadd = p;
  }
  s->closure = c;
  return LDG_OK;
}

}  // extern "C"

extern "C" {

int ldg_abi_version(void) { return LDG_ABI_VERSION; }

const char* ldg_error_string(int status) {
  switch (status) {
    case LDG_OK: return "LDG_OK";
    case LDG_ERR_INVALID: return "LDG_ERR_INVALID";
    case LDG_ERR_CUDA: return "LDG_ERR_CUDA";
    case LDG_ERR_NOMEM: return "LDG_ERR_NOMEM";
    case LDG_ERR_NONFINITE: return "LDG_ERR_NONFINITE";
    case LDG_ERR_UNSUPPORTED: return "LDG_ERR_UNSUPPORTED";
    case LDG_ERR_NODEVICE: return "LDG_ERR_NODEVICE";
    case LDG_ERR_TIMEOUT: return "LDG_ERR_TIMEOUT";
    case LDG_ERR_IO: return "LDG_ERR_IO";
  }
  return "LDG_ERR_UNKNOWN";
}

const char* ldg_last_error_message(void) { return g_last_error.c_str(); }

int ldg_config_default(ldg_config* c) {
  if (!c) return fail(LDG_ERR_INVALID, "null config");
  std::memset(c, 0, sizeof(*c));
  c->p = 2;  // Solver() delegates to p=2, dtSnaps=10, tf=1, L=1 (solver.cpp:4)
  c->nx = c->ny = c->nz = 10;
  c->L = 1.0;
  c->tf = 1.0;
  c->dt_snaps = 10;
  c->Re = 1600.0;
  c->Pr = .71;
  c->gamma = 1.4;
  c->Ma = 0.1;
  c->cfl = 0.01;
  c->precision = LDG_FP64;
  c->device = 0;
  c->check_finite = 1;
  c->use_box = 0;
  return LDG_OK;
}

int ldg_create(const ldg_config* cfg, ldg_solver** out) {
  if (!cfg || !out) return fail(LDG_ERR_INVALID, "null argument");
  *out = nullptr;
  const ldg_config& c = *cfg;
  Problem pb;
  std::string err;
  int pst = setup_problem(c, &pb, &err);
  if (pst != LDG_OK) return fail(pst, err);
  ldg_solver* s = new (std::nothrow) ldg_solver();
  if (!s) return fail(LDG_ERR_NOMEM, "host allocation");
  s->cfg = c;
  s->N = pb.N;
  s->n = pb.n;
  s->nf = pb.nf;
  s->nE = pb.nE;
  s->o1 = pb.o1;
  for (int l = 0; l < 3; ++l) {
    s->lo[l] = pb.lo[l];
    s->hi[l] = pb.hi[l];
  }
  s->p0 = pb.p0;
  s->T0 = pb.T0;
  s->dt = pb.dt;
  s->tf = pb.tf;
  s->timesteps = pb.timesteps;
  for (int i = 0; i < kMaxN; ++i) s->xi[i] = pb.xi[i];
  s->ops = pb.ops;
  const int N = s->N;
  s->o64 = make_opst<double>(s->ops, N);
  s->odd = make_opst<dd>(s->ops, N);
  s->mixed = c.precision == LDG_MIXED_F32X2;

  int st;
  if (cudaSetDevice(c.device) != cudaSuccess) {
    delete s;
    return fail(LDG_ERR_CUDA, "cudaSetDevice");
  }
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return fail(LDG_ERR_CUDA, "cudaStreamCreate");
  }
  const size_t ns = state_count(s);
  const size_t nE = s->nE;
  if ((st = dmalloc(s, &s->Un, ns)) || (st = dmalloc(s, &s->Uacc, ns)) || (st = dmalloc(s, &s->Us, ns)) ||
      (st = dmalloc(s, &s->Q, nE * kNQ * s->n)) || (st = dmalloc(s, &s->Tq, nE * 3 * kNQ * s->nf)) ||
      (st = dmalloc(s, &s->Fm, nE * 3 * kNS * s->nf)) ||
      (st = dmalloc(s, &s->Tu[0], nE * 6 * kNS * s->nf)) || (st = dmalloc(s, &s->Tu[1], nE * 6 * kNS * s->nf)) ||
      (st = dmalloc(s, &s->nodal, ns)) || (st = dmalloc(s, &s->diag, nE * 2)) || (st = dmalloc(s, &s->ens, nE)) ||
      (st = dmalloc(s, &s->red, 8))) {
    free_all(s);
    delete s;
    return st;
  }
  if (cudaMalloc((void**)&s->flag, sizeof(int)) != cudaSuccess) {
    free_all(s);
    delete s;
    return fail(LDG_ERR_NOMEM, "flag");
  }
  cudaError_t ae = d_attrs(N);
  if (ae != cudaSuccess) {
    free_all(s);
    delete s;
    return fail(LDG_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(ae));
  }
  if ((st = ensure_ke_capacity(s, s->timesteps + 1)) || (st = ldg_set_initial_condition(s))) {
    free_all(s);
    delete s;
    return st;
  }
  *out = s;
  return LDG_OK;
}

int ldg_destroy(ldg_solver* s) {
  if (!s) return LDG_OK;
  cudaSetDevice(s->cfg.device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
  return LDG_OK;
}

int ldg_get_info(const ldg_solver* s, ldg_info* info) {
  if (!s || !info) return fail(LDG_ERR_INVALID, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->p = s->cfg.p;
  info->dofs = s->n;
  info->nf = s->nf;
  info->nx = s->cfg.nx;
  info->ny = s->cfg.ny;
  info->nz = s->cfg.nz;
  info->nelements = s->nE;
  info->dt = s->dt;
  info->timesteps = s->timesteps;
  info->step = s->step;
  info->time = s->step * s->dt;
  info->device_bytes = s->bytes;
  info->precision = s->cfg.precision;
  return LDG_OK;
}

int ldg_set_initial_condition(ldg_solver* s) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  Problem pb;
  pb.cfg = s->cfg;
  pb.N = s->N;
  pb.n = s->n;
  pb.nf = s->nf;
  pb.nE = s->nE;
  for (int i = 0; i < kMaxN; ++i) pb.xi[i] = s->xi[i];
  for (int l = 0; l < 3; ++l) {
    pb.lo[l] = s->lo[l];
    pb.hi[l] = s->hi[l];
  }
  pb.p0 = s->p0;
  pb.T0 = s->T0;
  LDG_CUDA(launch_initial_condition(pb, s->nodal, s->stream));
  s->step = 0;
  return load_state_from_nodal(s);
}

int ldg_set_transfer_chunks(ldg_solver* s, int chunks) {
  if (!s || chunks < 1 || chunks > kMaxXferChunks) return fail(LDG_ERR_INVALID, "transfer chunks must be 1..64");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  LDG_CUDA(cudaStreamSynchronize(s->stream));
  if (s->xfer) LDG_CUDA(cudaStreamSynchronize(s->xfer));
  s->xfer_chunks = chunks;
  return LDG_OK;
}

int ldg_set_state(ldg_solver* s, const double* u, int where) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  return upload_gauss(s, u, where, s->Un, s->mixed ? (void*)s->Us : nullptr, s->Tu[s->cur], s->mixed);
}

int ldg_get_state(ldg_solver* s, double* u, int where) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  return download_gauss(s, s->Un, u, where);
}

int ldg_rhs(ldg_solver* s, const double* u_curr, double* k, int where) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  // Work in scratch buffers so the solver state (Un, Us, Tu[cur]) is kept:
  // the FP64 input goes to Uacc, the stage-input pair copy (mixed path) to
  // the nodal buffer.
  double* Tu = s->Tu[1 - s->cur];
  int st = upload_gauss(s, u_curr, where, s->Uacc, s->mixed ? (void*)s->nodal : nullptr, Tu, s->mixed);
  if (st) return st;
  const void* Uin = s->mixed ? (const void*)s->nodal : (const void*)s->Uacc;
  LDG_CUDA(s_grad(s, s->mixed, Uin, Tu, nullptr));
  StageCall c;
  if (s->closure) {  // the RHS the RK stages use: plain LDG plus the learned correction
    st = closure_correction(s->closure, solver_view(s), (const double*)Uin, s->Q, s->Kadd, s->stream);
    if (st) return st;
    c.Kadd = s->Kadd;
  }
  c.Us = Uin;
  c.Q = s->Q;
  c.Tu = Tu;
  c.Tq = s->Tq;
  c.Fm = s->Fm;
  c.Kout = s->Us;  // FP64 RHS in the stage buffer (restored below on the mixed path)
  c.stage = -1;
  LDG_CUDA(s_rhs(s, s->mixed, c));
  if ((st = download_gauss(s, s->Us, k, where))) return st;
  if (s->mixed)  // Us held the pair copy of Un: rebuild it
    LDG_CUDA(s_traces(s, true, s->Un, s->Us, s->Tu[1 - s->cur]));
  return LDG_OK;
}

}  // extern "C"

namespace {

// Plane-aligned chunk c of `chunks` over the elements: whole z-planes
// [nz c / chunks, nz (c+1) / chunks), so that an element's -z neighbour
// lies in its own chunk or the one before (except plane 0's, in the last).
void plane_chunk(const ldg_solver* s, int chunks, int c, int* e0, int* e1) {
  const long P = (long)s->cfg.nx * s->cfg.ny;
  *e0 = (int)(P * ((long)s->cfg.nz * c / chunks));
  *e1 = (int)(P * ((long)s->cfg.nz * (c + 1) / chunks));
}

// The RK4 steps of ldg_step.  first_grad_done: stage 0's gradient pass of
// the first step has run already (ldg_advance_host overlaps it with the
// upload).  u_out (host): the last stage's RHS pass runs in plane chunks and
// each chunk's new state is transformed and copied out on the copy stream
// as soon as it is written; the caller synchronises the copy stream.
int step_loop(ldg_solver* s, int nsteps, bool first_grad_done, double* u_out) {
  const bool mixed = s->mixed;
  const long per = (long)kNS * s->n;
  const int chunks = std::max(1, std::min(s->xfer_chunks, s->cfg.nz));
  for (int it = 0; it < nsteps; ++it) {
    const int cur = s->cur;
    for (int stage = 0; stage < 4; ++stage) {
      // Stage input: the FP64 state on the FP64 path at stage 0, otherwise
      // the stage buffer (on the mixed path it holds the FP32-pair copy).
      const void* Uin = (stage == 0 && !mixed) ? (const void*)s->Un : (const void*)s->Us;
      double* Tu_in = s->Tu[(stage & 1) ? 1 - cur : cur];
      double* Tu_out = s->Tu[(stage & 1) ? cur : 1 - cur];
      if (!(first_grad_done && it == 0 && stage == 0)) {
        LDG_CUDA(tic(s, 0));
        LDG_CUDA(s_grad(s, mixed, Uin, Tu_in, nullptr));
        LDG_CUDA(toc(s));
      }
      if (s->closure) {
        int cst = closure_correction(s->closure, solver_view(s), (const double*)Uin, s->Q, s->Kadd, s->stream);
        if (cst) return cst;
      }
      StageCall c;
      c.Kadd = s->closure ? s->Kadd : nullptr;
      c.Us = Uin;
      c.Q = s->Q;
      c.Tu = Tu_in;
      c.Tq = s->Tq;
      c.Fm = s->Fm;
      c.Un = s->Un;
      c.Uacc = s->Uacc;
      c.Unext = (stage < 3 || mixed) ? (void*)s->Us : nullptr;
      c.Tu_out = Tu_out;
      c.diag = stage == 3 ? s->diag : nullptr;
      c.flag = s->cfg.check_finite ? s->flag : nullptr;
      c.cacc = s->dt * kRkB[stage];
      c.cnext = stage < 3 ? s->dt * kRkA[stage] : 0.0;
      c.stage = stage;
      if (u_out && it == nsteps - 1 && stage == 3) {
        for (int k = 0; k < chunks; ++k) {
          int e0, e1;
          plane_chunk(s, chunks, k, &e0, &e1);
          if (e1 == e0) continue;
          LDG_CUDA(tic(s, 1));
          LDG_CUDA(s_rhs(s, mixed, c, e0, e1));
          LDG_CUDA(toc(s));
          // the chunk's new state (Uacc) in the reference layout, to the host
          LDG_CUDA(d_transform(s->N, s->Uacc + e0 * per, s->nodal + e0 * per, e1 - e0, s->ops, 1, s->stream));
          LDG_CUDA(cudaEventRecord(s->xev[k], s->stream));
          LDG_CUDA(cudaStreamWaitEvent(s->xfer, s->xev[k], 0));
          LDG_CUDA(cudaMemcpyAsync(u_out + e0 * per, s->nodal + e0 * per, (size_t)(e1 - e0) * per * sizeof(double),
                                   cudaMemcpyDeviceToHost, s->xfer));
        }
      } else {
        LDG_CUDA(tic(s, 1));
        LDG_CUDA(s_rhs(s, mixed, c));
        LDG_CUDA(toc(s));
      }
    }
    // After four stages Tu[cur] holds the traces of Uacc = u^{n+1}.
    std::swap(s->Un, s->Uacc);
    // computeKE after the step (solver.cpp:437).
    LDG_CUDA(tic(s, 2));
    k_reduce<<<1, 1024, 0, s->stream>>>(s->diag, s->nE, 2, 0, s->ops.ke_norm, s->ke_dev + s->step);
    LDG_CUDA(cudaGetLastError());
    LDG_CUDA(toc(s));
    s->step += 1;
    if (s->timing && s->ev_used > 4096) LDG_CUDA(harvest_times(s));
  }
  return LDG_OK;
}

int check_finite_flag(ldg_solver* s) {
  if (!s->cfg.check_finite) return LDG_OK;
  int h = 0;
  LDG_CUDA(cudaMemcpyAsync(&h, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  LDG_CUDA(cudaStreamSynchronize(s->stream));
  if (h) return fail(LDG_ERR_NONFINITE, "non-finite value in the state");
  return LDG_OK;
}

}  // namespace

extern "C" {

int ldg_step(ldg_solver* s, int nsteps) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  if (nsteps < 0) return fail(LDG_ERR_INVALID, "negative step count");
  if (nsteps == 0) return LDG_OK;
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  int st = ensure_ke_capacity(s, s->step + nsteps + 1);
  if (st) return st;
  if (s->cfg.check_finite) LDG_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), s->stream));
  if ((st = step_loop(s, nsteps, false, nullptr))) return st;
  return check_finite_flag(s);
}

int ldg_advance_host(ldg_solver* s, const double* u_in, double* u_out, int nsteps) {
  if (!s || !u_in || !u_out) return fail(LDG_ERR_INVALID, "ldg_advance_host: null argument");
  if (nsteps < 1) return fail(LDG_ERR_INVALID, "ldg_advance_host: nsteps must be at least 1");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  int st;
  if (s->closure) {  // the closure needs the whole gradient before any RHS: the plain sequence
    if ((st = ldg_set_state(s, u_in, LDG_HOST)) || (st = ldg_step(s, nsteps))) return st;
    return ldg_get_state(s, u_out, LDG_HOST);
  }
  if ((st = ensure_ke_capacity(s, s->step + nsteps + 1)) || (st = ensure_xfer(s))) return st;
  if (s->cfg.check_finite) LDG_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), s->stream));
  const bool mixed = s->mixed;
  const long per = (long)kNS * s->n;
  const int chunks = std::max(1, std::min(s->xfer_chunks, s->cfg.nz));
  const void* Uin0 = mixed ? (const void*)s->Us : (const void*)s->Un;
  double* Tu0 = s->Tu[s->cur];
  // 1. Upload in plane chunks: copy (copy stream), transform and traces
  //    (solver stream).  Stage 0's gradient pass of chunk c needs the traces
  //    of its -z neighbours, which lie in chunks c-1 and c, so it follows
  //    chunk c's upload; chunk 0's neighbours across the periodic wrap
  //    arrive with the last chunk, so its gradient pass goes last.
  LDG_CUDA(cudaEventRecord(s->xev[kMaxXferChunks], s->stream));
  LDG_CUDA(cudaStreamWaitEvent(s->xfer, s->xev[kMaxXferChunks], 0));
  for (int c = 0; c < chunks; ++c) {
    int e0, e1;
    plane_chunk(s, chunks, c, &e0, &e1);
    if (e1 == e0) continue;
    LDG_CUDA(cudaMemcpyAsync(s->nodal + e0 * per, u_in + e0 * per, (size_t)(e1 - e0) * per * sizeof(double),
                             cudaMemcpyHostToDevice, s->xfer));
    LDG_CUDA(cudaEventRecord(s->xev[c], s->xfer));
    LDG_CUDA(cudaStreamWaitEvent(s->stream, s->xev[c], 0));
    LDG_CUDA(d_transform(s->N, s->nodal + e0 * per, s->Un + e0 * per, e1 - e0, s->ops, 0, s->stream));
    LDG_CUDA(s_traces_range(s, mixed, s->Un, mixed ? (void*)s->Us : nullptr, Tu0, e0, e1 - e0));
    if (c > 0) {
      LDG_CUDA(tic(s, 0));
      LDG_CUDA(s_grad(s, mixed, Uin0, Tu0, nullptr, e0, e1));
      LDG_CUDA(toc(s));
    }
  }
  {
    int e0, e1;
    plane_chunk(s, chunks, 0, &e0, &e1);
    LDG_CUDA(tic(s, 0));
    LDG_CUDA(s_grad(s, mixed, Uin0, Tu0, nullptr, e0, e1));
    LDG_CUDA(toc(s));
  }
  // 2. The steps; the last stage's RHS pass feeds the download chunk by chunk.
  if ((st = step_loop(s, nsteps, true, u_out))) return st;
  LDG_CUDA(cudaStreamSynchronize(s->xfer));
  return check_finite_flag(s);
}

int ldg_time_step(ldg_solver* s) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  const long long every = s->snap_every;
  while (s->step < s->timesteps) {
    long long left = s->timesteps - s->step;
    if (every > 0) {
      // snapshot <file>.<k> before step k*every (solver.cpp:366-381)
      if (s->step % every == 0) {
        int st = ldg_write_xyzv(s, s->snap_file.c_str(), (int)(s->step / every));
        if (st) return st;
      }
      left = std::min(left, every - s->step % every);
    }
    int chunk = (int)std::min<long long>(left, 1 << 20);
    int st = ldg_step(s, chunk);
    if (st) return st;
  }
  return ldg_synchronize(s);
}

int ldg_set_snapshots(ldg_solver* s, const char* filename, int every) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  if (!filename || !*filename || every <= 0) {
    s->snap_file.clear();
    s->snap_every = 0;
    return LDG_OK;
  }
  s->snap_file = filename;
  s->snap_every = every;
  return LDG_OK;
}

int ldg_diagnostics(ldg_solver* s, double* ke_ref, double* ke, double* enstrophy) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  // Enstrophy from the FP64 LDG gradient of the current state (traces
  // rebuilt in FP64 in the spare trace buffer); KE from Un.
  double* Tu = s->Tu[1 - s->cur];
  LDG_CUDA(s_traces(s, false, s->Un, nullptr, Tu));
  LDG_CUDA(s_grad(s, false, s->Un, Tu, s->ens));
  LDG_CUDA(d_ke(s->N, s->Un, s->diag, s->ops, s->stream));
  k_reduce<<<1, 1024, 0, s->stream>>>(s->diag, s->nE, 2, 0, s->ops.ke_norm, s->red + 0);
  k_reduce<<<1, 1024, 0, s->stream>>>(s->diag, s->nE, 2, 1, s->ops.ke_norm, s->red + 1);
  k_reduce<<<1, 1024, 0, s->stream>>>(s->ens, s->nE, 1, 0, s->ops.ke_norm, s->red + 2);
  LDG_CUDA(cudaGetLastError());
  double h[3];
  LDG_CUDA(cudaMemcpyAsync(h, s->red, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  LDG_CUDA(cudaStreamSynchronize(s->stream));
  if (ke_ref) *ke_ref = h[0];
  if (ke) *ke = h[1];
  if (enstrophy) *enstrophy = h[2];
  return LDG_OK;
}

int ldg_ke_history(ldg_solver* s, double* ke, int max, int* count) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  if (count) *count = (int)s->step;
  int m = (int)std::min<long long>(max, s->step);
  if (m > 0 && ke) {
    LDG_CUDA(cudaMemcpyAsync(ke, s->ke_dev, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LDG_CUDA(cudaStreamSynchronize(s->stream));
  }
  return LDG_OK;
}

int ldg_ke_dissipation(ldg_solver* s, double* eps, int max, int* count) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  long long avail = s->step > 2 ? s->step - 2 : 0;
  if (count) *count = (int)avail;
  int m = (int)std::min<long long>(max, avail);
  if (m > 0 && eps) {
    std::vector<double> ke(m + 2);
    int st = ldg_ke_history(s, ke.data(), m + 2, nullptr);
    if (st) return st;
    for (int i = 0; i < m; ++i) eps[i] = -(ke[i + 2] - ke[i]) / (2 * s->dt);  // solver.cpp:438-440
  }
  return LDG_OK;
}

int ldg_synchronize(ldg_solver* s) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(cudaStreamSynchronize(s->stream));
  return LDG_OK;
}

void* ldg_stream(ldg_solver* s) { return s ? (void*)s->stream : nullptr; }

int ldg_enable_kernel_timing(ldg_solver* s, int enable) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(harvest_times(s));
  s->timing = enable != 0;
  return LDG_OK;
}

int ldg_kernel_times(ldg_solver* s, double* ms, long long* launches, int max_classes, int reset) {
  if (!s) return fail(LDG_ERR_INVALID, "null solver");
  LDG_CUDA(harvest_times(s));
  for (int i = 0; i < LDG_KERNEL_CLASSES && i < max_classes; ++i) {
    if (ms) ms[i] = s->kt_ms[i];
    if (launches) launches[i] = s->kt_n[i];
  }
  if (reset)
    for (int i = 0; i < LDG_KERNEL_CLASSES; ++i) {
      s->kt_ms[i] = 0;
      s->kt_n[i] = 0;
    }
  return LDG_OK;
}

int ldg_probe_fp64(int device, double* tflops, double* fma_per_sm_clk, double* sm_mhz) {
  if (!tflops) return fail(LDG_ERR_INVALID, "null output");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(LDG_ERR_NODEVICE, "no CUDA device");
  }
  LDG_CUDA(cudaSetDevice(device));
  int sms = 0;
  LDG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  // exactly one wave: as many 256-thread blocks per SM as fit
  int per_sm = 0;
  LDG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_chain, 256, 0));
  if (per_sm < 1) return fail(LDG_ERR_CUDA, "probe kernel does not fit an SM");
  const int blocks = sms * per_sm, threads = 256, iters = 2048;
  double* out = nullptr;
  long long* cyc = nullptr;
  int* smid = nullptr;
  LDG_CUDA(cudaMalloc((void**)&out, sizeof(double)));
  if (cudaMalloc((void**)&cyc, sizeof(long long) * blocks) != cudaSuccess ||
      cudaMalloc((void**)&smid, sizeof(int) * blocks) != cudaSuccess) {
    cudaFree(out);
    cudaFree(cyc);
    return fail(LDG_ERR_NOMEM, "probe buffer");
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_chain<<<blocks, threads>>>(out, cyc, smid, iters);  // warm-up
  cudaEventRecord(e0);
  k_fp64_chain<<<blocks, threads>>>(out, cyc, smid, iters);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
  std::vector<long long> hc(blocks);
  std::vector<int> hs(blocks);
  if (err == cudaSuccess) err = cudaMemcpy(hc.data(), cyc, sizeof(long long) * blocks, cudaMemcpyDeviceToHost);
  if (err == cudaSuccess) err = cudaMemcpy(hs.data(), smid, sizeof(int) * blocks, cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaFree(cyc);
  cudaFree(smid);
  if (err != cudaSuccess) return fail(LDG_ERR_CUDA, cudaGetErrorString(err));
  const double fmas_per_block = 16.0 * iters * threads;
  *tflops = 2.0 * fmas_per_block * blocks / (ms * 1e-3) / 1e12;
  // Per SM: the FMAs of the blocks it ran over the longest of their spans
  // (one wave, so they ran side by side); the median over SMs.
  std::vector<long long> span(1024, 0);
  std::vector<int> count(1024, 0);
  long long mx = 1;
  for (int b = 0; b < blocks; ++b) {
    const int id = hs[b] & 1023;
    span[id] = std::max(span[id], hc[b]);
    count[id] += 1;
    mx = std::max(mx, hc[b]);
  }
  std::vector<double> rate;
  for (int id = 0; id < 1024; ++id)
    if (count[id]) rate.push_back(count[id] * fmas_per_block / (double)span[id]);
  std::sort(rate.begin(), rate.end());
  if (fma_per_sm_clk) *fma_per_sm_clk = rate.empty() ? 0.0 : rate[rate.size() / 2];
  if (sm_mhz) *sm_mhz = (double)mx / (ms * 1e-3) / 1e6;
  return LDG_OK;
}

int ldg_probe_fp64_peak(int device, double* tflops) { return ldg_probe_fp64(device, tflops, nullptr, nullptr); }

int ldg_operators_1d(int p, double* x, double* w, double* A, double* Lp, double* Lm) {
  if (!x || !w || !A || !Lp || !Lm) return fail(LDG_ERR_INVALID, "null buffer");
  Ops1D o;
  if (!build_ops1d(p, &o)) return fail(LDG_ERR_INVALID, "order p outside 1..7");
  const int N = o.N;
  for (int i = 0; i < N; ++i) {
    x[i] = o.x[i];
    w[i] = o.w[i];
    Lp[i] = o.Lp[i];
    Lm[i] = o.Lm[i];
  }
  for (int i = 0; i < N * N; ++i) A[i] = o.A[i];
  return LDG_OK;
}

int ldg_probe_recip(int device, const double* x, double* r, double* rs, long n) {
  if (n < 0 || (n > 0 && (!x || !r || !rs))) return fail(LDG_ERR_INVALID, "null buffer");
  if (n == 0) return LDG_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(LDG_ERR_NODEVICE, "no CUDA device");
  }
  LDG_CUDA(cudaSetDevice(device));
  double* d = nullptr;
  LDG_CUDA(cudaMalloc((void**)&d, 3 * sizeof(double) * n));
  cudaError_t err = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    const long blocks = std::min<long>((n + 255) / 256, 152L * 16);
    k_recip<<<(int)blocks, 256>>>(d, d + n, d + 2 * n, n);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpy(r, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  if (err == cudaSuccess) err = cudaMemcpy(rs, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err != cudaSuccess) return fail(LDG_ERR_CUDA, cudaGetErrorString(err));
  return LDG_OK;
}

}  // extern "C"

namespace {
template <int N>
cudaError_t launch_contract(ldg_solver* s, int mode, const TcOps& tc) {
  constexpr int EPC = Cfg<N>::EPC;
  const int grid = (s->nE + EPC - 1) / EPC;
  if (mode == 0) {
    const size_t sm = sizeof(double) * EPC * kNS * Cfg<N>::n;
    k_contract_point<N, double><<<grid, Cfg<N>::T, sm, s->stream>>>(s->Un, s->Q, s->nE, s->o64, 0);
  } else if (mode <= 2) {
    const size_t sm = sizeof(double) * EPC * kNS * Cfg<N>::n;
    k_contract_point<N, dd><<<grid, Cfg<N>::T, sm, s->stream>>>((const float2*)s->Us, (float2*)s->Q, s->nE,
                                                                 s->odd, mode == 2);
  } else {
    if constexpr (N == 5) {
      static bool attr = false;
      const size_t sm = sizeof(double) * 2 * (kNS + kNQ) * Cfg<N>::n;
      if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_contract_tc<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
      }
      k_contract_tc<5><<<(s->nE + 1) / 2, 256, sm, s->stream>>>((const float2*)s->Us, (float2*)s->Q, s->nE, tc);
    } else {
      return cudaErrorInvalidValue;
    }
  }
  return cudaGetLastError();
}
cudaError_t d_contract(ldg_solver* s, int mode, const TcOps& tc) { LDG_DISPATCH(s->N, launch_contract<NN>(s, mode, tc)); }
}  // namespace

extern "C" {

int ldg_probe_contraction(ldg_solver* s, int mode, int reps, double* ms, double* max_rel_err) {
  if (!s || mode < 0 || mode > 3 || reps < 1) return fail(LDG_ERR_INVALID, "ldg_probe_contraction: bad arguments");
  if (mode == 3 && s->N != 5) return fail(LDG_ERR_UNSUPPORTED, "ldg_probe_contraction: the tensor-core mode is built for p=4");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  LDG_CUDA(d_attrs(s->N));
  const TcOps tc = make_tc_ops(s->ops, s->N);
  // the FP32-pair copy of the state (what the mixed path's stage 0 reads),
  // traces into the spare trace buffer; Q receives the contractions
  LDG_CUDA(s_traces(s, true, s->Un, s->Us, s->Tu[1 - s->cur]));
  const long long ne = std::min<long long>(s->nE, 2048);
  const size_t cnt = (size_t)ne * kNQ * s->n;
  std::vector<double> ref(cnt), got(cnt);
  LDG_CUDA(d_contract(s, 0, tc));
  LDG_CUDA(cudaMemcpyAsync(ref.data(), s->Q, cnt * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  LDG_CUDA(d_contract(s, mode, tc));  // warm-up, and the values compared
  LDG_CUDA(cudaMemcpyAsync(got.data(), s->Q, cnt * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  cudaEvent_t e0, e1;
  LDG_CUDA(cudaEventCreate(&e0));
  LDG_CUDA(cudaEventCreate(&e1));
  LDG_CUDA(cudaEventRecord(e0, s->stream));
  for (int r = 0; r < reps; ++r) LDG_CUDA(d_contract(s, mode, tc));
  LDG_CUDA(cudaEventRecord(e1, s->stream));
  LDG_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  LDG_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t / reps;
  double mx = 0.0, err = 0.0;
  for (size_t i = 0; i < cnt; ++i) {
    double v = got[i];
    if (mode > 0) {  // FP32 pairs
      float2 f;
      std::memcpy(&f, &got[i], sizeof(f));
      v = (double)f.x + (double)f.y;
    }
    mx = std::max(mx, std::fabs(ref[i]));
    err = std::max(err, std::fabs(v - ref[i]));
  }
  if (max_rel_err) *max_rel_err = mx > 0 ? err / mx : err;
  // the spare traces were overwritten with those of the pair copy of Un;
  // a mixed solver's stage buffer now holds that same pair copy
  return LDG_OK;
}

int ldg_save_checkpoint(ldg_solver* s, const char* path) {
  if (!s || !path || !*path) return fail(LDG_ERR_INVALID, "ldg_save_checkpoint: null solver or empty path");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  const size_t ns = state_count(s), nt = trace_count(s), nk = (size_t)s->step;
  std::vector<double> U(ns), T(nt), ke(nk);
  LDG_CUDA(cudaMemcpyAsync(U.data(), s->Un, ns * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  LDG_CUDA(cudaMemcpyAsync(T.data(), s->Tu[s->cur], nt * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  if (nk) LDG_CUDA(cudaMemcpyAsync(ke.data(), s->ke_dev, nk * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  LDG_CUDA(cudaStreamSynchronize(s->stream));
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.header_bytes = sizeof(CkptHeader);
  h.cfg = s->cfg;
  h.step = s->step;
  h.dt = s->dt;
  h.N = s->N;
  h.nE = s->nE;
  h.precision = s->mixed ? LDG_MIXED_F32X2 : LDG_FP64;
  h.state_bytes = (int64_t)(ns * sizeof(double));
  h.trace_bytes = (int64_t)(nt * sizeof(double));
  h.ke_count = (int64_t)nk;
  uint64_t hash = fnv1a(kFnvBasis, U.data(), ns * sizeof(double));
  hash = fnv1a(hash, T.data(), nt * sizeof(double));
  h.payload_hash = fnv1a(hash, ke.data(), nk * sizeof(double));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return fail(LDG_ERR_IO, "cannot open " + tmp + " for writing");
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(U.data(), sizeof(double), ns, f) == ns &&
            std::fwrite(T.data(), sizeof(double), nt, f) == nt &&
            (nk == 0 || std::fwrite(ke.data(), sizeof(double), nk, f) == nk);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    std::remove(tmp.c_str());
    return fail(LDG_ERR_IO, "short write to " + tmp);
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(LDG_ERR_IO, std::string("cannot rename ") + tmp + " to " + path);
  }
  return LDG_OK;
}

int ldg_checkpoint_config(const char* path, ldg_config* cfg) {
  if (!path || !cfg) return fail(LDG_ERR_INVALID, "ldg_checkpoint_config: null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(LDG_ERR_IO, std::string("cannot open ") + path);
  CkptHeader h;
  int st = read_header(f, path, &h);
  std::fclose(f);
  if (st) return st;
  *cfg = h.cfg;
  return LDG_OK;
}

int ldg_load_checkpoint(ldg_solver* s, const char* path) {
  if (!s || !path) return fail(LDG_ERR_INVALID, "ldg_load_checkpoint: null argument");
  LDG_CUDA(cudaSetDevice(s->cfg.device));
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(LDG_ERR_IO, std::string("cannot open ") + path);
  CkptHeader h;
  int st = read_header(f, path, &h);
  if (st) {
    std::fclose(f);
    return st;
  }
  const size_t ns = state_count(s), nt = trace_count(s);
  const int prec = s->mixed ? LDG_MIXED_F32X2 : LDG_FP64;
  if (!same_problem(h.cfg, s->cfg) || h.N != s->N || h.nE != s->nE || h.precision != prec || h.dt != s->dt) {
    std::fclose(f);
    return fail(LDG_ERR_INVALID, std::string("checkpoint ") + path +
                                     " is of another discretisation (order, mesh, box, physics, precision or dt)");
  }
  if (h.step < 0 || h.ke_count != h.step || h.state_bytes != (int64_t)(ns * sizeof(double)) ||
      h.trace_bytes != (int64_t)(nt * sizeof(double))) {
    std::fclose(f);
    return fail(LDG_ERR_IO, std::string("inconsistent checkpoint sizes in ") + path);
  }
  const size_t nk = (size_t)h.step;
  std::vector<double> U(ns), T(nt), ke(nk);
  bool ok = std::fread(U.data(), sizeof(double), ns, f) == ns && std::fread(T.data(), sizeof(double), nt, f) == nt &&
            (nk == 0 || std::fread(ke.data(), sizeof(double), nk, f) == nk) && std::fgetc(f) == EOF;
  std::fclose(f);
  if (!ok) return fail(LDG_ERR_IO, std::string("truncated or oversized checkpoint ") + path);
  uint64_t hash = fnv1a(kFnvBasis, U.data(), ns * sizeof(double));
  hash = fnv1a(hash, T.data(), nt * sizeof(double));
  if (fnv1a(hash, ke.data(), nk * sizeof(double)) != h.payload_hash)
    return fail(LDG_ERR_IO, std::string("checkpoint payload hash mismatch (corrupted): ") + path);
  if ((st = ensure_ke_capacity(s, (long long)nk + 1))) return st;
  LDG_CUDA(cudaMemcpyAsync(s->Un, U.data(), ns * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  if (s->mixed)  // the FP32-pair stage-0 copy of Un (its traces are replaced next)
    LDG_CUDA(s_traces(s, true, s->Un, s->Us, s->Tu[s->cur]));
  LDG_CUDA(cudaMemcpyAsync(s->Tu[s->cur], T.data(), nt * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  if (nk) LDG_CUDA(cudaMemcpyAsync(s->ke_dev, ke.data(), nk * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  LDG_CUDA(cudaStreamSynchronize(s->stream));
  s->step = (long long)nk;
  return LDG_OK;
}

}  // extern "C"
