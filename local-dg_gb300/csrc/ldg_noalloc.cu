// ldg_rhs_noalloc: the RHS evaluation of ldg_rhs for callers that cannot
// allocate device memory.
//
// Who needs it: host programs that embed this solver inside a framework
// which owns every byte of device memory -- a fixed arena reserved at start
// up, a caching allocator that already holds the GPU, or a real-time loop
// where a cudaMalloc (which can synchronise the device and fail under
// fragmentation) is not allowed.  Such a caller cannot create an ldg_solver
// handle, because ldg_create allocates the state, gradient and trace
// buffers.  This entry point takes the caller's input and output buffers and
// keeps its intermediate buffers (Gauss-point state, face traces, gradient,
// gradient traces) in one file-scope device array of fixed size.
//
// Properties:
//  * The array is LDG_NOALLOC_SCRATCH_BYTES (64 MiB) of static device memory.
//    Every GPU on which the library's device code is loaded holds it until
//    the process exits.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that
//    first call before any stream capture.
//  * All calls share the one array, and it keeps the previous call's
//    contents.  Every scratch region is written in full before it is read,
//    so nothing needs clearing between calls.  Calls whose GPU work overlaps
//    (on different streams, or from different threads) race on the array:
//    order them on one stream or synchronise between them.
//  * Calls no cudaMalloc, cudaFree or other allocating routine.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/ldg.h"
#include "ldg_kernels.cuh"
#include "ldg_ops.hpp"

using namespace ldg;

namespace ldg {
void set_last_error(const std::string& msg);  // ldg_capi.cu
}

namespace {

constexpr size_t kScratchDoubles = (size_t)LDG_NOALLOC_SCRATCH_BYTES / sizeof(double);
__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up once
// per device; the host-side symbol itself is not a device address).
cudaError_t scratch_address(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

template <int N>
cudaError_t run_rhs(const double* u, double* k, double* scratch, const DevOps& ops, const OpsT<double>& o,
                    cudaStream_t st) {
  using C = Cfg<N>;
  const int nE = ops.nE;
  const size_t ne = (size_t)nE;
  double* U = scratch;                       // [nE][5][n]    Gauss-point state, then K
  double* Tu = U + ne * kNS * C::n;          // [nE][6][5][nf] face traces of U
  double* Q = Tu + ne * 6 * kNS * C::nf;     // [nE][15][n]   gradient
  double* Tq = Q + ne * kNQ * C::n;          // [nE][3][15][nf] gradient minus-face traces
  double* Fm = Tq + ne * 3 * kNQ * C::nf;    // [nE][3][5][nf] minus-face Roe fluxes
  const size_t sm_tr = sizeof(double) * 2 * C::EPC * kNS * C::n;
  const size_t sm_trc = sizeof(double) * C::EPC * kNS * C::n;
  const size_t sm_g = sizeof(double) * C::EPC * grad_smem_values_per_element<N>();
  const size_t sm_r = sizeof(double) * C::EPC * (kNQ * C::n + 6 * kNS * C::nf);
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_transform<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_tr)) ||
      (e = cudaFuncSetAttribute(k_traces<N, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_trc)) ||
      (e = cudaFuncSetAttribute(k_grad<N, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_g)) ||
      (e = cudaFuncSetAttribute(k_rhs<N, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_r)))
    return e;
  const int grid = (nE + C::EPC - 1) / C::EPC;
  k_transform<N><<<grid, C::T, sm_tr, st>>>(u, U, nE, kNS, ops, 0);
  k_traces<N, double><<<grid, C::T, sm_trc, st>>>(U, nullptr, Tu, nE, o);
  k_grad<N, double><<<grid, C::T, sm_g, st>>>(U, Tu, Q, Tq, Fm, nullptr, ops, o, 0, ops.nE);
  StageArgs<double> a{};
  std::memset(&a, 0, sizeof(a));
  a.Us = U;
  a.Q = Q;
  a.Tu = Tu;
  a.Tq = Tq;
  a.Fm = Fm;
  a.Kout = U;  // each thread overwrites only the Gauss point it alone read
  a.stage = -1;
  k_rhs<N, double><<<grid, C::T, sm_r, st>>>(a, ops, o, 0, ops.nE);
  k_transform<N><<<grid, C::T, sm_tr, st>>>(U, k, nE, kNS, ops, 1);
  return cudaGetLastError();
}

int fail(int code, const std::string& msg) {
  ldg::set_last_error(msg);  // reported by ldg_last_error_message()
  return code;
}

}  // namespace

extern "C" int ldg_rhs_noalloc(const ldg_config* cfg, const double* u, double* k, void* stream) {
  if (!cfg || !u || !k) return fail(LDG_ERR_INVALID, "ldg_rhs_noalloc: null argument");
  const ldg_config& c = *cfg;
  if (c.p < 1 || c.p > 6) return fail(LDG_ERR_UNSUPPORTED, "ldg_rhs_noalloc: order p must be 1..6");
  if (c.nx < 3 || c.ny < 3 || c.nz < 3)
    return fail(LDG_ERR_INVALID, "ldg_rhs_noalloc: each direction needs at least 3 elements");
  if (!(c.Re > 0) || !(c.Pr > 0) || !(c.gamma > 1) || !(c.L > 0))
    return fail(LDG_ERR_INVALID, "ldg_rhs_noalloc: physical parameters must be positive (gamma > 1)");
  if (c.device < 0 || c.device >= kMaxDevices) return fail(LDG_ERR_INVALID, "ldg_rhs_noalloc: bad device");
  if (c.precision != LDG_FP64 && c.precision != LDG_MIXED_F32X2)
    return fail(LDG_ERR_INVALID, "ldg_rhs_noalloc: precision must be LDG_FP64 or LDG_MIXED_F32X2");
  if (c.precision != LDG_FP64)
    return fail(LDG_ERR_UNSUPPORTED, "ldg_rhs_noalloc: computes in FP64 only (precision LDG_FP64)");
  const int N = c.p + 1, n = N * N * N, nf = N * N;
  const long long nE = (long long)c.nx * c.ny * c.nz;
  const long long need = nE * (long long)(kNS * n + 6 * kNS * nf + kNQ * n + 3 * kNQ * nf + 3 * kNS * nf);
  if (need > (long long)kScratchDoubles)
    return fail(LDG_ERR_INVALID,
                "ldg_rhs_noalloc: mesh needs " + std::to_string(need * 8) + " bytes of scratch; the fixed scratch holds " +
                    std::to_string((long long)LDG_NOALLOC_SCRATCH_BYTES) + " bytes (at most " +
                    std::to_string((long long)kScratchDoubles / (need / nE)) + " elements at p=" +
                    std::to_string(c.p) + ")");
  Ops1D o1;
  if (!build_ops1d(c.p, &o1)) return fail(LDG_ERR_UNSUPPORTED, "ldg_rhs_noalloc: operator setup failed");
  DevOps ops;
  std::memset(&ops, 0, sizeof(ops));
  for (int i = 0; i < N * N; ++i) {
    ops.A[i] = o1.A[i];
    ops.B[i] = o1.B[i];
    ops.Bi[i] = o1.Bi[i];
  }
  for (int i = 0; i < N; ++i) {
    ops.lp[i] = o1.lp[i];
    ops.lm[i] = o1.lm[i];
    ops.Lp[i] = o1.Lp[i];
    ops.Lm[i] = o1.Lm[i];
    ops.w[i] = o1.w[i];
  }
  const double size = M_PI * c.L;
  const int nd[3] = {c.nx, c.ny, c.nz};
  double alpha[3];
  for (int l = 0; l < 3; ++l) {
    const double lo = c.use_box ? c.box_lo[l] : -size, hi = c.use_box ? c.box_hi[l] : size;
    alpha[l] = ((hi - lo) / nd[l]) / 2.0;
    if (!(alpha[l] > 0)) return fail(LDG_ERR_INVALID, "ldg_rhs_noalloc: empty box");
    ops.ia[l] = 1.0 / alpha[l];
  }
  ops.J = alpha[0] * alpha[1] * alpha[2];
  ops.inv_re = 1.0 / c.Re;
  ops.gamma = c.gamma;
  ops.g1 = (c.gamma == 1.4) ? 0.4 : c.gamma - 1.0;
  ops.kappa = c.gamma * (1.0 / c.Pr);
  ops.ke_norm = 1.0 / std::pow(2 * M_PI * c.L, 3.0);
  ops.nx = c.nx;
  ops.ny = c.ny;
  ops.nz = c.nz;
  ops.nE = (int)nE;
  const OpsT<double> o = make_opst<double>(ops, N);

  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    cudaGetLastError();
    return fail(LDG_ERR_NODEVICE, "ldg_rhs_noalloc: no CUDA device");
  }
  if (prev != c.device && cudaSetDevice(c.device) != cudaSuccess)
    return fail(LDG_ERR_CUDA, "ldg_rhs_noalloc: cudaSetDevice failed");
  double* scratch = nullptr;
  cudaError_t e = scratch_address(c.device, &scratch);
  if (e == cudaSuccess) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (N) {
      case 2: e = run_rhs<2>(u, k, scratch, ops, o, st); break;
      case 3: e = run_rhs<3>(u, k, scratch, ops, o, st); break;
      case 4: e = run_rhs<4>(u, k, scratch, ops, o, st); break;
      case 5: e = run_rhs<5>(u, k, scratch, ops, o, st); break;
      case 6: e = run_rhs<6>(u, k, scratch, ops, o, st); break;
      default: e = run_rhs<7>(u, k, scratch, ops, o, st); break;
    }
  }
  if (prev != c.device) cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(LDG_ERR_CUDA, std::string("ldg_rhs_noalloc: ") + cudaGetErrorString(e));
  return LDG_OK;
}
