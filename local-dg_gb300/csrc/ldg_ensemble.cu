// Batched ensemble: many independent Taylor-Green problems (different
// element counts, orders and Reynolds numbers) advanced together, one
// persistent launch per RK4 stage, each step replayed from a CUDA graph.
//
// Each launch drains a work queue of (member, element block) items: all
// gradient-pass items first, then all RHS items.  An RHS item of member i
// needs the gradient traces of i's neighbours, so its CTA waits (bounded
// spin) until all of i's gradient items are done.  Every gradient item was
// dequeued before any RHS item and runs to completion without waiting, so a
// wait depends only on CTAs that are already running: no grid-wide barrier
// or co-residency is needed.  A wait that exceeds its iteration limit (a
// runtime setting) sets the member's error flag and the CTA stops; the
// stage launches after it in the same graph see the flag and return at
// once, so the step stops at a stage boundary with the step's starting state
// Un intact.  The host then either reports LDG_ERR_TIMEOUT or (the default)
// recovers: it re-runs that step member by member with the solo kernels,
// which give the same bits, and carries on with the graphs.
//
// Every item runs the per-element device code of the solo kernels
// (grad_body / rhs_body), and the per-element arithmetic does not depend on
// the tile (elements per CTA), so each member's results are bitwise those of
// a solo ldg_step run with the same configuration.
//
// The autotuner times one stage for two tile shapes (128 or 256 threads per
// CTA: 4/2/1 or 9/4/2 elements per item for p = 2/3/4) and several
// persistent grid sizes, and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ldg.h"
#include "ldg_kernels.cuh"
#include "ldg_problem.hpp"

using namespace ldg;

namespace {

int fail(int code, const std::string& msg) {
  ldg::set_last_error(msg);
  return code;
}

#define ENS_CUDA(call)                                                               \
  do {                                                                               \
    cudaError_t err_ = (call);                                                       \
    if (err_ != cudaSuccess)                                                         \
      return fail(LDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_)); \
  } while (0)

const double kRkB[4] = {1 / 6.0, 1 / 3.0, 1 / 3.0, 1 / 6.0};
const double kRkA[3] = {0.5, 0.5, 1.0};
constexpr long long kDefaultWaitLimit = 1LL << 22;  // x ~100 ns sleeps: gives up after ~0.5 s

// Device-resident description of one member (one per state parity).
struct Member {
  DevOps ops;
  OpsT<double> o;
  int N;
  double* Un;
  double* Uacc;
  double* Us;
  double* Q;
  double* Tq;
  double* Fm;
  double* Tu[2];
  double* diag;
  double cacc[4];
  double cnext[3];
};

struct Item {
  int inst;
  int phase;  // 0 gradient, 1 RHS
  int e0;
  int ne;
};

// Elements per item for N = p+1 at BD threads per CTA.
__host__ __device__ constexpr int tile_epc(int N, int BD) {
  return BD == 256 ? (N == 3 ? 9 : N == 4 ? 4 : 2) : (N == 3 ? 4 : N == 4 ? 2 : 1);
}

template <int BD, int N>
__device__ void run_item(const Member& m, const Item& it, int stage, int cur, int* flag, double* smem) {
  constexpr int E = tile_epc(N, BD);
  static_assert(Cfg<N, E>::T == BD, "tile must fill the block");
  double* Tu_in = m.Tu[(stage & 1) ? 1 - cur : cur];
  double* Tu_out = m.Tu[(stage & 1) ? cur : 1 - cur];
  const double* Uin = stage == 0 ? m.Un : m.Us;
  if (it.phase == 0) {
    grad_body<N, double, E>(Uin, Tu_in, m.Q, m.Tq, m.Fm, nullptr, m.ops, m.o, it.e0, it.ne, smem);
  } else {
    StageArgs<double> a{};
    a.Us = Uin;
    a.Q = m.Q;
    a.Tu = Tu_in;
    a.Tq = m.Tq;
    a.Fm = m.Fm;
    a.Un = m.Un;
    a.Uacc = m.Uacc;
    a.Unext = stage < 3 ? m.Us : nullptr;
    a.Tu_out = Tu_out;
    a.Kout = nullptr;
    a.diag = stage == 3 ? m.diag : nullptr;
    a.flag = flag;
    a.cacc = m.cacc[stage];
    a.cnext = stage < 3 ? m.cnext[stage] : 0.0;
    a.stage = stage;
    rhs_body<N, double, E>(a, m.ops, m.o, it.e0, it.ne, smem);
  }
}

// err[0]: any wait gave up; err[1 + i]: a wait of member i gave up.
template <int BD>
__global__ void __launch_bounds__(BD) k_ensemble_stage(const Member* __restrict__ members,
                                                       const Item* __restrict__ items, int n_items, int* head,
                                                       int* done, const int* __restrict__ need, int stage, int cur,
                                                       int* flag, int* err, long long wait_limit) {
  extern __shared__ double smem[];
  __shared__ int s_item;
  __shared__ int s_ok;
  if (*(volatile int*)err) return;  // an earlier stage of this step gave up
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int idx = s_item;
    if (idx >= n_items) break;
    const Item it = items[idx];
    const Member& m = members[it.inst];
    if (it.phase == 1) {  // wait for the member's gradient pass (bounded)
      if (threadIdx.x == 0) {
        int ok = 1;
        long long spins = 0;
        while (atomicAdd(&done[it.inst], 0) < need[it.inst]) {
          if (++spins > wait_limit) {
            ok = 0;
            atomicOr(err, 1);
            atomicOr(err + 1 + it.inst, 1);
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
        s_ok = ok;
      }
      __syncthreads();
      if (!s_ok) return;  // nothing of this CTA is in flight
    }
    switch (m.N) {
      case 3: run_item<BD, 3>(m, it, stage, cur, flag, smem); break;
      case 4: run_item<BD, 4>(m, it, stage, cur, flag, smem); break;
      default: run_item<BD, 5>(m, it, stage, cur, flag, smem); break;
    }
    __threadfence();  // publish this item's stores before counting it
    __syncthreads();
    if (it.phase == 0 && threadIdx.x == 0) atomicAdd(&done[it.inst], 1);
  }
}

// Per-member KE after a step: the fixed-order compensated reduction of a
// solo run (k_reduce in ldg_capi.cu), into ke[member * cap + step].
__global__ void k_ensemble_ke(const Member* __restrict__ members, int count, const int* step, long long cap,
                              double* ke, const int* err) {
  __shared__ double ss[1024];
  __shared__ double sc[1024];
  const int i = blockIdx.x;
  if (i >= count || *(volatile const int*)err) return;
  const Member& m = members[i];
  double s = 0.0, c = 0.0;
  for (long j = threadIdx.x; j < m.ops.nE; j += blockDim.x) {
    double v = m.diag[j * 2];
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
  if (threadIdx.x == 0) ke[(long long)i * cap + *step] = m.ops.ke_norm * (ss[0] + sc[0]);
}

__global__ void k_ensemble_advance(int* step, const int* err) {
  if (!*(volatile const int*)err) *step += 1;
}

size_t smem_bytes(int BD) {
  size_t mx = 0;
  for (int N = 3; N <= 5; ++N) {
    const size_t E = tile_epc(N, BD), n = (size_t)N * N * N, nf = (size_t)N * N;
    // grad_body's layout (grad_smem_values_per_element) and rhs_body's
    mx = std::max(mx, sizeof(double) * E * (kNS * n + 2 * 3 * kNS * nf + kNQ * n + n));
    mx = std::max(mx, sizeof(double) * E * (kNQ * n + 6 * kNS * nf));
  }
  return mx;
}

}  // namespace

struct ldg_ensemble {
  int count = 0;
  int device = 0;
  std::vector<Problem> pbs;
  std::vector<Member> members;  // parity 0 (Un/Uacc as allocated)
  Member* d_members[2] = {nullptr, nullptr};  // parity 0 / 1 (Un and Uacc swapped)
  int parity = 0;
  Item* d_items[2] = {nullptr, nullptr};  // per tile shape
  int n_items[2] = {0, 0};
  int* d_need[2] = {nullptr, nullptr};
  int* d_head = nullptr;
  int* d_done = nullptr;
  int* d_flag = nullptr;
  int* d_err = nullptr;
  int* d_step = nullptr;
  double* d_ke = nullptr;
  double* d_nodal = nullptr;
  long long ke_cap = 0;
  long long step = 0;
  int tile = 1;  // 0: 128 threads, 1: 256 threads
  int grid = 0;  // persistent CTAs
  int sms = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};  // one captured step per parity
  std::vector<void*> allocs;
  size_t bytes = 0;
  float tune_ms[2][4] = {{0}};
  int tune_grid[4] = {0};
  long long wait_limit = kDefaultWaitLimit;
  int recover = 1;              // re-run a step that gave up, member by member
  long long recovered = 0;      // steps re-run so far
  std::vector<int> stalled;     // members whose gradient target is raised (test hook)
};

namespace {

int ens_alloc(ldg_ensemble* e, void** p, size_t bytes) {
  cudaError_t err = cudaMalloc(p, bytes);
  if (err != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(LDG_ERR_NOMEM, "ensemble: cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  }
  e->allocs.push_back(*p);
  e->bytes += bytes;
  return LDG_OK;
}

void ens_free(ldg_ensemble* e) {
  for (int k = 0; k < 2; ++k)
    if (e->exec[k]) cudaGraphExecDestroy(e->exec[k]);
  for (void* p : e->allocs) cudaFree(p);
  e->allocs.clear();
  if (e->stream) cudaStreamDestroy(e->stream);
}

int enqueue_stage(ldg_ensemble* e, int stage, int parity, int tile, int grid) {
  ENS_CUDA(cudaMemsetAsync(e->d_head, 0, sizeof(int), e->stream));
  ENS_CUDA(cudaMemsetAsync(e->d_done, 0, sizeof(int) * e->count, e->stream));
  // The trace buffers alternate per stage and four stages restore them, so
  // the current-trace index is 0 at every step start.
  if (tile)
    k_ensemble_stage<256><<<grid, 256, smem_bytes(256), e->stream>>>(e->d_members[parity], e->d_items[1],
                                                                     e->n_items[1], e->d_head, e->d_done,
                                                                     e->d_need[1], stage, 0, e->d_flag, e->d_err,
                                                                     e->wait_limit);
  else
    k_ensemble_stage<128><<<grid, 128, smem_bytes(128), e->stream>>>(e->d_members[parity], e->d_items[0],
                                                                     e->n_items[0], e->d_head, e->d_done,
                                                                     e->d_need[0], stage, 0, e->d_flag, e->d_err,
                                                                     e->wait_limit);
  ENS_CUDA(cudaGetLastError());
  return LDG_OK;
}

// One RK4 step of every member, for the given state parity.
int enqueue_step(ldg_ensemble* e, int parity) {
  int st;
  for (int stage = 0; stage < 4; ++stage)
    if ((st = enqueue_stage(e, stage, parity, e->tile, e->grid))) return st;
  k_ensemble_ke<<<e->count, 1024, 0, e->stream>>>(e->d_members[parity], e->count, e->d_step, e->ke_cap, e->d_ke,
                                                   e->d_err);
  k_ensemble_advance<<<1, 1, 0, e->stream>>>(e->d_step, e->d_err);
  ENS_CUDA(cudaGetLastError());
  return LDG_OK;
}

int capture_graphs(ldg_ensemble* e) {
  for (int k = 0; k < 2; ++k) {
    if (e->exec[k]) {
      cudaGraphExecDestroy(e->exec[k]);
      e->exec[k] = nullptr;
    }
    cudaGraph_t g = nullptr;
    ENS_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int st = enqueue_step(e, k);
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (st) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    ENS_CUDA(ce);
    ce = cudaGraphInstantiate(&e->exec[k], g, 0);
    cudaGraphDestroy(g);
    ENS_CUDA(ce);
  }
  return LDG_OK;
}

int ensure_ke(ldg_ensemble* e, long long need) {
  if (need <= e->ke_cap) return LDG_OK;
  long long cap = e->ke_cap ? e->ke_cap : 1024;
  while (cap < need) cap *= 2;
  void* p;
  int st = ens_alloc(e, &p, sizeof(double) * cap * e->count);
  if (st) return st;
  double* nk = (double*)p;
  if (e->d_ke) {
    ENS_CUDA(cudaMemcpy2DAsync(nk, cap * sizeof(double), e->d_ke, e->ke_cap * sizeof(double),
                               e->ke_cap * sizeof(double), e->count, cudaMemcpyDeviceToDevice, e->stream));
    ENS_CUDA(cudaStreamSynchronize(e->stream));
  }
  e->d_ke = nk;
  e->ke_cap = cap;
  return capture_graphs(e);  // the graphs bake in d_ke and ke_cap
}

// Times one stage (stage 0 only reads Un and the current traces, so
// repeating it leaves the state unchanged) for every tile shape and grid.
int autotune(ldg_ensemble* e) {
  cudaEvent_t a, b;
  ENS_CUDA(cudaEventCreate(&a));
  ENS_CUDA(cudaEventCreate(&b));
  const int mult[4] = {1, 2, 4, 8};
  float best = 1e30f;
  for (int tile = 0; tile < 2; ++tile)
    for (int g = 0; g < 4; ++g) {
      const int grid = e->sms * mult[g];
      e->tune_grid[g] = grid;
      int st = enqueue_stage(e, 0, e->parity, tile, grid);  // warm-up
      if (st) return st;
      ENS_CUDA(cudaEventRecord(a, e->stream));
      for (int r = 0; r < 3; ++r)
        if ((st = enqueue_stage(e, 0, e->parity, tile, grid))) return st;
      ENS_CUDA(cudaEventRecord(b, e->stream));
      ENS_CUDA(cudaEventSynchronize(b));
      float ms = 0.f;
      ENS_CUDA(cudaEventElapsedTime(&ms, a, b));
      e->tune_ms[tile][g] = ms / 3;
      if (ms < best) {
        best = ms;
        e->tile = tile;
        e->grid = grid;
      }
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return LDG_OK;
}

int check_flags(ldg_ensemble* e) {
  int h[2] = {0, 0};
  ENS_CUDA(cudaMemcpyAsync(&h[0], e->d_flag, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(cudaMemcpyAsync(&h[1], e->d_err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  if (h[1]) return fail(LDG_ERR_TIMEOUT, "ensemble: a dependency wait exceeded its limit");
  if (h[0]) return fail(LDG_ERR_NONFINITE, "ensemble: non-finite value in a member's state");
  return LDG_OK;
}

// The host copy of member i for state parity p (Un and Uacc swapped for p=1).
Member member_at(const ldg_ensemble* e, int i, int parity) {
  Member m = e->members[i];
  if (parity) std::swap(m.Un, m.Uacc);
  return m;
}

// After a step that gave up: every member's step-start state Un is intact,
// but the stages may have overwritten the traces of Un (the trace buffers
// alternate per stage).  Rebuild them so that the step can start again.
int restore_traces(ldg_ensemble* e, int parity) {
  for (int i = 0; i < e->count; ++i) {
    const Member m = member_at(e, i, parity);
    ENS_CUDA(launch_traces_fp64(m.N, m.Un, m.Tu[0], m.ops.nE, m.o, e->stream));
  }
  return LDG_OK;
}

// Re-runs the step that starts at state parity `parity`, member by member,
// with the solo kernels ldg_step launches (the same per-element arithmetic,
// so the same bits as an uninterrupted ensemble step), then its KE and the
// device step counter.  The error flags must be clear.
int recover_step(ldg_ensemble* e, int parity) {
  for (int i = 0; i < e->count; ++i) {
    const Member m = member_at(e, i, parity);
    for (int stage = 0; stage < 4; ++stage) {
      const double* Uin = stage == 0 ? m.Un : m.Us;
      double* Tu_in = m.Tu[(stage & 1) ? 1 : 0];
      double* Tu_out = m.Tu[(stage & 1) ? 0 : 1];
      ENS_CUDA(launch_grad_fp64(m.N, Uin, Tu_in, m.Q, m.Tq, m.Fm, m.ops, m.o, e->stream));
      StageArgs<double> a{};
      a.Us = Uin;
      a.Q = m.Q;
      a.Tu = Tu_in;
      a.Tq = m.Tq;
      a.Fm = m.Fm;
      a.Un = m.Un;
      a.Uacc = m.Uacc;
      a.Unext = stage < 3 ? m.Us : nullptr;
      a.Tu_out = Tu_out;
      a.diag = stage == 3 ? m.diag : nullptr;
      a.flag = e->d_flag;
      a.cacc = m.cacc[stage];
      a.cnext = stage < 3 ? m.cnext[stage] : 0.0;
      a.stage = stage;
      ENS_CUDA(launch_rhs_fp64(m.N, a, m.ops, m.o, e->stream));
    }
  }
  k_ensemble_ke<<<e->count, 1024, 0, e->stream>>>(e->d_members[parity], e->count, e->d_step, e->ke_cap, e->d_ke,
                                                   e->d_err);
  k_ensemble_advance<<<1, 1, 0, e->stream>>>(e->d_step, e->d_err);
  ENS_CUDA(cudaGetLastError());
  return LDG_OK;
}

// Raises (on) or restores the gradient-item target of member i in both
// tile shapes' need arrays.
int set_need_offset(ldg_ensemble* e, int i, int delta) {
  for (int tile = 0; tile < 2; ++tile) {
    int v = 0;
    ENS_CUDA(cudaMemcpyAsync(&v, e->d_need[tile] + i, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    ENS_CUDA(cudaStreamSynchronize(e->stream));
    v += delta;
    ENS_CUDA(cudaMemcpyAsync(e->d_need[tile] + i, &v, sizeof(int), cudaMemcpyHostToDevice, e->stream));
    ENS_CUDA(cudaStreamSynchronize(e->stream));
  }
  return LDG_OK;
}

}  // namespace

extern "C" {

int ldg_ensemble_create(const ldg_config* cfgs, int count, ldg_ensemble** out) {
  if (!cfgs || !out || count <= 0) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  *out = nullptr;
  const int device = cfgs[0].device;
  for (int i = 0; i < count; ++i) {
    if (cfgs[i].p < 2 || cfgs[i].p > 4) return fail(LDG_ERR_UNSUPPORTED, "ensemble members need p in 2..4");
    if (cfgs[i].precision != LDG_FP64) return fail(LDG_ERR_UNSUPPORTED, "ensemble members are FP64");
    if (cfgs[i].device != device) return fail(LDG_ERR_INVALID, "ensemble members must share a device");
  }
  ldg_ensemble* e = new ldg_ensemble();
  e->count = count;
  e->device = device;
  std::string err;
  int st = LDG_OK;
  auto bail = [&](int code) {
    ens_free(e);
    delete e;
    return code;
  };
  e->pbs.resize(count);
  for (int i = 0; i < count; ++i)
    if ((st = setup_problem(cfgs[i], &e->pbs[i], &err))) return bail(fail(st, "ensemble member " + std::to_string(i) + ": " + err));
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return bail(fail(LDG_ERR_CUDA, "ensemble: device/stream setup"));
  size_t max_state = 0;
  for (int i = 0; i < count; ++i) {
    const Problem& pb = e->pbs[i];
    Member m;
    std::memset(&m, 0, sizeof(m));
    m.ops = pb.ops;
    m.N = pb.N;
    m.o = make_opst<double>(m.ops, m.N);
    for (int s = 0; s < 4; ++s) m.cacc[s] = pb.dt * kRkB[s];  // as the solo path computes them
    for (int s = 0; s < 3; ++s) m.cnext[s] = pb.dt * kRkA[s];
    const size_t nE = pb.nE, n = pb.n, nf = pb.nf;
    void* p[9];
    const size_t sizes[9] = {nE * kNS * n, nE * kNS * n, nE * kNS * n, nE * kNQ * n, nE * 3 * kNQ * nf,
                             nE * 6 * kNS * nf, nE * 6 * kNS * nf, nE * 2, nE * 3 * kNS * nf};
    for (int k = 0; k < 9; ++k)
      if ((st = ens_alloc(e, &p[k], sizes[k] * sizeof(double)))) return bail(st);
    m.Un = (double*)p[0];
    m.Uacc = (double*)p[1];
    m.Us = (double*)p[2];
    m.Q = (double*)p[3];
    m.Tq = (double*)p[4];
    m.Tu[0] = (double*)p[5];
    m.Tu[1] = (double*)p[6];
    m.diag = (double*)p[7];
    m.Fm = (double*)p[8];
    max_state = std::max(max_state, nE * kNS * n);
    e->members.push_back(m);
  }
  void* p;
  if ((st = ens_alloc(e, &p, max_state * sizeof(double)))) return bail(st);
  e->d_nodal = (double*)p;
  for (int k = 0; k < 2; ++k) {
    if ((st = ens_alloc(e, &p, sizeof(Member) * count))) return bail(st);
    e->d_members[k] = (Member*)p;
  }
  int* ints[5];
  for (int k = 0; k < 5; ++k) {
    if ((st = ens_alloc(e, &p, sizeof(int) * (k == 1 ? count : k == 3 ? count + 1 : 1)))) return bail(st);
    ints[k] = (int*)p;
  }
  e->d_head = ints[0];
  e->d_done = ints[1];
  e->d_flag = ints[2];
  e->d_err = ints[3];
  e->d_step = ints[4];
  if (cudaMemsetAsync(e->d_flag, 0, sizeof(int), e->stream) ||
      cudaMemsetAsync(e->d_err, 0, sizeof(int) * (count + 1), e->stream) ||
      cudaMemsetAsync(e->d_step, 0, sizeof(int), e->stream))
    return bail(fail(LDG_ERR_CUDA, "ensemble: counters"));
  // Work items per tile shape: every member's gradient items, then RHS items.
  for (int tile = 0; tile < 2; ++tile) {
    std::vector<Item> items;
    std::vector<int> need(count);
    for (int phase = 0; phase < 2; ++phase)
      for (int i = 0; i < count; ++i) {
        const int E = tile_epc(e->pbs[i].N, tile ? 256 : 128);
        const int nE = e->pbs[i].nE;
        int k = 0;
        for (int e0 = 0; e0 < nE; e0 += E, ++k) items.push_back({i, phase, e0, std::min(E, nE - e0)});
        if (phase == 0) need[i] = k;
      }
    if ((st = ens_alloc(e, &p, sizeof(Item) * items.size()))) return bail(st);
    e->d_items[tile] = (Item*)p;
    if ((st = ens_alloc(e, &p, sizeof(int) * count))) return bail(st);
    e->d_need[tile] = (int*)p;
    e->n_items[tile] = (int)items.size();
    if (cudaMemcpyAsync(e->d_items[tile], items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice,
                        e->stream) ||
        cudaMemcpyAsync(e->d_need[tile], need.data(), sizeof(int) * count, cudaMemcpyHostToDevice, e->stream) ||
        cudaStreamSynchronize(e->stream))
      return bail(fail(LDG_ERR_CUDA, "ensemble: item upload"));
  }
  if (cudaFuncSetAttribute(k_ensemble_stage<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_bytes(256)) != cudaSuccess ||
      cudaFuncSetAttribute(k_ensemble_stage<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_bytes(128)) != cudaSuccess)
    return bail(fail(LDG_ERR_CUDA, "ensemble: shared-memory attribute"));
  // Member parity copies on the device.
  std::vector<Member> swapped = e->members;
  for (auto& m : swapped) std::swap(m.Un, m.Uacc);
  if (cudaMemcpyAsync(e->d_members[0], e->members.data(), sizeof(Member) * count, cudaMemcpyHostToDevice,
                      e->stream) ||
      cudaMemcpyAsync(e->d_members[1], swapped.data(), sizeof(Member) * count, cudaMemcpyHostToDevice, e->stream) ||
      cudaStreamSynchronize(e->stream))
    return bail(fail(LDG_ERR_CUDA, "ensemble: member upload"));
  // Initial conditions (Taylor-Green + seeded perturbation) and traces.
  for (int i = 0; i < count; ++i) {
    const Problem& pb = e->pbs[i];
    const Member& m = e->members[i];
    if (launch_initial_condition(pb, e->d_nodal, e->stream) != cudaSuccess ||
        launch_transform_any(pb.N, e->d_nodal, m.Un, pb.nE, pb.ops, 0, e->stream) != cudaSuccess ||
        launch_traces_fp64(pb.N, m.Un, m.Tu[0], pb.nE, m.o, e->stream) != cudaSuccess)
      return bail(fail(LDG_ERR_CUDA, "ensemble: initial condition"));
  }
  if ((st = autotune(e)) || (st = ensure_ke(e, 1024)) || (st = capture_graphs(e)) || (st = check_flags(e)))
    return bail(st);
  *out = e;
  return LDG_OK;
}

int ldg_ensemble_destroy(ldg_ensemble* e) {
  if (!e) return LDG_OK;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  ens_free(e);
  delete e;
  return LDG_OK;
}

int ldg_ensemble_step(ldg_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  if (nsteps == 0) return LDG_OK;
  ENS_CUDA(cudaSetDevice(e->device));
  int st = ensure_ke(e, e->step + nsteps + 1);
  if (st) return st;
  int left = nsteps;
  while (left > 0) {
    for (int it = 0; it < left; ++it) ENS_CUDA(cudaGraphLaunch(e->exec[(e->parity + it) & 1], e->stream));
    int h[2] = {0, 0};  // error flag, device step counter
    ENS_CUDA(cudaMemcpyAsync(&h[0], e->d_err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    ENS_CUDA(cudaMemcpyAsync(&h[1], e->d_step, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    ENS_CUDA(cudaStreamSynchronize(e->stream));
    // steps completed: the graphs after a failed stage return at once and
    // leave the device step counter where the failure happened
    const int done = h[0] ? (int)(h[1] - e->step) : left;
    e->parity ^= done & 1;  // u^{n+1} is in the other buffer
    e->step += done;
    left -= done;
    if (!h[0]) break;
    ENS_CUDA(cudaMemsetAsync(e->d_err, 0, sizeof(int) * (e->count + 1), e->stream));
    if ((st = restore_traces(e, e->parity))) return st;
    if (!e->recover) {
      ENS_CUDA(cudaStreamSynchronize(e->stream));
      return fail(LDG_ERR_TIMEOUT, "ensemble: a dependency wait exceeded its limit at step " +
                                       std::to_string(e->step) + "; the state is that step's start");
    }
    if ((st = recover_step(e, e->parity))) return st;
    e->parity ^= 1;
    e->step += 1;
    e->recovered += 1;
    left -= 1;
  }
  return check_flags(e);
}

int ldg_ensemble_set_wait_limit(ldg_ensemble* e, long long polls, int recover) {
  if (!e || polls < 0) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  ENS_CUDA(cudaSetDevice(e->device));
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  e->recover = recover ? 1 : 0;
  if (polls == e->wait_limit) return LDG_OK;
  e->wait_limit = polls;
  return capture_graphs(e);  // the limit is a launch argument the graphs bake in
}

int ldg_ensemble_recovered_steps(const ldg_ensemble* e, long long* steps) {
  if (!e || !steps) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  *steps = e->recovered;
  return LDG_OK;
}

int ldg_ensemble_inject_stall(ldg_ensemble* e, int member, int on) {
  if (!e || member < 0 || member >= e->count) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  ENS_CUDA(cudaSetDevice(e->device));
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  auto it = std::find(e->stalled.begin(), e->stalled.end(), member);
  const bool is_on = it != e->stalled.end();
  if (on && !is_on) {
    e->stalled.push_back(member);
    return set_need_offset(e, member, +1);
  }
  if (!on && is_on) {
    e->stalled.erase(it);
    return set_need_offset(e, member, -1);
  }
  return LDG_OK;
}

int ldg_ensemble_get_state(ldg_ensemble* e, int member, double* u, int where) {
  if (!e || member < 0 || member >= e->count || !u) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  ENS_CUDA(cudaSetDevice(e->device));
  const Problem& pb = e->pbs[member];
  const Member& m = e->members[member];
  const double* Un = e->parity ? m.Uacc : m.Un;
  ENS_CUDA(launch_transform_any(pb.N, Un, e->d_nodal, pb.nE, pb.ops, 1, e->stream));
  const size_t bytes = (size_t)pb.nE * kNS * pb.n * sizeof(double);
  ENS_CUDA(cudaMemcpyAsync(u, e->d_nodal, bytes, where == LDG_DEVICE ? cudaMemcpyDeviceToDevice
                                                                       : cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(cudaStreamSynchronize(e->stream));
  return LDG_OK;
}

int ldg_ensemble_ke_history(ldg_ensemble* e, int member, double* ke, int max, int* count) {
  if (!e || member < 0 || member >= e->count) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  if (count) *count = (int)e->step;
  const int m = (int)std::min<long long>(max, e->step);
  if (m > 0 && ke) {
    ENS_CUDA(cudaMemcpyAsync(ke, e->d_ke + (long long)member * e->ke_cap, m * sizeof(double),
                             cudaMemcpyDeviceToHost, e->stream));
    ENS_CUDA(cudaStreamSynchronize(e->stream));
  }
  return LDG_OK;
}

int ldg_ensemble_member_info(const ldg_ensemble* e, int member, ldg_info* info) {
  if (!e || !info || member < 0 || member >= e->count) return fail(LDG_ERR_INVALID, "ensemble: bad arguments");
  const Problem& pb = e->pbs[member];
  std::memset(info, 0, sizeof(*info));
  info->p = pb.cfg.p;
  info->dofs = pb.n;
  info->nf = pb.nf;
  info->nx = pb.cfg.nx;
  info->ny = pb.cfg.ny;
  info->nz = pb.cfg.nz;
  info->nelements = pb.nE;
  info->dt = pb.dt;
  info->timesteps = pb.timesteps;
  info->step = e->step;
  info->time = e->step * pb.dt;
  info->device_bytes = e->bytes;
  info->precision = LDG_FP64;
  return LDG_OK;
}

int ldg_ensemble_tuning(const ldg_ensemble* e, int* threads_per_cta, int* persistent_ctas, float* stage_ms,
                        int max) {
  if (!e) return fail(LDG_ERR_INVALID, "ensemble: null");
  if (threads_per_cta) *threads_per_cta = e->tile ? 256 : 128;
  if (persistent_ctas) *persistent_ctas = e->grid;
  if (stage_ms)
    for (int k = 0; k < 8 && k < max; ++k) stage_ms[k] = e->tune_ms[k / 4][k % 4];
  return LDG_OK;
}

void* ldg_ensemble_stream(ldg_ensemble* e) { return e ? (void*)e->stream : nullptr; }

}  // extern "C"
