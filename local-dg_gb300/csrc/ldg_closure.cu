// Learned closure: a per-element MLP that corrects the RHS of a coarse LDG
// solver toward the L2 projection of a fine solver's RHS.
//
// Data (ldg_closure_add_samples): the fine state u_f (Gauss basis) and its
// RHS K_f are L2-projected element-wise onto the coarse mesh (each coarse
// element is r^3 fine elements; the projection is exact with the fine Gauss
// rule).  The coarse solver evaluates its own gradient q and RHS K_c of the
// projected state u_c.  One sample per coarse element:
//   features  [u_c (5 x n), q (15 x n)]   (n = (p_c+1)^3 Gauss points)
//   target    P(K_f) - K_c                (5 x n)
// Solver in the loop (ldg_closure_project_state, then
// ldg_closure_add_samples_coarse): the coarse solver starts from P(u_f),
// runs on its own, and the samples take u_c from its state at the sample
// time, with the target P(K_f) - K_c(u_c) -- the states the coarse solver
// produces itself, which are what the closure sees when attached.
// Network: x -> GELU(W1 x + b1) -> GELU(W2 h + b2) -> W3 h + b3, inputs and
// outputs normalised per channel; BF16 weights and activations, FP32
// accumulation on the tensor cores (ldg_mlp.cuh), FP32 master weights with
// Adam.  In a coarse solver with the closure attached, every RK stage adds
// the de-normalised prediction to the RHS before the RK update, after two
// safeguards:
//   * fallback: an element whose normalised features leave the training
//     range (|x| > ood_sigma, 10 by default) or whose prediction is not
//     finite gets no correction (the plain LDG operator); such elements are
//     counted;
//   * energy stability (option `energy`, dissipative by default): the
//     component of the correction that would raise the element's kinetic
//     energy is removed.  With g_q = dKE/du at Gauss point q,
//     (-|v|^2/2, v, 0), the rate sum_q w_q g_q . d of a correction d is made
//     <= 0 by the smallest change in the element's L2 norm,
//     d <- d - lambda g with lambda = max(0, sum w g.d) / sum w g.g
//     (an element-wise form of backscatter clipping); projected elements
//     are counted.  The correction can then only dissipate kinetic energy.
//     The neutral mode removes the KE production whatever its sign.
// Training can add Gaussian noise to the normalised features (option
// input_noise), which makes the network less sensitive to the difference
// between projected fine states and the coarse solver's own states.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/ldg.h"
#include "ldg_closure.hpp"
#include "ldg_mlp.cuh"
#include "ldg_ops.hpp"

using namespace ldg;
using namespace ldg::mlp;

namespace ldg {
void set_last_error(const std::string& msg);
}

namespace {

int fail(int code, const std::string& msg) {
  ldg::set_last_error(msg);
  return code;
}

#define CL_CUDA(call)                                                                \
  do {                                                                               \
    cudaError_t err_ = (call);                                                       \
    if (err_ != cudaSuccess)                                                         \
      return fail(LDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_)); \
  } while (0)

constexpr int kChIn = 20;   // 5 state variables + 15 gradient components
constexpr int kChOut = 5;

// ------------------------------------------------------------ projection
// One CTA per coarse element: gathers the r^3 fine elements' Gauss values
// of nv variables into an (r Nf)^3 grid and contracts it with P1 (Nc x r Nf)
// along x, y, z.
__global__ void k_project(const double* __restrict__ Uf, double* __restrict__ Uc, int ncx, int ncy, int ncz,
                          int r, int Nf, int Nc, int nv, const double* __restrict__ P1) {
  extern __shared__ double sm[];
  const int M = r * Nf;  // fine points per direction in a coarse element
  double* g0 = sm;                      // nv * M^3
  double* g1 = g0 + (long)nv * M * M * M;  // nv * M * M * Nc
  double* g2 = g1 + (long)nv * M * M * Nc;  // nv * M * Nc * Nc
  const int ec = blockIdx.x;
  const int cx = ec % ncx, cy = (ec / ncx) % ncy, cz = ec / (ncx * ncy);
  const int nfx = ncx * r, nfy = ncy * r;
  const int nf3 = Nf * Nf * Nf, nc3 = Nc * Nc * Nc;
  for (int i = threadIdx.x; i < nv * M * M * M; i += blockDim.x) {
    const int v = i / (M * M * M);
    const int rem = i % (M * M * M);
    const int X = rem % M, Y = (rem / M) % M, Z = rem / (M * M);
    const int sx = X / Nf, sy = Y / Nf, sz = Z / Nf;
    const int qx = X % Nf, qy = Y % Nf, qz = Z % Nf;
    const long ef = (long)(r * cx + sx) + (long)nfx * ((r * cy + sy) + (long)nfy * (r * cz + sz));
    g0[i] = Uf[(ef * nv + v) * nf3 + qx + Nf * (qy + Nf * qz)];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nv * M * M * Nc; i += blockDim.x) {  // x: (v, a, Y, Z)
    const int v = i / (M * M * Nc);
    const int rem = i % (M * M * Nc);
    const int a = rem % Nc, Y = (rem / Nc) % M, Z = rem / (Nc * M);
    double s = 0.0;
    for (int X = 0; X < M; ++X) s = fma(P1[a * M + X], g0[(long)v * M * M * M + X + M * (Y + M * Z)], s);
    g1[i] = s;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nv * Nc * Nc * M; i += blockDim.x) {  // y: (v, a, b, Z)
    const int v = i / (Nc * Nc * M);
    const int rem = i % (Nc * Nc * M);
    const int a = rem % Nc, b = (rem / Nc) % Nc, Z = rem / (Nc * Nc);
    double s = 0.0;
    for (int Y = 0; Y < M; ++Y) s = fma(P1[b * M + Y], g1[(long)v * M * M * Nc + a + Nc * (Y + M * Z)], s);
    g2[i] = s;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nv * nc3; i += blockDim.x) {  // z: (v, a, b, c)
    const int v = i / nc3;
    const int rem = i % nc3;
    const int a = rem % Nc, b = (rem / Nc) % Nc, c = rem / (Nc * Nc);
    double s = 0.0;
    for (int Z = 0; Z < M; ++Z) s = fma(P1[c * M + Z], g2[(long)v * Nc * Nc * M + a + Nc * (b + Nc * Z)], s);
    Uc[((long)ec * nv + v) * nc3 + rem] = s;
  }
}

// Sample rows: features [U (5n), Q (15n)] and targets T - K (5n), float.
__global__ void k_make_rows(const double* __restrict__ U, const double* __restrict__ Q,
                            const double* __restrict__ KT, const double* __restrict__ Kc, int nE, int n,
                            float* __restrict__ X, float* __restrict__ Y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long in_dim = (long)kChIn * n, out_dim = (long)kChOut * n;
  if (i < (long)nE * in_dim) {
    const long e = i / in_dim, j = i % in_dim;
    X[i] = (float)(j < 5 * n ? U[e * 5 * n + j] : Q[e * 15 * n + (j - 5 * n)]);
  }
  if (i < (long)nE * out_dim) {
    Y[i] = (float)(KT[i] - Kc[i]);
  }
}

// Per-channel mean and standard deviation over rows x points (FP64 sums, one
// CTA per channel, fixed order).
__global__ void k_channel_stats(const float* __restrict__ D, long rows, int ch, int n, float* __restrict__ mean,
                                float* __restrict__ stdv) {
  __shared__ double s1[256], s2[256];
  const int c = blockIdx.x;
  double a = 0.0, b = 0.0;
  const long total = rows * n;
  for (long i = threadIdx.x; i < total; i += blockDim.x) {
    const long r = i / n, q = i % n;
    const double v = D[r * (long)ch * n + (long)c * n + q];
    a += v;
    b += v * v;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      s1[threadIdx.x] += s1[threadIdx.x + h];
      s2[threadIdx.x] += s2[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = s1[0] / (double)total;
    const double var = fmax(s2[0] / (double)total - m * m, 0.0);
    mean[c] = (float)m;
    stdv[c] = (float)fmax(sqrt(var), 1e-12);
  }
}

// SplitMix64 (Steele, Lea & Flood 2014) as a counter-based hash.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Standard normal deviate for counter i under key (Box-Muller on two
// hashed uniforms, the first in (0, 1]).
__device__ __forceinline__ float normal01(unsigned long long key, long i) {
  const unsigned long long a = mix64(key ^ (2ULL * (unsigned long long)i));
  const unsigned long long b = mix64(key ^ (2ULL * (unsigned long long)i + 1ULL));
  const float u1 = ((float)(a >> 40) + 1.f) * (1.f / 16777216.f);
  const float u2 = (float)(b >> 40) * (1.f / 16777216.f);
  return sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

// Gathers rows idx[] of raw features/targets and normalises them:
// Xb = bf16((x - mu_in) / sd_in + noise N(0, sigma^2)), Tn = (t - mu_out) / sd_out.
__global__ void k_gather_norm(const float* __restrict__ X, const float* __restrict__ Y, const long* __restrict__ idx,
                              int B, int n, const float* __restrict__ mi, const float* __restrict__ si,
                              const float* __restrict__ mo, const float* __restrict__ so,
                              __nv_bfloat16* __restrict__ Xb, float* __restrict__ Tn, float noise,
                              unsigned long long key) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long in_dim = (long)kChIn * n, out_dim = (long)kChOut * n;
  if (i < B * in_dim) {
    const long b = i / in_dim, j = i % in_dim;
    const int c = (int)(j / n);
    float x = (X[idx[b] * in_dim + j] - mi[c]) / si[c];
    if (noise > 0.f) x += noise * normal01(key, i);
    Xb[i] = __float2bfloat16(x);
  }
  if (Y && i < B * out_dim) {
    const long b = i / out_dim, j = i % out_dim;
    const int c = (int)(j / n);
    Tn[i] = (Y[idx[b] * out_dim + j] - mo[c]) / so[c];
  }
}

// Features of every element of a solver state for inference; ood[e] is set
// when a feature of element e is outside the training range (or not finite).
__global__ void k_features(const double* __restrict__ U, const double* __restrict__ Q, int nE, int n,
                           const float* __restrict__ mi, const float* __restrict__ si,
                           __nv_bfloat16* __restrict__ Xb, int* __restrict__ ood, float ood_sigma) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long in_dim = (long)kChIn * n;
  if (i >= (long)nE * in_dim) return;
  const long e = i / in_dim, j = i % in_dim;
  const int c = (int)(j / n);
  const double v = j < 5 * n ? U[e * 5 * n + j] : Q[e * 15 * n + (j - 5 * n)];
  const float x = ((float)v - mi[c]) / si[c];
  if (!(fabsf(x) <= ood_sigma)) ood[e] = 1;
  Xb[i] = __float2bfloat16(x);
}

struct GaussW {
  double w[8];
};

// De-normalised, energy-stable correction into the RHS term (one CTA per
// element, n <= 512 points).  Elements marked out of range or with a
// non-finite prediction get no correction.
__global__ void k_correction(const float* __restrict__ Yn, const double* __restrict__ U, int nE, int N,
                             const float* __restrict__ mo, const float* __restrict__ so, const GaussW gw,
                             const int* __restrict__ ood, int energy, double scale, double* __restrict__ Kadd,
                             unsigned long long* __restrict__ counters) {
  const int e = blockIdx.x;
  if (e >= nE) return;
  const int n = N * N * N, out_dim = kChOut * n;
  __shared__ int bad;
  __shared__ double sp[128], sg[128];
  if (threadIdx.x == 0) bad = ood[e];
  __syncthreads();
  for (int j = threadIdx.x; j < out_dim; j += blockDim.x)
    if (!isfinite(Yn[(long)e * out_dim + j])) bad = 1;
  __syncthreads();
  if (bad) {
    for (int j = threadIdx.x; j < out_dim; j += blockDim.x) Kadd[(long)e * out_dim + j] = 0.0;
    if (threadIdx.x == 0) atomicAdd(&counters[0], 1ULL);
    return;
  }
  // KE production of the correction, sum_q w_q g_q . d_q, and sum_q w_q |g_q|^2
  double pr = 0.0, gg = 0.0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const double* u = U + (long)e * 5 * n + q;
    const double ir = 1.0 / u[0];
    const double v0 = u[n] * ir, v1 = u[2 * n] * ir, v2 = u[3 * n] * ir;
    const double g0 = -0.5 * (v0 * v0 + v1 * v1 + v2 * v2);
    const double w = gw.w[q % N] * gw.w[(q / N) % N] * gw.w[q / (N * N)];
    double d[4];
    for (int c = 0; c < 4; ++c) d[c] = scale * (double)(Yn[(long)e * out_dim + c * n + q] * so[c] + mo[c]);
    pr += w * (g0 * d[0] + v0 * d[1] + v1 * d[2] + v2 * d[3]);
    gg += w * (g0 * g0 + v0 * v0 + v1 * v1 + v2 * v2);
  }
  sp[threadIdx.x] = pr;
  sg[threadIdx.x] = gg;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {  // fixed-order tree (deterministic)
    if (threadIdx.x < h) {
      sp[threadIdx.x] += sp[threadIdx.x + h];
      sg[threadIdx.x] += sg[threadIdx.x + h];
    }
    __syncthreads();
  }
  // energy 1: remove a KE-raising component; energy 2: remove the KE
  // production whatever its sign; energy 0: no projection
  const bool project = sg[0] > 0.0 && ((energy == 1 && sp[0] > 0.0) || (energy == 2 && sp[0] != 0.0));
  const double lambda = project ? sp[0] / sg[0] : 0.0;
  for (int j = threadIdx.x; j < out_dim; j += blockDim.x) {
    const int c = j / n, q = j % n;
    double d = scale * (double)(Yn[(long)e * out_dim + j] * so[c] + mo[c]);
    if (project && c < 4) {
      const double* u = U + (long)e * 5 * n + q;
      const double ir = 1.0 / u[0];
      const double v0 = u[n] * ir, v1 = u[2 * n] * ir, v2 = u[3 * n] * ir;
      const double g = c == 0 ? -0.5 * (v0 * v0 + v1 * v1 + v2 * v2) : (c == 1 ? v0 : (c == 2 ? v1 : v2));
      d -= lambda * g;
    }
    Kadd[(long)e * out_dim + j] = d;
  }
  if (project && threadIdx.x == 0) atomicAdd(&counters[1], 1ULL);
}

__global__ void k_f2bf(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, long count) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) y[i] = __float2bfloat16(x[i]);
}

// Per-row squared error of predictions against normalised targets, both
// plain (prediction 0 correction) and closure, in units of sd_out.
__global__ void k_eval_rows(const float* __restrict__ Yn, const float* __restrict__ Tn, int B, int n,
                            const float* __restrict__ mo, const float* __restrict__ so, double* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int out_dim = kChOut * n;
  double ep = 0.0, ec = 0.0;
  for (int j = 0; j < out_dim; ++j) {
    const int c = j / n;
    const double t = Tn[(long)b * out_dim + j];
    const double plain = (0.0 - mo[c]) / so[c];  // no correction
    ep += (t - plain) * (t - plain);
    ec += (t - Yn[(long)b * out_dim + j]) * (t - Yn[(long)b * out_dim + j]);
  }
  out[2 * b] = ep;
  out[2 * b + 1] = ec;
}

long ceil_div(long a, long b) { return (a + b - 1) / b; }

}  // namespace

struct ldg_closure {
  int p = 2, N = 3, n = 27, in_dim = 540, out_dim = 135, hidden = 128;
  int device = 0;
  cudaStream_t stream = nullptr;
  // parameters: W1 [H x in], b1 [H], W2 [H x H], b2 [H], W3 [out x H], b3 [out]
  long off[6] = {0, 0, 0, 0, 0, 0};
  long n_params = 0;
  float *theta = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16* wb = nullptr;  // bf16 copy (same offsets)
  int adam_t = 0;
  // normalisation
  float* stats = nullptr;  // mi[20], si[20], mo[5], so[5]
  bool stats_ready = false;
  // raw samples
  float* X = nullptr;
  float* Y = nullptr;
  long n_samples = 0, cap = 0;
  // batch workspace
  int wcap = 0;
  __nv_bfloat16 *Xb = nullptr, *H1 = nullptr, *H2 = nullptr, *dYb = nullptr, *dZ2b = nullptr, *dZ1b = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *Yo = nullptr, *Tn = nullptr, *dY = nullptr, *dH2 = nullptr, *dZ2 = nullptr,
        *dH1 = nullptr, *dZ1 = nullptr, *rowl = nullptr;
  long* idx = nullptr;
  double* evalbuf = nullptr;
  // projection scratch
  double *pf_K = nullptr, *pc_U = nullptr, *pc_KT = nullptr, *pc_K = nullptr;
  long pf_cap = 0, pc_cap = 0;
  unsigned long long* fallbacks = nullptr;  // [0] elements left uncorrected, [1] elements clipped
  int* ood = nullptr;                       // per element: features outside the training range
  double gw[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // Gauss weights of order p
  ldg_closure_options opt = {0.f, LDG_CLOSURE_ENERGY_DISSIPATIVE, 1.f, 10.f, 1.f, {0, 0, 0}};
};

namespace {

template <class T>
int cl_alloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(LDG_ERR_NOMEM, "closure: cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes");
  }
  return LDG_OK;
}

int ensure_workspace(ldg_closure* c, int B) {
  if (B <= c->wcap) return LDG_OK;
  int cap = std::max(B, 1024);
  void* ptrs[] = {c->Xb, c->H1, c->H2, c->dYb, c->dZ2b, c->dZ1b, c->Z1, c->Z2, c->Yo, c->Tn,
                  c->dY, c->dH2, c->dZ2, c->dH1, c->dZ1, c->rowl, c->idx, c->evalbuf, c->ood};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  const long H = c->hidden, I = c->in_dim, O = c->out_dim;
  int st;
  if ((st = cl_alloc(&c->Xb, (size_t)cap * I)) || (st = cl_alloc(&c->H1, (size_t)cap * H)) ||
      (st = cl_alloc(&c->H2, (size_t)cap * H)) || (st = cl_alloc(&c->dYb, (size_t)cap * O)) ||
      (st = cl_alloc(&c->dZ2b, (size_t)cap * H)) || (st = cl_alloc(&c->dZ1b, (size_t)cap * H)) ||
      (st = cl_alloc(&c->Z1, (size_t)cap * H)) || (st = cl_alloc(&c->Z2, (size_t)cap * H)) ||
      (st = cl_alloc(&c->Yo, (size_t)cap * O)) || (st = cl_alloc(&c->Tn, (size_t)cap * O)) ||
      (st = cl_alloc(&c->dY, (size_t)cap * O)) || (st = cl_alloc(&c->dH2, (size_t)cap * H)) ||
      (st = cl_alloc(&c->dZ2, (size_t)cap * H)) || (st = cl_alloc(&c->dH1, (size_t)cap * H)) ||
      (st = cl_alloc(&c->dZ1, (size_t)cap * H)) || (st = cl_alloc(&c->rowl, (size_t)cap)) ||
      (st = cl_alloc(&c->idx, (size_t)cap)) || (st = cl_alloc(&c->evalbuf, (size_t)cap * 2)) ||
      (st = cl_alloc(&c->ood, (size_t)cap)))
    return st;
  c->wcap = cap;
  return LDG_OK;
}

void gemm(const Mat& A, const Mat& B, float* C, long ldc, int M, int N, int K, int acc, cudaStream_t st) {
  dim3 grid((unsigned)ceil_div(N, kTN), (unsigned)ceil_div(M, kTM));
  k_gemm_bf16<<<grid, 128, 0, st>>>(A, B, C, ldc, M, N, K, acc);
}

// Forward pass on Xb (B rows): Z1, H1, Z2, H2, Yo.
cudaError_t forward(ldg_closure* c, int B) {
  const int I = c->in_dim, H = c->hidden, O = c->out_dim;
  const __nv_bfloat16* W1 = c->wb + c->off[0];
  const __nv_bfloat16* W2 = c->wb + c->off[2];
  const __nv_bfloat16* W3 = c->wb + c->off[4];
  cudaStream_t st = c->stream;
  gemm({c->Xb, I, 1}, {W1, 1, I}, c->Z1, H, B, H, I, 0, st);
  k_bias_act<<<(unsigned)ceil_div((long)B * H, 256), 256, 0, st>>>(c->Z1, c->theta + c->off[1], c->H1, B, H, 1);
  gemm({c->H1, H, 1}, {W2, 1, H}, c->Z2, H, B, H, H, 0, st);
  k_bias_act<<<(unsigned)ceil_div((long)B * H, 256), 256, 0, st>>>(c->Z2, c->theta + c->off[3], c->H2, B, H, 1);
  gemm({c->H2, H, 1}, {W3, 1, H}, c->Yo, O, B, O, H, 0, st);
  k_bias_act<<<(unsigned)ceil_div((long)B * O, 256), 256, 0, st>>>(c->Yo, c->theta + c->off[5], nullptr, B, O, 0);
  return cudaGetLastError();
}

// Backward pass from dY / dYb (B rows) into c->grad.
cudaError_t backward(ldg_closure* c, int B) {
  const int I = c->in_dim, H = c->hidden, O = c->out_dim;
  const __nv_bfloat16* W2 = c->wb + c->off[2];
  const __nv_bfloat16* W3 = c->wb + c->off[4];
  cudaStream_t st = c->stream;
  float* g = c->grad;
  // layer 3
  gemm({c->dYb, 1, O}, {c->H2, H, 1}, g + c->off[4], H, O, H, B, 0, st);  // dW3 = dY^T H2
  k_colsum<<<(unsigned)ceil_div(O, 128), 128, 0, st>>>(c->dY, B, O, g + c->off[5]);
  gemm({c->dYb, O, 1}, {W3, H, 1}, c->dH2, H, B, H, O, 0, st);             // dH2 = dY W3
  k_gelu_back<<<(unsigned)ceil_div((long)B * H, 256), 256, 0, st>>>(c->dH2, c->Z2, c->dZ2, c->dZ2b, (long)B * H);
  // layer 2
  gemm({c->dZ2b, 1, H}, {c->H1, H, 1}, g + c->off[2], H, H, H, B, 0, st);  // dW2 = dZ2^T H1
  k_colsum<<<(unsigned)ceil_div(H, 128), 128, 0, st>>>(c->dZ2, B, H, g + c->off[3]);
  gemm({c->dZ2b, H, 1}, {W2, H, 1}, c->dH1, H, B, H, H, 0, st);            // dH1 = dZ2 W2
  k_gelu_back<<<(unsigned)ceil_div((long)B * H, 256), 256, 0, st>>>(c->dH1, c->Z1, c->dZ1, c->dZ1b, (long)B * H);
  // layer 1
  gemm({c->dZ1b, 1, H}, {c->Xb, I, 1}, g + c->off[0], I, H, I, B, 0, st);  // dW1 = dZ1^T X
  k_colsum<<<(unsigned)ceil_div(H, 128), 128, 0, st>>>(c->dZ1, B, H, g + c->off[1]);
  return cudaGetLastError();
}

int refresh_bf16(ldg_closure* c) {
  k_f2bf<<<(unsigned)ceil_div(c->n_params, 256), 256, 0, c->stream>>>(c->theta, c->wb, c->n_params);
  CL_CUDA(cudaGetLastError());
  return LDG_OK;
}

int ensure_samples(ldg_closure* c, long need) {
  if (need <= c->cap) return LDG_OK;
  long cap = c->cap ? c->cap : 4096;
  while (cap < need) cap *= 2;
  float *nx = nullptr, *ny = nullptr;
  int st;
  if ((st = cl_alloc(&nx, (size_t)cap * c->in_dim)) || (st = cl_alloc(&ny, (size_t)cap * c->out_dim))) {
    if (nx) cudaFree(nx);
    return st;
  }
  if (c->X) {
    CL_CUDA(cudaMemcpyAsync(nx, c->X, sizeof(float) * c->n_samples * c->in_dim, cudaMemcpyDeviceToDevice, c->stream));
    CL_CUDA(cudaMemcpyAsync(ny, c->Y, sizeof(float) * c->n_samples * c->out_dim, cudaMemcpyDeviceToDevice, c->stream));
    CL_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(c->X);
    cudaFree(c->Y);
  }
  c->X = nx;
  c->Y = ny;
  c->cap = cap;
  return LDG_OK;
}

// 1-D projection matrix from r sub-intervals of Nf Gauss points onto Nc
// Gauss-Lagrange functions: P1[a][s*Nf+b] = (w_f[b]/r) L_a(xi_sb) / w_c[a],
// xi_sb = -1 + (2s + 1 + x_f[b]) / r.
std::vector<double> projection_1d(int pf, int pc, int r) {
  Ops1D of, oc;
  build_ops1d(pf, &of);
  build_ops1d(pc, &oc);
  const int Nf = pf + 1, Nc = pc + 1, M = r * Nf;
  std::vector<double> P(Nc * M);
  for (int a = 0; a < Nc; ++a)
    for (int s = 0; s < r; ++s)
      for (int b = 0; b < Nf; ++b) {
        const long double xi = -1.0L + (2.0L * s + 1.0L + of.x[b]) / r;
        long double L = 1.0L;
        for (int k = 0; k < Nc; ++k)
          if (k != a) L *= (xi - oc.x[k]) / ((long double)oc.x[a] - oc.x[k]);
        P[a * M + s * Nf + b] = (double)((of.w[b] / (long double)r) * L / oc.w[a]);
      }
  return P;
}

}  // namespace

namespace ldg {

int closure_check_solver(ldg_closure* c, const SolverView& v) {
  if (v.p != c->p) return fail(LDG_ERR_INVALID, "closure: order differs from the solver's");
  if (v.device != c->device) return fail(LDG_ERR_INVALID, "closure: device differs from the solver's");
  if (!c->stats_ready) return fail(LDG_ERR_INVALID, "closure: normalisation not finalised");
  return ensure_workspace(c, v.nE);
}

int closure_correction(ldg_closure* c, const SolverView& v, const double* U, const double* Q, double* Kadd,
                       cudaStream_t st) {
  cudaStream_t keep = c->stream;
  c->stream = st;  // run on the solver's stream
  int rc = ensure_workspace(c, v.nE);
  if (!rc) {
    const float* s = c->stats;
    cudaError_t e = cudaMemsetAsync(c->ood, 0, sizeof(int) * v.nE, st);
    if (e == cudaSuccess) {
      k_features<<<(unsigned)ceil_div((long)v.nE * c->in_dim, 256), 256, 0, st>>>(U, Q, v.nE, c->n, s, s + 20,
                                                                                   c->Xb, c->ood, c->opt.ood_sigma);
      e = forward(c, v.nE);
    }
    if (e == cudaSuccess) {
      GaussW gw;
      for (int i = 0; i < 8; ++i) gw.w[i] = c->gw[i];
      k_correction<<<v.nE, 128, 0, st>>>(c->Yo, U, v.nE, c->N, s + 40, s + 45, gw, c->ood, c->opt.energy,
                                         (double)c->opt.scale, Kadd, c->fallbacks);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) rc = fail(LDG_ERR_CUDA, std::string("closure inference: ") + cudaGetErrorString(e));
  }
  c->stream = keep;
  return rc;
}

}  // namespace ldg

extern "C" {

int ldg_closure_create(int p, int hidden, unsigned long long seed, int device, ldg_closure** out) {
  if (!out || p < 1 || p > 6 || hidden < 16 || hidden > 1024) return fail(LDG_ERR_INVALID, "closure: bad arguments");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(LDG_ERR_NODEVICE, "no CUDA device");
  }
  ldg_closure* c = new ldg_closure();
  c->p = p;
  c->N = p + 1;
  c->n = c->N * c->N * c->N;
  {
    Ops1D o1;
    if (!build_ops1d(p, &o1)) {
      delete c;
      return fail(LDG_ERR_UNSUPPORTED, "closure: no Gauss rule for this order");
    }
    for (int i = 0; i < c->N; ++i) c->gw[i] = o1.w[i];
  }
  c->in_dim = kChIn * c->n;
  c->out_dim = kChOut * c->n;
  c->hidden = hidden;
  c->device = device;
  const long I = c->in_dim, H = hidden, O = c->out_dim;
  c->off[0] = 0;
  c->off[1] = H * I;
  c->off[2] = c->off[1] + H;
  c->off[3] = c->off[2] + H * H;
  c->off[4] = c->off[3] + H;
  c->off[5] = c->off[4] + O * H;
  c->n_params = c->off[5] + O;
  int st;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) {
    delete c;
    return fail(LDG_ERR_CUDA, "closure: device/stream");
  }
  if ((st = cl_alloc(&c->theta, c->n_params)) || (st = cl_alloc(&c->grad, c->n_params)) ||
      (st = cl_alloc(&c->m, c->n_params)) || (st = cl_alloc(&c->v, c->n_params)) ||
      (st = cl_alloc(&c->wb, c->n_params)) || (st = cl_alloc(&c->stats, 64)) ||
      (st = cl_alloc(&c->fallbacks, 2))) {
    ldg_closure_destroy(c);
    return st;
  }
  // Initialisation: N(0, 1/fan_in) weights (last layer scaled by 0.1 so the
  // untrained correction is small), zero biases; seeded, deterministic.
  std::vector<float> h(c->n_params, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](long o, long rows, long cols, double scale) {
    std::normal_distribution<double> nd(0.0, scale / std::sqrt((double)cols));
    for (long i = 0; i < rows * cols; ++i) h[o + i] = (float)nd(rng);
  };
  fill(c->off[0], H, I, 1.0);
  fill(c->off[2], H, H, 1.0);
  fill(c->off[4], O, H, 0.1);
  std::vector<float> stats(64, 0.f);
  for (int i = 0; i < 20; ++i) stats[20 + i] = 1.f;
  for (int i = 0; i < 5; ++i) stats[45 + i] = 1.f;
  if (cudaMemcpy(c->theta, h.data(), sizeof(float) * c->n_params, cudaMemcpyHostToDevice) ||
      cudaMemset(c->m, 0, sizeof(float) * c->n_params) || cudaMemset(c->v, 0, sizeof(float) * c->n_params) ||
      cudaMemcpy(c->stats, stats.data(), sizeof(float) * 64, cudaMemcpyHostToDevice) ||
      cudaMemset(c->fallbacks, 0, 2 * sizeof(unsigned long long))) {
    ldg_closure_destroy(c);
    return fail(LDG_ERR_CUDA, "closure: initial upload");
  }
  if ((st = refresh_bf16(c)) || (st = ensure_workspace(c, 1024))) {
    ldg_closure_destroy(c);
    return st;
  }
  CL_CUDA(cudaStreamSynchronize(c->stream));
  *out = c;
  return LDG_OK;
}

int ldg_closure_destroy(ldg_closure* c) {
  if (!c) return LDG_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* ptrs[] = {c->theta, c->grad, c->m, c->v, c->wb, c->stats, c->X, c->Y, c->Xb, c->H1, c->H2,
                  c->dYb, c->dZ2b, c->dZ1b, c->Z1, c->Z2, c->Yo, c->Tn, c->dY, c->dH2, c->dZ2, c->dH1,
                  c->dZ1, c->rowl, c->idx, c->evalbuf, c->pf_K, c->pc_U, c->pc_KT, c->pc_K, c->fallbacks,
                  c->ood};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return LDG_OK;
}

namespace {

// What add_samples does with the coarse side.
enum class SampleMode {
  kProjected,  // features of the projected fine state (the coarse state is not touched)
  kCoarse,     // features of the coarse solver's own current state
  kSetState,   // no samples: the projected fine state becomes the coarse state
};

int add_samples_impl(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse, SampleMode mode) {
  if (!c || !fine || !coarse) return fail(LDG_ERR_INVALID, "closure: null argument");
  const SolverView f = solver_view(fine), k = solver_view(coarse);
  if (k.p != c->p) return fail(LDG_ERR_INVALID, "closure: coarse order differs");
  if (f.mixed || k.mixed) return fail(LDG_ERR_UNSUPPORTED, "closure data needs FP64 solvers");
  if (f.nx % k.nx || f.ny % k.ny || f.nz % k.nz || f.nx / k.nx != f.ny / k.ny || f.nx / k.nx != f.nz / k.nz)
    return fail(LDG_ERR_INVALID, "closure: the fine mesh must refine the coarse mesh uniformly");
  if (f.device != c->device || k.device != c->device) return fail(LDG_ERR_INVALID, "closure: devices differ");
  const int r = f.nx / k.nx, Nf = f.N, Nc = k.N;
  CL_CUDA(cudaSetDevice(c->device));
  // everything below runs on the coarse solver's stream after both
  // solvers' queued work
  CL_CUDA(cudaStreamSynchronize(f.stream));
  CL_CUDA(cudaStreamSynchronize(k.stream));
  cudaStream_t st = k.stream;
  const long fsz = (long)f.nE * 5 * f.n, csz = (long)k.nE * 5 * k.n;
  int rc;
  if (fsz > c->pf_cap) {
    if (c->pf_K) cudaFree(c->pf_K);
    if ((rc = cl_alloc(&c->pf_K, fsz))) return rc;
    c->pf_cap = fsz;
  }
  if (csz > c->pc_cap) {
    double* old[] = {c->pc_U, c->pc_KT, c->pc_K};
    for (double* p : old)
      if (p) cudaFree(p);
    if ((rc = cl_alloc(&c->pc_U, csz)) || (rc = cl_alloc(&c->pc_KT, csz)) || (rc = cl_alloc(&c->pc_K, csz))) return rc;
    c->pc_cap = csz;
  }
  std::vector<double> P1 = projection_1d(f.p, k.p, r);
  double* dP = nullptr;
  if ((rc = cl_alloc(&dP, P1.size()))) return rc;
  CL_CUDA(cudaMemcpyAsync(dP, P1.data(), sizeof(double) * P1.size(), cudaMemcpyHostToDevice, st));
  const int M = r * Nf;
  const size_t smem = sizeof(double) * 5 * ((size_t)M * M * M + (size_t)M * M * Nc + (size_t)M * Nc * Nc);
  CL_CUDA(cudaFuncSetAttribute(k_project, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (mode == SampleMode::kSetState) {
    k_project<<<k.nE, 256, smem, st>>>(f.Un, c->pc_U, k.nx, k.ny, k.nz, r, Nf, Nc, 5, dP);
    CL_CUDA(cudaGetLastError());
    rc = solver_set_gauss_state(coarse, c->pc_U);
    CL_CUDA(cudaStreamSynchronize(st));
    cudaFree(dP);
    return rc;
  }
  // fine RHS of the fine state (Gauss basis), projected onto the coarse mesh
  if ((rc = solver_rhs_gauss(fine, f.Un, c->pf_K))) return rc;
  CL_CUDA(cudaStreamSynchronize(f.stream));
  k_project<<<k.nE, 256, smem, st>>>(c->pf_K, c->pc_KT, k.nx, k.ny, k.nz, r, Nf, Nc, 5, dP);
  // the state whose features the sample carries
  if (mode == SampleMode::kProjected)
    k_project<<<k.nE, 256, smem, st>>>(f.Un, c->pc_U, k.nx, k.ny, k.nz, r, Nf, Nc, 5, dP);
  else
    CL_CUDA(cudaMemcpyAsync(c->pc_U, k.Un, sizeof(double) * csz, cudaMemcpyDeviceToDevice, st));
  CL_CUDA(cudaGetLastError());
  // coarse gradient and RHS of that state
  if ((rc = solver_rhs_gauss(coarse, c->pc_U, c->pc_K))) return rc;
  if ((rc = ensure_samples(c, c->n_samples + k.nE))) return rc;
  const long total = (long)k.nE * c->in_dim;
  k_make_rows<<<(unsigned)ceil_div(total, 256), 256, 0, st>>>(c->pc_U, k.Q, c->pc_KT, c->pc_K, k.nE, k.n,
                                                               c->X + c->n_samples * c->in_dim,
                                                               c->Y + c->n_samples * c->out_dim);
  CL_CUDA(cudaGetLastError());
  CL_CUDA(cudaStreamSynchronize(st));
  cudaFree(dP);
  c->n_samples += k.nE;
  return LDG_OK;
}

}  // namespace

int ldg_closure_add_samples(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse) {
  return add_samples_impl(c, fine, coarse, SampleMode::kProjected);
}

int ldg_closure_add_samples_coarse(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse) {
  return add_samples_impl(c, fine, coarse, SampleMode::kCoarse);
}

int ldg_closure_project_state(ldg_closure* c, ldg_solver* fine, ldg_solver* coarse) {
  return add_samples_impl(c, fine, coarse, SampleMode::kSetState);
}

int ldg_closure_sample_count(const ldg_closure* c, long long* count) {
  if (!c || !count) return fail(LDG_ERR_INVALID, "closure: null argument");
  *count = c->n_samples;
  return LDG_OK;
}

int ldg_closure_finalize_data(ldg_closure* c, long long first, long long count) {
  if (!c || first < 0 || count <= 0 || first + count > c->n_samples)
    return fail(LDG_ERR_INVALID, "closure: bad sample range");
  CL_CUDA(cudaSetDevice(c->device));
  k_channel_stats<<<kChIn, 256, 0, c->stream>>>(c->X + first * c->in_dim, count, kChIn, c->n, c->stats,
                                                c->stats + 20);
  k_channel_stats<<<kChOut, 256, 0, c->stream>>>(c->Y + first * c->out_dim, count, kChOut, c->n, c->stats + 40,
                                                 c->stats + 45);
  CL_CUDA(cudaGetLastError());
  CL_CUDA(cudaStreamSynchronize(c->stream));
  c->stats_ready = true;
  return LDG_OK;
}

int ldg_closure_train(ldg_closure* c, long long first, long long count, int iters, int batch, float lr,
                      unsigned long long seed, float* losses) {
  if (!c || iters < 0 || batch <= 0 || count <= 0 || first < 0 || first + count > c->n_samples)
    return fail(LDG_ERR_INVALID, "closure: bad training arguments");
  if (!c->stats_ready) return fail(LDG_ERR_INVALID, "closure: normalisation not finalised");
  CL_CUDA(cudaSetDevice(c->device));
  int rc;
  if ((rc = ensure_workspace(c, batch))) return rc;
  std::mt19937_64 rng(seed);
  std::uniform_int_distribution<long long> pick(first, first + count - 1);
  std::vector<long> idx(batch);
  float* d_loss = nullptr;
  if ((rc = cl_alloc(&d_loss, std::max(iters, 1)))) return rc;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float* s = c->stats;
  for (int it = 0; it < iters; ++it) {
    for (int b = 0; b < batch; ++b) idx[b] = (long)pick(rng);
    CL_CUDA(cudaMemcpyAsync(c->idx, idx.data(), sizeof(long) * batch, cudaMemcpyHostToDevice, c->stream));
    k_gather_norm<<<(unsigned)ceil_div((long)batch * c->in_dim, 256), 256, 0, c->stream>>>(
        c->X, c->Y, c->idx, batch, c->n, s, s + 20, s + 40, s + 45, c->Xb, c->Tn, c->opt.input_noise,
        seed * 0x100000001B3ULL + (unsigned long long)it);
    CL_CUDA(forward(c, batch));
    k_mse_grad<<<(unsigned)ceil_div(batch, 128), 128, 0, c->stream>>>(c->Yo, c->Tn, c->dY, c->dYb, batch,
                                                                      c->out_dim, c->rowl);
    k_colsum<<<1, 1, 0, c->stream>>>(c->rowl, batch, 1, d_loss + it);
    CL_CUDA(backward(c, batch));
    c->adam_t += 1;
    const float c1 = 1.f - std::pow(b1, (float)c->adam_t), c2 = 1.f - std::pow(b2, (float)c->adam_t);
    // cosine decay from lr to lr * lr_final over the call (constant when lr_final = 1)
    const float frac = iters > 1 ? (float)it / (float)(iters - 1) : 0.f;
    const float lr_it = lr * (c->opt.lr_final + (1.f - c->opt.lr_final) * 0.5f * (1.f + std::cos(3.14159265f * frac)));
    k_adam<<<(unsigned)ceil_div(c->n_params, 256), 256, 0, c->stream>>>(
        c->theta, c->grad, c->m, c->v, c->wb, nullptr, 1, 1, c->n_params, lr_it, b1, b2, eps, c1, c2);
    CL_CUDA(cudaGetLastError());
    // the bf16 copies of the biases are unused; the weights' are refreshed
    // by k_adam (same offsets)
  }
  if (losses && iters > 0)
    CL_CUDA(cudaMemcpyAsync(losses, d_loss, sizeof(float) * iters, cudaMemcpyDeviceToHost, c->stream));
  CL_CUDA(cudaStreamSynchronize(c->stream));
  cudaFree(d_loss);
  return LDG_OK;
}

int ldg_closure_evaluate(ldg_closure* c, long long first, long long count, double* err_plain, double* err_closure) {
  if (!c || first < 0 || count <= 0 || first + count > c->n_samples)
    return fail(LDG_ERR_INVALID, "closure: bad sample range");
  if (!c->stats_ready) return fail(LDG_ERR_INVALID, "closure: normalisation not finalised");
  CL_CUDA(cudaSetDevice(c->device));
  const int B = (int)std::min<long long>(count, 8192);
  int rc;
  if ((rc = ensure_workspace(c, B))) return rc;
  double sp = 0.0, sc = 0.0;
  std::vector<long> idx(B);
  std::vector<double> rows(2 * (size_t)B);
  const float* s = c->stats;
  for (long long b0 = first; b0 < first + count; b0 += B) {
    const int nb = (int)std::min<long long>(B, first + count - b0);
    for (int i = 0; i < nb; ++i) idx[i] = (long)(b0 + i);
    CL_CUDA(cudaMemcpyAsync(c->idx, idx.data(), sizeof(long) * nb, cudaMemcpyHostToDevice, c->stream));
    k_gather_norm<<<(unsigned)ceil_div((long)nb * c->in_dim, 256), 256, 0, c->stream>>>(
        c->X, c->Y, c->idx, nb, c->n, s, s + 20, s + 40, s + 45, c->Xb, c->Tn, 0.f, 0ULL);
    CL_CUDA(forward(c, nb));
    k_eval_rows<<<(unsigned)ceil_div(nb, 128), 128, 0, c->stream>>>(c->Yo, c->Tn, nb, c->n, s + 40, s + 45,
                                                                    c->evalbuf);
    CL_CUDA(cudaMemcpyAsync(rows.data(), c->evalbuf, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, c->stream));
    CL_CUDA(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nb; ++i) {
      sp += rows[2 * i];
      sc += rows[2 * i + 1];
    }
  }
  const double denom = (double)count * c->out_dim;
  if (err_plain) *err_plain = sp / denom;
  if (err_closure) *err_closure = sc / denom;
  return LDG_OK;
}

int ldg_closure_param_count(const ldg_closure* c, long long* count) {
  if (!c || !count) return fail(LDG_ERR_INVALID, "closure: null argument");
  *count = c->n_params;
  return LDG_OK;
}

int ldg_closure_get_params(ldg_closure* c, float* out) {
  if (!c || !out) return fail(LDG_ERR_INVALID, "closure: null argument");
  CL_CUDA(cudaMemcpyAsync(out, c->theta, sizeof(float) * c->n_params, cudaMemcpyDeviceToHost, c->stream));
  CL_CUDA(cudaStreamSynchronize(c->stream));
  return LDG_OK;
}

int ldg_closure_set_params(ldg_closure* c, const float* in) {
  if (!c || !in) return fail(LDG_ERR_INVALID, "closure: null argument");
  CL_CUDA(cudaMemcpyAsync(c->theta, in, sizeof(float) * c->n_params, cudaMemcpyHostToDevice, c->stream));
  // new parameters restart the optimiser
  CL_CUDA(cudaMemsetAsync(c->m, 0, sizeof(float) * c->n_params, c->stream));
  CL_CUDA(cudaMemsetAsync(c->v, 0, sizeof(float) * c->n_params, c->stream));
  c->adam_t = 0;
  int rc = refresh_bf16(c);
  if (rc) return rc;
  CL_CUDA(cudaStreamSynchronize(c->stream));
  return LDG_OK;
}

int ldg_closure_get_stats(ldg_closure* c, float* out50) {
  if (!c || !out50) return fail(LDG_ERR_INVALID, "closure: null argument");
  CL_CUDA(cudaMemcpyAsync(out50, c->stats, sizeof(float) * 50, cudaMemcpyDeviceToHost, c->stream));
  CL_CUDA(cudaStreamSynchronize(c->stream));
  return LDG_OK;
}

int ldg_closure_mlp_forward(ldg_closure* c, const float* x, float* y, int batch) {
  if (!c || !x || !y || batch <= 0) return fail(LDG_ERR_INVALID, "closure: bad arguments");
  CL_CUDA(cudaSetDevice(c->device));
  int rc;
  if ((rc = ensure_workspace(c, batch))) return rc;
  float* dx = nullptr;
  if ((rc = cl_alloc(&dx, (size_t)batch * c->in_dim))) return rc;
  CL_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * batch * c->in_dim, cudaMemcpyHostToDevice, c->stream));
  k_f2bf<<<(unsigned)ceil_div((long)batch * c->in_dim, 256), 256, 0, c->stream>>>(dx, c->Xb, (long)batch * c->in_dim);
  CL_CUDA(forward(c, batch));
  CL_CUDA(cudaMemcpyAsync(y, c->Yo, sizeof(float) * batch * c->out_dim, cudaMemcpyDeviceToHost, c->stream));
  CL_CUDA(cudaStreamSynchronize(c->stream));
  cudaFree(dx);
  return LDG_OK;
}

int ldg_closure_mlp_backward(ldg_closure* c, const float* x, const float* dy, int batch, float* grad) {
  if (!c || !x || !dy || !grad || batch <= 0) return fail(LDG_ERR_INVALID, "closure: bad arguments");
  CL_CUDA(cudaSetDevice(c->device));
  int rc;
  if ((rc = ensure_workspace(c, batch))) return rc;
  float* dx = nullptr;
  if ((rc = cl_alloc(&dx, (size_t)batch * c->in_dim))) return rc;
  CL_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * batch * c->in_dim, cudaMemcpyHostToDevice, c->stream));
  k_f2bf<<<(unsigned)ceil_div((long)batch * c->in_dim, 256), 256, 0, c->stream>>>(dx, c->Xb, (long)batch * c->in_dim);
  CL_CUDA(forward(c, batch));
  CL_CUDA(cudaMemcpyAsync(c->dY, dy, sizeof(float) * batch * c->out_dim, cudaMemcpyHostToDevice, c->stream));
  k_f2bf<<<(unsigned)ceil_div((long)batch * c->out_dim, 256), 256, 0, c->stream>>>(c->dY, c->dYb,
                                                                                   (long)batch * c->out_dim);
  CL_CUDA(backward(c, batch));
  CL_CUDA(cudaMemcpyAsync(grad, c->grad, sizeof(float) * c->n_params, cudaMemcpyDeviceToHost, c->stream));
  CL_CUDA(cudaStreamSynchronize(c->stream));
  cudaFree(dx);
  return LDG_OK;
}

int ldg_closure_get_samples(ldg_closure* c, long long first, long long count, float* X, float* Y) {
  if (!c || first < 0 || count <= 0 || first + count > c->n_samples)
    return fail(LDG_ERR_INVALID, "closure: bad sample range");
  CL_CUDA(cudaSetDevice(c->device));
  if (X)
    CL_CUDA(cudaMemcpyAsync(X, c->X + first * c->in_dim, sizeof(float) * count * c->in_dim,
                            cudaMemcpyDeviceToHost, c->stream));
  if (Y)
    CL_CUDA(cudaMemcpyAsync(Y, c->Y + first * c->out_dim, sizeof(float) * count * c->out_dim,
                            cudaMemcpyDeviceToHost, c->stream));
  CL_CUDA(cudaStreamSynchronize(c->stream));
  return LDG_OK;
}

int ldg_closure_fallbacks(ldg_closure* c, long long* count) {
  return ldg_closure_counters(c, count, nullptr);
}

int ldg_closure_get_options(const ldg_closure* c, ldg_closure_options* o) {
  if (!c || !o) return fail(LDG_ERR_INVALID, "closure: null argument");
  *o = c->opt;
  return LDG_OK;
}

int ldg_closure_set_options(ldg_closure* c, const ldg_closure_options* o) {
  if (!c || !o) return fail(LDG_ERR_INVALID, "closure: null argument");
  if (!(o->input_noise >= 0.f) || o->energy < 0 || o->energy > 2 || !(o->scale >= 0.f) || !(o->ood_sigma > 0.f) ||
      !(o->lr_final > 0.f && o->lr_final <= 1.f))
    return fail(LDG_ERR_INVALID, "closure: bad options");
  c->opt = *o;
  return LDG_OK;
}

int ldg_closure_counters(ldg_closure* c, long long* fallbacks, long long* clipped) {
  if (!c || (!fallbacks && !clipped)) return fail(LDG_ERR_INVALID, "closure: null argument");
  unsigned long long h[2] = {0, 0};
  CL_CUDA(cudaMemcpy(h, c->fallbacks, sizeof(h), cudaMemcpyDeviceToHost));
  if (fallbacks) *fallbacks = (long long)h[0];
  if (clipped) *clipped = (long long)h[1];
  return LDG_OK;
}

}  // extern "C"
