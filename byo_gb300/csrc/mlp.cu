// mlp.cu -- the learned direction / update policy: a 16-32-32-5 FP32 MLP
// (ReLU, ReLU, linear) that predicts log-time of five actions:
//   0 push, 1 pull, 2 blocked      (per edgeMap round, from frontier statistics)
//   3 in-place merge, 4 rebuild    (per container update, from batch statistics)
// The choice never changes a result, only speed.  GBBS's m/20 rule stays the
// fallback (no trained network) and the arbiter: the network's pick replaces the
// rule's only when it predicts a gain of more than kArbiterMargin.
//
// Training is on the device with the kernels below: one CTA runs Adam over
// minibatches of kMb samples; activations of a minibatch sit in shared memory,
// every parameter's gradient is a short loop over the minibatch (no atomics),
// so the update is deterministic.  Loss: mean over the observed targets of
// (y - t)^2, targets t = log2(1 + time_us) / 16.
#include <cmath>
#include <cstring>
#include <vector>

#include "device.cuh"
#include "engine.h"
#include "internal.h"
#include "policy.cuh"

namespace byo {

constexpr int kMb = 128;

struct Mlp {
  float *d_params = nullptr;    // kParams, the network used for inference
  std::vector<float> h_params;  // host copy
  bool trained = false;
};

// ---------------------------------------------------------------- forward pieces
__device__ __forceinline__ void mlp_forward(const float *P, const float *x, float *h1, float *h2, float *y) {
  for (int j = 0; j < kH; j++) {
    float a = P[kB1 + j];
    for (int k = 0; k < kIn; k++) a = fmaf(P[kW1 + j * kIn + k], x[k], a);
    h1[j] = a > 0.f ? a : 0.f;
  }
  for (int j = 0; j < kH; j++) {
    float a = P[kB2 + j];
    for (int k = 0; k < kH; k++) a = fmaf(P[kW2 + j * kH + k], h1[k], a);
    h2[j] = a > 0.f ? a : 0.f;
  }
  for (int o = 0; o < kOut; o++) {
    float a = P[kB3 + o];
    for (int k = 0; k < kH; k++) a = fmaf(P[kW3 + o * kH + k], h2[k], a);
    y[o] = a;
  }
}

__global__ void k_mlp_forward(const float *__restrict__ P, const float *__restrict__ X, uint64_t n, float *Y) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    float x[kIn], h1[kH], h2[kH], y[kOut];
    for (int k = 0; k < kIn; k++) x[k] = X[i * kIn + k];
    mlp_forward(P, x, h1, h2, y);
    for (int o = 0; o < kOut; o++) Y[i * kOut + o] = y[o];
  }
}

// ---------------------------------------------------------------- training
// Shared-memory layout of one minibatch (kMb samples).
struct MbSmem {
  float x[kMb][kIn];
  float h1[kMb][kH];
  float h2[kMb][kH];
  float dy[kMb][kOut];
  float dh1[kMb][kH];
  float dh2[kMb][kH];
};

// Loss and gradient of one minibatch [i0, i1) (order given by perm); the
// gradient of every parameter is written to g (thread-owned parameters).
__device__ void mb_loss_grad(const float *P, const float *__restrict__ X, const float *__restrict__ Y,
                             const uint8_t *__restrict__ M, const uint32_t *__restrict__ perm, uint64_t i0,
                             uint64_t i1, float inv_cnt, MbSmem &S, float *g, float *loss_acc) {
  const int nb = (int)(i1 - i0);
  for (int s = threadIdx.x; s < kMb; s += blockDim.x) {
    if (s < nb) {
      const uint64_t i = perm ? perm[i0 + s] : i0 + s;
      float y[kOut];
      for (int k = 0; k < kIn; k++) S.x[s][k] = X[i * kIn + k];
      mlp_forward(P, S.x[s], S.h1[s], S.h2[s], y);
      float l = 0.f;
      for (int o = 0; o < kOut; o++) {
        const bool m = (M[i] >> o) & 1u;
        const float d = m ? y[o] - Y[i * kOut + o] : 0.f;
        l += d * d;
        S.dy[s][o] = 2.f * d * inv_cnt;
      }
      atomicAdd(loss_acc, l * inv_cnt);
    } else {
      for (int k = 0; k < kIn; k++) S.x[s][k] = 0.f;
      for (int k = 0; k < kH; k++) S.h1[s][k] = S.h2[s][k] = 0.f;
      for (int o = 0; o < kOut; o++) S.dy[s][o] = 0.f;
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < kMb; s += blockDim.x) {
    for (int j = 0; j < kH; j++) {
      float a = 0.f;
      for (int o = 0; o < kOut; o++) a = fmaf(P[kW3 + o * kH + j], S.dy[s][o], a);
      S.dh2[s][j] = S.h2[s][j] > 0.f ? a : 0.f;
    }
    for (int k = 0; k < kH; k++) {
      float a = 0.f;
      for (int j = 0; j < kH; j++) a = fmaf(P[kW2 + j * kH + k], S.dh2[s][j], a);
      S.dh1[s][k] = S.h1[s][k] > 0.f ? a : 0.f;
    }
  }
  __syncthreads();
  for (int p = threadIdx.x; p < kParams; p += blockDim.x) {
    float a = 0.f;
    if (p < kB1) {
      const int j = p / kIn, k = p % kIn;
      for (int s = 0; s < kMb; s++) a = fmaf(S.dh1[s][j], S.x[s][k], a);
    } else if (p < kW2) {
      const int j = p - kB1;
      for (int s = 0; s < kMb; s++) a += S.dh1[s][j];
    } else if (p < kB2) {
      const int j = (p - kW2) / kH, k = (p - kW2) % kH;
      for (int s = 0; s < kMb; s++) a = fmaf(S.dh2[s][j], S.h1[s][k], a);
    } else if (p < kW3) {
      const int j = p - kB2;
      for (int s = 0; s < kMb; s++) a += S.dh2[s][j];
    } else if (p < kB3) {
      const int o = (p - kW3) / kH, k = (p - kW3) % kH;
      for (int s = 0; s < kMb; s++) a = fmaf(S.dy[s][o], S.h2[s][k], a);
    } else {
      const int o = p - kB3;
      for (int s = 0; s < kMb; s++) a += S.dy[s][o];
    }
    g[p] = a;
  }
  __syncthreads();
}

// Whole-batch loss and gradient (mean over every observed target), summed
// minibatch by minibatch; used by the gradient check.
__global__ void __launch_bounds__(256) k_mlp_loss_grad(const float *__restrict__ P, const float *__restrict__ X,
                                                       const float *__restrict__ Y, const uint8_t *__restrict__ M,
                                                       uint64_t n, float inv_cnt, float *grad, float *loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  MbSmem &S = *reinterpret_cast<MbSmem *>(smem);
  float *g = reinterpret_cast<float *>(smem + sizeof(MbSmem));
  __shared__ float lacc;
  if (threadIdx.x == 0) lacc = 0.f;
  for (int p = threadIdx.x; p < kParams; p += blockDim.x) grad[p] = 0.f;
  __syncthreads();
  for (uint64_t i0 = 0; i0 < n; i0 += kMb) {
    const uint64_t i1 = i0 + kMb < n ? i0 + kMb : n;
    mb_loss_grad(P, X, Y, M, nullptr, i0, i1, inv_cnt, S, g, &lacc);
    for (int p = threadIdx.x; p < kParams; p += blockDim.x) grad[p] += g[p];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = lacc;
}

// Adam (Kingma & Ba 2015) over `epochs` passes; perm is reshuffled on the host
// side once (a fixed permutation keeps the run deterministic).
__global__ void __launch_bounds__(256) k_mlp_train(float *P, const float *__restrict__ X, const float *__restrict__ Y,
                                                   const uint8_t *__restrict__ M, const uint32_t *__restrict__ perm,
                                                   uint64_t n, uint32_t epochs, float lr, float *mom, float *vel,
                                                   float *loss_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  MbSmem &S = *reinterpret_cast<MbSmem *>(smem);
  float *g = reinterpret_cast<float *>(smem + sizeof(MbSmem));
  float *Ps = g + kParams;  // parameters in shared memory
  __shared__ float lacc;
  for (int p = threadIdx.x; p < kParams; p += blockDim.x) Ps[p] = P[p];
  __syncthreads();
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  uint64_t step = 0;
  for (uint32_t e = 0; e < epochs; e++) {
    if (threadIdx.x == 0) lacc = 0.f;
    __syncthreads();
    for (uint64_t i0 = 0; i0 < n; i0 += kMb) {
      const uint64_t i1 = i0 + kMb < n ? i0 + kMb : n;
      // per-minibatch mean over its observed targets
      float cnt = 0.f;
      for (uint64_t i = i0; i < i1; i++) cnt += (float)__popc((unsigned)M[perm[i]]);
      const float inv = cnt > 0.f ? 1.f / cnt : 0.f;
      mb_loss_grad(Ps, X, Y, M, perm, i0, i1, inv, S, g, &lacc);
      step++;
      const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
      for (int p = threadIdx.x; p < kParams; p += blockDim.x) {
        const float gp = g[p];
        const float m = b1 * mom[p] + (1.f - b1) * gp;
        const float v = b2 * vel[p] + (1.f - b2) * gp * gp;
        mom[p] = m;
        vel[p] = v;
        Ps[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0 && loss_out) loss_out[e] = lacc;
  }
  for (int p = threadIdx.x; p < kParams; p += blockDim.x) P[p] = Ps[p];
}

// ---------------------------------------------------------------- round policy (inference)
// Stand-alone launch of the round policy, for the frontier a traversal starts
// from (later rounds run it as the epilogue of their last kernel).
__global__ void k_round_policy(const float *__restrict__ P, RoundStats *st, float n, float m, float reached_before,
                               int dense, int has_net, int log) {
  round_policy_warp(P, st, n, m, reached_before, dense, has_net, log);
}

// ---------------------------------------------------------------- host side

static int policy_get(byo_ctx *ctx, Mlp **out) {
  if (!ctx->policy) {
    Mlp *p = new Mlp();
    p->h_params.assign(kParams, 0.f);
    cudaError_t e = cudaMalloc(&p->d_params, kParams * sizeof(float));
    if (e != cudaSuccess) {
      delete p;
      return set_error(ctx, BYO_ENOMEM, "policy params", e);
    }
    ctx->policy = p;
  }
  *out = ctx->policy;
  return BYO_OK;
}

void policy_destroy(Mlp *p) {
  if (!p) return;
  if (p->d_params) cudaFree(p->d_params);
  delete p;
}

bool policy_trained(const byo_ctx *ctx) { return ctx->policy && ctx->policy->trained; }
const float *policy_params(const byo_ctx *ctx) { return ctx->policy ? ctx->policy->d_params : nullptr; }

int round_policy(byo_graph *g, RoundStats *d_st, uint64_t reached_before, bool this_round_dense) {
  byo_ctx *ctx = g->ctx;
  const bool net = policy_trained(ctx);
  launch(ctx, k_round_policy, dim3(1), dim3(32), 0, policy_params(ctx), d_st, (float)g->n, (float)g->m,
         (float)reached_before, this_round_dense ? 1 : 0, net ? 1 : 0, ctx->time_rounds ? 1 : 0);
  return check_launch(ctx, "round_policy");
}

int policy_tail_args(byo_graph *g, unsigned int *done, uint64_t reached_before, bool this_round_dense,
                     PolicyTail *pt) {
  byo_ctx *ctx = g->ctx;
  pt->P = policy_params(ctx);
  pt->n = (float)g->n;
  pt->m = (float)g->m;
  pt->reached_before = (float)reached_before;
  pt->dense = this_round_dense ? 1 : 0;
  pt->has_net = policy_trained(ctx) ? 1 : 0;
  pt->on = 1;
  pt->log = ctx->time_rounds ? 1 : 0;
  pt->done = done;
  return BYO_OK;
}

// Xavier-uniform initialisation from a counter-based stream (seeded).
static void init_params(std::vector<float> &P, uint64_t seed) {
  auto u01 = [&](uint64_t i) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + (i + 1) * 0xD1B54A32D192ED03ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) / 9007199254740992.0;
  };
  P.assign(kParams, 0.f);
  auto fill = [&](int off, int fan_out, int fan_in) {
    const double a = std::sqrt(6.0 / (fan_in + fan_out));
    for (int i = 0; i < fan_out * fan_in; i++) P[off + i] = (float)((2.0 * u01(off + i) - 1.0) * a);
  };
  fill(kW1, kH, kIn);
  fill(kW2, kH, kH);
  fill(kW3, kOut, kH);
}

// Host mirror of the forward pass (the update policy runs once per batch).
static void forward_host(const std::vector<float> &P, const float *x, float *y) {
  float h1[kH], h2[kH];
  for (int j = 0; j < kH; j++) {
    float a = P[kB1 + j];
    for (int k = 0; k < kIn; k++) a = std::fmaf(P[kW1 + j * kIn + k], x[k], a);
    h1[j] = a > 0.f ? a : 0.f;
  }
  for (int j = 0; j < kH; j++) {
    float a = P[kB2 + j];
    for (int k = 0; k < kH; k++) a = std::fmaf(P[kW2 + j * kH + k], h1[k], a);
    h2[j] = a > 0.f ? a : 0.f;
  }
  for (int o = 0; o < kOut; o++) {
    float a = P[kB3 + o];
    for (int k = 0; k < kH; k++) a = std::fmaf(P[kW3 + o * kH + k], h2[k], a);
    y[o] = a;
  }
}

void update_features(uint64_t batch, uint64_t m, uint64_t slots, int sorted, int insert, float *x) {
  const float inv = 1.f / 32.f;
  for (int i = 0; i < kIn; i++) x[i] = 0.f;
  x[0] = std::log2((float)batch + 1.f) * inv;
  x[1] = std::log2((float)m + 1.f) * inv;
  x[2] = std::log2((float)slots + 1.f) * inv;
  x[3] = slots ? (float)m / (float)slots : 0.f;
  x[4] = m ? std::fmin((float)batch / (float)m, 4.f) : 4.f;
  x[5] = sorted ? 1.f : 0.f;
  x[6] = insert ? 1.f : 0.f;
  x[15] = 1.f;  // marks an update sample
}

// 0 = in-place merge (the default and fallback), 1 = rebuild
int update_strategy(byo_ctx *ctx, uint64_t batch, uint64_t m, uint64_t slots, int sorted, int insert) {
  if (!policy_trained(ctx)) return 0;
  float x[kIn], y[kOut];
  update_features(batch, m, slots, sorted, insert, x);
  forward_host(ctx->policy->h_params, x, y);
  return (y[3] - y[4] > kArbiterMargin) ? 1 : 0;
}

}  // namespace byo

using namespace byo;

extern "C" {

int byo_policy_set_params(byo_ctx *ctx, const float *h_params) {
  if (!ctx || !h_params) return BYO_EINVAL;
  Mlp *p = nullptr;
  BYO_TRY(policy_get(ctx, &p));
  p->h_params.assign(h_params, h_params + kParams);
  BYO_CU(ctx, cudaMemcpy(p->d_params, h_params, kParams * sizeof(float), cudaMemcpyHostToDevice));
  p->trained = true;
  return BYO_OK;
}

int byo_policy_get_params(byo_ctx *ctx, float *h_params) {
  if (!ctx || !h_params) return BYO_EINVAL;
  if (!ctx->policy) return set_error(ctx, BYO_ENOTSUP, "no policy");
  std::memcpy(h_params, ctx->policy->h_params.data(), kParams * sizeof(float));
  return BYO_OK;
}

int byo_policy_clear(byo_ctx *ctx) {
  if (!ctx) return BYO_EINVAL;
  if (ctx->policy) ctx->policy->trained = false;
  return BYO_OK;
}

int byo_policy_init_params(uint64_t seed, float *h_params) {
  if (!h_params) return BYO_EINVAL;
  std::vector<float> P;
  init_params(P, seed);
  std::memcpy(h_params, P.data(), kParams * sizeof(float));
  return BYO_OK;
}

struct DevArrays {
  float *X = nullptr, *Y = nullptr, *a = nullptr, *b = nullptr, *c = nullptr;
  uint8_t *M = nullptr;
  uint32_t *perm = nullptr;
  ~DevArrays() {
    for (void *q : {(void *)X, (void *)Y, (void *)a, (void *)b, (void *)c, (void *)M, (void *)perm})
      if (q) cudaFree(q);
  }
};

int byo_policy_forward(byo_ctx *ctx, const float *h_params, const float *h_x, uint64_t n, float *h_y) {
  if (!ctx || !h_params || (n && (!h_x || !h_y))) return BYO_EINVAL;
  if (!n) return BYO_OK;
  DevArrays d;
  BYO_CU(ctx, cudaMalloc(&d.a, kParams * 4));
  BYO_CU(ctx, cudaMalloc(&d.X, n * kIn * 4));
  BYO_CU(ctx, cudaMalloc(&d.Y, n * kOut * 4));
  BYO_CU(ctx, cudaMemcpy(d.a, h_params, kParams * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.X, h_x, n * kIn * 4, cudaMemcpyHostToDevice));
  launch(ctx, k_mlp_forward, dim3(grid_for(ctx, n, 128)), dim3(128), 0, (const float *)d.a, (const float *)d.X, n, d.Y);
  BYO_TRY(check_launch(ctx, "mlp forward"));
  BYO_CU(ctx, cudaMemcpyAsync(h_y, d.Y, n * kOut * 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  return BYO_OK;
}

static uint64_t count_targets(const uint8_t *m, uint64_t n) {
  uint64_t c = 0;
  for (uint64_t i = 0; i < n; i++)
    for (int o = 0; o < kOut; o++) c += (m[i] >> o) & 1u;
  return c;
}

int byo_policy_loss_grad(byo_ctx *ctx, const float *h_params, const float *h_x, const float *h_y,
                         const uint8_t *h_mask, uint64_t n, float *loss, float *h_grad) {
  if (!ctx || !h_params || !h_x || !h_y || !h_mask || !loss || !h_grad || !n) return BYO_EINVAL;
  DevArrays d;
  BYO_CU(ctx, cudaMalloc(&d.a, kParams * 4));
  BYO_CU(ctx, cudaMalloc(&d.b, (kParams + 1) * 4));
  BYO_CU(ctx, cudaMalloc(&d.X, n * kIn * 4));
  BYO_CU(ctx, cudaMalloc(&d.Y, n * kOut * 4));
  BYO_CU(ctx, cudaMalloc(&d.M, n));
  BYO_CU(ctx, cudaMemcpy(d.a, h_params, kParams * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.X, h_x, n * kIn * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.Y, h_y, n * kOut * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.M, h_mask, n, cudaMemcpyHostToDevice));
  const uint64_t cnt = count_targets(h_mask, n);
  const size_t smem = sizeof(MbSmem) + kParams * 4;
  BYO_CU(ctx, cudaFuncSetAttribute(k_mlp_loss_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  launch(ctx, k_mlp_loss_grad, dim3(1), dim3(256), smem, (const float *)d.a, (const float *)d.X, (const float *)d.Y,
         (const uint8_t *)d.M, n, cnt ? 1.f / (float)cnt : 0.f, d.b, d.b + kParams);
  BYO_TRY(check_launch(ctx, "mlp loss/grad"));
  std::vector<float> out(kParams + 1);
  BYO_CU(ctx, cudaMemcpyAsync(out.data(), d.b, (kParams + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  std::memcpy(h_grad, out.data(), kParams * 4);
  *loss = out[kParams];
  return BYO_OK;
}

int byo_policy_train(byo_ctx *ctx, const float *h_init, const float *h_x, const float *h_y, const uint8_t *h_mask,
                     uint64_t n, uint32_t epochs, float lr, uint64_t seed, float *h_loss_per_epoch) {
  if (!ctx || !h_x || !h_y || !h_mask || !n || !epochs) return BYO_EINVAL;
  Mlp *p = nullptr;
  BYO_TRY(policy_get(ctx, &p));
  std::vector<float> P0;
  if (h_init) P0.assign(h_init, h_init + kParams);
  else init_params(P0, seed);
  // fixed shuffle of the samples (Fisher-Yates on a counter-based stream)
  std::vector<uint32_t> perm(n);
  for (uint64_t i = 0; i < n; i++) perm[i] = (uint32_t)i;
  uint64_t z = seed ^ 0xA5A5A5A5ull;
  for (uint64_t i = n - 1; i > 0; i--) {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t r = z;
    r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
    r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
    r ^= r >> 31;
    std::swap(perm[i], perm[r % (i + 1)]);
  }
  DevArrays d;
  BYO_CU(ctx, cudaMalloc(&d.X, n * kIn * 4));
  BYO_CU(ctx, cudaMalloc(&d.Y, n * kOut * 4));
  BYO_CU(ctx, cudaMalloc(&d.M, n));
  BYO_CU(ctx, cudaMalloc(&d.perm, n * 4));
  BYO_CU(ctx, cudaMalloc(&d.a, kParams * 4));
  BYO_CU(ctx, cudaMalloc(&d.b, kParams * 4));
  BYO_CU(ctx, cudaMalloc(&d.c, (size_t)epochs * 4));
  BYO_CU(ctx, cudaMemcpy(d.X, h_x, n * kIn * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.Y, h_y, n * kOut * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.M, h_mask, n, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(d.perm, perm.data(), n * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemcpy(p->d_params, P0.data(), kParams * 4, cudaMemcpyHostToDevice));
  BYO_CU(ctx, cudaMemset(d.a, 0, kParams * 4));
  BYO_CU(ctx, cudaMemset(d.b, 0, kParams * 4));
  const size_t smem = sizeof(MbSmem) + 2 * kParams * 4;
  BYO_CU(ctx, cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  launch(ctx, k_mlp_train, dim3(1), dim3(256), smem, p->d_params, (const float *)d.X, (const float *)d.Y,
         (const uint8_t *)d.M, (const uint32_t *)d.perm, n, epochs, lr, d.a, d.b, d.c);
  BYO_TRY(check_launch(ctx, "mlp train"));
  p->h_params.resize(kParams);
  BYO_CU(ctx, cudaMemcpyAsync(p->h_params.data(), p->d_params, kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (h_loss_per_epoch)
    BYO_CU(ctx, cudaMemcpyAsync(h_loss_per_epoch, d.c, (size_t)epochs * 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  p->trained = true;
  return BYO_OK;
}

}  // extern "C"
