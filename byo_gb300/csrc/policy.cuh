// policy.cuh -- the direction policy's inference, one warp, device side.
//
// Network: 16-32-32-5 FP32 MLP (ReLU, ReLU, linear) predicting log-times of
// five actions: 0 push, 1 pull, 2 blocked (per edgeMap round), 3 in-place
// merge, 4 rebuild (per container update).  Parameters are packed as W1 [32x16],
// b1, W2 [32x32], b2, W3 [5x32], b3.  GBBS's m/20 rule
// (edge_map_data.h:254-307) is the fallback and the arbiter: the network's pick
// replaces the rule's only when it predicts a gain above kArbiterMargin.
#pragma once

#include <cuda_pipeline.h>

#include "device.cuh"
#include "engine.h"

namespace byo {

constexpr int kIn = 16, kH = 32, kOut = 5;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kOut * kH, kParams = kB3 + kOut;  // 1765
// The network must predict a gain of more than 2^(16*margin) - 1 (about 7%)
// over the rule's choice before it overrides it.
constexpr float kArbiterMargin = 0.006f;

// The network is consulted when the frontier's size plus out-degree is within
// kGateFactor of the m/20 threshold, when the round before was dense, or when
// the frontier holds a vertex of degree >= 4^kGateHubBin; other frontiers
// (few vertices of low degree) are left to the rule: they take a few
// microseconds whichever direction runs, about what evaluating the network
// costs.
constexpr unsigned long long kGateFactor = 64;
constexpr int kGateHubBin = 5;

// Frontier statistics of the round just finished -> features -> m/20 rule ->
// network -> the next round's mode, written into st (mode, feat).  Features
// are computed when the network is consulted or `log` asks for them.  P may
// point to shared memory.  Called by the 32 lanes of one warp; lane k computes
// feature k and hidden unit k.
__device__ __forceinline__ void round_policy_warp(const float *P, RoundStats *st, float n, float m,
                                                  float reached_before, int dense, int has_net, int log) {
  __shared__ float x[kIn], h1[kH], h2[kH], y[kOut];
  const int lane = threadIdx.x & 31;
  const unsigned long long fc = st->count, dc = st->outdeg;
  const unsigned long long nn = (unsigned long long)n, mm = (unsigned long long)m;
  // the GBBS rule (edge_map_data.h:263,291) for the next round
  const int fallback = ((dense && fc > nn / 10) || (fc + dc > mm / 20)) ? MODE_PULL : MODE_PUSH;
  bool hub = false;
  for (int b = kGateHubBin; b < 8; b++) hub |= st->hist[b] != 0;
  const bool consult = has_net && (dense || hub || (fc + dc) * kGateFactor > mm / 20);
  if (lane == 0) st->mode = (unsigned long long)fallback;
  if (!consult && !log) return;
  if (lane < kIn) {
    const float inv = 1.f / 32.f;
    const float f = (float)fc, d = (float)dc;
    float v = 0.f;
    if (lane == 0) v = log2f(f + 1.f) * inv;
    else if (lane == 1) v = log2f(d + 1.f) * inv;
    else if (lane == 2) v = log2f(fmaxf(n - reached_before - f, 0.f) + 1.f) * inv;
    else if (lane == 3) v = log2f(n + 1.f) * inv;
    else if (lane == 4) v = log2f(m + 1.f) * inv;
    else if (lane >= 6 && lane < 14) {
      float tot = 0.f;
      for (int i = 0; i < 8; i++) tot += (float)st->hist[i];
      v = tot > 0.f ? (float)st->hist[lane - 6] / tot : 0.f;
    } else if (lane == 14) v = (f + d) / (m / 20.f + 1.f);
    else if (lane == 15) v = f / (n + 1.f);
    x[lane] = v;
    st->feat[lane] = v;
  }
  __syncwarp();
  if (!consult) return;
  {
    float a = P[kB1 + lane];
    for (int k = 0; k < kIn; k++) a = fmaf(P[kW1 + lane * kIn + k], x[k], a);
    h1[lane] = a > 0.f ? a : 0.f;
  }
  __syncwarp();
  {
    float a = P[kB2 + lane];
    for (int k = 0; k < kH; k++) a = fmaf(P[kW2 + lane * kH + k], h1[k], a);
    h2[lane] = a > 0.f ? a : 0.f;
  }
  __syncwarp();
  if (lane < kOut) {
    float a = P[kB3 + lane];
    for (int k = 0; k < kH; k++) a = fmaf(P[kW3 + lane * kH + k], h2[k], a);
    y[lane] = a;
  }
  __syncwarp();
  if (lane == 0) {
    int best = 0;
    for (int o = 1; o < 3; o++)
      if (y[o] < y[best]) best = o;
    // the m/20 rule arbitrates: keep its choice unless the predicted gain is clear
    if (y[fallback] - y[best] <= kArbiterMargin) best = fallback;
    st->mode = (unsigned long long)best;
  }
}

// The network's parameters rounded up to whole 16-byte chunks.
constexpr int kParamChunks = (kParams * 4 + 15) / 16;

// Start of a round's last kernel: every block begins copying the parameters
// into shared memory (asynchronously, behind its own work), so that the block
// that finishes last evaluates the network without a trip to L2.  Kernels too
// small to hide the copy (pt.prefetch == 0) read the parameters in place.
__device__ __forceinline__ void policy_prefetch(const PolicyTail &pt, float4 *sP) {
  if (!pt.on || !pt.has_net || !pt.prefetch) return;
  for (int i = threadIdx.x; i < kParamChunks; i += blockDim.x)
    __pipeline_memcpy_async(sP + i, reinterpret_cast<const float4 *>(pt.P) + i, 16);
  __pipeline_commit();
}

// Epilogue of a round's last kernel: the last block to finish (all other
// blocks' statistics are visible to it) runs the policy with one warp.  Every
// thread of the block calls it.
__device__ __forceinline__ void policy_tail(const PolicyTail &pt, RoundStats *st, const float4 *sP) {
  if (!pt.on) return;
  __shared__ int last;
  if (pt.has_net && pt.prefetch) __pipeline_wait_prior(0);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(pt.done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x < 32) {
    __threadfence();
    round_policy_warp(pt.prefetch ? reinterpret_cast<const float *>(sP) : pt.P, st, pt.n, pt.m,
                      pt.reached_before, pt.dense, pt.has_net, pt.log);
    if (threadIdx.x == 0) *pt.done = 0;
  }
}

}  // namespace byo
