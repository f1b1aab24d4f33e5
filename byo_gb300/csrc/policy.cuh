// policy.cuh -- the direction policy's inference, one warp, device side.
//
// Network: 16-32-32-5 FP32 MLP (ReLU, ReLU, linear) predicting log-times of
// five actions: 0 push, 1 pull, 2 blocked (per edgeMap round), 3 in-place
// merge, 4 rebuild (per container update).  Parameters are packed as W1 [32x16],
// b1, W2 [32x32], b2, W3 [5x32], b3.  GBBS's m/20 rule
// (edge_map_data.h:254-307) is the fallback and the judge: the network's pick
// replaces the rule's only when it predicts a gain above kJudgeMargin.
#pragma once

#include "device.cuh"
#include "engine.h"

namespace byo {

constexpr int kIn = 16, kH = 32, kOut = 5;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kOut * kH, kParams = kB3 + kOut;  // 1765
// The network must predict a gain of more than 2^(16*margin) - 1 (about 7%)
// over the rule's choice before it overrides it.
constexpr float kJudgeMargin = 0.006f;

// A frontier whose size plus out-degree is below 1/kGateFactor of the m/20
// threshold is left to the rule: the network is not consulted there (such
// rounds take a few microseconds whichever direction runs, and evaluating the
// network would cost about as much as it could gain).
constexpr unsigned long long kGateFactor = 64;

// Frontier statistics of the round just finished -> features -> m/20 rule ->
// network -> the next round's mode, written into st (mode, feat).  Features
// are computed when the network is consulted or `log` asks for them.  Called
// by the 32 lanes of one warp; lane k computes hidden unit k.
__device__ __forceinline__ void round_policy_warp(const float *__restrict__ P, RoundStats *st, float n, float m,
                                                  float reached_before, int dense, int has_net, int log) {
  __shared__ float x[kIn], h1[kH], h2[kH], y[kOut];
  __shared__ int fallback, consult;
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    // the GBBS rule (edge_map_data.h:263,291) for the next round
    const unsigned long long fc = st->count, dc = st->outdeg;
    const unsigned long long nn = (unsigned long long)n, mm = (unsigned long long)m;
    fallback = ((dense && fc > nn / 10) || (fc + dc > mm / 20)) ? MODE_PULL : MODE_PUSH;
    st->mode = (unsigned long long)fallback;
    consult = has_net && (dense || (fc + dc) * kGateFactor > mm / 20);
  }
  __syncwarp();
  if (!consult && !log) return;
  if (lane == 0) {
    const float inv = 1.f / 32.f;
    const float f = (float)st->count, d = (float)st->outdeg;
    const float unvisited = n - reached_before - f;
    x[0] = log2f(f + 1.f) * inv;
    x[1] = log2f(d + 1.f) * inv;
    x[2] = log2f(fmaxf(unvisited, 0.f) + 1.f) * inv;
    x[3] = log2f(n + 1.f) * inv;
    x[4] = log2f(m + 1.f) * inv;
    x[5] = 0.f;
    float tot = 0.f;
    for (int i = 0; i < 8; i++) tot += (float)st->hist[i];
    for (int i = 0; i < 8; i++) x[6 + i] = tot > 0.f ? (float)st->hist[i] / tot : 0.f;
    x[14] = (f + d) / (m / 20.f + 1.f);
    x[15] = f / (n + 1.f);
    for (int i = 0; i < kIn; i++) st->feat[i] = x[i];
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
    // the m/20 rule judges: keep its choice unless the predicted gain is clear
    if (y[fallback] - y[best] <= kJudgeMargin) best = fallback;
    st->mode = (unsigned long long)best;
  }
}

// Epilogue of a round's last kernel: the last block to finish (all other
// blocks' statistics are visible to it) runs the policy with one warp.  Every
// thread of the block calls it.
__device__ __forceinline__ void policy_tail(const PolicyTail &pt, RoundStats *st) {
  if (!pt.on) return;
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(pt.done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x < 32) {
    __threadfence();
    round_policy_warp(pt.P, st, pt.n, pt.m, pt.reached_before, pt.dense, pt.has_net, pt.log);
    if (threadIdx.x == 0) *pt.done = 0;
  }
}

}  // namespace byo
