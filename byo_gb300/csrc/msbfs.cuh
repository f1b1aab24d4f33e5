// msbfs.cuh -- the 64-source bit-lane BFS as device code: its state, the
// traversal of one query by a co-resident grid (ms_bfs_body) and the levels
// pass (ms_levels_body).  msbfs.cu runs them as their own kernels; pma.cu's
// mixed stream runs them inside the persistent kernel that also applies
// update batches.  The algorithm is described at the top of msbfs.cu.
#pragma once

#include "device.cuh"
#include "gridsync.cuh"
#include "internal.h"

namespace byo {

constexpr int kMsBlock = 256;
constexpr int kLevelBits = 16;                   // bit planes of the levels (rounds < 2^16)
constexpr int kMsLog = 64;                       // rounds recorded for byo_last_rounds

struct MsCtl {
  unsigned long long cnt[3];   // |L_r| (slot r % 3)
  unsigned long long ldeg[3];  // slot sum of L_r
  unsigned long long lc[3];    // list fill: non-hubs from the front
  unsigned long long hc[3];    // list fill: hubs from the back
  unsigned long long lvalid[3];
  unsigned long long cc[2];    // hub chunks of L_r, by round parity
  unsigned long long tc[2];    // touched vertices of a push round, by parity
  unsigned long long nheavy, nmega, nmc;
  GridBar bar;
  unsigned int rounds, pushes;
  unsigned long long t0;               // globaltimer after the set-up phase
  unsigned long long rlog[kMsLog][4];  // per round: end time, push?, |F|, slots of F
};

struct MsArgs {
  const uint64_t *off;
  const uint32_t *slots;
  uint64_t n, nslots, full;
  uint64_t *seen, *A, *B, *X;
  uint32_t *L[3];          // frontier lists, slot r % 3 holds round r's
  uint64_t *C[2];          // hub chunks of a frontier (vertex << 32 | chunk), by parity
  uint64_t *MC;            // chunks of every vertex above hub_deg (pull)
  uint64_t ccap;           // capacity of each chunk list
  uint32_t *T, *H;         // touched list; heavy list (warp vertices front, hubs back)
  uint32_t *levels;        // [k][n]
  uint64_t *planes;        // [kLevelBits][n]: bit b of the level of each (source, vertex)
  const uint32_t *srcs;
  uint32_t k;
  MsCtl *ctl;
  uint32_t max_rounds, heavy_deg, hub_deg, push_div;
};

__device__ __forceinline__ uint64_t vload(const unsigned long long *p) {
  return *(const volatile unsigned long long *)p;
}
__device__ __forceinline__ uint64_t ldm(const uint64_t *p, uint64_t i) {
  return __ldcg((const unsigned long long *)p + i);
}
__device__ __forceinline__ void stm(uint64_t *p, uint64_t i, uint64_t x) {
  __stcg((unsigned long long *)p + i, (unsigned long long)x);
}

__device__ __forceinline__ uint64_t warp_or64(uint64_t x) {
  const unsigned lo = __reduce_or_sync(kFull, (unsigned)x);
  const unsigned hi = __reduce_or_sync(kFull, (unsigned)(x >> 32));
  return (uint64_t)hi << 32 | lo;
}

// Records round r as the level of the lanes' newly reached (source, vertex)
// pairs: ORs `got` into v's plane b for each bit b of r.  From round 2^16 on,
// one store per pair straight to the output, one store instruction per
// source bit present in the warp.  Warp-uniform call (r is uniform).
__device__ __forceinline__ void ms_levels(const MsArgs &a, uint32_t v, uint64_t got, uint32_t r) {
  if (r < (1u << kLevelBits)) {
    if (got)
      for (uint32_t m = r; m; m &= m - 1)
        atomicOr((unsigned long long *)a.planes + (uint64_t)(__ffs((int)m) - 1) * a.n + v,
                 (unsigned long long)got);
    return;
  }
  uint64_t any = warp_or64(got);
  while (any) {
    const int s = __ffsll((long long)any) - 1;
    any &= any - 1;
    if ((got >> s) & 1) __stcs(a.levels + (uint64_t)s * a.n + v, r);
  }
}

// Appends lanes' vertices to frontier list `slot` (non-hubs front, hubs back
// with their chunks in C[par]).  Warp-uniform call.
__device__ __forceinline__ void ms_list(const MsArgs &a, int slot, int par, bool has, uint32_t v, uint64_t d) {
  MsCtl *c = a.ctl;
  const bool hub = has && d > a.hub_deg;
  const uint64_t s1 = warp_append(has && !hub, &c->lc[slot]);
  if (has && !hub) a.L[slot][s1] = v;
  if (__ballot_sync(kFull, hub)) {
    const uint64_t s2 = warp_append(hub, &c->hc[slot]);
    if (hub) {
      a.L[slot][a.n - 1 - s2] = v;
      const uint64_t nch = (d + a.hub_deg - 1) / a.hub_deg;
      const uint64_t cb = atomicAdd(&c->cc[par], (unsigned long long)nch);
      if (cb + nch <= a.ccap)
        for (uint64_t t = 0; t < nch; t++) a.C[par][cb + t] = (uint64_t)v << 32 | t;
      else
        atomicOr(&c->bar.err, 2u);
    }
  }
}

// One warp pushes F[u] over slots [b, e) of u; with `track`, the first
// writer of X[v] appends v to the touched list.  Warp-uniform call.
__device__ __forceinline__ void ms_push_range(const MsArgs &a, uint64_t mu, uint64_t b, uint64_t e, int par,
                                              bool track) {
  const unsigned lane = threadIdx.x & 31;
  for (uint64_t base = b; base < e; base += 32) {
    const uint64_t j = base + lane;
    uint32_t v = kSentinel;
    bool first = false;
    if (j < e) {
      v = __ldg(a.slots + j);
      if (v != kSentinel) {
        const uint64_t add = mu & ~ldm(a.seen, v);
        if (add) {
          if (track)
            first = atomicOr((unsigned long long *)a.X + v, (unsigned long long)add) == 0;
          else
            atomicOr((unsigned long long *)a.X + v, (unsigned long long)add);
        }
      }
    }
    if (track) {
      const uint64_t slot = warp_append(first, &a.ctl->tc[par]);
      if (first) a.T[slot] = v;
    }
  }
}

// Adds per-thread counts of a round's frontier to slot `cur`, one atomic pair
// per block.
__device__ __forceinline__ void ms_count(MsCtl *c, int cur, uint64_t cnt, uint64_t deg) {
  __shared__ unsigned long long red[2][32];
  cnt = warp_sum(cnt);
  deg = warp_sum(deg);
  const unsigned w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = cnt;
    red[1][w] = deg;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long x = 0, y = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
      x += red[0][i];
      y += red[1][i];
    }
    if (x) atomicAdd(&c->cnt[cur], x);
    if (y) atomicAdd(&c->ldeg[cur], y);
  }
  __syncthreads();
}

// The traversal of one 64-source query by the whole (co-resident) grid, any
// block size up to 1024; its grid barriers are `bar`.  Returns when done or
// when a barrier gave up (bar->err set).
__device__ inline void ms_bfs_body(const MsArgs &a, GridBar *bar) {
  MsCtl *c = a.ctl;
  const unsigned int nb = gridDim.x;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t warp = tid >> 5, nwarps = nthr >> 5;
  const uint64_t n = a.n;

  // phase 0: zero the masks; list the warp vertices, the hubs and the hubs' chunks
  for (uint64_t i = tid; i < n; i += nthr) {
    stm(a.seen, i, 0);
    stm(a.A, i, 0);
    stm(a.B, i, 0);
    stm(a.X, i, 0);
    stm(a.planes, i, 0);  // plane 0; plane b is cleared before round 2^b
  }
  for (uint64_t base = warp * 32; base < n; base += nwarps * 32) {
    const uint64_t v = base + lane;
    const uint64_t d = v < n ? a.off[v + 1] - a.off[v] : 0;
    const bool heavy = d > a.heavy_deg && d <= a.hub_deg, mega = d > a.hub_deg;
    const uint64_t s1 = warp_append(heavy, &c->nheavy);
    if (heavy) a.H[s1] = (uint32_t)v;
    if (__ballot_sync(kFull, mega)) {
      const uint64_t s2 = warp_append(mega, &c->nmega);
      if (mega) {
        a.H[n - 1 - s2] = (uint32_t)v;
        const uint64_t nch = (d + a.hub_deg - 1) / a.hub_deg;
        const uint64_t cb = atomicAdd(&c->nmc, (unsigned long long)nch);
        if (cb + nch <= a.ccap)
          for (uint64_t t = 0; t < nch; t++) a.MC[cb + t] = v << 32 | t;
        else
          atomicOr(&c->bar.err, 2u);
      }
    }
  }
  if (!grid_sync(bar, nb)) return;
  // the seeds form L_0 (sources may repeat)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (uint32_t s = 0; s < a.k; s++) {
      const uint32_t v = a.srcs[s];
      if (ldm(a.A, v) == 0) {
        const uint64_t d = a.off[v + 1] - a.off[v];
        if (d > a.hub_deg) {
          a.L[0][n - 1 - c->hc[0]++] = v;
          const uint64_t nch = (d + a.hub_deg - 1) / a.hub_deg;
          for (uint64_t t = 0; t < nch && c->cc[0] < a.ccap; t++) a.C[0][c->cc[0]++] = (uint64_t)v << 32 | t;
        } else {
          a.L[0][c->lc[0]++] = v;
        }
        c->cnt[0]++;
        c->ldeg[0] += d;
      }
      stm(a.A, v, ldm(a.A, v) | 1ull << s);
      stm(a.seen, v, ldm(a.seen, v) | 1ull << s);
    }
    c->lvalid[0] = 1;
    c->lvalid[2] = 1;  // an empty list: round 1 has nothing to clear
  }
  if (!grid_sync(bar, nb)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) c->t0 = globaltimer_ns();
  const uint64_t nheavy = vload(&c->nheavy), nmega = vload(&c->nmega), nmc = vload(&c->nmc);

  uint64_t *F = a.A, *N = a.B;
  uint32_t r = 1;
  for (; r <= a.max_rounds; r++) {
    const int cur = r % 3, prv = (r + 2) % 3, old = (r + 1) % 3;
    const int par = r & 1, ppar = par ^ 1;
    const uint64_t fcnt = vload(&c->cnt[prv]);
    if (fcnt == 0) break;
    const uint64_t fdeg = vload(&c->ldeg[prv]);
    const bool push = fdeg + fcnt < a.nslots / a.push_div;
    if (push) {
      // a frontier with many edges is pushed without a touched list: its
      // touched vertices are found by a pass over X, and it leaves no list
      const bool dense = fdeg + fcnt >= n / 64;
      // phase A: a round that left no list of its frontier; collect it from F
      if (!vload(&c->lvalid[prv])) {
        for (uint64_t base = warp * 32; base < n; base += nwarps * 32) {
          const uint64_t v = base + lane;
          const bool has = v < n && ldm(F, v) != 0;
          ms_list(a, prv, ppar, has, (uint32_t)v, has ? a.off[v + 1] - a.off[v] : 0);
        }
        if (!grid_sync(bar, nb)) return;
      }
      // phase 1: free N of round r-2's entries; scatter L_{r-1} into X
      if (vload(&c->lvalid[old])) {
        const uint64_t lco = vload(&c->lc[old]), hco = vload(&c->hc[old]);
        for (uint64_t i = tid; i < lco + hco; i += nthr)
          stm(N, i < lco ? a.L[old][i] : a.L[old][n - 1 - (i - lco)], 0);
      } else {
        for (uint64_t i = tid; i < n; i += nthr) stm(N, i, 0);
      }
      const uint64_t lcp = vload(&c->lc[prv]);
      for (uint64_t i = warp; i < lcp; i += nwarps) {
        const uint32_t u = __ldcg(a.L[prv] + i);
        ms_push_range(a, ldm(F, u), a.off[u], a.off[u + 1], par, !dense);
      }
      const uint64_t ccp = vload(&c->cc[ppar]);
      for (uint64_t i = warp; i < ccp; i += nwarps) {
        const uint64_t e = ldm(a.C[ppar], i);
        const uint32_t u = (uint32_t)(e >> 32);
        const uint64_t b = a.off[u] + (uint64_t)(uint32_t)e * a.hub_deg;
        ms_push_range(a, ldm(F, u), b, min(b + a.hub_deg, a.off[u + 1]), par, !dense);
      }
      if (!grid_sync(bar, nb)) return;
      // phase 2: the touched vertices become the next frontier
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        c->cnt[old] = c->ldeg[old] = c->lc[old] = c->hc[old] = c->lvalid[old] = 0;
        c->cc[ppar] = 0;
        c->tc[ppar] = 0;
        c->lvalid[cur] = dense ? 0 : 1;
        c->pushes++;
      }
      uint64_t my_cnt = 0, my_deg = 0;
      if (dense) {
        for (uint64_t base = warp * 32; base < n; base += nwarps * 32) {
          const uint64_t v = base + lane;
          uint64_t got = 0;
          if (v < n) {
            got = ldm(a.X, v);
            if (got) {
              stm(a.X, v, 0);
              stm(a.seen, v, ldm(a.seen, v) | got);
              stm(N, v, got);
              my_cnt++;
              my_deg += a.off[v + 1] - a.off[v];
            }
          }
          ms_levels(a, (uint32_t)v, got, r);
        }
      } else {
        const uint64_t tcount = vload(&c->tc[par]);
        for (uint64_t base = warp * 32; base < tcount; base += nwarps * 32) {
          const uint64_t i = base + lane;
          uint32_t v = 0;
          uint64_t got = 0, d = 0;
          if (i < tcount) {
            v = __ldcg(a.T + i);
            got = ldm(a.X, v);
            stm(a.X, v, 0);
            stm(a.seen, v, ldm(a.seen, v) | got);
            stm(N, v, got);
            d = a.off[v + 1] - a.off[v];
            my_cnt++;
            my_deg += d;
          }
          ms_list(a, cur, par, i < tcount, v, d);
          ms_levels(a, v, got, r);
        }
      }
      ms_count(c, cur, my_cnt, my_deg);
    } else {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        c->cnt[old] = c->ldeg[old] = c->lc[old] = c->hc[old] = c->lvalid[old] = 0;
        c->cc[ppar] = 0;
        c->tc[ppar] = 0;
      }
      uint64_t my_cnt = 0, my_deg = 0;
      // light vertices: a thread each
      for (uint64_t base = warp * 32; base < n; base += nwarps * 32) {
        const uint64_t v = base + lane;
        uint64_t got = 0;
        if (v < n) {
          const uint64_t b = a.off[v], e = a.off[v + 1];
          if (e - b <= a.heavy_deg) {
            const uint64_t sv = ldm(a.seen, v);
            const uint64_t need = a.full & ~sv;
            if (need) {
              uint64_t j = b;
              for (; j + 4 <= e; j += 4) {
                const uint32_t u0 = __ldg(a.slots + j), u1 = __ldg(a.slots + j + 1);
                const uint32_t u2 = __ldg(a.slots + j + 2), u3 = __ldg(a.slots + j + 3);
                uint64_t f = u0 != kSentinel ? ldm(F, u0) : 0;
                f |= u1 != kSentinel ? ldm(F, u1) : 0;
                f |= u2 != kSentinel ? ldm(F, u2) : 0;
                f |= u3 != kSentinel ? ldm(F, u3) : 0;
                got |= f;
                if ((got & need) == need) break;
              }
              for (; j < e && (got & need) != need; j++) {
                const uint32_t u = __ldg(a.slots + j);
                if (u != kSentinel) got |= ldm(F, u);
              }
              got &= need;
              if (got) {
                stm(a.seen, v, sv | got);
                my_cnt++;
                my_deg += e - b;
              }
            }
            stm(N, v, got);
          }
        }
        ms_levels(a, (uint32_t)v, got, r);
      }
      // warp vertices
      for (uint64_t i = warp; i < nheavy; i += nwarps) {
        const uint32_t v = __ldcg(a.H + i);
        const uint64_t sv = ldm(a.seen, v);
        const uint64_t need = a.full & ~sv;
        const uint64_t b = a.off[v], e = a.off[v + 1];
        uint64_t got = 0;
        if (need) {
          for (uint64_t base = b; base < e; base += 32) {
            const uint64_t j = base + lane;
            uint64_t x = 0;
            if (j < e) {
              const uint32_t u = __ldg(a.slots + j);
              if (u != kSentinel) x = ldm(F, u);
            }
            got |= warp_or64(x);
            if ((got & need) == need) break;
          }
          got &= need;
        }
        if (lane == 0) {
          stm(N, v, got);
          if (got) {
            stm(a.seen, v, sv | got);
            my_cnt++;
            my_deg += e - b;
          }
        }
        ms_levels(a, v, lane == 0 ? got : 0, r);
      }
      // hubs: a warp per chunk, partial ORs meet in X
      for (uint64_t i = warp; i < nmc; i += nwarps) {
        const uint64_t ch = ldm(a.MC, i);
        const uint32_t v = (uint32_t)(ch >> 32);
        const uint64_t need = a.full & ~ldm(a.seen, v);
        if (!need) continue;
        const uint64_t b = a.off[v] + (uint64_t)(uint32_t)ch * a.hub_deg;
        const uint64_t e = min(b + a.hub_deg, a.off[v + 1]);
        uint64_t got = 0;
        uint32_t it = 0;
        for (uint64_t base = b; base < e; base += 32, it++) {
          const uint64_t j = base + lane;
          uint64_t x = 0;
          if (j < e) {
            const uint32_t u = __ldg(a.slots + j);
            if (u != kSentinel) x = ldm(F, u);
          }
          got |= warp_or64(x);
          if ((got & need) == need) break;
          if ((it & 7) == 7 && ((got | ldm(a.X, v)) & need) == need) break;
        }
        got &= need;
        if (lane == 0 && (got & ~ldm(a.X, v))) atomicOr((unsigned long long *)a.X + v, (unsigned long long)got);
      }
      if (nmega) {
        if (!grid_sync(bar, nb)) return;
        for (uint64_t base = warp * 32; base < nmega; base += nwarps * 32) {
          const uint64_t i = base + lane;
          uint32_t v = 0;
          uint64_t got = 0;
          if (i < nmega) {
            v = __ldcg(a.H + n - 1 - i);
            got = ldm(a.X, v);
            stm(a.X, v, 0);
            stm(N, v, got);
            if (got) {
              stm(a.seen, v, ldm(a.seen, v) | got);
              my_cnt++;
              my_deg += a.off[v + 1] - a.off[v];
            }
          }
          ms_levels(a, v, got, r);
        }
      }
      ms_count(c, cur, my_cnt, my_deg);
    }
    // the plane that round r + 1 is the first to use
    if (((r + 1) & r) == 0 && r + 1 < (1u << kLevelBits)) {
      uint64_t *pl = a.planes + (uint64_t)(__ffs((int)(r + 1)) - 1) * n;
      for (uint64_t i = tid; i < n; i += nthr) stm(pl, i, 0);
    }
    if (!grid_sync(bar, nb)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0 && r <= kMsLog) {
      c->rlog[r - 1][0] = globaltimer_ns();
      c->rlog[r - 1][1] = push;
      c->rlog[r - 1][2] = fcnt;
      c->rlog[r - 1][3] = fdeg;
    }
    uint64_t *t = F;
    F = N;
    N = t;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) c->rounds = r - 1;
}

// Bits 0..7 of x spread to the low bit of bytes 0..7 (SWAR: the byte is
// copied into every byte lane, lane i keeps bit i, and a carry-free add
// turns each lane's kept bit into its top bit, shifted down to bit 0).
__device__ __forceinline__ uint64_t spread8(uint64_t x) {
  const uint64_t t = ((x & 0xFFull) * 0x0101010101010101ull) & 0x8040201008040201ull;
  return ((t + 0x7F7F7F7F7F7F7F7Full) >> 7) & 0x0101010101010101ull;
}

// One (source, vertex) level: a zero level is the source itself, a pair
// reached from round 2^16 on (already written) or a pair never reached.
__device__ __forceinline__ void ms_store_level(const MsArgs &a, uint32_t s, uint64_t v, uint32_t lv,
                                               uint64_t sv) {
  if (!lv) {
    if (__ldg(a.srcs + s) == (uint32_t)v) lv = 0;
    else if ((sv >> s) & 1) return;  // reached after round 2^16 - 1: written by the traversal
    else lv = kSentinel;
  }
  __stcs(a.levels + (uint64_t)s * a.n + v, lv);
}

// The levels from the bit planes, a thread per vertex: level of (s, v) =
// sum over planes b of bit s of plane b, << b.  Up to 8 planes (levels below
// 256) the levels of 8 sources at a time are assembled as bytes of one word,
// a spread8 per plane; deeper traversals take them bit by bit.  Per source a
// warp stores 32 consecutive words.
__device__ inline void ms_levels_body(const MsArgs &a, uint64_t tid, uint64_t nthr) {
  const uint32_t last = a.ctl->rounds;
  const int used = last ? min(32 - __clz((int)last), kLevelBits) : 0;
  const uint64_t n = a.n;
  const uint32_t k = a.k;
  for (uint64_t v = tid; v < n; v += nthr) {
    const uint64_t sv = __ldcs(a.seen + v);
    if (used <= 8) {
      uint64_t pl[8];
#pragma unroll
      for (int b = 0; b < 8; b++) pl[b] = b < used ? __ldcs(a.planes + (uint64_t)b * n + v) : 0;
      for (uint32_t s0 = 0; s0 < k; s0 += 8) {
        uint64_t packed = 0;
#pragma unroll
        for (int b = 0; b < 8; b++) packed |= spread8(pl[b] >> s0) << b;
#pragma unroll
        for (uint32_t i = 0; i < 8; i++)
          if (s0 + i < k) ms_store_level(a, s0 + i, v, (uint32_t)(packed >> (8 * i)) & 0xFFu, sv);
      }
    } else {
      for (uint32_t s = 0; s < k; s++) {
        uint32_t lv = 0;
        for (int b = 0; b < used; b++) lv |= (uint32_t)((__ldg(a.planes + (uint64_t)b * n + v) >> s) & 1) << b;
        ms_store_level(a, s, v, lv, sv);
      }
    }
  }
}


// The work arrays of a query over graph view g (its own slots: the PMA's
// leaves with their gaps, or a CSR), sized for k sources; srcs, levels and
// ctl are left to the caller.
int ms_args_setup(byo_graph *g, uint32_t k, MsArgs *a);

}  // namespace byo
