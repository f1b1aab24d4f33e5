// msbfs.cu -- 64-source BFS packed into bit lanes, run by one persistent
// cooperative kernel.
//
// Each vertex carries 64-bit masks: seen (sources that reached it), and the
// frontier masks of two consecutive rounds, F (read) and N (written).  BFS
// levels do not depend on the order in which a round's ORs happen, so every
// source's levels equal those of a single-source BFS (BFS.h:47-64) from it.
// The union frontier of all lanes chooses the direction of each round, as
// edgeMapData does for one source (edge_map_data.h:254-307):
//
//   push  every frontier vertex u ORs F[u] & ~seen[v] into an accumulator
//         X[v] of each neighbour; the first writer of X[v] appends v to a
//         touched list, and a second phase turns the touched vertices into
//         the next frontier and its list.  A frontier vertex takes a warp;
//         hubs (more than hub_deg slots) are cut into chunks of hub_deg
//         slots, a warp per chunk.
//   pull  every vertex that still misses some source ORs the F masks of its
//         neighbours, stopping once every missing bit is found.  Up to
//         heavy_deg slots a thread takes the vertex, up to hub_deg a warp;
//         above that its slots are cut into chunks, a warp each, whose ORs
//         meet in X[v] and are settled after a grid barrier.  A pull round
//         writes every N[v] and keeps only the frontier's size and slot sum,
//         reduced per block, so no single counter is contended.
//
// A push round needs the list of its input frontier: it has one when the
// previous round was a push, otherwise it first collects it from F.  It also
// needs N free of the entries of two rounds before, which it clears from that
// round's list, or wholesale when that round was a pull.  Levels are kept as
// bit planes: when round r reaches sources `got` at v, got is ORed into
// plane b of v for every bit b of r (16 planes, rounds below 2^16; later
// rounds write their levels straight to the output).  A last kernel turns
// each vertex's planes into its 64 levels and writes them source-major, a
// warp storing 32 consecutive words per source, with BYO_NONE for pairs never
// reached; the traversal itself makes no scattered output stores.  Rounds are
// separated by a grid
// barrier of the project's own whose wait is bounded in time: a barrier that
// does not complete sets an error flag and every block leaves.
#include <algorithm>
#include <vector>

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
  __shared__ unsigned long long red[2][kMsBlock / 32];
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
    for (int i = 0; i < kMsBlock / 32; i++) {
      x += red[0][i];
      y += red[1][i];
    }
    if (x) atomicAdd(&c->cnt[cur], x);
    if (y) atomicAdd(&c->ldeg[cur], y);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kMsBlock, 5) k_ms_bfs(MsArgs a) {
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
  if (!grid_sync(&c->bar, nb)) return;
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
  if (!grid_sync(&c->bar, nb)) return;
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
        if (!grid_sync(&c->bar, nb)) return;
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
      if (!grid_sync(&c->bar, nb)) return;
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
        if (!grid_sync(&c->bar, nb)) return;
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
    if (!grid_sync(&c->bar, nb)) return;
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
__global__ void __launch_bounds__(256) k_ms_levels(const MsArgs a) {
  if (a.ctl->bar.err) return;
  const uint32_t last = a.ctl->rounds;
  const int used = last ? min(32 - __clz((int)last), kLevelBits) : 0;
  const uint64_t n = a.n;
  const uint32_t k = a.k;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
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

int bfs_multi_run(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint32_t *rounds) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  if (k == 0 || k > 64) return set_error(ctx, BYO_EINVAL, "bfs_multi: 1 <= k <= 64 sources");
  for (uint32_t s = 0; s < k; s++)
    if (h_srcs[s] >= n) return set_error(ctx, BYO_EINVAL, "bfs_multi: source >= n");
  if (n >= (1ull << 32) - 1) return set_error(ctx, BYO_EINVAL, "bfs_multi: n too large");
  const byo_tuning t = effective_tuning(g);
  MsArgs a = {};
  a.off = g->d_off;
  a.slots = g->d_slots;
  a.n = n;
  a.nslots = g->nslots;
  a.full = k == 64 ? ~0ull : ((1ull << k) - 1);
  a.k = k;
  a.max_rounds = 0xFFFFFFF0u;
  a.heavy_deg = t.ms_heavy_deg;
  a.hub_deg = t.ms_hub_deg;
  a.push_div = t.ms_push_div;
  // chunks of a set of distinct vertices above hub_deg: sum of ceil(d / hub_deg) <= 2 * slots / hub_deg
  const uint64_t nchunks = 2 * g->nslots / a.hub_deg + 64;
  a.ccap = nchunks;
  uint64_t *masks;
  BYO_TRY(ws(g, WS_LP, 4 * n + 4, &masks));  // seen | A | B | X
  a.seen = masks;
  a.A = masks + n;
  a.B = masks + 2 * n;
  a.X = masks + 3 * n;
  uint32_t *lists;
  BYO_TRY(ws(g, WS_FRONT_LIST_A, 3 * n + 4, &lists));
  for (int i = 0; i < 3; i++) a.L[i] = lists + i * n;
  uint32_t *th;
  BYO_TRY(ws(g, WS_FRONT_LIST_B, 2 * n + 4, &th));
  a.T = th;
  a.H = th + n;
  uint64_t *chunks;
  BYO_TRY(ws(g, WS_DEFER, 3 * nchunks, &chunks));
  a.C[0] = chunks;
  a.C[1] = chunks + nchunks;
  a.MC = chunks + 2 * nchunks;
  uint32_t *misc;
  BYO_TRY(ws(g, WS_MISC, 64 + sizeof(MsCtl) / 4 + 8, &misc));  // sources, then the control block
  a.srcs = misc;
  a.ctl = (MsCtl *)(misc + 64);
  a.levels = d_levels;
  BYO_TRY(ws(g, WS_MS_LEVELS, (size_t)kLevelBits * n, &a.planes));
  BYO_CU(ctx, cudaMemcpyAsync(misc, h_srcs, k * 4, cudaMemcpyHostToDevice, ctx->stream));
  BYO_CU(ctx, cudaMemsetAsync(a.ctl, 0, sizeof(MsCtl), ctx->stream));
  if (ctx->bar_limit_ms || ctx->bar_extra) {  // the barrier test hook
    const unsigned int hb[2] = {ctx->bar_limit_ms, ctx->bar_extra};
    BYO_CU(ctx, cudaMemcpyAsync(&a.ctl->bar.limit_ms, hb, sizeof(hb), cudaMemcpyHostToDevice, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));  // hb is on the stack
  }
  // co-resident grid for the cooperative launch
  int per_sm = 0;
  BYO_CU(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_bfs, kMsBlock, 0));
  if (per_sm < 1) return set_error(ctx, BYO_EDEVICE, "bfs_multi: kernel cannot be resident");
  const unsigned int grid = (unsigned int)std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t)per_sm * ctx->num_sms, (n + kMsBlock - 1) / kMsBlock));
  void *args[] = {(void *)&a};
  const bool timed = !ctx->ktag.empty() && ktimer_begin(ctx, "bfs_multi");
  BYO_CU(ctx, cudaLaunchCooperativeKernel((const void *)k_ms_bfs, dim3(grid), dim3(kMsBlock), args, 0, ctx->stream));
  launch(ctx, k_ms_levels, dim3(grid_for(ctx, n, 256)), dim3(256), 0, a);
  ctx->launches++;
  if (timed) ktimer_end(ctx);
  MsCtl *h = nullptr;
  BYO_TRY(pinned(ctx, sizeof(MsCtl), (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (h->bar.err & 2u) return set_error(ctx, BYO_EDEVICE, "bfs_multi: hub chunk list overflow");
  if (h->bar.err) return set_error(ctx, BYO_ETIMEDOUT, "bfs_multi: grid barrier timed out");
  if (rounds) *rounds = h->rounds;
  ctx->rounds.clear();
  uint64_t prev = h->t0;
  for (uint32_t r = 0; r < h->rounds && r < (uint32_t)kMsLog; r++) {
    byo_round_log e = {};
    e.round = r + 1;
    e.mode = h->rlog[r][1] ? 0 : 1;
    e.frontier = h->rlog[r][2];
    e.frontier_deg = h->rlog[r][3];
    e.ms = (float)((double)(h->rlog[r][0] - prev) * 1e-6);
    prev = h->rlog[r][0];
    ctx->rounds.push_back(e);
  }
  return check_launch(ctx, "bfs_multi");
}

}  // namespace byo
