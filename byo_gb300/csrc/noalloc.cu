// noalloc.cu -- BFS over a caller-owned device CSR that allocates nothing.
//
// Some callers cannot let a library allocate device memory: hosts whose memory
// manager reserves the whole GPU up front and hands out sub-ranges itself (a
// database buffer pool, a JVM or Go runtime that owns one big device arena).
// A cudaMalloc from inside the library would either fail (the arena already
// holds the memory) or take memory the host's manager does not know about.
// For them byo_bfs_csr_noalloc runs the same direction-optimising BFS as
// byo_bfs (same parents and levels) with every piece of traversal state in one
// file-scope device array, g_bfs_scratch, of fixed size: room for
// BYO_NOALLOC_MAX_VERTICES (2^20) vertices at 16.4 bytes per vertex
// (16.4 MiB).  Every GPU that loads this library keeps that array until the
// process exits.
//
// The call is host-synchronous: after each round it copies the next
// frontier's size back to pageable host memory and synchronises the caller's
// stream, and it returns when the result is in the output arrays.
//
// The array is shared by every call on a device and keeps what the last call
// left in it; each call re-initialises what must start at zero.  Calls that
// overlap on the GPU (two streams, or two host threads) race on it and give
// wrong results; callers must serialise them.  The first call on a device
// looks the array's device address up (cudaGetSymbolAddress) with that device
// current and caches it per (device, CUDA context); a context created after a
// cudaDeviceReset is a new key, so the address is looked up again there.
#include <mutex>

#include "../../include/byo_gpu.h"
#include "device.cuh"

namespace {

using byo::kFull;
using byo::lane_id;
using byo::warp_append;

constexpr uint64_t kMaxV = BYO_NOALLOC_MAX_VERTICES;
constexpr uint64_t kMaxW = kMaxV / 32;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint64_t kNone64 = ~0ull;

// byte layout of the scratch array
constexpr size_t kOffLp = 0;                               // uint64[kMaxV] level<<32 | parent
constexpr size_t kOffList = kOffLp + 8 * kMaxV;            // uint32[2][kMaxV] frontier lists
constexpr size_t kOffBits = kOffList + 2 * 4 * kMaxV;      // uint32[2][kMaxW] frontier bitmaps
constexpr size_t kOffVisited = kOffBits + 2 * 4 * kMaxW;   // uint32[kMaxW]
constexpr size_t kOffStats = kOffVisited + 4 * kMaxW;      // uint64[4]: count, outdeg
constexpr size_t kScratchBytes = kOffStats + 64;

static __device__ __align__(256) unsigned char g_bfs_scratch[kScratchBytes];

struct Scratch {
  uint64_t *lp;
  uint32_t *list[2];
  uint32_t *bits[2];
  uint32_t *visited;
  unsigned long long *stats;
};

Scratch carve(void *base) {
  unsigned char *b = static_cast<unsigned char *>(base);
  Scratch s;
  s.lp = reinterpret_cast<uint64_t *>(b + kOffLp);
  s.list[0] = reinterpret_cast<uint32_t *>(b + kOffList);
  s.list[1] = s.list[0] + kMaxV;
  s.bits[0] = reinterpret_cast<uint32_t *>(b + kOffBits);
  s.bits[1] = s.bits[0] + kMaxW;
  s.visited = reinterpret_cast<uint32_t *>(b + kOffVisited);
  s.stats = reinterpret_cast<unsigned long long *>(b + kOffStats);
  return s;
}

// ---------------------------------------------------------------- kernels

__global__ void k_na_init(uint64_t *lp, uint32_t *visited, uint32_t *bits0, uint32_t *bits1, uint32_t *list0,
                          unsigned long long *stats, uint64_t n, uint32_t src) {
  const uint64_t W = (n + 31) / 32;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    lp[i] = i == src ? (uint64_t)src : kNone64;
    if (i < W) {
      const uint32_t w = i == (src >> 5) ? 1u << (src & 31) : 0u;
      visited[i] = w;
      bits0[i] = w;
      bits1[i] = 0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    list0[0] = src;
    stats[0] = stats[1] = 0;
  }
}

// one warp per frontier vertex; the smallest (level, parent) wins per vertex
__global__ void __launch_bounds__(256) k_na_push(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbrs,
                                                 const uint32_t *__restrict__ F, uint64_t fsize, uint64_t *lp,
                                                 const uint32_t *__restrict__ visited, uint32_t *out_list,
                                                 uint32_t *out_bits, unsigned long long *stats, uint64_t lvl) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t dsum = 0;
  for (uint64_t i = gw; i < fsize; i += nw) {
    const uint32_t u = F[i];
    const uint64_t b = off[u], e = off[u + 1];
    for (uint64_t base = b; base < e; base += 32) {
      const uint64_t j = base + lane_id();
      bool emit = false;
      uint32_t v = 0;
      if (j < e) {
        v = nbrs[j];
        if (!((__ldcg(visited + (v >> 5)) >> (v & 31)) & 1u)) {
          unsigned long long old = atomicMin((unsigned long long *)(lp + v), (unsigned long long)(lvl | u));
          emit = old == kNone64;
        }
      }
      const uint64_t slot = warp_append(emit, stats);
      if (emit) {
        out_list[slot] = v;
        atomicOr(out_bits + (v >> 5), 1u << (v & 31));
        dsum += off[v + 1] - off[v];
      }
    }
  }
  dsum = byo::warp_sum(dsum);
  if (lane_id() == 0 && dsum) atomicAdd(stats + 1, (unsigned long long)dsum);
}

// one thread per unvisited vertex, first frontier neighbour in sorted order
__global__ void __launch_bounds__(256) k_na_pull(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbrs,
                                                 const uint32_t *__restrict__ Fbits, uint64_t n, uint64_t *lp,
                                                 uint32_t *visited, uint32_t *out_list, uint32_t *out_bits,
                                                 unsigned long long *stats, uint64_t lvl) {
  const uint64_t W = (n + 31) / 32;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t dsum = 0;
  for (uint64_t w = gw; w < W; w += nw) {
    const uint32_t vword = visited[w];
    if (vword == kFull) continue;
    const uint64_t v = w * 32 + lane_id();
    bool found = false;
    uint32_t parent = 0;
    if (v < n && !((vword >> lane_id()) & 1u)) {
      for (uint64_t j = off[v]; j < off[v + 1]; j++) {
        const uint32_t u = nbrs[j];
        if ((__ldg(Fbits + (u >> 5)) >> (u & 31)) & 1u) {
          found = true;
          parent = u;
          break;
        }
      }
    }
    if (found) lp[v] = lvl | parent;
    const unsigned fb = __ballot_sync(kFull, found);
    if (lane_id() == 0 && fb) {
      out_bits[w] = fb;
      visited[w] = vword | fb;
    }
    const uint64_t slot = warp_append(found, stats);
    if (found) {
      out_list[slot] = (uint32_t)v;
      dsum += off[v + 1] - off[v];
    }
  }
  dsum = byo::warp_sum(dsum);
  if (lane_id() == 0 && dsum) atomicAdd(stats + 1, (unsigned long long)dsum);
}

__global__ void k_na_mark(const uint32_t *__restrict__ list, const unsigned long long *stats, uint32_t *visited) {
  const uint64_t cnt = stats[0];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x)
    atomicOr(visited + (list[i] >> 5), 1u << (list[i] & 31));
}

__global__ void k_na_clear(const uint32_t *__restrict__ list, uint64_t cnt, uint32_t *bits) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x)
    bits[list[i] >> 5] = 0;
}

__global__ void k_na_extract(const uint64_t *__restrict__ lp, uint64_t n, uint32_t *parent, uint32_t *level) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = lp[i];
    if (parent) parent[i] = x == kNone64 ? kNone : (uint32_t)x;
    if (level) level[i] = x == kNone64 ? kNone : (uint32_t)(x >> 32);
  }
}

// ---------------------------------------------------------------- set-up

std::mutex g_mu;
// Device address of g_bfs_scratch per device ordinal, valid for the CUDA
// context current when it was looked up (a reset destroys the context and
// reloads the module, so the address is looked up again for a new context).
void *g_addr[256];
void *g_addr_ctx[256];

typedef int (*CtxGetCurrentFn)(void **);

// The current CUDA context (driver handle), or null when the driver entry
// point is unavailable (then the cache is keyed on the device alone).
void *current_context() {
  static CtxGetCurrentFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  void *c = nullptr;
  if (fn && fn(&c) != 0) c = nullptr;
  return c;
}

int scratch_for_current_device(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
    cudaGetLastError();
    return BYO_EDEVICE;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  void *cx = current_context();
  if (!g_addr[dev] || !cx || g_addr_ctx[dev] != cx) {
    // The runtime makes the device's primary context current here if no
    // context is current yet; the key is read again afterwards.
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_bfs_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return BYO_EDEVICE;
    }
    g_addr[dev] = p;
    g_addr_ctx[dev] = current_context();
  }
  *out = g_addr[dev];
  return BYO_OK;
}

int grid_of(uint64_t work, int block) {
  uint64_t g = (work + block - 1) / block;
  if (g > 4096) g = 4096;
  return g < 1 ? 1 : (int)g;
}

}  // namespace

extern "C" int byo_bfs_csr_noalloc(const uint64_t *d_offsets, const uint32_t *d_nbrs, uint64_t n, uint64_t m,
                                   uint32_t src, uint32_t *d_parent, uint32_t *d_level, void *stream,
                                   uint32_t *rounds) {
  if (!d_offsets || (m && !d_nbrs) || (!d_parent && !d_level)) return BYO_EINVAL;
  if (n == 0 || n > kMaxV || src >= n) return BYO_EINVAL;
  void *base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc != BYO_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Scratch s = carve(base);
  const uint64_t W = (n + 31) / 32;
  uint64_t consumed = 0;  // size of the frontier whose bits sit in the next bitmap
  uint64_t deg_src[2] = {0, 0};
  k_na_init<<<grid_of(n, 256), 256, 0, st>>>(s.lp, s.visited, s.bits[0], s.bits[1], s.list[0], s.stats, n, src);
  if (cudaGetLastError() != cudaSuccess) return BYO_EDEVICE;
  if (cudaMemcpyAsync(deg_src, d_offsets + src, 16, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return BYO_EDEVICE;
  }
  uint64_t fsize = 1, outdeg = deg_src[1] - deg_src[0];
  bool dense = false;
  int cur = 0;
  uint32_t r = 1, nr = 0;
  while (fsize > 0) {
    // the GBBS rule (edge_map_data.h:254-307): dense when the frontier came
    // from a dense round and holds more than n/10 vertices, or when
    // |F| + sum of its degrees exceeds m/20
    const bool pull = (dense && fsize > n / 10) || (fsize + outdeg > m / 20);
    if (!pull && outdeg == 0) break;
    const int nxt = cur ^ 1;
    // the next bitmap still holds the frontier before `cur`
    if (nr > 0) k_na_clear<<<grid_of(consumed + 1, 256), 256, 0, st>>>(s.list[nxt], consumed, s.bits[nxt]);
    if (cudaMemsetAsync(s.stats, 0, 16, st) != cudaSuccess) {
      cudaGetLastError();
      return BYO_EDEVICE;
    }
    const uint64_t lvl = (uint64_t)r << 32;
    if (pull) {
      k_na_pull<<<grid_of(W * 32, 256), 256, 0, st>>>(d_offsets, d_nbrs, s.bits[cur], n, s.lp, s.visited,
                                                     s.list[nxt], s.bits[nxt], s.stats, lvl);
    } else {
      k_na_push<<<grid_of(fsize * 32, 256), 256, 0, st>>>(d_offsets, d_nbrs, s.list[cur], fsize, s.lp, s.visited,
                                                         s.list[nxt], s.bits[nxt], s.stats, lvl);
      k_na_mark<<<grid_of(outdeg + 1, 256), 256, 0, st>>>(s.list[nxt], s.stats, s.visited);
    }
    consumed = fsize;
    // a launch that failed to start leaves no sticky error: catch it here,
    // before the round's counts are read back
    if (cudaGetLastError() != cudaSuccess) return BYO_EDEVICE;
    unsigned long long got[2] = {0, 0};
    if (cudaMemcpyAsync(got, s.stats, 16, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      return BYO_EDEVICE;
    }
    fsize = got[0];
    outdeg = got[1];
    dense = pull;
    cur = nxt;
    r++;
    nr++;
  }
  k_na_extract<<<grid_of(n, 256), 256, 0, st>>>(s.lp, n, d_parent, d_level);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) return BYO_EDEVICE;
  if (rounds) *rounds = nr;
  return BYO_OK;
}
