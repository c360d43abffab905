// Device forms of the hypergraph formats on either side of the refinement:
//
//   createInverse (shared/utils.cpp:32-56)   the net -> pins CSR of a vertex ->
//       nets CSR, each net's pins in ascending vertex id: a histogram of the
//       pins per net, an exclusive scan, a scatter with one cursor per net
//       and a sort of each net's pins (warps, CTAs, or CTAs merging sorted
//       chunks by rank, by the net's size);
//   net thinning (CN/cn.cpp:201-268)          the nets below both size bounds,
//       renumbered in order, and every vertex's kept nets in its own order:
//       flags, scans and compactions;
//   BFS ordering (shared/utils.cpp:433-536, the one-thread walk of
//       shared/utils.cpp:538-590)             levels in discovery order: a
//       frontier vertex i walks its nets in vertex -> nets order and a net's
//       pins in ascending id, so a newly reached vertex's key is the smallest
//       (frontier position, pair index) that reaches it, and the next frontier
//       is the reached vertices sorted by key.  A net's pins are all reached
//       from the first (frontier position, net) that walks it, so each net is
//       walked once per search.
//
// All of it is integer work bound by HBM bandwidth and atomics; the results
// are the host forms' bit for bit.

#include "fp_device.cuh"
#include "fp_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace fp {

namespace {

constexpr unsigned kAllLanes = 0xffffffffu;

// ------------------------------------------------------------- exclusive scan
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr long long kScanTile = (long long)kScanThreads * kScanItems;

// Exclusive scan of one tile of `in` into `out`; the tile's total into
// sums[blockIdx.x].  Values and totals fit 32 bits (pins < 2^31).
__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const uint32_t* in, uint32_t* out, uint32_t* sums,
                                                                 long long n) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t t = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    v[i] = base + i < n ? in[base + i] : 0u;
    t += v[i];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = t;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(kAllLanes, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t x = warp_tot[lane];
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(kAllLanes, x, off);
      if (lane >= off) x += y;
    }
    warp_tot[lane] = x;   // inclusive warp totals
  }
  __syncthreads();
  uint32_t run = incl - t + (w > 0 ? warp_tot[w - 1] : 0u);
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = warp_tot[31];
}

__global__ void scan_add_kernel(uint32_t* out, const uint32_t* offs, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanTile];
}

// Scratch words scan_exclusive needs for n values.
size_t scan_scratch(long long n) {
  size_t s = 0;
  while (n > kScanTile) {
    n = (n + kScanTile - 1) / kScanTile;
    s += (size_t)n * 2;
  }
  return s + 2;
}

// out[i] = in[0] + ... + in[i-1] (in and out may alias).
cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, long long n, uint32_t* scratch, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long tiles = (n + kScanTile - 1) / kScanTile;
  uint32_t* sums = scratch;
  scan_tile_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, sums, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || tiles == 1) return e;
  e = scan_exclusive(sums, sums, tiles, scratch + tiles * 2, st);   // sums -> their offsets
  if (e != cudaSuccess) return e;
  scan_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, sums, n);
  return cudaGetLastError();
}

// ------------------------------------------------------------- segmented sort
// Ascending sort of each segment [off[s], off[s+1]) of `a`.  Segments of up to
// 32 items: one warp (bitonic network over the lanes); up to kSortTile: one
// CTA (bitonic in shared memory); longer: one CTA sorts its tiles and places
// every item at its rank (its index in its tile plus, for each other tile, the
// items below it there: a binary search); items are distinct.
constexpr int kSortThreads = 512;
constexpr int kSortTile = 4096;

template <class T>
__device__ __forceinline__ T max_item() { return ~T(0); }

// Lists of the segments the CTA kernels sort: [0] count of mid, [1] of long.
template <class T>
__global__ void sort_small_kernel(T* a, const uint32_t* off, int nseg, int* mid, int* lng, int* cnt) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = w; s < nseg; s += nw) {
    const uint32_t b = off[s], n = off[s + 1] - b;
    if (n <= 1) continue;
    if (n > 32) {
      if (lane == 0) {
        if (n <= (uint32_t)kSortTile) mid[atomicAdd(&cnt[0], 1)] = s;
        else lng[atomicAdd(&cnt[1], 1)] = s;
      }
      continue;
    }
    T x = (uint32_t)lane < n ? a[b + lane] : max_item<T>();
    for (int k = 2; k <= 32; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        const T y = __shfl_xor_sync(kAllLanes, x, j);
        const bool up = (lane & k) == 0;
        const bool lower = (lane & j) == 0;
        // the lower lane of a pair keeps the min in an ascending run
        x = (lower == up) ? (x < y ? x : y) : (x < y ? y : x);
      }
    if ((uint32_t)lane < n) a[b + lane] = x;
  }
}

// Bitonic sort of n <= kSortTile items in shared memory (padded to a power of two).
template <class T>
__device__ void cta_sort(T* buf, int n) {
  int m = 1;
  while (m < n) m <<= 1;
  for (int i = n + threadIdx.x; i < m; i += blockDim.x) buf[i] = max_item<T>();
  __syncthreads();
  for (int k = 2; k <= m; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const T x = buf[i], y = buf[p];
          const bool up = (i & k) == 0;
          if ((x > y) == up) { buf[i] = y; buf[p] = x; }
        }
      }
      __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(kSortThreads) sort_mid_kernel(T* a, const uint32_t* off, const int* mid,
                                                                const int* cnt) {
  __shared__ T buf[kSortTile];
  const int nm = cnt[0];
  for (int i = blockIdx.x; i < nm; i += gridDim.x) {
    const int s = mid[i];
    const uint32_t b = off[s];
    const int n = (int)(off[s + 1] - b);
    for (int k = threadIdx.x; k < n; k += blockDim.x) buf[k] = a[b + k];
    cta_sort(buf, n);
    for (int k = threadIdx.x; k < n; k += blockDim.x) a[b + k] = buf[k];
    __syncthreads();
  }
}

// First index in the ascending t[0, n) with t[idx] >= x.
template <class T>
__device__ __forceinline__ int lower_bound_items(const T* t, int n, T x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (t[m] < x) lo = m + 1; else hi = m;
  }
  return lo;
}

// Long segments: the chunks (kSortTile items) of all of them and then all
// their items are spread over the grid.  lpre[i] / ipre[i]: chunks / items of
// the long segments before list entry i (one thread fills them; the long
// segments are few).
__global__ void sort_long_prefix_kernel(const uint32_t* off, const int* lng, const int* cnt, int* lpre,
                                        long long* ipre) {
  const int nl = cnt[1];
  int c = 0;
  long long it = 0;
  for (int i = 0; i < nl; i++) {
    lpre[i] = c;
    ipre[i] = it;
    const uint32_t n = off[lng[i] + 1] - off[lng[i]];
    c += (int)((n + kSortTile - 1) / kSortTile);
    it += n;
  }
  lpre[nl] = c;
  ipre[nl] = it;
}

// The list entry i with pre[i] <= x < pre[i + 1].
template <class P>
__device__ __forceinline__ int entry_of(const P* pre, int n, P x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int m = (lo + hi + 1) >> 1;
    if (pre[m] <= x) lo = m; else hi = m - 1;
  }
  return lo;
}

template <class T>
__global__ void __launch_bounds__(kSortThreads) sort_long_chunks_kernel(T* a, const uint32_t* off, const int* lng,
                                                                        const int* cnt, const int* lpre) {
  __shared__ T buf[kSortTile];
  const int nl = cnt[1];
  if (nl == 0) return;
  const int nch = lpre[nl];
  for (int g = blockIdx.x; g < nch; g += gridDim.x) {
    const int i = entry_of(lpre, nl, g);
    const uint32_t b = off[lng[i]];
    const int n = (int)(off[lng[i] + 1] - b);
    const int c0 = (g - lpre[i]) * kSortTile;
    const int m = min(kSortTile, n - c0);
    for (int k = threadIdx.x; k < m; k += blockDim.x) buf[k] = a[b + c0 + k];
    cta_sort(buf, m);
    for (int k = threadIdx.x; k < m; k += blockDim.x) a[b + c0 + k] = buf[k];
    __syncthreads();
  }
}

// Every item of a long segment to its rank: its index in its chunk plus the
// items below it in each other chunk (binary searches; items are distinct).
template <class T>
__global__ void sort_long_rank_kernel(const T* a, T* tmp, const uint32_t* off, const int* lng, const int* cnt,
                                      const long long* ipre) {
  const int nl = cnt[1];
  if (nl == 0) return;
  const long long tot = ipre[nl];
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < tot;
       x += (long long)gridDim.x * blockDim.x) {
    const int i = entry_of(ipre, nl, x);
    const uint32_t b = off[lng[i]];
    const int n = (int)(off[lng[i] + 1] - b);
    const int k = (int)(x - ipre[i]);
    const T* seg = a + b;
    const T v = seg[k];
    const int c = k / kSortTile;
    int r = k - c * kSortTile;
    for (int c0 = 0; c0 < n; c0 += kSortTile)
      if (c0 != c * kSortTile) r += lower_bound_items(seg + c0, min(kSortTile, n - c0), v);
    tmp[b + r] = v;
  }
}

template <class T>
__global__ void sort_long_copy_kernel(T* a, const T* tmp, const uint32_t* off, const int* lng, const int* cnt,
                                      const long long* ipre) {
  const int nl = cnt[1];
  if (nl == 0) return;
  const long long tot = ipre[nl];
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < tot;
       x += (long long)gridDim.x * blockDim.x) {
    const int i = entry_of(ipre, nl, x);
    const uint32_t b = off[lng[i]] + (uint32_t)(x - ipre[i]);
    a[b] = tmp[b];
  }
}

// List scratch of segmented_sort for nseg segments, in ints: the mid and long
// lists, the long segments' chunk prefix (nseg + 1) and, 8-byte aligned, their
// item prefix (nseg + 1 long longs).
size_t sort_ipre_at(int nseg) { return (3 * (size_t)std::max(nseg, 1) + 2 + 1) & ~size_t(1); }
size_t sort_list_ints(int nseg) { return sort_ipre_at(nseg) + 2 * ((size_t)std::max(nseg, 1) + 1); }

template <class T>
cudaError_t segmented_sort(T* a, T* tmp, const uint32_t* off, int nseg, int* lists, int* cnt, int num_sms,
                           cudaStream_t st) {
  if (nseg <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int) * 2, st);
  if (e != cudaSuccess) return e;
  int* mid = lists;
  int* lng = lists + nseg;
  int* lpre = lists + 2 * (size_t)nseg;                                 // nseg + 1
  long long* ipre = reinterpret_cast<long long*>(lists + sort_ipre_at(nseg));
  const int blocks = std::max(1, std::min((nseg + 7) / 8, num_sms * 16));
  sort_small_kernel<T><<<blocks, 256, 0, st>>>(a, off, nseg, mid, lng, cnt);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  sort_mid_kernel<T><<<num_sms * 2, kSortThreads, 0, st>>>(a, off, mid, cnt);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  sort_long_prefix_kernel<<<1, 1, 0, st>>>(off, lng, cnt, lpre, ipre);
  sort_long_chunks_kernel<T><<<num_sms * 2, kSortThreads, 0, st>>>(a, off, lng, cnt, lpre);
  sort_long_rank_kernel<T><<<num_sms * 8, 256, 0, st>>>(a, tmp, off, lng, cnt, ipre);
  sort_long_copy_kernel<T><<<num_sms * 8, 256, 0, st>>>(a, tmp, off, lng, cnt, ipre);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- createInverse
__global__ void count_pins_kernel(const uint32_t* vnets, long long pins, uint32_t* cnt) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pins; k += (long long)gridDim.x * blockDim.x)
    atomicAdd(&cnt[vnets[k]], 1u);
}

// The vertex of pin slot k: the last v with vptr[v] <= k.
__device__ __forceinline__ int owner_of(const uint32_t* vptr, int nov, uint32_t k) {
  int lo = 0, hi = nov - 1;
  while (lo < hi) {
    const int m = (lo + hi + 1) >> 1;
    if (vptr[m] <= k) lo = m; else hi = m - 1;
  }
  return lo;
}

__global__ void scatter_pins_kernel(const uint32_t* vptr, const uint32_t* vnets, int nov, long long pins,
                                    const uint32_t* nptr, uint32_t* cursor, uint32_t* npins) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pins;
       k += (long long)gridDim.x * blockDim.x) {
    const uint32_t e = vnets[k];
    const int v = owner_of(vptr, nov, (uint32_t)k);
    npins[nptr[e] + atomicAdd(&cursor[e], 1u)] = (uint32_t)v;
  }
}

// ------------------------------------------------------------------- thinning
__global__ void thin_flags_kernel(const uint32_t* nptr, int noe, double size_lim, int thin_min, uint32_t* keep,
                                  uint32_t* kept_size) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < noe; e += gridDim.x * blockDim.x) {
    const int degree = (int)(nptr[e + 1] - nptr[e]);
    const bool k = (double)degree < size_lim && degree < thin_min;   // CN/cn.cpp:226
    keep[e] = k ? 1u : 0u;
    kept_size[e] = k ? (uint32_t)degree : 0u;
  }
}

// Kept nets' pins and sources at their new places (renum = scan of keep;
// toff = scan of the kept sizes, by old net index).
__global__ void thin_nets_kernel(const uint32_t* nptr, const uint32_t* npins, const int* src, int noe,
                                 const uint32_t* keep, const uint32_t* renum, const uint32_t* toff, uint32_t* tpins,
                                 int* tsrc) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int e = w; e < noe; e += nw) {
    if (!keep[e]) continue;
    const uint32_t r = renum[e], b = nptr[e], n = nptr[e + 1] - b, t = toff[e];
    for (uint32_t j = lane; j < n; j += 32) tpins[t + j] = npins[b + j];
    if (lane == 0) tsrc[r] = src[e];
  }
}

// Each vertex's kept nets, renumbered, in its own order: slot k of the
// vertex -> nets CSR goes to the scan of the kept slots before it.
__global__ void thin_slot_flags_kernel(const uint32_t* vnets, long long pins, const uint32_t* keep, uint32_t* sflag) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pins; k += (long long)gridDim.x * blockDim.x)
    sflag[k] = keep[vnets[k]];
}

__global__ void thin_slot_write_kernel(const uint32_t* vnets, long long pins, const uint32_t* keep,
                                       const uint32_t* renum, const uint32_t* sscan, uint32_t* tvnets) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pins;
       k += (long long)gridDim.x * blockDim.x) {
    const uint32_t e = vnets[k];
    if (keep[e]) tvnets[sscan[k]] = renum[e];
  }
}

__global__ void thin_vptr_kernel(const uint32_t* vptr, int nov, const uint32_t* sscan, uint32_t* tvptr) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v <= nov; v += gridDim.x * blockDim.x) tvptr[v] = sscan[vptr[v]];
}

// ------------------------------------------------------------------------ BFS
// Per search: dist (-1 unreached), net_key (first (frontier position, net
// index) that walks the net this level), vkey (smallest (frontier position,
// pair index) that reaches the vertex this level).
struct BfsBuf {
  int* dist;
  unsigned long long* net_key;   // [noe]
  unsigned char* net_done;       // [noe] walked in an earlier level
  unsigned long long* vkey;      // [nov]
  uint32_t* vpre;                // [pins] pins of the vertex's earlier nets (pair index of a net's first pin)
  int* frontier;                 // [nov]
  int* next_nets;                // [noe] nets walked this level
  unsigned long long* items;     // [nov] (pair index << 32) | vertex of the reached vertices
  unsigned long long* sort_tmp;  // [nov]
  uint32_t* bucket;              // [nov + 1] reached vertices per frontier position, then offsets
  uint32_t* cursor;              // [nov]
  uint32_t* foff;                // [nov + 1] nets of the frontier positions before each
  int* lists;                    // [sort_list_ints(nov)]
  int* cnt;                      // [8]: [0,1] sort lists, [2] nets this level, [3] reached, [4] min id
  uint32_t* scan_tmp;
};

__global__ void bfs_start_kernel(BfsBuf B, int nov, int noe, int s) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < max(nov, noe); v += gridDim.x * blockDim.x) {
    if (v < nov) {
      B.dist[v] = v == s ? 0 : -1;
      B.vkey[v] = ~0ull;
    }
    if (v < noe) {
      B.net_key[v] = ~0ull;
      B.net_done[v] = 0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) B.frontier[0] = s;
}

// Nets per frontier position, scanned into foff (nf + 1) by the caller.
__global__ void bfs_fdeg_kernel(BfsBuf B, const uint32_t* vptr, int nf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nf; i += gridDim.x * blockDim.x)
    B.foff[i] = i < nf ? vptr[B.frontier[i] + 1] - vptr[B.frontier[i]] : 0u;
}

// (a) every (frontier position i, net index k) pair bids for its net; the
// pairs are spread over the grid (a vertex may have millions of nets).
__global__ void bfs_bid_kernel(BfsBuf B, const uint32_t* vptr, const uint32_t* vnets, int nf) {
  const uint32_t tot = B.foff[nf];
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
    const int i = entry_of(B.foff, nf, t);
    const uint32_t k = t - B.foff[i];
    const uint32_t e = vnets[vptr[B.frontier[i]] + k];
    if (!B.net_done[e]) atomicMin(&B.net_key[e], ((unsigned long long)i << 32) | k);
  }
}

// (b) the nets bid for this level, listed once: the bid of (i, k) for net e
// wins iff net_key[e] == (i, k).
__global__ void bfs_list_nets_kernel(BfsBuf B, const uint32_t* vptr, const uint32_t* vnets, int nf) {
  const uint32_t tot = B.foff[nf];
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
    const int i = entry_of(B.foff, nf, t);
    const uint32_t k = t - B.foff[i];
    const uint32_t e = vnets[vptr[B.frontier[i]] + k];
    if (!B.net_done[e] && B.net_key[e] == (((unsigned long long)i << 32) | k)) {
      B.next_nets[atomicAdd(&B.cnt[2], 1)] = (int)e;
      B.net_done[e] = 1;
    }
  }
}

// (c) every listed net walks its pins: an unreached pin bids (i, pair index).
__global__ void bfs_walk_kernel(BfsBuf B, const uint32_t* vptr, const uint32_t* nptr, const uint32_t* npins) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int nn = B.cnt[2];
  for (int x = w; x < nn; x += nw) {
    const int e = B.next_nets[x];
    const unsigned long long nk = B.net_key[e];
    const int i = (int)(nk >> 32);
    const uint32_t k = (uint32_t)nk;
    const int v = B.frontier[i];
    const uint32_t q0 = B.vpre[vptr[v] + k];
    const uint32_t b = nptr[e], n = nptr[e + 1] - b;
    for (uint32_t j = lane; j < n; j += 32) {
      const uint32_t u = npins[b + j];
      if (B.dist[u] < 0) atomicMin(&B.vkey[u], ((unsigned long long)i << 32) | (q0 + j));
    }
  }
}

// (d) the reached vertices: their distance, and one count per frontier position.
__global__ void bfs_reached_kernel(BfsBuf B, int nov, int level) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nov; u += gridDim.x * blockDim.x) {
    const unsigned long long k = B.vkey[u];
    if (k == ~0ull || B.dist[u] >= 0) continue;
    B.dist[u] = level;
    atomicAdd(&B.bucket[(int)(k >> 32)], 1u);
    atomicAdd(&B.cnt[3], 1);
  }
}

// (e) the reached vertices into their frontier position's bucket, as
// (pair index, vertex) items, and keys cleared for the next level.
__global__ void bfs_bucket_kernel(BfsBuf B, int nov, int level) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nov; u += gridDim.x * blockDim.x) {
    const unsigned long long k = B.vkey[u];
    if (k == ~0ull) continue;
    B.vkey[u] = ~0ull;
    if (B.dist[u] != level) continue;
    const int i = (int)(k >> 32);
    B.items[B.bucket[i] + atomicAdd(&B.cursor[i], 1u)] = ((k & 0xffffffffull) << 32) | (unsigned)u;
  }
}

__global__ void bfs_next_kernel(BfsBuf B, int n, int* order, int at) {
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
    const int u = (int)(B.items[x] & 0xffffffffull);
    B.frontier[x] = u;
    if (order) order[at + x] = u;
    atomicMin(&B.cnt[4], u);
  }
}

__global__ void vpre_fill_kernel(const uint32_t* vnets, const uint32_t* nptr, long long pins, uint32_t* vpre) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pins; k += (long long)gridDim.x * blockDim.x)
    vpre[k] = nptr[vnets[k] + 1] - nptr[vnets[k]];
}

// The scan ran over all slots (modulo 2^32); a vertex's own prefix is the
// difference to its first slot's value, which fits 32 bits.
__global__ void vpre_base_kernel(const uint32_t* vptr, int nov, long long pins, const uint32_t* vpre,
                                 uint32_t* base) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nov; v += gridDim.x * blockDim.x)
    base[v] = (long long)vptr[v] < pins ? vpre[vptr[v]] : 0u;
}

__global__ void vpre_rebase_kernel(const uint32_t* vptr, int nov, long long pins, const uint32_t* base,
                                   uint32_t* vpre) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pins;
       k += (long long)gridDim.x * blockDim.x)
    vpre[k] -= base[owner_of(vptr, nov, (uint32_t)k)];
}

__global__ void bfs_set_kernel(int* cnt) {
  cnt[2] = 0;
  cnt[3] = 0;
  cnt[4] = 0x7fffffff;
}

__global__ void bfs_first_kernel(int* order, int s) { order[0] = s; }

// Owner of a set of device buffers, freed on scope exit (after the caller
// synchronised its stream).
struct DevBufs {
  std::vector<void*> p;
  cudaError_t err = cudaSuccess;
  template <class T>
  T* get(size_t n) {
    if (err != cudaSuccess) return nullptr;
    void* q = nullptr;
    err = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (err != cudaSuccess) return nullptr;
    p.push_back(q);
    return static_cast<T*>(q);
  }
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
};

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return FP_OK;
  if (e == cudaErrorMemoryAllocation) return FP_ERR_NOMEM;
  return FP_ERR_CUDA;
}

int grid_for(long long n, int num_sms) {
  return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)num_sms * 16));
}

// The net -> pins CSR (pins ascending per net) of a device vertex -> nets CSR.
cudaError_t transpose(const uint32_t* vptr, const uint32_t* vnets, int nov, int noe, long long pins, uint32_t* nptr,
                      uint32_t* npins, uint32_t* cursor, uint32_t* scan_tmp, int* lists, int* cnt,
                      uint32_t* sort_tmp, int num_sms, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(nptr, 0, sizeof(uint32_t) * ((size_t)noe + 1), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * std::max(noe, 1), st);
  if (e != cudaSuccess) return e;
  if (pins > 0) {
    count_pins_kernel<<<grid_for(pins, num_sms), 256, 0, st>>>(vnets, pins, nptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if ((e = scan_exclusive(nptr, nptr, (long long)noe + 1, scan_tmp, st)) != cudaSuccess) return e;
  if (pins > 0) {
    scatter_pins_kernel<<<grid_for(pins, num_sms), 256, 0, st>>>(vptr, vnets, nov, pins, nptr, cursor, npins);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return segmented_sort<uint32_t>(npins, sort_tmp, nptr, noe, lists, cnt, num_sms, st);
}

// Host checks that keep every device index in bounds.
bool vertex_csr_ok(int nov, int noe, long long pins, const uint32_t* vptr, const uint32_t* vnets) {
  if (nov <= 0 || noe < 0 || pins < 0 || pins >= (1ll << 31) || !vptr || (pins > 0 && !vnets)) return false;
  if (vptr[0] != 0 || (long long)vptr[nov] != pins) return false;
  for (int v = 0; v < nov; v++)
    if (vptr[v + 1] < vptr[v]) return false;
  for (long long k = 0; k < pins; k++)
    if (vnets[k] >= (uint32_t)noe) return false;
  return true;
}

}  // namespace

int create_inverse_device(int device, cudaStream_t st, int num_sms, int nov, int noe, long long pins,
                          const uint32_t* vptr_h, const uint32_t* vnets_h, uint32_t* nptr_h, uint32_t* npins_h) {
  if (!vertex_csr_ok(nov, noe, pins, vptr_h, vnets_h) || !nptr_h || (pins > 0 && !npins_h)) return FP_ERR_INVALID;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return status_of(e);
  DevBufs M;
  uint32_t* vptr = M.get<uint32_t>((size_t)nov + 1);
  uint32_t* vnets = M.get<uint32_t>(pins);
  uint32_t* nptr = M.get<uint32_t>((size_t)noe + 1);
  uint32_t* npins = M.get<uint32_t>(pins);
  uint32_t* cursor = M.get<uint32_t>(noe);
  uint32_t* stmp = M.get<uint32_t>(scan_scratch((long long)noe + 1));
  int* lists = M.get<int>(sort_list_ints(noe));
  int* cnt = M.get<int>(8);
  uint32_t* sort_tmp = M.get<uint32_t>(pins);
  if (M.err != cudaSuccess) return status_of(M.err);
  e = cudaMemcpyAsync(vptr, vptr_h, sizeof(uint32_t) * ((size_t)nov + 1), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && pins > 0)
    e = cudaMemcpyAsync(vnets, vnets_h, sizeof(uint32_t) * pins, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = transpose(vptr, vnets, nov, noe, pins, nptr, npins, cursor, stmp, lists, cnt, sort_tmp, num_sms, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(nptr_h, nptr, sizeof(uint32_t) * ((size_t)noe + 1), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && pins > 0)
    e = cudaMemcpyAsync(npins_h, npins, sizeof(uint32_t) * pins, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return status_of(e);
}

int thin_nets_device(int device, cudaStream_t st, int num_sms, const fp_hypergraph* h, double size_lim,
                     int thin_min, HostGraph& out) {
  const int nov = h->nov, noe = h->noe;
  const long long pins = h->pins;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return status_of(e);
  DevBufs M;
  uint32_t* vptr = M.get<uint32_t>((size_t)nov + 1);
  uint32_t* vnets = M.get<uint32_t>(pins);
  uint32_t* nptr = M.get<uint32_t>((size_t)noe + 1);
  uint32_t* npins = M.get<uint32_t>(pins);
  int* src = M.get<int>(noe);
  uint32_t* keep = M.get<uint32_t>((size_t)noe + 1);
  uint32_t* renum = M.get<uint32_t>((size_t)noe + 1);
  uint32_t* toff = M.get<uint32_t>((size_t)noe + 1);   // kept sizes, then their offsets (old net order)
  uint32_t* tpins = M.get<uint32_t>(pins);
  int* tsrc = M.get<int>(noe);
  uint32_t* tvptr = M.get<uint32_t>((size_t)nov + 1);
  uint32_t* tvnets = M.get<uint32_t>(pins);
  uint32_t* sscan = M.get<uint32_t>((size_t)pins + 1);   // kept slots of the vertex -> nets CSR, scanned
  uint32_t* stmp = M.get<uint32_t>(scan_scratch(std::max<long long>(std::max(noe, nov), pins) + 1));
  if (M.err != cudaSuccess) return status_of(M.err);
  auto up = [&](void* d, const void* s, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(d, s, bytes, cudaMemcpyHostToDevice, st);
  };
  up(vptr, h->vptr, sizeof(uint32_t) * ((size_t)nov + 1));
  up(vnets, h->vnets, sizeof(uint32_t) * pins);
  up(nptr, h->nptr, sizeof(uint32_t) * ((size_t)noe + 1));
  up(npins, h->npins, sizeof(uint32_t) * pins);
  up(src, h->src, sizeof(int) * noe);
  if (e == cudaSuccess) e = cudaMemsetAsync(keep + noe, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(toff + noe, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess && noe > 0) {
    thin_flags_kernel<<<grid_for(noe, num_sms), 256, 0, st>>>(nptr, noe, size_lim, thin_min, keep, toff);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = scan_exclusive(keep, renum, (long long)noe + 1, stmp, st);
  if (e == cudaSuccess) e = scan_exclusive(toff, toff, (long long)noe + 1, stmp, st);
  uint32_t tot[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[0], renum + noe, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[1], toff + noe, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && noe > 0) {
    thin_nets_kernel<<<grid_for((long long)noe * 32, num_sms), 256, 0, st>>>(nptr, npins, src, noe, keep, renum,
                                                                             toff, tpins, tsrc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(sscan + pins, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess && pins > 0) {
    thin_slot_flags_kernel<<<grid_for(pins, num_sms), 256, 0, st>>>(vnets, pins, keep, sscan);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = scan_exclusive(sscan, sscan, pins + 1, stmp, st);
  if (e == cudaSuccess && pins > 0) {
    thin_slot_write_kernel<<<grid_for(pins, num_sms), 256, 0, st>>>(vnets, pins, keep, renum, sscan, tvnets);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    thin_vptr_kernel<<<grid_for((long long)nov + 1, num_sms), 256, 0, st>>>(vptr, nov, sscan, tvptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return status_of(e);
  const int tnoe = (int)tot[0];
  const long long tpn = (long long)tot[1];
  out = HostGraph();
  out.nov = nov;
  out.noe = tnoe;
  out.pins = tpn;
  out.vptr.resize((size_t)nov + 1);
  out.vnets.resize(tpn);
  out.nptr.resize((size_t)tnoe + 1);
  out.npins.resize(tpn);
  out.src.resize(tnoe);
  std::vector<uint32_t> toff_h((size_t)noe + 1), keep_h((size_t)noe);
  auto down = [&](void* d, const void* s, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToHost, st);
  };
  down(out.vptr.data(), tvptr, sizeof(uint32_t) * ((size_t)nov + 1));
  down(out.vnets.data(), tvnets, sizeof(uint32_t) * tpn);
  down(out.npins.data(), tpins, sizeof(uint32_t) * tpn);
  down(out.src.data(), tsrc, sizeof(int) * tnoe);
  down(toff_h.data(), toff, sizeof(uint32_t) * ((size_t)noe + 1));
  down(keep_h.data(), keep, sizeof(uint32_t) * noe);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return status_of(e);
  int r = 0;
  for (int x = 0; x < noe; x++)
    if (keep_h[x]) out.nptr[r++] = toff_h[x];
  out.nptr[tnoe] = (uint32_t)tpn;
  if (h->weights) out.weights.assign(h->weights, h->weights + nov);
  return FP_OK;
}

int bfs_order_device(int device, cudaStream_t st, int num_sms, const fp_hypergraph* h, int start, int* ordering,
                     int* far_out) {
  const int nov = h->nov, noe = h->noe;
  const long long pins = h->pins;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return status_of(e);
  DevBufs M;
  uint32_t* vptr = M.get<uint32_t>((size_t)nov + 1);
  uint32_t* vnets = M.get<uint32_t>(pins);
  uint32_t* nptr = M.get<uint32_t>((size_t)noe + 1);
  uint32_t* npins = M.get<uint32_t>(pins);
  const size_t nmax = (size_t)std::max(nov, noe);
  uint32_t* cursor = M.get<uint32_t>(nmax);
  uint32_t* stmp = M.get<uint32_t>(scan_scratch((long long)nmax + 1));
  int* lists = M.get<int>(sort_list_ints((int)nmax));
  uint32_t* sort32 = M.get<uint32_t>(pins);
  int* order = M.get<int>(nov);
  BfsBuf B{};
  B.dist = M.get<int>(nov);
  B.net_key = M.get<unsigned long long>(noe);
  B.net_done = M.get<unsigned char>(noe);
  B.vkey = M.get<unsigned long long>(nov);
  B.vpre = M.get<uint32_t>(pins);
  B.frontier = M.get<int>(nov);
  B.next_nets = M.get<int>(noe);
  B.items = M.get<unsigned long long>(nov);
  B.sort_tmp = M.get<unsigned long long>(nov);
  B.bucket = M.get<uint32_t>((size_t)nov + 1);
  B.foff = M.get<uint32_t>((size_t)nov + 1);
  B.cursor = cursor;
  B.lists = lists;
  B.cnt = M.get<int>(8);
  B.scan_tmp = stmp;
  if (M.err != cudaSuccess) return status_of(M.err);
  e = cudaMemcpyAsync(vptr, h->vptr, sizeof(uint32_t) * ((size_t)nov + 1), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && pins > 0)
    e = cudaMemcpyAsync(vnets, h->vnets, sizeof(uint32_t) * pins, cudaMemcpyHostToDevice, st);
  // createInverse's order: each net's pins ascending
  if (e == cudaSuccess)
    e = transpose(vptr, vnets, nov, noe, pins, nptr, npins, cursor, stmp, lists, B.cnt, sort32, num_sms, st);
  // vpre: the pair index of the first pin of each of a vertex's nets
  if (e == cudaSuccess && pins > 0) {
    vpre_fill_kernel<<<grid_for(pins, num_sms), 256, 0, st>>>(vnets, nptr, pins, B.vpre);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = scan_exclusive(B.vpre, B.vpre, pins, stmp, st);
    if (e == cudaSuccess) {
      vpre_base_kernel<<<grid_for(nov, num_sms), 256, 0, st>>>(vptr, nov, pins, B.vpre, cursor);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      vpre_rebase_kernel<<<grid_for(pins, num_sms), 256, 0, st>>>(vptr, nov, pins, cursor, B.vpre);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) return status_of(e);
  int* h_cnt = nullptr;
  if ((e = cudaMallocHost(&h_cnt, sizeof(int) * 8)) != cudaSuccess) return status_of(e);
  struct PinnedFree {
    int* p;
    ~PinnedFree() { cudaFreeHost(p); }
  } pf{h_cnt};
  // One search from s: returns the lowest id of the last level and the number
  // of vertices reached; lists them in `ord` (device) if not null.
  auto search = [&](int s, int* ord, int* far, int* reached) -> cudaError_t {
    cudaError_t x = cudaSuccess;
    bfs_start_kernel<<<grid_for(std::max(nov, noe), num_sms), 256, 0, st>>>(B, nov, noe, s);
    if ((x = cudaGetLastError()) != cudaSuccess) return x;
    if (ord) {
      bfs_first_kernel<<<1, 1, 0, st>>>(ord, s);
      if ((x = cudaGetLastError()) != cudaSuccess) return x;
    }
    int nf = 1, level = 0, total = 1;
    *far = s;
    for (;;) {
      level++;
      if ((x = cudaMemsetAsync(B.bucket, 0, sizeof(uint32_t) * ((size_t)nf + 1), st)) != cudaSuccess) return x;
      if ((x = cudaMemsetAsync(B.cursor, 0, sizeof(uint32_t) * nf, st)) != cudaSuccess) return x;
      bfs_set_kernel<<<1, 1, 0, st>>>(B.cnt);
      bfs_fdeg_kernel<<<grid_for((long long)nf + 1, num_sms), 256, 0, st>>>(B, vptr, nf);
      if ((x = cudaGetLastError()) != cudaSuccess) return x;
      if ((x = scan_exclusive(B.foff, B.foff, (long long)nf + 1, B.scan_tmp, st)) != cudaSuccess) return x;
      bfs_bid_kernel<<<num_sms * 16, 256, 0, st>>>(B, vptr, vnets, nf);
      bfs_list_nets_kernel<<<num_sms * 16, 256, 0, st>>>(B, vptr, vnets, nf);
      bfs_walk_kernel<<<num_sms * 8, 256, 0, st>>>(B, vptr, nptr, npins);
      bfs_reached_kernel<<<grid_for(nov, num_sms), 256, 0, st>>>(B, nov, level);
      if ((x = cudaGetLastError()) != cudaSuccess) return x;
      if ((x = cudaMemcpyAsync(h_cnt, B.cnt, sizeof(int) * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return x;
      if ((x = cudaStreamSynchronize(st)) != cudaSuccess) return x;
      const int got = h_cnt[3];
      if (got == 0) break;
      if ((x = scan_exclusive(B.bucket, B.bucket, (long long)nf + 1, B.scan_tmp, st)) != cudaSuccess) return x;
      bfs_bucket_kernel<<<grid_for(nov, num_sms), 256, 0, st>>>(B, nov, level);
      if ((x = cudaGetLastError()) != cudaSuccess) return x;
      if ((x = segmented_sort<unsigned long long>(B.items, B.sort_tmp, B.bucket, nf, B.lists, B.cnt, num_sms, st)) !=
          cudaSuccess)
        return x;
      bfs_set_kernel<<<1, 1, 0, st>>>(B.cnt);
      bfs_next_kernel<<<grid_for(got, num_sms), 256, 0, st>>>(B, got, ord, total);
      if ((x = cudaGetLastError()) != cudaSuccess) return x;
      if ((x = cudaMemcpyAsync(h_cnt, B.cnt, sizeof(int) * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return x;
      if ((x = cudaStreamSynchronize(st)) != cudaSuccess) return x;
      *far = h_cnt[4];
      total += got;
      nf = got;
    }
    *reached = total;
    return cudaSuccess;
  };
  int f1 = 0, f2 = 0, f3 = 0, reached = 0;
  if ((e = search(start, nullptr, &f1, &reached)) != cudaSuccess) return status_of(e);
  if ((e = search(f1, nullptr, &f2, &reached)) != cudaSuccess) return status_of(e);
  if ((e = cudaMemsetAsync(order, 0xff, sizeof(int) * nov, st)) != cudaSuccess) return status_of(e);
  if ((e = search(f2, order, &f3, &reached)) != cudaSuccess) return status_of(e);
  e = cudaMemcpyAsync(ordering, order, sizeof(int) * nov, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return status_of(e);
  if (far_out) {
    far_out[0] = f1;
    far_out[1] = f2;
  }
  return reached == nov ? FP_OK : FP_ERR_UNSUPPORTED;
}

}  // namespace fp
