// Helpers shared by the speculative (grid-wide) refinement kernels.
#pragma once

#include "fp_device.cuh"

#include <cooperative_groups.h>

namespace fp {
namespace spec {

namespace cg = cooperative_groups;

constexpr int kSThreads = 256;
constexpr int kSWarps = kSThreads / 32;
constexpr int kNone = 0x7fffffff;
constexpr unsigned kAll = 0xffffffffu;

// Global nanosecond timer (per-phase time statistics).
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Loads of state that other SMs write (L2, not the SM's L1).
template <class T>
__device__ __forceinline__ T lds(const T* p) { return __ldcg(p); }

// Grid-wide barrier of a co-resident (cooperatively launched) grid with a
// bounded wait.  bar[0] = arrivals, bar[2] = abort flag.  Every CTA adds to
// bar[0] once per barrier: CTA 0 adds 2^31 - (gridDim.x - 1), the others 1, so
// bit 31 flips exactly when the last CTA arrives and the low bits return to
// their value -- no reset, one atomic per CTA.  Returns false in every thread
// of the CTA if the wait gave up (another CTA stopped arriving) or another CTA
// aborted; the kernel then reports FP_ERR_DEVICE_TIMEOUT through `status` and
// returns.
//
// Failure-detection test hooks (fp_debug_barrier_fault; both zero unless a
// test sets them): bar[1] = n > 0 makes the grid's last CTA leave at its n-th
// barrier without arriving, as a CTA that stopped would; bar[3] > 0 replaces
// the poll limit, so that the other CTAs give up after that many polls.
// Per-warp / per-CTA timing statistics (atomics in the hot loops): collected
// only by builds with FP_TIMING_STATS defined.
#ifdef FP_TIMING_STATS
constexpr bool kTimingStats = true;
#else
constexpr bool kTimingStats = false;
#endif

constexpr unsigned kBarrierSpins = 1u << 21;   // polls of an L2 line with 32 ns naps: about a second or more

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Barriers this CTA has entered in this launch (thread 0 only); a kernel
// calls barrier_start() before its first grid_barrier.
static __shared__ unsigned s_barriers;
__device__ __forceinline__ void barrier_start() {
  if (threadIdx.x == 0) s_barriers = 0;
}

__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned n = ++s_barriers;
    const unsigned leave_at = __ldcg(&bar[1]);
    if (leave_at != 0u && n == leave_at && blockIdx.x == gridDim.x - 1) {
      ok = 0;   // test hook: this CTA stops arriving
    } else {
      const unsigned limit = __ldcg(&bar[3]) != 0u ? __ldcg(&bar[3]) : kBarrierSpins;
      const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
      __threadfence();
      const unsigned old = atomicAdd(&bar[0], inc);
      unsigned spins = 0;
      while (((old ^ ld_acquire(&bar[0])) & 0x80000000u) == 0u) {
        if ((++spins & 255u) == 0u && (ld_acquire(&bar[2]) != 0u || spins > limit)) {
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
      if (!ok) {
        atomicExch(&bar[2], 1u);
        atomicCAS(status, 0, -4);   // FP_ERR_DEVICE_TIMEOUT
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ int warp_sum(int x) {
  for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(kAll, x, off);
  return x;
}
__device__ __forceinline__ int warp_min(int x) {
  for (int off = 16; off; off >>= 1) x = min(x, __shfl_xor_sync(kAll, x, off));
  return x;
}
__device__ __forceinline__ int warp_max(int x) {
  for (int off = 16; off; off >>= 1) x = max(x, __shfl_xor_sync(kAll, x, off));
  return x;
}
__device__ __forceinline__ long long warp_sum64(long long x) {
  for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(kAll, x, off);
  return x;
}

__device__ __forceinline__ LdgKey warp_ldg_argmax(LdgKey k) {
  for (int off = 16; off; off >>= 1) {
    LdgKey o = shfl_key(k, off);
    if (ldg_better(o, k)) k = o;
  }
  return k;
}

struct Carve {
  unsigned char* p;
  template <class T>
  __device__ T* take(size_t n) {
    T* r = reinterpret_cast<T*>(p);
    p += (n * sizeof(T) + 15) & ~size_t(15);
    return r;
  }
};

// First index of the ascending list `pos_list` (n entries) with value >= x.
__device__ __forceinline__ int lower_bound_pos(const int* pos_list, int n, int x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&pos_list[mid]) < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Contiguous share [*b, *e) of a vertex's deg nets for warp wi of nw warps
// (balances vertices with few large nets across the warps of a group).
__device__ __forceinline__ void net_range(int deg, int wi, int nw, int* b, int* e) {
  const int g = (deg + nw - 1) / nw;
  *b = min(wi * g, deg);
  *e = min(*b + g, deg);
}

// Adds to the warp's part tally the nets [nb, min(nb + 32, deg)) of a vertex
// (base: its offset in vnets; deg: the end of the warp's nets): for every listed part, the number of
// nets listing it (cnt) and the (net index, slot) of its first sighting (first);
// returns this lane's count of nets where `own` has exactly one pin.  Slots of
// the 32 nets are flattened across the warp (inclusive scan of list lengths).
__device__ __forceinline__ int tally_batch(const DevInstance& I, int own, uint32_t base, int nb, int deg, int* cnt,
                                           unsigned long long* first) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  const int k = nb + lane;
  int s = 0, n = 0;
  if (k < deg) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    s = (int)__ldg(&I.nptr[e]);
    const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
    n = lds(&I.ep_len[e]);
    if (n < 0 || n > cap) { dev_fail(I.status, kDevErrInvalid); n = 0; }
  }
  int incl = n;
  for (int off = 1; off < 32; off <<= 1) {
    const int t = __shfl_up_sync(kAll, incl, off);
    if (lane >= off) incl += t;
  }
  const int total = __shfl_sync(kAll, incl, 31);
  int c1 = 0;
  // kU slots per lane per step: the loads of one step are independent, which
  // keeps kU requests per lane in flight (the walk is latency-bound otherwise).
  constexpr int kU = 4;
  for (int f0 = 0; f0 < total; f0 += 32 * kU) {
    int aa[kU], key_net[kU], key_slot[kU], pp[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int f = f0 + u * 32 + lane;
      int lo = 0, hi = 31;
#pragma unroll
      for (int it = 0; it < 5; it++) {
        const int mid = (lo + hi) >> 1;
        const int val = __shfl_sync(kAll, incl, mid);
        if (f < val) hi = mid; else lo = mid + 1;
      }
      const int sl = __shfl_sync(kAll, s, lo);
      const int nl = __shfl_sync(kAll, n, lo);
      const int il = __shfl_sync(kAll, incl, lo);
      const int j = f - (il - nl);              // slot within net nb + lo
      key_net[u] = nb + lo;
      key_slot[u] = j;
      aa[u] = f < total ? sl + j : -1;          // slot address, -1 past the end
    }
    int cc[kU];
    // parts and counts are loaded together: no second round trip for own's count
#pragma unroll
    for (int u = 0; u < kU; u++) {
      pp[u] = aa[u] >= 0 ? lds(&I.ep_part[aa[u]]) : -1;
      cc[u] = aa[u] >= 0 ? lds(&I.ep_cnt[aa[u]]) : 0;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (aa[u] < 0) continue;
      const int p = pp[u];
      if ((unsigned)p >= (unsigned)K) {
        dev_fail(I.status, kDevErrInvalid);
        continue;
      }
      atomicAdd(&cnt[p], 1);
      atomicMin(&first[p], ((unsigned long long)key_net[u] << 32) | (unsigned)key_slot[u]);
      if (p == own && cc[u] == 1) c1++;
    }
  }
  return c1;
}

// Record of one (vertex, net) pair of a vertex about to move own -> d, one
// 32-bit word at the pair's vnets index: the slot of `own` in the net's list,
// the slot of `d` (kNoSlot: not listed), own's count there is 1 (the move takes
// own off the list), v is the net's source.  The slots stay valid until the
// move is committed: a net whose part set changes has no other mover in the
// round, and count-only moves never move slots.
constexpr uint32_t kNoSlot = 0x1fffu;   // slots < K <= 4096
__device__ __forceinline__ uint32_t rec_pack(int jo, int jd, bool rem, bool src) {
  return (uint32_t)jo | ((uint32_t)(jd < 0 ? kNoSlot : (uint32_t)jd) << 13) | (rem ? 1u << 26 : 0u) |
         (src ? 1u << 27 : 0u);
}
__device__ __forceinline__ int rec_jo(uint32_t r) { return (int)(r & 0x1fffu); }
__device__ __forceinline__ int rec_jd(uint32_t r) {
  const uint32_t j = (r >> 13) & 0x1fffu;
  return j == kNoSlot ? -1 : (int)j;
}
__device__ __forceinline__ bool rec_rem(uint32_t r) { return (r >> 26) & 1u; }
__device__ __forceinline__ bool rec_add(uint32_t r) { return ((r >> 13) & 0x1fffu) == kNoSlot; }
__device__ __forceinline__ bool rec_src(uint32_t r) { return (r >> 27) & 1u; }
// The move changes the net's part set (or, with volumes, the net's send side).
__device__ __forceinline__ bool rec_setchange(uint32_t r, bool vol) {
  return rec_rem(r) || rec_add(r) || (vol && rec_src(r));
}

// Writes the records of nets [nb, nb + 32) of v for the move own -> d into
// rec[base + k].  Slots of the 32 lists are flattened across the warp as in
// tally_batch.  sj / sd / sc: 32 ints each of per-warp scratch.  Returns the
// record of this lane's net nb + lane and its net id in *e_out (-1 past deg).
__device__ __forceinline__ uint32_t locate_batch(const DevInstance& I, uint32_t* rec, int v, int own, int d,
                                                 uint32_t base, int nb, int deg, int* sj, int* sd, int* sc,
                                                 int* e_out) {
  const int lane = threadIdx.x & 31;
  const int k = nb + lane;
  int s = 0, n = 0, e = -1;
  if (k < deg) {
    e = (int)__ldg(&I.vnets[base + k]);
    s = (int)__ldg(&I.nptr[e]);
    const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
    n = lds(&I.ep_len[e]);
    if (n < 0 || n > cap) { dev_fail(I.status, kDevErrInvalid); n = 0; }
  }
  sj[lane] = -1;
  sd[lane] = -1;
  sc[lane] = 0;
  int incl = n;
  for (int off = 1; off < 32; off <<= 1) {
    const int t = __shfl_up_sync(kAll, incl, off);
    if (lane >= off) incl += t;
  }
  const int total = __shfl_sync(kAll, incl, 31);
  __syncwarp();
  constexpr int kU = 4;
  for (int f0 = 0; f0 < total; f0 += 32 * kU) {
    int aa[kU], kn[kU], kj[kU], pp[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int f = f0 + u * 32 + lane;
      int lo = 0, hi = 31;
#pragma unroll
      for (int it = 0; it < 5; it++) {
        const int mid = (lo + hi) >> 1;
        const int val = __shfl_sync(kAll, incl, mid);
        if (f < val) hi = mid; else lo = mid + 1;
      }
      const int sl = __shfl_sync(kAll, s, lo);
      const int nl = __shfl_sync(kAll, n, lo);
      const int il = __shfl_sync(kAll, incl, lo);
      kn[u] = lo;
      kj[u] = f - (il - nl);
      aa[u] = f < total ? sl + kj[u] : -1;
    }
    int cc[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      pp[u] = aa[u] >= 0 ? lds(&I.ep_part[aa[u]]) : -1;
      cc[u] = aa[u] >= 0 ? lds(&I.ep_cnt[aa[u]]) : 0;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (aa[u] < 0) continue;
      // own and d are listed at most once per net: one writer per entry
      if (pp[u] == own) {
        sj[kn[u]] = kj[u];
        sc[kn[u]] = cc[u] == 1;
      }
      if (pp[u] == d) sd[kn[u]] = kj[u];
    }
  }
  __syncwarp();
  uint32_t r = 0;
  if (k < deg) {
    const int jo = sj[lane];
    if (jo < 0) {
      dev_fail(I.status, kDevErrInvalid);   // v's own part must be listed on v's nets
    } else {
      r = rec_pack(jo, sd[lane], sc[lane] != 0, __ldg(&I.src[e]) == v);
      rec[base + k] = r;
    }
  }
  __syncwarp();
  *e_out = e;
  return r;
}

// Volume arrays updated while a vertex moves (MSV: send only; MSRV: both).
struct Vol {
  int* send;
  int* recv;
};

// commit_net with the slots taken from the move's record (no list search).
__device__ __forceinline__ void commit_rec(const DevInstance& I, int v, int own, int d, int e, uint32_t r,
                                           const Vol* vol) {
  const int s = (int)__ldg(&I.nptr[e]);
  const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
  int n = lds(&I.ep_len[e]);
  const int jo = rec_jo(r);
  int jd = rec_jd(r);
  if (jo >= n || jd >= n || n > cap || (jd < 0 && n == cap && !rec_rem(r))) {
    dev_fail(I.status, kDevErrInvalid);
    return;
  }
  const int sv = vol ? __ldg(&I.src[e]) : -1;
  const int sp = (vol && sv != v) ? lds(&I.part_vec[sv]) : d;
  if (vol && sv == v) atomicAdd(&vol->send[own], -(n - 1));
  const int co = atomicAdd(&I.ep_cnt[s + jo], -1) - 1;
  if (co == 0) {
    const int last = n - 1;
    I.ep_part[s + jo] = lds(&I.ep_part[s + last]);
    I.ep_cnt[s + jo] = lds(&I.ep_cnt[s + last]);
    I.ep_part[s + last] = -1;
    I.ep_cnt[s + last] = 0;
    if (jd == last) jd = jo;
    n = last;
    if (vol && sv != v) {
      atomicAdd(&vol->send[sp], -1);
      if (vol->recv) atomicAdd(&vol->recv[own], -1);
    }
  } else {
    if (vol && vol->recv && sv == v) atomicAdd(&vol->recv[own], 1);
  }
  if (vol && sv == v) atomicAdd(&vol->send[d], n - 1);
  if (jd >= 0) {
    atomicAdd(&I.ep_cnt[s + jd], 1);
    if (vol && vol->recv && sv == v) atomicAdd(&vol->recv[d], -1);
  } else {
    I.ep_part[s + n] = d;
    I.ep_cnt[s + n] = 1;
    n++;
    if (vol) {
      atomicAdd(&vol->send[sp], 1);
      if (vol->recv && sv != v) atomicAdd(&vol->recv[d], 1);
    }
  }
  if (co == 0 || jd < 0) I.ep_len[e] = n;
}

// One thread applies vertex v's move own -> d to net e: the reference's
// REMOVAL (decrement, swap-with-last when the count reaches zero) then ADDING
// (increment or append), TV/partition.cpp:388-436, with the send / received
// volume bookkeeping of MGV/partition.cpp:376-449 and MSRV/partition.cpp:387-483.
__device__ __forceinline__ void commit_net(const DevInstance& I, int v, int own, int d, int e, const Vol* vol) {
  const int s = (int)__ldg(&I.nptr[e]);
  const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
  int n = lds(&I.ep_len[e]);
  int jo = -1, jd = -1;
  for (int j = 0; j < n && (jo < 0 || jd < 0); j++) {
    const int p = lds(&I.ep_part[s + j]);
    if (p == own) jo = j;
    if (p == d) jd = j;
  }
  if (jo < 0 || n > cap || (jd < 0 && n == cap && lds(&I.ep_cnt[s + jo]) > 1)) {
    dev_fail(I.status, kDevErrInvalid);
    return;
  }
  const int sv = vol ? __ldg(&I.src[e]) : -1;
  const int sp = (vol && sv != v) ? lds(&I.part_vec[sv]) : d;
  if (vol && sv == v) atomicAdd(&vol->send[own], -(n - 1));
  // Counts change atomically: movers committed in the same round may share a net
  // on which they only shift counts (their part sets are disjoint there).
  const int co = atomicAdd(&I.ep_cnt[s + jo], -1) - 1;
  if (co == 0) {
    const int last = n - 1;
    I.ep_part[s + jo] = lds(&I.ep_part[s + last]);
    I.ep_cnt[s + jo] = lds(&I.ep_cnt[s + last]);
    I.ep_part[s + last] = -1;
    I.ep_cnt[s + last] = 0;
    if (jd == last) jd = jo;
    n = last;
    if (vol && sv != v) {
      atomicAdd(&vol->send[sp], -1);
      if (vol->recv) atomicAdd(&vol->recv[own], -1);
    }
  } else {
    if (vol && vol->recv && sv == v) atomicAdd(&vol->recv[own], 1);
  }
  if (vol && sv == v) atomicAdd(&vol->send[d], n - 1);
  if (jd >= 0) {
    atomicAdd(&I.ep_cnt[s + jd], 1);
    if (vol && vol->recv && sv == v) atomicAdd(&vol->recv[d], -1);
  } else {
    I.ep_part[s + n] = d;
    I.ep_cnt[s + n] = 1;
    n++;
    if (vol) {
      atomicAdd(&vol->send[sp], 1);
      if (vol->recv && sv != v) atomicAdd(&vol->recv[d], 1);
    }
  }
  I.ep_len[e] = n;
}

// One warp applies v's move own -> d to the list of net e (REMOVAL then ADDING,
// as commit_net, without volumes); the lanes search the slots of own and d
// together.  The net must have no other mover at the same time.  Returns the
// list length after the move (every lane).
__device__ __forceinline__ int commit_net_warp(const DevInstance& I, int own, int d, int e) {
  const int lane = threadIdx.x & 31;
  const int s = (int)__ldg(&I.nptr[e]);
  const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
  int n = lds(&I.ep_len[e]);
  int jo = -1, jd = -1;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    const int p = j < n ? lds(&I.ep_part[s + j]) : -1;
    const unsigned mo = __ballot_sync(kAll, p == own);
    const unsigned md = __ballot_sync(kAll, p == d);
    if (mo && jo < 0) jo = j0 + __ffs(mo) - 1;
    if (md && jd < 0) jd = j0 + __ffs(md) - 1;
  }
  const int co = jo >= 0 ? lds(&I.ep_cnt[s + jo]) : 0;
  if (jo < 0 || n > cap || (jd < 0 && n == cap && co > 1)) {
    if (lane == 0) dev_fail(I.status, kDevErrInvalid);
    return n;
  }
  if (lane == 0) {
    if (co == 1) {
      const int last = n - 1;
      I.ep_part[s + jo] = lds(&I.ep_part[s + last]);
      I.ep_cnt[s + jo] = lds(&I.ep_cnt[s + last]);
      I.ep_part[s + last] = -1;
      I.ep_cnt[s + last] = 0;
      if (jd == last) jd = jo;
      n = last;
    } else {
      I.ep_cnt[s + jo] = co - 1;
    }
    if (jd >= 0) {
      I.ep_cnt[s + jd] = lds(&I.ep_cnt[s + jd]) + 1;
    } else {
      I.ep_part[s + n] = d;
      I.ep_cnt[s + n] = 1;
      n++;
    }
    I.ep_len[e] = n;
  }
  n = __shfl_sync(kAll, n, 0);
  __syncwarp();
  return n;
}

// Least-loaded part (lowest index on ties) and the second smallest size, for
// the LDG fallback (TV/partition.cpp:118-132) and its drift margin.
__device__ __forceinline__ void block_min_part(const int* sizes, int K, unsigned long long* scr, int* minpart,
                                               int* minsize, int* second) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned long long mk = ~0ull;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    const unsigned long long key = ((unsigned long long)((unsigned)sizes[p] ^ 0x80000000u) << 32) | (unsigned)p;
    mk = key < mk ? key : mk;
  }
  for (int off = 16; off; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(kAll, mk, off);
    mk = o < mk ? o : mk;
  }
  __syncthreads();
  if (lane == 0) scr[wib] = mk;
  __syncthreads();
  mk = scr[0];
  for (int x = 1; x < (int)(blockDim.x >> 5); x++) mk = scr[x] < mk ? scr[x] : mk;
  const int mp = (int)(mk & 0xffffffffu);
  int s2 = 0x7fffffff;
  for (int p = threadIdx.x; p < K; p += blockDim.x)
    if (p != mp) s2 = min(s2, sizes[p]);
  s2 = warp_min(s2);
  __syncthreads();
  if (lane == 0) scr[wib] = (unsigned long long)(unsigned)s2;
  __syncthreads();
  int m2 = 0x7fffffff;
  for (int x = 0; x < (int)(blockDim.x >> 5); x++) m2 = min(m2, (int)(unsigned)scr[x]);
  __syncthreads();
  *minpart = mp;
  *minsize = sizes[mp];
  *second = m2;
}

}  // namespace spec
}  // namespace fp
