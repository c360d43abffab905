// Refinement kernels: one persistent CTA per instance that walks the reference's
// visiting order exactly (every decision reads the state left by all earlier
// moves, as the sequential CPU refinement does) and spreads the work of each
// vertex over the CTA: warps scan the vertex's nets, the part tables live in
// shared memory, and the argmax runs as a block reduction with the reference's
// tie-break.  Results are bit-identical to the reference's partition().
//
//   TV   : TV/partition.cpp:307-440      CN  : CN/partition.cpp:245-377
//   TM   : TM/partition.cpp:300-593      MSM : MSM/partition.cpp:347-656
//   MSV  : MGV/partition.cpp:222-477     MSRV: MSRV/partition.cpp:240-517

#include "fp_device.cuh"

namespace fp {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_id() { return threadIdx.x >> 5; }

// Dynamic shared memory carving (8-byte aligned chunks).
struct Carve {
  unsigned char* p;
  template <class T>
  __device__ T* take(int n) {
    T* r = reinterpret_cast<T*>(p);
    size_t bytes = ((size_t)n * sizeof(T) + 15) & ~size_t(15);
    p += bytes;
    return r;
  }
};

// Scan of the nets of vertex v: for every part the number of v's nets that list
// it (cnt) and the (net index, slot) where v first sees it (first); c1 counts
// the nets in which v is the only pin of its own part.
__device__ void scan_parts(const DevInstance& I, int own, uint32_t base, int deg, int* cnt,
                           unsigned long long* first, int* c1) {
  const int lane = lane_id();
  int local_c1 = 0;
  for (int i = warp_id(); i < deg; i += kWarps) {
    const int e = (int)I.vnets[base + i];
    const int s = (int)I.nptr[e];
    const int cap = (int)I.nptr[e + 1] - s;
    int n = I.ep_len[e];
    if (n > cap) { dev_fail(I.status, kDevErrInvalid); n = cap; }
    for (int j = lane; j < n; j += 32) {
      const int p = I.ep_part[s + j];
      if ((unsigned)p >= (unsigned)I.K) { dev_fail(I.status, kDevErrInvalid); continue; }
      atomicAdd(&cnt[p], 1);
      atomicMin(&first[p], ((unsigned long long)i << 32) | (unsigned)j);
      if (c1 && p == own && I.ep_cnt[s + j] == 1) local_c1++;
    }
  }
  if (c1 && local_c1) atomicAdd(c1, local_c1);
}

// Volume bookkeeping applied while a vertex moves (MSV / MSRV); NULL for the
// other metrics.
struct VolHooks {
  int* send;
  int* recv;   // NULL for MSV
};

// Moves vertex v from part `own` to part `d` on every one of its nets: the
// reference's REMOVAL loop (decrement, swap-with-last when the count reaches
// zero) followed by its ADDING loop (increment or append), one warp per net.
// Volume hooks follow MGV/partition.cpp:376-449 and MSRV/partition.cpp:387-483.
__device__ void move_lists(const DevInstance& I, int v, int own, int d, uint32_t base, int deg,
                           const VolHooks* vh) {
  const int lane = lane_id();
  for (int i = warp_id(); i < deg; i += kWarps) {
    const int e = (int)I.vnets[base + i];
    const int s = (int)I.nptr[e];
    int n = I.ep_len[e];
    int jo = -1, jd = -1;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      const int p = j < n ? I.ep_part[s + j] : -1;
      const unsigned bo = __ballot_sync(kFull, p == own);
      const unsigned bd = __ballot_sync(kFull, p == d);
      if (bo && jo < 0) jo = j0 + __ffs(bo) - 1;
      if (bd && jd < 0) jd = j0 + __ffs(bd) - 1;
    }
    const int cap = (int)I.nptr[e + 1] - s;
    if (jo < 0 || n > cap || (jd < 0 && n == cap && I.ep_cnt[s + jo] > 1)) {
      // The list does not hold v's part, or has no free slot: the state is
      // inconsistent.  Report it and leave the net untouched.
      if (lane == 0) dev_fail(I.status, kDevErrInvalid);
      continue;
    }
    if (lane == 0) {
      const int sv = vh ? I.src[e] : -1;
      const int sp = (vh && sv != v) ? I.part_vec[sv] : d;
      if (vh && sv == v) atomicAdd(&vh->send[own], -(n - 1));
      {
        const int co = I.ep_cnt[s + jo] - 1;
        if (co == 0) {
          const int last = n - 1;
          I.ep_part[s + jo] = I.ep_part[s + last];
          I.ep_cnt[s + jo] = I.ep_cnt[s + last];
          I.ep_part[s + last] = -1;
          I.ep_cnt[s + last] = 0;
          if (jd == last) jd = jo;
          n = last;
          if (vh && sv != v) {
            atomicAdd(&vh->send[sp], -1);
            if (vh->recv) atomicAdd(&vh->recv[own], -1);
          }
        } else {
          I.ep_cnt[s + jo] = co;
          if (vh && vh->recv && sv == v) atomicAdd(&vh->recv[own], 1);
        }
      }
      if (vh && sv == v) atomicAdd(&vh->send[d], n - 1);
      if (jd >= 0) {
        I.ep_cnt[s + jd] += 1;
        if (vh && vh->recv && sv == v) atomicAdd(&vh->recv[d], -1);
      } else {
        I.ep_part[s + n] = d;
        I.ep_cnt[s + n] = 1;
        n++;
        if (vh) {
          atomicAdd(&vh->send[sp], 1);
          if (vh->recv && sv != v) atomicAdd(&vh->recv[d], 1);
        }
      }
      I.ep_len[e] = n;
    }
  }
}

__device__ __forceinline__ void zero_ints(int* a, int n, int val) {
  for (int p = threadIdx.x; p < n; p += blockDim.x) a[p] = val;
}
__device__ __forceinline__ void zero_u64(unsigned long long* a, int n, unsigned long long val) {
  for (int p = threadIdx.x; p < n; p += blockDim.x) a[p] = val;
}

__device__ __forceinline__ int block_max_int(int x, unsigned long long* scratch) {
  // max via min of the complemented, sign-biased value
  unsigned long long key = (unsigned long long)(~((unsigned)x ^ 0x80000000u));
  key = block_min_u64(key, scratch);
  return (int)((~(unsigned)key) ^ 0x80000000u);
}

// ------------------------------------------------------------------ TV

__global__ void __launch_bounds__(kThreads, 1) refine_tv_kernel(DevInstance I, int passes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ LdgKey kscr[kWarps];
  __shared__ unsigned long long uscr[kWarps];
  __shared__ int c1_s, moves_s;
  const int K = I.K;
  Carve cv{smem_raw};
  int* sizes = cv.take<int>(K);
  int* marker = cv.take<int>(K);
  int* cnt = cv.take<int>(K);
  unsigned long long* first = cv.take<unsigned long long>(K);
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    sizes[p] = I.part_sizes[p];
    marker[p] = I.marker[p];
  }
  __syncthreads();
  for (int it = 0; it < passes; it++) {
    if (threadIdx.x == 0) moves_s = 0;
    for (int z = 0; z < I.nov; z++) {
      const int v = I.order[z];
      const int own = I.part_vec[v];
      const uint32_t base = I.vptr[v];
      const int deg = (int)(I.vptr[v + 1] - base);
      zero_ints(cnt, K, 0);
      zero_u64(first, K, ~0ull);
      if (threadIdx.x == 0) c1_s = 0;
      __syncthreads();
      scan_parts(I, own, base, deg, cnt, first, &c1_s);
      __syncthreads();
      // Active parts are those seen in this scan whose marker was not already v
      // (the reference's marker array persists across passes, so a part whose
      // last scan was v's own previous visit does not become active).
      LdgKey best{-1.0, 0, -1, ~0ull};
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const int c = cnt[p];
        if (c > 0) {
          const bool stale = marker[p] == v;
          marker[p] = v;
          if (!stale) {
            LdgKey k{ldg_score(c - (p == own ? 1 : 0), sizes[p], I.C), sizes[p], p, first[p]};
            if (ldg_better(k, best)) best = k;
          }
        }
      }
      best = block_ldg_argmax(best, kscr);
      int d = best.part;
      if (d < 0) d = block_min_loaded(sizes, K, uscr);
      if (sizes[d] > I.max_pw) d = own;
      if (sizes[d] < I.min_pw) d = own;
      bool accept = false;
      if (d != own) accept = c1_s >= deg - cnt[d];
      __syncthreads();
      if (accept) {
        if (threadIdx.x == 0) {
          I.part_vec[v] = d;
          sizes[own] -= I.w[v];
          sizes[d] += I.w[v];
          moves_s++;
        }
        move_lists(I, v, own, d, base, deg, nullptr);
        __syncthreads();
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) I.moves[it] = moves_s;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    I.part_sizes[p] = sizes[p];
    I.marker[p] = marker[p];
  }
}

// ------------------------------------------------------------------ MSV / MSRV

__global__ void __launch_bounds__(kThreads, 1) refine_vol_kernel(DevInstance I, int passes, int rv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ LdgKey kscr[kWarps];
  __shared__ unsigned long long uscr[kWarps];
  __shared__ int moves_s, maxv_s, cc_s, count_s;
  __shared__ VolHooks vh;
  const int K = I.K;
  Carve cv{smem_raw};
  int* sizes = cv.take<int>(K);
  int* cnt = cv.take<int>(K);
  unsigned long long* first = cv.take<unsigned long long>(K);
  int* gains = cv.take<int>(K);
  int* losses = cv.take<int>(K);
  int* send = cv.take<int>(K);
  int* recv = cv.take<int>(K);
  int* mark = cv.take<int>(K);
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    sizes[p] = I.part_sizes[p];
    send[p] = I.send[p];
    recv[p] = rv ? I.recv[p] : 0;
  }
  if (threadIdx.x == 0) {
    vh.send = send;
    vh.recv = rv ? recv : nullptr;
  }
  __syncthreads();
  for (int it = 0; it < passes; it++) {
    // Max-volume parts at the start of the pass (MGV/partition.cpp:211-234).
    {
      int mx = -2147483647 - 1;
      for (int p = threadIdx.x; p < K; p += blockDim.x) mx = max(mx, send[p] + recv[p]);
      mx = block_max_int(mx, uscr);
      int local = 0;
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const bool is_max = send[p] + recv[p] == mx;
        mark[p] = is_max ? 1 : -1;
        local += is_max;
      }
      if (threadIdx.x == 0) { maxv_s = mx; cc_s = 1; count_s = 0; moves_s = 0; }
      __syncthreads();
      if (local) atomicAdd(&count_s, local);
      __syncthreads();
    }
    for (int z = 0; z < I.nov; z++) {
      const int v = I.order[z];
      const int own = I.part_vec[v];
      const uint32_t base = I.vptr[v];
      const int deg = (int)(I.vptr[v + 1] - base);
      zero_ints(cnt, K, 0);
      zero_u64(first, K, ~0ull);
      zero_ints(gains, K, 0);
      zero_ints(losses, K, 0);
      __syncthreads();
      scan_parts(I, own, base, deg, cnt, first, nullptr);
      __syncthreads();
      // The marker array is reset every pass, so every part seen is active.
      LdgKey best{-1.0, 0, -1, ~0ull};
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const int c = cnt[p];
        if (c > 0) {
          LdgKey k{ldg_score(c - (p == own ? 1 : 0), sizes[p], I.C), sizes[p], p, first[p]};
          if (ldg_better(k, best)) best = k;
        }
      }
      best = block_ldg_argmax(best, kscr);
      int d = best.part;
      if (d < 0) d = block_min_loaded(sizes, K, uscr);
      if (d == own) continue;  // uniform across the block
      // Gains and losses per part (MGV/partition.cpp:294-337, MSRV/partition.cpp:303-350).
      {
        const int lane = lane_id();
        for (int i = warp_id(); i < deg; i += kWarps) {
          const int e = (int)I.vnets[base + i];
          const int s = (int)I.nptr[e];
          const int n = I.ep_len[e];
          bool oc1 = false, fd = false;
          for (int j = lane; j < n; j += 32) {
            const int p = I.ep_part[s + j];
            if (p == own && I.ep_cnt[s + j] == 1) oc1 = true;
            if (p == d) fd = true;
          }
          oc1 = __any_sync(kFull, oc1);
          fd = __any_sync(kFull, fd);
          if (lane == 0) {
            const int sv = I.src[e];
            const int sp = I.part_vec[sv];
            if (sv == v) {
              atomicAdd(&gains[own], n - 1);
              atomicAdd(&losses[d], n - 1);
            }
            if (oc1) {
              if (sv != v) {
                atomicAdd(&gains[sp], 1);
                if (rv) atomicAdd(&gains[own], 1);
              } else {
                atomicAdd(&losses[d], -1);
              }
            }
            if (!fd) {
              if (sv != v) {
                atomicAdd(&losses[sp], 1);
                if (rv) atomicAdd(&losses[d], 1);
              } else {
                atomicAdd(&losses[d], 1);
              }
            }
          }
        }
      }
      __syncthreads();
      const int mx = maxv_s, cc = cc_s;
      bool bad = false;
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const int g = gains[p], l = losses[p];
        if (mark[p] == cc) bad |= rv ? (g <= l) : (g < l);
        else bad |= (send[p] + recv[p] + (l - g) >= mx);
      }
      bad = __syncthreads_or(bad);
      if (bad) continue;
      if (threadIdx.x == 0) {
        I.part_vec[v] = d;
        sizes[own] -= I.w[v];
        sizes[d] += I.w[v];
        moves_s++;
      }
      __syncthreads();
      move_lists(I, v, own, d, base, deg, &vh);
      __syncthreads();
      if (!rv) {
        // MSV recomputes the max parts after every move (MGV/partition.cpp:453-472).
        int m2 = -2147483647 - 1;
        for (int p = threadIdx.x; p < K; p += blockDim.x) m2 = max(m2, send[p]);
        m2 = block_max_int(m2, uscr);
        for (int p = threadIdx.x; p < K; p += blockDim.x) mark[p] = send[p] == m2 ? 1 : -1;
        if (threadIdx.x == 0) { maxv_s = m2; cc_s = 1; }
        __syncthreads();
      } else {
        // MSRV rescans only when an old max part changed, against the old maximum,
        // without resetting the list (MSRV/partition.cpp:486-513).
        bool changed = false;
        for (int p = threadIdx.x; p < K; p += blockDim.x)
          if (mark[p] == cc && send[p] + recv[p] != mx) changed = true;
        changed = __syncthreads_or(changed);
        if (changed) {
          int m2 = -2147483647 - 1;
          for (int p = threadIdx.x; p < K; p += blockDim.x) m2 = max(m2, send[p] + recv[p]);
          m2 = block_max_int(m2, uscr);
          if (m2 >= mx) {
            const int ncc = m2 > mx ? cc + 1 : cc;
            int local = 0;
            for (int p = threadIdx.x; p < K; p += blockDim.x)
              if (send[p] + recv[p] == m2) { mark[p] = ncc; local++; }
            __syncthreads();
            if (threadIdx.x == 0) {
              if (m2 > mx) count_s = 0;
              maxv_s = m2;
              cc_s = ncc;
            }
            __syncthreads();
            if (local) atomicAdd(&count_s, local);
            __syncthreads();
            if (threadIdx.x == 0 && count_s > K) dev_fail(I.status, kDevErrUnsupported);
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) I.moves[it] = moves_s;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    I.part_sizes[p] = sizes[p];
    I.send[p] = send[p];
    if (rv) I.recv[p] = recv[p];
  }
}

// ------------------------------------------------------------------ TM / MSM

// conn[a][b] += delta with the message count and the zero masks kept exact.
// The number of 0->1 minus 1->0 crossings of a +-1 walk equals the change of
// [value >= 1], and the parity of zero crossings the change of [value == 0],
// so per-operation updates are exact whatever the order of the operations.
__device__ __forceinline__ void conn_add(const DevInstance& I, int* msgs, int a, int b, int delta) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const int old = atomicAdd(&I.conn[(size_t)a * K + b], delta);
  const int now = old + delta;
  if (delta > 0 && old == 0) atomicAdd(&msgs[a], 1);
  if (delta < 0 && old == 1) atomicAdd(&msgs[a], -1);
  if ((old == 0) != (now == 0)) {
    atomicXor(&I.zrow[(size_t)a * words + (b >> 5)], 1u << (b & 31));
    atomicXor(&I.zcol[(size_t)b * words + (a >> 5)], 1u << (a & 31));
  }
  if ((old == 1) != (now == 1)) {   // same parity argument for [value == 1]
    atomicXor(&I.c1row[(size_t)a * words + (b >> 5)], 1u << (b & 31));
    atomicXor(&I.c1col[(size_t)b * words + (a >> 5)], 1u << (a & 31));
  }
}

__global__ void __launch_bounds__(kThreads, 1) refine_msg_kernel(DevInstance I, int passes, int msm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long uscr[kWarps];
  __shared__ int moves_s, gain_s, has_gain_s, maxv_s, nmax_s, nsnd_s;
  const int K = I.K;
  const int words = (K + 31) >> 5;
  Carve cv{smem_raw};
  int* sizes = cv.take<int>(K);
  int* msgs = cv.take<int>(K);
  int* gains = cv.take<int>(K);         // MSM: per-part gains
  unsigned long long* fsnd = cv.take<unsigned long long>(K);  // first non-source net per sender part
  uint32_t* R = cv.take<uint32_t>(words);   // receiver parts
  uint32_t* S = cv.take<uint32_t>(words);   // sender parts
  int* maxlist = cv.take<int>(K);
  int* sndlist = cv.take<int>(K);
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    sizes[p] = I.part_sizes[p];
    msgs[p] = I.msgs[p];
  }
  __syncthreads();
  const int lane = lane_id();
  for (int it = 0; it < passes; it++) {
    if (threadIdx.x == 0) moves_s = 0;
    for (int v = 0; v < I.nov; v++) {
      const int own = I.part_vec[v];
      const uint32_t base = I.vptr[v];
      const int deg = (int)(I.vptr[v + 1] - base);
      zero_u64(fsnd, K, ~0ull);
      if (msm) zero_ints(gains, K, 0);
      for (int x = threadIdx.x; x < words; x += blockDim.x) { R[x] = 0; S[x] = 0; }
      if (threadIdx.x == 0) { gain_s = 0; has_gain_s = 0; }
      __syncthreads();
      // Receivers, senders and the source-side gain (TM/partition.cpp:320-393).
      int g_local = 0;
      for (int i = warp_id(); i < deg; i += kWarps) {
        const int e = (int)I.vnets[base + i];
        const int s = (int)I.nptr[e];
        const int n = I.ep_len[e];
        const int sv = I.src[e];
        if (sv == v) {
          for (int j = lane; j < n; j += 32) {
            const int t = I.ep_part[s + j];
            if ((unsigned)t >= (unsigned)K) { dev_fail(I.status, kDevErrInvalid); continue; }
            if (t == own) {
              if (I.ep_cnt[s + j] > 1) atomicOr(&R[own >> 5], 1u << (own & 31));
            } else {
              atomicOr(&R[t >> 5], 1u << (t & 31));
              // gain_loss_2d[own][t] is 1 at this point (raised once per listed
              // part, lowered after each net), so the test is conn == 1.
              if (I.conn[(size_t)own * K + t] == 1) g_local++;
            }
          }
        } else {
          const int ps = I.part_vec[sv];
          bool oc1 = false;
          for (int j = lane; j < n; j += 32)
            if (I.ep_part[s + j] == own && I.ep_cnt[s + j] == 1) oc1 = true;
          oc1 = __any_sync(kFull, oc1);
          if (lane == 0) {
            atomicOr(&S[ps >> 5], 1u << (ps & 31));
            atomicMin(&fsnd[ps], ((unsigned long long)i << 1) | (oc1 ? 1ull : 0ull));
          }
        }
      }
      if (g_local) {
        if (msm) atomicAdd(&gains[own], g_local);
        else atomicAdd(&gain_s, g_local);
        atomicOr(&has_gain_s, 1);
      }
      __syncthreads();
      // Sender-side gain: only the first net of each sender part is tested.
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const unsigned long long f = fsnd[p];
        if (f != ~0ull && (f & 1ull) && I.conn[(size_t)p * K + own] == 1) {
          if (msm) atomicAdd(&gains[p], 1);
          else atomicAdd(&gain_s, 1);
          atomicOr(&has_gain_s, 1);
        }
      }
      __syncthreads();
      int bestk = -1;
      if (!msm) {
        const int gain = gain_s;
        if (gain > 0) {
          // best = first k with the largest gain - loss > 0 among parts below
          // capacity (TM/partition.cpp:408-450).
          unsigned long long key = ~0ull;
          for (int k = threadIdx.x; k < K; k += blockDim.x) {
            if (k == own || !((double)sizes[k] < I.C)) continue;
            int loss = 0;
            const uint32_t* zr = I.zrow + (size_t)k * words;
            const uint32_t* zc = I.zcol + (size_t)k * words;
            for (int x = 0; x < words; x++) {
              uint32_t self = (x == (k >> 5)) ? ~(1u << (k & 31)) : ~0u;
              loss += __popc(R[x] & zr[x] & self) + __popc(S[x] & zc[x] & self);
            }
            const int imp = gain - loss;
            if (imp > 0) {
              const unsigned long long kk = ((unsigned long long)(0x7fffffff - imp) << 32) | (unsigned)k;
              key = kk < key ? kk : key;
            }
          }
          key = block_min_u64(key, uscr);
          if (key != ~0ull) bestk = (int)(key & 0xffffffffu);
        }
      } else if (has_gain_s) {
        // MSM (MSM/partition.cpp:360-520): the max-message parts must all gain
        // more than they lose, no other part may reach the max, best total
        // improvement wins, first k on ties.
        int mx = -2147483647 - 1;
        for (int p = threadIdx.x; p < K; p += blockDim.x) mx = max(mx, msgs[p]);
        mx = block_max_int(mx, uscr);
        if (threadIdx.x == 0) { maxv_s = mx; nmax_s = 0; nsnd_s = 0; }
        __syncthreads();
        bool zero_gain_max = false;
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
          if (msgs[p] == mx) {
            maxlist[atomicAdd(&nmax_s, 1)] = p;
            if (gains[p] <= 0) zero_gain_max = true;
          } else if ((S[p >> 5] >> (p & 31)) & 1u) {
            sndlist[atomicAdd(&nsnd_s, 1)] = p;
          }
        }
        zero_gain_max = __syncthreads_or(zero_gain_max);
        if (!zero_gain_max) {
          const int nmax = nmax_s, nsnd = nsnd_s;
          unsigned long long key = ~0ull;
          for (int k = threadIdx.x; k < K; k += blockDim.x) {
            if (k == own) continue;
            const uint32_t* zr = I.zrow + (size_t)k * words;
            int Lk = 0;
            for (int x = 0; x < words; x++) Lk += __popc(R[x] & zr[x]);
            bool good = true;
            int imp = 0;
            bool k_is_max = false;
            for (int q = 0; q < nmax && good; q++) {
              const int m = maxlist[q];
              int l = (m == k) ? Lk : 0;
              if (m == k) k_is_max = true;
              if ((S[m >> 5] >> (m & 31)) & 1u)
                l += (I.zrow[(size_t)m * words + (k >> 5)] >> (k & 31)) & 1u;
              if (gains[m] <= l) good = false;
              imp += gains[m] - l;
            }
            bool k_is_snd = false;
            for (int q = 0; q < nsnd && good; q++) {
              const int sp = sndlist[q];
              int l = (int)((I.zrow[(size_t)sp * words + (k >> 5)] >> (k & 31)) & 1u);
              if (sp == k) { l += Lk; k_is_snd = true; }
              if (msgs[sp] + (l - gains[sp]) >= mx) good = false;
            }
            if (good && !k_is_max && !k_is_snd) {
              if (msgs[k] + (Lk - gains[k]) >= mx) good = false;
            }
            if (good) {
              const unsigned long long kk = ((unsigned long long)(0x7fffffff - imp) << 32) | (unsigned)k;
              key = kk < key ? kk : key;
            }
          }
          key = block_min_u64(key, uscr);
          if (key != ~0ull) bestk = (int)(key & 0xffffffffu);
        }
      }
      __syncthreads();
      if (bestk < 0) continue;
      const int d = bestk;
      if (threadIdx.x == 0) {
        I.part_vec[v] = d;
        sizes[own] -= I.w[v];
        sizes[d] += I.w[v];
        moves_s++;
      }
      __syncthreads();
      move_lists(I, v, own, d, base, deg, nullptr);
      __syncthreads();
      // Connection updates on the final lists (TM/partition.cpp:519-587).
      for (int i = warp_id(); i < deg; i += kWarps) {
        const int e = (int)I.vnets[base + i];
        const int s = (int)I.nptr[e];
        const int n = I.ep_len[e];
        const int sv = I.src[e];
        if (sv == v) {
          for (int j = lane; j < n; j += 32) {
            const int t = I.ep_part[s + j];
            if (t != d) conn_add(I, msgs, d, t, 1);
            if (t != own && t != d) conn_add(I, msgs, own, t, -1);
            if (t == d && I.ep_cnt[s + j] > 1) conn_add(I, msgs, own, t, -1);
          }
        } else {
          const int sn = I.part_vec[sv];
          bool dc1 = false, fo = false;
          for (int j = lane; j < n; j += 32) {
            const int t = I.ep_part[s + j];
            if (t == d && I.ep_cnt[s + j] == 1) dc1 = true;
            if (t == own) fo = true;
          }
          dc1 = __any_sync(kFull, dc1);
          fo = __any_sync(kFull, fo);
          if (lane == 0) {
            if (dc1) conn_add(I, msgs, sn, d, 1);
            if (!fo) conn_add(I, msgs, sn, own, -1);
          }
        }
      }
      __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x == 0) I.moves[it] = moves_s;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    I.part_sizes[p] = sizes[p];
    I.msgs[p] = msgs[p];
  }
}

// ------------------------------------------------------------------ CN

__global__ void __launch_bounds__(kThreads, 1) refine_cn_kernel(DevInstance I, int passes) {
  __shared__ unsigned long long uscr[kWarps];
  __shared__ int moves_s, nold_s;
  __shared__ int oldpins[kThreads];
  const int lane = lane_id();
  for (int it = 0; it < passes; it++) {
    if (threadIdx.x == 0) moves_s = 0;
    __syncthreads();
    for (int e0 = 0; e0 < I.noe; e0 += kThreads) {
      const int e1 = min(e0 + kThreads, I.noe);
      int from = e0;
      while (true) {
        // Next net with exactly two parts, scanning in id order.
        const int e = from + (int)threadIdx.x;
        unsigned long long key = ~0ull;
        if (e < e1 && I.ep_len[e] == 2) key = (unsigned long long)e;
        key = block_min_u64(key, uscr);
        if (key == ~0ull) break;
        const int net = (int)key;
        from = net + 1;
        const int s = (int)I.nptr[net];
        const int p1 = I.ep_part[s], c1 = I.ep_cnt[s];
        const int p2 = I.ep_part[s + 1], c2 = I.ep_cnt[s + 1];
        const int oldp = c1 < c2 ? p1 : p2;
        const int newp = c1 < c2 ? p2 : p1;
        const int pb = (int)I.nptr[net], pe = (int)I.nptr[net + 1];
        // Does any pin on the smaller side touch an uncut net (CN/partition.cpp:291-309)?
        bool cut = false;
        for (int k = pb + warp_id(); k < pe; k += kWarps) {
          const int u = (int)I.npins[k];
          if (I.part_vec[u] != oldp) continue;
          for (uint32_t j = I.vptr[u] + lane; j < I.vptr[u + 1]; j += 32)
            if (I.ep_len[I.vnets[j]] == 1) cut = true;
        }
        cut = __syncthreads_or(cut);
        if (cut) continue;
        // Move the smaller side's pins to the other part, in net pin order.
        for (int k0 = pb; k0 < pe; k0 += kThreads) {
          const int k = k0 + (int)threadIdx.x;
          const bool is_old = k < pe && I.part_vec[I.npins[k]] == oldp;
          if (threadIdx.x == 0) nold_s = 0;
          __syncthreads();
          // ordered compaction of this chunk
          const unsigned b = __ballot_sync(kFull, is_old);
          __shared__ int wcount[kWarps];
          if (lane == 0) wcount[warp_id()] = __popc(b);
          __syncthreads();
          if (is_old) {
            int off = 0;
            for (int w2 = 0; w2 < warp_id(); w2++) off += wcount[w2];
            off += __popc(b & ((1u << lane) - 1u));
            oldpins[off] = (int)I.npins[k];
          }
          if (threadIdx.x == 0) {
            int t = 0;
            for (int w2 = 0; w2 < kWarps; w2++) t += wcount[w2];
            nold_s = t;
          }
          __syncthreads();
          const int nold = nold_s;
          for (int q = 0; q < nold; q++) {
            const int u = oldpins[q];
            const uint32_t ub = I.vptr[u];
            const int udeg = (int)(I.vptr[u + 1] - ub);
            if (threadIdx.x == 0) {
              I.part_vec[u] = newp;
              I.part_sizes[oldp] -= I.w[u];
              I.part_sizes[newp] += I.w[u];
              moves_s++;
            }
            move_lists(I, u, oldp, newp, ub, udeg, nullptr);
            __syncthreads();
          }
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) I.moves[it] = moves_s;
  }
}

}  // namespace

size_t refine_smem_bytes(int metric, int K) {
  auto a = [](size_t n) { return (n + 15) & ~size_t(15); };
  const size_t ki = a(sizeof(int) * (size_t)K), ku = a(sizeof(unsigned long long) * (size_t)K);
  const size_t kw = a(sizeof(uint32_t) * (size_t)((K + 31) / 32));
  switch (metric) {
    case 1: return 3 * ki + ku;                  // TV
    case 4: case 5: return 7 * ki + ku;          // MSV, MSRV
    case 2: case 3: return 5 * ki + ku + 2 * kw; // TM, MSM
    default: return 0;                           // CN
  }
}

cudaError_t launch_refine(const DevInstance& I, int passes, cudaStream_t st) {
  const size_t smem = refine_smem_bytes(I.metric, I.K);
  cudaError_t err = cudaSuccess;
  switch (I.metric) {
    case 1:
      err = cudaFuncSetAttribute(refine_tv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err == cudaSuccess) refine_tv_kernel<<<1, kThreads, smem, st>>>(I, passes);
      break;
    case 4:
    case 5:
      err = cudaFuncSetAttribute(refine_vol_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err == cudaSuccess) refine_vol_kernel<<<1, kThreads, smem, st>>>(I, passes, I.metric == 5);
      break;
    case 2:
    case 3:
      err = cudaFuncSetAttribute(refine_msg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err == cudaSuccess) refine_msg_kernel<<<1, kThreads, smem, st>>>(I, passes, I.metric == 3);
      break;
    case 0:
      refine_cn_kernel<<<1, kThreads, 0, st>>>(I, passes);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  if (err != cudaSuccess) return err;
  return cudaGetLastError();
}

}  // namespace fp
