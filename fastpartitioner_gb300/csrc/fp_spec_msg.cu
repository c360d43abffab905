// Speculative grid-wide refinement for the message metrics: TM
// (TM/partition.cpp:300-593) and MSM (MSM/partition.cpp:347-656).  Both walk the
// vertices in id order.
//
// Moves are rare for these metrics, so a round is simple: every warp of the
// grid evaluates a window of vertices against the current state (gain from the
// K x K connection counts, loss per candidate part from the zero masks of that
// matrix); the first mover ends the window, all vertices before it are
// non-movers decided on exactly the sequential state, and the mover's move --
// lists, connection counts, message counts, zero masks -- is applied by warps
// of the whole grid.  Vertices with more than 256 nets get a round of
// their own in which the whole grid computes their gain sets.

#include "fp_spec_common.cuh"

namespace fp {

namespace {

using namespace spec;

constexpr int kBig = 1000000000;

// conn[a][b] += delta with the message count and the zero masks kept exact
// (0->1 minus 1->0 crossings of a +-1 walk give the change of [value >= 1], and
// the parity of zero crossings the change of [value == 0], whatever the order).
__device__ __forceinline__ void conn_add_g(const DevInstance& I, int a, int b, int delta) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const int old = atomicAdd(&I.conn[(size_t)a * K + b], delta);
  const int now = old + delta;
  if (delta > 0 && old == 0) atomicAdd(&I.msgs[a], 1);
  if (delta < 0 && old == 1) atomicAdd(&I.msgs[a], -1);
  if ((old == 0) != (now == 0)) {
    atomicXor(&I.zrow[(size_t)a * words + (b >> 5)], 1u << (b & 31));
    atomicXor(&I.zcol[(size_t)b * words + (a >> 5)], 1u << (a & 31));
  }
}

// Per-warp scratch of one evaluation.
struct MsgWarp {
  uint32_t* R;               // receiver parts (bitmask)
  uint32_t* S;               // sender parts (bitmask)
  unsigned long long* fsnd;  // first non-source net per sender part: (net index << 1) | own-alone
  int* gains;                // MSM: gains per part
  int* maxl;                 // MSM: scratch lists
  int* sndl;
};

// Receivers, senders and the source-side gain over nets [nb, nb + 32) of v
// (TM/partition.cpp:320-393).  Returns this lane's source-side gain count.
__device__ int msg_batch(const DevInstance& I, int v, int own, uint32_t base, int nb, int deg, const MsgWarp& Wk,
                         unsigned* oc1mask) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  const int k = nb + lane;
  int s = 0, n = 0, sv = -1;
  if (k < deg) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    s = (int)__ldg(&I.nptr[e]);
    n = lds(&I.ep_len[e]);
    sv = __ldg(&I.src[e]);
  }
  if (lane == 0) *oc1mask = 0u;
  __syncwarp();
  int incl = n;
  for (int off = 1; off < 32; off <<= 1) {
    const int t = __shfl_up_sync(kAll, incl, off);
    if (lane >= off) incl += t;
  }
  const int total = __shfl_sync(kAll, incl, 31);
  int g = 0;
  for (int f0 = 0; f0 < total; f0 += 32) {
    const int f = f0 + lane;
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
    const int svl = __shfl_sync(kAll, sv, lo);
    if (f < total) {
      const int a = sl + f - (il - nl);
      const int t = lds(&I.ep_part[a]);
      if ((unsigned)t >= (unsigned)K) {
        dev_fail(I.status, kDevErrInvalid);
      } else if (svl == v) {
        if (t == own) {
          if (lds(&I.ep_cnt[a]) > 1) atomicOr(&Wk.R[own >> 5], 1u << (own & 31));
        } else {
          atomicOr(&Wk.R[t >> 5], 1u << (t & 31));
          // gain_loss_2d[own][t] is 1 here (raised once per listed part, lowered
          // after each net, TM/partition.cpp:347-369): the test is conn == 1.
          if (lds(&I.conn[(size_t)own * K + t]) == 1) g++;
        }
      } else if (t == own && lds(&I.ep_cnt[a]) == 1) {
        atomicOr(oc1mask, 1u << lo);
      }
    }
  }
  __syncwarp();
  if (k < deg && sv != v) {
    const int ps = lds(&I.part_vec[sv]);
    atomicOr(&Wk.S[ps >> 5], 1u << (ps & 31));
    atomicMin(&Wk.fsnd[ps], ((unsigned long long)k << 1) | ((*oc1mask >> lane) & 1u));
  }
  __syncwarp();
  return g;
}

// TM decision: first k below capacity with the largest gain - loss > 0
// (TM/partition.cpp:408-450).  One warp (lanes over k) or, with pstep =
// blockDim.x, one CTA (each thread returns its partial key).
__device__ unsigned long long tm_best_partial(const DevInstance& I, const int* sizes, const uint32_t* R,
                                              const uint32_t* S, int own, int gain, int k0, int kstep) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  unsigned long long key = ~0ull;
  for (int k = k0; k < K; k += kstep) {
    if (k == own || !((double)sizes[k] < I.C)) continue;
    const uint32_t* zr = I.zrow + (size_t)k * words;
    const uint32_t* zc = I.zcol + (size_t)k * words;
    int loss = 0;
    for (int x = 0; x < words; x++) {
      const uint32_t self = (x == (k >> 5)) ? ~(1u << (k & 31)) : ~0u;
      loss += __popc(R[x] & lds(&zr[x]) & self) + __popc(S[x] & lds(&zc[x]) & self);
    }
    const int imp = gain - loss;
    if (imp > 0) {
      const unsigned long long kk = ((unsigned long long)(0x7fffffff - imp) << 32) | (unsigned)k;
      key = kk < key ? kk : key;
    }
  }
  return key;
}

// MSM decision for candidate k (MSM/partition.cpp:460-520): every max-message
// part must gain more than it loses, no other part may reach the maximum; the
// total improvement over the max parts is returned (-1: not good).
__device__ int msm_eval_k(const DevInstance& I, const int* msgs, const int* gains, const uint32_t* R, const uint32_t* S,
                          const int* maxl, int nmax, const int* sndl, int nsnd, int mx, int k) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const uint32_t* zr = I.zrow + (size_t)k * words;
  int Lk = 0;
  for (int x = 0; x < words; x++) Lk += __popc(R[x] & lds(&zr[x]));
  int imp = 0;
  bool k_max = false;
  for (int q = 0; q < nmax; q++) {
    const int m = maxl[q];
    int l = m == k ? Lk : 0;
    if (m == k) k_max = true;
    if ((S[m >> 5] >> (m & 31)) & 1u) l += (lds(&I.zrow[(size_t)m * words + (k >> 5)]) >> (k & 31)) & 1u;
    if (gains[m] <= l) return -1;
    imp += gains[m] - l;
  }
  bool k_snd = false;
  for (int q = 0; q < nsnd; q++) {
    const int sp = sndl[q];
    int l = (int)((lds(&I.zrow[(size_t)sp * words + (k >> 5)]) >> (k & 31)) & 1u);
    if (sp == k) { l += Lk; k_snd = true; }
    if (msgs[sp] + (l - gains[sp]) >= mx) return -1;
  }
  if (!k_max && !k_snd && msgs[k] + (Lk - gains[k]) >= mx) return -1;
  return imp;
}

// Move of one net by one thread: lists (commit_net), then the connection
// updates on the net's final list (TM/partition.cpp:519-587).
__device__ void msg_commit_net(const DevInstance& I, int v, int own, int d, int e) {
  commit_net(I, v, own, d, e, nullptr);
  const int s = (int)__ldg(&I.nptr[e]);
  const int n = lds(&I.ep_len[e]);
  const int sv = __ldg(&I.src[e]);
  if (sv == v) {
    for (int j = 0; j < n; j++) {
      const int t = lds(&I.ep_part[s + j]);
      if (t != d) conn_add_g(I, d, t, 1);
      if (t != own && t != d) conn_add_g(I, own, t, -1);
      if (t == d && lds(&I.ep_cnt[s + j]) > 1) conn_add_g(I, own, t, -1);
    }
  } else {
    const int sn = lds(&I.part_vec[sv]);
    bool dc1 = false, fo = false;
    for (int j = 0; j < n; j++) {
      const int t = lds(&I.ep_part[s + j]);
      if (t == d && lds(&I.ep_cnt[s + j]) == 1) dc1 = true;
      if (t == own) fo = true;
    }
    if (dc1) conn_add_g(I, sn, d, 1);
    if (!fo) conn_add_g(I, sn, own, -1);
  }
}

__global__ void __launch_bounds__(kSThreads) spec_msg_kernel(DevInstance I, SpecBuf B, int passes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long uscr[kSWarps];
  __shared__ int iscr[kSWarps];
  __shared__ unsigned oc1m[kSWarps];
  __shared__ int s_mx, s_nmax, s_best;
  const bool msm = I.metric == 3;
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  Carve cv{smem_raw};
  int* sizes_s = cv.take<int>(K);
  int* msgs_s = cv.take<int>(K);
  int* maxl_s = cv.take<int>(K);                        // max-message parts (MSM)
  uint32_t* R_b = cv.take<uint32_t>((size_t)words * kSWarps);
  uint32_t* S_b = cv.take<uint32_t>((size_t)words * kSWarps);
  unsigned long long* fs_b = cv.take<unsigned long long>((size_t)K * kSWarps);
  int* gains_b = cv.take<int>((size_t)K * kSWarps);
  int* sndl_b = cv.take<int>((size_t)K * kSWarps);
  MsgWarp Wk{R_b + (size_t)wib * words, S_b + (size_t)wib * words, fs_b + (size_t)wib * K,
             gains_b + (size_t)wib * K, maxl_s, sndl_b + (size_t)wib * K};
  unsigned long long tA = gtimer();
  int heavy_round = 0;
  int round = 0;
  for (int it = 0; it < passes; it++) {
    int pos = 0;
    int W = min(nwarps, B.wmax);
    int hidx = 0;
    while (pos < I.nov) {
      // ------------------------------------------------------------ round state
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        sizes_s[p] = lds(&I.part_sizes[p]);
        msgs_s[p] = lds(&I.msgs[p]);
      }
      __syncthreads();
      if (msm) {
        // max-message parts, recomputed for every vertex by the reference
        // (MSM/partition.cpp:368-386); they change only with moves.
        int mx = -2147483647 - 1;
        for (int p = threadIdx.x; p < K; p += blockDim.x) mx = max(mx, msgs_s[p]);
        mx = warp_max(mx);
        if (lane == 0) iscr[wib] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
          int m = iscr[0];
          for (int x = 1; x < kSWarps; x++) m = max(m, iscr[x]);
          s_mx = m;
          int c = 0;
          for (int p = 0; p < K; p++)
            if (msgs_s[p] == m) maxl_s[c++] = p;
          s_nmax = c;
        }
        __syncthreads();
      }
      while (hidx < B.nheavy && __ldg(&B.heavy_pos[hidx]) < pos) hidx++;
      const int next_heavy = hidx < B.nheavy ? __ldg(&B.heavy_pos[hidx]) : I.nov;

      if (next_heavy == pos) {
        // ========================================================== heavy round
        const int hp = heavy_round & 1;
        int* hg = B.hgain + hp * K;            // MSM gains / TM: [0] gain
        uint32_t* hR = reinterpret_cast<uint32_t*>(B.hloss + hp * K);      // words <= K
        uint32_t* hS = reinterpret_cast<uint32_t*>(B.hadelta + hp * K);
        unsigned long long* hf = B.hfirst + hp * K;
        int* hmisc = B.hmisc + hp * 8;
        const int v = pos;
        const int own = lds(&I.part_vec[v]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        for (int x = lane; x < words; x += 32) { Wk.R[x] = 0; Wk.S[x] = 0; }
        for (int p = lane; p < K; p += 32) Wk.fsnd[p] = ~0ull;
        __syncwarp();
        int g = 0;
        for (int nb = gw * 32; nb < deg; nb += nwarps * 32) g += msg_batch(I, v, own, base, nb, deg, Wk, &oc1m[wib]);
        g = warp_sum(g);
        __syncthreads();
        for (int x = threadIdx.x; x < words; x += blockDim.x) {
          uint32_t r = 0, s = 0;
          for (int y = 0; y < kSWarps; y++) { r |= R_b[(size_t)y * words + x]; s |= S_b[(size_t)y * words + x]; }
          if (r) atomicOr(&hR[x], r);
          if (s) atomicOr(&hS[x], s);
        }
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
          unsigned long long f = ~0ull;
          for (int y = 0; y < kSWarps; y++) f = min(f, fs_b[(size_t)y * K + p]);
          if (f != ~0ull) atomicMin(&hf[p], f);
        }
        if (lane == 0 && g) atomicAdd(&hmisc[0], g);
        if (!grid_barrier(B.bar, I.status)) return;
        // every CTA: full sets, sender gains, decision
        uint32_t* R = R_b;   // warp 0's arrays hold the global sets
        uint32_t* S = S_b;
        for (int x = threadIdx.x; x < words; x += blockDim.x) { R[x] = lds(&hR[x]); S[x] = lds(&hS[x]); }
        int* gains = gains_b;
        for (int p = threadIdx.x; p < K; p += blockDim.x) gains[p] = 0;
        __syncthreads();
        int gsum = 0;
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
          const unsigned long long f = lds(&hf[p]);
          if (f != ~0ull && (f & 1ull) && lds(&I.conn[(size_t)p * K + own]) == 1) {
            if (msm) gains[p] += 1;
            else gsum++;
          }
        }
        gsum = warp_sum(gsum);
        if (lane == 0) iscr[wib] = gsum;
        __syncthreads();
        int gain_total = lds(&hmisc[0]);
        for (int x = 0; x < kSWarps; x++) gain_total += iscr[x];
        __syncthreads();
        int best = -1;
        if (!msm) {
          if (gain_total > 0) {
            unsigned long long key = tm_best_partial(I, sizes_s, R, S, own, gain_total, threadIdx.x, blockDim.x);
            key = block_min_u64(key, uscr);
            if (key != ~0ull) best = (int)(key & 0xffffffffu);
          }
        } else {
          if (threadIdx.x == 0) gains[own] += lds(&hmisc[0]);
          __syncthreads();
          bool has_gain = false;
          for (int p = threadIdx.x; p < K; p += blockDim.x) has_gain |= gains[p] > 0;
          has_gain = __syncthreads_or(has_gain);
          if (has_gain) {
            // sender parts that are not max parts
            __shared__ int s_nsnd;
            if (threadIdx.x == 0) {
              int c = 0;
              for (int p = 0; p < K; p++)
                if (((S[p >> 5] >> (p & 31)) & 1u) && msgs_s[p] != s_mx) sndl_b[c++] = p;
              s_nsnd = c;
            }
            __syncthreads();
            unsigned long long key = ~0ull;
            for (int k = threadIdx.x; k < K; k += blockDim.x) {
              if (k == own) continue;
              const int imp = msm_eval_k(I, msgs_s, gains, R, S, maxl_s, s_nmax, sndl_b, s_nsnd, s_mx, k);
              if (imp >= 0) {
                const unsigned long long kk = ((unsigned long long)(0x7fffffff - imp) << 32) | (unsigned)k;
                key = kk < key ? kk : key;
              }
            }
            key = block_min_u64(key, uscr);
            if (key != ~0ull) best = (int)(key & 0xffffffffu);
          }
        }
        if (!grid_barrier(B.bar, I.status)) return;
        if (best >= 0) {
          for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < deg; i += gridDim.x * blockDim.x)
            msg_commit_net(I, v, own, best, (int)__ldg(&I.vnets[base + i]));
          if (blockIdx.x == 0 && threadIdx.x == 0) {
            I.part_vec[v] = best;
            const int wv = __ldg(&I.w[v]);
            atomicAdd(&I.part_sizes[own], -wv);
            atomicAdd(&I.part_sizes[best], wv);
            atomicAdd((unsigned long long*)&I.moves[it], 1ull);
          }
        }
        {
          const int op = hp ^ 1;
          for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K; p += gridDim.x * blockDim.x) {
            B.hgain[op * K + p] = 0;
            B.hloss[op * K + p] = 0;
            B.hadelta[op * K + p] = 0;
            B.hfirst[op * K + p] = ~0ull;
          }
          if (blockIdx.x == 0 && threadIdx.x < 8) B.hmisc[op * 8 + threadIdx.x] = 0;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) B.ctl[(round & 1) ^ 1] = kNone;
        pos += 1;
        heavy_round++;
        round++;
        if (!grid_barrier(B.bar, I.status)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          B.stats[1]++;
          const unsigned long long tH = gtimer();
          B.stats[19] += tH - tA;
          tA = tH;
        }
        continue;
      }

      // ============================================================ light round
      const int end_w = min(min(pos + W, I.nov), next_heavy);
      const int par = round & 1;
      for (int v = pos + gw; v < end_w; v += nwarps) {
        const int own = lds(&I.part_vec[v]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        for (int x = lane; x < words; x += 32) { Wk.R[x] = 0; Wk.S[x] = 0; }
        for (int p = lane; p < K; p += 32) { Wk.fsnd[p] = ~0ull; Wk.gains[p] = 0; }
        __syncwarp();
        int g = 0;
        for (int nb = 0; nb < deg; nb += 32) g += msg_batch(I, v, own, base, nb, deg, Wk, &oc1m[wib]);
        g = warp_sum(g);
        int gs = 0;
        for (int p = lane; p < K; p += 32) {
          const unsigned long long f = Wk.fsnd[p];
          if (f != ~0ull && (f & 1ull) && lds(&I.conn[(size_t)p * K + own]) == 1) {
            if (msm) Wk.gains[p] += 1;
            else gs++;
          }
        }
        gs = warp_sum(gs);
        __syncwarp();
        int best = -1;
        if (!msm) {
          const int gain = g + gs;
          if (gain > 0) {
            unsigned long long key = tm_best_partial(I, sizes_s, Wk.R, Wk.S, own, gain, lane, 32);
            for (int off = 16; off; off >>= 1) {
              const unsigned long long o2 = __shfl_xor_sync(kAll, key, off);
              key = o2 < key ? o2 : key;
            }
            if (key != ~0ull) best = (int)(key & 0xffffffffu);
          }
        } else {
          if (lane == 0) Wk.gains[own] += g;
          __syncwarp();
          bool has_gain = false;
          bool zero_gain_max = false;
          for (int p = lane; p < K; p += 32) has_gain |= Wk.gains[p] > 0;
          for (int q = lane; q < s_nmax; q += 32) zero_gain_max |= Wk.gains[maxl_s[q]] <= 0;
          has_gain = __any_sync(kAll, has_gain);
          zero_gain_max = __any_sync(kAll, zero_gain_max);
          if (has_gain && !zero_gain_max) {
            int nsnd = 0;
            for (int p0 = 0; p0 < K; p0 += 32) {
              const int p = p0 + lane;
              const bool ok = p < K && ((Wk.S[p >> 5] >> (p & 31)) & 1u) && msgs_s[p] != s_mx;
              const unsigned m = __ballot_sync(kAll, ok);
              if (ok) Wk.sndl[nsnd + __popc(m & ((1u << lane) - 1u))] = p;
              nsnd += __popc(m);
            }
            __syncwarp();
            unsigned long long key = ~0ull;
            for (int k = lane; k < K; k += 32) {
              if (k == own) continue;
              const int imp = msm_eval_k(I, msgs_s, Wk.gains, Wk.R, Wk.S, maxl_s, s_nmax, Wk.sndl, nsnd, s_mx, k);
              if (imp >= 0) {
                const unsigned long long kk = ((unsigned long long)(0x7fffffff - imp) << 32) | (unsigned)k;
                key = kk < key ? kk : key;
              }
            }
            for (int off = 16; off; off >>= 1) {
              const unsigned long long o2 = __shfl_xor_sync(kAll, key, off);
              key = o2 < key ? o2 : key;
            }
            if (key != ~0ull) best = (int)(key & 0xffffffffu);
          }
        }
        if (best >= 0 && lane == 0) {
          B.dec[v - pos] = (own << 16) | best;
          atomicMin(&B.ctl[par], v);
        }
        __syncwarp();
      }
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tE = gtimer();
        B.stats[16] += tE - tA;
        tA = tE;
      }
      // ---- commit the first mover (if any); the window ends after it
      const int f = lds(&B.ctl[par]);
      int end = end_w;
      if (f != kNone) {
        end = f + 1;
        const int pk = lds(&B.dec[f - pos]);
        const int own = pk >> 16, d = pk & 0xffff;
        const uint32_t base = __ldg(&I.vptr[f]);
        const int deg = (int)(__ldg(&I.vptr[f + 1]) - base);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < deg; i += gridDim.x * blockDim.x)
          msg_commit_net(I, f, own, d, (int)__ldg(&I.vnets[base + i]));
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          I.part_vec[f] = d;
          const int wv = __ldg(&I.w[f]);
          atomicAdd(&I.part_sizes[own], -wv);
          atomicAdd(&I.part_sizes[d], wv);
          atomicAdd((unsigned long long*)&I.moves[it], 1ull);
          B.stats[2]++;
        }
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        B.ctl[par ^ 1] = kNone;
        B.stats[0]++;
        B.stats[9] += end - pos;
        B.stats[f == kNone ? 3 : 8]++;
      }
      if (f == kNone) {
        if (end_w == pos + W) W = min(2 * W, B.wmax);
      } else {
        W = max(256, min(B.wmax, 2 * (f - pos + 1)));
      }
      pos = end;
      round++;
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tC = gtimer();
        B.stats[18] += tC - tA;
        tA = tC;
      }
    }
  }
}

}  // namespace

size_t spec_msg_smem_bytes(int K) {
  auto a = [](size_t n) { return (n + 15) & ~size_t(15); };
  const size_t words = (size_t)(K + 31) / 32;
  return 3 * a(sizeof(int) * K) + 2 * a(sizeof(uint32_t) * words * kSWarps) +
         a(sizeof(unsigned long long) * (size_t)K * kSWarps) + 2 * a(sizeof(int) * (size_t)K * kSWarps);
}

cudaError_t launch_spec_msg(const DevInstance& I, const SpecBuf& B, int passes, int num_sms, cudaStream_t st,
                            int* grid_out) {
  const size_t smem = spec_msg_smem_bytes(I.K);
  const void* fn = (const void*)spec_msg_kernel;
  cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSThreads, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = per_sm * num_sms;
  if (grid * kSWarps > B.max_warps) grid = B.max_warps / kSWarps;
  if (grid_out) *grid_out = grid;
  DevInstance Ic = I;
  SpecBuf Bc = B;
  int p = passes;
  void* args[] = {&Ic, &Bc, &p};
  err = cudaLaunchCooperativeKernel(fn, grid, kSThreads, args, smem, st);
  if (err != cudaSuccess) return err;
  return cudaGetLastError();
}

}  // namespace fp
