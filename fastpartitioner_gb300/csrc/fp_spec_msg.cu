// Speculative grid-wide refinement for the message metrics: TM
// (TM/partition.cpp:300-593) and MSM (MSM/partition.cpp:347-656).  Both walk the
// vertices in id order.
//
// Moves are rare for these metrics, so a round is simple: the warps of the
// grid evaluate a window of vertices against the current state and the first
// mover ends the window.  Every vertex before it is a non-mover decided on
// exactly the sequential state, and the mover's move (lists, connection counts,
// message counts, masks) is applied by warps of the whole grid.
//
// Evaluation reads the K x K connection counts only through bit masks:
// conn == 1 (gains, TM/partition.cpp:347-391) by the row and column of the
// vertex's own part, and conn == 0 (losses per candidate part,
// TM/partition.cpp:408-450) staged in shared memory when K <= 256.  Vertices
// are classed by work like the LDG engine: light ones are evaluated by one
// warp, medium ones by one CTA, the heaviest (up to gmax per window) by all
// warps of the grid, whose slices meet in global sets that one CTA per vertex
// decides from after a grid barrier.

#include "fp_spec_common.cuh"

namespace fp {

namespace {

using namespace spec;

constexpr int kStageK = 256;   // zero masks staged in shared memory up to this K

// conn[a][b] += delta with the message count, the zero masks and the conn == 1
// masks kept exact: the 0->1 minus 1->0 crossings of a +-1 walk give the change
// of [value >= 1], and the parity of crossings into or out of a value gives the
// change of [value == x], whatever the order of concurrent updates.
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
  if ((old == 1) != (now == 1)) {
    atomicXor(&I.c1row[(size_t)a * words + (b >> 5)], 1u << (b & 31));
    atomicXor(&I.c1col[(size_t)b * words + (a >> 5)], 1u << (a & 31));
  }
}

// A word of a zero mask, staged in shared memory or read from L2.
__device__ __forceinline__ uint32_t zword(const uint32_t* p, bool staged) { return staged ? *p : lds(p); }

struct Masks {
  const uint32_t* zr;   // conn == 0 by row (K x words)
  const uint32_t* zc;   // conn == 0 by column
  bool staged;
};

// Per-warp scratch of one evaluation.
struct MsgWarp {
  uint32_t* R;               // receiver parts (bitmask)
  uint32_t* S;               // sender parts (bitmask)
  unsigned long long* fsnd;  // first non-source net per sender part: (net index << 1) | own-alone
  int* gains;                // MSM: gains per part
  int* sndl;                 // MSM: sender parts that are not max parts
  uint32_t* c1r;             // conn[own][*] == 1
  uint32_t* c1c;             // conn[*][own] == 1
};

__device__ __forceinline__ bool bit(const uint32_t* m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }

// Clears the warp's scratch and loads the conn == 1 row and column of own.
__device__ __forceinline__ void msg_begin(const DevInstance& I, const MsgWarp& Wk, int own, bool msm) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  const int words = (K + 31) >> 5;
  for (int x = lane; x < words; x += 32) {
    Wk.R[x] = 0;
    Wk.S[x] = 0;
    Wk.c1r[x] = lds(&I.c1row[(size_t)own * words + x]);
    Wk.c1c[x] = lds(&I.c1col[(size_t)own * words + x]);
  }
  for (int p = lane; p < K; p += 32) {
    Wk.fsnd[p] = ~0ull;
    if (msm) Wk.gains[p] = 0;
  }
  __syncwarp();
}

// Receivers, senders and the source-side gain over nets [nb, min(nb + 32, nend))
// of v (TM/partition.cpp:320-393).  Slots are flattened across the warp and
// loaded 4 per lane per step with their counts.  Returns this lane's
// source-side gain count.
__device__ int msg_batch(const DevInstance& I, int v, int own, uint32_t base, int nb, int nend, const MsgWarp& Wk,
                         unsigned* oc1mask) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  const int k = nb + lane;
  int s = 0, n = 0, sv = -1, ps = -1;
  if (k < nend) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    s = (int)__ldg(&I.nptr[e]);
    const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
    n = lds(&I.ep_len[e]);
    sv = __ldg(&I.src[e]);
    if (sv != v) ps = lds(&I.part_vec[sv]);
    if (n < 0 || n > cap || (sv != v && (unsigned)ps >= (unsigned)K)) {
      dev_fail(I.status, kDevErrInvalid);
      n = 0;
      ps = 0;
    }
  }
  if (lane == 0) *oc1mask = 0u;
  int incl = n;
  for (int off = 1; off < 32; off <<= 1) {
    const int t = __shfl_up_sync(kAll, incl, off);
    if (lane >= off) incl += t;
  }
  const int total = __shfl_sync(kAll, incl, 31);
  __syncwarp();
  int g = 0;
  constexpr int kU = 4;
  for (int f0 = 0; f0 < total; f0 += 32 * kU) {
    int aa[kU], lo_[kU], src_[kU], pp[kU], cc[kU];
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
      src_[u] = __shfl_sync(kAll, sv, lo) == v;
      lo_[u] = lo;
      aa[u] = f < total ? sl + f - (il - nl) : -1;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      pp[u] = aa[u] >= 0 ? lds(&I.ep_part[aa[u]]) : -1;
      cc[u] = aa[u] >= 0 ? lds(&I.ep_cnt[aa[u]]) : 0;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (aa[u] < 0) continue;
      const int t = pp[u];
      if ((unsigned)t >= (unsigned)K) {
        dev_fail(I.status, kDevErrInvalid);
      } else if (src_[u]) {
        if (t == own) {
          if (cc[u] > 1) atomicOr(&Wk.R[own >> 5], 1u << (own & 31));
        } else {
          atomicOr(&Wk.R[t >> 5], 1u << (t & 31));
          // gain_loss_2d[own][t] is 1 here (raised once per listed part, lowered
          // after each net, TM/partition.cpp:347-369): the test is conn == 1.
          if (bit(Wk.c1r, t)) g++;
        }
      } else if (t == own && cc[u] == 1) {
        atomicOr(oc1mask, 1u << lo_[u]);
      }
    }
  }
  __syncwarp();
  if (k < nend && sv != v) {
    atomicOr(&Wk.S[ps >> 5], 1u << (ps & 31));
    atomicMin(&Wk.fsnd[ps], ((unsigned long long)k << 1) | ((*oc1mask >> lane) & 1u));
  }
  __syncwarp();
  return g;
}

// TM: the part k below capacity with the largest gain - loss > 0, lowest k on
// ties (TM/partition.cpp:408-450); threads k0, k0 + kstep, ... each return a
// partial key (~0: none).
__device__ unsigned long long tm_best_partial(const DevInstance& I, const Masks& M, const int* sizes,
                                              const uint32_t* R, const uint32_t* S, int own, int gain, int k0,
                                              int kstep) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  unsigned long long key = ~0ull;
  for (int k = k0; k < K; k += kstep) {
    if (k == own || !((double)sizes[k] < I.C)) continue;
    const uint32_t* zr = M.zr + (size_t)k * words;
    const uint32_t* zc = M.zc + (size_t)k * words;
    int loss = 0;
    for (int x = 0; x < words; x++) {
      const uint32_t self = (x == (k >> 5)) ? ~(1u << (k & 31)) : ~0u;
      loss += __popc(R[x] & zword(&zr[x], M.staged) & self) + __popc(S[x] & zword(&zc[x], M.staged) & self);
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
__device__ int msm_eval_k(const DevInstance& I, const Masks& M, const int* msgs, const int* gains, const uint32_t* R,
                          const uint32_t* S, const int* maxl, int nmax, const int* sndl, int nsnd, int mx, int k) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const uint32_t* zr = M.zr + (size_t)k * words;
  int Lk = 0;
  for (int x = 0; x < words; x++) Lk += __popc(R[x] & zword(&zr[x], M.staged));
  int imp = 0;
  bool k_max = false;
  for (int q = 0; q < nmax; q++) {
    const int m = maxl[q];
    int l = m == k ? Lk : 0;
    if (m == k) k_max = true;
    if (bit(S, m)) l += (zword(&M.zr[(size_t)m * words + (k >> 5)], M.staged) >> (k & 31)) & 1u;
    if (gains[m] <= l) return -1;
    imp += gains[m] - l;
  }
  bool k_snd = false;
  for (int q = 0; q < nsnd; q++) {
    const int sp = sndl[q];
    int l = (int)((zword(&M.zr[(size_t)sp * words + (k >> 5)], M.staged) >> (k & 31)) & 1u);
    if (sp == k) { l += Lk; k_snd = true; }
    if (msgs[sp] + (l - gains[sp]) >= mx) return -1;
  }
  if (!k_max && !k_snd && msgs[k] + (Lk - gains[k]) >= mx) return -1;
  return imp;
}

__device__ __forceinline__ unsigned long long msm_key(int imp, int k) {
  return ((unsigned long long)(0x7fffffff - imp) << 32) | (unsigned)k;
}

// Round state shared by the evaluations of a CTA.
struct MsgRound {
  const int* sizes;
  const int* msgs;
  const int* maxl;   // max-message parts (MSM)
  int nmax, mx;
};

// Decision of one warp for v from its scratch (g: source-side gain count).
// rec (if not null) receives the decision record's gain and loss: TM's gain
// and the loss at the chosen part (TM/partition.cpp:330-450), MSM's gain
// vector summed and the chosen part's improvement (MSM/partition.cpp:388-518).
__device__ int msg_decide_warp(const DevInstance& I, const Masks& M, const MsgRound& Rd, const MsgWarp& Wk, int own,
                               int g, bool msm, int2* rec = nullptr) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  int gs = 0;
  for (int p = lane; p < K; p += 32) {
    const unsigned long long f = Wk.fsnd[p];
    if (f != ~0ull && (f & 1ull) && bit(Wk.c1c, p)) {
      if (msm) Wk.gains[p] += 1;
      else gs++;
    }
  }
  gs = warp_sum(gs);
  __syncwarp();
  unsigned long long key = ~0ull;
  if (!msm) {
    const int gain = g + gs;
    if (gain > 0) key = tm_best_partial(I, M, Rd.sizes, Wk.R, Wk.S, own, gain, lane, 32);
  } else {
    if (lane == 0) Wk.gains[own] += g;
    __syncwarp();
    bool has_gain = false, zero_gain_max = false;
    for (int p = lane; p < K; p += 32) has_gain |= Wk.gains[p] > 0;
    for (int q = lane; q < Rd.nmax; q += 32) zero_gain_max |= Wk.gains[Rd.maxl[q]] <= 0;
    has_gain = __any_sync(kAll, has_gain);
    zero_gain_max = __any_sync(kAll, zero_gain_max);
    if (has_gain && !zero_gain_max) {
      int nsnd = 0;
      for (int p0 = 0; p0 < K; p0 += 32) {
        const int p = p0 + lane;
        const bool ok = p < K && bit(Wk.S, p) && Rd.msgs[p] != Rd.mx;
        const unsigned m = __ballot_sync(kAll, ok);
        if (ok) Wk.sndl[nsnd + __popc(m & ((1u << lane) - 1u))] = p;
        nsnd += __popc(m);
      }
      __syncwarp();
      for (int k = lane; k < K; k += 32) {
        if (k == own) continue;
        const int imp = msm_eval_k(I, M, Rd.msgs, Wk.gains, Wk.R, Wk.S, Rd.maxl, Rd.nmax, Wk.sndl, nsnd, Rd.mx, k);
        if (imp >= 0) key = min(key, msm_key(imp, k));
      }
    }
  }
  for (int off = 16; off; off >>= 1) {
    const unsigned long long o2 = __shfl_xor_sync(kAll, key, off);
    key = o2 < key ? o2 : key;
  }
  if (rec) {
    const int imp = key != ~0ull ? 0x7fffffff - (int)(key >> 32) : -1;
    if (!msm) {
      const int gain = g + gs;
      *rec = make_int2(gain, key != ~0ull ? gain - imp : 0);
    } else {
      int gsum = 0;
      for (int p = lane; p < K; p += 32) gsum += Wk.gains[p];
      *rec = make_int2(warp_sum(gsum), imp);
    }
  }
  return key != ~0ull ? (int)(key & 0xffffffffu) : -1;
}

// Decision of the whole CTA from the combined scratch of warp 0 (R, S, fsnd;
// g: the CTA's source-side gain count).  uscr / iscr: per-warp scratch.
__device__ int msg_decide_cta(const DevInstance& I, const Masks& M, const MsgRound& Rd, const MsgWarp& W0, int own,
                              int g, bool msm, unsigned long long* uscr, int* iscr, int2* rec = nullptr) {
  __shared__ int s_nsnd;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int K = I.K;
  int gs = 0;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    const unsigned long long f = W0.fsnd[p];
    const bool gp = f != ~0ull && (f & 1ull) && bit(W0.c1c, p);
    if (msm) W0.gains[p] = (gp ? 1 : 0) + (p == own ? g : 0);
    else gs += gp;
  }
  gs = warp_sum(gs);
  __syncthreads();
  if (lane == 0) iscr[wib] = gs;
  __syncthreads();
  int gs_t = 0;
  for (int x = 0; x < (int)(blockDim.x >> 5); x++) gs_t += iscr[x];
  unsigned long long key = ~0ull;
  if (!msm) {
    const int gain = g + gs_t;
    if (gain > 0) key = tm_best_partial(I, M, Rd.sizes, W0.R, W0.S, own, gain, threadIdx.x, blockDim.x);
  } else {
    bool has_gain = false, zgm = false;
    for (int p = threadIdx.x; p < K; p += blockDim.x) has_gain |= W0.gains[p] > 0;
    for (int q = threadIdx.x; q < Rd.nmax; q += blockDim.x) zgm |= W0.gains[Rd.maxl[q]] <= 0;
    has_gain = __syncthreads_or(has_gain);
    zgm = __syncthreads_or(zgm);
    if (has_gain && !zgm) {
      if (threadIdx.x == 0) {
        int c = 0;
        for (int p = 0; p < K; p++)
          if (bit(W0.S, p) && Rd.msgs[p] != Rd.mx) W0.sndl[c++] = p;
        s_nsnd = c;
      }
      __syncthreads();
      for (int k = threadIdx.x; k < K; k += blockDim.x) {
        if (k == own) continue;
        const int imp = msm_eval_k(I, M, Rd.msgs, W0.gains, W0.R, W0.S, Rd.maxl, Rd.nmax, W0.sndl, s_nsnd, Rd.mx, k);
        if (imp >= 0) key = min(key, msm_key(imp, k));
      }
    }
  }
  key = block_min_u64(key, uscr);
  if (rec) {
    const int imp = key != ~0ull ? 0x7fffffff - (int)(key >> 32) : -1;
    if (!msm) {
      const int gain = g + gs_t;
      *rec = make_int2(gain, key != ~0ull ? gain - imp : 0);
    } else {
      int gsum = 0;
      for (int p = threadIdx.x; p < K; p += blockDim.x) gsum += W0.gains[p];
      gsum = warp_sum(gsum);
      __syncthreads();
      if (lane == 0) iscr[wib] = gsum;
      __syncthreads();
      int t = 0;
      for (int x = 0; x < (int)(blockDim.x >> 5); x++) t += iscr[x];
      __syncthreads();
      *rec = make_int2(t, imp);
    }
  }
  return key != ~0ull ? (int)(key & 0xffffffffu) : -1;
}

// Combines the scratch of all warps of the CTA into warp 0's (R, S by OR,
// fsnd by minimum); the caller synchronises before and after.
__device__ __forceinline__ void msg_combine(const DevInstance& I, uint32_t* R_b, uint32_t* S_b,
                                            unsigned long long* fs_b) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  for (int x = threadIdx.x; x < words; x += blockDim.x) {
    uint32_t r = 0, s = 0;
    for (int y = 0; y < kSWarps; y++) { r |= R_b[(size_t)y * words + x]; s |= S_b[(size_t)y * words + x]; }
    R_b[x] = r;
    S_b[x] = s;
  }
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    unsigned long long f = ~0ull;
    for (int y = 0; y < kSWarps; y++) f = min(f, fs_b[(size_t)y * K + p]);
    fs_b[p] = f;
  }
}

// Move of v own -> d on net e by one warp: the list (commit_net_warp), then the
// connection updates on the net's final list (TM/partition.cpp:519-587).
__device__ void msg_commit_net_warp(const DevInstance& I, int v, int own, int d, int e) {
  const int lane = threadIdx.x & 31;
  const int n = commit_net_warp(I, own, d, e);
  const int s = (int)__ldg(&I.nptr[e]);
  const int sv = __ldg(&I.src[e]);
  if (sv == v) {
    for (int j = lane; j < n; j += 32) {
      const int t = lds(&I.ep_part[s + j]);
      if (t != d) conn_add_g(I, d, t, 1);
      if (t != own && t != d) conn_add_g(I, own, t, -1);
      if (t == d && lds(&I.ep_cnt[s + j]) > 1) conn_add_g(I, own, t, -1);
    }
  } else {
    bool dc1 = false, fo = false;
    for (int j = lane; j < n; j += 32) {
      const int t = lds(&I.ep_part[s + j]);
      if (t == d && lds(&I.ep_cnt[s + j]) == 1) dc1 = true;
      if (t == own) fo = true;
    }
    dc1 = __any_sync(kAll, dc1);
    fo = __any_sync(kAll, fo);
    if (lane == 0) {
      const int sn = lds(&I.part_vec[sv]);
      if (dc1) conn_add_g(I, sn, d, 1);
      if (!fo) conn_add_g(I, sn, own, -1);
    }
  }
  __syncwarp();
}

// The move of v by the whole grid: one warp per net, then v's part and sizes.
__device__ void msg_commit_grid(const DevInstance& I, int v, int own, int d, int gw, int nwarps, int it) {
  const uint32_t base = __ldg(&I.vptr[v]);
  const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
  for (int i = gw; i < deg; i += nwarps) msg_commit_net_warp(I, v, own, d, (int)__ldg(&I.vnets[base + i]));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    I.part_vec[v] = d;
    const int wv = __ldg(&I.w[v]);
    atomicAdd(&I.part_sizes[own], -wv);
    atomicAdd(&I.part_sizes[d], wv);
    atomicAdd((unsigned long long*)&I.moves[it], 1ull);
  }
}

// Three CTAs per SM (the compiler's own choice otherwise varies with the code
// and can spill).
__global__ void __launch_bounds__(kSThreads, 3) spec_msg_kernel(DevInstance I, SpecBuf B, int passes) {
  barrier_start();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long uscr[kSWarps];
  __shared__ int iscr[kSWarps];
  __shared__ unsigned oc1m[kSWarps];
  __shared__ int s_mx, s_nmax, s_stop;
  __shared__ int s_gz[kMaxGridVerts], s_go[kMaxGridVerts], s_gd[kMaxGridVerts];
  __shared__ uint32_t s_gb[kMaxGridVerts];
  const bool msm = I.metric == 3;
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  const bool staged = K <= kStageK;
  Carve cv{smem_raw};
  int* sizes_s = cv.take<int>(K);
  int* msgs_s = cv.take<int>(K);
  int* maxl_s = cv.take<int>(K);                        // max-message parts (MSM)
  uint32_t* R_b = cv.take<uint32_t>((size_t)words * kSWarps);
  uint32_t* S_b = cv.take<uint32_t>((size_t)words * kSWarps);
  uint32_t* c1r_b = cv.take<uint32_t>((size_t)words * kSWarps);
  uint32_t* c1c_b = cv.take<uint32_t>((size_t)words * kSWarps);
  unsigned long long* fs_b = cv.take<unsigned long long>((size_t)K * kSWarps);
  int* gains_b = cv.take<int>((size_t)K * kSWarps);
  int* sndl_b = cv.take<int>((size_t)K * kSWarps);
  uint32_t* zr_s = staged ? cv.take<uint32_t>((size_t)K * words) : nullptr;
  uint32_t* zc_s = staged ? cv.take<uint32_t>((size_t)K * words) : nullptr;
  const Masks M{staged ? zr_s : I.zrow, staged ? zc_s : I.zcol, staged};
  const MsgWarp Wk{R_b + (size_t)wib * words, S_b + (size_t)wib * words, fs_b + (size_t)wib * K,
                   gains_b + (size_t)wib * K, sndl_b + (size_t)wib * K, c1r_b + (size_t)wib * words,
                   c1c_b + (size_t)wib * words};
  const MsgWarp W0{R_b, S_b, fs_b, gains_b, sndl_b, c1r_b, c1c_b};
  unsigned long long tA = gtimer();
  int heavy_round = 0;
  int round = 0;
  bool dirty = true;   // staged masks out of date (a move was committed)
  for (int it = 0; it < passes; it++) {
    // decision records of the last pass: a vertex evaluated before the window's
    // first mover saw the final state; one after it is evaluated again later
    const bool logp = I.recs != nullptr && it == passes - 1;
    int pos = 0;
    // window length: one position per warp to start, doubled after a window
    // without a mover, twice the distance to the mover after one
    int W = min(nwarps, B.wmax_msg);
    int hidx = 0;
    while (pos < I.nov) {
      // ------------------------------------------------------------ round state
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        sizes_s[p] = lds(&I.part_sizes[p]);
        msgs_s[p] = lds(&I.msgs[p]);
      }
      if (staged && dirty) {
        for (int x = threadIdx.x; x < K * words; x += blockDim.x) {
          zr_s[x] = lds(&I.zrow[x]);
          zc_s[x] = lds(&I.zcol[x]);
        }
      }
      dirty = false;
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
      const MsgRound Rd{sizes_s, msgs_s, maxl_s, msm ? s_nmax : 0, msm ? s_mx : 0};
      while (hidx < B.nheavy && __ldg(&B.heavy_pos[hidx]) < pos) hidx++;

      // ================================================================= round
      // A window holds up to gmax whole-grid vertices and ends before the next
      // one, or at its first mover.
      int end_w = min(pos + W, I.nov);
      if (hidx + B.gmax < B.nheavy) end_w = min(end_w, (int)__ldg(&B.heavy_pos[hidx + B.gmax]));
      int ns = 0;
      while (ns < B.gmax && hidx + ns < B.nheavy && __ldg(&B.heavy_pos[hidx + ns]) < end_w) ns++;
      const int hp = heavy_round & 1;   // whole-grid sets, double-buffered by parity
      // slot j of this parity: K words at hslot(j) (receivers in hloss, senders in
      // hadelta, first non-source nets in hfirst), 8 words of hmisc at hmslot(j)
      auto hslot = [&](int j) { return ((size_t)hp * kMaxGridVerts + j) * K; };
      auto hmslot = [&](int j) { return (hp * kMaxGridVerts + j) * 8; };
      const unsigned long long tR = gtimer();
      if ((int)threadIdx.x < ns) {
        const int v = __ldg(&B.heavy_pos[hidx + threadIdx.x]);
        const uint32_t b = __ldg(&I.vptr[v]);
        s_gz[threadIdx.x] = v;
        s_go[threadIdx.x] = lds(&I.part_vec[v]);
        s_gb[threadIdx.x] = b;
        s_gd[threadIdx.x] = (int)(__ldg(&I.vptr[v + 1]) - b);
      }
      __syncthreads();
      // ---- tally slices of the whole-grid vertices, combined per CTA
      for (int j = 0; j < ns; j++) {
        const int v = s_gz[j], own = s_go[j], deg = s_gd[j];
        const uint32_t base = s_gb[j];
        uint32_t* hR = reinterpret_cast<uint32_t*>(B.hloss + hslot(j));      // words <= K
        uint32_t* hS = reinterpret_cast<uint32_t*>(B.hadelta + hslot(j));
        unsigned long long* hf = B.hfirst + hslot(j);
        msg_begin(I, Wk, own, msm);
        int g = 0;
        {
          int n0, n1;
          net_range(deg, gw, nwarps, &n0, &n1);
          for (int nb = n0; nb < n1; nb += 32) g += msg_batch(I, v, own, base, nb, n1, Wk, &oc1m[wib]);
        }
        g = warp_sum(g);
        __syncthreads();
        msg_combine(I, R_b, S_b, fs_b);
        __syncthreads();
        for (int x = threadIdx.x; x < words; x += blockDim.x) {
          if (R_b[x]) atomicOr(&hR[x], R_b[x]);
          if (S_b[x]) atomicOr(&hS[x], S_b[x]);
        }
        for (int p = threadIdx.x; p < K; p += blockDim.x)
          if (fs_b[p] != ~0ull) atomicMin(&hf[p], fs_b[p]);
        if (lane == 0 && g) atomicAdd(&B.hmisc[hmslot(j)], g);
        __syncthreads();   // the per-warp scratch serves the next vertex and the evaluations below
      }
      if (kTimingStats && ns && threadIdx.x == 0) atomicMax(&B.stats[38], gtimer() - tR);

      const int par = round & 1;
      const int span = end_w - pos;
      const int q = (span + nwarps - 1) / nwarps;
      const int z0 = min(pos + gw * q, end_w);
      const int z1 = min(z0 + q, end_w);
      for (int v = z0; v < z1; v++) {
        if (__ldg(&B.vclass[v]) != 0) continue;   // medium vertex: evaluated by the whole CTA below
        if (lds(&B.ctl[par]) < v) break;           // an earlier mover ends the window
        const int own = lds(&I.part_vec[v]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        msg_begin(I, Wk, own, msm);
        int g = 0;
        for (int nb = 0; nb < deg; nb += 32) g += msg_batch(I, v, own, base, nb, deg, Wk, &oc1m[wib]);
        g = warp_sum(g);
        int2 rec;
        const int best = msg_decide_warp(I, M, Rd, Wk, own, g, msm, logp ? &rec : nullptr);
        if (logp && lane == 0) I.recs[v] = make_int4(best, rec.x, rec.y, best >= 0);
        if (best >= 0) {
          if (lane == 0) {
            B.dec[v - pos] = (own << 16) | best;
            atomicMin(&B.ctl[par], v);
          }
          break;
        }
      }
      // medium vertices of this CTA's positions
      const int cz0 = min(pos + blockIdx.x * kSWarps * q, end_w);
      const int cz1 = min(cz0 + kSWarps * q, end_w);
      for (int mi = lower_bound_pos(B.mid_pos, B.nmid, cz0); mi < B.nmid; mi++) {
        const int v = __ldg(&B.mid_pos[mi]);
        if (v >= cz1) break;
        __syncthreads();
        if (threadIdx.x == 0) s_stop = lds(&B.ctl[par]) < v;
        __syncthreads();
        if (s_stop) break;
        const int own = lds(&I.part_vec[v]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        msg_begin(I, Wk, own, msm);
        int g = 0;
        {
          int n0, n1;
          net_range(deg, wib, kSWarps, &n0, &n1);
          for (int nb = n0; nb < n1; nb += 32) g += msg_batch(I, v, own, base, nb, n1, Wk, &oc1m[wib]);
        }
        g = warp_sum(g);
        __syncthreads();
        if (lane == 0) iscr[wib] = g;
        msg_combine(I, R_b, S_b, fs_b);
        __syncthreads();
        int gt = 0;
        for (int x = 0; x < kSWarps; x++) gt += iscr[x];
        int2 rec;
        const int best = msg_decide_cta(I, M, Rd, W0, own, gt, msm, uscr, iscr, logp ? &rec : nullptr);
        if (logp && threadIdx.x == 0) I.recs[v] = make_int4(best, rec.x, rec.y, best >= 0);
        if (best >= 0) {
          if (threadIdx.x == 0) {
            B.dec[v - pos] = (own << 16) | best;
            atomicMin(&B.ctl[par], v);
          }
          break;
        }
      }
      __syncthreads();
      if (kTimingStats && threadIdx.x == 0) atomicMax(&B.stats[36], gtimer() - tR);
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tE = gtimer();
        B.stats[16] += tE - tA;
        tA = tE;
        // per-window maxima over CTAs (no CTA writes these again before the next window)
        B.stats[32] += B.stats[36];
        B.stats[34] += B.stats[38];
        B.stats[36] = 0;
        B.stats[38] = 0;
      }
      if (ns) {
        // ---- the whole-grid vertices before the first mover: CTA j decides
        // vertex j from the global sets (one read of the first mover per CTA:
        // other CTAs may lower it meanwhile)
        if (threadIdx.x == 0) s_stop = lds(&B.ctl[par]);
        __syncthreads();
        const int f0 = s_stop;
        for (int j = blockIdx.x; j < ns; j += gridDim.x) {
          const int v = s_gz[j], own = s_go[j];
          if (v > f0) break;
          const size_t hs = hslot(j);
          for (int x = threadIdx.x; x < words; x += blockDim.x) {
            R_b[x] = lds(reinterpret_cast<const uint32_t*>(B.hloss + hs) + x);
            S_b[x] = lds(reinterpret_cast<const uint32_t*>(B.hadelta + hs) + x);
            c1c_b[x] = lds(&I.c1col[(size_t)own * words + x]);
          }
          for (int p = threadIdx.x; p < K; p += blockDim.x) fs_b[p] = lds(&B.hfirst[hs + p]);
          __syncthreads();
          int2 rec;
          const int best =
              msg_decide_cta(I, M, Rd, W0, own, lds(&B.hmisc[hmslot(j)]), msm, uscr, iscr, logp ? &rec : nullptr);
          if (logp && threadIdx.x == 0) I.recs[v] = make_int4(best, rec.x, rec.y, best >= 0);
          if (best >= 0 && threadIdx.x == 0) {
            B.dec[v - pos] = (own << 16) | best;
            atomicMin(&B.ctl[par], v);
          }
          __syncthreads();
        }
        if (!grid_barrier(B.bar, I.status)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          const unsigned long long tH = gtimer();
          B.stats[19] += tH - tA;
          tA = tH;
        }
      }
      // ---- commit the first mover (if any); the window ends after it
      const int f = lds(&B.ctl[par]);
      int end = end_w;
      if (f != kNone) {
        end = f + 1;
        const int pk = lds(&B.dec[f - pos]);
        msg_commit_grid(I, f, pk >> 16, pk & 0xffff, gw, nwarps, it);
        if (blockIdx.x == 0 && threadIdx.x == 0) B.stats[2]++;
        dirty = true;
      }
      if (ns) {
        // the other parity's sets are cleared for the next window with
        // whole-grid vertices
        const size_t ob = (size_t)(hp ^ 1) * kMaxGridVerts * K;
        for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kMaxGridVerts * K; p += gridDim.x * blockDim.x) {
          B.hloss[ob + p] = 0;
          B.hadelta[ob + p] = 0;
          B.hfirst[ob + p] = ~0ull;
        }
        if (blockIdx.x == 0 && threadIdx.x < 8 * kMaxGridVerts) B.hmisc[(hp ^ 1) * 8 * kMaxGridVerts + threadIdx.x] = 0;
        heavy_round++;
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        B.ctl[par ^ 1] = kNone;
        B.stats[0]++;
        B.stats[1] += ns;
        B.stats[9] += end - pos;
        B.stats[f == kNone ? 3 : 8]++;
      }
      W = f == kNone ? min(2 * W, B.wmax_msg) : max(min(nwarps, B.wmax_msg), min(B.wmax_msg, 2 * (end - pos)));
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
  size_t b = 3 * a(sizeof(int) * K) + 4 * a(sizeof(uint32_t) * words * kSWarps) +
             a(sizeof(unsigned long long) * (size_t)K * kSWarps) + 2 * a(sizeof(int) * (size_t)K * kSWarps);
  if (K <= kStageK) b += 2 * a(sizeof(uint32_t) * (size_t)K * words);
  return b;
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
