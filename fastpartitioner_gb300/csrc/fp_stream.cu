// Streaming initial partitions on the device: the LDG streams of TV
// (TV/partition.cpp:207-264, LDG2 without a current part), MSV
// (MGV/partition.cpp:122-189) and MSRV (MSRV/partition.cpp:123-196), and CN's
// stream (CN/partition.cpp:132-221), in stream_ldg_kernel; the
// message-greedy streams of TM and MSM (TM/partition.cpp:87-250,
// MSM/partition.cpp:146-309) in stream_msg_kernel, further down.
//
// The reference places the vertices one by one in visiting order: a vertex
// scores every part listed on its nets (the number of its nets listing it,
// times 1 - size / C), takes the best (ties: the smaller part, then the part
// seen first), or the least-loaded part when none scores, and then adds itself
// to its nets' lists: a count increment where the part is listed, an append
// where it is not.  CN scores only the nets with one listed part (uncut nets),
// by that part.  A later decision reads the part sets of its nets (an
// increment changes no score and no first sighting) and the part sizes.
//
// One cooperative kernel runs the stream in windows of the next positions,
// like the refinement engine:
//
//   A  evaluate  every warp tallies its positions' nets against the lists at
//                the window start, decides with the window-start sizes, finds
//                its part's slot in each net and claims the nets it will
//                append to (round-stamped, never cleared);
//   B  validate  a position keeps its decision iff no earlier position of the
//                window appends to one of its nets and the decision taken again
//                with the exact sizes at its place (the window-start sizes plus
//                the earlier placements) is the same.  The window ends at the
//                first conflict; at the first changed decision it either ends
//                too (that position commits last, with its exact decision) or,
//                with StreamArgs::walk, one warp walks on in order with exact
//                sizes, taking every change (a change that appends where the
//                old decision did not claims those nets, and the later
//                positions are checked against the claims again);
//   C  commit    the positions before the cut are applied at once: on any net
//                at most one of them appends (a later reader of that net is
//                invalid), the others increment counts at their recorded slots
//                (changed decisions locate theirs again).
//
// Vertices without nets read only the sizes.  When all of them weigh 0 (vertex
// weight = degree) they are not positions: after each window's commit they take
// the least-loaded part of the sizes at their place.  A position is evaluated
// by a warp, by a CTA when its lists are long (kStreamCtaWork entries or more),
// and a vertex with many nets (kStreamHeavy or more, or kStreamGridWork list
// entries) is a window of its own, evaluated and committed by the whole grid.

#include "fp_spec_common.cuh"

#include <algorithm>

namespace fp {

namespace {

using namespace spec;

constexpr int kCN = 0;
constexpr int kTV = 1;
constexpr int kMSV = 4;
constexpr int kMSRV = 5;

// CN's tally of the nets [nb, min(nb + 32, deg)) of a vertex: the part of
// every net with exactly one listed part, the number of such nets per part and
// the first such net (CN/partition.cpp:150-170).
__device__ __forceinline__ void tally_uncut(const DevInstance& I, uint32_t base, int nb, int deg, int* cnt,
                                            unsigned long long* first) {
  const int k = nb + (threadIdx.x & 31);
  if (k >= deg) return;
  const int e = (int)__ldg(&I.vnets[base + k]);
  if (lds(&I.ep_len[e]) != 1) return;
  const int p = lds(&I.ep_part[__ldg(&I.nptr[e])]);
  if ((unsigned)p >= (unsigned)I.K) {
    dev_fail(I.status, kDevErrInvalid);
    return;
  }
  atomicAdd(&cnt[p], 1);
  atomicMin(&first[p], (unsigned long long)k << 32);
}

// The stream's tally of nets [nb, min(nb + 32, deg)) into cnt / first.
__device__ __forceinline__ void tally_stream(const DevInstance& I, bool cn, uint32_t base, int nb, int deg, int* cnt,
                                             unsigned long long* first) {
  if (cn) tally_uncut(I, base, nb, deg, cnt, first);
  else tally_batch(I, -1, base, nb, deg, cnt, first);
}

__device__ __forceinline__ unsigned long long skey(int round, int pos) {
  return ((unsigned long long)(unsigned)round << 32) | (0xffffffffu - (unsigned)pos);
}
// Did a position before `pos` of this round claim net e (it appends to it)?
__device__ __forceinline__ bool claimed_before(const SpecBuf& B, int round, int e, int pos) {
  const unsigned long long c = lds(&B.claim64[e]);
  return (int)(c >> 32) == round && (int)(0xffffffffu - (unsigned)(c & 0xffffffffu)) < pos;
}

// Candidate entry: part (12 bits), nets listing it (16), first sighting: net
// index (16) and slot (20).  Positions hold fewer than kStreamHeavy nets.
__device__ __forceinline__ unsigned long long sc_entry(int p, int c, unsigned long long f) {
  return ((unsigned long long)p << 52) | ((unsigned long long)c << 36) | (((f >> 32) & 0xffffull) << 20) |
         (f & 0xfffffull);
}

// Exact LDG pick of one warp over candidate entries (part, count, first),
// sizes sz0[p] + (dsz ? dsz[p] : 0): the best positive score, ties to the
// smaller part, then the first seen; -1 if no part scores (TV/partition.cpp:
// 98-117).
__device__ int pick_entries(const DevInstance& I, const unsigned long long* cl, int nc, const int* sz0,
                            const int* dsz) {
  const int lane = threadIdx.x & 31;
  LdgKey best{-1.0, 0, -1, ~0ull};
  for (int i = lane; i < nc; i += 32) {
    const unsigned long long ent = lds(&cl[i]);
    const int p = (int)(ent >> 52);
    const int c = (int)((ent >> 36) & 0xffffull);
    const unsigned long long f = (((ent >> 20) & 0xffffull) << 32) | (ent & 0xfffffull);
    const int sz = sz0[p] + (dsz ? dsz[p] : 0);
    const LdgKey k{ldg_score(c, sz, I.C), sz, p, f};
    if (ldg_better(k, best)) best = k;
  }
  best = warp_ldg_argmax(best);
  return best.part;
}

// Least-loaded part of sz0 + dsz, lowest index on ties (one warp).
__device__ int least_loaded(const int* sz0, const int* dsz, int K) {
  const int lane = threadIdx.x & 31;
  unsigned long long mk = ~0ull;
  for (int p = lane; p < K; p += 32) {
    const int sz = sz0[p] + (dsz ? dsz[p] : 0);
    const unsigned long long key = ((unsigned long long)((unsigned)sz ^ 0x80000000u) << 32) | (unsigned)p;
    mk = key < mk ? key : mk;
  }
  for (int off = 16; off; off >>= 1) {
    const unsigned long long x = __shfl_xor_sync(kAll, mk, off);
    mk = x < mk ? x : mk;
  }
  return (int)(mk & 0xffffffffu);
}

// Slot of part d in each of the nets [nb, min(nb + 32, deg)) of a vertex, -1
// where d is not listed; lane i gets net nb + i's.  The lists' entries are
// walked flattened across the warp, kU loads per lane in flight, as in
// tally_batch.  sd: 32 ints of per-warp scratch.
__device__ int locate_part(const DevInstance& I, uint32_t base, int nb, int deg, int d, int* sd) {
  const int lane = threadIdx.x & 31;
  const int k = nb + lane;
  int s = 0, n = 0;
  if (k < deg) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    s = (int)__ldg(&I.nptr[e]);
    const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
    n = lds(&I.ep_len[e]);
    if (n < 0 || n > cap) { dev_fail(I.status, kDevErrInvalid); n = 0; }
  }
  sd[lane] = -1;
  int incl = n;
  for (int off = 1; off < 32; off <<= 1) {
    const int t = __shfl_up_sync(kAll, incl, off);
    if (lane >= off) incl += t;
  }
  const int total = __shfl_sync(kAll, incl, 31);
  __syncwarp();
  constexpr int kU = 4;
  for (int f0 = 0; f0 < total; f0 += 32 * kU) {
    int aa[kU], kn[kU], kj[kU];
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
    int pp[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) pp[u] = aa[u] >= 0 ? lds(&I.ep_part[aa[u]]) : -1;
#pragma unroll
    for (int u = 0; u < kU; u++)
      if (aa[u] >= 0 && pp[u] == d) sd[kn[u]] = kj[u];   // d is listed once per net: one writer
  }
  __syncwarp();
  const int j = sd[lane];
  __syncwarp();
  return k < deg ? j : -1;
}

// Adds one pin of part d to net e at slot `slot` (-1 / kNoSlot: append).
__device__ __forceinline__ void place_net(const DevInstance& I, int e, int d, int slot) {
  const int s = (int)__ldg(&I.nptr[e]);
  if (slot >= 0 && slot != (int)kNoSlot) {
    atomicAdd(&I.ep_cnt[s + slot], 1);
  } else {
    const int n = lds(&I.ep_len[e]);
    const int cap = (int)__ldg(&I.nptr[e + 1]) - s;
    if (n >= cap) {
      dev_fail(I.status, kDevErrInvalid);
      return;
    }
    I.ep_part[s + n] = d;
    I.ep_cnt[s + n] = 1;
    I.ep_len[e] = n + 1;
  }
}

// Candidates of window offset o from a tally (cnt / first over K parts), in
// ascending part order, and its decision with the window-start sizes (the
// least-loaded part minpart when no part scores); writes cand, ncand, dec, wt
// and the weight's mlist entry.  One warp; returns the decision.
__device__ int decide_position(const DevInstance& I, const SpecBuf& B, const int* sizes_s, int minpart,
                               const int* cnt, const unsigned long long* first, int o, int wv, int par,
                               int* nc_out) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  unsigned long long* cl = B.cand + (size_t)o * K;
  int nc = 0;
  LdgKey best{-1.0, 0, -1, ~0ull};
  for (int p0 = 0; p0 < K; p0 += 32) {
    const int p = p0 + lane;
    const int c = p < K ? cnt[p] : 0;
    const unsigned m = __ballot_sync(kAll, c > 0);
    if (c > 0) {
      cl[nc + __popc(m & ((1u << lane) - 1u))] = sc_entry(p, c, first[p]);
      const LdgKey k{ldg_score(c, sizes_s[p], I.C), sizes_s[p], p, first[p]};
      if (ldg_better(k, best)) best = k;
    }
    nc += __popc(m);
  }
  best = warp_ldg_argmax(best);
  const int d = best.part >= 0 ? best.part : minpart;
  *nc_out = nc;
  if (lane == 0) {
    B.ncand[o] = nc;
    B.dec[o] = d;
    B.wt[o] = wv;
    B.flag[o] = 0;
    if (wv) {
      const int i = atomicAdd(&B.mcnt[par], 1);
      B.mlist[i] = make_int4(o, wv, d, 0);
      B.midx[o] = i;
    }
  }
  __syncwarp();
  return d;
}

// The records of d in the nets [n0, n1) of a vertex (one warp) and the claims
// of the nets d is appended to.
// With claim_all every net is claimed (and counted as appended to): any
// other decision's appends are then a subset.
__device__ int record_slots(const DevInstance& I, const SpecBuf& B, const StreamArgs& S, uint32_t base, int n0,
                            int n1, int d, int round, int z, int* sd, bool claim_all) {
  const int lane = threadIdx.x & 31;
  int napp = 0;
  for (int nb = n0; nb < n1; nb += 32) {
    const int j = locate_part(I, base, nb, n1, d, sd);
    const int k = nb + lane;
    const bool app = k < n1 && (j < 0 || claim_all);
    if (k < n1) {
      S.rec[base + k] = j >= 0 ? (uint32_t)j : kNoSlot;
      if (app) atomicMax(&B.claim64[(int)__ldg(&I.vnets[base + k])], skey(round, z));
    }
    napp += __popc(__ballot_sync(kAll, app));
  }
  return napp;   // every lane
}

// The walk takes a changed decision d of position z that appends where the old
// one did not: the nets d is appended to are claimed for z (the earliest
// claim wins), and the walk checks every later position against the claims
// again.  One warp.
__device__ void claim_appends(const DevInstance& I, const SpecBuf& B, int v, int round, int z, int d, int* sd) {
  const int lane = threadIdx.x & 31;
  const uint32_t base = __ldg(&I.vptr[v]);
  const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
  for (int nb = 0; nb < deg; nb += 32) {
    const int j = locate_part(I, base, nb, deg, d, sd);
    const int k = nb + lane;
    if (k < deg && j < 0) atomicMax(&B.claim64[(int)__ldg(&I.vnets[base + k])], skey(round, z));
  }
}

// Does an earlier position of the round claim one of position z's nets (v's)?
// One warp; every lane gets the answer.
__device__ bool conflicts_now(const DevInstance& I, const SpecBuf& B, int v, int round, int z) {
  const int lane = threadIdx.x & 31;
  const uint32_t base = __ldg(&I.vptr[v]);
  const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
  bool conf = false;
  for (int k = lane; k < deg && !conf; k += 32) conf = claimed_before(B, round, (int)__ldg(&I.vnets[base + k]), z);
  return __any_sync(kAll, conf);
}

// Nets of window offset o listing part d (its candidate entry's count; 0 if d
// is not a candidate).  One warp.
__device__ int cand_count(const SpecBuf& B, int K, int o, int d) {
  const int lane = threadIdx.x & 31;
  const unsigned long long* cl = B.cand + (size_t)o * K;
  const int nc = lds(&B.ncand[o]);
  int c = 0;
  for (int i = lane; i < nc; i += 32) {
    const unsigned long long ent = lds(&cl[i]);
    if ((int)(ent >> 52) == d) c = (int)((ent >> 36) & 0xffffull);
  }
  return warp_max(c);
}

// The vertices without nets [k0, k1) of the iso list take the least-loaded
// part of sz (TV: the size of that part above max_pw would make the reference
// use part -1: unsupported).  One warp; *amin caches the argmin (-1: stale).
__device__ void place_iso(const DevInstance& I, const StreamArgs& S, const int* sz, int k0, int k1, int* amin) {
  if (k0 >= k1) return;
  const int lane = threadIdx.x & 31;
  if (*amin < 0) *amin = least_loaded(sz, nullptr, I.K);
  const int d = *amin;
  if (I.metric == kTV && sz[d] > I.max_pw) {
    if (lane == 0) dev_fail(I.status, kDevErrUnsupported);
    return;
  }
  for (int k = k0 + lane; k < k1; k += 32) I.part_vec[__ldg(&S.iso_list[k])] = d;
}

__global__ void __launch_bounds__(kSThreads, 2) stream_ldg_kernel(DevInstance I, SpecBuf B, StreamArgs S) {
  barrier_start();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long uscr[kSWarps];
  __shared__ int s_minpart, s_minsize, s_second, s_dec, s_napp, s_nc;
  const int K = I.K;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gthreads = gridDim.x * blockDim.x;
  const bool tv = I.metric == kTV;
  const bool cn = I.metric == kCN;   // no marker and no TV clamp
  Carve cv{smem_raw};
  int* sizes_s = cv.take<int>(K);
  int* dsz_cta = cv.take<int>(K);
  int* cnt_b = cv.take<int>((size_t)K * kSWarps);
  unsigned long long* first_b = cv.take<unsigned long long>((size_t)K * kSWarps);
  int* sd_b = cv.take<int>(32 * kSWarps);
  int* cnt = cnt_b + (size_t)wib * K;
  unsigned long long* first = first_b + (size_t)wib * K;
  int* sd = sd_b + 32 * wib;
  const bool stats = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long t0 = stats ? gtimer() : 0ull;
  auto lap = [&](int slot) {   // block 0's time since the last lap into stats[slot]
    if (stats) {
      const unsigned long long t = gtimer();
      B.stats[slot] += t - t0;
      t0 = t;
    }
  };

  int pos = 0, round = 1, hidx = 0;
  int W = min(nwarps, B.wmax);
  while (pos < S.npos) {
    const int par = round & 1;
    // ------------------------------------------------------------ round state
    for (int p = threadIdx.x; p < K; p += blockDim.x) sizes_s[p] = lds(&I.part_sizes[p]);
    __syncthreads();
    block_min_part(sizes_s, K, uscr, &s_minpart, &s_minsize, &s_second);
    __syncthreads();
    while (hidx < S.nheavy && __ldg(&S.heavy_pos[hidx]) < pos) hidx++;
    if (hidx < S.nheavy && __ldg(&S.heavy_pos[hidx]) == pos) {
      // ================================================ a vertex with many nets
      const int v = __ldg(&S.porder[pos]);
      const uint32_t base = __ldg(&I.vptr[v]);
      const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
      for (int p = lane; p < K; p += 32) { cnt[p] = 0; first[p] = ~0ull; }
      __syncwarp();
      {
        int n0, n1;
        net_range(deg, gw, nwarps, &n0, &n1);
        for (int nb = n0; nb < n1; nb += 32) tally_stream(I, cn, base, nb, n1, cnt, first);
      }
      __syncthreads();
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        int c = 0;
        unsigned long long f = ~0ull;
        for (int x = 0; x < kSWarps; x++) {
          c += cnt_b[(size_t)x * K + p];
          const unsigned long long fx = first_b[(size_t)x * K + p];
          f = fx < f ? fx : f;
        }
        if (c) {
          atomicAdd(&B.hcnt[p], c);
          atomicMin(&B.hfirst[p], f);
        }
      }
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0) {
        if (wib == 0) {
          LdgKey best{-1.0, 0, -1, ~0ull};
          for (int p = lane; p < K; p += 32) {
            const int c = lds(&B.hcnt[p]);
            if (c <= 0) continue;
            const LdgKey k{ldg_score(c, sizes_s[p], I.C), sizes_s[p], p, lds(&B.hfirst[p])};
            if (ldg_better(k, best)) best = k;
          }
          best = warp_ldg_argmax(best);
          const int d = best.part >= 0 ? best.part : s_minpart;
          if (lane == 0) {
            if (tv && sizes_s[d] > I.max_pw) dev_fail(I.status, kDevErrUnsupported);
            B.dec[0] = d;
          }
        }
        if (!cn)
          for (int p = threadIdx.x; p < K; p += blockDim.x)
            if (lds(&B.hcnt[p]) > 0) atomicMax(&S.mark_pos[p], pos);
      }
      if (!grid_barrier(B.bar, I.status)) return;
      const int d = lds(&B.dec[0]);
      const int wv = __ldg(&I.w[v]);
      {
        int n0, n1;
        net_range(deg, gw, nwarps, &n0, &n1);
        for (int nb = n0; nb < n1; nb += 32) {
          const int j = locate_part(I, base, nb, n1, d, sd);
          if (nb + lane < n1) place_net(I, (int)__ldg(&I.vnets[base + nb + lane]), d, j);
        }
      }
      if (gtid == 0) {
        I.part_vec[v] = d;
        if (wv) atomicAdd(&I.part_sizes[d], wv);
      }
      if (S.niso && gw == 0) {
        // the vertices without nets before and after this one
        int* sz = cnt;
        for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p];
        __syncwarp();
        int amin = -1;
        if (pos == 0) place_iso(I, S, sz, 0, __ldg(&S.iso_before[0]), &amin);
        __syncwarp();
        if (lane == 0) sz[d] += wv;
        __syncwarp();
        amin = wv ? -1 : amin;
        place_iso(I, S, sz, __ldg(&S.iso_before[pos]), __ldg(&S.iso_before[pos + 1]), &amin);
      }
      for (int p = gtid; p < K; p += gthreads) {
        B.hcnt[p] = 0;
        B.hfirst[p] = ~0ull;
      }
      if (gtid == 0) {   // the next round's cut words and placements, as a window leaves them
        B.ctl[4 + (par ^ 1)] = kNone;
        B.ctl[2 + (par ^ 1)] = kNone;
        B.mcnt[par ^ 1] = 0;
      }
      pos++;
      round++;
      if (!grid_barrier(B.bar, I.status)) return;
      if (stats) B.stats[1]++;
      lap(19);
      continue;
    }

    // ================================================================= window
    int end_w = min(pos + W, S.npos);
    if (hidx < S.nheavy) end_w = min(end_w, (int)__ldg(&S.heavy_pos[hidx]));
    const int span = end_w - pos;
    const int q = (span + nwarps - 1) / nwarps;
    const int z0 = min(pos + gw * q, end_w);
    const int z1 = min(z0 + q, end_w);
    // ---- A: evaluate: light positions by their warps, medium positions by
    // CTAs from the end of the grid
    for (int z = z0; z < z1; z++) {
      if (__ldg(&S.pclass[z]) != 0) continue;
      const int o = z - pos;
      const int v = __ldg(&S.porder[z]);
      const uint32_t base = __ldg(&I.vptr[v]);
      const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
      for (int p = lane; p < K; p += 32) { cnt[p] = 0; first[p] = ~0ull; }
      __syncwarp();
      for (int nb = 0; nb < deg; nb += 32) tally_stream(I, cn, base, nb, deg, cnt, first);
      __syncwarp();
      int nc;
      const int d = decide_position(I, B, sizes_s, s_minpart, cnt, first, o, __ldg(&I.w[v]), par, &nc);
      // CN: a position without candidates decides by the sizes alone; it
      // claims all its nets, so that a changed decision adds no claim
      const int napp = record_slots(I, B, S, base, 0, deg, d, round, z, sd, cn && nc == 0);
      if (lane == 0) B.slack[o] = napp;   // nets the decision appends to
      __syncwarp();
    }
    if (S.nmid) {
      const int i0 = lower_bound_pos(S.mid_pos, S.nmid, pos);
      const int i1 = lower_bound_pos(S.mid_pos, S.nmid, end_w);
      for (int i = i0 + (int)(gridDim.x - 1 - blockIdx.x); i < i1; i += gridDim.x) {
        const int z = __ldg(&S.mid_pos[i]);
        const int o = z - pos;
        const int v = __ldg(&S.porder[z]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        int n0, n1;
        net_range(deg, wib, kSWarps, &n0, &n1);
        __syncthreads();   // the tallies of the CTA's previous position are read
        for (int p = lane; p < K; p += 32) { cnt[p] = 0; first[p] = ~0ull; }
        __syncwarp();
        for (int nb = n0; nb < n1; nb += 32) tally_stream(I, cn, base, nb, n1, cnt, first);
        __syncthreads();
        for (int p = threadIdx.x; p < K; p += blockDim.x) {   // warp 0's arrays hold the sums
          int c = 0;
          unsigned long long f = ~0ull;
          for (int x = 0; x < kSWarps; x++) {
            c += cnt_b[(size_t)x * K + p];
            const unsigned long long fx = first_b[(size_t)x * K + p];
            f = fx < f ? fx : f;
          }
          cnt_b[p] = c;
          first_b[p] = f;
        }
        __syncthreads();
        if (wib == 0) {
          int nc;
          const int d = decide_position(I, B, sizes_s, s_minpart, cnt_b, first_b, o, __ldg(&I.w[v]), par, &nc);
          if (lane == 0) {
            s_dec = d;
            s_nc = nc;
          }
        }
        if (threadIdx.x == 0) s_napp = 0;
        __syncthreads();
        const int napp = record_slots(I, B, S, base, n0, n1, s_dec, round, z, sd, cn && s_nc == 0);
        if (lane == 0) atomicAdd(&s_napp, napp);
        __syncthreads();
        if (threadIdx.x == 0) B.slack[o] = s_napp;
      }
    }
    if (!grid_barrier(B.bar, I.status)) return;
    lap(16);
    // ---- B: validate.  B1 (every warp): the first position with a claim
    // conflict, and the first whose decision changes with the exact sizes
    // (or needs a TV part above max_pw) if every earlier one keeps its own.
    // B2 (one warp, only if such a change comes before the first conflict):
    // walk the positions from it in order with exact sizes, taking each
    // changed decision whose appends are a subset of the old one's (no new
    // claims), and end the window at the first change that is not -- that
    // position commits last, with its exact decision -- or at the conflict.
    int* const cut_w = &B.ctl[4 + par];
    int* const flip_w = &B.ctl[2 + par];
    const int cz0 = min(pos + blockIdx.x * kSWarps * q, end_w);
    const int cta_o0 = cz0 - pos;
    {
      for (int p = threadIdx.x; p < K; p += blockDim.x) dsz_cta[p] = 0;
      __syncthreads();
      const int nm = lds(&B.mcnt[par]);
      for (int i = threadIdx.x; i < nm; i += blockDim.x) {
        const int4 m = lds(&B.mlist[i]);
        if (m.x < cta_o0) atomicAdd(&dsz_cta[m.z], m.y);
      }
      __syncthreads();
      bool decided = false;   // this warp found its first change: later ones only check conflicts
      for (int z = z0; z < z1; z++) {
        const int o = z - pos;
        const int v = __ldg(&S.porder[z]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        bool conf = false;
        for (int k = lane; k < deg && !conf; k += 32)
          conf = claimed_before(B, round, (int)__ldg(&I.vnets[base + k]), z);
        if (__any_sync(kAll, conf)) {
          if (lane == 0) atomicMin(cut_w, (z << 3) | 5);
          break;
        }
        if (decided) continue;
        // the exact sizes here if no earlier decision changes: the window-start
        // sizes, the placements before this CTA's positions, those of this
        // CTA's positions before z
        int* dsz = cnt;
        for (int p = lane; p < K; p += 32) dsz[p] = dsz_cta[p];
        __syncwarp();
        for (int o2 = cta_o0 + lane; o2 < o; o2 += 32) {
          const int w = lds(&B.wt[o2]);
          if (w) atomicAdd(&dsz[lds(&B.dec[o2])], w);
        }
        __syncwarp();
        int d2 = pick_entries(I, B.cand + (size_t)o * K, lds(&B.ncand[o]), sizes_s, dsz);
        if (d2 < 0) d2 = least_loaded(sizes_s, dsz, K);
        const bool clamp = tv && sizes_s[d2] + dsz[d2] > I.max_pw;
        if (d2 != lds(&B.dec[o]) || clamp) {
          if (lane == 0) {
            B.dfix[o] = d2;
            atomicMin(flip_w, (z << 3) | (clamp ? 7 : 2));
          }
          decided = true;
        }
        __syncwarp();
      }
    }
    if (!grid_barrier(B.bar, I.status)) return;
    lap(17);
    const int cutw = lds(cut_w), flipw = lds(flip_w);
    const int zc = cutw == kNone ? end_w : min(cutw >> 3, end_w);
    const int zf = flipw == kNone ? end_w : min(flipw >> 3, end_w);
    int cut = zc, cutc = zc;
    if (zf < zc && !S.walk) {
      // the first change ends the window: it commits last with its exact
      // decision (a TV clamp does not commit)
      cut = zf;
      cutc = (flipw & 7) == 2 ? zf + 1 : zf;
    } else if (zf < zc) {
      if (blockIdx.x == 0 && wib == 0) {
        int* sz = cnt;
        for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p];
        __syncwarp();
        const int nm = lds(&B.mcnt[par]);
        for (int i = lane; i < nm; i += 32) {
          const int4 m = lds(&B.mlist[i]);
          if (m.x < zf - pos) atomicAdd(&sz[m.z], m.y);
        }
        __syncwarp();
        int c1 = zc, c2 = zc;
        bool stop = false, reclaim = false;
        // 32 positions at a time: their scalar words one per lane, and the
        // next position's first 32 candidates loaded while one is decided
        for (int zb = zf; zb < zc && !stop; zb += 32) {
          const int zl = zb + lane, ol = zl - pos;
          const bool in = zl < zc;
          const int nc_l = in ? lds(&B.ncand[ol]) : 0;
          const int d_l = in ? lds(&B.dec[ol]) : 0;
          const int w_l = in ? lds(&B.wt[ol]) : 0;
          const int na_l = in ? lds(&B.slack[ol]) : 0;
          int deg_l = 0, v_l = 0;
          if (in) {
            v_l = __ldg(&S.porder[zl]);
            deg_l = (int)(__ldg(&I.vptr[v_l + 1]) - __ldg(&I.vptr[v_l]));
          }
          const int nb = min(32, zc - zb);
          unsigned long long ent = 0;
          {
            const int nc0 = __shfl_sync(kAll, nc_l, 0);
            if (lane < nc0) ent = lds(&B.cand[(size_t)(zb - pos) * K + lane]);
          }
          for (int j = 0; j < nb; j++) {
            const int z = zb + j, o = z - pos;
            const int nc = __shfl_sync(kAll, nc_l, j);
            const int d = __shfl_sync(kAll, d_l, j);
            const int w = __shfl_sync(kAll, w_l, j);
            const int napp = __shfl_sync(kAll, na_l, j);
            const int deg = __shfl_sync(kAll, deg_l, j);
            const int vz = __shfl_sync(kAll, v_l, j);
            const int ncn = __shfl_sync(kAll, nc_l, (j + 1) & 31);
            if (reclaim && conflicts_now(I, B, vz, round, z)) {   // a taken change appends to one of its nets
              c1 = c2 = z;
              stop = true;
              break;
            }
            unsigned long long ent_next = 0;
            if (j + 1 < nb && lane < ncn) ent_next = lds(&B.cand[(size_t)(o + 1) * K + lane]);
            LdgKey best{-1.0, 0, -1, ~0ull};
            for (int i = lane; i < nc; i += 32) {
              const unsigned long long e = i < 32 ? ent : lds(&B.cand[(size_t)o * K + i]);
              const int p = (int)(e >> 52);
              const int c = (int)((e >> 36) & 0xffffull);
              const unsigned long long f = (((e >> 20) & 0xffffull) << 32) | (e & 0xfffffull);
              const LdgKey k{ldg_score(c, sz[p], I.C), sz[p], p, f};
              if (ldg_better(k, best)) best = k;
            }
            best = warp_ldg_argmax(best);
            const int d2 = best.part >= 0 ? best.part : least_loaded(sz, nullptr, K);
            ent = ent_next;
            if (tv && sz[d2] > I.max_pw) {   // the reference would use part -1
              c1 = c2 = z;
              stop = true;
              break;
            }
            if (d2 != d) {
              // the old decision appended to every net, or the new one to none:
              // no new claim; else the new appends are claimed
              const bool safe = napp == deg || (!cn && cand_count(B, K, o, d2) == deg);
              if (!safe) {
                claim_appends(I, B, vz, round, z, d2, sd);
                reclaim = true;
              }
              if (lane == 0) {
                B.dec[o] = d2;
                B.flag[o] = 1;   // its records are d's: located again at commit
                if (w) B.mlist[lds(&B.midx[o])].z = d2;
                B.stats[9]++;
              }
            }
            __syncwarp();
            if (lane == 0 && w) sz[d2] += w;
            __syncwarp();
          }
        }
        if (lane == 0) {
          B.ctl[6] = c1;
          B.ctl[7] = c2;
        }
      }
      if (!grid_barrier(B.bar, I.status)) return;
      lap(20);
      cut = lds(&B.ctl[6]);
      cutc = lds(&B.ctl[7]);
      // the placements before each CTA's positions, with the changed decisions
      for (int p = threadIdx.x; p < K; p += blockDim.x) dsz_cta[p] = 0;
      __syncthreads();
      const int nm = lds(&B.mcnt[par]);
      for (int i = threadIdx.x; i < nm; i += blockDim.x) {
        const int4 m = lds(&B.mlist[i]);
        if (m.x < cta_o0) atomicAdd(&dsz_cta[m.z], m.y);
      }
      __syncthreads();
    }
    if (cut <= pos) {
      // the window's first position needs a part above max_pw: the reference
      // would place it in part -1
      if (gtid == 0) dev_fail(I.status, tv ? kDevErrUnsupported : kDevErrInvalid);
      return;
    }
    // ---- C: commit the positions before the cut (and a flip at the cut)
    for (int z = z0; z < min(z1, cutc); z++) {
      const int o = z - pos;
      const int v = __ldg(&S.porder[z]);
      const uint32_t base = __ldg(&I.vptr[v]);
      const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
      const int d = z == cut ? lds(&B.dfix[o]) : lds(&B.dec[o]);
      if (z == cut || lds(&B.flag[o])) {
        for (int nb = 0; nb < deg; nb += 32) {
          const int j = locate_part(I, base, nb, deg, d, sd);
          if (nb + lane < deg) place_net(I, (int)__ldg(&I.vnets[base + nb + lane]), d, j);
        }
      } else {
        for (int k = lane; k < deg; k += 32)
          place_net(I, (int)__ldg(&I.vnets[base + k]), d, (int)lds(&S.rec[base + k]));
      }
      if (!cn) {
        const unsigned long long* cl = B.cand + (size_t)o * K;
        const int nc = lds(&B.ncand[o]);
        for (int i = lane; i < nc; i += 32) atomicMax(&S.mark_pos[(int)(lds(&cl[i]) >> 52)], z);
      }
      if (lane == 0) {
        I.part_vec[v] = d;
        const int wv = lds(&B.wt[o]);
        if (wv) atomicAdd(&I.part_sizes[d], wv);
      }
    }
    if (S.niso) {
      // the vertices without nets between the committed positions: the
      // least-loaded part of the exact sizes at their place
      const int zb = min(z1, cutc);
      if (z0 < zb || (pos == 0 && gw == 0)) {
        const int cta_o0 = min(pos + blockIdx.x * kSWarps * q, end_w) - pos;
        int* sz = cnt;
        for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p] + dsz_cta[p];
        __syncwarp();
        for (int o2 = cta_o0 + lane; o2 < z0 - pos; o2 += 32) {
          const int w = lds(&B.wt[o2]);
          if (w) atomicAdd(&sz[lds(&B.dec[o2])], w);
        }
        __syncwarp();
        int amin = -1;
        if (pos == 0 && gw == 0) place_iso(I, S, sz, 0, __ldg(&S.iso_before[0]), &amin);
        for (int z = z0; z < zb; z++) {
          const int o = z - pos;
          const int w = lds(&B.wt[o]);
          if (w) {
            __syncwarp();
            if (lane == 0) sz[z == cut ? lds(&B.dfix[o]) : lds(&B.dec[o])] += w;
            __syncwarp();
            amin = -1;
          }
          place_iso(I, S, sz, __ldg(&S.iso_before[z]), __ldg(&S.iso_before[z + 1]), &amin);
        }
      }
    }
    if (gw == 0 && lane == 0) {
      B.ctl[4 + (par ^ 1)] = kNone;
      B.ctl[2 + (par ^ 1)] = kNone;
      B.mcnt[par ^ 1] = 0;
    }
    if (stats) {
      B.stats[0]++;
      B.stats[2] += cutc - pos;
      if (cutc > cut) B.stats[5]++;                       // a change with new appends
      else if (cut < end_w) B.stats[8]++;                 // a conflict
    }
    if (cutc >= end_w) {
      if (end_w == pos + W) W = min(2 * W, B.wmax);
    } else {
      W = max(256, min(B.wmax, 2 * (cutc - pos)));
    }
    pos = cutc;
    round++;
    if (!grid_barrier(B.bar, I.status)) return;
    lap(18);
  }
  // TV's marker: the last vertex that saw each part (TV/partition.cpp:218-226)
  if (blockIdx.x == 0 && !cn)
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
      const int z = lds(&S.mark_pos[p]);
      I.marker[p] = z >= 0 ? __ldg(&S.porder[z]) : -1;
    }
}

// Send (and, MSRV, received) volumes of the streamed lists: the source's part
// sends to every other listed part (MGV/partition.cpp:159-184).
// Nothing is counted after a failed stream (its part vector is incomplete).
__global__ void stream_volumes_kernel(DevInstance I, int rv) {
  if (*I.status != 0) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < I.noe; e += gridDim.x * blockDim.x) {
    const int sp = I.part_vec[__ldg(&I.src[e])];
    if ((unsigned)sp >= (unsigned)I.K) continue;
    const int s = (int)__ldg(&I.nptr[e]);
    const int n = I.ep_len[e];
    for (int j = 0; j < n; j++) {
      const int p = I.ep_part[s + j];
      if (p == sp || (unsigned)p >= (unsigned)I.K) continue;
      atomicAdd(&I.send[sp], 1);
      if (rv) atomicAdd(&I.recv[p], 1);
    }
  }
}

// ============================================================== TM / MSM
// The message-greedy stream (TM/partition.cpp:87-250, MSM/partition.cpp:
// 146-309).  A vertex v reads: the source parts of its nets whose source is
// placed (the active parts), the part lists of the nets it is the source of
// (its own nets), which connection counts are positive in the active parts'
// rows and in the listed parts' columns, and the part sizes.  It saves, in
// part k, one message per active part sp with conn[sp][k] > 0 and one per
// (own net, listed part p) with conn[k][p] > 0; it takes the part below
// capacity that saves the most (ties: the smaller part, then the lower
// index), else the least-loaded part.  Placing v appends or increments its
// nets' lists, makes v's part the source part of its own nets, and raises
// conn[sp][d] (1 if it was 0, else +1 where d is new on the net) and
// conn[d][p] (+1 per own net listing p), counting a message where an entry
// leaves 0.
//
// A window position is invalid when an earlier one appends to or is the
// source of one of its nets (claims), or makes an entry positive in a row or
// column it reads (first such position per row and per column, by round
// parity).  Among the committed positions an entry that was 0 at the window
// start is therefore raised by one position only, so its first-event rule is
// applied by that position alone; the other entries only add.

// Record of a (vertex, net) pair: the chosen part's slot (13 bits; kNoSlot:
// appended), the net's source part at the window start plus one (11 bits; 0:
// the source is not placed), the vertex is the net's source (bit 24).
__device__ __forceinline__ uint32_t mrec(int slot, int sp, bool own) {
  return (uint32_t)(slot < 0 ? (int)kNoSlot : slot) | ((uint32_t)(sp + 1) << 13) | (own ? 1u << 24 : 0u);
}
__device__ __forceinline__ int mrec_slot(uint32_t r) { return (int)(r & 0x1fffu); }
__device__ __forceinline__ int mrec_sp(uint32_t r) { return (int)((r >> 13) & 0x7ffu) - 1; }
__device__ __forceinline__ bool mrec_own(uint32_t r) { return (r >> 24) & 1u; }

__device__ __forceinline__ bool bit_of(const uint32_t* m, int b) { return (m[b >> 5] >> (b & 31)) & 1u; }

struct MsgKey {
  int sv, sz, k;   // k = -1: none
};
__device__ __forceinline__ bool msg_better(const MsgKey& a, const MsgKey& b) {
  if (a.k < 0) return false;
  if (b.k < 0) return true;
  if (a.sv != b.sv) return a.sv > b.sv;
  if (a.sz != b.sz) return a.sz < b.sz;
  return a.k < b.k;
}
__device__ __forceinline__ MsgKey warp_msg_best(MsgKey x) {
  for (int off = 16; off; off >>= 1) {
    MsgKey o;
    o.sv = __shfl_xor_sync(kAll, x.sv, off);
    o.sz = __shfl_xor_sync(kAll, x.sz, off);
    o.k = __shfl_xor_sync(kAll, x.k, off);
    if (msg_better(o, x)) x = o;
  }
  return x;
}

// Messages part k saves for the active parts `act` and the own-net parts
// `own` with multiplicities `mult` (conn > 0 masks prow / pcol).
// The masks are read from shared memory (a copy staged at the round start)
// when kStaged, else from global memory past L1.
constexpr int kMsgStageK = 256;
template <bool kStaged>
__device__ __forceinline__ uint32_t mask_word(const uint32_t* p) { return kStaged ? *p : __ldcg(p); }

template <bool kStaged>
__device__ __forceinline__ int msg_saved(const uint32_t* prow, const uint32_t* pcol, int words, int k,
                                         const uint32_t* act, const uint32_t* own, const int* mult) {
  int sv = 0;
  const uint32_t* col = pcol + (size_t)k * words;
  const uint32_t* row = prow + (size_t)k * words;
  for (int w = 0; w < words; w++) {
    sv += __popc(act[w] & mask_word<kStaged>(&col[w]));
    uint32_t x = own[w] & mask_word<kStaged>(&row[w]);
    while (x) {
      const int b = __ffs(x) - 1;
      x &= x - 1;
      sv += mult[w * 32 + b];
    }
  }
  return sv;
}

// Nets [n0, n1) of v: active source parts into act, own nets' listed parts
// into own / mult (one warp; act, own, mult shared by the warps that call it).
__device__ void msg_scan_nets(const DevInstance& I, int v, uint32_t base, int n0, int n1, uint32_t* act,
                              uint32_t* own, int* mult) {
  const int lane = threadIdx.x & 31;
  for (int k = n0 + lane; k < n1; k += 32) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    const int s = __ldg(&I.src[e]);
    if (s == v) {
      const int sl = (int)__ldg(&I.nptr[e]);
      const int n = lds(&I.ep_len[e]);
      for (int j = 0; j < n; j++) {
        const int p = lds(&I.ep_part[sl + j]);
        if ((unsigned)p >= (unsigned)I.K) { dev_fail(I.status, kDevErrInvalid); continue; }
        atomicAdd(&mult[p], 1);
        atomicOr(&own[p >> 5], 1u << (p & 31));
      }
    } else {
      const int sp = lds(&I.part_vec[s]);
      if (sp >= 0) atomicOr(&act[sp >> 5], 1u << (sp & 31));
    }
  }
}

// Records of v's nets [n0, n1) for decision d (slot, source part, own net)
// and, with claim, the claims of the nets v appends to or is the source of.
__device__ int msg_records(const DevInstance& I, const SpecBuf& B, const StreamArgs& S, int v, uint32_t base,
                           int n0, int n1, int d, bool claim, int round, int z, int* sd) {
  const int lane = threadIdx.x & 31;
  int napp = 0;
  for (int nb = n0; nb < n1; nb += 32) {
    const int j = locate_part(I, base, nb, n1, d, sd);
    const int k = nb + lane;
    if (k < n1) {
      const int e = (int)__ldg(&I.vnets[base + k]);
      const int s = __ldg(&I.src[e]);
      const bool own = s == v;
      const int sp = own ? -1 : lds(&I.part_vec[s]);
      S.rec[base + k] = mrec(j, sp, own);
      if (claim && (j < 0 || own)) atomicMax(&B.claim64[e], skey(round, z));
    }
    napp += __popc(__ballot_sync(kAll, k < n1 && j < 0));
  }
  return napp;   // nets d is appended to, every lane
}

// The entries position z (decision d) makes positive, by the window-start
// masks: (sp, d) for active sp != d, (d, p) for own-net parts p != d; their
// rows and columns' first positions (one warp).
__device__ void msg_mark_new(const StreamArgs& S, int K, int words, int par, int z, int d, const uint32_t* act,
                             const uint32_t* own) {
  const int lane = threadIdx.x & 31;
  bool any_d_col = false, any_d_row = false;
  for (int k = lane; k < K; k += 32) {
    if (k == d) continue;
    if (bit_of(act, k) && !((__ldcg(&S.prow[(size_t)k * words + (d >> 5)]) >> (d & 31)) & 1u)) {
      atomicMin(&S.rowpos[par * K + k], z);
      any_d_col = true;
    }
    if (bit_of(own, k) && !((__ldcg(&S.prow[(size_t)d * words + (k >> 5)]) >> (k & 31)) & 1u)) {
      atomicMin(&S.colpos[par * K + k], z);
      any_d_row = true;
    }
  }
  if (__any_sync(kAll, any_d_col) && lane == 0) atomicMin(&S.colpos[par * K + d], z);
  if (__any_sync(kAll, any_d_row) && lane == 0) atomicMin(&S.rowpos[par * K + d], z);
}

__device__ __forceinline__ void set_pos_bit(const StreamArgs& S, int words, int a, int b) {
  atomicOr(&S.prow[(size_t)a * words + (b >> 5)], 1u << (b & 31));
  atomicOr(&S.pcol[(size_t)b * words + (a >> 5)], 1u << (a & 31));
}

// Commit of v's connection updates for decision d over nets [n0, n1) of the
// warp, before v's lists change.  first[K]: first net index per active part
// (filled by the caller over all of v's nets), zs[K]: conn[sp][d] was 0.
__device__ void msg_commit_act(const DevInstance& I, const StreamArgs& S, int words, int d, uint32_t base, int n0,
                               int n1, const int* first, const int* zs, int slot_override_d, int* sd) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  for (int nb = n0; nb < n1; nb += 32) {
    // d's slot: the record's, or located again (a flip committed with another part)
    const int jl = slot_override_d ? locate_part(I, base, nb, n1, d, sd) : 0;
    const int k = nb + lane;
    if (k >= n1) continue;
    const uint32_t r = lds(&S.rec[base + k]);
    const int sp = mrec_sp(r);
    if (sp < 0 || sp == d) continue;
    const bool dc1 = slot_override_d ? jl < 0 : mrec_slot(r) == (int)kNoSlot;   // d is new on the net
    const bool is_first = first[sp] == k;
    const int add = is_first ? (zs[sp] ? 1 : (dc1 ? 1 : 0)) : (dc1 ? 1 : 0);
    if (add) atomicAdd(&I.conn[(size_t)sp * K + d], add);
    if (is_first && zs[sp]) {
      atomicAdd(&I.msgs[sp], 1);
      set_pos_bit(S, words, sp, d);
    }
  }
}

__global__ void __launch_bounds__(kSThreads, 2) stream_msg_kernel(DevInstance I, SpecBuf B, StreamArgs S) {
  barrier_start();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long uscr[kSWarps];
  __shared__ int s_minpart, s_minsize, s_second, s_dec;
  __shared__ MsgKey s_best[kSWarps];
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  Carve cv{smem_raw};
  int* sizes_s = cv.take<int>(K);
  int* dsz_cta = cv.take<int>(K);
  int* a_b = cv.take<int>((size_t)K * kSWarps);        // per warp: multiplicities / sizes / first nets
  int* b_b = cv.take<int>((size_t)K * kSWarps);        // per warp: zero-start flags
  uint32_t* act_b = cv.take<uint32_t>((size_t)words * kSWarps);
  uint32_t* own_b = cv.take<uint32_t>((size_t)words * kSWarps);
  int* sd_b = cv.take<int>(32 * kSWarps);
  int* ca = cv.take<int>(K);                           // CTA: multiplicities, then first nets
  int* cb = cv.take<int>(K);                           // CTA: zero-start flags
  uint32_t* cact = cv.take<uint32_t>(words);
  uint32_t* cown = cv.take<uint32_t>(words);
  const bool staged = K <= kMsgStageK;
  uint32_t* sprow = cv.take<uint32_t>(staged ? (size_t)K * words : 0);   // the round's conn > 0 masks
  uint32_t* spcol = cv.take<uint32_t>(staged ? (size_t)K * words : 0);
  int* wa = a_b + (size_t)wib * K;
  int* wb = b_b + (size_t)wib * K;
  uint32_t* wact = act_b + (size_t)wib * words;
  uint32_t* wown = own_b + (size_t)wib * words;
  int* sd = sd_b + 32 * wib;
  const bool stats = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long t0 = stats ? gtimer() : 0ull;
  auto lap = [&](int slot) {
    if (stats) {
      const unsigned long long t = gtimer();
      B.stats[slot] += t - t0;
      t0 = t;
    }
  };

  int pos = 0, round = 1, hidx = 0;
  int W = min(nwarps, S.msg_wmax);
  while (pos < S.npos) {
    const int par = round & 1;
    for (int p = threadIdx.x; p < K; p += blockDim.x) sizes_s[p] = lds(&I.part_sizes[p]);
    if (staged)
      for (int x = threadIdx.x; x < K * words; x += blockDim.x) {
        sprow[x] = __ldcg(&S.prow[x]);
        spcol[x] = __ldcg(&S.pcol[x]);
      }
    __syncthreads();
    block_min_part(sizes_s, K, uscr, &s_minpart, &s_minsize, &s_second);
    __syncthreads();
    while (hidx < S.nheavy && __ldg(&S.heavy_pos[hidx]) < pos) hidx++;
    if (hidx < S.nheavy && __ldg(&S.heavy_pos[hidx]) == pos) {
      // ======================= a vertex with many nets: CTA 0 places it alone
      if (blockIdx.x == 0) {
        const int v = __ldg(&S.porder[pos]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        int n0, n1;
        net_range(deg, wib, kSWarps, &n0, &n1);
        for (int p = threadIdx.x; p < K; p += blockDim.x) ca[p] = 0;
        for (int x = threadIdx.x; x < words; x += blockDim.x) { cact[x] = 0; cown[x] = 0; }
        __syncthreads();
        msg_scan_nets(I, v, base, n0, n1, cact, cown, ca);
        __syncthreads();
        MsgKey best{0, 0, -1};
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
          const int sv = staged ? msg_saved<true>(sprow, spcol, words, k, cact, cown, ca)
                                : msg_saved<false>(S.prow, S.pcol, words, k, cact, cown, ca);
          if ((double)sizes_s[k] < I.C) {
            const MsgKey c{sv, sizes_s[k], k};
            if (msg_better(c, best)) best = c;
          }
        }
        best = warp_msg_best(best);
        if (lane == 0) s_best[wib] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
          MsgKey b = s_best[0];
          for (int x = 1; x < kSWarps; x++)
            if (msg_better(s_best[x], b)) b = s_best[x];
          s_dec = b.k >= 0 ? b.k : s_minpart;
        }
        __syncthreads();
        const int d = s_dec;
        // own-net messages: conn[d][p] += multiplicity, a message where it was 0
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
          const int m = ca[p];
          if (m > 0 && p != d) {
            const bool z0 = !((__ldcg(&S.prow[(size_t)d * words + (p >> 5)]) >> (p & 31)) & 1u);
            atomicAdd(&I.conn[(size_t)d * K + p], m);
            if (z0) {
              atomicAdd(&I.msgs[d], 1);
              set_pos_bit(S, words, d, p);
            }
          }
        }
        // records (no claims: the window holds this position alone)
        msg_records(I, B, S, v, base, n0, n1, d, false, round, pos, sd);
        __syncthreads();
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
          ca[p] = 0x7fffffff;
          cb[p] = p != d && !((__ldcg(&S.prow[(size_t)p * words + (d >> 5)]) >> (d & 31)) & 1u);
        }
        __syncthreads();
        for (int k = n0 + lane; k < n1; k += 32) {
          const int sp = mrec_sp(lds(&S.rec[base + k]));
          if (sp >= 0 && sp != d) atomicMin(&ca[sp], k);
        }
        __syncthreads();
        msg_commit_act(I, S, words, d, base, n0, n1, ca, cb, 0, sd);
        __syncthreads();
        for (int k = n0 + lane; k < n1; k += 32)
          place_net(I, (int)__ldg(&I.vnets[base + k]), d, mrec_slot(lds(&S.rec[base + k])));
        if (threadIdx.x == 0) {
          I.part_vec[v] = d;
          const int wv = __ldg(&I.w[v]);
          if (wv) atomicAdd(&I.part_sizes[d], wv);
        }
        if (S.niso && wib == 0) {
          int* sz = wa;
          for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p];
          __syncwarp();
          int amin = -1;
          if (pos == 0) place_iso(I, S, sz, 0, __ldg(&S.iso_before[0]), &amin);
          __syncwarp();
          const int wv = __ldg(&I.w[v]);
          if (lane == 0) sz[d] += wv;
          __syncwarp();
          amin = wv ? -1 : amin;
          place_iso(I, S, sz, __ldg(&S.iso_before[pos]), __ldg(&S.iso_before[pos + 1]), &amin);
        }
      }
      if (gtid == 0) {
        B.ctl[4 + (par ^ 1)] = kNone;
        B.ctl[2 + (par ^ 1)] = kNone;
        B.mcnt[par ^ 1] = 0;
      }
      for (int p = gtid; p < K; p += gridDim.x * blockDim.x) {
        S.rowpos[(par ^ 1) * K + p] = kNone;
        S.colpos[(par ^ 1) * K + p] = kNone;
      }
      pos++;
      round++;
      if (!grid_barrier(B.bar, I.status)) return;
      if (stats) B.stats[1]++;
      lap(19);
      continue;
    }

    // ================================================================= window
    int end_w = min(pos + W, S.npos);
    if (hidx < S.nheavy) end_w = min(end_w, (int)__ldg(&S.heavy_pos[hidx]));
    const int span = end_w - pos;
    const int q = (span + nwarps - 1) / nwarps;
    const int z0 = min(pos + gw * q, end_w);
    const int z1 = min(z0 + q, end_w);
    // ---- A: evaluate
    for (int z = z0; z < z1; z++) {
      const int o = z - pos;
      const int v = __ldg(&S.porder[z]);
      const uint32_t base = __ldg(&I.vptr[v]);
      const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
      for (int p = lane; p < K; p += 32) wa[p] = 0;
      for (int x = lane; x < words; x += 32) { wact[x] = 0; wown[x] = 0; }
      __syncwarp();
      msg_scan_nets(I, v, base, 0, deg, wact, wown, wa);
      __syncwarp();
      MsgKey best{0, 0, -1};
      int* sv_out = S.saved + (size_t)o * K;
      for (int k = lane; k < K; k += 32) {
        const int sv = staged ? msg_saved<true>(sprow, spcol, words, k, wact, wown, wa)
                              : msg_saved<false>(S.prow, S.pcol, words, k, wact, wown, wa);
        sv_out[k] = sv;
        if ((double)sizes_s[k] < I.C) {
          const MsgKey c{sv, sizes_s[k], k};
          if (msg_better(c, best)) best = c;
        }
      }
      best = warp_msg_best(best);
      const int d = best.k >= 0 ? best.k : s_minpart;
      const int napp = msg_records(I, B, S, v, base, 0, deg, d, true, round, z, sd);
      msg_mark_new(S, K, words, par, z, d, wact, wown);
      for (int x = lane; x < words; x += 32) {
        S.actm[(size_t)o * words + x] = wact[x];
        S.ownm[(size_t)o * words + x] = wown[x];
      }
      const int wv = __ldg(&I.w[v]);
      if (lane == 0) {
        B.dec[o] = d;
        B.wt[o] = wv;
        B.flag[o] = 0;
        B.slack[o] = napp;
        if (wv) {
          const int i = atomicAdd(&B.mcnt[par], 1);
          B.mlist[i] = make_int4(o, wv, d, 0);
          B.midx[o] = i;
        }
      }
      __syncwarp();
    }
    if (!grid_barrier(B.bar, I.status)) return;
    lap(16);
    // ---- B: validate, as in the LDG stream: B1 finds the first conflict
    // (claims, or a row / column an earlier position makes positive) and the
    // first decision that changes with the exact sizes; B2 walks from that
    // change to the conflict on one warp, taking each change whose appends are
    // a subset of the old decision's, and stopping at a position that reads a
    // row or column a taken change makes positive.
    int* const cut_w = &B.ctl[4 + par];
    int* const flip_w = &B.ctl[2 + par];
    const int cz0 = min(pos + blockIdx.x * kSWarps * q, end_w);
    const int cta_o0 = cz0 - pos;
    {
      for (int p = threadIdx.x; p < K; p += blockDim.x) dsz_cta[p] = 0;
      __syncthreads();
      const int nm = lds(&B.mcnt[par]);
      for (int i = threadIdx.x; i < nm; i += blockDim.x) {
        const int4 m = lds(&B.mlist[i]);
        if (m.x < cta_o0) atomicAdd(&dsz_cta[m.z], m.y);
      }
      __syncthreads();
      bool decided = false;
      for (int z = z0; z < z1; z++) {
        const int o = z - pos;
        const int v = __ldg(&S.porder[z]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        bool conf = false;
        for (int k = lane; k < deg && !conf; k += 32)
          conf = claimed_before(B, round, (int)__ldg(&I.vnets[base + k]), z);
        for (int k = lane; k < K && !conf; k += 32) {
          if (bit_of(S.actm + (size_t)o * words, k) && lds(&S.rowpos[par * K + k]) < z) conf = true;
          if (bit_of(S.ownm + (size_t)o * words, k) && lds(&S.colpos[par * K + k]) < z) conf = true;
        }
        if (__any_sync(kAll, conf)) {
          if (lane == 0) atomicMin(cut_w, (z << 3) | 5);
          break;
        }
        if (decided) continue;
        int* dsz = wa;
        for (int p = lane; p < K; p += 32) dsz[p] = dsz_cta[p];
        __syncwarp();
        for (int o2 = cta_o0 + lane; o2 < o; o2 += 32) {
          const int w = lds(&B.wt[o2]);
          if (w) atomicAdd(&dsz[lds(&B.dec[o2])], w);
        }
        __syncwarp();
        MsgKey best{0, 0, -1};
        const int* sv_in = S.saved + (size_t)o * K;
        for (int k = lane; k < K; k += 32) {
          const int sz = sizes_s[k] + dsz[k];
          if ((double)sz < I.C) {
            const MsgKey c{lds(&sv_in[k]), sz, k};
            if (msg_better(c, best)) best = c;
          }
        }
        best = warp_msg_best(best);
        const int d2 = best.k >= 0 ? best.k : least_loaded(sizes_s, dsz, K);
        if (d2 != lds(&B.dec[o])) {
          if (lane == 0) atomicMin(flip_w, (z << 3) | 2);
          decided = true;
        }
        __syncwarp();
      }
    }
    if (!grid_barrier(B.bar, I.status)) return;
    lap(17);
    const int cutw = lds(cut_w), flipw = lds(flip_w);
    const int zc = cutw == kNone ? end_w : min(cutw >> 3, end_w);
    const int zf = flipw == kNone ? end_w : min(flipw >> 3, end_w);
    int cut = zc, cutc = zc;
    if (zf < zc) {
      if (blockIdx.x == 0 && wib == 0) {
        int* sz = wa;
        uint32_t* rows_new = wact;   // rows / columns a taken change makes positive
        uint32_t* cols_new = wown;
        for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p];
        for (int x = lane; x < words; x += 32) { rows_new[x] = 0; cols_new[x] = 0; }
        __syncwarp();
        const int nm = lds(&B.mcnt[par]);
        for (int i = lane; i < nm; i += 32) {
          const int4 m = lds(&B.mlist[i]);
          if (m.x < zf - pos) atomicAdd(&sz[m.z], m.y);
        }
        __syncwarp();
        int c1 = zc, c2 = zc;
        bool stop = false, reclaim = false;
        constexpr int kSv = kMsgStageK / 32;   // saved values a lane prefetches (K <= kMsgStageK)
        // 32 positions at a time: their scalar words one per lane; the next
        // position's saved messages loaded while one is decided (K <= 256)
        for (int zb = zf; zb < zc && !stop; zb += 32) {
          const int zl = zb + lane, ol = zl - pos;
          const bool in = zl < zc;
          const int d_l = in ? lds(&B.dec[ol]) : 0;
          const int w_l = in ? lds(&B.wt[ol]) : 0;
          const int na_l = in ? lds(&B.slack[ol]) : 0;
          int deg_l = 0, v_l = 0;
          if (in) {
            v_l = __ldg(&S.porder[zl]);
            deg_l = (int)(__ldg(&I.vptr[v_l + 1]) - __ldg(&I.vptr[v_l]));
          }
          const int nb = min(32, zc - zb);
          int sv[kSv], svn[kSv];
#pragma unroll
          for (int u = 0; u < kSv; u++) {
            const int k = lane + 32 * u;
            sv[u] = staged && k < K ? lds(&S.saved[(size_t)(zb - pos) * K + k]) : 0;
          }
          for (int j = 0; j < nb; j++) {
            const int z = zb + j, o = z - pos;
            const int d = __shfl_sync(kAll, d_l, j);
            const int w = __shfl_sync(kAll, w_l, j);
            const int napp = __shfl_sync(kAll, na_l, j);
            const int deg = __shfl_sync(kAll, deg_l, j);
            const int vz = __shfl_sync(kAll, v_l, j);
#pragma unroll
            for (int u = 0; u < kSv; u++) {
              const int k = lane + 32 * u;
              svn[u] = staged && k < K && j + 1 < nb ? lds(&S.saved[(size_t)(o + 1) * K + k]) : 0;
            }
            const uint32_t* am = S.actm + (size_t)o * words;
            const uint32_t* om = S.ownm + (size_t)o * words;
            bool conf = false;
            for (int x = lane; x < words; x += 32)
              if ((lds(&am[x]) & rows_new[x]) || (lds(&om[x]) & cols_new[x])) conf = true;
            if (__any_sync(kAll, conf) || (reclaim && conflicts_now(I, B, vz, round, z))) {
              c1 = c2 = z;
              stop = true;
              break;
            }
            MsgKey best{0, 0, -1};
            if (staged) {
#pragma unroll
              for (int u = 0; u < kSv; u++) {
                const int k = lane + 32 * u;
                if (k < K && (double)sz[k] < I.C) {
                  const MsgKey c{sv[u], sz[k], k};
                  if (msg_better(c, best)) best = c;
                }
              }
            } else {
              const int* sv_in = S.saved + (size_t)o * K;
              for (int k = lane; k < K; k += 32)
                if ((double)sz[k] < I.C) {
                  const MsgKey c{lds(&sv_in[k]), sz[k], k};
                  if (msg_better(c, best)) best = c;
                }
            }
            best = warp_msg_best(best);
            const int d2 = best.k >= 0 ? best.k : least_loaded(sz, nullptr, K);
#pragma unroll
            for (int u = 0; u < kSv; u++) sv[u] = svn[u];
            if (d2 != d) {
              if (napp != deg) {   // new appends: claimed; later positions check them
                claim_appends(I, B, vz, round, z, d2, sd);
                reclaim = true;
              }
              bool ncol = false, nrow = false;
              for (int k = lane; k < K; k += 32) {
                if (k == d2) continue;
                if (((lds(&am[k >> 5]) >> (k & 31)) & 1u) &&
                    !((__ldcg(&S.prow[(size_t)k * words + (d2 >> 5)]) >> (d2 & 31)) & 1u)) {
                  atomicOr(&rows_new[k >> 5], 1u << (k & 31));
                  ncol = true;
                }
                if (((lds(&om[k >> 5]) >> (k & 31)) & 1u) &&
                    !((__ldcg(&S.prow[(size_t)d2 * words + (k >> 5)]) >> (k & 31)) & 1u)) {
                  atomicOr(&cols_new[k >> 5], 1u << (k & 31));
                  nrow = true;
                }
              }
              const bool any_c = __any_sync(kAll, ncol), any_r = __any_sync(kAll, nrow);
              if (lane == 0) {
                if (any_c) atomicOr(&cols_new[d2 >> 5], 1u << (d2 & 31));
                if (any_r) atomicOr(&rows_new[d2 >> 5], 1u << (d2 & 31));
                B.dec[o] = d2;
                B.flag[o] = 1;
                if (w) B.mlist[lds(&B.midx[o])].z = d2;
                B.stats[9]++;
              }
            }
            __syncwarp();
            if (lane == 0 && w) sz[d2] += w;
            __syncwarp();
          }
        }
        if (lane == 0) {
          B.ctl[6] = c1;
          B.ctl[7] = c2;
        }
      }
      if (!grid_barrier(B.bar, I.status)) return;
      lap(20);
      cut = lds(&B.ctl[6]);
      cutc = lds(&B.ctl[7]);
      for (int p = threadIdx.x; p < K; p += blockDim.x) dsz_cta[p] = 0;
      __syncthreads();
      const int nm = lds(&B.mcnt[par]);
      for (int i = threadIdx.x; i < nm; i += blockDim.x) {
        const int4 m = lds(&B.mlist[i]);
        if (m.x < cta_o0) atomicAdd(&dsz_cta[m.z], m.y);
      }
      __syncthreads();
    }
    if (cut <= pos) {
      if (gtid == 0) dev_fail(I.status, kDevErrInvalid);
      return;
    }
    // ---- C: commit
    for (int z = z0; z < min(z1, cutc); z++) {
      const int o = z - pos;
      const int v = __ldg(&S.porder[z]);
      const uint32_t base = __ldg(&I.vptr[v]);
      const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
      const bool fl = z == cut || lds(&B.flag[o]);   // records of another part: located again
      const int d = z == cut ? lds(&B.dfix[o]) : lds(&B.dec[o]);
      // own-net messages from the window-start lists (before v's placement)
      for (int p = lane; p < K; p += 32) wa[p] = 0;
      for (int x = lane; x < words; x += 32) { wact[x] = 0; wown[x] = 0; }
      __syncwarp();
      for (int k = lane; k < deg; k += 32) {
        const uint32_t r = lds(&S.rec[base + k]);
        if (!mrec_own(r)) continue;
        const int e = (int)__ldg(&I.vnets[base + k]);
        const int sl = (int)__ldg(&I.nptr[e]);
        const int n = lds(&I.ep_len[e]);
        for (int j = 0; j < n; j++) {
          const int pp = lds(&I.ep_part[sl + j]);
          if ((unsigned)pp < (unsigned)K) atomicAdd(&wa[pp], 1);
        }
      }
      __syncwarp();
      for (int p = lane; p < K; p += 32) {
        const int m = wa[p];
        if (m > 0 && p != d) {
          const bool z0b = !((__ldcg(&S.prow[(size_t)d * words + (p >> 5)]) >> (p & 31)) & 1u);
          atomicAdd(&I.conn[(size_t)d * K + p], m);
          if (z0b) {
            atomicAdd(&I.msgs[d], 1);
            set_pos_bit(S, words, d, p);
          }
        }
      }
      __syncwarp();
      // active-source messages: first net per source part, zero-start flags
      for (int p = lane; p < K; p += 32) {
        wa[p] = 0x7fffffff;
        wb[p] = p != d && !((__ldcg(&S.prow[(size_t)p * words + (d >> 5)]) >> (d & 31)) & 1u);
      }
      __syncwarp();
      for (int k = lane; k < deg; k += 32) {
        const int sp = mrec_sp(lds(&S.rec[base + k]));
        if (sp >= 0 && sp != d) atomicMin(&wa[sp], k);
      }
      __syncwarp();
      msg_commit_act(I, S, words, d, base, 0, deg, wa, wb, fl ? 1 : 0, sd);
      __syncwarp();
      if (fl) {
        for (int nb = 0; nb < deg; nb += 32) {
          const int j = locate_part(I, base, nb, deg, d, sd);
          if (nb + lane < deg) place_net(I, (int)__ldg(&I.vnets[base + nb + lane]), d, j);
        }
      } else {
        for (int k = lane; k < deg; k += 32)
          place_net(I, (int)__ldg(&I.vnets[base + k]), d, mrec_slot(lds(&S.rec[base + k])));
      }
      if (lane == 0) {
        I.part_vec[v] = d;
        const int wv = lds(&B.wt[o]);
        if (wv) atomicAdd(&I.part_sizes[d], wv);
      }
      __syncwarp();
    }
    if (S.niso) {
      const int zb = min(z1, cutc);
      if (z0 < zb || (pos == 0 && gw == 0)) {
        const int cta_o0 = min(pos + blockIdx.x * kSWarps * q, end_w) - pos;
        int* sz = wa;
        for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p] + dsz_cta[p];
        __syncwarp();
        for (int o2 = cta_o0 + lane; o2 < z0 - pos; o2 += 32) {
          const int w = lds(&B.wt[o2]);
          if (w) atomicAdd(&sz[lds(&B.dec[o2])], w);
        }
        __syncwarp();
        int amin = -1;
        if (pos == 0 && gw == 0) place_iso(I, S, sz, 0, __ldg(&S.iso_before[0]), &amin);
        for (int z = z0; z < zb; z++) {
          const int o = z - pos;
          const int w = lds(&B.wt[o]);
          if (w) {
            __syncwarp();
            if (lane == 0) sz[z == cut ? lds(&B.dfix[o]) : lds(&B.dec[o])] += w;
            __syncwarp();
            amin = -1;
          }
          place_iso(I, S, sz, __ldg(&S.iso_before[z]), __ldg(&S.iso_before[z + 1]), &amin);
        }
      }
    }
    if (gtid == 0) {
      B.ctl[4 + (par ^ 1)] = kNone;
      B.ctl[2 + (par ^ 1)] = kNone;
      B.mcnt[par ^ 1] = 0;
    }
    for (int p = gtid; p < K; p += gridDim.x * blockDim.x) {
      S.rowpos[(par ^ 1) * K + p] = kNone;
      S.colpos[(par ^ 1) * K + p] = kNone;
    }
    if (stats) {
      B.stats[0]++;
      B.stats[2] += cutc - pos;
      if (cutc > cut) B.stats[5]++;
      else if (cut < end_w) B.stats[8]++;
    }
    if (cutc >= end_w) {
      if (end_w == pos + W) W = min(2 * W, S.msg_wmax);
    } else {
      W = min(S.msg_wmax, max(256, 2 * (cutc - pos)));
    }
    pos = cutc;
    round++;
    if (!grid_barrier(B.bar, I.status)) return;
    lap(18);
  }
}

// The refinement's masks of the streamed connection counts: zero and one, by
// row and by column.
__global__ void stream_conn_masks_kernel(DevInstance I) {
  const int K = I.K;
  const int words = (K + 31) >> 5;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < (long long)K * words;
       x += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(x / words), w = (int)(x % words);
    uint32_t zr = 0, zc = 0, c1r = 0, c1c = 0;
    for (int b = 0; b < 32; b++) {
      const int k = w * 32 + b;
      if (k >= K) break;
      const int r = I.conn[(size_t)a * K + k];   // row a, column k
      const int c = I.conn[(size_t)k * K + a];   // column a, row k
      if (r == 0) zr |= 1u << b;
      if (r == 1) c1r |= 1u << b;
      if (c == 0) zc |= 1u << b;
      if (c == 1) c1c |= 1u << b;
    }
    I.zrow[x] = zr;
    I.zcol[x] = zc;
    I.c1row[x] = c1r;
    I.c1col[x] = c1c;
  }
}

}  // namespace

size_t stream_smem_bytes(int K) {
  auto a = [](size_t n) { return (n + 15) & ~size_t(15); };
  return 2 * a(sizeof(int) * K) + a(sizeof(int) * (size_t)K * kSWarps) +
         a(sizeof(unsigned long long) * (size_t)K * kSWarps) + a(sizeof(int) * 32 * kSWarps);
}

size_t stream_msg_smem_bytes(int K) {
  auto a = [](size_t n) { return (n + 15) & ~size_t(15); };
  const size_t words = (size_t)(K + 31) / 32;
  return 2 * a(sizeof(int) * K) + 2 * a(sizeof(int) * (size_t)K * kSWarps) + 2 * a(sizeof(uint32_t) * words * kSWarps) +
         a(sizeof(int) * 32 * kSWarps) + 2 * a(sizeof(int) * K) + 2 * a(sizeof(uint32_t) * words) +
         (K <= kMsgStageK ? 2 * a(sizeof(uint32_t) * K * words) : 0);
}

cudaError_t launch_stream_msg(const DevInstance& I, const SpecBuf& B, const StreamArgs& S, int num_sms,
                              cudaStream_t st) {
  const size_t smem = stream_msg_smem_bytes(I.K);
  const void* fn = (const void*)stream_msg_kernel;
  cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSThreads, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = per_sm * num_sms;
  if (grid * kSWarps > B.max_warps) grid = B.max_warps / kSWarps;
  DevInstance Ic = I;
  SpecBuf Bc = B;
  StreamArgs Sc = S;
  void* args[] = {&Ic, &Bc, &Sc};
  err = cudaLaunchCooperativeKernel(fn, grid, kSThreads, args, smem, st);
  if (err != cudaSuccess) return err;
  const long long n = (long long)I.K * ((I.K + 31) / 32);
  stream_conn_masks_kernel<<<(int)std::min<long long>((n + 255) / 256, (long long)num_sms * 8), 256, 0, st>>>(I);
  return cudaGetLastError();
}

cudaError_t launch_stream_ldg(const DevInstance& I, const SpecBuf& B, const StreamArgs& S, int num_sms,
                              cudaStream_t st) {
  const size_t smem = stream_smem_bytes(I.K);
  const void* fn = (const void*)stream_ldg_kernel;
  cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSThreads, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = per_sm * num_sms;
  if (grid * kSWarps > B.max_warps) grid = B.max_warps / kSWarps;
  DevInstance Ic = I;
  SpecBuf Bc = B;
  StreamArgs Sc = S;
  void* args[] = {&Ic, &Bc, &Sc};
  err = cudaLaunchCooperativeKernel(fn, grid, kSThreads, args, smem, st);
  if (err != cudaSuccess) return err;
  if (I.metric == kMSV || I.metric == kMSRV) {
    stream_volumes_kernel<<<num_sms * 4, 256, 0, st>>>(I, I.metric == kMSRV ? 1 : 0);
    err = cudaGetLastError();
  }
  return err;
}

}  // namespace fp
