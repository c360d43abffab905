// Speculative grid-wide refinement for the LDG metrics: TV (TV/partition.cpp:
// 307-440), MSV (MGV/partition.cpp:222-477) and MSRV (MSRV/partition.cpp:240-517).
//
// The reference walks the vertices one by one; every decision reads the state
// left by all earlier moves.  Here one persistent cooperative kernel runs all
// passes as a sequence of rounds.  A round covers a window of the next vertices
// in visiting order:
//
//   A  evaluate   every warp of the grid decides its vertices against the
//                 current state, as if each were next.  A mover claims its nets
//                 (part-set-changing or count-only), and every vertex records
//                 how much part-size / volume drift its outcome tolerates.
//   B  validate   a vertex keeps its outcome iff nothing it read can have
//                 changed: no earlier mover of the window changed the part set
//                 of one of its nets, or the count of its own part there; the
//                 weight moved before it stays within its size slack (the LDG
//                 argmax, its tie-breaks and TV's clamps cannot flip); the
//                 volumes stay within its volume slack; if it would leave its
//                 part, no earlier mover touched a max-volume part; for TV, no
//                 stale marker can apply.  The first invalid position cuts the
//                 window (MSV / MSRV fix a position whose decision the size
//                 drift flipped in place and validate again from it).
//   C  commit     all movers before the cut are applied at once -- on any net
//                 they either are alone or only shift counts, which commute --
//                 and the next window starts at the cut.
//
// Every committed outcome therefore equals the reference's sequential outcome.
//
// A mover's slots (own part, destination) in each of its nets' lists are found
// once, by a flattened pass over the slots (locate_batch), and recorded per
// (vertex, net); the gain / loss terms and the commit then take O(1) per net.
// Vertices are classed by work (list slots over their nets, host-side): light
// ones are evaluated by one warp, medium ones by one CTA, and the heaviest (up
// to gmax per window) by all warps of the grid, which split the tally, the gain
// / loss sums and the move in two extra grid phases of the window.

#include "fp_spec_common.cuh"

namespace fp {

namespace {

using namespace spec;

constexpr int kTV = 1, kMSV = 4, kMSRV = 5;
constexpr int kBig = 1000000000;

struct RoundCtx {
  const int* sizes;
  const float* penf;   // 1 - size / C in float (off by < 4e-7 * (1 + size / C))
  const int* marker;
  const int* vol;
  const int* mark;
  int minpart, minsize, second, maxv, cc;
  float Cf;            // C rounded to float
};

// LDG argmax over the tallied parts (TV/partition.cpp:98-145 with TV's clamps,
// MGV/partition.cpp:28-65 without), executed by one warp, plus the part-size
// drift under which the outcome cannot change.
//
// Scores are first formed in float from the float penalty 1 - size / C, which
// is off by less than 4e-7 * (1 + size / C); a score of count c is bounded
// within tol = 1e-6 * c * (1 + |size / C|).  The exact double score (the
// reference's arithmetic) and the tie-breaks are then evaluated only for parts
// whose upper bound reaches the largest lower bound: a set that holds the
// exact argmax and all its ties.  The slack bounds use lower bounds of the
// score gaps (a low bound only costs an exact re-check).
__device__ __forceinline__ float score_tol(int c, float pf) { return (float)c * 1e-6f * (1.0f + fabsf(1.0f - pf)); }
__device__ __forceinline__ int slack_divf(float a, float b) {
  const float x = __fdiv_rn(a, b) * (1.0f - 1e-5f) - 1.0f;
  if (!(x > -1.0f)) return -1;
  if (x > 1.0e9f) return kBig;
  return (int)floorf(x);
}

// Candidate entry of a part for the exact re-check: part (12 bits), count
// without the vertex itself (16 bits), first sighting (net index, 16 bits;
// slot, 20 bits).  A vertex whose count or first net index does not fit (one
// with 65536 nets or more) stores no list: ncand = -1.
__device__ __forceinline__ unsigned long long cand_entry(int p, int c, unsigned long long f) {
  return ((unsigned long long)p << 52) | ((unsigned long long)c << 36) | (((f >> 32) & 0xffffull) << 20) |
         (f & 0xfffffull);
}

// One warp.  The tallied parts (count > 0, no stale TV marker) are first
// compacted, in ascending order, into list (K ints of warp scratch); cand /
// *ncand (if cand is not null) receive their re-check entries and scan (if not
// null) TV's scanned-part bits.  The bound, exact and slack passes then walk
// only the compacted parts.
__device__ int ldg_decide(const DevInstance& I, const RoundCtx& R, const int* cnt, const unsigned long long* first,
                          int metric, int v, int own, bool first_of_window, int* list, unsigned long long* cand,
                          int* ncand, uint32_t* scan, bool* special, int* slack_out) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int K = I.K;
  const bool tv = metric == kTV;
  int nc = 0;
  bool sp = false, wide = false;
#pragma unroll 4
  for (int p0 = 0; p0 < K; p0 += 32) {
    const int p = p0 + lane;
    const int c = p < K ? cnt[p] : 0;
    const bool stale = tv && c > 0 && R.marker[p] == v;
    sp |= stale;
    const bool ok = c > 0 && !stale;
    const unsigned m = __ballot_sync(kAll, ok);
    if (ok) {
      const int i = nc + __popc(m & below);
      list[i] = p;
      if (cand) {
        const unsigned long long f = first[p];
        wide |= c > 0xffff || (f >> 32) > 0xffffull;
        cand[i] = cand_entry(p, c - (p == own ? 1 : 0), f);
      }
    }
    if (scan) {
      const unsigned ms = __ballot_sync(kAll, c > 0);
      if (lane == 0) scan[p0 >> 5] = ms;
    }
    nc += __popc(m);
  }
  wide = __any_sync(kAll, wide);
  if (cand && lane == 0) *ncand = wide ? -1 : nc;
  *special = __any_sync(kAll, sp) && !first_of_window;
  __syncwarp();
  float fb = 0.0f;   // largest lower bound of a score (0: none positive for sure)
  bool any = false;
  for (int i = lane; i < nc; i += 32) {
    const int p = list[i];
    const int cc = cnt[p] - (p == own ? 1 : 0);
    if (cc > 0) {
      const float pf = R.penf[p];
      const float f = __fmul_rn((float)cc, pf), t = score_tol(cc, pf);
      fb = fmaxf(fb, f - t);
      any |= f + t > 0.0f;
    }
  }
  for (int off = 16; off; off >>= 1) fb = fmaxf(fb, __shfl_xor_sync(kAll, fb, off));
  LdgKey best{-1.0, 0, -1, ~0ull};
  float sbest = 0.0f;   // a lower bound of the winner's exact score, in float
  if (__any_sync(kAll, any)) {
    // Parts whose upper bound reaches the largest lower bound: the argmax and
    // all its ties are among them.  A single one with a positive lower bound
    // is the argmax outright (every other score lies below fb); otherwise the
    // exact double scores (TV/partition.cpp:103-104) and tie-breaks decide.
    int nnear = 0, np = -1;
    float nlo = 0.0f;
    for (int i = lane; i < nc; i += 32) {
      const int p = list[i];
      const int cc = cnt[p] - (p == own ? 1 : 0);
      if (cc <= 0) continue;
      const float pf = R.penf[p];
      const float f = __fmul_rn((float)cc, pf), t = score_tol(cc, pf);
      if (!(f + t > 0.0f) || f + t < fb) continue;
      nnear++;
      np = p;
      nlo = f - t;
    }
    const int tot = __reduce_add_sync(kAll, nnear);
    const unsigned hn = __ballot_sync(kAll, nnear > 0);
    const int src = __ffs(hn) - 1;
    const float lo1 = __shfl_sync(kAll, nlo, src);
    if (tot == 1 && lo1 > 0.0f) {
      best.part = __shfl_sync(kAll, np, src);
      sbest = lo1;
    } else {
      for (int i = lane; i < nc; i += 32) {
        const int p = list[i];
        const int cc = cnt[p] - (p == own ? 1 : 0);
        if (cc <= 0) continue;
        const float pf = R.penf[p];
        const float f = __fmul_rn((float)cc, pf), t = score_tol(cc, pf);
        if (!(f + t > 0.0f) || f + t < fb) continue;   // cannot be a positive best
        const double pen = __dsub_rn(1.0, __ddiv_rn((double)R.sizes[p], I.C));   // TV/partition.cpp:103-104
        LdgKey k{__dmul_rn((double)cc, pen), R.sizes[p], p, first[p]};
        if (ldg_better(k, best)) best = k;
      }
      best = warp_ldg_argmax(best);
      sbest = (float)best.score;
    }
  }
  const int d0 = best.part >= 0 ? best.part : R.minpart;
  int d = d0;
  if (tv) {
    if (R.sizes[d] > I.max_pw) d = own;
    if (R.sizes[d] < I.min_pw) d = own;
  }
  // Drift margins: every part's size may move by at most D.  All conditions are
  // monotone in D.
  int sl = kBig;
  const float Cf = R.Cf;
  if (best.part >= 0) {
    const int w = best.part;
    const int cw = cnt[w] - (w == own ? 1 : 0);
    const float Swf = sbest;
    sl = min(sl, slack_divf(Swf * (1.0f - 1e-6f) * Cf, (float)cw) - 1);   // stays positive
    for (int i = lane; i < nc; i += 32) {
      const int q = list[i];
      if (q == w) continue;
      const int cq = cnt[q] - (q == own ? 1 : 0);
      if (cq <= 0) continue;
      const float pq = R.penf[q];
      const float fq = __fmul_rn((float)cq, pq) + score_tol(cq, pq);   // above the exact score
      const float diff = Swf - fq - 1e-6f * (fabsf(Swf) + fabsf(fq));   // below the exact gap
      if (!(diff > 0.0f)) { sl = -1; continue; }                       // (near) tie: size / order decide
      sl = min(sl, slack_divf(diff * Cf, (float)(cw + cq)) - 1);
    }
  } else {
    for (int i = lane; i < nc; i += 32) {
      const int q = list[i];
      if (cnt[q] - (q == own ? 1 : 0) <= 0) continue;
      // size - C, shrunk past float rounding of C
      const float x = (float)R.sizes[q] - Cf - 1e-6f * Cf - 1.0f;
      sl = min(sl, (!(x > -1.0f) ? -1 : x > 1.0e9f ? kBig : (int)floorf(x)) - 1);   // stays non-positive
    }
    sl = min(sl, (R.second - R.minsize - 1) / 2);                 // least-loaded part stays
  }
  if (tv) {
    const int s0 = R.sizes[d0];
    sl = min(sl, s0 > I.max_pw ? s0 - I.max_pw - 1 : I.max_pw - s0);
    const int d1 = s0 > I.max_pw ? own : d0;
    const int s1 = R.sizes[d1];
    sl = min(sl, s1 < I.min_pw ? I.min_pw - s1 - 1 : s1 - I.min_pw);
  }
  sl = warp_min(sl);
  *slack_out = max(sl, -1);
  return d;
}

// The LDG decision of the vertex at window offset o again, from its stored
// candidates and the exact part sizes at that position: round-start sizes plus
// the moves of the window's movers before o -- those before offset o_from
// already summed per part in dsz_cta (the CTA's share), the rest read from the
// window records -- gathered in the warp's K-int scratch dsz.  One warp.
// Returns -1 if the vertex has no candidate list (65536 nets or more).
__device__ int ldg_recheck(const DevInstance& I, const RoundCtx& R, const SpecBuf& B, int o, int own, int metric,
                           int* dsz, const int* dsz_cta, int o_from) {
  const int lane = threadIdx.x & 31;
  const int K = I.K;
  for (int p = lane; p < K; p += 32) dsz[p] = dsz_cta[p];
  __syncwarp();
  for (int o2 = o_from + lane; o2 < o; o2 += 32) {
    const int w = lds(&B.wt[o2]);   // 0 unless a mover
    const int pk = lds(&B.dec[o2]);
    if (w == 0) continue;
    atomicAdd(&dsz[pk & 0xffff], w);
    atomicAdd(&dsz[pk >> 16], -w);
  }
  __syncwarp();
  const unsigned long long* cl = B.cand + (size_t)o * K;
  const int nc = lds(&B.ncand[o]);
  if (nc < 0) return -1;   // no list (65536 nets or more): the caller cuts
  // Float scores first: the float penalty 1 - sz / C is off by less than
  // 4e-7 * (1 + sz / C), so a score of count c by less than c times that; the
  // bound used is 1e-6 * c * (1 + sz / C).  Exact double scores only for
  // candidates whose upper bound reaches the largest lower bound.
  const float Cf = R.Cf;
  float fb = 0.0f;
  for (int i = lane; i < nc; i += 32) {
    const unsigned long long ent = lds(&cl[i]);
    const int p = (int)(ent >> 52);
    const int c = (int)((ent >> 36) & 0xffffull);
    const float xf = __fdiv_rn((float)(R.sizes[p] + dsz[p]), Cf);
    fb = fmaxf(fb, __fmul_rn((float)c, 1.0f - xf) - (float)c * 1e-6f * (1.0f + fabsf(xf)));
  }
  for (int off = 16; off; off >>= 1) fb = fmaxf(fb, __shfl_xor_sync(kAll, fb, off));
  // a single part reaching fb > 0 is the argmax outright (as in ldg_decide)
  int nnear = 0, np = -1;
  for (int i = lane; i < nc; i += 32) {
    const unsigned long long ent = lds(&cl[i]);
    const int p = (int)(ent >> 52);
    const int c = (int)((ent >> 36) & 0xffffull);
    const float xf = __fdiv_rn((float)(R.sizes[p] + dsz[p]), Cf);
    if (__fmul_rn((float)c, 1.0f - xf) + (float)c * 1e-6f * (1.0f + fabsf(xf)) < fb) continue;   // cannot be best
    nnear++;
    np = p;
  }
  LdgKey best{-1.0, 0, -1, ~0ull};
  if (fb > 0.0f && __reduce_add_sync(kAll, nnear) == 1) {
    best.part = __shfl_sync(kAll, np, __ffs(__ballot_sync(kAll, nnear > 0)) - 1);
  } else {
    for (int i = lane; i < nc; i += 32) {
      const unsigned long long ent = lds(&cl[i]);
      const int p = (int)(ent >> 52);
      const int c = (int)((ent >> 36) & 0xffffull);
      const int sz = R.sizes[p] + dsz[p];
      const float xf = __fdiv_rn((float)sz, Cf);
      if (__fmul_rn((float)c, 1.0f - xf) + (float)c * 1e-6f * (1.0f + fabsf(xf)) < fb) continue;   // cannot be best
      const unsigned long long f = (((ent >> 20) & 0xffffull) << 32) | (ent & 0xfffffull);
      const double pen = __dsub_rn(1.0, __ddiv_rn((double)sz, I.C));
      LdgKey k{__dmul_rn((double)c, pen), sz, p, f};
      if (ldg_better(k, best)) best = k;
    }
    best = warp_ldg_argmax(best);
  }
  int d0 = best.part;
  if (d0 < 0) {
    unsigned long long mk = ~0ull;
    for (int p = lane; p < K; p += 32) {
      const int sz = R.sizes[p] + dsz[p];
      const unsigned long long key = ((unsigned long long)((unsigned)sz ^ 0x80000000u) << 32) | (unsigned)p;
      mk = key < mk ? key : mk;
    }
    for (int off = 16; off; off >>= 1) {
      const unsigned long long x = __shfl_xor_sync(kAll, mk, off);
      mk = x < mk ? x : mk;
    }
    d0 = (int)(mk & 0xffffffffu);
  }
  int d = d0;
  if (metric == kTV) {
    if (R.sizes[d] + dsz[d] > I.max_pw) d = own;
    if (R.sizes[d] + dsz[d] < I.min_pw) d = own;
  }
  __syncwarp();
  return d;
}

// The reference's gains / losses of the move own -> d on net e
// (MGV/partition.cpp:294-337, MSRV/partition.cpp:303-350) and the exact change
// of every part's volume that commit_rec will make (adelta), from the net's
// record r.
__device__ __forceinline__ void net_terms(const DevInstance& I, bool rv, int v, int own, int d, int e, uint32_t r,
                                          int* gains, int* losses, int* adelta) {
  const int n = lds(&I.ep_len[e]);
  const bool rem = rec_rem(r), add = rec_add(r);
  const int sv = __ldg(&I.src[e]);
  const int sp = sv == v ? own : lds(&I.part_vec[sv]);
  if (sv == v) {
    atomicAdd(&gains[own], n - 1);
    atomicAdd(&losses[d], n - 1);
  }
  if (rem) {
    if (sv != v) {
      atomicAdd(&gains[sp], 1);
      if (rv) atomicAdd(&gains[own], 1);
    } else {
      atomicAdd(&losses[d], -1);
    }
  }
  if (add) {
    if (sv != v) {
      atomicAdd(&losses[sp], 1);
      if (rv) atomicAdd(&losses[d], 1);
    } else {
      atomicAdd(&losses[d], 1);
    }
  }
  const int n1 = rem ? n - 1 : n;
  if (sv == v) {
    atomicAdd(&adelta[own], -(n - 1));
    atomicAdd(&adelta[d], n1 - 1);
  }
  if (rem) {
    if (sv != v) {
      atomicAdd(&adelta[sp], -1);
      if (rv) atomicAdd(&adelta[own], -1);
    }
  } else if (rv && sv == v) {
    atomicAdd(&adelta[own], 1);
  }
  if (!add) {
    if (rv && sv == v) atomicAdd(&adelta[d], -1);
  } else {
    atomicAdd(&adelta[sv == v ? d : sp], 1);
    if (rv && sv != v) atomicAdd(&adelta[d], 1);
  }
}

// Records of v's nets for the move own -> d; warp wi of a group of nw warps
// takes a contiguous share of the nets (net_range).  With volumes (MSV / MSRV) the
// gain / loss / volume terms are added to the warp's arrays.  loc: the warp's
// 96 ints of scratch.
__device__ void locate_all(const DevInstance& I, const SpecBuf& B, int metric, int v, int own, int d,
                           uint32_t base, int deg, int wi, int nw, int* loc, int* gains, int* losses, int* adelta) {
  const bool vol = metric != kTV, rv = metric == kMSRV;
  int n0, n1;
  net_range(deg, wi, nw, &n0, &n1);
  for (int nb = n0; nb < n1; nb += 32) {
    int e;
    const uint32_t r = locate_batch(I, B.rec, v, own, d, base, nb, n1, loc, loc + 32, loc + 64, &e);
    if (vol && e >= 0) net_terms(I, rv, v, own, d, e, r, gains, losses, adelta);
  }
}

// Count claims, exactly: an open-addressed table from (net, part) to the first
// window position of a count-only mover that changes that part's count on that
// net.  Movers insert in evaluation and clear the slots they recorded at
// commit, so the table is empty between rounds.  A probe longer than kProbe
// marks the round (ctab_over), whose checks then fall back to the part mask.
constexpr int kProbe = 32;
__device__ __forceinline__ uint32_t ctab_hash(int e, int p) {
  uint32_t h = (uint32_t)e * 0x9E3779B1u ^ ((uint32_t)p * 0x85EBCA77u);
  return h ^ (h >> 15);
}
__device__ __forceinline__ unsigned long long ctab_keyof(int e, int p) {
  return ((unsigned long long)(unsigned)e << 12) | (unsigned)p;
}
__device__ uint32_t ctab_insert(const SpecBuf& B, int e, int p, int z, int par) {
  const unsigned long long key = ctab_keyof(e, p);
  uint32_t s = ctab_hash(e, p) & B.ctab_mask;
  for (int i = 0; i < kProbe; i++) {
    const unsigned long long prev = atomicCAS(&B.ctab_key[s], ~0ull, key);
    if (prev == ~0ull || prev == key) {
      atomicMin(&B.ctab_pos[s], z);
      atomicAdd(&B.ctab_cnt[s], 1);
      return s;
    }
    s = (s + 1) & B.ctab_mask;
  }
  atomicExch(&B.ctab_over[par], 1);
  return ~0u;
}
// First position of a count-only mover on (e, p) and the number of such movers
// in the round (*n); kNone if none, -1 if unknown.
__device__ int ctab_find(const SpecBuf& B, int e, int p, int* n) {
  const unsigned long long key = ctab_keyof(e, p);
  uint32_t s = ctab_hash(e, p) & B.ctab_mask;
  for (int i = 0; i < kProbe; i++) {
    const unsigned long long k = lds(&B.ctab_key[s]);
    if (k == key) {
      *n = lds(&B.ctab_cnt[s]);
      return lds(&B.ctab_pos[s]);
    }
    if (k == ~0ull) return kNone;
    s = (s + 1) & B.ctab_mask;
  }
  return -1;
}

// Claims of the mover at position z on its nets k0, k0 + kstep, ...: a change
// of the part set (or, with volumes, of the source's side) takes claim_m, a
// count-only change claim_c, the bits of the two parts and their table entries.
__device__ __forceinline__ void claim_nets(const DevInstance& I, const SpecBuf& B, bool vol, int z, int own, int d,
                                           uint32_t base, int deg, int k0, int kstep, int par) {
  const uint32_t bits = (1u << (own & 31)) | (1u << (d & 31));
  for (int k = k0; k < deg; k += kstep) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    if (rec_setchange(lds(&B.rec[base + k]), vol)) {
      atomicMin(&B.claim_m[e], z);
    } else {
      atomicMin(&B.claim_c[e], z);
      atomicOr(&B.mask_c[e], bits);
      const uint32_t s1 = ctab_insert(B, e, own, z, par);
      const uint32_t s2 = ctab_insert(B, e, d, z, par);
      B.rec_slot[base + k] = make_uint2(s1, s2);
    }
  }
}

// Appends a mover of window offset o to the round's list.
__device__ __forceinline__ void list_mover(const SpecBuf& B, int par, int o, int wv, int pk) {
  const int i = atomicAdd(&B.mcnt[par], 1);
  B.mlist[i] = make_int4(o, wv, pk, 0);
  B.midx[o] = i;
}

__device__ __forceinline__ void ctab_clear(const SpecBuf& B, uint2 sl) {
  if (sl.x != ~0u) { B.ctab_key[sl.x] = ~0ull; B.ctab_pos[sl.x] = kNone; B.ctab_cnt[sl.x] = 0; }
  if (sl.y != ~0u) { B.ctab_key[sl.y] = ~0ull; B.ctab_pos[sl.y] = kNone; B.ctab_cnt[sl.y] = 0; }
}

// Clears the claims of a vertex on its nets k0, k0 + kstep, ... (commit phase):
// cur, those of its current move (its records and rec_slot); old, those of a
// move an in-window fix replaced (rec_slot2).
__device__ __forceinline__ void unclaim_nets(const DevInstance& I, const SpecBuf& B, bool vol, uint32_t base, int deg,
                                             int k0, int kstep, bool cur = true, bool old = false) {
  for (int k = k0; k < deg; k += kstep) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    B.claim_m[e] = kNone;
    B.claim_c[e] = kNone;
    B.mask_c[e] = 0;
    if (cur && !rec_setchange(lds(&B.rec[base + k]), vol)) ctab_clear(B, lds(&B.rec_slot[base + k]));
    if (old) ctab_clear(B, lds(&B.rec_slot2[base + k]));
  }
}

// Did an earlier mover of the window change something the vertex at z read on
// its nets k0, k0 + kstep, ...?  0: nothing; 5: a part set; 6: the count of
// z's own part where it matters; 7: z (a mover) changes the part set of a net
// whose counts an earlier mover changes.
//
// Counts enter a decision only through "own has exactly one pin on the net",
// and only when the vertex would move (cand: decision != own; its move records
// hold own's slot).  Before the commit the count c it saw is still in place;
// earlier count-only moves can make it 1 only if c == 1 or if at least c - 1
// of the round's count-only movers touch (net, own).
__device__ __forceinline__ int conflicts(const DevInstance& I, const SpecBuf& B, bool vol, int z, int own,
                                         bool cand, bool mover, uint32_t base, int deg, int k0, int kstep, bool ov) {
  const unsigned ob = 1u << (own & 31);
  int conf = 0;
  for (int k = k0; k < deg && !conf; k += kstep) {
    const int e = (int)__ldg(&I.vnets[base + k]);
    if (lds(&B.claim_m[e]) < z) {
      conf = 5;
    } else if (cand && lds(&B.claim_c[e]) < z) {
      bool hit;
      if (ov) {
        hit = (lds(&B.mask_c[e]) & ob) != 0;
      } else {
        int n = 0;
        const int fp = ctab_find(B, e, own, &n);
        if (fp < 0) {
          hit = true;
        } else if (fp >= z) {
          hit = false;
        } else {
          const int c = lds(&I.ep_cnt[(int)__ldg(&I.nptr[e]) + rec_jo(lds(&B.rec[base + k]))]);
          hit = c <= 1 || n >= c - 1;
        }
      }
      if (hit) conf = 6;
      else if (mover && rec_setchange(lds(&B.rec[base + k]), vol)) conf = 7;
    }
  }
  return conf;
}

// Per-thread partial of the MSV / MSRV accept test (MGV/partition.cpp:339-362,
// MSRV/partition.cpp:352-376) over parts p0, p0 + pstep, ...
struct AcceptPart {
  bool failM, failN, mt;
  int fsl, msl, vd;
};

__device__ AcceptPart accept_partial(const RoundCtx& R, const int* gains, const int* losses, const int* adelta, int K,
                                     bool rv, int p0, int pstep) {
  AcceptPart a{false, false, false, -1, kBig, 0};
  for (int p = p0; p < K; p += pstep) {
    const int g = gains[p], l = losses[p];
    const int t = R.vol[p] + l - g;
    if (R.mark[p] == R.cc) {
      if (rv ? (g <= l) : (g < l)) a.failM = true;
      if (adelta[p] != 0) a.mt = true;
    } else {
      if (t >= R.maxv) { a.failN = true; a.fsl = max(a.fsl, t - R.maxv); }
      a.msl = min(a.msl, R.maxv - 1 - t);
    }
    a.vd = max(a.vd, abs(adelta[p]));
  }
  return a;
}

// Outcome and volume slack: accepted -> stays accepted while no non-max part
// rises by more than msl; rejected on a max part -> local, stays rejected;
// rejected only on non-max parts -> stays rejected while the worst of them
// drops by at most fsl.
__device__ __forceinline__ void accept_final(bool failM, bool failN, int fsl, int msl, bool* good, int* vslack) {
  *good = !failM && !failN;
  *vslack = *good ? msl : (failM ? kBig : fsl);
}

__device__ __forceinline__ int block_reduce_max(int x, int* scr) {
  x = warp_max(x);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scr[threadIdx.x >> 5] = x;
  __syncthreads();
  int r = scr[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); i++) r = max(r, scr[i]);
  __syncthreads();
  return r;
}
__device__ __forceinline__ int block_reduce_sum(int x, int* scr) {
  x = warp_sum(x);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scr[threadIdx.x >> 5] = x;
  __syncthreads();
  int s = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += scr[i];
  __syncthreads();
  return s;
}
__device__ __forceinline__ int block_reduce_min(int x, int* scr) {
  return -block_reduce_max(-x, scr);
}

// Evaluation of a medium vertex at position z by the whole CTA: the warps split
// the tally, warp 0 decides, the warps split the locate pass and the gain /
// loss terms.  Writes the same per-position record as a warp evaluation (flag
// bit 2 marks it).
__device__ void cta_eval_ldg(const DevInstance& I, const SpecBuf& B, const RoundCtx& R, int metric, int z, int pos,
                             int par, int q, int* cnt_b, unsigned long long* first_b, int* gains_b, int* losses_b,
                             int* adelta_b, int* iscr, int* s_mw, int* s_mv, int* loc_b, bool logp) {
  __shared__ int sh[4];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const bool vol = metric != kTV, rv = metric == kMSRV;
  const int o = z - pos;
  const int v = __ldg(&B.porder[z]);
  const int own = lds(&I.part_vec[v]);
  const uint32_t base = __ldg(&I.vptr[v]);
  const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
  int* cnt = cnt_b + (size_t)wib * K;
  unsigned long long* first = first_b + (size_t)wib * K;
  const long long t0 = clock64();
  for (int p = lane; p < K; p += 32) { cnt[p] = 0; first[p] = ~0ull; }
  __syncwarp();
  int c1 = 0;
  {
    int n0, n1;
    net_range(deg, wib, kSWarps, &n0, &n1);
    for (int nb = n0; nb < n1; nb += 32) c1 += tally_batch(I, own, base, nb, n1, cnt, first);
  }
  c1 = warp_sum(c1);
  __syncthreads();
  if (lane == 0) iscr[wib] = c1;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
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
  int c1t = 0;
  for (int x = 0; x < kSWarps; x++) c1t += iscr[x];
  const long long t1 = clock64();
  if (wib == 0) {
    bool special;
    int slack;
    const int d = ldg_decide(I, R, cnt_b, first_b, metric, v, own, z == pos, gains_b, B.cand + (size_t)o * K,
                             &B.ncand[o], metric == kTV ? B.scan + (size_t)o * words : nullptr, &special, &slack);
    if (lane == 0) {
      sh[0] = d;
      sh[1] = special ? 1 : 0;
      sh[2] = slack;
    }
  }
  __syncthreads();
  const long long t2 = clock64();
  const int d = sh[0];
  const bool special = sh[1] != 0;
  const int slack = sh[2];
  bool mover = false, mt = false;
  int vs = kBig, vdd = 0;
  int rg = 0, rl = 0;   // decision record (with the log on)
  if (d != own) {
    // TV moves iff the leave gain covers the arrival loss; MSV / MSRV need the
    // accept test on the gain / loss sums.
    if (metric == kTV) {
      rg = c1t;
      rl = deg - cnt_b[d];
    }
    const bool need = metric == kTV ? c1t >= deg - cnt_b[d] : true;
    mover = metric == kTV && need;
    {   // records for every decision that moves: own's slot per net serves the validation
      int* gains = gains_b + (size_t)wib * K;
      int* losses = losses_b + (size_t)wib * K;
      int* adelta = adelta_b + (size_t)wib * K;
      if (vol) {
        for (int p = lane; p < K; p += 32) { gains[p] = 0; losses[p] = 0; adelta[p] = 0; }
        __syncwarp();
      }
      locate_all(I, B, metric, v, own, d, base, deg, wib, kSWarps, loc_b + wib * 96, gains, losses, adelta);
      __syncthreads();
      if (vol) {
        for (int p = threadIdx.x; p < K; p += blockDim.x) {
          int g = 0, l = 0, a = 0;
          for (int x = 0; x < kSWarps; x++) {
            g += gains_b[(size_t)x * K + p];
            l += losses_b[(size_t)x * K + p];
            a += adelta_b[(size_t)x * K + p];
          }
          gains_b[p] = g;
          losses_b[p] = l;
          adelta_b[p] = a;
        }
        __syncthreads();
        const AcceptPart a = accept_partial(R, gains_b, losses_b, adelta_b, K, rv, threadIdx.x, blockDim.x);
        const bool fM = __syncthreads_or(a.failM);
        const bool fN = __syncthreads_or(a.failN);
        const bool amt = __syncthreads_or(a.mt);
        const int fsl = block_reduce_max(a.fsl, iscr);
        const int msl = block_reduce_min(a.msl, iscr);
        vdd = block_reduce_max(a.vd, iscr);
        bool good;
        accept_final(fM, fN, fsl, msl, &good, &vs);
        mover = good;
        mt = mover && amt;
        if (logp) {
          int g = 0, l = 0;
          for (int p = threadIdx.x; p < K; p += blockDim.x) { g += gains_b[p]; l += losses_b[p]; }
          rg = block_reduce_sum(g, iscr);
          rl = block_reduce_sum(l, iscr);
        }
      }
    }
  }
  if (mover) {
    claim_nets(I, B, vol, z, own, d, base, deg, threadIdx.x, blockDim.x, par);
    if (threadIdx.x == 0) {
      if (mt) atomicMin(&B.ctl[2 + par], z);
      list_mover(B, par, o, __ldg(&I.w[v]), (own << 16) | d);
    }
  }
  if (threadIdx.x == 0) {
    const int wv = mover ? __ldg(&I.w[v]) : 0;
    if (logp) { B.rgain[o] = rg; B.rloss[o] = rl; }
    B.dec[o] = (own << 16) | d;
    B.flag[o] = (unsigned char)((mover ? 1 : 0) | (special ? 2 : 0) | 4);
    B.slack[o] = slack;
    B.vslack[o] = vs;
    B.wt[o] = wv;
    B.vd[o] = mover ? vdd : 0;
    // CTA evaluation statistics (cycles): tally and merge / decision / the rest
    const long long t3 = clock64();
    if (kTimingStats) {
      atomicAdd(&B.stats[29], (unsigned long long)(t1 - t0));
      atomicAdd(&B.stats[30], (unsigned long long)(t2 - t1));
      atomicAdd(&B.stats[31], (unsigned long long)(t3 - t2));
      atomicAdd(&B.stats[40], 1ull);
    }
    const int owner = o / q - (int)blockIdx.x * kSWarps;   // warp of this CTA owning position z
    s_mw[owner] += wv;
    s_mv[owner] += mover ? vdd : 0;
  }
  __syncthreads();
}

// Validation of a medium vertex by the whole CTA (the warp validation's rules).
__device__ void cta_validate_ldg(const DevInstance& I, const SpecBuf& B, const RoundCtx& R, int metric, int z, int pos,
                                 int q, int par, int mtpos, long long pre_w, long long pre_v, const int* cw,
                                 const int* cv, int* dsz, const int* dsz_cta, int o_from, bool check_nets,
                                 int* cut) {
  __shared__ long long shd[2];
  __shared__ int shw;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int o = z - pos;
  const int fl = lds(&B.flag[o]);
  const int pk = lds(&B.dec[o]);
  const int own = pk >> 16, d = pk & 0xffff;
  const int v = __ldg(&B.porder[z]);
  if (wib == 0) {
    // drift before z: earlier CTAs, this CTA's warps before the owner (cw / cv),
    // the owner's positions before z
    const int owner = o / q;
    long long D = 0, V = 0;
    for (int x = lane; x < owner - (int)blockIdx.x * kSWarps; x += 32) {
      D += cw[x];
      V += cv[x];
    }
    for (int o2 = owner * q + lane; o2 < o; o2 += 32) {
      D += lds(&B.wt[o2]);
      V += lds(&B.vd[o2]);
    }
    D = warp_sum64(D);
    V = warp_sum64(V);
    if (lane == 0) {
      shd[0] = pre_w + D;
      shd[1] = pre_v + V;
      shw = ((fl & 2) && z != pos) ? 1 : 0;
    }
  }
  __syncthreads();
  const long long D = shd[0], V = shd[1];
  const bool recheck = shw == 0 && D > max(lds(&B.slack[o]), 0);
  __syncthreads();   // every thread has read shw before warp 0 may change it
  if (recheck) {
    if (wib == 0) {
      const int d2 = ldg_recheck(I, R, B, o, own, metric, dsz, dsz_cta, o_from);
      if (lane == 0 && d2 != d) shw = 2;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && shw == 0) shw = V > max(lds(&B.vslack[o]), 0) ? 3 : (mtpos < z && d != own) ? 4 : 0;
  __syncthreads();
  int why = shw;
  if (why == 0 && check_nets) {
    const uint32_t base = __ldg(&I.vptr[v]);
    const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
    const int conf = conflicts(I, B, metric != kTV, z, own, d != own, fl & 1, base, deg, threadIdx.x, blockDim.x,
                               lds(&B.ctab_over[par]) != 0);
    const int c5 = __syncthreads_or(conf == 5), c6 = __syncthreads_or(conf == 6), c7 = __syncthreads_or(conf == 7);
    why = c5 ? 5 : c6 ? 6 : c7 ? 7 : 0;
  }
  if (why && threadIdx.x == 0) atomicMin(cut, (z << 3) | why);
  __syncthreads();
}

// In-window fix of the light vertex at position z (window offset o) whose size
// check failed: its decision becomes the exact one (dfix, taken with the sizes
// the committed prefix leaves), and the move records, the accept test and the
// claims are redone for it.  The replaced move's claims stay (a superset keeps
// every later check conservative); their table slots go to rec_slot2 for the
// commit.  One warp, the warp gw owning position z.
__device__ void fix_position(const DevInstance& I, const SpecBuf& B, const RoundCtx& R, int metric, int z, int o,
                             int par, int gw, int* loc, int* gains, int* losses, int* adelta, bool logp) {
  const int lane = threadIdx.x & 31;
  const bool vol = metric != kTV, rv = metric == kMSRV;
  const int K = I.K;
  const int v = __ldg(&B.porder[z]);
  const uint32_t base = __ldg(&I.vptr[v]);
  const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
  const int fl = lds(&B.flag[o]);
  const int own = lds(&B.dec[o]) >> 16;
  const int d = lds(&B.dfix[o]);
  const bool had = (fl & 1) != 0;
  if (had) {
    for (int k = lane; k < deg; k += 32)
      B.rec_slot2[base + k] =
          rec_setchange(lds(&B.rec[base + k]), vol) ? make_uint2(~0u, ~0u) : lds(&B.rec_slot[base + k]);
  }
  bool mover = false, mt = false, good = false;
  int vs = kBig, vdd = 0;
  if (d != own) {
    for (int p = lane; p < K; p += 32) { gains[p] = 0; losses[p] = 0; adelta[p] = 0; }
    __syncwarp();
    locate_all(I, B, metric, v, own, d, base, deg, 0, 1, loc, gains, losses, adelta);
    __syncwarp();
    const AcceptPart a = accept_partial(R, gains, losses, adelta, K, rv, lane, 32);
    const bool fM = __any_sync(kAll, a.failM);
    const bool fN = __any_sync(kAll, a.failN);
    accept_final(fM, fN, warp_max(a.fsl), warp_min(a.msl), &good, &vs);
    mover = good;
    mt = mover && __any_sync(kAll, a.mt);
    vdd = warp_max(a.vd);
  }
  __syncwarp();
  if (logp) {
    int rg = 0, rl = 0;
    if (d != own) {
      for (int p = lane; p < K; p += 32) { rg += gains[p]; rl += losses[p]; }
      rg = warp_sum(rg);
      rl = warp_sum(rl);
    }
    if (lane == 0) { B.rgain[o] = rg; B.rloss[o] = rl; }
  }
  if (mover) {
    claim_nets(I, B, vol, z, own, d, base, deg, lane, 32, par);
    if (lane == 0 && mt) atomicMin(&B.ctl[2 + par], z);
  }
  if (lane == 0) {
    const int wv = mover ? __ldg(&I.w[v]) : 0;
    const int vn = mover ? vdd : 0;
    if (had) B.mlist[lds(&B.midx[o])] = make_int4(o, wv, (own << 16) | d, 0);   // the replaced mover's entry
    else if (mover) list_mover(B, par, o, wv, (own << 16) | d);
    B.wsum[gw] += wv - lds(&B.wt[o]);
    B.vsum[gw] += vn - lds(&B.vd[o]);
    B.dec[o] = (own << 16) | d;
    B.flag[o] = (unsigned char)((fl & 10) | (mover ? 1 : 0) | (good ? 16 : 0) | 32 | (had ? 64 : 0));
    B.slack[o] = kBig;   // exact: no size check again
    B.vslack[o] = vs;
    B.wt[o] = wv;
    B.vd[o] = vn;
  }
  __syncwarp();
}

static_assert(kMaxGridVerts <= kSWarps, "one warp decides each whole-grid vertex of a window");

// Two CTAs per SM: without the hint the compiler trades registers for a third
// CTA and spills, which measured slower.
__global__ void __launch_bounds__(kSThreads, 2) spec_ldg_kernel(DevInstance I, SpecBuf B, int passes) {
  barrier_start();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long uscr[kSWarps];
  __shared__ int iscr[kSWarps];
  __shared__ int s_minpart, s_minsize, s_second, s_maxv, s_cc, s_count;
  // the window's whole-grid vertices: position, vertex, own part, first net
  // index, degree, decision, stale-marker risk, size slack
  __shared__ int s_gz[kMaxGridVerts], s_gv[kMaxGridVerts], s_go[kMaxGridVerts], s_gd[kMaxGridVerts];
  __shared__ uint32_t s_gb[kMaxGridVerts];
  __shared__ int s_gdec[kMaxGridVerts], s_gspec[kMaxGridVerts], s_gslk[kMaxGridVerts];
  __shared__ long long s_pre_w, s_pre_v;
  __shared__ unsigned long long uscr2[kSWarps];
  __shared__ int s_cw[kSWarps], s_cv[kSWarps], s_mt, s_nm;   // this CTA's warps' sums, round words
  __shared__ int s_mw[kSWarps], s_mv[kSWarps];
  __shared__ int loc_b[kSWarps * 96];   // per-warp locate scratch
  const int metric = I.metric;
  const bool vol = metric != kTV;
  const bool rv = metric == kMSRV;
  const int K = I.K;
  const int words = (K + 31) >> 5;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  const float Cf = (float)I.C;
  Carve cv{smem_raw};
  int* sizes_s = cv.take<int>(K);
  float* penf_s = cv.take<float>(K);
  int* marker_s = cv.take<int>(K);
  int* vol_s = cv.take<int>(K);
  int* mark_s = cv.take<int>(K);
  int* cnt_b = cv.take<int>((size_t)K * kSWarps);                    // per-warp arrays, warp x at x*K
  unsigned long long* first_b = cv.take<unsigned long long>((size_t)K * kSWarps);
  int* gains_b = cv.take<int>((size_t)K * kSWarps);
  int* losses_b = cv.take<int>((size_t)K * kSWarps);
  int* adelta_b = cv.take<int>((size_t)K * kSWarps);
  int* cnt = cnt_b + (size_t)wib * K;
  unsigned long long* first = first_b + (size_t)wib * K;
  int* gains = gains_b + (size_t)wib * K;
  int* losses = losses_b + (size_t)wib * K;
  int* adelta = adelta_b + (size_t)wib * K;
  int* loc = loc_b + wib * 96;
  Vol V{I.send, rv ? I.recv : nullptr};

  const bool vfix = metric == kMSV || metric == kMSRV;
  int round = 0;
  int heavy_round = 0;
  int vr = 0;   // validation passes (parity selects the cut word)
  unsigned long long tA = gtimer();
  for (int it = 0; it < passes; it++) {
    const bool logp = I.recs != nullptr && it == passes - 1;   // decision records of the last pass
    int pos = 0;
    int W = min(nwarps, B.wmax);
    int hidx = 0;
    bool pass_start = true;
    bool prev_maxtouch = false;
    while (pos < B.npos) {
      const int par = round & 1;
      // ------------------------------------------------------------ round state
      for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const int sz = lds(&I.part_sizes[p]);
        sizes_s[p] = sz;
        penf_s[p] = 1.0f - __fdiv_rn((float)sz, Cf);
        if (metric == kTV) {
          // a part scanned in the last window takes its last scanner as marker
          // (block 0 stores it; the others read only parts not scanned there)
          const unsigned long long ml = lds(&B.mlast[p]);
          if (round > 0 && (int)(ml >> 32) == round) {
            const int mv = __ldg(&B.porder[(int)(ml & 0xffffffffu)]);
            marker_s[p] = mv;
            if (blockIdx.x == 0) I.marker[p] = mv;
          } else {
            marker_s[p] = lds(&I.marker[p]);
          }
        }
        if (vol) vol_s[p] = lds(&I.send[p]) + (rv ? lds(&I.recv[p]) : 0);
      }
      __syncthreads();
      block_min_part(sizes_s, K, uscr, &s_minpart, &s_minsize, &s_second);
      if (vol) {
        // Max-volume parts.  MSV rescans after every move (MGV/partition.cpp:
        // 453-472); MSRV rescans only when an old max part changed, against the
        // old maximum, appending to its list (MSRV/partition.cpp:486-513).
        int mx = -2147483647 - 1;
        for (int p = threadIdx.x; p < K; p += blockDim.x) mx = max(mx, vol_s[p]);
        mx = warp_max(mx);
        if (lane == 0) iscr[wib] = mx;
        __syncthreads();
        mx = iscr[0];
        for (int x = 1; x < kSWarps; x++) mx = max(mx, iscr[x]);
        __syncthreads();
        if (!rv || pass_start) {
          int local = 0;
          for (int p = threadIdx.x; p < K; p += blockDim.x) {
            const bool m = vol_s[p] == mx;
            mark_s[p] = m ? 1 : -1;
            local += m;
          }
          local = warp_sum(local);
          if (lane == 0) iscr[wib] = local;
          __syncthreads();
          if (threadIdx.x == 0) {
            int c = 0;
            for (int x = 0; x < kSWarps; x++) c += iscr[x];
            s_maxv = mx;
            s_cc = 1;
            s_count = c;
          }
          __syncthreads();
        } else if (prev_maxtouch) {
          bool changed = false;
          for (int p = threadIdx.x; p < K; p += blockDim.x)
            if (mark_s[p] == s_cc && vol_s[p] != s_maxv) changed = true;
          changed = __syncthreads_or(changed);
          if (changed && mx >= s_maxv) {
            const int ncc = mx > s_maxv ? s_cc + 1 : s_cc;
            int local = 0;
            for (int p = threadIdx.x; p < K; p += blockDim.x)
              if (vol_s[p] == mx) { mark_s[p] = ncc; local++; }
            local = warp_sum(local);
            if (lane == 0) iscr[wib] = local;
            __syncthreads();
            if (threadIdx.x == 0) {
              int c = 0;
              for (int x = 0; x < kSWarps; x++) c += iscr[x];
              s_count = (mx > s_maxv ? 0 : s_count) + c;
              s_maxv = mx;
              s_cc = ncc;
              if (s_count > K) dev_fail(I.status, kDevErrUnsupported);  // the reference overruns max_parts
            }
            __syncthreads();
          }
        }
      }
      __syncthreads();
      const RoundCtx R{sizes_s, penf_s, marker_s, vol_s, mark_s, s_minpart, s_minsize, s_second, s_maxv, s_cc, Cf};
      if (blockIdx.x == 0 && threadIdx.x == 0) B.stats[20] += gtimer() - tA;
      pass_start = false;
      prev_maxtouch = false;
      while (hidx < B.nheavy && __ldg(&B.heavy_pos[hidx]) < pos) hidx++;

      // ================================================================= round
      // A window holds up to gmax whole-grid vertices and ends before the next
      // one.
      int end_w = min(pos + W, B.npos);
      if (hidx + B.gmax < B.nheavy) end_w = min(end_w, (int)__ldg(&B.heavy_pos[hidx + B.gmax]));
      int ns = 0;
      while (ns < B.gmax && hidx + ns < B.nheavy && __ldg(&B.heavy_pos[hidx + ns]) < end_w) ns++;
      const int span = end_w - pos;
      const int q = (span + nwarps - 1) / nwarps;
      const int z0 = min(pos + gw * q, end_w);
      const int z1 = min(z0 + q, end_w);
      const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gthreads = gridDim.x * blockDim.x;
      const int hp = heavy_round & 1;   // whole-grid tallies, double-buffered by parity
      // slot j of this parity: K entries at hslot(j), 8 words of hmisc at hmslot(j)
      auto hslot = [&](int j) { return ((size_t)hp * kMaxGridVerts + j) * K; };
      auto hmslot = [&](int j) { return (hp * kMaxGridVerts + j) * 8; };
      const unsigned long long tR = gtimer();
      if ((int)threadIdx.x < ns) {
        const int z = __ldg(&B.heavy_pos[hidx + threadIdx.x]);
        const int v = __ldg(&B.porder[z]);
        const uint32_t b = __ldg(&I.vptr[v]);
        s_gz[threadIdx.x] = z;
        s_gv[threadIdx.x] = v;
        s_go[threadIdx.x] = lds(&I.part_vec[v]);
        s_gb[threadIdx.x] = b;
        s_gd[threadIdx.x] = (int)(__ldg(&I.vptr[v + 1]) - b);
      }
      __syncthreads();
      // ---- A1: tally slices of the whole-grid vertices, pre-reduced per CTA
      for (int j = 0; j < ns; j++) {
        const int own_s = s_go[j], deg_s = s_gd[j];
        const uint32_t base_s = s_gb[j];
        int* hcnt = B.hcnt + hslot(j);
        unsigned long long* hfirst = B.hfirst + hslot(j);
        for (int p = lane; p < K; p += 32) { cnt[p] = 0; first[p] = ~0ull; }
        __syncwarp();
        int c1 = 0;
        {
          int n0, n1;
          net_range(deg_s, gw, nwarps, &n0, &n1);
          for (int nb = n0; nb < n1; nb += 32) c1 += tally_batch(I, own_s, base_s, nb, n1, cnt, first);
        }
        c1 = warp_sum(c1);
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
            atomicAdd(&hcnt[p], c);
            atomicMin(&hfirst[p], f);
          }
        }
        if (lane == 0 && c1) atomicAdd(&B.hmisc[hmslot(j)], c1);
        __syncthreads();   // the per-warp arrays serve the next vertex and the evaluations below
      }
      if (kTimingStats && ns && threadIdx.x == 0) atomicMax(&B.stats[38], gtimer() - tR);
      // ---- A: evaluate
      int wsum = 0, vsum = 0;
      const long long cA = clock64();
      long long cV = 0;
      int nV = 0;
      for (int z = z0; z < z1; z++) {
        const int o = z - pos;
        const int v = __ldg(&B.porder[z]);
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        if (__ldg(&B.vclass[v]) != 0) continue;   // medium vertex: evaluated by the whole CTA below
        const long long cz = clock64();
        const int own = lds(&I.part_vec[v]);
        for (int p = lane; p < K; p += 32) { cnt[p] = 0; first[p] = ~0ull; }
        __syncwarp();
        int c1 = 0;
        for (int nb = 0; nb < deg; nb += 32) c1 += tally_batch(I, own, base, nb, deg, cnt, first);
        __syncwarp();
        c1 = warp_sum(c1);
        const long long cT = clock64();
        bool special;
        int slack;
        // candidates (part, count, first sighting) for an exact re-check of the
        // decision if the part sizes drift beyond its slack; TV's scanned parts
        const int d = ldg_decide(I, R, cnt, first, metric, v, own, z == pos, gains, B.cand + (size_t)o * K,
                                 &B.ncand[o], metric == kTV ? B.scan + (size_t)o * words : nullptr, &special, &slack);
        const long long cD = clock64();
        // An isolated vertex (no nets, weight 0) changes nothing a later position
        // reads; if its decision flips under the window's size drift, validation
        // corrects it in place instead of cutting.  Its accept outcome does not
        // depend on the destination (all gains and losses are zero).
        const bool iso = deg == 0 && __ldg(&I.w[v]) == 0;
        bool mover = false, mt = false, good = metric == kTV;
        int vs = kBig, vdd = 0;
        if (metric == kTV) {
          if (d != own) {
            mover = c1 >= deg - cnt[d];
            // the records also serve the validation (own's slot per net)
            locate_all(I, B, metric, v, own, d, base, deg, 0, 1, loc, nullptr, nullptr, nullptr);
          }
        } else if (d != own || iso) {
          for (int p = lane; p < K; p += 32) { gains[p] = 0; losses[p] = 0; adelta[p] = 0; }
          __syncwarp();
          if (d != own) locate_all(I, B, metric, v, own, d, base, deg, 0, 1, loc, gains, losses, adelta);
          __syncwarp();
          AcceptPart a = accept_partial(R, gains, losses, adelta, K, rv, lane, 32);
          const bool fM = __any_sync(kAll, a.failM);
          const bool fN = __any_sync(kAll, a.failN);
          accept_final(fM, fN, warp_max(a.fsl), warp_min(a.msl), &good, &vs);
          mover = good && d != own;
          mt = mover && __any_sync(kAll, a.mt);
          vdd = warp_max(a.vd);
        }
        __syncwarp();
        if (logp) {
          // decision record: TV's leave gain / arrival loss (TV/partition.cpp:355-378),
          // MSV / MSRV's gain and loss vectors summed (MGV/partition.cpp:294-337)
          int rg = 0, rl = 0;
          if (d != own) {
            if (metric == kTV) {
              rg = c1;
              rl = deg - cnt[d];
            } else {
              for (int p = lane; p < K; p += 32) { rg += gains[p]; rl += losses[p]; }
              rg = warp_sum(rg);
              rl = warp_sum(rl);
            }
          }
          if (lane == 0) { B.rgain[o] = rg; B.rloss[o] = rl; }
        }
        const int wv = mover ? __ldg(&I.w[v]) : 0;
        if (mover) {
          claim_nets(I, B, vol, z, own, d, base, deg, lane, 32, par);
          if (lane == 0) {
            if (mt) atomicMin(&B.ctl[2 + par], z);
            list_mover(B, par, o, wv, (own << 16) | d);
          }
        }
        if (lane == 0) {
          B.dec[o] = (own << 16) | d;   // own read now: part_vec changes in the commit phase
          B.flag[o] = (unsigned char)((mover ? 1 : 0) | (special ? 2 : 0) | (iso ? 8 : 0) | (good ? 16 : 0));
          B.slack[o] = slack;
          B.vslack[o] = vs;
          B.wt[o] = wv;
          B.vd[o] = mover ? vdd : 0;
        }
        wsum += wv;
        vsum += mover ? vdd : 0;
        if (kTimingStats && lane == 0) {
          atomicAdd(&B.stats[41], (unsigned long long)(cT - cz));
          atomicAdd(&B.stats[42], (unsigned long long)(cD - cT));
          atomicAdd(&B.stats[43], (unsigned long long)(clock64() - cD));
        }
        cV += clock64() - cz;
        nV++;
        __syncwarp();
      }
      if (kTimingStats && lane == 0 && nV) {
        // per-window statistics (cycles): slowest warp, and all light evaluations
        atomicMax(&B.stats[22], (unsigned long long)(clock64() - cA));
        atomicAdd(&B.stats[25], (unsigned long long)cV);
        atomicAdd(&B.stats[26], (unsigned long long)nV);
      }
      // medium vertices of this CTA's positions: the CTA evaluates them together
      if (threadIdx.x < kSWarps) { s_mw[threadIdx.x] = 0; s_mv[threadIdx.x] = 0; }
      __syncthreads();
      const long long cM = clock64();
      const int cz0 = min(pos + blockIdx.x * kSWarps * q, end_w);
      const int cz1 = min(cz0 + kSWarps * q, end_w);
      for (int mi = lower_bound_pos(B.mid_pos, B.nmid, cz0); mi < B.nmid; mi++) {
        const int z = __ldg(&B.mid_pos[mi]);
        if (z >= cz1) break;
        cta_eval_ldg(I, B, R, metric, z, pos, par, q, cnt_b, first_b, gains_b, losses_b, adelta_b, iscr, s_mw, s_mv,
                     loc_b, logp);
      }
      __syncthreads();
      if (kTimingStats && threadIdx.x == 0) {
        const long long dm = clock64() - cM;
        if (dm > 2000) atomicMax(&B.stats[24], (unsigned long long)dm);
        atomicMax(&B.stats[36], gtimer() - tR);
      }
      if (ns) {
        if (!grid_barrier(B.bar, I.status)) return;
        const unsigned long long tG = gtimer();
        // ---- A2: decisions of the whole-grid vertices, taken in every CTA from
        // the global tallies (warp j decides vertex j; each is first of the
        // window or not, like any position), then their locate / gain-loss slices
        for (int j = 0; j < ns; j++) {
          const size_t hs = hslot(j);
          for (int p = threadIdx.x; p < K; p += blockDim.x) {
            cnt_b[(size_t)j * K + p] = lds(&B.hcnt[hs + p]);
            first_b[(size_t)j * K + p] = lds(&B.hfirst[hs + p]);
          }
        }
        __syncthreads();
        if (wib < ns) {
          const int j = wib;
          const int zs = s_gz[j], vsup = s_gv[j], own_s = s_go[j];
          const int* cj = cnt_b + (size_t)j * K;
          const unsigned long long* fj = first_b + (size_t)j * K;
          bool special;
          int slack;
          // block 0 keeps the candidates for an exact re-check, TV's scanned parts
          const int os = zs - pos;
          const bool b0 = blockIdx.x == 0;
          const int d = ldg_decide(I, R, cj, fj, metric, vsup, own_s, zs == pos, gains_b + (size_t)j * K,
                                   b0 ? B.cand + (size_t)os * K : nullptr, b0 ? &B.ncand[os] : nullptr,
                                   b0 && metric == kTV ? B.scan + (size_t)os * words : nullptr, &special, &slack);
          if (lane == 0) { s_gdec[j] = d; s_gspec[j] = special ? 1 : 0; s_gslk[j] = slack; }
        }
        __syncthreads();
        for (int j = 0; j < ns; j++) {
          const int d = s_gdec[j], own_s = s_go[j];
          if (d == own_s) continue;   // records for every decision that moves (the validation reads own's slots)
          const size_t hs = hslot(j);
          if (vol) {
            for (int p = lane; p < K; p += 32) { gains[p] = 0; losses[p] = 0; adelta[p] = 0; }
            __syncwarp();
          }
          locate_all(I, B, metric, s_gv[j], own_s, d, s_gb[j], s_gd[j], gw, nwarps, loc, gains, losses, adelta);
          if (vol) {
            __syncthreads();
            for (int p = threadIdx.x; p < K; p += blockDim.x) {
              int g = 0, l = 0, a = 0;
              for (int x = 0; x < kSWarps; x++) {
                g += gains_b[(size_t)x * K + p];
                l += losses_b[(size_t)x * K + p];
                a += adelta_b[(size_t)x * K + p];
              }
              if (g) atomicAdd(&B.hgain[hs + p], g);
              if (l) atomicAdd(&B.hloss[hs + p], l);
              if (a) atomicAdd(&B.hadelta[hs + p], a);
            }
            __syncthreads();   // the per-warp arrays serve the next vertex
          }
        }
        if (!grid_barrier(B.bar, I.status)) return;
        // ---- A3: accept tests (MSV / MSRV) in every CTA, claims, the records
        for (int j = 0; j < ns; j++) {
          const size_t hs = hslot(j);
          const int zs = s_gz[j], vsup = s_gv[j], own_s = s_go[j], deg_s = s_gd[j], d = s_gdec[j];
          const uint32_t base_s = s_gb[j];
          const int os = zs - pos;
          const bool need = d != own_s &&
                            (metric == kTV ? lds(&B.hmisc[hmslot(j)]) >= deg_s - cnt_b[(size_t)j * K + d] : true);
          bool mover = metric == kTV && need, mt = false;
          int vs = kBig, vdd = 0;
          int rg = 0, rl = 0;   // decision record (with the log on)
          if (metric == kTV && d != own_s) {
            rg = lds(&B.hmisc[hmslot(j)]);
            rl = deg_s - cnt_b[(size_t)j * K + d];
          }
          if (vol && need) {
            for (int p = threadIdx.x; p < K; p += blockDim.x) {
              gains_b[p] = lds(&B.hgain[hs + p]);
              losses_b[p] = lds(&B.hloss[hs + p]);
              adelta_b[p] = lds(&B.hadelta[hs + p]);
            }
            __syncthreads();
            const AcceptPart a = accept_partial(R, gains_b, losses_b, adelta_b, K, rv, threadIdx.x, blockDim.x);
            const bool fM = __syncthreads_or(a.failM);
            const bool fN = __syncthreads_or(a.failN);
            const bool amt = __syncthreads_or(a.mt);
            const int fsl = block_reduce_max(a.fsl, iscr);
            const int msl = block_reduce_min(a.msl, iscr);
            vdd = block_reduce_max(a.vd, iscr);
            bool good;
            accept_final(fM, fN, fsl, msl, &good, &vs);
            mover = good;
            mt = mover && amt;
            if (logp) {
              int g = 0, l = 0;
              for (int p = threadIdx.x; p < K; p += blockDim.x) { g += gains_b[p]; l += losses_b[p]; }
              rg = block_reduce_sum(g, iscr);
              rl = block_reduce_sum(l, iscr);
            }
          }
          if (mover) claim_nets(I, B, vol, zs, own_s, d, base_s, deg_s, gtid, gthreads, par);
          const int wv = mover ? __ldg(&I.w[vsup]) : 0;
          if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (logp) { B.rgain[os] = rg; B.rloss[os] = rl; }
            B.dec[os] = (own_s << 16) | d;
            B.flag[os] = (unsigned char)((mover ? 1 : 0) | (s_gspec[j] ? 2 : 0) | 4);
            B.slack[os] = s_gslk[j];
            B.vslack[os] = vs;
            B.wt[os] = wv;
            B.vd[os] = mover ? vdd : 0;
            if (mover) {
              if (mt) atomicMin(&B.ctl[2 + par], zs);
              list_mover(B, par, os, wv, (own_s << 16) | d);
            }
          }
          // the warp owning position zs carries its weight and volume change
          const int owner = os / q;
          if (threadIdx.x == 0 && owner / kSWarps == (int)blockIdx.x) {
            s_mw[owner % kSWarps] += wv;
            s_mv[owner % kSWarps] += mover ? vdd : 0;
          }
          __syncthreads();
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) B.stats[33] += gtimer() - tG;
      }
      if (lane == 0) {
        B.wsum[gw] = wsum + s_mw[wib];
        B.vsum[gw] = vsum + s_mv[wib];
      }
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tE = gtimer();
        B.stats[16] += tE - tA;
        tA = tE;
        B.stats[21] += B.stats[22];   // no CTA writes these again before the next phase A
        B.stats[22] = 0;
        B.stats[23] += B.stats[24];
        B.stats[24] = 0;
      }
      int cutw;
      for (int zfix = pos, nfix = 0;; nfix++) {
        int* const cut_w = &B.ctl[4 + (vr & 1)];
        // ---- B: validate.  Prefix sums of moved weight and volume drift over the
        // warps before this one (warps own consecutive position ranges).
        // Positions before zfix are known valid (an earlier pass of the window).
        const unsigned long long tV = gtimer();
        long long Dw, Vw;
        {
          // one round of independent loads: the earlier warps' sums, this CTA's
          // warps' sums, the round words
          long long pw = 0, pv = 0;
          const int lim = blockIdx.x * kSWarps;
          for (int g = threadIdx.x; g < lim; g += blockDim.x) {
            pw += lds(&B.wsum[g]);
            pv += lds(&B.vsum[g]);
          }
          if (threadIdx.x < kSWarps) {
            s_cw[threadIdx.x] = lds(&B.wsum[lim + threadIdx.x]);
            s_cv[threadIdx.x] = lds(&B.vsum[lim + threadIdx.x]);
          }
          if (threadIdx.x == 0) {
            s_mt = lds(&B.ctl[2 + par]);
            s_nm = lds(&B.mcnt[par]);
          }
          pw = warp_sum64(pw);
          pv = warp_sum64(pv);
          if (lane == 0) {
            uscr[wib] = (unsigned long long)pw;
            uscr2[wib] = (unsigned long long)pv;
          }
          __syncthreads();
          long long a = 0, b = 0;
          for (int x = 0; x < kSWarps; x++) {
            a += (long long)uscr[x];
            b += (long long)uscr2[x];
          }
          if (threadIdx.x == 0) {
            s_pre_w = a;
            s_pre_v = b;
          }
          Dw = a;
          Vw = b;
          for (int x = 0; x < wib; x++) {
            Dw += s_cw[x];
            Vw += s_cv[x];
          }
        }
        const int mtpos = s_mt;
        const int nm = s_nm;
        const unsigned long long tV1 = gtimer();
        // part-size changes of the window's movers before this CTA's first position
        // (phase-A scratch gains_b is free now)
        int* dsz_cta = gains_b;
        const int cta_o0 = cz0 - pos;
        for (int p = threadIdx.x; p < K; p += blockDim.x) dsz_cta[p] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < nm; i += blockDim.x) {
          const int4 m = lds(&B.mlist[i]);
          if (m.x >= cta_o0 || m.y == 0) continue;
          atomicAdd(&dsz_cta[m.z & 0xffff], m.y);
          atomicAdd(&dsz_cta[m.z >> 16], -m.y);
        }
        __syncthreads();
        const bool ov = lds(&B.ctab_over[par]) != 0;
        for (int z = z0; z < z1; z++) {
          const int o = z - pos;
          // the position's words in one round of independent loads
          const int wz = lds(&B.wt[o]), vz = lds(&B.vd[o]);
          const int fl = lds(&B.flag[o]);
          const int slk = lds(&B.slack[o]), vslk = lds(&B.vslack[o]);
          int pk = lds(&B.dec[o]);
          const int v = __ldg(&B.porder[z]);
          if (z < zfix || (fl & 4)) {      // valid already / medium vertex, validated by the CTA below
            Dw += wz;
            Vw += vz;
            continue;
          }
          const uint32_t base = __ldg(&I.vptr[v]);
          const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
          const int own = pk >> 16;
          int why = ((fl & 2) && z != pos) ? 1 : 0;
          if (!why && Dw > max(slk, 0)) {
            // beyond the slack: decide again with the exact sizes at this position
            const int d2 = ldg_recheck(I, R, B, o, own, metric, cnt, dsz_cta, cta_o0);
            if (d2 != (pk & 0xffff)) {
              if (fl & 8) {
                // isolated vertex: take the exact decision (no weight, no nets, so
                // no later position sees the difference)
                pk = (own << 16) | d2;
                if (lane == 0) {
                  B.dec[o] = pk;
                  B.flag[o] = (unsigned char)((fl & ~1) | ((fl & 16) && d2 != own ? 1 : 0));
                }
              } else {
                why = 2;
                if (lane == 0) B.dfix[o] = d2;
              }
            }
          }
          // the max-volume parts enter only the accept test of a vertex whose
          // decision leaves its part (MSRV/partition.cpp:308-400,
          // MGV/partition.cpp:292-362), and they change only with a move
          if (!why) why = Vw > max(vslk, 0) ? 3 : (mtpos < z && (pk & 0xffff) != own) ? 4 : 0;
          if (!why) {
            const int c = conflicts(I, B, vol, z, own, (pk & 0xffff) != own, fl & 1, base, deg, lane, 32, ov);
            const int c5 = __any_sync(kAll, c == 5), c6 = __any_sync(kAll, c == 6), c7 = __any_sync(kAll, c == 7);
            why = c5 ? 5 : c6 ? 6 : c7 ? 7 : 0;
          }
          if (why) {
            if (lane == 0) atomicMin(cut_w, (z << 3) | why);   // position, then cut reason
            break;
          }
          Dw += wz;
          Vw += vz;
        }
        __syncthreads();
        const unsigned long long tV2 = gtimer();
        for (int mi = lower_bound_pos(B.mid_pos, B.nmid, cz0); mi < B.nmid; mi++) {
          const int z = __ldg(&B.mid_pos[mi]);
          if (z >= cz1) break;
          if (z < zfix) continue;
          cta_validate_ldg(I, B, R, metric, z, pos, q, par, mtpos, s_pre_w, s_pre_v, s_cw, s_cv, cnt_b, dsz_cta,
                           cta_o0, true, cut_w);
        }
        for (int j = 0; j < ns; j++) {
          // a whole-grid vertex: its nets checked by every thread, the rest by the
          // CTA owning its position
          const int zs = s_gz[j], own_s = s_go[j];
          if (zs < zfix) continue;
          const int os = zs - pos;
          const int fl = lds(&B.flag[os]);
          const int c = conflicts(I, B, vol, zs, own_s, (lds(&B.dec[os]) & 0xffff) != own_s, fl & 1, s_gb[j], s_gd[j],
                                  gtid, gthreads, lds(&B.ctab_over[par]) != 0);
          if (c) atomicMin(cut_w, (zs << 3) | c);
          if (zs >= cz0 && zs < cz1)
            cta_validate_ldg(I, B, R, metric, zs, pos, q, par, mtpos, s_pre_w, s_pre_v, s_cw, s_cv, cnt_b, dsz_cta,
                             cta_o0, false, cut_w);
        }
        __syncthreads();
        if (kTimingStats && threadIdx.x == 0) {
          const unsigned long long tV3 = gtimer();
          atomicMax(&B.stats[39], tV3 - tV);
          // per-pass phase times of this CTA: prefix sums, light positions, the rest
          atomicAdd(&B.stats[45], tV1 - tV);
          atomicAdd(&B.stats[46], tV2 - tV1);
          atomicAdd(&B.stats[47], tV3 - tV2);
        }
        if (!grid_barrier(B.bar, I.status)) return;
        cutw = lds(cut_w);
        if (blockIdx.x == 0 && threadIdx.x == 0) B.ctl[4 + ((vr + 1) & 1)] = kNone;   // the next pass's word
        vr++;
        // a size flip of a light position (MSV / MSRV): fix it and validate again
        bool fix = vfix && nfix < B.maxfix && cutw != kNone && (cutw & 7) == 2;
        const int zc = cutw >> 3;
        if (fix) fix = zc < end_w && __ldg(&B.vclass[__ldg(&B.porder[zc])]) == 0;
        if (!fix) break;
        if (gw == (zc - pos) / q)
          fix_position(I, B, R, metric, zc, zc - pos, par, gw, loc, gains, losses, adelta, logp);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          B.stats[44]++;
          B.stats[35] += B.stats[39];
          B.stats[39] = 0;
        }
        if (!grid_barrier(B.bar, I.status)) return;
        zfix = zc;
      }
      // ---- C: commit every mover before the cut.
      const int cut = cutw == kNone ? end_w : min(cutw >> 3, end_w);
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tB = gtimer();
        B.stats[0]++;
        const int why = cutw == kNone ? 0 : (cutw & 7);
        B.stats[why <= 5 ? 3 + why : 21 + why]++;   // 6, 7: slots 27, 28
        B.stats[9] += cut - pos;
        // per-window maxima over CTAs (no CTA writes these again before the next phase A)
        B.stats[32] += B.stats[36];
        B.stats[34] += B.stats[38];
        B.stats[35] += B.stats[39];
        B.stats[36] = 0;
        B.stats[38] = 0;
        B.stats[39] = 0;
        B.stats[17] += tB - tA;
        tA = tB;
      }
      if (cut <= pos) {             // no progress: inconsistent claims; stop (all CTAs agree)
        if (threadIdx.x == 0) dev_fail(I.status, kDevErrInvalid);
        return;
      }
      const int mt_c = lds(&B.ctl[2 + par]);
      if (logp) {
        // decision records of this warp's committed positions
        for (int z = z0 + lane; z < min(z1, cut); z += 32) {
          const int o = z - pos;
          const int fl = lds(&B.flag[o]);
          I.recs[__ldg(&B.porder[z])] =
              make_int4(lds(&B.dec[o]) & 0xffff, lds(&B.rgain[o]), lds(&B.rloss[o]), fl & 1);
        }
      }
      for (int z = z0; z < z1; z++) {
        const int o = z - pos;
        const int fl = lds(&B.flag[o]);
        if (!(fl & (1 | 64)) || (fl & 4)) continue;   // claims held: a mover or a replaced mover
        const int v = __ldg(&B.porder[z]);
        const int pk = lds(&B.dec[o]);
        const int own = pk >> 16, d = pk & 0xffff;
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        if ((fl & 1) && z < cut) {
          for (int k = lane; k < deg; k += 32)
            commit_rec(I, v, own, d, (int)__ldg(&I.vnets[base + k]), lds(&B.rec[base + k]), vol ? &V : nullptr);
          if (lane == 0) {
            atomicAdd(&B.stats[2], 1ull);
            I.part_vec[v] = d;
            const int wv = __ldg(&I.w[v]);
            atomicAdd(&I.part_sizes[own], -wv);
            atomicAdd(&I.part_sizes[d], wv);
            atomicAdd((unsigned long long*)&I.moves[it], 1ull);
          }
        }
        unclaim_nets(I, B, vol, base, deg, lane, 32, fl & 1, fl & 64);
      }
      for (int mi = lower_bound_pos(B.mid_pos, B.nmid, cz0); mi < B.nmid; mi++) {
        const int z = __ldg(&B.mid_pos[mi]);
        if (z >= cz1) break;
        const int o = z - pos;
        const int fl = lds(&B.flag[o]);
        if (!(fl & 1)) continue;
        const int v = __ldg(&B.porder[z]);
        const int pk = lds(&B.dec[o]);
        const int own = pk >> 16, d = pk & 0xffff;
        const uint32_t base = __ldg(&I.vptr[v]);
        const int deg = (int)(__ldg(&I.vptr[v + 1]) - base);
        if (z < cut) {
          for (int k = threadIdx.x; k < deg; k += blockDim.x)
            commit_rec(I, v, own, d, (int)__ldg(&I.vnets[base + k]), lds(&B.rec[base + k]), vol ? &V : nullptr);
          if (threadIdx.x == 0) {
            atomicAdd(&B.stats[2], 1ull);
            I.part_vec[v] = d;
            const int wv = __ldg(&I.w[v]);
            atomicAdd(&I.part_sizes[own], -wv);
            atomicAdd(&I.part_sizes[d], wv);
            atomicAdd((unsigned long long*)&I.moves[it], 1ull);
          }
        }
        unclaim_nets(I, B, vol, base, deg, threadIdx.x, blockDim.x);
      }
      for (int j = 0; j < ns; j++) {
        // a whole-grid vertex, by every thread
        const int zs = s_gz[j], vsup = s_gv[j], own_s = s_go[j], deg_s = s_gd[j];
        const uint32_t base_s = s_gb[j];
        const int os = zs - pos;
        if (lds(&B.flag[os]) & 1) {
          const int pk = lds(&B.dec[os]);
          const int d = pk & 0xffff;
          if (zs < cut) {
            for (int i = gtid; i < deg_s; i += gthreads)
              commit_rec(I, vsup, own_s, d, (int)__ldg(&I.vnets[base_s + i]), lds(&B.rec[base_s + i]),
                         vol ? &V : nullptr);
            if (gtid == 0) {
              atomicAdd(&B.stats[2], 1ull);
              I.part_vec[vsup] = d;
              const int wv = __ldg(&I.w[vsup]);
              atomicAdd(&I.part_sizes[own_s], -wv);
              atomicAdd(&I.part_sizes[d], wv);
              atomicAdd((unsigned long long*)&I.moves[it], 1ull);
            }
          }
          unclaim_nets(I, B, vol, base_s, deg_s, gtid, gthreads);
        }
      }
      if (B.niso && (metric != kMSRV || logp)) {
        // Vertices without nets, weight 0 (positions hold only the others):
        // each takes the least-loaded part at its place in the visiting order
        // (TV: unless the clamps keep it home) and changes nothing a later
        // decision reads, so they are decided here, after the cut, from the
        // exact sizes between the committed positions (MSRV never moves them;
        // there they are walked only for the decision records).
        int* dsz = gains_b;   // the committed movers' size changes before this CTA's first position
        const int cta_o0 = cz0 - pos;
        for (int p = threadIdx.x; p < K; p += blockDim.x) dsz[p] = 0;
        __syncthreads();
        const int nmv = lds(&B.mcnt[par]);
        for (int i = threadIdx.x; i < nmv; i += blockDim.x) {
          const int4 m = lds(&B.mlist[i]);
          if (m.x >= cta_o0 || m.y == 0) continue;
          atomicAdd(&dsz[m.z & 0xffff], m.y);
          atomicAdd(&dsz[m.z >> 16], -m.y);
        }
        __syncthreads();
        const int zb = min(z1, cut);
        if (z0 < zb) {
          int* sz = cnt;   // this warp's sizes, at its current position
          for (int p = lane; p < K; p += 32) sz[p] = sizes_s[p] + dsz[p];
          __syncwarp();
          for (int o2 = cta_o0 + lane; o2 < z0 - pos; o2 += 32) {
            const int w = lds(&B.wt[o2]);
            if (w == 0) continue;
            const int pk = lds(&B.dec[o2]);
            atomicAdd(&sz[pk & 0xffff], w);
            atomicAdd(&sz[pk >> 16], -w);
          }
          __syncwarp();
          int amin = -1;
          long long nmoved = 0;
          auto group = [&](int k0, int k1) {
            if (k0 >= k1) return;
            if (amin < 0) {
              unsigned long long mk = ~0ull;
              for (int p = lane; p < K; p += 32) {
                const unsigned long long key = ((unsigned long long)((unsigned)sz[p] ^ 0x80000000u) << 32) | (unsigned)p;
                mk = key < mk ? key : mk;
              }
              for (int off = 16; off; off >>= 1) {
                const unsigned long long x = __shfl_xor_sync(kAll, mk, off);
                mk = x < mk ? x : mk;
              }
              amin = (int)(mk & 0xffffffffu);
            }
            const int sa = sz[amin];
            const bool home = metric == kTV && (sa > I.max_pw || sa < I.min_pw);
            for (int k = k0 + lane; k < k1; k += 32) {
              const int v = __ldg(&B.iso_list[k]);
              const int own = lds(&I.part_vec[v]);
              const int d = home ? own : amin;
              const bool mv = d != own && metric != kMSRV;
              if (mv) {
                I.part_vec[v] = d;
                nmoved++;
              }
              if (logp) I.recs[v] = make_int4(d, 0, 0, mv ? 1 : 0);
            }
          };
          if (pos == 0 && gw == 0) group(0, __ldg(&B.iso_before[0]));   // before the pass's first position
          for (int z = z0; z < zb; z++) {
            const int o = z - pos;
            const int w = lds(&B.wt[o]);
            if (w != 0) {
              __syncwarp();
              if (lane == 0) {
                const int pk = lds(&B.dec[o]);
                sz[pk & 0xffff] += w;
                sz[pk >> 16] -= w;
              }
              __syncwarp();
              amin = -1;
            }
            group(__ldg(&B.iso_before[z]), __ldg(&B.iso_before[z + 1]));
          }
          nmoved = warp_sum64(nmoved);
          if (lane == 0 && nmoved) {
            atomicAdd((unsigned long long*)&I.moves[it], (unsigned long long)nmoved);
            atomicAdd(&B.stats[2], (unsigned long long)nmoved);
          }
        }
        __syncthreads();
      }
      if (ns) {
        // the other parity's tallies are cleared for the next window with
        // whole-grid vertices
        const size_t ob = (size_t)(hp ^ 1) * kMaxGridVerts * K;
        for (int p = gtid; p < kMaxGridVerts * K; p += gthreads) {
          B.hcnt[ob + p] = 0;
          B.hfirst[ob + p] = ~0ull;
          B.hgain[ob + p] = 0;
          B.hloss[ob + p] = 0;
          B.hadelta[ob + p] = 0;
        }
        if (gtid < 8 * kMaxGridVerts) B.hmisc[(hp ^ 1) * 8 * kMaxGridVerts + gtid] = 0;
        if (gtid == 0) B.stats[1] += ns;
        heavy_round++;
      }
      if (metric == kTV) {
        // marker = last scanner of each part among the committed positions: each
        // warp offers the last of its own positions per part, stamped with the
        // window (round + 1), and the next round state reads the maximum
        const int zc = min(z1, cut);
        const unsigned long long stamp = (unsigned long long)(round + 1) << 32;
        for (int wd = lane; wd < words; wd += 32) {
          uint32_t seen = 0;
          for (int z = zc - 1; z >= z0 && seen != ~0u; z--) {
            uint32_t m = lds(&B.scan[(size_t)(z - pos) * words + wd]) & ~seen;
            seen |= m;
            while (m) {
              const int b = __ffs(m) - 1;
              m &= m - 1;
              atomicMax(&B.mlast[wd * 32 + b], stamp | (unsigned)z);
            }
          }
        }
      }
      if (gw == 0 && lane == 0) {
        B.ctl[2 + (par ^ 1)] = kNone;
        B.ctab_over[par ^ 1] = 0;
        B.mcnt[par ^ 1] = 0;
      }
      prev_maxtouch = mt_c < cut;
      if (cut == end_w) {
        if (end_w == pos + W) W = min(2 * W, B.wmax);
      } else {
        // regrow from the last valid length
        W = min(B.wmax, max(B.wmin > 0 ? B.wmin : nwarps, B.wgrow * (cut - pos)));
      }
      pos = cut;
      round++;
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tC = gtimer();
        B.stats[18] += tC - tA;
        tA = tC;
      }
    }
  }
  if (metric == kTV && blockIdx.x == 0) {
    // markers of the last window (the loop's final barrier made them visible)
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
      const unsigned long long ml = lds(&B.mlast[p]);
      if (round > 0 && (int)(ml >> 32) == round) I.marker[p] = __ldg(&B.porder[(int)(ml & 0xffffffffu)]);
    }
  }
}

}  // namespace

size_t spec_ldg_smem_bytes(int K) {
  auto a = [](size_t n) { return (n + 15) & ~size_t(15); };
  const size_t k4 = a(sizeof(int) * K);
  return 5 * k4 + 4 * a(sizeof(int) * (size_t)K * kSWarps) + a(sizeof(unsigned long long) * (size_t)K * kSWarps);
}

cudaError_t launch_spec_ldg(const DevInstance& I, const SpecBuf& B, int passes, int num_sms, cudaStream_t st,
                            int* grid_out) {
  const size_t smem = spec_ldg_smem_bytes(I.K);
  const void* fn = (const void*)spec_ldg_kernel;
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
