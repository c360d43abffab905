// Speculative grid-wide refinement for CN (CN/partition.cpp:245-377): the walk
// goes over the nets in id order; a net with exactly two parts moves all pins
// of its smaller side to the other part, unless one of those pins is in a net
// that is not cut.
//
// A round covers a window of nets; every warp decides its nets against the
// current state.  Claims are stamped with the round number, so they never need
// to be cleared.  A net that will move pins ("acting") claims every net of
// those pins (its write set); a later net is invalid if anything it read --
// its own part list, the uncut net that kept it from acting, or the nets of
// its smaller side -- was claimed by an earlier acting net.  The first invalid
// net cuts the window; acting nets before the cut are applied concurrently
// (their write sets are disjoint).
//
// An acting net moves its pins one at a time in the reference, each move
// updating every net of the pin.  All of them move old -> new, so the k moves
// that land on one net have a result that depends on k only (cn_apply_net);
// the commit counts the moves per net, then updates each touched net once.

#include "fp_spec_common.cuh"

namespace fp {

namespace {

using namespace spec;

// Round-stamped claim: the latest round wins, then the smallest position.
__device__ __forceinline__ unsigned long long ckey(int round, int pos) {
  return ((unsigned long long)(unsigned)round << 32) | (0xffffffffu - (unsigned)pos);
}
// Did a net position earlier than `pos` claim net x in this round?
__device__ __forceinline__ bool claim_before(const SpecBuf& B, int round, int x, int pos) {
  const unsigned long long c = lds(&B.claim64[x]);
  return (int)(c >> 32) == round && (int)(0xffffffffu - (unsigned)(c & 0xffffffffu)) < pos;
}

// Walk of the (pin, net) pairs of net e's pins [pb, pe) on part oldp, 32 pins
// at a time, the pairs flattened across the warp with 4 loads in flight per
// lane.
//   kMode 0: returns a net of those pins that is not cut (-1: none);
//   kMode 1: claims every such net for position e and records the pins to move
//            (window offset o, round parity par); returns -1;
//   kMode 2: returns 1 if an acting net before e claimed one of them, else -1.
// Modes 0 and 2 stop early when *stop (shared by the warps splitting a net's
// pins) is set.
// gstop: the same in global memory (the grid's warps splitting a net).
template <int kMode>
__device__ int cn_walk_range(const DevInstance& I, const SpecBuf& B, int e, int pb, int pe, int oldp, int round,
                             int o, int par, const volatile int* stop, const int* gstop = nullptr) {
  const int lane = threadIdx.x & 31;
  for (int b0 = pb; b0 < pe; b0 += 32) {
    if (kMode != 1 && stop && __shfl_sync(kAll, *stop, 0)) return -1;   // warp-uniform: lane 0's read
    if (kMode != 1 && gstop && __shfl_sync(kAll, lds(gstop), 0)) return -1;
    const int k = b0 + lane;
    int u = -1, d = 0;
    uint32_t ub = 0;
    if (k < pe) {
      u = (int)__ldg(&I.npins[k]);
      if (lds(&I.part_vec[u]) == oldp) {
        ub = __ldg(&I.vptr[u]);
        d = (int)(__ldg(&I.vptr[u + 1]) - ub);
      } else {
        u = -1;
      }
    }
    if (kMode == 0) {
      // a pin's cached witness: a net of the pin found uncut before; still
      // uncut, it ends the search without walking the pin's nets (hub pins
      // lie on millions of nets)
      const int w = u >= 0 ? lds(&B.cn_wit[u]) : -1;
      const int hit = (w >= 0 && lds(&I.ep_len[w]) == 1) ? w : -1;
      const unsigned m = __ballot_sync(kAll, hit >= 0);
      if (m) return __shfl_sync(kAll, hit, __ffs(m) - 1);
    }
    if (kMode == 1 && u >= 0) B.cn_moved[atomicAdd(&B.cn_cnt[par], 1)] = make_int2(u, o);
    int incl = d;
    for (int off = 1; off < 32; off <<= 1) {
      const int t = __shfl_up_sync(kAll, incl, off);
      if (lane >= off) incl += t;
    }
    const int total = __shfl_sync(kAll, incl, 31);
    constexpr int kU = 4;
    for (int f0 = 0; f0 < total; f0 += 32 * kU) {
      int xs[kU];
#pragma unroll
      for (int q = 0; q < kU; q++) {
        const int f = f0 + q * 32 + lane;
        int lo = 0, hi = 31;
#pragma unroll
        for (int it = 0; it < 5; it++) {
          const int mid = (lo + hi) >> 1;
          const int val = __shfl_sync(kAll, incl, mid);
          if (f < val) hi = mid; else lo = mid + 1;
        }
        const uint32_t bl = __shfl_sync(kAll, ub, lo);
        const int dl = __shfl_sync(kAll, d, lo);
        const int il = __shfl_sync(kAll, incl, lo);
        xs[q] = f < total ? (int)__ldg(&I.vnets[bl + (uint32_t)(f - (il - dl))]) : -1;
      }
      if (kMode == 0) {
        int hit = -1, hq = 0;
#pragma unroll
        for (int q = 0; q < kU; q++)
          if (xs[q] >= 0 && hit < 0 && lds(&I.ep_len[xs[q]]) == 1) { hit = xs[q]; hq = q; }
        const unsigned m = __ballot_sync(kAll, hit >= 0);
        if (m) {
          const int src = __ffs(m) - 1;
          const int x = __shfl_sync(kAll, hit, src);
          // the pin of that pair keeps it as its witness
          const int f = f0 + __shfl_sync(kAll, hq, src) * 32 + src;
          int lo = 0, hi = 31;
#pragma unroll
          for (int it = 0; it < 5; it++) {
            const int mid = (lo + hi) >> 1;
            const int val = __shfl_sync(kAll, incl, mid);
            if (f < val) hi = mid; else lo = mid + 1;
          }
          const int uw = __shfl_sync(kAll, u, lo);
          if (lane == 0 && uw >= 0) B.cn_wit[uw] = x;
          return x;
        }
      } else if (kMode == 1) {
#pragma unroll
        for (int q = 0; q < kU; q++)
          if (xs[q] >= 0) atomicMax(&B.claim64[xs[q]], ckey(round, e));
      } else {
        bool c = false;
#pragma unroll
        for (int q = 0; q < kU; q++)
          if (xs[q] >= 0 && claim_before(B, round, xs[q], e)) c = true;
        if (__any_sync(kAll, c)) return 1;
      }
    }
  }
  return -1;
}

template <int kMode>
__device__ __forceinline__ int cn_walk(const DevInstance& I, const SpecBuf& B, int e, int oldp, int round, int o,
                                       int par) {
  return cn_walk_range<kMode>(I, B, e, (int)__ldg(&I.nptr[e]), (int)__ldg(&I.nptr[e + 1]), oldp, round, o, par,
                              nullptr);
}

// Warp gw's contiguous share (of nw warps) of net e's pins.
__device__ __forceinline__ void cn_grid_share(const DevInstance& I, int e, int gw, int nw, int* pb, int* pe) {
  const int b = (int)__ldg(&I.nptr[e]), n = (int)__ldg(&I.nptr[e + 1]) - b;
  const int g = (n + nw - 1) / nw;
  *pb = b + min(gw * g, n);
  *pe = b + min(gw * g + g, n);
}

// Two-part test of net e (CN/partition.cpp:262-270): old (smaller side) and
// new parts, false if the net does not span exactly two parts.
__device__ __forceinline__ bool cn_two(const DevInstance& I, int e, int* oldp, int* newp, int* oldc = nullptr) {
  if (lds(&I.ep_len[e]) != 2) return false;
  const int s = (int)__ldg(&I.nptr[e]);
  const int p1 = lds(&I.ep_part[s]), c1 = lds(&I.ep_cnt[s]);
  const int p2 = lds(&I.ep_part[s + 1]), c2 = lds(&I.ep_cnt[s + 1]);
  *oldp = c1 < c2 ? p1 : p2;
  *newp = c1 < c2 ? p2 : p1;
  if (oldc) *oldc = c1 < c2 ? c1 : c2;
  return true;
}

// Warp wib's contiguous share of net e's pins.
__device__ __forceinline__ void cn_pin_share(const DevInstance& I, int e, int* pb, int* pe) {
  const int b = (int)__ldg(&I.nptr[e]), n = (int)__ldg(&I.nptr[e + 1]) - b;
  const int g = (n + kSWarps - 1) / kSWarps, w = (int)(threadIdx.x >> 5);
  *pb = b + min(w * g, n);
  *pe = b + min(w * g + g, n);
}

// Evaluation of a net with many pins by the whole CTA: the warps split its
// pins (cn_eval's rules), then the claims of an acting net.
__device__ void cn_eval_cta(const DevInstance& I, const SpecBuf& B, int e, int o, int round, int par, bool logp) {
  __shared__ int sh_two, sh_old, sh_new, sh_unc, sh_cold;
  __shared__ volatile int sh_stop;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    sh_two = 0;
    sh_unc = -1;
    sh_stop = 0;
    if (lds(&I.ep_len[e]) == 2) {
      const int s = (int)__ldg(&I.nptr[e]);
      const int p1 = lds(&I.ep_part[s]), c1 = lds(&I.ep_cnt[s]);
      const int p2 = lds(&I.ep_part[s + 1]), c2 = lds(&I.ep_cnt[s + 1]);
      sh_two = 1;
      sh_old = c1 < c2 ? p1 : p2;
      sh_new = c1 < c2 ? p2 : p1;
      sh_cold = c1 < c2 ? c1 : c2;
    }
  }
  __syncthreads();
  int act = 0;
  const int oldp = sh_two ? sh_old : 0, newp = sh_two ? sh_new : 0;
  if (sh_two) {
    int pb, pe;
    cn_pin_share(I, e, &pb, &pe);
    const int hit = cn_walk_range<0>(I, B, e, pb, pe, oldp, 0, 0, 0, &sh_stop);
    if (hit >= 0 && lane == 0) {
      atomicCAS(&sh_unc, -1, hit);   // any uncut net is a witness
      sh_stop = 1;
    }
    __syncthreads();
    act = sh_unc < 0;
    if (act) cn_walk_range<1>(I, B, e, pb, pe, oldp, round, o, par, nullptr);
  }
  if (threadIdx.x == 0) {
    B.dec[o] = (oldp << 16) | newp;
    B.flag[o] = (unsigned char)act;
    B.slack[o] = sh_unc;   // the uncut net that blocks the move (-1: none)
    if (logp) B.rgain[o] = sh_two ? sh_cold : -1;
  }
  __syncthreads();
}

// Validation of a net with many pins by the whole CTA (the warp loop's rules);
// a conflict lowers the cut word.
__device__ void cn_validate_cta(const DevInstance& I, const SpecBuf& B, int e, int o, int round, int* cut) {
  __shared__ volatile int sh_conf;
  const int lane = threadIdx.x & 31;
  const int act = lds(&B.flag[o]);
  if (threadIdx.x == 0) {
    int c = claim_before(B, round, e, e) ? 1 : 0;
    const int unc = lds(&B.slack[o]);
    if (unc >= 0 && claim_before(B, round, unc, e)) c = 1;
    sh_conf = c;
  }
  __syncthreads();
  if (act && !sh_conf) {
    int pb, pe;
    cn_pin_share(I, e, &pb, &pe);
    if (cn_walk_range<2>(I, B, e, pb, pe, lds(&B.dec[o]) >> 16, round, 0, 0, &sh_conf) > 0 && lane == 0) sh_conf = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0 && sh_conf) atomicMin(cut, (e << 3) | 5);
  __syncthreads();
}

// Evaluation of net e (one warp).  Returns 0 (no move), 1 (acting), and the
// old / new parts; *uncut = a net proving "no move" (-1 if e is not two-part).
__device__ int cn_eval(const DevInstance& I, const SpecBuf& B, int e, int* oldp_o, int* newp_o, int* uncut,
                       int* oldc_o) {
  *uncut = -1;
  *oldc_o = -1;
  if (lds(&I.ep_len[e]) != 2) return 0;
  const int s = (int)__ldg(&I.nptr[e]);
  const int p1 = lds(&I.ep_part[s]), c1 = lds(&I.ep_cnt[s]);
  const int p2 = lds(&I.ep_part[s + 1]), c2 = lds(&I.ep_cnt[s + 1]);
  const int oldp = c1 < c2 ? p1 : p2;
  const int newp = c1 < c2 ? p2 : p1;
  *oldp_o = oldp;
  *newp_o = newp;
  *oldc_o = c1 < c2 ? c1 : c2;
  // any pin on the smaller side with a net that is not cut?
  *uncut = cn_walk<0>(I, B, e, oldp, 0, 0, 0);
  return *uncut < 0 ? 1 : 0;
}

// k moves oldp -> newp of pins of net x, each the reference's REMOVAL then
// ADDING on x's list (CN/partition.cpp:311-370), applied at once by one warp:
// the lanes find the two slots, lane 0 replays the k steps.  Only the first
// step can append newp and only the last can remove oldp, so the k-fold result
// follows from the counts.
__device__ void cn_apply_net(const DevInstance& I, int x, int oldp, int newp, int k) {
  const int lane = threadIdx.x & 31;
  const int s = (int)__ldg(&I.nptr[x]);
  const int cap = (int)__ldg(&I.nptr[x + 1]) - s;
  int n = lds(&I.ep_len[x]);
  int jo = -1, jd = -1;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    const int p = j < n ? lds(&I.ep_part[s + j]) : -1;
    const unsigned mo = __ballot_sync(kAll, p == oldp);
    const unsigned md = __ballot_sync(kAll, p == newp);
    if (mo && jo < 0) jo = j0 + __ffs(mo) - 1;
    if (md && jd < 0) jd = j0 + __ffs(md) - 1;
  }
  if (lane == 0) {
    int co = jo >= 0 ? lds(&I.ep_cnt[s + jo]) : 0;
    int cd = jd >= 0 ? lds(&I.ep_cnt[s + jd]) : 0;
    if (jo < 0 || n > cap || co < k || k < 1) {
      dev_fail(I.status, kDevErrInvalid);
    } else {
      bool ok = true;
      // oldp's count reached zero: the last entry fills its slot
      auto remove_old = [&]() {
        const int last = n - 1;
        if (last != jo) {
          if (last == jd) {
            I.ep_part[s + jo] = newp;
            jd = jo;
          } else {
            I.ep_part[s + jo] = lds(&I.ep_part[s + last]);
            I.ep_cnt[s + jo] = lds(&I.ep_cnt[s + last]);
          }
        }
        I.ep_part[s + last] = -1;
        I.ep_cnt[s + last] = 0;
        n = last;
        jo = -1;
      };
      auto append_new = [&]() {
        if (n >= cap) { ok = false; return; }
        jd = n;
        cd = 1;
        I.ep_part[s + jd] = newp;
        n++;
      };
      if (jd >= 0) {
        co -= k;
        cd += k;
        if (co == 0) remove_old();
      } else {
        co -= 1;   // first move
        if (co == 0) {
          remove_old();
          append_new();   // k == 1
        } else {
          append_new();
          co -= k - 1;    // the other k - 1 moves
          cd += k - 1;
          if (co == 0) remove_old();
        }
      }
      if (!ok) {
        dev_fail(I.status, kDevErrInvalid);
      } else {
        if (jo >= 0) I.ep_cnt[s + jo] = co;
        I.ep_cnt[s + jd] = cd;
        I.ep_len[x] = n;
      }
    }
  }
  __syncwarp();
}

// Three CTAs per SM: without the hint the compiler spills to fit more.
__global__ void __launch_bounds__(kSThreads, 3) spec_cn_kernel(DevInstance I, SpecBuf B, int passes) {
  barrier_start();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  // the window's grid-evaluated nets: id, two-part, old and new part
  __shared__ int s_ge[kMaxGridVerts], s_gt[kMaxGridVerts], s_go[kMaxGridVerts], s_gn[kMaxGridVerts];
  unsigned long long tA = gtimer();
  int round = 1;   // claims of round 0 (the cleared array) never match
  int heavy_round = 0;
  __shared__ int s_gc[kMaxGridVerts];
  for (int it = 0; it < passes; it++) {
    // decision records of the last pass: (new part, pins moved, old part,
    // acting) of a two-part net, (-1, 0, -1, 0) of any other net
    const bool logp = I.recs != nullptr && it == passes - 1;
    int pos = 0;
    int W = min(nwarps * 4, B.wmax);
    int hidx = 0;
    while (pos < I.noe) {
      const int par = round & 1;
      // a window holds up to gmax nets evaluated by the grid and ends before the next
      while (hidx < B.nheavy && __ldg(&B.heavy_pos[hidx]) < pos) hidx++;
      int end_w = min(pos + W, I.noe);
      if (hidx + B.gmax < B.nheavy) end_w = min(end_w, (int)__ldg(&B.heavy_pos[hidx + B.gmax]));
      int ns = 0;
      while (ns < B.gmax && hidx + ns < B.nheavy && __ldg(&B.heavy_pos[hidx + ns]) < end_w) ns++;
      const int hp = heavy_round & 1;
      // slot j of this parity in hmisc: [0] uncut witness + 1 (0: none), [1] conflict
      auto hm = [&](int j) { return B.hmisc + (hp * kMaxGridVerts + j) * 8; };
      if ((int)threadIdx.x < ns) {
        const int e = __ldg(&B.heavy_pos[hidx + threadIdx.x]);
        int op = 0, np = 0, oc = -1;
        s_ge[threadIdx.x] = e;
        s_gt[threadIdx.x] = cn_two(I, e, &op, &np, &oc) ? 1 : 0;
        s_go[threadIdx.x] = op;
        s_gn[threadIdx.x] = np;
        s_gc[threadIdx.x] = oc;
      }
      __syncthreads();
      // ---- A0: the grid's warps split the pins of each grid net (uncut search)
      for (int j = 0; j < ns; j++) {
        if (!s_gt[j]) continue;
        int pb, pe;
        cn_grid_share(I, s_ge[j], gw, nwarps, &pb, &pe);
        const int hit = cn_walk_range<0>(I, B, s_ge[j], pb, pe, s_go[j], 0, 0, 0, nullptr, hm(j));
        if (hit >= 0 && lane == 0) atomicCAS(hm(j), 0, hit + 1);
      }
      const int span = end_w - pos;
      const int q = (span + nwarps - 1) / nwarps;
      const int z0 = min(pos + gw * q, end_w);
      const int z1 = min(z0 + q, end_w);
      // ---- A: evaluate; acting nets claim the nets of the pins they move
      for (int e = z0; e < z1; e++) {
        const int o = e - pos;
        if ((int)(__ldg(&I.nptr[e + 1]) - __ldg(&I.nptr[e])) > B.cn_big) continue;   // the CTA evaluates it below
        int oldp = 0, newp = 0, unc = -1, oldc = -1;
        const int act = cn_eval(I, B, e, &oldp, &newp, &unc, &oldc);
        if (act) cn_walk<1>(I, B, e, oldp, round, o, par);
        if (lane == 0) {
          B.dec[o] = (oldp << 16) | newp;
          B.flag[o] = (unsigned char)act;
          B.slack[o] = unc;   // the uncut net that blocks the move (-1: none)
          if (logp) B.rgain[o] = oldc;
        }
        __syncwarp();
      }
      // nets with many pins of this CTA's positions: the whole CTA each
      const int cz0 = min(pos + blockIdx.x * kSWarps * q, end_w);
      const int cz1 = min(cz0 + kSWarps * q, end_w);
      for (int mi = lower_bound_pos(B.mid_pos, B.nmid, cz0); mi < B.nmid; mi++) {
        const int e = __ldg(&B.mid_pos[mi]);
        if (e >= cz1) break;
        cn_eval_cta(I, B, e, e - pos, round, par, logp);
      }
      if (!grid_barrier(B.bar, I.status)) return;
      if (ns) {
        // ---- A1: an acting grid net's claims and pins, split across the grid
        for (int j = 0; j < ns; j++) {
          const int e = s_ge[j], o = e - pos;
          const int unc = lds(hm(j)) - 1;
          const int act = s_gt[j] && unc < 0;
          if (act) {
            int pb, pe;
            cn_grid_share(I, e, gw, nwarps, &pb, &pe);
            cn_walk_range<1>(I, B, e, pb, pe, s_go[j], round, o, par, nullptr);
          }
          if (blockIdx.x == 0 && threadIdx.x == 0) {
            B.dec[o] = s_gt[j] ? (s_go[j] << 16) | s_gn[j] : 0;
            B.flag[o] = (unsigned char)act;
            B.slack[o] = s_gt[j] ? unc : -1;
            if (logp) B.rgain[o] = s_gt[j] ? s_gc[j] : -1;
          }
        }
        if (!grid_barrier(B.bar, I.status)) return;
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tE = gtimer();
        B.stats[16] += tE - tA;
        tA = tE;
      }
      // ---- B: validate against earlier acting nets' claims
      for (int e = z0; e < z1; e++) {
        const int o = e - pos;
        if ((int)(__ldg(&I.nptr[e + 1]) - __ldg(&I.nptr[e])) > B.cn_big) continue;   // validated by the CTA below
        const int act = lds(&B.flag[o]);
        bool conf = false;
        if (lane == 0) {
          if (claim_before(B, round, e, e)) conf = true;
          const int unc = lds(&B.slack[o]);
          if (unc >= 0 && claim_before(B, round, unc, e)) conf = true;
        }
        conf = __any_sync(kAll, conf);   // warp-uniform before the pin loop's votes
        if (act && !conf) conf = cn_walk<2>(I, B, e, lds(&B.dec[o]) >> 16, round, 0, 0) > 0;
        conf = __any_sync(kAll, conf);
        if (conf) {
          if (lane == 0) atomicMin(&B.ctl[par], (e << 3) | 5);
          break;
        }
      }
      __syncthreads();
      for (int mi = lower_bound_pos(B.mid_pos, B.nmid, cz0); mi < B.nmid; mi++) {
        const int e = __ldg(&B.mid_pos[mi]);
        if (e >= cz1) break;
        cn_validate_cta(I, B, e, e - pos, round, &B.ctl[par]);
      }
      for (int j = 0; j < ns; j++) {
        // a grid net: its own list and witness by every warp (cheap), its
        // moving pins' nets split across the grid
        const int e = s_ge[j], o = e - pos;
        const int unc = lds(&B.slack[o]);
        bool conf = claim_before(B, round, e, e) || (unc >= 0 && claim_before(B, round, unc, e));
        if (!conf && lds(&B.flag[o])) {
          int pb, pe;
          cn_grid_share(I, e, gw, nwarps, &pb, &pe);
          conf = cn_walk_range<2>(I, B, e, pb, pe, s_go[j], round, 0, 0, nullptr, hm(j) + 1) > 0;
          if (conf && lane == 0) atomicExch(hm(j) + 1, 1);
        }
        if (conf && lane == 0) atomicMin(&B.ctl[par], (e << 3) | 5);
      }
      if (!grid_barrier(B.bar, I.status)) return;
      const int cutw = lds(&B.ctl[par]);
      const int cut = cutw == kNone ? end_w : min(cutw >> 3, end_w);
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tB = gtimer();
        B.stats[0]++;
        B.stats[cutw == kNone ? 3 : 8]++;
        B.stats[9] += cut - pos;
        B.stats[17] += tB - tA;
        tA = tB;
      }
      if (cut <= pos) {
        if (threadIdx.x == 0) dev_fail(I.status, kDevErrInvalid);
        return;
      }
      if (logp) {
        for (int e = z0 + lane; e < min(z1, cut); e += 32) {
          const int o = e - pos;
          const int oc = lds(&B.rgain[o]);
          const int act = lds(&B.flag[o]) & 1;
          const int pk = lds(&B.dec[o]);
          I.recs[e] = oc >= 0 ? make_int4(pk & 0xffff, act ? oc : 0, pk >> 16, act) : make_int4(-1, 0, -1, 0);
        }
      }
      // ---- C1: pins of acting nets before the cut: part, sizes, moves per net
      const int nmv = lds(&B.cn_cnt[par]);
      for (int i = gw; i < nmv; i += nwarps) {
        const int2 mv = lds(&B.cn_moved[i]);
        if (pos + mv.y >= cut) continue;
        const int u = mv.x;
        const int pk = lds(&B.dec[mv.y]);
        const uint32_t ub = __ldg(&I.vptr[u]), ue = __ldg(&I.vptr[u + 1]);
        for (uint32_t j = ub + lane; j < ue; j += 32) {
          const int x = (int)__ldg(&I.vnets[j]);
          if (atomicAdd(&B.cn_kcnt[x], 1) == 0) B.cn_nets[atomicAdd(&B.cn_cnt[2 + par], 1)] = make_int2(x, pk);
        }
        if (lane == 0) {
          const int oldp = pk >> 16, newp = pk & 0xffff;
          I.part_vec[u] = newp;
          const int wv = __ldg(&I.w[u]);
          atomicAdd(&I.part_sizes[oldp], -wv);
          atomicAdd(&I.part_sizes[newp], wv);
          atomicAdd((unsigned long long*)&I.moves[it], 1ull);
          atomicAdd(&B.stats[2], 1ull);
        }
      }
      if (!grid_barrier(B.bar, I.status)) return;
      // ---- C2: every touched net once, with all of its moves
      const int nnet = lds(&B.cn_cnt[2 + par]);
      for (int i = gw; i < nnet; i += nwarps) {
        const int2 xe = lds(&B.cn_nets[i]);
        const int k = lds(&B.cn_kcnt[xe.x]);
        cn_apply_net(I, xe.x, xe.y >> 16, xe.y & 0xffff, k);
        if (lane == 0) B.cn_kcnt[xe.x] = 0;
      }
      if (gw == 0 && lane == 0) {
        B.ctl[par ^ 1] = kNone;
        B.cn_cnt[par ^ 1] = 0;
        B.cn_cnt[2 + (par ^ 1)] = 0;
      }
      if (ns) {
        // the other parity's grid-net words, for the next window with grid nets
        if (blockIdx.x == 0 && threadIdx.x < 8 * kMaxGridVerts) B.hmisc[(hp ^ 1) * 8 * kMaxGridVerts + threadIdx.x] = 0;
        if (blockIdx.x == 0 && threadIdx.x == 0) B.stats[1] += ns;
        heavy_round++;
      }
      if (cut == end_w) {
        if (end_w == pos + W) W = min(2 * W, B.wmax);
      } else {
        W = max(1024, min(B.wmax, 2 * (cut - pos)));
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
}

}  // namespace

cudaError_t launch_spec_cn(const DevInstance& I, const SpecBuf& B, int passes, int num_sms, cudaStream_t st,
                           int* grid_out) {
  const void* fn = (const void*)spec_cn_kernel;
  int per_sm = 0;
  cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSThreads, 0);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = per_sm * num_sms;
  if (grid * kSWarps > B.max_warps) grid = B.max_warps / kSWarps;
  if (grid_out) *grid_out = grid;
  DevInstance Ic = I;
  SpecBuf Bc = B;
  int p = passes;
  void* args[] = {&Ic, &Bc, &p};
  err = cudaLaunchCooperativeKernel(fn, grid, kSThreads, args, 0, st);
  if (err != cudaSuccess) return err;
  return cudaGetLastError();
}

}  // namespace fp
