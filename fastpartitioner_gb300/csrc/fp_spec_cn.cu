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
// (their write sets are disjoint), each moving its pins in net pin order.

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

// Evaluation of net e (one warp).  Returns 0 (no move), 1 (acting), and the
// old / new parts; *uncut = a net proving "no move" (-1 if e is not two-part).
__device__ int cn_eval(const DevInstance& I, int e, int* oldp_o, int* newp_o, int* uncut) {
  const int lane = threadIdx.x & 31;
  *uncut = -1;
  if (lds(&I.ep_len[e]) != 2) return 0;
  const int s = (int)__ldg(&I.nptr[e]);
  const int p1 = lds(&I.ep_part[s]), c1 = lds(&I.ep_cnt[s]);
  const int p2 = lds(&I.ep_part[s + 1]), c2 = lds(&I.ep_cnt[s + 1]);
  const int oldp = c1 < c2 ? p1 : p2;
  const int newp = c1 < c2 ? p2 : p1;
  *oldp_o = oldp;
  *newp_o = newp;
  const int pb = (int)__ldg(&I.nptr[e]), pe = (int)__ldg(&I.nptr[e + 1]);
  // any pin on the smaller side with a net that is not cut?
  for (int k = pb; k < pe; k++) {
    const int u = (int)__ldg(&I.npins[k]);
    if (lds(&I.part_vec[u]) != oldp) continue;
    const uint32_t ub = __ldg(&I.vptr[u]), ue = __ldg(&I.vptr[u + 1]);
    for (uint32_t j0 = ub; j0 < ue; j0 += 32) {
      const uint32_t j = j0 + lane;
      const int x = j < ue ? (int)__ldg(&I.vnets[j]) : -1;
      const bool unc = x >= 0 && lds(&I.ep_len[x]) == 1;
      const unsigned m = __ballot_sync(kAll, unc);
      if (m) {
        *uncut = __shfl_sync(kAll, x, __ffs(m) - 1);
        return 0;
      }
    }
  }
  return 1;
}

__global__ void __launch_bounds__(kSThreads) spec_cn_kernel(DevInstance I, SpecBuf B, int passes) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSWarps + wib;
  const int nwarps = gridDim.x * kSWarps;
  unsigned long long tA = gtimer();
  int round = 1;   // claims of round 0 (the cleared array) never match
  for (int it = 0; it < passes; it++) {
    int pos = 0;
    int W = min(nwarps * 4, B.wmax);
    while (pos < I.noe) {
      const int par = round & 1;
      const int end_w = min(pos + W, I.noe);
      const int span = end_w - pos;
      const int q = (span + nwarps - 1) / nwarps;
      const int z0 = min(pos + gw * q, end_w);
      const int z1 = min(z0 + q, end_w);
      // ---- A: evaluate; acting nets claim the nets of the pins they move
      for (int e = z0; e < z1; e++) {
        const int o = e - pos;
        int oldp = 0, newp = 0, unc = -1;
        const int act = cn_eval(I, e, &oldp, &newp, &unc);
        if (act) {
          const int pb = (int)__ldg(&I.nptr[e]), pe = (int)__ldg(&I.nptr[e + 1]);
          for (int k = pb; k < pe; k++) {
            const int u = (int)__ldg(&I.npins[k]);
            if (lds(&I.part_vec[u]) != oldp) continue;
            const uint32_t ub = __ldg(&I.vptr[u]), ue = __ldg(&I.vptr[u + 1]);
            for (uint32_t j = ub + lane; j < ue; j += 32) atomicMax(&B.claim64[__ldg(&I.vnets[j])], ckey(round, e));
          }
        }
        if (lane == 0) {
          B.dec[o] = (oldp << 16) | newp;
          B.flag[o] = (unsigned char)act;
          B.slack[o] = unc;   // the uncut net that blocks the move (-1: none)
        }
        __syncwarp();
      }
      if (!grid_barrier(B.bar, I.status)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long tE = gtimer();
        B.stats[16] += tE - tA;
        tA = tE;
      }
      // ---- B: validate against earlier acting nets' claims
      for (int e = z0; e < z1; e++) {
        const int o = e - pos;
        const int act = lds(&B.flag[o]);
        bool conf = false;
        if (lane == 0) {
          if (claim_before(B, round, e, e)) conf = true;
          const int unc = lds(&B.slack[o]);
          if (unc >= 0 && claim_before(B, round, unc, e)) conf = true;
        }
        conf = __any_sync(kAll, conf);   // warp-uniform before the pin loop's votes
        if (act && !conf) {
          const int oldp = lds(&B.dec[o]) >> 16;
          const int pb = (int)__ldg(&I.nptr[e]), pe = (int)__ldg(&I.nptr[e + 1]);
          for (int k = pb; k < pe && !conf; k++) {
            const int u = (int)__ldg(&I.npins[k]);
            if (lds(&I.part_vec[u]) != oldp) continue;
            const uint32_t ub = __ldg(&I.vptr[u]), ue = __ldg(&I.vptr[u + 1]);
            for (uint32_t j = ub + lane; j < ue; j += 32)
              if (claim_before(B, round, (int)__ldg(&I.vnets[j]), e)) conf = true;
            conf = __any_sync(kAll, conf);
          }
        }
        conf = __any_sync(kAll, conf);
        if (conf) {
          if (lane == 0) atomicMin(&B.ctl[par], (e << 3) | 5);
          break;
        }
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
      // ---- C: apply acting nets before the cut; clear every acting net's claims
      for (int e = z0; e < z1; e++) {
        const int o = e - pos;
        if (!lds(&B.flag[o])) continue;
        const int pk = lds(&B.dec[o]);
        const int oldp = pk >> 16, newp = pk & 0xffff;
        const int pb = (int)__ldg(&I.nptr[e]), pe = (int)__ldg(&I.nptr[e + 1]);
        if (e < cut) {
          // pins on the smaller side, in net pin order (CN/partition.cpp:311-370);
          // the side was fixed before any of them moved
          for (int k = pb; k < pe; k++) {
            const int u = (int)__ldg(&I.npins[k]);
            if (lds(&B.flag[o]) && lds(&I.part_vec[u]) != oldp) continue;
            const uint32_t ub = __ldg(&I.vptr[u]), ue = __ldg(&I.vptr[u + 1]);
            for (uint32_t j = ub + lane; j < ue; j += 32) commit_net(I, u, oldp, newp, (int)__ldg(&I.vnets[j]), nullptr);
            __syncwarp();
            if (lane == 0) {
              I.part_vec[u] = newp;
              const int wv = __ldg(&I.w[u]);
              atomicAdd(&I.part_sizes[oldp], -wv);
              atomicAdd(&I.part_sizes[newp], wv);
              atomicAdd((unsigned long long*)&I.moves[it], 1ull);
              atomicAdd(&B.stats[2], 1ull);
            }
            __syncwarp();
          }
        }
      }
      if (gw == 0 && lane == 0) B.ctl[par ^ 1] = kNone;
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
