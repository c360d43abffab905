// Streaming initial partitioners (host side).
//
// Each metric's partition_gpu() in the reference first runs its CPU streaming
// partitioner and then hands the resulting state to the GPU; the same split is
// kept here.  These produce the refinement input: part vector, ordered per-net
// part lists, part sizes, and the metric's auxiliary state.
//
//   LDG stream  (TV, MSV, MSRV): TV/partition.cpp:207-264, MGV/partition.cpp:122-189,
//                                MSRV/partition.cpp:123-196
//   CN stream   (uncut nets):    CN/partition.cpp:132-221
//   message-greedy (TM, MSM):    TM/partition.cpp:87-250, MSM/partition.cpp:146-309

#include "fp_internal.h"

#include <algorithm>

namespace fp {

namespace {

inline int list_find(const int* part, int len, int p) {
  for (int j = 0; j < len; j++)
    if (part[j] == p) return j;
  return -1;
}

// Increments part p in net e, appending it when absent.  Returns the slot.
inline int list_add(HostState& st, int e, int p) {
  int s = st.ep_start[e];
  int j = list_find(&st.ep_part[s], st.ep_len[e], p);
  if (j >= 0) {
    st.ep_cnt[s + j]++;
    return j;
  }
  j = st.ep_len[e]++;
  st.ep_part[s + j] = p;
  st.ep_cnt[s + j] = 1;
  return j;
}

// list_add when `left` more of the current vertex's nets are known to list p
// (a vertex lists no net twice): once they are found, p is appended to the
// remaining nets without a search.
inline int list_add_known(HostState& st, int e, int p, int& left) {
  const int s = st.ep_start[e];
  if (left > 0) {
    const int j = list_find(&st.ep_part[s], st.ep_len[e], p);
    if (j >= 0) {
      st.ep_cnt[s + j]++;
      left--;
      return j;
    }
  }
  const int j = st.ep_len[e]++;
  st.ep_part[s + j] = p;
  st.ep_cnt[s + j] = 1;
  return j;
}

// The streams read, per (vertex, net) pair in visiting order, the net's list
// header and then its list: two dependent misses on a random net.  A cursor
// walks the same pair sequence ahead of the stream and requests both early:
// headers kHdrAhead pairs ahead, lists (their header now cached) kListAhead
// pairs ahead.
struct PairAhead {
  const Problem& pb;
  const HostState& st;
  int z = 0;
  uint32_t i = 0, end = 0;
  PairAhead(const Problem& p, const HostState& s) : pb(p), st(s) { seek(0); }
  void seek(int zz) {
    const HostGraph& g = *pb.g;
    for (z = zz; z < g.nov; z++) {
      const int v = pb.order[z];
      i = g.vptr[v];
      end = g.vptr[v + 1];
      if (i < end) return;
    }
  }
  // Net of the cursor's pair, or -1 past the last pair; then one pair on.
  int next() {
    if (z >= pb.g->nov) return -1;
    const int e = (int)pb.g->vnets[i];
    if (++i == end) seek(z + 1);
    return e;
  }
};

constexpr int kHdrAhead = 64;
constexpr int kListAhead = 16;

struct Prefetcher {
  PairAhead hdr, list;
  Prefetcher(const Problem& pb, const HostState& st) : hdr(pb, st), list(pb, st) {
    for (int k = 0; k < kHdrAhead; k++) header(hdr.next());
    for (int k = 0; k < kListAhead; k++) body(list.next());
  }
  void header(int e) {
    if (e < 0) return;
    __builtin_prefetch(&hdr.st.ep_len[e]);
    __builtin_prefetch(&hdr.st.ep_start[e]);
  }
  void body(int e) {
    if (e < 0) return;
    const int s = list.st.ep_start[e];
    __builtin_prefetch(&list.st.ep_part[s]);
    __builtin_prefetch(&list.st.ep_cnt[s]);
  }
  // Called once per pair the stream reads.
  void step() {
    header(hdr.next());
    body(list.next());
  }
};

// The least-loaded part (the lowest index among the smallest sizes), the
// streams' fallback: a tournament tree over the K part sizes, updated after each
// assignment in O(log K).  Most vertices of a heavy-tailed instance have no
// nets and take this fallback, so a scan of all K sizes per vertex would
// dominate the stream.
struct LeastLoaded {
  const std::vector<int>& sizes;
  int n = 1;
  std::vector<int> win;   // win[x]: winning part of node x's subtree, -1 = padding
  explicit LeastLoaded(const std::vector<int>& s) : sizes(s) {
    const int K = (int)s.size();
    while (n < K) n <<= 1;
    win.assign(2 * (size_t)n, -1);
    for (int k = 0; k < K; k++) win[n + k] = k;
    for (int x = n - 1; x >= 1; x--) win[x] = pick(win[2 * x], win[2 * x + 1]);
  }
  // a from the left subtree (lower indices), b from the right one
  int pick(int a, int b) const {
    if (a < 0) return b;
    if (b < 0) return a;
    return sizes[b] < sizes[a] ? b : a;
  }
  void changed(int k) {
    for (int x = (n + k) >> 1; x >= 1; x >>= 1) win[x] = pick(win[2 * x], win[2 * x + 1]);
  }
  int argmin() const { return win[1]; }
};

// LDG decision over the parts seen by the current vertex, in first-seen order:
// highest score * (1 - size / C) above zero, ties to the smaller part, then to
// the earlier part; if no part scores, the least loaded part (lowest index).
int ldg_decide(const Problem& pb, const HostState& st, const std::vector<int>& seen, int nseen,
               const std::vector<int>& count, const LeastLoaded& least) {
  double best = 0;
  int arg = -1;
  for (int i = 0; i < nseen; i++) {
    int p = seen[i];
    // Sizes are never negative, so a score is at most its count: a part whose
    // count is below the best score can neither beat nor tie it.
    if (arg >= 0 && count[p] < best) continue;
    double pen = 1 - (1.0 * st.part_sizes[p] / pb.C);
    double sc = (double)count[p] * pen;
    if (sc > 0 && (arg == -1 || sc > best || (sc == best && st.part_sizes[p] < st.part_sizes[arg]))) {
      best = sc;
      arg = p;
    }
  }
  return arg >= 0 ? arg : least.argmin();
}

void state_alloc(const Problem& pb, HostState& st) {
  const HostGraph& g = *pb.g;
  st.part_vec.assign(g.nov, -1);
  st.part_sizes.assign(pb.K, 0);
  st.ep_start.assign(g.nptr.begin(), g.nptr.end());
  st.ep_len.assign(g.noe, 0);
  st.ep_part.assign(g.pins, -1);
  st.ep_cnt.assign(g.pins, 0);
  st.marker.assign(pb.K, -1);
  st.send.assign(pb.K, 0);
  st.recv.assign(pb.K, 0);
  st.msgs.assign(pb.K, 0);
  st.conn.clear();
}

int stream_ldg(const Problem& pb, HostState& st) {
  const HostGraph& g = *pb.g;
  const int K = pb.K;
  const bool vol = pb.metric == FP_METRIC_MSV || pb.metric == FP_METRIC_MSRV;
  const bool rv = pb.metric == FP_METRIC_MSRV;
  const int max_pw = (int)(pb.xw + (pb.xw * 0.1));
  // count[p]: listed entries of part p over v's nets (zero between vertices);
  // seen: the parts in first-seen order (one spare slot for the branch-free
  // append).  marker[p] = v for every part v saw, as the reference leaves it.
  std::vector<int> seen(K + 1), count(K, 0);
  LeastLoaded least(st.part_sizes);
  Prefetcher pf(pb, st);
  for (int z = 0; z < g.nov; z++) {
    const int v = pb.order[z];
    int nseen = 0;
    for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      pf.step();
      const int e = (int)g.vnets[i];
      const int* lp = &st.ep_part[st.ep_start[e]];
      const int len = st.ep_len[e];
      for (int j = 0; j < len; j++) {
        const int p = lp[j];
        seen[nseen] = p;
        nseen += count[p]++ == 0;
      }
    }
    const int d = ldg_decide(pb, st, seen, nseen, count, least);
    // TV's LDG2 sends a part above max_pw back to the vertex's current part,
    // which is -1 during the stream (TV/partition.cpp:135-138).
    if (pb.metric == FP_METRIC_TV && st.part_sizes[d] > max_pw) return FP_ERR_UNSUPPORTED;
    int left = count[d];   // nets of v that list d
    for (int i = 0; i < nseen; i++) {
      st.marker[seen[i]] = v;
      count[seen[i]] = 0;
    }
    st.part_sizes[d] += pb.w[v];
    if (pb.w[v]) least.changed(d);
    st.part_vec[v] = d;
    for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      const int e = (int)g.vnets[i];
      if (!vol) {
        list_add_known(st, e, d, left);
        continue;
      }
      const int s = st.ep_start[e];
      const int sv = g.src[e];
      const int sp = st.part_vec[sv];
      if (sv == v) {
        for (int j = 0; j < st.ep_len[e]; j++) {
          const int p = st.ep_part[s + j];
          if (p != sp) {
            st.send[sp]++;
            if (rv) st.recv[p]++;
          }
        }
      }
      const int before = st.ep_len[e];
      list_add_known(st, e, d, left);
      if (st.ep_len[e] != before && sv != v && sp != -1) {
        st.send[sp]++;
        if (rv) st.recv[d]++;
      }
    }
  }
  return FP_OK;
}

int stream_cn(const Problem& pb, HostState& st) {
  const HostGraph& g = *pb.g;
  std::vector<int> seen(pb.K), count(pb.K, 0), mark(pb.K, -1);
  LeastLoaded least(st.part_sizes);
  Prefetcher pf(pb, st);
  for (int z = 0; z < g.nov; z++) {
    const int v = pb.order[z];
    int nseen = 0;
    for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      pf.step();
      const int e = (int)g.vnets[i];
      if (st.ep_len[e] != 1) continue;
      const int p = st.ep_part[st.ep_start[e]];
      if (mark[p] != v) { mark[p] = v; count[p] = 1; seen[nseen++] = p; }
      else count[p]++;
    }
    const int d = ldg_decide(pb, st, seen, nseen, count, least);
    st.part_sizes[d] += pb.w[v];
    if (pb.w[v]) least.changed(d);
    st.part_vec[v] = d;
    for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_add(st, (int)g.vnets[i], d);
  }
  return FP_OK;
}

int stream_msg(const Problem& pb, HostState& st) {
  const HostGraph& g = *pb.g;
  const int K = pb.K;
  st.conn.assign((size_t)K * K, 0);
  if (pb.metric == FP_METRIC_MSM)
    for (int i = 0; i < K; i++) st.conn[(size_t)i * K + i] = -1;
  // conn > 0 as bit sets by row and by column.  The stream only raises
  // connection counts, so a bit is set once, when its count leaves 0.
  const int W = (K + 63) / 64;
  std::vector<uint64_t> prow((size_t)K * W, 0), pcol((size_t)K * W, 0);
  std::vector<int> rowcnt(K, 0), colcnt(K, 0);      // set bits per row / column
  auto set_pos = [&](int a, int b) {
    prow[(size_t)a * W + (b >> 6)] |= 1ull << (b & 63);
    pcol[(size_t)b * W + (a >> 6)] |= 1ull << (a & 63);
    rowcnt[a]++;
    colcnt[b]++;
  };
  std::vector<int> saved(K);
  const uint64_t last_mask = (K & 63) ? (1ull << (K & 63)) - 1 : ~0ull;
  // saved[k] -= amount for every k < K whose bit in `bits` is clear
  auto sub_zeros = [&](const uint64_t* bits, int amount) {
    for (int x = 0; x < W; x++) {
      uint64_t zb = ~bits[x];
      if (x == W - 1) zb &= last_mask;
      for (; zb; zb &= zb - 1) saved[x * 64 + __builtin_ctzll(zb)] -= amount;
    }
  };
  std::vector<int> smark(K, -1), src_part(g.noe, -1), mult(K, 0);
  std::vector<int> act_parts, act_nets, own_nets, mparts, dcount;
  std::vector<uint64_t> act(W), planes;
  LeastLoaded least(st.part_sizes);
  for (int z = 0; z < g.nov; z++) {
    const int v = pb.order[z];
    act_parts.clear();
    act_nets.clear();
    own_nets.clear();
    for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      const int e = (int)g.vnets[i];
      if (g.src[e] == v) own_nets.push_back(e);
      const int sp = src_part[e];
      if (sp != -1) {
        if (smark[sp] != v) { smark[sp] = v; act_parts.push_back(sp); }
        act_nets.push_back((int)(i - g.vptr[v]));   // index among v's nets
      }
    }
    // Part saving the most messages among parts below capacity; ties to the
    // smaller part, then the lower index.  saved(k) counts the active source
    // parts sp with conn[sp][k] > 0, and over the vertex's own nets every
    // listed part p with conn[k][p] > 0 (TM/partition.cpp:113-150): the first
    // sum is a popcount of column k under the active-part mask, the second one
    // of row k under the bit planes of each part's multiplicity.
    std::fill(act.begin(), act.end(), 0);
    for (int sp : act_parts) act[sp >> 6] |= 1ull << (sp & 63);
    mparts.clear();
    int mmax = 0;
    for (int e : own_nets) {
      const int s = st.ep_start[e];
      for (int j = 0; j < st.ep_len[e]; j++) {
        const int p = st.ep_part[s + j];
        if (mult[p]++ == 0) mparts.push_back(p);
        mmax = std::max(mmax, mult[p]);
      }
    }
    int best = -1, arg = -1;
    // With no active source part and no listed part on its own nets, a vertex
    // saves nothing anywhere: the loop below would pick the smallest part below
    // capacity (lowest index first), which is the least-loaded part, the same
    // as the fallback when no part is below capacity.
    const bool idle = act_parts.empty() && mmax == 0;
    int nplanes = 0;
    while ((mmax >> nplanes) != 0) nplanes++;
    // The same saved(k) two ways, the cheaper per vertex: popcounts over every
    // part (K * W * (1 + planes) words), or -- once most counts are positive --
    // the largest possible saving less the clear bits of the active parts'
    // rows (conn[sp][k] == 0) and of the listed parts' columns
    // (conn[k][p] == 0, weighted by the part's multiplicity).
    long long zcost = K;
    for (int sp : act_parts) zcost += W + (K - rowcnt[sp]);
    for (int p : mparts) zcost += W + (K - colcnt[p]);
    if (!idle && zcost < (long long)K * W * (1 + nplanes)) {
      int msum = 0;
      for (int p : mparts) msum += mult[p];
      std::fill(saved.begin(), saved.end(), (int)act_parts.size() + msum);
      for (int sp : act_parts) sub_zeros(&prow[(size_t)sp * W], 1);
      for (int p : mparts) sub_zeros(&pcol[(size_t)p * W], mult[p]);
      for (int p : mparts) mult[p] = 0;
      for (int k = 0; k < K; k++) {
        if (!(st.part_sizes[k] < pb.C)) continue;
        if (saved[k] > best || (saved[k] == best && st.part_sizes[k] < st.part_sizes[arg])) { best = saved[k]; arg = k; }
      }
    } else {
      planes.assign((size_t)nplanes * W, 0);
      for (int p : mparts)
        for (int b = 0; b < nplanes; b++)
          if ((mult[p] >> b) & 1) planes[(size_t)b * W + (p >> 6)] |= 1ull << (p & 63);
      for (int p : mparts) mult[p] = 0;
      for (int k = idle ? K : 0; k < K; k++) {
        if (!(st.part_sizes[k] < pb.C)) continue;
        const uint64_t* col = &pcol[(size_t)k * W];
        const uint64_t* row = &prow[(size_t)k * W];
        int sv = 0;
        for (int x = 0; x < W; x++) sv += __builtin_popcountll(col[x] & act[x]);
        for (int b = 0; b < nplanes; b++) {
          int c = 0;
          for (int x = 0; x < W; x++) c += __builtin_popcountll(row[x] & planes[(size_t)b * W + x]);
          sv += c << b;
        }
        if (sv > best || (sv == best && st.part_sizes[k] < st.part_sizes[arg])) { best = sv; arg = k; }
      }
    }
    const int d = arg >= 0 ? arg : least.argmin();
    st.part_vec[v] = d;
    st.part_sizes[d] += pb.w[v];
    if (pb.w[v]) least.changed(d);
    // d's count in each of v's nets after adding v (the reference looks it up
    // again, TM/partition.cpp:210-223)
    dcount.resize(g.vptr[v + 1] - g.vptr[v]);
    for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      const int e = (int)g.vnets[i];
      const int j = list_add(st, e, d);
      dcount[i - g.vptr[v]] = st.ep_cnt[st.ep_start[e] + j];
    }
    for (int k : act_nets) {
      const int e = (int)g.vnets[g.vptr[v] + k];
      const int sp = src_part[e];
      if (sp == d) continue;
      int& c = st.conn[(size_t)sp * K + d];
      if (c == 0) {
        st.msgs[sp]++;
        c = 1;
        set_pos(sp, d);
      } else if (dcount[k] == 1) {
        c++;
      }
    }
    for (int e : own_nets) {
      src_part[e] = d;
      const int s = st.ep_start[e];
      for (int j = 0; j < st.ep_len[e]; j++) {
        const int p = st.ep_part[s + j];
        if (p == d) continue;
        int& c = st.conn[(size_t)d * K + p];
        if (c == 0) { st.msgs[d]++; c = 1; set_pos(d, p); }
        else c++;
      }
    }
  }
  return FP_OK;
}

}  // namespace

int initial_partition(const Problem& pb, HostState& st) {
  state_alloc(pb, st);
  switch (pb.metric) {
    case FP_METRIC_TV:
    case FP_METRIC_MSV:
    case FP_METRIC_MSRV: return stream_ldg(pb, st);
    case FP_METRIC_CN: return stream_cn(pb, st);
    case FP_METRIC_TM:
    case FP_METRIC_MSM: return stream_msg(pb, st);
    default: return FP_ERR_INVALID;
  }
}

}  // namespace fp
