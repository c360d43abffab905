// FastPartitioner CPU oracle -- TEST INFRASTRUCTURE ONLY.
//
// This file is the parity checker for the GB300 refinement engine.  It restates,
// single-threaded and loop for loop, the reference's sequential CPU path for the
// six metrics (streaming initial partition, REFI_ITER refinement passes, and the
// six metric evaluators).  Only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / reference legs may load it; the product library never links or
// calls it.
//
// Parity of this restatement is pinned against the reference itself: the recipe
// in oracle/Makefile compiles the reference's own partition.cpp / metric.cpp from
// its source tree into oracle/_ref/, and tests/golden/make_golden.py records the
// reference's final part vectors, per-net part lists and metric values on seeded
// inputs.  tests/test_oracle_golden.py checks this file against those fixtures.
//
// Reference files followed (paths inside the FastPartitioner tree):
//   TV   : TV/partition.cpp:89-145 (LDG2), 147-264 (initial), 307-440 (refine)
//   CN   : CN/partition.cpp:80-221 (initial), 245-377 (refine)
//   TM   : TM/partition.cpp:11-250 (initial), 300-593 (refine)
//   MSM  : MSM/partition.cpp:69-309 (initial), 347-656 (refine)
//   MSV  : MGV/partition.cpp:28-65 (LDG), 68-189 (initial), 222-477 (refine)
//   MSRV : MSRV/partition.cpp:26-64 (LDG), 66-196 (initial), 240-517 (refine)
//   metrics: shared/metric.cpp:3-391, inverse CSR shared/utils.cpp:32-56
//
// Extensions (both reduce exactly to the reference when left at their defaults):
//   * vertex weights: part_sizes += w(v); W = sum of w, C = (W/K) * eps_factor,
//     max_pw/min_pw use W/K where the reference uses nov/K.  weights == NULL means
//     unit weights, i.e. the reference.
//   * eps_factor: the reference hard-codes 1.05.

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <climits>
#include <vector>
#include <chrono>
#include <algorithm>

extern "C" {

typedef struct {
  int nov, noe;
  long long pins;
  const unsigned* vptr;    // nov+1, vertex -> nets CSR offsets
  const unsigned* vnets;   // pins, nets of each vertex in visiting order
  const unsigned* nptr;    // noe+1, net -> pins CSR offsets (CN refinement order)
  const unsigned* npins;   // pins
  const int* src;          // noe, source vertex of each net
  const int* weights;      // nov or NULL (unit weights)
  const int* ordering;     // nov or NULL (identity)
} fpo_hg;

typedef struct {
  // inputs
  int metric;              // 0=CN 1=TV 2=TM 3=MSM 4=MSV 5=MSRV
  int K;
  double eps_factor;       // reference: 1.05
  int passes;              // REFI_ITER
  int refine;              // REFI_OPT
  // outputs (caller allocated; any may be NULL)
  int* part_vec_init;      // nov
  int* ep_len_init;        // noe
  int* ep_part_init;       // pins
  int* ep_cnt_init;        // pins
  int* part_vec;           // nov
  int* ep_len;             // noe
  int* ep_part;            // pins
  int* ep_cnt;             // pins
  long long metrics_init[6];   // TV, CN, TM, MSM(MGM), MSV(MGV), MSRV(MGAV)
  long long metrics_final[6];
  long long moves[64];         // accepted moves per pass (first 64 passes)
  double refine_seconds;       // the reference's "Refinement took" span
  int status;                  // 0 ok, <0 error
  // decision records of the last refinement pass (caller allocated, nov
  // entries -- noe for CN -- or NULL); their meaning per metric is that of
  // fp_get_decisions in include/fastpart.h
  int* rec_dest;
  int* rec_gain;
  int* rec_loss;
  int* rec_moved;
} fpo_run;

}  // extern "C"

namespace {

enum { M_CN = 0, M_TV = 1, M_TM = 2, M_MSM = 3, M_MSV = 4, M_MSRV = 5 };

// Decision records of the last pass: one entry per visited vertex (per net for
// CN), written by the refinements below when `on` (the pass is the last one).
struct Records {
  int *dest = nullptr, *gain = nullptr, *loss = nullptr, *moved = nullptr;
  bool on = false;
  void put(int i, int d, int g, int l, bool mv) const {
    if (!on) return;
    if (dest) dest[i] = d;
    if (gain) gain[i] = g;
    if (loss) loss[i] = l;
    if (moved) moved[i] = mv ? 1 : 0;
  }
};

struct HG {
  int nov, noe;
  long long pins;
  const unsigned *vptr, *vnets, *nptr, *npins;
  const int* src;
  std::vector<int> w;      // per-vertex weight
  std::vector<int> order;
  long long W;             // total weight
};

// Per-net ordered part lists: ep_start[e] .. ep_start[e] + ep_len[e] hold the
// parts present in net e in the reference's insertion / swap-with-last order.
struct Lists {
  std::vector<int> start, len, part, cnt;
};

struct Ctx {
  const HG* g;
  int K;
  double C;
  int xw;                  // W / K (integer division, as nov / K in the reference)
  Lists L;
  std::vector<int> part_vec, part_sizes;
};

void lists_init(Ctx& c) {
  const HG& g = *c.g;
  c.L.start.assign(g.noe + 1, 0);
  c.L.len.assign(g.noe, 0);
  c.L.part.assign(g.pins, -1);
  c.L.cnt.assign(g.pins, 0);
  // Net offsets from the vertex -> nets CSR (TV/partition.cpp:178-197).
  for (int v = 0; v < g.nov; v++)
    for (unsigned k = g.vptr[v]; k < g.vptr[v + 1]; k++) c.L.start[g.vnets[k] + 1]++;
  for (int e = 1; e <= g.noe; e++) c.L.start[e] += c.L.start[e - 1];
  c.part_vec.assign(g.nov, -1);
  c.part_sizes.assign(c.K, 0);
}

// "Update the edge part info": add one pin of part `d` to net e
// (TV/partition.cpp:240-263).
inline void list_add(Lists& L, int e, int d) {
  int s = L.start[e], n = L.len[e];
  for (int j = 0; j < n; j++)
    if (L.part[s + j] == d) { L.cnt[s + j]++; return; }
  L.part[s + n] = d;
  L.cnt[s + n] = 1;
  L.len[e]++;
}

// "REMOVAL": remove one pin of part `p` from net e, swap-with-last when its
// count reaches zero (TV/partition.cpp:388-411).  Returns true if p left e.
inline bool list_remove(Lists& L, int e, int p) {
  int s = L.start[e], n = L.len[e];
  for (int j = 0; j < n; j++) {
    if (L.part[s + j] == p) {
      if (--L.cnt[s + j] == 0) {
        L.part[s + j] = L.part[s + n - 1];
        L.cnt[s + j] = L.cnt[s + n - 1];
        L.part[s + n - 1] = -1;
        L.cnt[s + n - 1] = 0;
        L.len[e]--;
        return true;
      }
      return false;
    }
  }
  return false;
}

int min_loaded(const std::vector<int>& sizes, int K) {
  int best = INT_MAX, idx = -1;
  for (int i = 0; i < K; i++)
    if (sizes[i] < best) { best = sizes[i]; idx = i; }
  return idx;
}

// LDG argmax over active parts (TV/partition.cpp:98-132, MGV/partition.cpp:28-64).
int ldg_argmax(const Ctx& c, const std::vector<int>& active, int nact,
               const std::vector<double>& scores) {
  double max_val = 0;
  int max_index = -1;
  for (int i = 0; i < nact; i++) {
    int p = active[i];
    double penalty = 1 - (1.0 * c.part_sizes[p] / c.C);
    double score = scores[p] * penalty;
    if (score > 0) {
      if (max_index == -1 || score > max_val ||
          (score == max_val && c.part_sizes[p] < c.part_sizes[max_index])) {
        max_val = score;
        max_index = p;
      }
    }
  }
  if (max_index == -1) max_index = min_loaded(c.part_sizes, c.K);
  return max_index;
}

// Score gather shared by the LDG streams and refinements (TV/partition.cpp:318-338).
// marker/scores persist across calls exactly as the reference's arrays do.
int gather_scores(const Ctx& c, int v, std::vector<int>& marker, std::vector<double>& scores,
                  std::vector<int>& active) {
  const HG& g = *c.g;
  int nact = 0;
  for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
    int e = g.vnets[i];
    int s = c.L.start[e], n = c.L.len[e];
    for (int j = 0; j < n; j++) {
      int p = c.L.part[s + j];
      if (marker[p] != v) {
        scores[p] = 1;
        marker[p] = v;
        active[nact++] = p;
      } else {
        scores[p]++;
      }
    }
  }
  return nact;
}

// ---------------------------------------------------------------- metrics
// shared/metric.cpp, evaluated on the ordered part lists + part vector.
void eval_metrics(const Ctx& c, long long out[6]) {
  const HG& g = *c.g;
  const int K = c.K;
  // TV_Refined (metric.cpp:70-86) and CN (metric.cpp:3-14).
  long long tv = 0, cn = 0;
  for (int e = 0; e < g.noe; e++) {
    int distinct = 0;
    for (int j = c.L.start[e]; j < c.L.start[e + 1]; j++)
      if (c.L.cnt[j] > 0) distinct++;
    if (distinct > 0) tv += distinct - 1;
    if (c.L.len[e] > 1) cn++;
  }
  // TM_scratch / MGM_scratch (metric.cpp:122-284): distinct (part(src), p) pairs.
  std::vector<char> conn((size_t)K * K, 0);
  std::vector<long long> msgs(K, 0);
  for (int e = 0; e < g.noe; e++) {
    int k = c.part_vec[g.src[e]];
    for (int j = 0; j < c.L.len[e]; j++) {
      int p = c.L.part[c.L.start[e] + j];
      if (p != k && !conn[(size_t)k * K + p]) { conn[(size_t)k * K + p] = 1; msgs[k]++; }
    }
  }
  long long tm = 0, msm = -1;
  for (int k = 0; k < K; k++) { tm += msgs[k]; if (msgs[k] > msm) msm = msgs[k]; }
  // MGV_Scratch (metric.cpp:301-335): send[part(src)] += len-1 once per occurrence
  // of src among the net's pins.  MGAV_Scratch (metric.cpp:353-391).
  std::vector<long long> send(K, 0), send2(K, 0), recv(K, 0);
  for (int e = 0; e < g.noe; e++) {
    int sv = g.src[e];
    for (unsigned j = g.nptr[e]; j < g.nptr[e + 1]; j++)
      if ((int)g.npins[j] == sv) send[c.part_vec[sv]] += c.L.len[e] - 1;
    int sp = c.part_vec[sv];
    send2[sp] += c.L.len[e] - 1;
    for (int j = 0; j < c.L.len[e]; j++) {
      int p = c.L.part[c.L.start[e] + j];
      if (p != sp) recv[p]++;
    }
  }
  long long msv = -1, msrv = -1;
  for (int k = 0; k < K; k++) {
    if (send[k] > msv) msv = send[k];
    if (send2[k] + recv[k] > msrv) msrv = send2[k] + recv[k];
  }
  out[0] = tv; out[1] = cn; out[2] = tm; out[3] = msm; out[4] = msv; out[5] = msrv;
}

// ---------------------------------------------------------------- initial streams

// LDG stream of TV (LDG2 with clamps), MSV and MSRV (plain LDG, volume bookkeeping).
void initial_ldg(Ctx& c, int metric, std::vector<int>& marker, std::vector<int>& send,
                 std::vector<int>& recv, int& status) {
  const HG& g = *c.g;
  std::vector<int> active(c.K);
  std::vector<double> scores(c.K, 0.0);
  const int max_pw = (int)(c.xw + (c.xw * 0.1));
  for (int z = 0; z < g.nov; z++) {
    int v = g.order[z];
    int nact = gather_scores(c, v, marker, scores, active);
    int d = ldg_argmax(c, active, nact, scores);
    if (metric == M_TV && c.part_sizes[d] > max_pw) {
      // LDG2 would assign part_vec[v] == -1 here (TV/partition.cpp:135-138):
      // undefined behaviour in the reference, rejected here.
      status = -3;
      return;
    }
    c.part_sizes[d] += g.w[v];
    c.part_vec[v] = d;
    for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      int e = g.vnets[i];
      int s = c.L.start[e], n = c.L.len[e];
      bool found = false;
      if (metric == M_TV) {
        list_add(c.L, e, d);
        continue;
      }
      // MGV/partition.cpp:151-181, MSRV/partition.cpp:151-194.
      int sv = g.src[e];
      int sp = c.part_vec[sv];
      for (int j = 0; j < n; j++) {
        int p = c.L.part[s + j];
        if (sv == v && p != sp) {
          send[sp]++;
          if (metric == M_MSRV) recv[p]++;
        }
        if (p == d) { found = true; c.L.cnt[s + j]++; }
      }
      if (!found) {
        c.L.part[s + n] = d;
        c.L.cnt[s + n] = 1;
        c.L.len[e]++;
        if (sv != v && sp != -1) {
          send[sp]++;
          if (metric == M_MSRV) recv[d]++;
        }
      }
    }
  }
}

// CN stream: LDG over uncut nets only (CN/partition.cpp:132-221).
void initial_cn(Ctx& c) {
  const HG& g = *c.g;
  std::vector<int> marker(c.K, -1), active(c.K);
  std::vector<double> scores(c.K, 0.0);
  for (int z = 0; z < g.nov; z++) {
    int v = g.order[z];
    int nact = 0;
    for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      int e = g.vnets[i];
      if (c.L.len[e] == 1) {
        int p = c.L.part[c.L.start[e]];
        if (marker[p] != v) { scores[p] = 1; marker[p] = v; active[nact++] = p; }
        else scores[p]++;
      }
    }
    int d = ldg_argmax(c, active, nact, scores);
    c.part_sizes[d] += g.w[v];
    c.part_vec[v] = d;
    for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_add(c.L, g.vnets[i], d);
  }
}

// Message-greedy stream of TM / MSM (TM/partition.cpp:87-250, MSM/partition.cpp:146-309).
// conn is K x K, row-major; diagonal is 0 (TM) or -1 (MSM).
void initial_msg(Ctx& c, std::vector<int>& conn, std::vector<int>& msgs) {
  const HG& g = *c.g;
  const int K = c.K;
  std::vector<int> src_marker(K, -1), src_node_parts(g.noe, -1);
  std::vector<int> active_src, active_src_net, src_update;
  for (int z = 0; z < g.nov; z++) {
    int v = g.order[z];
    active_src.clear(); active_src_net.clear(); src_update.clear();
    for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
      int e = g.vnets[i];
      if (g.src[e] == v) src_update.push_back(e);
      if (src_node_parts[e] != -1) {
        if (src_marker[src_node_parts[e]] != v) {
          src_marker[src_node_parts[e]] = v;
          active_src.push_back(src_node_parts[e]);
        }
        active_src_net.push_back(e);
      }
    }
    int max_saved = -1, max_index = -1;
    for (int k = 0; k < K; k++) {
      if (c.part_sizes[k] < c.C) {
        int saved = 0;
        for (int sp : active_src)
          if (conn[(size_t)sp * K + k] > 0) saved++;
        for (int e : src_update) {
          int s = c.L.start[e], n = c.L.len[e];
          for (int j = 0; j < n; j++)
            if (conn[(size_t)k * K + c.L.part[s + j]] > 0) saved++;
        }
        if (saved > max_saved || (saved == max_saved && c.part_sizes[k] < c.part_sizes[max_index])) {
          max_index = k;
          max_saved = saved;
        }
      }
    }
    if (max_index == -1) max_index = min_loaded(c.part_sizes, K);
    int d = max_index;
    c.part_vec[v] = d;
    c.part_sizes[d] += g.w[v];
    for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_add(c.L, g.vnets[i], d);
    for (int e : active_src_net) {
      int sp = src_node_parts[e];
      if (sp == d) continue;
      int& cc = conn[(size_t)sp * K + d];
      if (cc == 0) { msgs[sp]++; cc = 1; }
      else {
        int s = c.L.start[e], n = c.L.len[e];
        for (int j = 0; j < n; j++) {
          if (c.L.part[s + j] == d) {
            if (c.L.cnt[s + j] == 1) cc++;
            break;
          }
        }
      }
    }
    for (int e : src_update) {
      src_node_parts[e] = d;
      int s = c.L.start[e], n = c.L.len[e];
      for (int j = 0; j < n; j++) {
        int p = c.L.part[s + j];
        if (p == d) continue;
        int& cc = conn[(size_t)d * K + p];
        if (cc == 0) { msgs[d]++; cc = 1; }
        else cc++;
      }
    }
  }
}

// ---------------------------------------------------------------- refinements

// Moves v from its part to d on every net (REMOVAL then ADDING).
void move_lists(Ctx& c, int v, int own, int d) {
  const HG& g = *c.g;
  for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_remove(c.L, g.vnets[i], own);
  for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_add(c.L, g.vnets[i], d);
}

// TV refinement (TV/partition.cpp:307-440).  `marker` carries over from the
// initial stream and across passes, as in the reference.
void refine_tv(Ctx& c, int passes, std::vector<int>& marker, long long* moves, Records rec) {
  const HG& g = *c.g;
  std::vector<int> active(c.K);
  std::vector<double> scores(c.K, 0.0);
  const int max_pw = (int)(c.xw + (c.xw * 0.1));
  const int min_pw = (int)(c.xw - (c.xw * 0.1));
  for (int it = 0; it < passes; it++) {
    long long mv = 0;
    rec.on = it == passes - 1;
    for (int z = 0; z < g.nov; z++) {
      int v = g.order[z];
      int own = c.part_vec[v];
      int nact = gather_scores(c, v, marker, scores, active);
      scores[own]--;
      int d = ldg_argmax(c, active, nact, scores);
      if (c.part_sizes[d] > max_pw) d = c.part_vec[v];
      if (c.part_sizes[d] < min_pw && c.part_vec[v] != -1) d = c.part_vec[v];
      if (own == d) {
        rec.put(v, d, 0, 0, false);
        continue;
      }
      int leave_gain = 0, arrival_loss = 0;
      for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        int e = g.vnets[i];
        int s = c.L.start[e], n = c.L.len[e];
        bool found = false;
        for (int j = 0; j < n; j++) {
          if (c.L.part[s + j] == own && c.L.cnt[s + j] == 1) leave_gain++;
          else if (c.L.part[s + j] == d) found = true;
        }
        if (!found) arrival_loss++;
      }
      rec.put(v, d, leave_gain, arrival_loss, leave_gain >= arrival_loss);
      if (leave_gain >= arrival_loss) {
        mv++;
        c.part_vec[v] = d;
        c.part_sizes[own] -= g.w[v];
        c.part_sizes[d] += g.w[v];
        move_lists(c, v, own, d);
      }
    }
    if (it < 64) moves[it] = mv;
  }
}

// CN refinement (CN/partition.cpp:245-377), net-centric, nets in id order.
void refine_cn(Ctx& c, int passes, long long* moves, Records rec) {
  const HG& g = *c.g;
  std::vector<int> push(g.nov);
  for (int it = 0; it < passes; it++) {
    long long mv = 0;
    rec.on = it == passes - 1;
    for (int e = 0; e < g.noe; e++) {
      if (c.L.len[e] != 2) {
        rec.put(e, -1, 0, -1, false);
        continue;
      }
      int s = c.L.start[e];
      int p1 = c.L.part[s], c1 = c.L.cnt[s];
      int p2 = c.L.part[s + 1], c2 = c.L.cnt[s + 1];
      int oldp, newp;
      if (c1 < c2) { oldp = p1; newp = p2; } else { oldp = p2; newp = p1; }
      int np = 0;
      bool not_in_cut = false;
      for (unsigned k = g.nptr[e]; !not_in_cut && k < g.nptr[e + 1]; k++) {
        int u = g.npins[k];
        if (c.part_vec[u] == oldp) {
          push[np++] = u;
          for (unsigned j = g.vptr[u]; j < g.vptr[u + 1]; j++) {
            if (c.L.len[g.vnets[j]] == 1) { not_in_cut = true; break; }
          }
        }
      }
      rec.put(e, newp, not_in_cut ? 0 : np, oldp, !not_in_cut);
      if (!not_in_cut) {
        for (int q = 0; q < np; q++) {
          int u = push[q];
          int own = c.part_vec[u];
          c.part_vec[u] = newp;
          c.part_sizes[own] -= g.w[u];
          c.part_sizes[newp] += g.w[u];
          move_lists(c, u, own, newp);
          mv++;
        }
      }
    }
    if (it < 64) moves[it] = mv;
  }
}

// Shared commit of TM / MSM: lists, then the K x K connection counts and the
// per-part message counts (TM/partition.cpp:457-591).
void commit_msg(Ctx& c, int v, int own, int d, std::vector<int>& conn, std::vector<int>& msgs) {
  const HG& g = *c.g;
  const int K = c.K;
  c.part_vec[v] = d;
  c.part_sizes[own] -= g.w[v];
  c.part_sizes[d] += g.w[v];
  for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_remove(c.L, g.vnets[i], own);
  for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) list_add(c.L, g.vnets[i], d);
  for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
    int e = g.vnets[i];
    int s = c.L.start[e], n = c.L.len[e];
    if (g.src[e] == v) {
      for (int j = 0; j < n; j++) {
        int t = c.L.part[s + j];
        if (t != d) {
          if (++conn[(size_t)d * K + t] == 1) msgs[d]++;
        }
        if (t != own && t != d) {
          if (--conn[(size_t)own * K + t] == 0) msgs[own]--;
        }
        if (t == d && c.L.cnt[s + j] > 1) {
          if (--conn[(size_t)own * K + t] == 0) msgs[own]--;
        }
      }
    } else {
      int sn = c.part_vec[g.src[e]];
      bool found = false;
      for (int j = 0; j < n; j++) {
        if (c.L.part[s + j] == d && c.L.cnt[s + j] == 1) {
          if (++conn[(size_t)sn * K + d] == 1) msgs[sn]++;
        }
        if (c.L.part[s + j] == own) found = true;
      }
      if (!found) {
        if (--conn[(size_t)sn * K + own] == 0) msgs[sn]--;
      }
    }
  }
}

// TM refinement (TM/partition.cpp:300-593); vertices in id order.
void refine_tm(Ctx& c, int passes, std::vector<int>& conn, std::vector<int>& msgs, long long* moves,
               Records rec) {
  const HG& g = *c.g;
  const int K = c.K;
  std::vector<int> receivers(K), senders(K);
  for (int it = 0; it < passes; it++) {
    long long mv = 0;
    rec.on = it == passes - 1;
    std::vector<int> mrec(K, -1), msnd(K, -1);
    for (int v = 0; v < g.nov; v++) {
      int best = -1, best_imp = 0;
      int own = c.part_vec[v];
      int gain = 0, nrec = 0, nsnd = 0;
      for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        int e = g.vnets[i];
        int s = c.L.start[e], n = c.L.len[e];
        if (g.src[e] == v) {
          for (int j = 0; j < n; j++) {
            int t = c.L.part[s + j];
            if (t == own && c.L.cnt[s + j] > 1 && mrec[own] != v) { receivers[nrec++] = own; mrec[own] = v; }
            if (t != own) {
              if (mrec[t] != v) { receivers[nrec++] = t; mrec[t] = v; }
              // gain_loss_2d[own][t] is 1 here: it is raised once per listed part and
              // lowered again after each net (TM/partition.cpp:347-369).
              int cc = conn[(size_t)own * K + t];
              if (cc == 1 || cc == 1) gain++;
            }
          }
        } else {
          int ps = c.part_vec[g.src[e]];
          if (msnd[ps] != v) {
            senders[nsnd++] = ps;
            msnd[ps] = v;
            for (int j = 0; j < n; j++)
              if (c.L.part[s + j] == own && c.L.cnt[s + j] == 1 && conn[(size_t)ps * K + own] == 1) gain++;
          }
        }
      }
      if (gain > 0) {
        for (int k = 0; k < K; k++) {
          if (c.part_sizes[k] >= c.C) continue;
          if (k == own) continue;
          int loss = 0;
          for (int i = 0; i < nrec; i++) {
            int r = receivers[i];
            if (r == k) continue;
            if (conn[(size_t)k * K + r] == 0) loss++;
          }
          for (int i = 0; i < nsnd; i++) {
            int sp = senders[i];
            if (sp == k) continue;
            if (conn[(size_t)sp * K + k] == 0) loss++;
          }
          if (gain > loss && gain - loss > best_imp) { best = k; best_imp = gain - loss; }
        }
      }
      rec.put(v, best, gain, best != -1 ? gain - best_imp : 0, best != -1);
      if (best != -1) {
        mv++;
        commit_msg(c, v, own, best, conn, msgs);
      }
    }
    if (it < 64) moves[it] = mv;
  }
}

// MSM refinement (MSM/partition.cpp:347-656); vertices in id order.
void refine_msm(Ctx& c, int passes, std::vector<int>& conn, std::vector<int>& msgs, long long* moves,
                Records rec) {
  const HG& g = *c.g;
  const int K = c.K;
  std::vector<int> gains(K), losses(K), max_parts(K), mmark(K), receivers(K), senders(K);
  for (int it = 0; it < passes; it++) {
    long long mv = 0;
    rec.on = it == passes - 1;
    std::vector<int> mrec(K, -1), msnd(K, -1);
    for (int v = 0; v < g.nov; v++) {
      int best = -1, best_imp = -1;
      int own = c.part_vec[v];
      std::fill(gains.begin(), gains.end(), 0);
      std::fill(mmark.begin(), mmark.end(), -1);
      bool has_gain = false;
      int nrec = 0, nsnd = 0;
      int max_mes = -1, nmax = 0, mcc = 0;
      for (int i = 0; i < K; i++) {
        if (msgs[i] > max_mes) { nmax = 1; max_parts[0] = i; max_mes = msgs[i]; mcc++; mmark[i] = mcc; }
        else if (msgs[i] == max_mes) { max_parts[nmax++] = i; mmark[i] = mcc; }
      }
      for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        int e = g.vnets[i];
        int s = c.L.start[e], n = c.L.len[e];
        if (g.src[e] == v) {
          for (int j = 0; j < n; j++) {
            int t = c.L.part[s + j];
            if (t == own && c.L.cnt[s + j] > 1 && mrec[own] != v) { receivers[nrec++] = own; mrec[own] = v; }
            if (t != own) {
              if (mrec[t] != v) { receivers[nrec++] = t; mrec[t] = v; }
              if (conn[(size_t)own * K + t] == 1) { gains[own]++; has_gain = true; }
            }
          }
        } else {
          int ps = c.part_vec[g.src[e]];
          if (msnd[ps] != v) {
            senders[nsnd++] = ps;
            msnd[ps] = v;
            for (int j = 0; j < n; j++)
              if (c.L.part[s + j] == own && c.L.cnt[s + j] == 1 && conn[(size_t)ps * K + own] == 1) {
                gains[ps]++;
                has_gain = true;
              }
          }
        }
      }
      if (has_gain) {
        for (int k = 0; k < K; k++) {
          if (k == own) continue;
          std::fill(losses.begin(), losses.end(), 0);
          for (int i = 0; i < nrec; i++)
            if (conn[(size_t)k * K + receivers[i]] == 0) losses[k]++;
          for (int i = 0; i < nsnd; i++)
            if (conn[(size_t)senders[i] * K + k] == 0) losses[senders[i]]++;
          bool good = true;
          int imp = 0;
          for (int i = 0; i < nmax; i++) {
            int m = max_parts[i];
            if (gains[m] <= losses[m]) { good = false; break; }
            imp += gains[m] - losses[m];
          }
          for (int i = 0; good && i < K; i++) {
            if (mmark[i] == mcc) continue;
            if (msgs[i] + (losses[i] - gains[i]) >= max_mes) good = false;
          }
          if (good && imp > best_imp) { best = k; best_imp = imp; }
        }
      }
      if (rec.on) {
        int gsum = 0;
        for (int p = 0; p < K; p++) gsum += gains[p];
        rec.put(v, best, gsum, best_imp, best != -1);
      }
      if (best != -1) {
        mv++;
        commit_msg(c, v, own, best, conn, msgs);
      }
    }
    if (it < 64) moves[it] = mv;
  }
}

// Max-volume scan shared by MSV / MSRV (MGV/partition.cpp:456-471).
struct MaxSet {
  std::vector<int> parts, mark;
  int count = 0, val = -1, cc = 0;
  bool overflow = false;
};

// MSV (MGV) refinement (MGV/partition.cpp:222-477) and MSRV refinement
// (MSRV/partition.cpp:240-517).  recv is ignored for MSV.
void refine_vol(Ctx& c, int metric, int passes, std::vector<int>& send, std::vector<int>& recv,
                long long* moves, int& status, Records rec) {
  const HG& g = *c.g;
  const int K = c.K;
  const bool rv = (metric == M_MSRV);
  std::vector<int> marker(K, -1), active(K), gains(K, 0), losses(K, 0);
  std::vector<double> scores(K, 0.0);
  MaxSet M;
  M.parts.assign(K, 0);
  M.mark.assign(K, -1);
  auto vol = [&](int i) { return rv ? send[i] + recv[i] : send[i]; };
  auto full_scan = [&]() {
    M.count = 0; M.val = -1; M.cc = 0;
    std::fill(M.mark.begin(), M.mark.end(), -1);
    for (int i = 0; i < K; i++) {
      int x = vol(i);
      if (x > M.val) { M.count = 1; M.parts[0] = i; M.val = x; M.cc++; M.mark[i] = M.cc; }
      else if (x == M.val) { M.parts[M.count++] = i; M.mark[i] = M.cc; }
    }
  };
  for (int it = 0; it < passes; it++) {
    long long mv = 0;
    rec.on = it == passes - 1;
    std::fill(marker.begin(), marker.end(), -1);
    full_scan();
    for (int z = 0; z < g.nov; z++) {
      int v = g.order[z];
      int own = c.part_vec[v];
      std::fill(gains.begin(), gains.end(), 0);
      std::fill(losses.begin(), losses.end(), 0);
      int nact = gather_scores(c, v, marker, scores, active);
      scores[own]--;
      int d = ldg_argmax(c, active, nact, scores);
      if (own == d) {
        rec.put(v, d, 0, 0, false);
        continue;
      }
      for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        int e = g.vnets[i];
        int s = c.L.start[e], n = c.L.len[e];
        int sv = g.src[e];
        int sp = c.part_vec[sv];
        if (sv == v) {
          gains[own] += n - 1;
          losses[d] += n - 1;
        }
        bool found = false;
        for (int j = 0; j < n; j++) {
          if (c.L.part[s + j] == own && c.L.cnt[s + j] == 1) {
            if (sv != v) {
              gains[sp]++;
              if (rv) gains[own]++;
            } else {
              losses[d]--;
            }
          }
          if (c.L.part[s + j] == d) found = true;
        }
        if (!found) {
          if (sv != v) {
            losses[sp]++;
            if (rv) losses[d]++;
          } else {
            losses[d]++;
          }
        }
      }
      bool good = true;
      for (int i = 0; i < M.count; i++) {
        int m = M.parts[i];
        if (rv ? (gains[m] <= losses[m]) : (gains[m] < losses[m])) { good = false; break; }
      }
      for (int i = 0; good && i < K; i++) {
        if (M.mark[i] == M.cc) continue;
        if (vol(i) + (losses[i] - gains[i]) >= M.val) good = false;
      }
      if (rec.on) {
        int gsum = 0, lsum = 0;
        for (int p = 0; p < K; p++) { gsum += gains[p]; lsum += losses[p]; }
        rec.put(v, d, gsum, lsum, good);
      }
      if (!good) continue;
      mv++;
      c.part_vec[v] = d;
      c.part_sizes[own] -= g.w[v];
      c.part_sizes[d] += g.w[v];
      // REMOVING (no break in the reference; the part occurs once per list).
      for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        int e = g.vnets[i];
        int s = c.L.start[e], n = c.L.len[e];
        int sv = g.src[e];
        int sp = c.part_vec[sv];
        if (sv == v) send[own] -= n - 1;
        for (int j = 0; j < n; j++) {
          if (c.L.part[s + j] == own) {
            c.L.cnt[s + j]--;
            if (c.L.cnt[s + j] == 0) {
              c.L.part[s + j] = c.L.part[s + n - 1];
              c.L.cnt[s + j] = c.L.cnt[s + n - 1];
              c.L.part[s + n - 1] = -1;
              c.L.cnt[s + n - 1] = 0;
              c.L.len[e]--;
              n--;
              if (sv != v) {
                send[sp]--;
                if (rv) recv[own]--;
              }
            } else if (rv && sv == v) {
              recv[own]++;
            }
          }
        }
      }
      // ADDING.
      for (unsigned i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        int e = g.vnets[i];
        int s = c.L.start[e], n = c.L.len[e];
        int sv = g.src[e];
        int sp = c.part_vec[sv];
        if (sv == v) send[sp] += n - 1;
        bool found = false;
        for (int j = 0; j < n; j++) {
          if (c.L.part[s + j] == d) {
            found = true;
            c.L.cnt[s + j]++;
            if (rv && sv == v) recv[d]--;
            break;
          }
        }
        if (!found) {
          c.L.part[s + n] = d;
          c.L.cnt[s + n] = 1;
          c.L.len[e]++;
          send[sp]++;
          if (rv && sv != v) recv[d]++;
        }
      }
      if (!rv) {
        full_scan();
      } else {
        // MSRV/partition.cpp:486-513: rescan only when an old max part changed;
        // the count is not reset, so entries can repeat.
        bool changed = false;
        for (int i = 0; i < M.count; i++)
          if (M.val != vol(M.parts[i])) changed = true;
        for (int i = 0; changed && i < K; i++) {
          int x = vol(i);
          if (x > M.val) { M.count = 1; M.parts[0] = i; M.val = x; M.cc++; M.mark[i] = M.cc; }
          else if (x == M.val) {
            if (M.count >= K) { status = -4; return; }  // reference writes past max_parts[K-1]
            M.parts[M.count++] = i;
            M.mark[i] = M.cc;
          }
        }
      }
    }
    if (it < 64) moves[it] = mv;
  }
}

}  // namespace

extern "C" int fpo_partition(const fpo_hg* in, fpo_run* r) {
  r->status = 0;
  if (!in || !r || r->K < 2 || in->nov <= 0 || in->noe < 0 || r->metric < 0 || r->metric > 5) {
    r->status = -1;
    return -1;
  }
  HG g;
  g.nov = in->nov; g.noe = in->noe; g.pins = in->pins;
  g.vptr = in->vptr; g.vnets = in->vnets; g.nptr = in->nptr; g.npins = in->npins; g.src = in->src;
  g.w.resize(g.nov);
  g.W = 0;
  for (int v = 0; v < g.nov; v++) { g.w[v] = in->weights ? in->weights[v] : 1; g.W += g.w[v]; }
  g.order.resize(g.nov);
  for (int z = 0; z < g.nov; z++) g.order[z] = in->ordering ? in->ordering[z] : z;

  Ctx c;
  c.g = &g;
  c.K = r->K;
  c.xw = (int)(g.W / r->K);
  if (c.xw < 1) { r->status = -2; return -2; }
  c.C = c.xw * r->eps_factor;
  lists_init(c);

  const int K = c.K;
  const int m = r->metric;
  std::vector<int> marker(K, -1), send(K, 0), recv(K, 0), msgs(K, 0);
  std::vector<int> conn;
  int status = 0;
  if (m == M_TV || m == M_MSV || m == M_MSRV) {
    initial_ldg(c, m, marker, send, recv, status);
  } else if (m == M_CN) {
    initial_cn(c);
  } else {
    conn.assign((size_t)K * K, 0);
    if (m == M_MSM)
      for (int i = 0; i < K; i++) conn[(size_t)i * K + i] = -1;
    initial_msg(c, conn, msgs);
  }
  if (status) { r->status = status; return status; }

  if (r->part_vec_init) std::memcpy(r->part_vec_init, c.part_vec.data(), sizeof(int) * g.nov);
  if (r->ep_len_init) std::memcpy(r->ep_len_init, c.L.len.data(), sizeof(int) * g.noe);
  if (r->ep_part_init) std::memcpy(r->ep_part_init, c.L.part.data(), sizeof(int) * g.pins);
  if (r->ep_cnt_init) std::memcpy(r->ep_cnt_init, c.L.cnt.data(), sizeof(int) * g.pins);
  eval_metrics(c, r->metrics_init);

  std::memset(r->moves, 0, sizeof(r->moves));
  auto t0 = std::chrono::steady_clock::now();
  Records rec;
  rec.dest = r->rec_dest;
  rec.gain = r->rec_gain;
  rec.loss = r->rec_loss;
  rec.moved = r->rec_moved;
  if (r->refine && r->passes > 0) {
    switch (m) {
      case M_TV: refine_tv(c, r->passes, marker, r->moves, rec); break;
      case M_CN: refine_cn(c, r->passes, r->moves, rec); break;
      case M_TM: refine_tm(c, r->passes, conn, msgs, r->moves, rec); break;
      case M_MSM: refine_msm(c, r->passes, conn, msgs, r->moves, rec); break;
      default: refine_vol(c, m, r->passes, send, recv, r->moves, status, rec); break;
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  r->refine_seconds = std::chrono::duration<double>(t1 - t0).count();
  if (status) { r->status = status; return status; }

  if (r->part_vec) std::memcpy(r->part_vec, c.part_vec.data(), sizeof(int) * g.nov);
  if (r->ep_len) std::memcpy(r->ep_len, c.L.len.data(), sizeof(int) * g.noe);
  if (r->ep_part) std::memcpy(r->ep_part, c.L.part.data(), sizeof(int) * g.pins);
  if (r->ep_cnt) std::memcpy(r->ep_cnt, c.L.cnt.data(), sizeof(int) * g.pins);
  eval_metrics(c, r->metrics_final);
  return 0;
}
