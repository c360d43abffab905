// Host side of the C ABI that needs no GPU: generated and file-backed
// hypergraphs, and the drop-in partition_gpu() driver.

#include "fp_internal.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <fstream>
#include <sstream>
#include <string>
#include <memory>
#include <new>
#include <vector>
#include <algorithm>

namespace {

using fp::HostGraph;

// Net -> pins from vertex -> nets, pins in ascending vertex order per net
// (the reference's createInverse, shared/utils.cpp:32-56).
void build_net_csr(HostGraph& g) {
  g.nptr.assign(g.noe + 1, 0);
  for (long long k = 0; k < g.pins; k++) g.nptr[g.vnets[k] + 1]++;
  for (int e = 0; e < g.noe; e++) g.nptr[e + 1] += g.nptr[e];
  g.npins.assign(g.pins, 0);
  std::vector<uint32_t> fill(g.nptr.begin(), g.nptr.end() - 1);
  for (int v = 0; v < g.nov; v++)
    for (uint32_t k = g.vptr[v]; k < g.vptr[v + 1]; k++) g.npins[fill[g.vnets[k]]++] = (uint32_t)v;
}

void choose_sources(HostGraph& g, int rule) {
  g.src.assign(g.noe, -1);
  for (int e = 0; e < g.noe; e++) {
    if (g.nptr[e] == g.nptr[e + 1]) continue;
    const uint32_t* b = &g.npins[g.nptr[e]];
    const uint32_t* en = &g.npins[g.nptr[e + 1]];
    g.src[e] = rule == 0 ? (int)*std::min_element(b, en) : (int)*b;
  }
}

// PaToH-like text: "index_base nov noe pins" then one line of vertex ids per
// file net (shared/hypergraph_rw.cpp:97-183).  Produces the file's own
// net -> pins CSR (lines as given).
bool parse_text(const std::string& path, int& nov, int& noe, long long& pins, std::vector<uint32_t>& lptr,
                std::vector<uint32_t>& lids) {
  std::ifstream in(path);
  if (!in) return false;
  in.seekg(0, std::ios::end);
  const long long bytes = (long long)in.tellg();
  in.seekg(0, std::ios::beg);
  int base = 0;
  long long lnov = 0, lnoe = 0;
  in >> base >> lnov >> lnoe >> pins;
  // counts the library can hold (int32 ids, fewer than 2^31 pins)
  if (!in || bytes < 0 || lnov <= 0 || lnov > INT32_MAX || lnoe < 0 || lnoe > INT32_MAX || pins < 0 ||
      pins >= (1ll << 31))
    return false;
  nov = (int)lnov;
  noe = (int)lnoe;
  const int salt = base == 0 ? 0 : -1;
  std::string line;
  std::getline(in, line);
  lptr.assign(1, 0);
  lids.clear();
  lids.reserve((size_t)std::min<long long>(pins, bytes / 2 + 1));   // an id takes two bytes at least
  while ((int)lptr.size() - 1 < noe && std::getline(in, line)) {
    std::istringstream iss(line);
    long long x;
    size_t before = lids.size();
    while (iss >> x) {
      long long id = x + salt;
      if (id < 0 || id >= nov) return false;
      lids.push_back((uint32_t)id);
    }
    if (lids.size() != before) lptr.push_back((uint32_t)lids.size());
  }
  noe = (int)lptr.size() - 1;
  return (long long)lids.size() == pins;
}

// <path>.plbin: u32 noe, u32 nov, i64 pins, then per line its cumulative end
// and its ids (shared/hypergraph_rw.cpp:185-240).
bool read_plbin(const std::string& path, int& nov, int& noe, long long& pins, std::vector<uint32_t>& lptr,
                std::vector<uint32_t>& lids) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  in.seekg(0, std::ios::end);
  const long long bytes = (long long)in.tellg();
  in.seekg(0, std::ios::beg);
  uint32_t unoe = 0, unov = 0;
  in.read((char*)&unoe, 4);
  in.read((char*)&unov, 4);
  in.read((char*)&pins, 8);
  // the file holds 16 header bytes, 4 per line and 4 per id
  if (!in || unoe > INT32_MAX || unov == 0 || unov > INT32_MAX || pins < 0 || pins >= (1ll << 31) ||
      16 + 4 * ((long long)unoe + pins) > bytes)
    return false;
  noe = (int)unoe;
  nov = (int)unov;
  lptr.assign((size_t)noe + 1, 0);
  lids.resize((size_t)pins);
  uint32_t prev = 0;
  for (int e = 0; e < noe; e++) {
    uint32_t end = 0;
    in.read((char*)&end, 4);
    if (!in || end < prev || end > (uint64_t)pins) return false;
    lptr[e + 1] = end;
    if (end > prev) in.read((char*)&lids[prev], (std::streamsize)(end - prev) * 4);
    if (!in) return false;
    prev = end;
  }
  for (uint32_t x : lids)
    if (x >= (uint32_t)nov) return false;
  return prev == (uint64_t)pins;
}

bool write_plbin(const std::string& path, int nov, int noe, long long pins, const std::vector<uint32_t>& lptr,
                 const std::vector<uint32_t>& lids) {
  std::ofstream out(path, std::ios::binary);
  if (!out) return false;
  uint32_t unoe = (uint32_t)noe, unov = (uint32_t)nov;
  out.write((const char*)&unoe, 4);
  out.write((const char*)&unov, 4);
  out.write((const char*)&pins, 8);
  for (int e = 0; e < noe; e++) {
    uint32_t end = lptr[e + 1];
    out.write((const char*)&end, 4);
    out.write((const char*)&lids[lptr[e]], (std::streamsize)(lptr[e + 1] - lptr[e]) * 4);
  }
  return (bool)out;
}

}  // namespace

namespace fp {

int make_problem(const fp_hypergraph* h, int K, int metric, double eps_factor, HostGraph& g, Problem& pb) {
  if (metric < 0 || metric > 5 || K < 2 || K > kMaxK || !(eps_factor > 0)) return FP_ERR_INVALID;
  const int rc = fp_validate(h);
  if (rc) return rc;
  g.nov = h->nov;
  g.noe = h->noe;
  g.pins = h->pins;
  g.vptr.assign(h->vptr, h->vptr + h->nov + 1);
  g.vnets.assign(h->vnets, h->vnets + h->pins);
  g.nptr.assign(h->nptr, h->nptr + h->noe + 1);
  g.npins.assign(h->npins, h->npins + h->pins);
  g.src.assign(h->src, h->src + h->noe);
  pb.g = &g;
  pb.K = K;
  pb.metric = metric;
  pb.eps_factor = eps_factor;
  pb.w.resize(g.nov);
  long long W = 0;
  for (int v = 0; v < g.nov; v++) { pb.w[v] = h->weights ? h->weights[v] : 1; W += pb.w[v]; }
  if (h->weights) g.weights = pb.w;
  pb.order.resize(g.nov);
  for (int z = 0; z < g.nov; z++) pb.order[z] = h->ordering ? h->ordering[z] : z;
  pb.xw = (int)(W / K);
  if (pb.xw < 1) return FP_ERR_INVALID;
  pb.C = pb.xw * eps_factor;
  return FP_OK;
}

// Checks a caller-built refinement state in the reference's layout against the
// hypergraph and converts it into the engine's host state.  ep_ends[e] is
// lambda(e), the number of parts listed for net e: the stream increments it
// from 0 (TV/partition.cpp:1066-1075) and the metric code reads it as that count
// (shared/metric.cpp:3-14,57-68).  ep_starts must equal the net offsets.
int state_from_caller(const HostGraph& g, const Problem& pb, const fp_state* s, HostState& st) {
  if (!s || !s->part_vec || !s->ep_starts || !s->ep_ends || !s->ep_parts || !s->ep_cnt) return FP_ERR_INVALID;
  const int K = pb.K, metric = pb.metric, nov = g.nov, noe = g.noe;
  const bool msg = metric == FP_METRIC_TM || metric == FP_METRIC_MSM;
  st.part_vec.assign(s->part_vec, s->part_vec + nov);
  st.part_sizes.assign(K, 0);
  for (int v = 0; v < nov; v++) {
    const int p = st.part_vec[v];
    if (p < 0 || p >= K) return FP_ERR_INVALID;
    st.part_sizes[p] += pb.w[v];
  }
  if (s->part_sizes)
    for (int p = 0; p < K; p++)
      if (s->part_sizes[p] != st.part_sizes[p]) return FP_ERR_INVALID;
  st.ep_start.assign(g.nptr.begin(), g.nptr.end());
  st.ep_len.assign(noe, 0);
  st.ep_part.assign(g.pins, -1);
  st.ep_cnt.assign(g.pins, 0);
  // Every list must hold exactly the parts of the net's pins with their counts
  // (the reference's checkMe invariant, MSM/partition.cpp:2-68).
  std::vector<int> mark(K, -1), count(K, 0), listed(K, -1);
  for (int e = 0; e < noe; e++) {
    const int b = (int)g.nptr[e], size = (int)(g.nptr[e + 1] - g.nptr[e]);
    if (s->ep_starts[e] != b) return FP_ERR_INVALID;
    const int len = s->ep_ends[e];   // lambda(e): the list length, as the reference keeps it
    if (len < 1 || len > size || len > K) return FP_ERR_INVALID;
    int distinct = 0;
    for (int k = b; k < b + size; k++) {
      const int p = st.part_vec[g.npins[k]];
      if (mark[p] != e) { mark[p] = e; count[p] = 0; distinct++; }
      count[p]++;
    }
    if (distinct != len) return FP_ERR_INVALID;
    for (int j = 0; j < len; j++) {
      const int p = s->ep_parts[b + j], c = s->ep_cnt[b + j];
      if (p < 0 || p >= K || mark[p] != e || listed[p] == e || count[p] != c) return FP_ERR_INVALID;
      listed[p] = e;
      st.ep_part[b + j] = p;
      st.ep_cnt[b + j] = c;
    }
    st.ep_len[e] = len;
  }
  st.marker.assign(K, -1);
  if (s->marker)
    for (int p = 0; p < K; p++) {
      if (s->marker[p] < -1 || s->marker[p] >= nov) return FP_ERR_INVALID;
      st.marker[p] = s->marker[p];
    }
  // Volumes and messages: as given, else the count over the lists; the arrays
  // a metric does not keep stay zero (send: MSV, MSRV; recv: MSRV).
  const bool keep_send = metric == FP_METRIC_MSV || metric == FP_METRIC_MSRV;
  const bool keep_recv = metric == FP_METRIC_MSRV;
  st.send.assign(K, 0);
  st.recv.assign(K, 0);
  st.msgs.assign(K, 0);
  if (msg) st.conn.assign((size_t)K * K, 0);
  for (int e = 0; e < noe; e++) {
    const int sp = st.part_vec[g.src[e]];
    const int b = st.ep_start[e];
    for (int j = 0; j < st.ep_len[e]; j++) {
      const int p = st.ep_part[b + j];
      if (p == sp) continue;
      if (keep_send) st.send[sp]++;
      if (keep_recv) st.recv[p]++;
      if (msg) st.conn[(size_t)sp * K + p]++;
    }
  }
  if (msg) {
    if (metric == FP_METRIC_MSM)
      for (int p = 0; p < K; p++) st.conn[(size_t)p * K + p] = -1;   // MSM/partition.cpp:101
    if (s->conn) st.conn.assign(s->conn, s->conn + (size_t)K * K);
    for (int a = 0; a < K; a++)
      for (int b = 0; b < K; b++)
        if (a != b && st.conn[(size_t)a * K + b] > 0) st.msgs[a]++;
    if (s->msgs) st.msgs.assign(s->msgs, s->msgs + K);
  }
  if (s->send && keep_send) st.send.assign(s->send, s->send + K);
  if (s->recv && keep_recv) st.recv.assign(s->recv, s->recv + K);
  return FP_OK;
}

}  // namespace fp

extern "C" {

int fp_stream_partition(const fp_hypergraph* h, int32_t K, int32_t metric, double eps_factor, fp_state* out) {
  return fp::guarded([&]() -> int {
    if (!h || !out) return FP_ERR_INVALID;
    fp::HostGraph g;
    fp::Problem pb;
    int rc = fp::make_problem(h, K, metric, eps_factor, g, pb);
    if (rc) return rc;
    fp::HostState st;
    rc = fp::initial_partition(pb, st);
    if (rc) return rc;
    const size_t KK = (size_t)K * K;
    if (out->part_vec) std::copy(st.part_vec.begin(), st.part_vec.end(), out->part_vec);
    if (out->ep_starts)
      for (int e = 0; e < g.noe; e++) out->ep_starts[e] = (int)g.nptr[e];
    if (out->ep_ends)
      std::copy(st.ep_len.begin(), st.ep_len.end(), out->ep_ends);
    if (out->ep_parts) std::copy(st.ep_part.begin(), st.ep_part.end(), out->ep_parts);
    if (out->ep_cnt) std::copy(st.ep_cnt.begin(), st.ep_cnt.end(), out->ep_cnt);
    if (out->part_sizes) std::copy(st.part_sizes.begin(), st.part_sizes.end(), out->part_sizes);
    if (out->marker) std::copy(st.marker.begin(), st.marker.end(), out->marker);
    if (out->send) std::copy(st.send.begin(), st.send.end(), out->send);
    if (out->recv) std::copy(st.recv.begin(), st.recv.end(), out->recv);
    if (out->msgs) std::copy(st.msgs.begin(), st.msgs.end(), out->msgs);
    if (out->conn) {
      if (st.conn.size() == KK) std::copy(st.conn.begin(), st.conn.end(), out->conn);
      else std::fill(out->conn, out->conn + KK, 0);
    }
    return FP_OK;
  });
}


int fp_check_state(const fp_hypergraph* h, int32_t K, int32_t metric, double eps_factor, const fp_state* st) {
  return fp::guarded([&]() -> int {
    if (!h || !st) return FP_ERR_INVALID;
    fp::HostGraph g;
    fp::Problem pb;
    int rc = fp::make_problem(h, K, metric, eps_factor, g, pb);
    if (rc) return rc;
    fp::HostState hs;
    return fp::state_from_caller(g, pb, st, hs);
  });
}

int fp_generate(const fp_gen_params* p, fp_graph** out) {
  return fp::guarded([&]() -> int {
    if (!p || !out) return FP_ERR_INVALID;
    *out = nullptr;
    fp::GenParams gp;
    gp.nov = p->nov; gp.noe = p->noe;
    gp.size_lo = p->size_lo; gp.size_hi = p->size_hi;
    gp.size_alpha = p->size_alpha; gp.pin_beta = p->pin_beta;
    gp.src_rule = p->src_rule; gp.sort_pins = p->sort_pins; gp.weight_rule = p->weight_rule;
    gp.seed = p->seed;
    std::unique_ptr<fp_graph> g(new (std::nothrow) fp_graph);
    if (!g) return FP_ERR_NOMEM;
    int rc = fp::generate(gp, g->g);
    if (rc) return rc;
    *out = g.release();
    return FP_OK;
  });
}

int fp_graph_from_nets(int32_t nov, int32_t noe, const uint32_t* nptr, const uint32_t* npins, const int32_t* src,
                       fp_graph** out) {
  return fp::guarded([&]() -> int {
    if (!out || nov <= 0 || noe < 0 || !nptr || nptr[0] != 0 || (!npins && nptr[noe] > 0)) return FP_ERR_INVALID;
    *out = nullptr;
    for (int e = 0; e < noe; e++)
      if (nptr[e + 1] < nptr[e]) return FP_ERR_INVALID;
    std::unique_ptr<fp_graph> gg(new (std::nothrow) fp_graph);
    if (!gg) return FP_ERR_NOMEM;
    HostGraph& g = gg->g;
    g.nov = nov;
    g.noe = noe;
    g.pins = nptr[noe];
    g.nptr.assign(nptr, nptr + noe + 1);
    g.npins.assign(npins, npins + g.pins);
    for (uint32_t x : g.npins)
      if (x >= (uint32_t)nov) return FP_ERR_INVALID;
    if (src) g.src.assign(src, src + noe);
    else choose_sources(g, 0);
    fp::build_vertex_csr(g);
    *out = gg.release();
    return FP_OK;
  });
}

int fp_graph_from_vertices(int32_t nov, int32_t noe, const uint32_t* vptr, const uint32_t* vnets, const int32_t* src,
                           fp_graph** out) {
  return fp::guarded([&]() -> int {
    if (!out || nov <= 0 || noe < 0 || !vptr || vptr[0] != 0 || (!vnets && vptr[nov] > 0)) return FP_ERR_INVALID;
    *out = nullptr;
    for (int v = 0; v < nov; v++)
      if (vptr[v + 1] < vptr[v]) return FP_ERR_INVALID;
    std::unique_ptr<fp_graph> gg(new (std::nothrow) fp_graph);
    if (!gg) return FP_ERR_NOMEM;
    HostGraph& g = gg->g;
    g.nov = nov;
    g.noe = noe;
    g.pins = vptr[nov];
    g.vptr.assign(vptr, vptr + nov + 1);
    g.vnets.assign(vnets, vnets + g.pins);
    for (uint32_t x : g.vnets)
      if (x >= (uint32_t)noe) return FP_ERR_INVALID;
    build_net_csr(g);
    if (src) g.src.assign(src, src + noe);
    else choose_sources(g, 0);
    *out = gg.release();
    return FP_OK;
  });
}

int fp_bfs_order(const fp_hypergraph* h, int32_t start, int32_t* ordering, int32_t* far_out) {
  return fp::guarded([&]() -> int {
    if (!h || !ordering) return FP_ERR_INVALID;
    int rc = fp_validate(h);
    if (rc) return rc;
    const int nov = h->nov, noe = h->noe;
    if (start < 0 || start >= nov) return FP_ERR_INVALID;
    // net -> pins with the pins of a net in ascending vertex id: the order the
    // reference's createInverse builds and its BFS walks (shared/utils.cpp:32-56)
    std::vector<uint32_t> iptr(noe + 1, 0), ipins(h->pins);
    for (long long k = 0; k < h->pins; k++) iptr[h->vnets[k] + 1]++;
    for (int e = 0; e < noe; e++) iptr[e + 1] += iptr[e];
    {
      std::vector<uint32_t> fill(iptr.begin(), iptr.end() - 1);
      for (int v = 0; v < nov; v++)
        for (uint32_t k = h->vptr[v]; k < h->vptr[v + 1]; k++) ipins[fill[h->vnets[k]]++] = (uint32_t)v;
    }
    // One level at a time, frontier in discovery order: a vertex's nets in
    // vertex -> nets order, a net's pins in ascending id (the one-thread walk of
    // topDown, shared/utils.cpp:538-590).
    std::vector<int> dist(nov), queue, next;
    auto bfs = [&](int s, int32_t* order) {
      std::fill(dist.begin(), dist.end(), -1);
      queue.assign(1, s);
      dist[s] = 0;
      int n = 0, level = 0;
      if (order) order[n++] = s;
      while (!queue.empty()) {
        next.clear();
        for (int v : queue)
          for (uint32_t k = h->vptr[v]; k < h->vptr[v + 1]; k++) {
            const uint32_t e = h->vnets[k];
            for (uint32_t j = iptr[e]; j < iptr[e + 1]; j++) {
              const int u = (int)ipins[j];
              if (dist[u] < 0) {
                dist[u] = level + 1;
                next.push_back(u);
              }
            }
          }
        if (next.empty()) break;
        level++;
        if (order)
          for (int u : next) order[n++] = u;
        queue.swap(next);
      }
      return n;
    };
    // the farthest vertex: the lowest id at the largest distance
    // (bfsFarthest_queue_par, shared/utils.cpp:433-480)
    auto farthest = [&]() {
      int f = -1, fd = -1;
      for (int i = 0; i < nov; i++)
        if (dist[i] > fd) { f = i; fd = dist[i]; }
      return f;
    };
    bfs(start, nullptr);
    const int f1 = farthest();
    bfs(f1, nullptr);
    const int f2 = farthest();
    for (int i = 0; i < nov; i++) ordering[i] = -1;
    const int reached = bfs(f2, ordering);   // bfsOrdering_queue_par, shared/utils.cpp:482-536
    if (far_out) { far_out[0] = f1; far_out[1] = f2; }
    return reached == nov ? FP_OK : FP_ERR_UNSUPPORTED;
  });
}

int fp_thin_nets(const fp_hypergraph* h, int32_t thin_mean, int32_t thin_min, fp_graph** out) {
  return fp::guarded([&]() -> int {
    if (!h || !out) return FP_ERR_INVALID;
    *out = nullptr;
    const int rc = fp_validate(h);
    if (rc) return rc;
    const int nov = h->nov, noe = h->noe;
    // mean net size in float, as the driver computes it: pins / (noe + .0f)
    const double mean = noe > 0 ? (double)((float)h->pins / ((float)noe + 0.0f)) : 0.0;
    std::unique_ptr<fp_graph> gg(new (std::nothrow) fp_graph);
    if (!gg) return FP_ERR_NOMEM;
    HostGraph& g = gg->g;
    g.nov = nov;
    std::vector<int> renum(noe, -1);
    g.nptr.assign(1, 0);
    for (int e = 0; e < noe; e++) {
      const int degree = (int)(h->nptr[e + 1] - h->nptr[e]);
      if (degree < thin_mean * mean && degree < thin_min) {
        renum[e] = (int)g.src.size();
        g.npins.insert(g.npins.end(), h->npins + h->nptr[e], h->npins + h->nptr[e + 1]);
        g.nptr.push_back((uint32_t)g.npins.size());
        g.src.push_back(h->src[e]);
      }
    }
    g.noe = (int)g.src.size();
    g.pins = (long long)g.npins.size();
    // each vertex keeps its kept nets in its own net order, renumbered
    g.vptr.assign(nov + 1, 0);
    g.vnets.reserve(g.pins);
    for (int v = 0; v < nov; v++) {
      for (uint32_t k = h->vptr[v]; k < h->vptr[v + 1]; k++)
        if (renum[h->vnets[k]] >= 0) g.vnets.push_back((uint32_t)renum[h->vnets[k]]);
      g.vptr[v + 1] = (uint32_t)g.vnets.size();
    }
    if (h->weights) g.weights.assign(h->weights, h->weights + nov);
    *out = gg.release();
    return FP_OK;
  });
}

int fp_read_patohlike(const char* path, int32_t transpose, int32_t write_cache, fp_graph** out) {
  return fp::guarded([&]() -> int {
    if (!path || !out) return FP_ERR_INVALID;
    *out = nullptr;
    int nov = 0, noe = 0;
    long long pins = 0;
    std::vector<uint32_t> lptr, lids;
    const std::string bin = std::string(path) + ".plbin";
    bool ok = read_plbin(bin, nov, noe, pins, lptr, lids);
    if (!ok) {
      if (!parse_text(path, nov, noe, pins, lptr, lids)) return FP_ERR_IO;
      if (write_cache) write_plbin(bin, nov, noe, pins, lptr, lids);
    }
    std::unique_ptr<fp_graph> gg(new (std::nothrow) fp_graph);
    if (!gg) return FP_ERR_NOMEM;
    HostGraph& g = gg->g;
    g.pins = pins;
    if (transpose) {
      // File lines are nets (TV/tv.cpp:51-80, CN/cn.cpp:154-177).
      g.nov = nov;
      g.noe = noe;
      g.nptr = std::move(lptr);
      g.npins = std::move(lids);
      fp::build_vertex_csr(g);
    } else {
      // File lines are vertices, ids are nets (TM/tm.cpp:65): needs a square file.
      if (nov != noe) return FP_ERR_INVALID;
      g.nov = noe;
      g.noe = nov;
      g.vptr = std::move(lptr);
      g.vnets = std::move(lids);
      build_net_csr(g);
    }
    choose_sources(g, 0);
    *out = gg.release();
    return FP_OK;
  });
}

int fp_write_patohlike(const fp_graph* gg, const char* path) {
  return fp::guarded([&]() -> int {
    if (!gg || !path) return FP_ERR_INVALID;
    const HostGraph& g = gg->g;
    FILE* f = std::fopen(path, "w");
    if (!f) return FP_ERR_IO;
    std::fprintf(f, "0 %d %d %lld\n", g.nov, g.noe, g.pins);
    for (int e = 0; e < g.noe; e++) {
      for (uint32_t k = g.nptr[e]; k < g.nptr[e + 1]; k++)
        std::fprintf(f, k + 1 < g.nptr[e + 1] ? "%u " : "%u", g.npins[k]);
      std::fputc('\n', f);
    }
    return std::fclose(f) == 0 ? FP_OK : FP_ERR_IO;
  });
}

int fp_graph_view(const fp_graph* gg, fp_hypergraph* v) {
  return fp::guarded([&]() -> int {
    if (!gg || !v) return FP_ERR_INVALID;
    const HostGraph& g = gg->g;
    v->nov = g.nov;
    v->noe = g.noe;
    v->pins = g.pins;
    v->vptr = g.vptr.data();
    v->vnets = g.vnets.data();
    v->nptr = g.nptr.data();
    v->npins = g.npins.data();
    v->src = g.src.data();
    v->weights = g.weights.empty() ? nullptr : g.weights.data();
    v->ordering = nullptr;
    return FP_OK;
  });
}

int fp_graph_destroy(fp_graph* g) {
  return fp::guarded([&]() -> int {
    if (!g) return FP_ERR_INVALID;
    delete g;
    return FP_OK;
  });
}

// Drop-in body of the reference's partition_gpu(): host stream, metric lines,
// REFI_ITER device passes, metric lines again (e.g. TV/partition.cpp:984-1184).
int fp_partition_gpu(int32_t metric, const uint32_t* row_ptr, const uint32_t* col_ind, const uint32_t* net_appearence,
                     int32_t nov, int32_t noe, int64_t pins, const int32_t* edge_wgths, const int32_t* src_nodes,
                     int32_t K, const int32_t* ordering, const char* f_name, int32_t REFI_OPT, int32_t REFI_ITER,
                     const uint32_t* row_ptr_inv, const uint32_t* col_ind_inv, int32_t* part_vec_out,
                     int64_t* metrics_out) {
  return fp::guarded([&]() -> int {
    (void)edge_wgths;      // unused by the reference as well
    (void)net_appearence;  // net sizes follow from the CSR
    (void)f_name;
    if (!row_ptr || !col_ind || !src_nodes || nov <= 0 || noe < 0 || pins < 0) return FP_ERR_INVALID;
    HostGraph g;
    g.nov = nov;
    g.noe = noe;
    g.pins = pins;
    g.vptr.assign(row_ptr, row_ptr + nov + 1);
    g.vnets.assign(col_ind, col_ind + pins);
    fp_ctx* ctx = nullptr;
    int rc = fp_ctx_create(0, &ctx);
    if (rc) return rc;
    if (row_ptr_inv && col_ind_inv) {
      g.nptr.assign(row_ptr_inv, row_ptr_inv + noe + 1);
      g.npins.assign(col_ind_inv, col_ind_inv + pins);
    } else {
      // the reference's createInverse, on the device (fp_create_inverse)
      g.nptr.resize((size_t)noe + 1);
      g.npins.resize((size_t)std::max<long long>(pins, 1));
      rc = fp_create_inverse(ctx, nov, noe, pins, row_ptr, col_ind, g.nptr.data(), g.npins.data());
      g.npins.resize(pins);
      if (rc) { fp_ctx_destroy(ctx); return rc; }
    }
    g.src.assign(src_nodes, src_nodes + noe);
    fp_hypergraph h;
    h.nov = nov;
    h.noe = noe;
    h.pins = pins;
    h.vptr = g.vptr.data();
    h.vnets = g.vnets.data();
    h.nptr = g.nptr.data();
    h.npins = g.npins.data();
    h.src = g.src.data();
    h.weights = nullptr;
    h.ordering = ordering;

    fp_instance* inst = nullptr;
    rc = fp_instance_create(ctx, &h, K, metric, 1.05, &inst);
    if (rc) { fp_ctx_destroy(ctx); return rc; }
    int64_t before[6] = {0}, after[6] = {-1, -1, -1, -1, -1, -1};
    static const char* names[6] = {"TV", "CN", "TM", "MGM", "MGV", "MGAV"};
    if ((rc = fp_initial_partition(inst)) == FP_OK && (rc = fp_metrics(inst, before)) == FP_OK) {
      for (int i = 0; i < 6; i++) std::printf("%s : %lld\n", names[i], (long long)before[i]);
      auto t0 = std::chrono::steady_clock::now();
      if (REFI_OPT) rc = fp_refine(inst, REFI_ITER);
      auto t1 = std::chrono::steady_clock::now();
      if (rc == FP_OK) {
        std::printf("Refinement took : %g seconds.\n", std::chrono::duration<double>(t1 - t0).count());
        if (REFI_OPT) rc = fp_metrics(inst, after);
      }
      if (rc == FP_OK) {
        for (int i = 0; i < 6; i++) std::printf("After Refinement %s : %lld\n", names[i], (long long)after[i]);
        for (int i = 0; i < 6; i++) {
          if (REFI_OPT)
            std::printf("Improved Percentage %s : %g\n", names[i], 100.0 - ((double)after[i] / before[i]) * 100);
          else
            std::printf("Improved Percentage %s : -1\n", names[i]);
        }
        std::printf("Iterated for : %d times\n", REFI_OPT ? REFI_ITER : 0);
        if (part_vec_out) rc = fp_get_partition(inst, part_vec_out);
        if (metrics_out) {
          for (int i = 0; i < 6; i++) { metrics_out[i] = before[i]; metrics_out[6 + i] = after[i]; }
        }
      }
    }
    std::fflush(stdout);
    fp_instance_destroy(inst);
    fp_ctx_destroy(ctx);
    return rc;
  });
}

}  // extern "C"
