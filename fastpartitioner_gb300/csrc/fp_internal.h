// Internal host-side types shared by the library's translation units.
#pragma once

#include <cstdint>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fastpart.h"

namespace fp {

// A hypergraph owned by the host library: vertex -> nets and net -> pins CSRs,
// one source vertex per net, optional vertex weights.
struct HostGraph {
  int nov = 0, noe = 0;
  long long pins = 0;
  std::vector<uint32_t> vptr, vnets, nptr, npins;
  std::vector<int> src, weights;
};

struct GenParams {
  int nov = 0, noe = 0;
  int size_lo = 2, size_hi = 2;
  double size_alpha = 0;   // > 0: clipped Zipf net sizes; else uniform
  double pin_beta = 0;     // > 0: Zipf pin popularity; else uniform pins
  int src_rule = 0;        // 0: lowest-id pin, 1: first drawn pin
  int sort_pins = 1;       // sort each net's pins by vertex id
  int weight_rule = 0;     // 0: unit weights, 1: weight = vertex degree
  uint64_t seed = 0;
};

int generate(const GenParams& p, HostGraph& g);
void build_vertex_csr(HostGraph& g);

// Refinement state laid out exactly as the device engine consumes it.
struct HostState {
  std::vector<int> part_vec;     // nov
  std::vector<int> part_sizes;   // K (weighted sizes)
  std::vector<int> ep_start;     // noe + 1, net slot offsets (= net sizes prefix)
  std::vector<int> ep_len;       // noe, parts present in the net
  std::vector<int> ep_part;      // pins, ordered part list per net
  std::vector<int> ep_cnt;       // pins, pins of that part in the net
  std::vector<int> marker;       // K, TV: last vertex that scanned each part
  std::vector<int> send, recv;   // K, MSV / MSRV volumes
  std::vector<int> conn;         // K*K, TM / MSM connection counts (row-major)
  std::vector<int> msgs;         // K, TM / MSM messages per part
};

struct Problem {
  const HostGraph* g;
  int K;
  int metric;
  double eps_factor;
  std::vector<int> w;      // per-vertex weight
  std::vector<int> order;  // visiting order
  int xw;                  // (sum of weights) / K
  double C;                // xw * eps_factor
};

// Streaming initial partitioners (host).  Return FP_OK or an error code.
int initial_partition(const Problem& pb, HostState& st);

// Largest K the library supports (13-bit list slots in the device records).
constexpr int kMaxK = 4096;

// Copies a validated hypergraph into g and fills pb (weights, visiting order,
// xw = W / K, C = xw * eps_factor) as the reference derives them.
int make_problem(const fp_hypergraph* h, int K, int metric, double eps_factor, HostGraph& g, Problem& pb);

// Checks a caller's state in the reference's layout (fp_state: ep_ends[e] is
// the number of parts listed for net e) against g and pb and converts it into
// the engine's host state; FP_ERR_INVALID if it is not the recount of part_vec.
int state_from_caller(const HostGraph& g, const Problem& pb, const fp_state* s, HostState& st);

// Runs an entry point's body and turns a C++ exception into a status code, so
// that nothing thrown crosses the C ABI: a failed allocation is FP_ERR_NOMEM,
// anything else FP_ERR_INVALID.  `on_throw` releases what the body had built.
template <class Body, class Cleanup>
int guarded(Body&& body, Cleanup&& on_throw) noexcept {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    on_throw();
    return FP_ERR_NOMEM;
  } catch (...) {
    on_throw();
    return FP_ERR_INVALID;
  }
}

template <class Body>
int guarded(Body&& body) noexcept {
  return guarded(std::forward<Body>(body), [] {});
}

}  // namespace fp

// Opaque handle of the public header: a host-owned hypergraph.
struct fp_graph {
  fp::HostGraph g;
};
