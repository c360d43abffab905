// Seeded synthetic hypergraph generator for the workloads FastPartitioner's
// refinement is measured on (no public dataset is used: every instance is drawn
// from a stated distribution with a fixed seed).
//
//   net sizes : uniform [lo, hi]  or  Zipf(alpha) on {1, 2, ...} clipped to [lo, hi]
//   pins      : uniform over vertices, or proportional to a Zipf(beta) popularity
//               whose ranks are randomly permuted over vertex ids; no vertex is
//               drawn twice within a net
//   source    : lowest-id pin, or first drawn pin
//
// The vertex -> nets CSR is the transpose of the net -> pins CSR with nets in
// ascending id order per vertex, which is what FastPartitioner's TV and CN drivers
// build (TV/tv.cpp:56-80).
//
// Randomness: splitmix64-seeded xoshiro256**; uniform doubles from the top 53 bits.

#include "fp_internal.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#include <numeric>

namespace fp {

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) {
      x += 0x9E3779B97F4A7C15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s[i] = z ^ (z >> 31);
    }
  }
  static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  inline uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // Unbiased integer in [0, n) (Lemire's multiply-shift with rejection).
  inline uint64_t below(uint64_t n) {
    uint64_t x = next();
    __uint128_t m = (__uint128_t)x * n;
    uint64_t l = (uint64_t)m;
    if (l < n) {
      uint64_t t = (0 - n) % n;
      while (l < t) {
        x = next();
        m = (__uint128_t)x * n;
        l = (uint64_t)m;
      }
    }
    return (uint64_t)(m >> 64);
  }
};

// Walker alias table over arbitrary non-negative weights.
struct Alias {
  std::vector<double> prob;
  std::vector<uint32_t> alias;
  void build(const std::vector<double>& w) {
    size_t n = w.size();
    prob.assign(n, 0.0);
    alias.assign(n, 0);
    double sum = 0;
    for (double x : w) sum += x;
    std::vector<double> scaled(n);
    std::vector<uint32_t> small, large;
    small.reserve(n);
    large.reserve(n);
    for (size_t i = 0; i < n; i++) {
      scaled[i] = w[i] * (double)n / sum;
      (scaled[i] < 1.0 ? small : large).push_back((uint32_t)i);
    }
    while (!small.empty() && !large.empty()) {
      uint32_t s = small.back(); small.pop_back();
      uint32_t l = large.back();
      prob[s] = scaled[s];
      alias[s] = l;
      scaled[l] = (scaled[l] + scaled[s]) - 1.0;
      if (scaled[l] < 1.0) { large.pop_back(); small.push_back(l); }
    }
    for (uint32_t i : large) prob[i] = 1.0;
    for (uint32_t i : small) prob[i] = 1.0;
  }
  inline uint32_t sample(Rng& r) const {
    uint32_t i = (uint32_t)r.below(prob.size());
    return r.uniform() < prob[i] ? i : alias[i];
  }
};

// Zipf(alpha) on {1, 2, ...} clipped to [lo, hi]: mass above hi is put on hi,
// mass below lo on lo.
std::vector<double> clipped_zipf_weights(double alpha, int lo, int hi) {
  // zeta(alpha) by direct summation plus an Euler-Maclaurin tail.
  const int N = std::max(hi, 1 << 20);
  double head = 0;
  for (int s = N; s >= 1; s--) head += std::pow((double)s, -alpha);
  double tail = std::pow((double)N, 1.0 - alpha) / (alpha - 1.0) - 0.5 * std::pow((double)N, -alpha);
  double zeta = head + tail;
  std::vector<double> w(hi - lo + 1, 0.0);
  double below = 0, inside = 0;
  for (int s = 1; s < lo; s++) below += std::pow((double)s, -alpha);
  for (int s = lo; s <= hi; s++) {
    w[s - lo] = std::pow((double)s, -alpha);
    inside += w[s - lo];
  }
  w[0] += below;
  w[hi - lo] += std::max(0.0, zeta - below - inside);
  return w;
}

}  // namespace

int generate(const GenParams& p, HostGraph& g) {
  if (p.nov <= 0 || p.noe < 0 || p.size_lo < 1 || p.size_hi < p.size_lo || p.size_hi > p.nov)
    return FP_ERR_INVALID;
  Rng rng(p.seed);
  g.nov = p.nov;
  g.noe = p.noe;

  // Net sizes.
  std::vector<int> sizes(p.noe);
  if (p.size_alpha > 0) {
    Alias a;
    a.build(clipped_zipf_weights(p.size_alpha, p.size_lo, p.size_hi));
    for (int e = 0; e < p.noe; e++) sizes[e] = p.size_lo + (int)a.sample(rng);
  } else {
    for (int e = 0; e < p.noe; e++) sizes[e] = p.size_lo + (int)rng.below(p.size_hi - p.size_lo + 1);
  }
  g.nptr.assign(p.noe + 1, 0);
  for (int e = 0; e < p.noe; e++) g.nptr[e + 1] = g.nptr[e] + (uint32_t)sizes[e];
  long long pins = g.nptr[p.noe];
  g.pins = pins;
  g.npins.assign(pins, 0);

  // Pin sampler.
  Alias pop;
  std::vector<uint32_t> rank_to_vertex;
  const bool zipf_pins = p.pin_beta > 0;
  if (zipf_pins) {
    std::vector<double> w(p.nov);
    for (int r = 0; r < p.nov; r++) {
      double x = (double)(r + 1);
      w[r] = 1.0 / std::pow(x, p.pin_beta);
    }
    pop.build(w);
    rank_to_vertex.resize(p.nov);
    std::iota(rank_to_vertex.begin(), rank_to_vertex.end(), 0u);
    for (int i = p.nov - 1; i > 0; i--) std::swap(rank_to_vertex[i], rank_to_vertex[rng.below(i + 1)]);
  }
  std::vector<int> stamp(p.nov, -1);
  for (int e = 0; e < p.noe; e++) {
    uint32_t* out = &g.npins[g.nptr[e]];
    int s = sizes[e];
    for (int k = 0; k < s;) {
      uint32_t v = zipf_pins ? rank_to_vertex[pop.sample(rng)] : (uint32_t)rng.below(p.nov);
      if (stamp[v] == e) continue;
      stamp[v] = e;
      out[k++] = v;
    }
  }

  // Sources, then the pin order the workload asks for.
  g.src.assign(p.noe, -1);
  for (int e = 0; e < p.noe; e++) {
    uint32_t* b = &g.npins[g.nptr[e]];
    uint32_t* en = &g.npins[g.nptr[e + 1]];
    if (b == en) continue;
    if (p.src_rule == 0) g.src[e] = (int)*std::min_element(b, en);
    else g.src[e] = (int)*b;
    if (p.sort_pins) std::sort(b, en);
  }
  build_vertex_csr(g);

  g.weights.clear();
  if (p.weight_rule == 1) {
    g.weights.resize(p.nov);
    for (int v = 0; v < p.nov; v++) g.weights[v] = (int)(g.vptr[v + 1] - g.vptr[v]);
  }
  return FP_OK;
}

void build_vertex_csr(HostGraph& g) {
  g.vptr.assign(g.nov + 1, 0);
  for (long long k = 0; k < g.pins; k++) g.vptr[g.npins[k] + 1]++;
  for (int v = 0; v < g.nov; v++) g.vptr[v + 1] += g.vptr[v];
  g.vnets.assign(g.pins, 0);
  std::vector<uint32_t> fill(g.vptr.begin(), g.vptr.end() - 1);
  for (int e = 0; e < g.noe; e++)
    for (uint32_t k = g.nptr[e]; k < g.nptr[e + 1]; k++) g.vnets[fill[g.npins[k]]++] = (uint32_t)e;
}

}  // namespace fp
