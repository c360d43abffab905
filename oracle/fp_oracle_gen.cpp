// Workload generator of the oracle -- TEST INFRASTRUCTURE ONLY.
//
// bench.py's reference arm runs the reference's own partition_par() on the same
// seeded synthetic instance as the GPU arm without loading the product library,
// so the instance is drawn here and written straight to the .fphg file that the
// reference harness (ref_harness.cpp) reads.  The draws must be the product
// generator's, bit for bit (tests/test_oracle_gen.py compares the files):
//
//   RNG        xoshiro256** seeded by four splitmix64 outputs; a uniform double
//              from the top 53 bits; an integer below n by Lemire's
//              multiply-shift with rejection
//   net sizes  uniform [lo, hi] or a Walker alias table over Zipf(alpha) on
//              {1, 2, ...} clipped to [lo, hi] (mass below lo on lo, above hi on hi;
//              zeta by summation down from max(hi, 2^20) plus an Euler-Maclaurin tail)
//   pins       uniform, or an alias table over Zipf(beta) popularity by rank with
//              ranks shuffled over vertex ids (Fisher-Yates from the top); a
//              vertex drawn twice in one net is drawn again
//   source     lowest-id pin (rule 0) or first drawn pin (rule 1); pins sorted
//              per net when asked
//   vertices   vertex -> nets is the transpose, nets ascending per vertex
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <numeric>
#include <vector>

namespace {

struct Xoshiro {
  uint64_t s[4];
  explicit Xoshiro(uint64_t seed) {
    uint64_t x = seed;
    for (auto& w : s) {
      x += 0x9E3779B97F4A7C15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      w = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t out = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return out;
  }
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  uint64_t below(uint64_t n) {
    __uint128_t m = (__uint128_t)next() * n;
    if ((uint64_t)m < n) {
      const uint64_t floor = (0 - n) % n;
      while ((uint64_t)m < floor) m = (__uint128_t)next() * n;
    }
    return (uint64_t)(m >> 64);
  }
};

// Walker's alias method: the index with probability weight[i] / sum.
struct AliasTable {
  std::vector<double> keep;
  std::vector<uint32_t> other;
  explicit AliasTable(const std::vector<double>& weight) {
    const size_t n = weight.size();
    keep.assign(n, 0.0);
    other.assign(n, 0);
    double total = 0;
    for (double x : weight) total += x;
    std::vector<double> q(n);
    std::vector<uint32_t> lo, hi;
    for (size_t i = 0; i < n; i++) {
      q[i] = weight[i] * (double)n / total;
      if (q[i] < 1.0) lo.push_back((uint32_t)i);
      else hi.push_back((uint32_t)i);
    }
    while (!lo.empty() && !hi.empty()) {
      const uint32_t a = lo.back();
      lo.pop_back();
      const uint32_t b = hi.back();
      keep[a] = q[a];
      other[a] = b;
      q[b] = (q[b] + q[a]) - 1.0;
      if (q[b] < 1.0) {
        hi.pop_back();
        lo.push_back(b);
      }
    }
    for (uint32_t i : hi) keep[i] = 1.0;
    for (uint32_t i : lo) keep[i] = 1.0;
  }
  uint32_t draw(Xoshiro& r) const {
    const uint32_t i = (uint32_t)r.below(keep.size());
    return r.unit() < keep[i] ? i : other[i];
  }
};

std::vector<double> zipf_clipped(double alpha, int lo, int hi) {
  const int top = std::max(hi, 1 << 20);
  double zeta = 0;
  for (int k = top; k >= 1; k--) zeta += std::pow((double)k, -alpha);
  zeta += std::pow((double)top, 1.0 - alpha) / (alpha - 1.0) - 0.5 * std::pow((double)top, -alpha);
  std::vector<double> w(hi - lo + 1);
  double under = 0, in = 0;
  for (int k = 1; k < lo; k++) under += std::pow((double)k, -alpha);
  for (int k = lo; k <= hi; k++) {
    w[k - lo] = std::pow((double)k, -alpha);
    in += w[k - lo];
  }
  w[0] += under;
  w[hi - lo] += std::max(0.0, zeta - under - in);
  return w;
}

}  // namespace

// Draws the instance and writes it as an FPHG1 file (magic, nov, noe, pins,
// vptr, vnets, nptr, npins, src).  Returns 0, or -1 on bad parameters or I/O.
extern "C" int fpo_generate_fphg(int nov, int noe, int size_lo, int size_hi, double size_alpha, double pin_beta,
                                 int src_rule, int sort_pins, unsigned long long seed, const char* path) {
  if (nov <= 0 || noe < 0 || size_lo < 1 || size_hi < size_lo || size_hi > nov) return -1;
  Xoshiro rng(seed);
  std::vector<uint32_t> nptr(noe + 1, 0);
  {
    std::vector<int> size(noe);
    if (size_alpha > 0) {
      AliasTable t(zipf_clipped(size_alpha, size_lo, size_hi));
      for (int e = 0; e < noe; e++) size[e] = size_lo + (int)t.draw(rng);
    } else {
      for (int e = 0; e < noe; e++) size[e] = size_lo + (int)rng.below(size_hi - size_lo + 1);
    }
    for (int e = 0; e < noe; e++) nptr[e + 1] = nptr[e] + (uint32_t)size[e];
  }
  const long long pins = nptr[noe];
  std::vector<uint32_t> npins(pins);
  std::vector<uint32_t> id_of_rank;
  std::vector<double> pop;
  if (pin_beta > 0) {
    pop.resize(nov);
    for (int r = 0; r < nov; r++) pop[r] = 1.0 / std::pow((double)(r + 1), pin_beta);
  }
  AliasTable popularity(pin_beta > 0 ? pop : std::vector<double>{1.0});
  if (pin_beta > 0) {
    id_of_rank.resize(nov);
    std::iota(id_of_rank.begin(), id_of_rank.end(), 0u);
    for (int i = nov - 1; i > 0; i--) std::swap(id_of_rank[i], id_of_rank[rng.below(i + 1)]);
  }
  std::vector<int> seen(nov, -1);
  for (int e = 0; e < noe; e++) {
    for (uint32_t k = nptr[e]; k < nptr[e + 1];) {
      const uint32_t v = pin_beta > 0 ? id_of_rank[popularity.draw(rng)] : (uint32_t)rng.below(nov);
      if (seen[v] == e) continue;
      seen[v] = e;
      npins[k++] = v;
    }
  }
  std::vector<int> src(noe, -1);
  for (int e = 0; e < noe; e++) {
    uint32_t* b = npins.data() + nptr[e];
    uint32_t* en = npins.data() + nptr[e + 1];
    if (b == en) continue;
    src[e] = src_rule == 0 ? (int)*std::min_element(b, en) : (int)*b;
    if (sort_pins) std::sort(b, en);
  }
  std::vector<uint32_t> vptr(nov + 1, 0), vnets(pins);
  for (long long k = 0; k < pins; k++) vptr[npins[k] + 1]++;
  for (int v = 0; v < nov; v++) vptr[v + 1] += vptr[v];
  {
    std::vector<uint32_t> at(vptr.begin(), vptr.end() - 1);
    for (int e = 0; e < noe; e++)
      for (uint32_t k = nptr[e]; k < nptr[e + 1]; k++) vnets[at[npins[k]]++] = (uint32_t)e;
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return -1;
  bool ok = std::fwrite("FPHG1\0\0\0", 1, 8, f) == 8;
  ok = ok && std::fwrite(&nov, 4, 1, f) == 1 && std::fwrite(&noe, 4, 1, f) == 1 && std::fwrite(&pins, 8, 1, f) == 1;
  ok = ok && std::fwrite(vptr.data(), 4, vptr.size(), f) == vptr.size();
  ok = ok && std::fwrite(vnets.data(), 4, vnets.size(), f) == vnets.size();
  ok = ok && std::fwrite(nptr.data(), 4, nptr.size(), f) == nptr.size();
  ok = ok && std::fwrite(npins.data(), 4, npins.size(), f) == npins.size();
  ok = ok && std::fwrite(src.data(), 4, src.size(), f) == src.size();
  return std::fclose(f) == 0 && ok ? 0 : -1;
}
