// Seeded random constraint networks for the propagation engine's tests and
// benchmarks: model-B binary networks (as used by the reference's rand-2-*
// fixtures, samples/bench/rand-2-23), ternary positive tables, and the uneven
// multi-instance mix. Header-only so the engine, the benchmark driver and the
// test checkers all generate byte-identical instances from the same seed on
// any host (no libstdc++ distributions: every draw below is defined here).
//
// Value a of variable x is bit (a & 63) of word (a >> 6) of x's domain, LSB
// first, exactly the layout of the reference's IntVar::bit_doms_
// (include/Network.h:102-108). Bits at or beyond a domain's size are zero.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <unordered_set>
#include <vector>

#ifdef __CUDACC__
#define CPGEN_HD __host__ __device__
#else
#define CPGEN_HD
#endif

namespace cpgen {

CPGEN_HD inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Sequential stream used for structure (scopes, per-constraint tightness,
// tuples, removed values).
struct Stream {
  uint64_t s;
  explicit Stream(uint64_t seed) : s(mix64(seed ^ 0x5eed5eed5eedull)) {}
  uint64_t next() {
    s += 0x9e3779b97f4a7c15ull;
    return mix64(s);
  }
  // Uniform in [0, k).
  uint64_t below(uint64_t k) {
    return static_cast<uint64_t>((static_cast<unsigned __int128>(next()) * k) >> 64);
  }
  // Uniform in [0, 1).
  double unit() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }
};

inline int words_for(int d) { return d <= 0 ? 1 : (d + 63) / 64; }

// One constraint network. Binary relations are stored as support bit-rows:
// for constraint c with scope (x, y), row a (a < dom[x]) holds W words whose
// bit b is set iff (x=a, y=b) is an allowed tuple. Tables are positive
// (supports) tuple lists of any arity.
struct Instance {
  int n = 0;
  int W = 1;                        // u64 words per domain (max over variables)
  std::vector<int> dom;             // domain size per variable
  std::vector<uint64_t> init;       // n*W initial domain words
  std::vector<int> bx, by;          // binary scopes
  std::vector<int64_t> brow_off;    // word offset of constraint c's rows
  std::vector<uint64_t> brows;      // all binary support rows
  std::vector<int> tarity;          // table arity
  std::vector<int64_t> tscope_off;  // offset into tscope
  std::vector<int> tscope;          // table scopes
  std::vector<int> tntup;           // tuples per table
  std::vector<int64_t> ttup_off;    // offset into ttup (in ints)
  std::vector<int> ttup;            // tuples, row-major (arity ints each)
  std::vector<uint64_t> bseed;      // per binary constraint: relation seed
  std::vector<uint32_t> bthr;       // per binary constraint: tightness threshold

  int n_bin() const { return static_cast<int>(bx.size()); }
  int n_tab() const { return static_cast<int>(tarity.size()); }
  bool bit(int x, int a) const { return (init[size_t(x) * W + (a >> 6)] >> (a & 63)) & 1ull; }
  const uint64_t* row(int c, int a) const { return &brows[brow_off[c] + int64_t(a) * W]; }
  int64_t num_values() const {
    int64_t s = 0;
    for (int d : dom) s += d;
    return s;
  }
  // Total tuple count (binary relations counted by support bits).
  int64_t bin_tuples(int c) const {
    int64_t s = 0;
    for (int a = 0; a < dom[bx[c]]; ++a)
      for (int w = 0; w < W; ++w) s += __builtin_popcountll(row(c, a)[w]);
    return s;
  }
};

inline void init_full_domains(Instance& I) {
  I.init.assign(size_t(I.n) * I.W, 0);
  for (int x = 0; x < I.n; ++x)
    for (int a = 0; a < I.dom[x]; ++a) I.init[size_t(x) * I.W + (a >> 6)] |= 1ull << (a & 63);
}

// Support word w of row a of a binary relation with tightness threshold thr16
// (a tuple is forbidden iff a 16-bit uniform draw is below thr16). Counter
// based, so any word can be generated independently.
CPGEN_HD inline uint64_t relation_word(uint64_t cseed, int a, int w, uint32_t thr16, int dom_y) {
  uint64_t out = 0;
  for (int q = 0; q < 16; ++q) {
    const uint64_t h = mix64(cseed ^ mix64((uint64_t(uint32_t(a)) << 32) | (uint64_t(w) << 8) | uint64_t(q)));
    for (int k = 0; k < 4; ++k) {
      const uint32_t u = uint32_t(h >> (16 * k)) & 0xffffu;
      if (u >= thr16) out |= 1ull << (4 * q + k);
    }
  }
  const int lo = w * 64;
  if (dom_y - lo < 64) out &= (dom_y - lo <= 0) ? 0ull : ((1ull << (dom_y - lo)) - 1ull);
  return out;
}

inline uint32_t tightness_threshold(double p) {
  double t = std::floor(p * 65536.0 + 0.5);
  if (t < 0) t = 0;
  if (t > 65536) t = 65536;
  return uint32_t(t);
}

// Appends e binary constraints on distinct unordered variable pairs drawn
// uniformly; constraint c forbids each tuple independently with probability
// p_c, p_c uniform in [p_lo, p_hi] (p_lo == p_hi gives a fixed tightness).
// make_rows = false records each constraint's seed and threshold (bseed,
// bthr) without materialising the rows, for generators that build the rows
// on a GPU with the same relation_word.
inline void add_random_binary(Instance& I, int64_t e, double p_lo, double p_hi, Stream& S,
                              uint64_t seed, bool make_rows = true) {
  const int64_t total = int64_t(I.n) * (I.n - 1) / 2;
  if (e > total) throw std::invalid_argument("more binary constraints than variable pairs");
  std::unordered_set<uint64_t> seen;
  seen.reserve(size_t(e) * 2 + 16);
  const int64_t first = I.n_bin();
  while (I.n_bin() - first < e) {
    int x = int(S.below(I.n)), y = int(S.below(I.n));
    if (x == y) continue;
    if (x > y) std::swap(x, y);
    const uint64_t key = (uint64_t(x) << 32) | uint64_t(y);
    if (!seen.insert(key).second) continue;
    I.bx.push_back(x);
    I.by.push_back(y);
  }
  for (int64_t c = first; c < I.n_bin(); ++c) {
    const double p = (p_lo == p_hi) ? p_lo : p_lo + (p_hi - p_lo) * S.unit();
    const uint32_t thr = tightness_threshold(p);
    const uint64_t cseed = mix64(seed ^ mix64(0xB1A5B1A5ull + uint64_t(c)));
    const int x = I.bx[c], y = I.by[c];
    I.bseed.push_back(cseed);
    I.bthr.push_back(thr);
    if (!make_rows) continue;
    I.brow_off.push_back(int64_t(I.brows.size()));
    for (int a = 0; a < I.dom[x]; ++a)
      for (int w = 0; w < I.W; ++w) I.brows.push_back(w < words_for(I.dom[y]) ? relation_word(cseed, a, w, thr, I.dom[y]) : 0ull);
  }
}

// Appends k positive tables of the given arity on distinct sorted scopes,
// each with `ntup` distinct tuples drawn uniformly without replacement from
// the Cartesian product of the scope's domains.
inline void add_random_tables(Instance& I, int k, int arity, int ntup, Stream& S) {
  std::unordered_set<uint64_t> scopes;
  std::vector<int> sc(arity);
  int made = 0;
  while (made < k) {
    for (int i = 0; i < arity; ++i) sc[i] = int(S.below(I.n));
    std::sort(sc.begin(), sc.end());
    bool distinct = true;
    for (int i = 1; i < arity; ++i) distinct &= sc[i] != sc[i - 1];
    if (!distinct) continue;
    uint64_t key = 0;
    for (int i = 0; i < arity; ++i) key = key * 1000003ull + uint64_t(sc[i]);
    if (!scopes.insert(key).second) continue;
    double space = 1;
    for (int i = 0; i < arity; ++i) space *= I.dom[sc[i]];
    const int want = int(std::min<double>(ntup, space));
    I.tarity.push_back(arity);
    I.tscope_off.push_back(int64_t(I.tscope.size()));
    for (int i = 0; i < arity; ++i) I.tscope.push_back(sc[i]);
    I.ttup_off.push_back(int64_t(I.ttup.size()));
    I.tntup.push_back(want);
    std::unordered_set<uint64_t> tuples;
    tuples.reserve(size_t(want) * 2 + 16);
    std::vector<int> t(arity);
    while (int(tuples.size()) < want) {
      uint64_t code = 0;
      for (int i = 0; i < arity; ++i) {
        t[i] = int(S.below(I.dom[sc[i]]));
        code = code * uint64_t(I.dom[sc[i]]) + uint64_t(t[i]);
      }
      if (!tuples.insert(code).second) continue;
      for (int i = 0; i < arity; ++i) I.ttup.push_back(t[i]);
    }
    ++made;
  }
}

// Clears round(frac * total values) distinct (variable, value) bits.
inline void remove_random_values(Instance& I, double frac, Stream& S) {
  if (frac <= 0) return;
  std::vector<int64_t> ids;
  ids.reserve(size_t(I.num_values()));
  for (int x = 0; x < I.n; ++x)
    for (int a = 0; a < I.dom[x]; ++a) ids.push_back(int64_t(x) << 16 | a);
  const int64_t k = int64_t(std::floor(frac * double(ids.size()) + 0.5));
  for (int64_t i = 0; i < k; ++i) {
    const int64_t j = i + int64_t(S.below(uint64_t(ids.size() - i)));
    std::swap(ids[i], ids[j]);
    const int x = int(ids[i] >> 16), a = int(ids[i] & 0xffff);
    I.init[size_t(x) * I.W + (a >> 6)] &= ~(1ull << (a & 63));
  }
}

inline Instance empty_instance(int n, int d) {
  Instance I;
  I.n = n;
  I.dom.assign(n, d);
  I.W = words_for(d);
  init_full_domains(I);
  return I;
}

// Model-B random binary network: n variables with uniform domain size d,
// e constraints on distinct pairs, tightness uniform in [p_lo, p_hi], then a
// fraction `remove` of all (variable, value) pairs cleared.
inline Instance random_binary(int n, int d, int64_t e, double p_lo, double p_hi, double remove,
                              uint64_t seed, bool make_rows = true) {
  Instance I = empty_instance(n, d);
  Stream S(seed);
  add_random_binary(I, e, p_lo, p_hi, S, seed, make_rows);
  remove_random_values(I, remove, S);
  return I;
}

// Binary network plus ternary positive tables (the mixed-arity GAC workload).
inline Instance random_mixed(int n, int d, int64_t e, double p_lo, double p_hi, int k3, int ntup,
                             double remove, uint64_t seed) {
  Instance I = empty_instance(n, d);
  Stream S(seed);
  add_random_binary(I, e, p_lo, p_hi, S, seed);
  add_random_tables(I, k3, 3, ntup, S);
  remove_random_values(I, remove, S);
  return I;
}

// Per-instance seed of instance `index` in a batch built from `base_seed`.
inline uint64_t batch_seed(uint64_t base_seed, uint64_t index) { return base_seed * 1000003ull + index; }

// Shape of one instance of the uneven multi-instance batch: n uniform in
// [n_lo, n_hi], d uniform over {8,16,32,64,128,256} capped at d_cap, edge
// density uniform in [0.05, 0.3] of all pairs, tightness uniform in [0.2, 0.6].
struct UnevenShape {
  int n;
  int d;
  int64_t e;
  double p;
};

inline UnevenShape uneven_shape(uint64_t seed, int n_lo = 20, int n_hi = 400, int d_cap = 256) {
  Stream S(seed ^ 0xA11CEull);
  static const int kD[6] = {8, 16, 32, 64, 128, 256};
  UnevenShape s;
  s.n = n_lo + int(S.below(uint64_t(n_hi - n_lo + 1)));
  int choices = 0;
  while (choices < 6 && kD[choices] <= d_cap) ++choices;
  s.d = kD[S.below(uint64_t(choices < 1 ? 1 : choices))];
  const double density = 0.05 + 0.25 * S.unit();
  const int64_t pairs = int64_t(s.n) * (s.n - 1) / 2;
  s.e = std::max<int64_t>(1, std::min<int64_t>(pairs, int64_t(std::floor(density * double(pairs) + 0.5))));
  s.p = 0.2 + 0.4 * S.unit();
  return s;
}

inline Instance uneven_instance(uint64_t seed, int n_lo = 20, int n_hi = 400, int d_cap = 256,
                                bool make_rows = true) {
  const UnevenShape s = uneven_shape(seed, n_lo, n_hi, d_cap);
  return random_binary(s.n, s.d, s.e, s.p, s.p, 0.0, seed, make_rows);
}

// FNV-1a over every array of the instance: a fingerprint stored beside golden
// results so that a change of generator is caught instead of silently
// comparing different networks.
inline uint64_t fingerprint(const Instance& I) {
  uint64_t h = 1469598103934665603ull;
  auto eat = [&](const void* p, size_t nbytes) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < nbytes; ++i) h = (h ^ b[i]) * 1099511628211ull;
  };
  eat(&I.n, sizeof(int));
  eat(&I.W, sizeof(int));
  eat(I.dom.data(), I.dom.size() * sizeof(int));
  eat(I.init.data(), I.init.size() * 8);
  eat(I.bx.data(), I.bx.size() * sizeof(int));
  eat(I.by.data(), I.by.size() * sizeof(int));
  eat(I.brows.data(), I.brows.size() * 8);
  eat(I.tarity.data(), I.tarity.size() * sizeof(int));
  eat(I.tscope.data(), I.tscope.size() * sizeof(int));
  eat(I.tntup.data(), I.tntup.size() * sizeof(int));
  eat(I.ttup.data(), I.ttup.size() * sizeof(int));
  return h;
}

}  // namespace cpgen
