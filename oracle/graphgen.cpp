// ORACLE — test infrastructure only.  Independent restatement of the seeded
// synthetic-graph generators the benchmark workloads are defined on, so that
// the CPU reference arm and the checkers can build the benchmark graphs
// without loading the product library.
//
// Algorithm (Graph500-style recursive-quadrant RMAT with a counter-based
// RNG, as the workload definition states): draw i of edge_factor * 2^scale
// draws starts from x = splitmix64(seed) ^ (i * 0xA24BAED4963EE407) and, for
// each of the `scale` levels, advances x = splitmix64(x) and picks the
// quadrant from u = (x >> 11) * 2^-53 against a, a+b, a+b+c (source bit,
// destination bit).  Self loops are dropped, symmetrisation adds the reverse
// of every drawn edge, duplicates are removed, and each row lists its
// destinations in ascending order.  Edge weights are 1 + (splitmix64(wseed ^
// (k * 0xD1B54A32D192ED03)) mod 255) for the k-th edge of the final CSR, with
// wseed = splitmix64(seed ^ 0x77656967687473).  The mirror partition is the
// edge-balanced contiguous split: vertex v goes to the first partition p for
// which v's cumulative (edges + vertices) weight stays below (p+1)/M of the
// total.
//
// This file builds the CSR differently from the product generator: every
// draw becomes a (source << scale | destination) key, the keys are radix-sorted
// (LSD, 16-bit digits, all threads) and deduplicated, and the rows follow
// from the sorted keys.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int nthreads_of(int t) {
  if (t > 0) return t;
  const unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

template <class F>
void run_threads(int n, F&& f) {
  std::vector<std::thread> ts;
  for (int t = 1; t < n; ++t) ts.emplace_back([&f, t] { f(t); });
  f(0);
  for (auto& th : ts) th.join();
}

struct OrcGraph {
  uint32_t V = 0;
  std::vector<uint64_t> ro;
  std::vector<uint32_t> col, w;
};

// Stable LSD radix sort of 64-bit keys over their low `bits` bits.
void radix_sort(std::vector<uint64_t>& keys, int bits, int nt) {
  const size_t n = keys.size();
  std::vector<uint64_t> tmp(n);
  constexpr int D = 16;
  constexpr size_t B = (size_t)1 << D;
  std::vector<std::vector<size_t>> hist(nt, std::vector<size_t>(B));
  for (int shift = 0; shift < bits; shift += D) {
    const uint64_t* in = keys.data();
    uint64_t* out = tmp.data();
    run_threads(nt, [&](int t) {
      std::fill(hist[t].begin(), hist[t].end(), 0);
      const size_t b = n * t / nt, e = n * (t + 1) / nt;
      for (size_t i = b; i < e; ++i) ++hist[t][(in[i] >> shift) & (B - 1)];
    });
    // offsets: digit-major, then thread order (stability)
    size_t run = 0;
    for (size_t d = 0; d < B; ++d)
      for (int t = 0; t < nt; ++t) {
        const size_t c = hist[t][d];
        hist[t][d] = run;
        run += c;
      }
    run_threads(nt, [&](int t) {
      const size_t b = n * t / nt, e = n * (t + 1) / nt;
      std::vector<size_t>& h = hist[t];
      for (size_t i = b; i < e; ++i) out[h[(in[i] >> shift) & (B - 1)]++] = in[i];
    });
    keys.swap(tmp);
  }
}

}  // namespace

extern "C" {

uint64_t orc_rmat_seed(uint32_t scale, uint32_t edge_factor) {
  return 0x6772756Eull ^ ((uint64_t)scale << 8) ^ (uint64_t)edge_factor;
}

void* orc_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                   int symmetrize, int weighted, int threads) {
  if (scale == 0 || scale > 31 || edge_factor == 0) return nullptr;
  const int nt = nthreads_of(threads);
  const uint32_t V = 1u << scale;
  const uint64_t draws = (uint64_t)edge_factor << scale;
  const double ab = a + b, abc = a + b + c;
  const uint64_t key0 = mix64(seed);
  const uint64_t per = symmetrize ? 2 : 1;
  std::vector<uint64_t> keys(draws * per);
  std::vector<size_t> kept(nt);
  run_threads(nt, [&](int t) {
    const uint64_t lo = draws * t / nt, hi = draws * (t + 1) / nt;
    uint64_t* out = keys.data() + lo * per;
    size_t k = 0;
    for (uint64_t i = lo; i < hi; ++i) {
      uint64_t x = key0 ^ (i * 0xA24BAED4963EE407ull);
      uint32_t s = 0, d = 0;
      for (uint32_t l = 0; l < scale; ++l) {
        x = mix64(x);
        const double u = (double)(x >> 11) * (1.0 / 9007199254740992.0);
        const uint32_t sb = u >= ab ? 1u : 0u;
        const uint32_t db = (u >= a && u < ab) || u >= abc ? 1u : 0u;
        s = (s << 1) | sb;
        d = (d << 1) | db;
      }
      if (s == d) continue;
      out[k++] = ((uint64_t)s << scale) | d;
      if (symmetrize) out[k++] = ((uint64_t)d << scale) | s;
    }
    kept[t] = k;
  });
  // close the gaps left by dropped self loops
  size_t n = kept[0];
  for (int t = 1; t < nt; ++t) {
    const uint64_t lo = draws * t / nt;
    std::memmove(keys.data() + n, keys.data() + lo * per, sizeof(uint64_t) * kept[t]);
    n += kept[t];
  }
  keys.resize(n);
  radix_sort(keys, 2 * (int)scale, nt);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  OrcGraph* g = new OrcGraph;
  g->V = V;
  g->ro.assign((size_t)V + 1, 0);
  g->col.resize(keys.size());
  const uint64_t dmask = ((uint64_t)1 << scale) - 1;
  for (size_t i = 0; i < keys.size(); ++i) {
    ++g->ro[(keys[i] >> scale) + 1];
    g->col[i] = (uint32_t)(keys[i] & dmask);
  }
  for (uint32_t v = 0; v < V; ++v) g->ro[v + 1] += g->ro[v];
  if (weighted) {
    const uint64_t wseed = mix64(seed ^ 0x77656967687473ull);
    g->w.resize(g->col.size());
    const size_t m = g->w.size();
    run_threads(nt, [&](int t) {
      const size_t b = m * t / nt, e = m * (t + 1) / nt;
      for (size_t k = b; k < e; ++k) g->w[k] = 1u + (uint32_t)(mix64(wseed ^ (k * 0xD1B54A32D192ED03ull)) % 255u);
    });
  }
  return g;
}

uint32_t orc_graph_num_vertices(const void* h) { return static_cast<const OrcGraph*>(h)->V; }
uint64_t orc_graph_num_edges(const void* h) { return static_cast<const OrcGraph*>(h)->col.size(); }

// Copies the CSR out (w may be null; it is left untouched for an unweighted
// graph).
void orc_graph_copy(const void* h, uint64_t* ro, uint32_t* col, uint32_t* w) {
  const OrcGraph* g = static_cast<const OrcGraph*>(h);
  std::memcpy(ro, g->ro.data(), sizeof(uint64_t) * g->ro.size());
  if (!g->col.empty()) std::memcpy(col, g->col.data(), sizeof(uint32_t) * g->col.size());
  if (w && !g->w.empty()) std::memcpy(w, g->w.data(), sizeof(uint32_t) * g->w.size());
}

void orc_graph_free(void* h) { delete static_cast<OrcGraph*>(h); }

void orc_partition_edge_balanced(uint32_t V, const uint64_t* ro, uint32_t M, uint32_t* part) {
  const double total = (double)ro[V] + (double)V;
  uint32_t p = 0;
  for (uint32_t v = 0; v < V; ++v) {
    const double before = (double)ro[v] + (double)v;
    while (p + 1 < M && before >= total * (double)(p + 1) / M) ++p;
    part[v] = p;
  }
}

}  // extern "C"
