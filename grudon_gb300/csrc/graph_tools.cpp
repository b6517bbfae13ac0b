// Host graph tools: seeded RMAT / Erdos-Renyi / grid generators, CSR build
// (dedupe, self-loop removal, symmetrisation), Galois .gr and MatrixMarket
// I/O, and the mirror-partition file format.
//
// The reference reads graphs with galois::graphs::readGraph (.gr binary CSR,
// src/DistributedGraph.cpp:49,571) and partition files with one integer per
// line (include/partitioning_engine/Partitioner.hpp:89-105).  Generation is
// counter-based (SplitMix64 keyed by edge index), so the produced CSR is
// identical for any thread count and on any host architecture.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/grudon_gpu.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Uniform double in [0,1) from 53 high bits.
inline double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

// Unbiased-enough bounded draw (Lemire multiply-high).
inline uint32_t bounded(uint64_t r, uint32_t n) {
  return (uint32_t)(((unsigned __int128)r * n) >> 64);
}

int hw_threads(int threads) {
  if (threads > 0) return threads;
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

void parallel_for(int nthreads, uint64_t n, const std::function<void(uint64_t, uint64_t)>& fn) {
  if (nthreads <= 1 || n < 4096) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> ts;
  uint64_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    uint64_t b = (uint64_t)t * chunk, e = std::min<uint64_t>(n, b + chunk);
    if (b >= e) break;
    ts.emplace_back([&, b, e] { fn(b, e); });
  }
  for (auto& t : ts) t.join();
}

// Dynamic scheduling over [0,n) in chunks (rows of very uneven cost).
void parallel_dynamic(int nthreads, uint64_t n, uint64_t grain,
                      const std::function<void(uint64_t, uint64_t)>& fn) {
  if (nthreads <= 1 || n <= grain) {
    fn(0, n);
    return;
  }
  std::atomic<uint64_t> next{0};
  std::vector<std::thread> ts;
  for (int t = 0; t < nthreads; ++t)
    ts.emplace_back([&] {
      for (;;) {
        uint64_t b = next.fetch_add(grain);
        if (b >= n) break;
        fn(b, std::min(n, b + grain));
      }
    });
  for (auto& t : ts) t.join();
}

// Edge source: fills (src,dst) for draw index i; returns false to drop it.
using EdgeFn = std::function<bool(uint64_t, uint32_t&, uint32_t&)>;

grd_host_graph* alloc_graph(uint32_t V, uint64_t E, bool weighted) {
  grd_host_graph* g = (grd_host_graph*)std::calloc(1, sizeof(grd_host_graph));
  if (!g) return nullptr;
  g->num_vertices = V;
  g->num_edges = E;
  g->row_offsets = (uint64_t*)std::malloc(sizeof(uint64_t) * ((size_t)V + 1));
  g->col_indices = (uint32_t*)std::malloc(sizeof(uint32_t) * (E ? E : 1));
  g->weights = weighted ? (uint32_t*)std::malloc(sizeof(uint32_t) * (E ? E : 1)) : nullptr;
  if (!g->row_offsets || !g->col_indices || (weighted && !g->weights)) {
    grd_graph_free(g);
    return nullptr;
  }
  return g;
}

void assign_weights(grd_host_graph* g, uint64_t seed, int nthreads) {
  if (!g->weights) return;
  const uint64_t wseed = splitmix64(seed ^ 0x77656967687473ull);  // "weights"
  uint32_t* w = g->weights;
  parallel_for(nthreads, g->num_edges, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) w[i] = 1u + (uint32_t)(splitmix64(wseed ^ (i * 0xD1B54A32D192ED03ull)) % 255u);
  });
}

// Two-pass counting-sort CSR build from a regenerable edge stream, then
// per-row sort + unique.  The result depends only on the edge multiset.
int build_csr(uint32_t V, uint64_t draws, bool symmetrize, bool weighted, uint64_t seed,
              int nthreads, const EdgeFn& edge, grd_host_graph** out) {
  std::vector<std::atomic<uint32_t>> deg(V);
  for (auto& d : deg) d.store(0, std::memory_order_relaxed);
  parallel_for(nthreads, draws, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) {
      uint32_t s, d;
      if (!edge(i, s, d) || s == d) continue;
      deg[s].fetch_add(1, std::memory_order_relaxed);
      if (symmetrize) deg[d].fetch_add(1, std::memory_order_relaxed);
    }
  });
  std::vector<uint64_t> off((size_t)V + 1, 0);
  for (uint32_t v = 0; v < V; ++v) off[v + 1] = off[v] + deg[v].load(std::memory_order_relaxed);
  const uint64_t raw = off[V];
  std::vector<uint32_t> tmp;
  try {
    tmp.resize(raw ? raw : 1);
  } catch (const std::bad_alloc&) {
    return GRD_E_OOM;
  }
  std::vector<std::atomic<uint64_t>> cur(V);
  for (uint32_t v = 0; v < V; ++v) cur[v].store(off[v], std::memory_order_relaxed);
  parallel_for(nthreads, draws, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) {
      uint32_t s, d;
      if (!edge(i, s, d) || s == d) continue;
      tmp[cur[s].fetch_add(1, std::memory_order_relaxed)] = d;
      if (symmetrize) tmp[cur[d].fetch_add(1, std::memory_order_relaxed)] = s;
    }
  });
  std::vector<uint32_t> ndeg(V);
  parallel_dynamic(nthreads, V, 4096, [&](uint64_t b, uint64_t e) {
    for (uint64_t v = b; v < e; ++v) {
      uint32_t* p = tmp.data() + off[v];
      uint32_t* q = tmp.data() + off[v + 1];
      std::sort(p, q);
      ndeg[v] = (uint32_t)(std::unique(p, q) - p);
    }
  });
  uint64_t E = 0;
  for (uint32_t v = 0; v < V; ++v) E += ndeg[v];
  grd_host_graph* g = alloc_graph(V, E, weighted);
  if (!g) return GRD_E_OOM;
  g->seed = seed;
  g->row_offsets[0] = 0;
  for (uint32_t v = 0; v < V; ++v) g->row_offsets[v + 1] = g->row_offsets[v] + ndeg[v];
  parallel_for(nthreads, V, [&](uint64_t b, uint64_t e) {
    for (uint64_t v = b; v < e; ++v)
      std::memcpy(g->col_indices + g->row_offsets[v], tmp.data() + off[v], sizeof(uint32_t) * ndeg[v]);
  });
  assign_weights(g, seed, nthreads);
  *out = g;
  return GRD_OK;
}

}  // namespace

extern "C" {

uint64_t grd_rmat_seed(uint32_t scale, uint32_t edge_factor) {
  return 0x6772756Eull ^ ((uint64_t)scale << 8) ^ (uint64_t)edge_factor;
}

int grd_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                 int symmetrize, int weighted, int threads, grd_host_graph** out) {
  if (!out || scale == 0 || scale > 31 || edge_factor == 0) return GRD_E_INVALID;
  if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0)) return GRD_E_INVALID;
  *out = nullptr;
  const uint32_t V = 1u << scale;
  const uint64_t draws = (uint64_t)edge_factor << scale;
  const double ab = a + b, abc = a + b + c;
  const uint64_t key = splitmix64(seed);
  EdgeFn fn = [=](uint64_t i, uint32_t& s, uint32_t& d) {
    uint64_t x = key ^ (i * 0xA24BAED4963EE407ull);
    uint32_t src = 0, dst = 0;
    for (uint32_t l = 0; l < scale; ++l) {
      x = splitmix64(x);
      double r = u01(x);
      uint32_t sb = 0, db = 0;
      if (r < a) {
      } else if (r < ab) {
        db = 1;
      } else if (r < abc) {
        sb = 1;
      } else {
        sb = 1;
        db = 1;
      }
      src = (src << 1) | sb;
      dst = (dst << 1) | db;
    }
    s = src;
    d = dst;
    return true;
  };
  return build_csr(V, draws, symmetrize != 0, weighted != 0, seed, hw_threads(threads), fn, out);
}

int grd_gen_er(uint32_t num_vertices, uint32_t edge_factor, uint64_t seed, int symmetrize, int weighted,
               int threads, grd_host_graph** out) {
  if (!out || num_vertices == 0 || edge_factor == 0) return GRD_E_INVALID;
  *out = nullptr;
  const uint64_t draws = (uint64_t)edge_factor * num_vertices;
  const uint64_t key = splitmix64(seed ^ 0x45524552ull);
  const uint32_t n = num_vertices;
  EdgeFn fn = [=](uint64_t i, uint32_t& s, uint32_t& d) {
    uint64_t x = splitmix64(key ^ (i * 0xA24BAED4963EE407ull));
    s = bounded(x, n);
    d = bounded(splitmix64(x), n);
    return true;
  };
  return build_csr(n, draws, symmetrize != 0, weighted != 0, seed, hw_threads(threads), fn, out);
}

int grd_gen_grid(uint32_t k, uint64_t seed, int weighted, int threads, grd_host_graph** out) {
  if (!out || k == 0 || (uint64_t)k * k > 0xFFFFFFFFull) return GRD_E_INVALID;
  *out = nullptr;
  const uint32_t V = k * k;
  // Rows are produced directly in ascending-neighbour order.
  std::vector<uint32_t> ndeg(V);
  for (uint32_t v = 0; v < V; ++v) {
    uint32_t r = v / k, c = v % k;
    ndeg[v] = (r > 0) + (c > 0) + (c + 1 < k) + (r + 1 < k);
  }
  uint64_t E = 0;
  for (uint32_t v = 0; v < V; ++v) E += ndeg[v];
  grd_host_graph* g = alloc_graph(V, E, weighted != 0);
  if (!g) return GRD_E_OOM;
  g->seed = seed;
  g->row_offsets[0] = 0;
  for (uint32_t v = 0; v < V; ++v) g->row_offsets[v + 1] = g->row_offsets[v] + ndeg[v];
  int nt = hw_threads(threads);
  parallel_for(nt, V, [&](uint64_t b, uint64_t e) {
    for (uint64_t v = b; v < e; ++v) {
      uint32_t r = (uint32_t)(v / k), c = (uint32_t)(v % k);
      uint32_t* p = g->col_indices + g->row_offsets[v];
      if (r > 0) *p++ = (uint32_t)v - k;
      if (c > 0) *p++ = (uint32_t)v - 1;
      if (c + 1 < k) *p++ = (uint32_t)v + 1;
      if (r + 1 < k) *p++ = (uint32_t)v + k;
    }
  });
  assign_weights(g, seed, nt);
  *out = g;
  return GRD_OK;
}

int grd_graph_from_csr(const grd_csr* csr, grd_host_graph** out) {
  if (!csr || !out || !csr->row_offsets || (csr->num_edges && !csr->col_indices)) return GRD_E_INVALID;
  *out = nullptr;
  const uint32_t V = csr->num_vertices;
  if (csr->row_offsets[0] != 0 || csr->row_offsets[V] != csr->num_edges) return GRD_E_INVALID;
  for (uint32_t v = 0; v < V; ++v)
    if (csr->row_offsets[v + 1] < csr->row_offsets[v]) return GRD_E_INVALID;
  for (uint64_t i = 0; i < csr->num_edges; ++i)
    if (csr->col_indices[i] >= V) return GRD_E_INVALID;
  grd_host_graph* g = alloc_graph(V, csr->num_edges, csr->weights != nullptr);
  if (!g) return GRD_E_OOM;
  std::memcpy(g->row_offsets, csr->row_offsets, sizeof(uint64_t) * ((size_t)V + 1));
  if (csr->num_edges) std::memcpy(g->col_indices, csr->col_indices, sizeof(uint32_t) * csr->num_edges);
  if (csr->weights && csr->num_edges) std::memcpy(g->weights, csr->weights, sizeof(uint32_t) * csr->num_edges);
  *out = g;
  return GRD_OK;
}

void grd_graph_free(grd_host_graph* g) {
  if (!g) return;
  std::free(g->row_offsets);
  std::free(g->col_indices);
  std::free(g->weights);
  std::free(g);
}

// ---- Galois .gr version 1: u64 version, u64 sizeof(edge data), u64 V,
// u64 E, u64 row_end[V], u32 dst[E], u32 pad if E odd, edge data[E]. ------
int grd_write_gr(const grd_host_graph* g, const char* path) {
  if (!g || !path) return GRD_E_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) return GRD_E_IO;
  uint64_t hdr[4] = {1, g->weights ? 4u : 0u, g->num_vertices, g->num_edges};
  bool ok = std::fwrite(hdr, sizeof hdr, 1, f) == 1;
  ok = ok && (g->num_vertices == 0 ||
              std::fwrite(g->row_offsets + 1, sizeof(uint64_t), g->num_vertices, f) == g->num_vertices);
  ok = ok && (g->num_edges == 0 || std::fwrite(g->col_indices, sizeof(uint32_t), g->num_edges, f) == g->num_edges);
  if (ok && g->weights) {
    uint32_t pad = 0;
    if (g->num_edges & 1) ok = std::fwrite(&pad, 4, 1, f) == 1;
    ok = ok && (g->num_edges == 0 || std::fwrite(g->weights, sizeof(uint32_t), g->num_edges, f) == g->num_edges);
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GRD_OK : GRD_E_IO;
}

int grd_read_gr(const char* path, grd_host_graph** out) {
  if (!path || !out) return GRD_E_INVALID;
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return GRD_E_IO;
  uint64_t hdr[4];
  if (std::fread(hdr, sizeof hdr, 1, f) != 1 || hdr[0] != 1 || (hdr[1] != 0 && hdr[1] != 4) ||
      hdr[2] > 0xFFFFFFFFull) {
    std::fclose(f);
    return GRD_E_IO;
  }
  const uint32_t V = (uint32_t)hdr[2];
  const uint64_t E = hdr[3];
  grd_host_graph* g = alloc_graph(V, E, hdr[1] == 4);
  if (!g) {
    std::fclose(f);
    return GRD_E_OOM;
  }
  bool ok = true;
  g->row_offsets[0] = 0;
  if (V) ok = std::fread(g->row_offsets + 1, sizeof(uint64_t), V, f) == V;
  if (ok && E) ok = std::fread(g->col_indices, sizeof(uint32_t), E, f) == E;
  if (ok && g->weights) {
    uint32_t pad;
    if (E & 1) ok = std::fread(&pad, 4, 1, f) == 1;
    if (ok && E) ok = std::fread(g->weights, sizeof(uint32_t), E, f) == E;
  }
  std::fclose(f);
  for (uint32_t v = 0; ok && v < V; ++v) ok = g->row_offsets[v + 1] >= g->row_offsets[v];
  ok = ok && g->row_offsets[V] == E;
  for (uint64_t i = 0; ok && i < E; ++i) ok = g->col_indices[i] < V;
  if (!ok) {
    grd_graph_free(g);
    return GRD_E_IO;
  }
  *out = g;
  return GRD_OK;
}

// MatrixMarket coordinate, 1-based; the third column (if any) is the weight.
int grd_write_mtx(const grd_host_graph* g, const char* path) {
  if (!g || !path) return GRD_E_INVALID;
  FILE* f = std::fopen(path, "w");
  if (!f) return GRD_E_IO;
  bool ok = std::fprintf(f, "%%%%MatrixMarket matrix coordinate %s general\n%u %u %llu\n",
                         g->weights ? "integer" : "pattern", g->num_vertices, g->num_vertices,
                         (unsigned long long)g->num_edges) > 0;
  for (uint32_t v = 0; ok && v < g->num_vertices; ++v)
    for (uint64_t i = g->row_offsets[v]; ok && i < g->row_offsets[v + 1]; ++i)
      ok = (g->weights ? std::fprintf(f, "%u %u %u\n", v + 1, g->col_indices[i] + 1, g->weights[i])
                       : std::fprintf(f, "%u %u\n", v + 1, g->col_indices[i] + 1)) > 0;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GRD_OK : GRD_E_IO;
}

int grd_read_mtx(const char* path, grd_host_graph** out) {
  if (!path || !out) return GRD_E_INVALID;
  *out = nullptr;
  FILE* f = std::fopen(path, "r");
  if (!f) return GRD_E_IO;
  char line[512];
  bool weighted = false, have_banner = false;
  unsigned long long nr = 0, nc = 0, nnz = 0;
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == '%') {
      if (!have_banner && std::strstr(line, "MatrixMarket")) {
        have_banner = true;
        weighted = !std::strstr(line, "pattern");
      }
      continue;
    }
    if (std::sscanf(line, "%llu %llu %llu", &nr, &nc, &nnz) == 3) break;
    std::fclose(f);
    return GRD_E_IO;
  }
  if (nr == 0 || nr != nc || nr > 0xFFFFFFFFull) {
    std::fclose(f);
    return GRD_E_IO;
  }
  std::vector<uint64_t> key;
  std::vector<uint32_t> wv;
  key.reserve(nnz);
  for (unsigned long long k = 0; k < nnz; ++k) {
    unsigned long long s, d;
    double w = 1;
    if (!std::fgets(line, sizeof line, f)) break;
    int n = std::sscanf(line, "%llu %llu %lf", &s, &d, &w);
    if (n < 2 || s == 0 || d == 0 || s > nr || d > nr) {
      std::fclose(f);
      return GRD_E_IO;
    }
    key.push_back(((s - 1) << 32) | (d - 1));
    wv.push_back((uint32_t)w);
  }
  std::fclose(f);
  if (key.size() != nnz) return GRD_E_IO;
  std::vector<uint64_t> order(nnz);
  for (uint64_t i = 0; i < nnz; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint64_t x, uint64_t y) { return key[x] < key[y]; });
  const uint32_t V = (uint32_t)nr;
  std::vector<uint64_t> keep;
  for (uint64_t i = 0; i < nnz; ++i) {
    uint64_t k = key[order[i]];
    if ((k >> 32) == (k & 0xFFFFFFFFull)) continue;
    if (!keep.empty() && key[keep.back()] == k) continue;
    keep.push_back(order[i]);
  }
  grd_host_graph* g = alloc_graph(V, keep.size(), weighted);
  if (!g) return GRD_E_OOM;
  std::fill(g->row_offsets, g->row_offsets + V + 1, 0);
  for (uint64_t i = 0; i < keep.size(); ++i) {
    uint64_t k = key[keep[i]];
    g->row_offsets[(k >> 32) + 1]++;
    g->col_indices[i] = (uint32_t)(k & 0xFFFFFFFFull);
    if (weighted) g->weights[i] = wv[keep[i]];
  }
  for (uint32_t v = 0; v < V; ++v) g->row_offsets[v + 1] += g->row_offsets[v];
  *out = g;
  return GRD_OK;
}

int grd_partition_edge_balanced(const grd_host_graph* g, uint32_t num_memory, uint32_t* part) {
  if (!g || !part || num_memory == 0) return GRD_E_INVALID;
  const uint32_t V = g->num_vertices;
  const uint64_t E = g->num_edges;
  // Contiguous gid ranges; boundary p is the first vertex whose cumulative
  // (edges + vertices) weight reaches p/M of the total, so both edge-heavy
  // hubs and long low-degree tails are balanced.
  const double total = (double)E + (double)V;
  uint32_t p = 0;
  for (uint32_t v = 0; v < V; ++v) {
    double before = (double)g->row_offsets[v] + (double)v;
    while (p + 1 < num_memory && before >= total * (double)(p + 1) / num_memory) ++p;
    part[v] = p;
  }
  return GRD_OK;
}

int grd_write_partition_file(const uint32_t* part, uint32_t n, const char* path) {
  if (!part || !path) return GRD_E_INVALID;
  FILE* f = std::fopen(path, "w");
  if (!f) return GRD_E_IO;
  bool ok = true;
  for (uint32_t i = 0; ok && i < n; ++i) ok = std::fprintf(f, "%u\n", part[i]) > 0;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GRD_OK : GRD_E_IO;
}

// Unlike the reference (which logs and leaves the partition vector
// zero-filled on a missing file, Partitioner.hpp:92-96), a missing, short or
// out-of-range file is an error.
int grd_read_partition_file(const char* path, uint32_t n, uint32_t num_memory, uint32_t* part) {
  if (!path || !part || num_memory == 0) return GRD_E_INVALID;
  FILE* f = std::fopen(path, "r");
  if (!f) return GRD_E_IO;
  for (uint32_t i = 0; i < n; ++i) {
    long long x;
    if (std::fscanf(f, "%lld", &x) != 1 || x < 0 || x >= (long long)num_memory) {
      std::fclose(f);
      return GRD_E_IO;
    }
    part[i] = (uint32_t)x;
  }
  std::fclose(f);
  return GRD_OK;
}

}  // extern "C"
