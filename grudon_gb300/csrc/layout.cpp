// Partition layout build (host).  See layout.hpp for the slot order contract.
#include "layout.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <functional>
#include <thread>

namespace grd {
namespace {

void par_for(int nt, uint64_t n, const std::function<void(uint64_t, uint64_t)>& fn) {
  if (nt <= 1 || n < 65536) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> ts;
  uint64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    uint64_t b = (uint64_t)t * chunk, e = std::min<uint64_t>(n, b + chunk);
    if (b >= e) break;
    ts.emplace_back([&, b, e] { fn(b, e); });
  }
  for (auto& t : ts) t.join();
}

inline uint32_t popc64(uint64_t x) { return (uint32_t)__builtin_popcountll(x); }

}  // namespace

std::string build_layout(uint32_t V, uint64_t E, const uint64_t* ro, const uint32_t* col,
                         const uint32_t* weights, const uint32_t* mirror_part, uint32_t M, Layout& L,
                         int threads) {
  int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
  if (M == 0 || M > 1024) return "num_memory must be in [1, 1024]";
  if (V == 0) return "graph has no vertices";
  if (!ro) return "row_offsets is NULL";
  if (E && !col) return "col_indices is NULL";
  if (E >= 0xFFFFFFF0ull) return "more than 2^32-16 edges: 32-bit edge offsets would overflow";
  if (ro[0] != 0 || ro[V] != E) return "row_offsets[0] must be 0 and row_offsets[V] must equal num_edges";
  for (uint32_t v = 0; v < V; ++v)
    if (ro[v + 1] < ro[v]) return "row_offsets is not monotone";
  std::atomic<bool> bad_col{false};
  par_for(nt, E, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i)
      if (col[i] >= V) bad_col.store(true, std::memory_order_relaxed);
  });
  if (bad_col.load()) return "col_indices holds an id >= num_vertices";

  L = Layout();
  L.V = V;
  L.E = E;
  L.M = M;
  L.weighted = weights != nullptr;
  L.mirror.resize(V);
  for (uint32_t v = 0; v < V; ++v) {
    uint32_t p = mirror_part ? mirror_part[v] : v % M;  // NaivePartitioner: gid % M
    if (p >= M) return "mirror partition id >= num_memory";
    L.mirror[v] = p;
  }
  L.outdeg.resize(V);
  for (uint32_t v = 0; v < V; ++v) L.outdeg[v] = (uint32_t)(ro[v + 1] - ro[v]);

  // Owned vertices per partition, ascending gid; own_slot = rank in partition.
  L.n_owned.assign(M, 0);
  L.n_proxy.assign(M, 0);
  L.part_edges.assign(M, 0);
  std::vector<uint32_t> own_slot(V);
  for (uint32_t v = 0; v < V; ++v) {
    own_slot[v] = L.n_owned[L.mirror[v]]++;
    L.part_edges[L.mirror[v]] += L.outdeg[v];
  }

  // Proxy discovery: destinations of p's edges mastered in another mirror
  // partition (cross_node_mirrors, src/DistributedGraph.cpp:345-349).
  const uint64_t W = ((uint64_t)V + 63) / 64;
  std::vector<std::vector<uint64_t>> bm(M, std::vector<uint64_t>(W, 0));
  par_for(nt, V, [&](uint64_t b, uint64_t e) {
    for (uint64_t u = b; u < e; ++u) {
      const uint32_t p = L.mirror[u];
      uint64_t* bp = bm[p].data();
      for (uint64_t i = ro[u]; i < ro[u + 1]; ++i) {
        const uint32_t d = col[i];
        if (L.mirror[d] != p) {
          const uint64_t bit = 1ull << (d & 63);
          if (!(__atomic_load_n(&bp[d >> 6], __ATOMIC_RELAXED) & bit))
            __atomic_fetch_or(&bp[d >> 6], bit, __ATOMIC_RELAXED);
        }
      }
    }
  });
  std::vector<std::vector<uint32_t>> pre(M, std::vector<uint32_t>(W + 1, 0));
  for (uint32_t p = 0; p < M; ++p) {
    for (uint64_t w = 0; w < W; ++w) pre[p][w + 1] = pre[p][w] + popc64(bm[p][w]);
    L.n_proxy[p] = pre[p][W];
  }

  // Slot bases, tile aligned.
  L.slot_base.assign(M, 0);
  uint64_t S = 0;
  for (uint32_t p = 0; p < M; ++p) {
    L.slot_base[p] = (uint32_t)S;
    uint64_t T = (uint64_t)L.n_owned[p] + L.n_proxy[p];
    uint64_t padded = std::max<uint64_t>(TILE_SLOTS, (T + TILE_SLOTS - 1) / TILE_SLOTS * TILE_SLOTS);
    S += padded;
    if (S >= 0xFFFFFFF0ull) return "slot space exceeds 2^32";
  }
  L.S = S;
  L.slot_gid.assign(S, INVALID);
  {
    std::vector<uint32_t> fill(M, 0);
    for (uint32_t v = 0; v < V; ++v) {
      uint32_t p = L.mirror[v];
      L.slot_gid[L.slot_base[p] + fill[p]++] = v;
    }
    for (uint32_t p = 0; p < M; ++p) {
      uint32_t k = L.slot_base[p] + L.n_owned[p];
      for (uint64_t w = 0; w < W; ++w) {
        uint64_t x = bm[p][w];
        while (x) {
          int b = __builtin_ctzll(x);
          x &= x - 1;
          L.slot_gid[k++] = (uint32_t)(w * 64 + b);
        }
      }
    }
  }

  // Out-edge CSR over global slots.
  L.row_off.assign(S + 1, 0);
  for (uint64_t s = 0; s < S; ++s) {
    uint32_t g = L.slot_gid[s];
    uint32_t deg = 0;
    if (g != INVALID) {
      uint32_t p = L.mirror[g];
      // owned iff this slot is g's owned slot (proxies of g live in other partitions)
      if (s == (uint64_t)L.slot_base[p] + own_slot[g]) deg = L.outdeg[g];
    }
    L.row_off[s + 1] = L.row_off[s] + deg;
  }
  L.col.resize(E ? E : 1);
  if (L.weighted) L.wgt.resize(E ? E : 1);
  par_for(nt, V, [&](uint64_t b, uint64_t e) {
    for (uint64_t u = b; u < e; ++u) {
      const uint32_t p = L.mirror[u];
      const uint64_t s = (uint64_t)L.slot_base[p] + own_slot[u];
      uint64_t o = L.row_off[s];
      for (uint64_t i = ro[u]; i < ro[u + 1]; ++i, ++o) {
        const uint32_t d = col[i];
        uint32_t ds;
        if (L.mirror[d] == p) {
          ds = L.slot_base[p] + own_slot[d];
        } else {
          const uint64_t w = d >> 6;
          ds = L.slot_base[p] + L.n_owned[p] + pre[p][w] + popc64(bm[p][w] & ((1ull << (d & 63)) - 1));
        }
        L.col[o] = ds;
        if (L.weighted) L.wgt[o] = weights[i];
      }
    }
  });

  // Static hub work items: rows with more than HUB_DEGREE edges, cut at
  // absolute edge indices that are multiples of HUB_CHUNK (so every chunk
  // interior is 16-byte aligned for vector loads).
  for (uint64_t s = 0; s < S; ++s) {
    uint32_t e0 = L.row_off[s], e1 = L.row_off[s + 1];
    if (e1 - e0 <= HUB_DEGREE) continue;
    uint32_t a = e0;
    while (a < e1) {
      uint32_t nxt = (a / HUB_CHUNK + 1) * HUB_CHUNK;
      uint32_t b = std::min(e1, nxt);
      L.hubs.push_back(HubChunk{(uint32_t)s, a, b});
      a = b;
    }
  }

  // Tiles.
  const uint64_t nt_tiles = S / TILE_SLOTS;
  L.tile_part.resize(nt_tiles);
  L.tile_first.resize(nt_tiles);
  for (uint32_t p = 0; p < M; ++p) {
    uint64_t t0 = L.slot_base[p] / TILE_SLOTS;
    uint64_t t1 = (p + 1 < M) ? L.slot_base[p + 1] / TILE_SLOTS : nt_tiles;
    for (uint64_t t = t0; t < t1; ++t) {
      L.tile_part[t] = p;
      L.tile_first[t] = (uint32_t)t0;
    }
  }
  return std::string();
}

// In-edge view, built on demand (pull traversal, PR_PULL).  Sources are
// visited in ascending slot order, so every in-list is sorted by source.
void build_in_edges(Layout& L) {
  if (!L.in_off.empty()) return;
  const uint64_t S = L.S;
  L.in_off.assign(S + 1, 0);
  for (uint64_t i = 0; i < L.E; ++i) L.in_off[L.col[i] + 1]++;
  for (uint64_t s = 0; s < S; ++s) L.in_off[s + 1] += L.in_off[s];
  L.in_src.resize(L.E ? L.E : 1);
  if (L.weighted) L.in_wgt.resize(L.E ? L.E : 1);
  std::vector<uint32_t> cur(L.in_off.begin(), L.in_off.end() - 1);
  for (uint64_t s = 0; s < S; ++s) {
    for (uint32_t i = L.row_off[s]; i < L.row_off[s + 1]; ++i) {
      uint32_t d = L.col[i];
      uint32_t o = cur[d]++;
      L.in_src[o] = (uint32_t)s;
      if (L.weighted) L.in_wgt[o] = L.wgt[i];
    }
  }
  L.in_hubs.clear();
  L.in_meds.clear();
  for (uint64_t s = 0; s < S; ++s) {
    const uint32_t d = L.in_off[s + 1] - L.in_off[s];
    if (d > PULL_HUB)
      L.in_hubs.push_back(HubChunk{(uint32_t)s, L.in_off[s], L.in_off[s + 1]});
    else if (d > PULL_MED)
      L.in_meds.push_back(HubChunk{(uint32_t)s, L.in_off[s], L.in_off[s + 1]});
  }
}

}  // namespace grd
