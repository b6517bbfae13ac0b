// Partition layout built on the GPU from the uploaded CSR: the
// DistributedGraph ctor's proxy discovery, translation tables and local
// graphs (src/DistributedGraph.cpp:285-785) as scans, one stable radix sort
// and edge-parallel maps.  The result is identical, array for array, to the
// host build of layout.cpp (same slot order: per partition its owned gids
// ascending, then its proxies ascending; same edge order; same hub and
// in-list order), so every round gives identical results on either.
//
// Phase A (sizes): mirror ids and out-degrees, the source of every edge (a
// max-scan of row-start marks), proxy bitmaps (one bit per partition and gid,
// atomicOr), their popcount prefix, and the owned order of each partition (a
// stable radix sort of (partition, gid)).  The host reads the per-partition
// counts, places the partitions and allocates the resident arrays.
// Phase B (fill): slot -> gid, gid -> owned slot, row offsets (a scan of the
// slot degrees), the relabelled columns and weights, hub work items.
// The in-edge view (pull) is a stable radix sort of (destination slot, edge)
// over the relabelled columns, so every in-list keeps ascending sources.
//
// The proxy bitmaps take M * V / 8 bytes, so the device build serves up to
// 64 memory partitions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/grudon_gpu.h"
#include "ctx.hpp"
#include "devprim.cuh"
#include "kernels.cuh"
#include "layout.hpp"

using namespace grd;
using namespace grd::prim;

namespace {

constexpr uint32_t DEV_MAX_PARTS = 64;
constexpr int LT = 256;  // threads of the element-wise layout kernels

enum LayErr : uint32_t { E_ROWS = 1u, E_COL = 2u, E_MIRROR = 4u };

// Stream-ordered scratch, released when the build returns.
struct Scratch {
  grd_ctx* ctx;
  std::vector<void*> ptrs;
  explicit Scratch(grd_ctx* c) : ctx(c) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, ctx->stream);
  }
  template <class T>
  int get(T** p, size_t count) {
    void* d = nullptr;
    const cudaError_t e = cudaMallocAsync(&d, sizeof(T) * std::max<size_t>(count, 1), ctx->stream);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      ctx->err = std::string("layout scratch allocation: ") + cudaGetErrorString(e);
      return GRD_E_OOM;
    }
    ptrs.push_back(d);
    *p = static_cast<T*>(d);
    return GRD_OK;
  }
};

uint32_t grid_of(const grd_ctx* ctx, uint64_t n) {
  const uint64_t b = (n + LT - 1) / LT;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(b, (uint64_t)ctx->num_sms * 16));
}

template <class Op>
int scan(grd_ctx* ctx, Scratch& tmp, const uint32_t* in, uint32_t* out, uint64_t n, bool inclusive,
         bool total_at_n) {
  if (n == 0) {
    if (total_at_n) CK(cudaMemsetAsync(out, 0, sizeof(uint32_t), ctx->stream));
    return GRD_OK;
  }
  const uint64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
  uint32_t* sums = nullptr;
  TRY(tmp.get(&sums, nt));
  k_scan_reduce<Op><<<(uint32_t)nt, SCAN_THREADS, 0, ctx->stream>>>(in, n, sums);
  k_scan_sums<Op><<<1, SCAN_THREADS, 0, ctx->stream>>>(sums, nt);
  k_scan_down<Op><<<(uint32_t)nt, SCAN_THREADS, 0, ctx->stream>>>(in, out, n, sums, inclusive ? 1 : 0,
                                                                  total_at_n ? 1 : 0);
  CK_LAUNCH();
  return GRD_OK;
}

int bits_for(uint64_t max_key) {
  int b = 0;
  while (b < 32 && (max_key >> b) != 0) ++b;
  return std::max(b, 1);
}

// Stable sort of n pairs by the low `bits` key bits; keys/vals are replaced
// by the buffers that hold the result (scratch or the originals).
int radix_sort(grd_ctx* ctx, Scratch& tmp, uint32_t*& keys, uint32_t*& vals, uint64_t n, int bits) {
  static_assert(RS_THREADS == RS_BINS, "one thread per digit in the scatter's prefix step");
  if (n <= 1) return GRD_OK;
  const uint64_t nt = (n + RS_TILE - 1) / RS_TILE;
  uint32_t *k2 = nullptr, *v2 = nullptr, *hist = nullptr;
  TRY(tmp.get(&k2, n));
  TRY(tmp.get(&v2, n));
  TRY(tmp.get(&hist, (uint64_t)RS_BINS * nt));
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<(uint32_t)nt, RS_THREADS, 0, ctx->stream>>>(keys, n, shift, hist, (uint32_t)nt);
    TRY(scan<OpAdd>(ctx, tmp, hist, hist, (uint64_t)RS_BINS * nt, false, false));
    k_rs_scatter<<<(uint32_t)nt, RS_THREADS, 0, ctx->stream>>>(keys, vals, n, shift, hist, (uint32_t)nt, k2, v2);
    CK_LAUNCH();
    std::swap(keys, k2);
    std::swap(vals, v2);
  }
  return GRD_OK;
}

// Per-partition constants of phase B.
struct PartInfo {
  uint32_t slot_base, n_owned, ostart, prebase;
};

struct CsrIn {
  const uint64_t* ro;
  const uint32_t* col;
  const uint32_t* w;
  const uint32_t* mir_in;  // nullptr: gid % M (NaivePartitioner)
  uint32_t V, M;
  uint64_t E;
};

// ---------------------------------------------------------------- phase A --
// Mirror id, out-degree and row-start mark of every vertex.  (Partition
// sizes come from the sorted partition ids, edge counts from the row
// offsets: no shared counter for every thread to contend on.)
__global__ void __launch_bounds__(LT) k_lay_vertex(CsrIn in, uint32_t* mir, uint32_t* outdeg, uint32_t* esrc,
                                                   uint32_t* err) {
  uint32_t bad = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < in.V; v += gridDim.x * blockDim.x) {
    uint32_t p = in.mir_in ? in.mir_in[v] : v % in.M;
    if (p >= in.M) {
      bad |= E_MIRROR;
      p = 0;
    }
    mir[v] = p;
    const uint64_t r0 = in.ro[v], r1 = in.ro[v + 1];
    uint64_t deg = 0;
    if (r1 < r0 || r1 > in.E) {
      bad |= E_ROWS;
    } else {
      deg = r1 - r0;
      if (deg) esrc[r0] = v;  // the row's first edge: source of the run that follows
    }
    outdeg[v] = (uint32_t)deg;
  }
  if (bad) atomicOr(err, bad);
}

// Proxy discovery (cross_node_mirrors, src/DistributedGraph.cpp:345-349): a
// destination mastered outside the source's partition sets its bit in that
// partition's bitmap.
__global__ void __launch_bounds__(LT) k_lay_proxy_bits(CsrIn in, const uint32_t* __restrict__ mir,
                                                       const uint32_t* __restrict__ esrc, unsigned long long* bm,
                                                       uint64_t W, uint32_t* err) {
  uint32_t bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < in.E;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t d = in.col[i];
    if (d >= in.V) {
      bad |= E_COL;
      continue;
    }
    const uint32_t p = mir[esrc[i]];
    if (mir[d] == p) continue;
    unsigned long long* word = bm + (uint64_t)p * W + (d >> 6);
    const unsigned long long bit = 1ull << (d & 63);
    if (!(__ldcg(word) & bit)) atomicOr(word, bit);
  }
  if (bad) atomicOr(err, bad);
}

__global__ void __launch_bounds__(LT) k_lay_popc(const unsigned long long* __restrict__ bm, uint64_t n,
                                                 uint32_t* cnt) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    cnt[i] = (uint32_t)__popcll(bm[i]);
}

__global__ void __launch_bounds__(LT) k_iota(uint32_t* a, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    a[i] = (uint32_t)i;
}

// Proxy prefix at each partition's first bitmap word (the partition's
// proxy count is the difference of two neighbours).
__global__ void k_lay_part_prefix(const uint32_t* __restrict__ pre, uint64_t W, uint32_t M, uint32_t* out) {
  for (uint32_t p = threadIdx.x; p <= M; p += blockDim.x) out[p] = pre[(uint64_t)p * W];
}

// ---------------------------------------------------------------- phase B --
__global__ void __launch_bounds__(LT) k_lay_owned(const uint32_t* __restrict__ sorted_gid,
                                                  const uint32_t* __restrict__ mir, uint32_t V,
                                                  const PartInfo* __restrict__ info, uint32_t* own_slot,
                                                  uint32_t* slot_gid) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
    const uint32_t v = sorted_gid[i];
    const PartInfo pi = info[mir[v]];
    const uint32_t s = pi.slot_base + (i - pi.ostart);
    own_slot[v] = s;
    slot_gid[s] = v;
  }
}

__global__ void __launch_bounds__(LT) k_lay_proxy_slots(const unsigned long long* __restrict__ bm,
                                                        const uint32_t* __restrict__ pre, uint64_t W, uint32_t M,
                                                        const PartInfo* __restrict__ info, uint32_t* slot_gid) {
  const uint64_t n = W * M;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long x = bm[i];
    if (!x) continue;
    const uint32_t p = (uint32_t)(i / W);
    const uint64_t w = i - (uint64_t)p * W;
    const PartInfo pi = info[p];
    uint32_t s = pi.slot_base + pi.n_owned + (pre[i] - pi.prebase);
    while (x) {
      const int b = __ffsll((long long)x) - 1;
      x &= x - 1;
      slot_gid[s++] = (uint32_t)(w * 64 + (uint64_t)b);
    }
  }
}

__global__ void __launch_bounds__(LT) k_lay_slot_deg(const uint32_t* __restrict__ slot_gid,
                                                     const uint32_t* __restrict__ own_slot,
                                                     const uint32_t* __restrict__ outdeg, uint64_t S, uint32_t* deg) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t g = slot_gid[s];
    deg[s] = (g != INVALID && own_slot[g] == (uint32_t)s) ? outdeg[g] : 0u;
  }
}

// Columns relabelled to slots of the source's partition: the destination's
// owned slot when it lives there, else its proxy slot (rank of its bit).
__global__ void __launch_bounds__(LT) k_lay_edges(CsrIn in, const uint32_t* __restrict__ mir,
                                                  const uint32_t* __restrict__ esrc,
                                                  const uint32_t* __restrict__ own_slot,
                                                  const uint32_t* __restrict__ row_off,
                                                  const unsigned long long* __restrict__ bm,
                                                  const uint32_t* __restrict__ pre, uint64_t W,
                                                  const PartInfo* __restrict__ info, uint32_t* col_out,
                                                  uint32_t* wgt_out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < in.E;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t u = esrc[i];
    const uint32_t p = mir[u];
    const uint32_t o = row_off[own_slot[u]] + (uint32_t)(i - in.ro[u]);
    const uint32_t d = in.col[i];
    uint32_t ds;
    if (mir[d] == p) {
      ds = own_slot[d];
    } else {
      const PartInfo pi = info[p];
      const uint64_t wi = (uint64_t)p * W + (d >> 6);
      ds = pi.slot_base + pi.n_owned + (pre[wi] - pi.prebase) + (uint32_t)__popcll(bm[wi] & ((1ull << (d & 63)) - 1ull));
    }
    col_out[o] = ds;
    if (in.w) wgt_out[o] = in.w[i];
  }
}

// Hub rows (more than HUB_DEGREE edges) cut at absolute multiples of
// HUB_CHUNK: count per slot, then fill at the scanned offsets.
__global__ void __launch_bounds__(LT) k_lay_hub_count(const uint32_t* __restrict__ row_off, uint64_t S,
                                                      uint32_t* cnt) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t e0 = row_off[s], e1 = row_off[s + 1];
    cnt[s] = (e1 - e0 > HUB_DEGREE) ? ((e1 - 1) / HUB_CHUNK - e0 / HUB_CHUNK + 1) : 0u;
  }
}

__global__ void __launch_bounds__(LT) k_lay_hub_fill(const uint32_t* __restrict__ row_off,
                                                     const uint32_t* __restrict__ off, uint64_t S, HubChunkD* hubs) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
    if (off[s + 1] == off[s]) continue;
    const uint32_t e1 = row_off[s + 1];
    uint32_t a = row_off[s], k = off[s];
    while (a < e1) {
      const uint32_t b = min(e1, (a / HUB_CHUNK + 1) * HUB_CHUNK);
      hubs[k++] = HubChunkD{(uint32_t)s, a, b};
      a = b;
    }
  }
}

// ------------------------------------------------------------ in-edges --
__global__ void __launch_bounds__(LT) k_lay_row_marks(const uint32_t* __restrict__ row_off, uint64_t S,
                                                      uint32_t* lsrc) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x)
    if (row_off[s + 1] > row_off[s]) lsrc[row_off[s]] = (uint32_t)s;
}

__global__ void __launch_bounds__(LT) k_lay_in_gather(const uint32_t* __restrict__ edge, uint64_t E,
                                                      const uint32_t* __restrict__ lsrc,
                                                      const uint32_t* __restrict__ wgt, uint32_t* in_src,
                                                      uint32_t* in_wgt) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t e = edge[k];
    in_src[k] = lsrc[e];
    if (wgt) in_wgt[k] = wgt[e];
  }
}

// Bounds of sorted keys: out[s] = first k with key[k] >= s, for s = 0..S
// (the in-edge offsets; the partition starts of the owned order).
__global__ void __launch_bounds__(LT) k_lay_in_off(const uint32_t* __restrict__ key, uint64_t E, uint64_t S,
                                                   uint32_t* in_off) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= E; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = k ? (uint64_t)key[k - 1] + 1 : 0;  // slots after the previous key
    const uint64_t hi = k < E ? (uint64_t)key[k] : S;      // up to and including this key
    for (uint64_t s = lo; s <= hi; ++s) in_off[s] = (uint32_t)k;
  }
}

__global__ void __launch_bounds__(LT) k_lay_in_class(const uint32_t* __restrict__ in_off, uint64_t S, uint32_t* ch,
                                                     uint32_t* cm) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t d = in_off[s + 1] - in_off[s];
    ch[s] = d > PULL_HUB ? 1u : 0u;
    cm[s] = (d > PULL_MED && d <= PULL_HUB) ? 1u : 0u;
  }
}

__global__ void __launch_bounds__(LT) k_lay_in_class_fill(const uint32_t* __restrict__ in_off, uint64_t S,
                                                          const uint32_t* __restrict__ oh,
                                                          const uint32_t* __restrict__ om, HubChunkD* hubs,
                                                          HubChunkD* meds) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
    const HubChunkD c{(uint32_t)s, in_off[s], in_off[s + 1]};
    if (oh[s + 1] != oh[s]) hubs[oh[s]] = c;
    if (om[s + 1] != om[s]) meds[om[s]] = c;
  }
}

std::string layout_error(uint32_t err) {
  if (err & E_ROWS) return "row_offsets is not monotone";
  if (err & E_COL) return "col_indices holds an id >= num_vertices";
  if (err & E_MIRROR) return "mirror partition id >= num_memory";
  return "invalid graph";
}

}  // namespace

// Checks the host-visible parts of a CSR for the device build.
int grd_scan_add_u32(grd_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, bool total_at_n) {
  Scratch tmp(ctx);
  return scan<OpAdd>(ctx, tmp, in, out, n, false, total_at_n);
}

int grd_scan_u32(grd_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, bool inclusive, bool total_at_n) {
  Scratch tmp(ctx);
  return scan<OpAdd>(ctx, tmp, in, out, n, inclusive, total_at_n);
}

int grd_device_layout_check(const grd_csr* graph, uint32_t M, std::string* why) {
  if (!graph) return *why = "graph is NULL", GRD_E_INVALID;
  if (M == 0 || M > DEV_MAX_PARTS) return *why = "the device layout build takes 1..64 memory partitions", GRD_E_INVALID;
  if (graph->num_vertices == 0) return *why = "graph has no vertices", GRD_E_INVALID;
  if (!graph->row_offsets) return *why = "row_offsets is NULL", GRD_E_INVALID;
  if (graph->num_edges && !graph->col_indices) return *why = "col_indices is NULL", GRD_E_INVALID;
  if (graph->num_edges >= 0xFFFFFFF0ull)
    return *why = "more than 2^32-16 edges: 32-bit edge offsets would overflow", GRD_E_INVALID;
  if (graph->row_offsets[0] != 0 || graph->row_offsets[graph->num_vertices] != graph->num_edges)
    return *why = "row_offsets[0] must be 0 and row_offsets[V] must equal num_edges", GRD_E_INVALID;
  return GRD_OK;
}

// Host->device copies of the caller's CSR arrays.  Copies straight from
// pageable memory ran at anything from 8 to 45 GB/s from one call to the next
// on the same arrays; so the arrays are first copied by host threads into a
// pinned staging area kept by the ctx, and the copy engine reads them from
// there, chunk by chunk, each chunk's copy overlapping the next chunk's
// host copy.
namespace {
struct StagedUpload {
  grd_ctx* ctx;
  cudaStream_t s;
  size_t used = 0;
  static constexpr size_t kChunk = size_t(256) << 20;
  static constexpr size_t kDirect = size_t(8) << 20;  // smaller arrays go straight from the caller
  int reserve(size_t bytes) {
    CK(cudaStreamSynchronize(s));  // no earlier copy still reads the area
    if (ctx->ingest_stage_bytes < bytes) {
      if (ctx->ingest_stage) CK(cudaFreeHost(ctx->ingest_stage));
      ctx->ingest_stage = nullptr;
      ctx->ingest_stage_bytes = 0;
      if (cudaHostAlloc((void**)&ctx->ingest_stage, bytes, cudaHostAllocDefault) != cudaSuccess) {
        (void)cudaGetLastError();
        ctx->ingest_stage = nullptr;  // copies then go straight from the caller's memory
        return GRD_OK;
      }
      ctx->ingest_stage_bytes = bytes;
    }
    return GRD_OK;
  }
  int copy(void* dst, const void* src, size_t bytes) {
    if (!bytes) return GRD_OK;
    if (bytes < kDirect || !ctx->ingest_stage || used + bytes > ctx->ingest_stage_bytes) {
      CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
      return GRD_OK;
    }
    unsigned char* stage = ctx->ingest_stage + used;
    used += (bytes + 255) / 256 * 256;
    const unsigned nt = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    for (size_t off = 0; off < bytes; off += kChunk) {
      const size_t n = std::min(kChunk, bytes - off);
      const size_t part = (n + nt - 1) / nt;
      std::vector<std::thread> th;
      for (unsigned t = 0; t < nt; ++t) {
        const size_t a = std::min(n, t * part), b = std::min(n, a + part);
        if (a < b)
          th.emplace_back([=] { std::memcpy(stage + off + a, static_cast<const unsigned char*>(src) + off + a, b - a); });
      }
      for (auto& x : th) x.join();
      CK(cudaMemcpyAsync(static_cast<unsigned char*>(dst) + off, stage + off, n, cudaMemcpyHostToDevice, s));
    }
    return GRD_OK;
  }
};
}  // namespace

// Uploads the CSR and builds the resident layout.  first: size the ctx's
// arrays from it; otherwise the partition sizes must equal the ctx's.
int grd_device_layout_build(grd_ctx* ctx, const grd_csr* graph, const uint32_t* mirror_part, bool first) {
  const uint32_t V = graph->num_vertices, M = ctx->L.M;
  const uint64_t E = graph->num_edges;
  const bool weighted = graph->weights != nullptr;
  if (!first && (V != ctx->L.V || E != ctx->L.E || weighted != ctx->L.weighted)) {
    ctx->err = "grd_ingest: the graph's size differs from the ctx's";
    return GRD_E_INVALID;
  }
  // A re-ingest overwrites the resident arrays as it goes; until it has
  // finished, the ctx refuses to run (a graph that turns out not to match
  // the ctx's partition, proxy or hub counts leaves it that way).
  ctx->layout_valid = false;
  ctx->layout_gen++;
  cudaStream_t s = ctx->stream;
  Scratch tmp(ctx);
  // inputs
  uint64_t* d_ro = nullptr;
  uint32_t *d_col = nullptr, *d_w = nullptr, *d_mir_in = nullptr;
  TRY(tmp.get(&d_ro, (uint64_t)V + 1));
  TRY(tmp.get(&d_col, E));
  StagedUpload up{ctx, s};
  TRY(up.reserve(sizeof(uint64_t) * ((uint64_t)V + 1) + sizeof(uint32_t) * E * (weighted ? 2 : 1) +
                 (mirror_part ? sizeof(uint32_t) * V : 0) + 4 * 256));
  TRY(up.copy(d_ro, graph->row_offsets, sizeof(uint64_t) * ((uint64_t)V + 1)));
  TRY(up.copy(d_col, graph->col_indices, sizeof(uint32_t) * E));
  uint64_t h2d = sizeof(uint64_t) * ((uint64_t)V + 1) + sizeof(uint32_t) * E;
  if (weighted) {
    TRY(tmp.get(&d_w, E));
    TRY(up.copy(d_w, graph->weights, sizeof(uint32_t) * E));
    h2d += sizeof(uint32_t) * E;
  }
  if (mirror_part) {
    TRY(tmp.get(&d_mir_in, V));
    TRY(up.copy(d_mir_in, mirror_part, sizeof(uint32_t) * V));
    h2d += sizeof(uint32_t) * V;
  }
  const CsrIn in{d_ro, d_col, d_w, d_mir_in, V, M, E};

  // ---- phase A
  const uint64_t W = ((uint64_t)V + 63) / 64;
  uint32_t *mir = nullptr, *esrc = nullptr, *err = nullptr, *outdeg = nullptr, *pcnt = nullptr, *pre = nullptr;
  uint32_t *pb = nullptr, *okeys = nullptr, *ovals = nullptr, *pstart = nullptr;
  unsigned long long* bm = nullptr;
  TRY(tmp.get(&mir, V));
  TRY(tmp.get(&esrc, E));
  TRY(tmp.get(&err, 1));
  TRY(tmp.get(&pstart, M + 1));
  TRY(tmp.get(&bm, W * M));
  TRY(tmp.get(&pcnt, W * M));
  TRY(tmp.get(&pre, W * M + 1));
  TRY(tmp.get(&pb, M + 1));
  TRY(tmp.get(&okeys, V));
  TRY(tmp.get(&ovals, V));
  if (first) {
    TRY(tmp.get(&outdeg, V));  // the ctx's outdeg array does not exist yet
  } else {
    outdeg = const_cast<uint32_t*>(ctx->g.outdeg);
  }
  CK(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
  CK(cudaMemsetAsync(bm, 0, sizeof(unsigned long long) * W * M, s));
  if (E) CK(cudaMemsetAsync(esrc, 0, sizeof(uint32_t) * E, s));
  k_lay_vertex<<<grid_of(ctx, V), LT, 0, s>>>(in, mir, outdeg, esrc, err);
  CK_LAUNCH();
  TRY(scan<OpMax>(ctx, tmp, esrc, esrc, E, true, false));
  k_lay_proxy_bits<<<grid_of(ctx, E), LT, 0, s>>>(in, mir, esrc, bm, W, err);
  k_lay_popc<<<grid_of(ctx, W * M), LT, 0, s>>>(bm, W * M, pcnt);
  CK_LAUNCH();
  TRY(scan<OpAdd>(ctx, tmp, pcnt, pre, W * M, false, true));
  k_lay_part_prefix<<<1, 128, 0, s>>>(pre, W, M, pb);
  CK(cudaMemcpyAsync(okeys, mir, sizeof(uint32_t) * V, cudaMemcpyDeviceToDevice, s));
  k_iota<<<grid_of(ctx, V), LT, 0, s>>>(ovals, V);
  CK_LAUNCH();
  uint32_t *sk = okeys, *sv = ovals;
  TRY(radix_sort(ctx, tmp, sk, sv, V, bits_for(M - 1)));  // owned gids, partition-major, ascending
  k_lay_in_off<<<grid_of(ctx, (uint64_t)V + 1), LT, 0, s>>>(sk, V, M, pstart);
  CK_LAUNCH();
  // sizes to the host
  std::vector<uint32_t> h_pb(M + 1), h_ps(M + 1);
  uint32_t h_err = 0;
  CK(cudaMemcpyAsync(h_ps.data(), pstart, sizeof(uint32_t) * (M + 1), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h_pb.data(), pb, sizeof(uint32_t) * (M + 1), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&h_err, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h_err) {
    ctx->err = layout_error(h_err);
    return GRD_E_INVALID;
  }
  Layout& L = ctx->L;
  std::vector<uint32_t> n_owned(M), n_proxy(M);
  for (uint32_t p = 0; p < M; ++p) {
    n_owned[p] = h_ps[p + 1] - h_ps[p];
    n_proxy[p] = h_pb[p + 1] - h_pb[p];
  }
  if (first) {
    L.n_owned = n_owned;
    L.n_proxy = n_proxy;
    L.slot_base.assign(M, 0);
    uint64_t S = 0;
    for (uint32_t p = 0; p < M; ++p) {
      L.slot_base[p] = (uint32_t)S;
      const uint64_t T = (uint64_t)n_owned[p] + n_proxy[p];
      S += std::max<uint64_t>(TILE_SLOTS, (T + TILE_SLOTS - 1) / TILE_SLOTS * TILE_SLOTS);
      if (S >= 0xFFFFFFF0ull) {
        ctx->err = "slot space exceeds 2^32";
        return GRD_E_INVALID;
      }
    }
    L.S = S;
    const uint64_t nt_tiles = S / TILE_SLOTS;
    L.tile_part.assign(nt_tiles, 0);
    L.tile_first.assign(nt_tiles, 0);
    for (uint32_t p = 0; p < M; ++p) {
      const uint64_t t0 = L.slot_base[p] / TILE_SLOTS;
      const uint64_t t1 = (p + 1 < M) ? L.slot_base[p + 1] / TILE_SLOTS : nt_tiles;
      for (uint64_t t = t0; t < t1; ++t) {
        L.tile_part[t] = p;
        L.tile_first[t] = (uint32_t)t0;
      }
    }
    TRY(grd_alloc_resident(ctx));
    CK(cudaMemcpyAsync((void*)ctx->g.outdeg, outdeg, sizeof(uint32_t) * V, cudaMemcpyDeviceToDevice, s));
    std::vector<uint32_t> T(M);
    for (uint32_t p = 0; p < M; ++p) T[p] = L.T(p);
    CK(cudaMemcpyAsync((void*)ctx->g.tile_part, L.tile_part.data(), sizeof(uint32_t) * nt_tiles,
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)ctx->g.part_base, L.slot_base.data(), sizeof(uint32_t) * M, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)ctx->g.part_T, T.data(), sizeof(uint32_t) * M, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)ctx->g.part_owned, L.n_owned.data(), sizeof(uint32_t) * M, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the pageable sources above are locals
  } else if (n_owned != L.n_owned || n_proxy != L.n_proxy) {
    ctx->err = "grd_ingest: the graph's partition sizes differ from the ctx's";
    return GRD_E_INVALID;
  }

  // ---- phase B
  const uint64_t S = L.S;
  std::vector<PartInfo> h_info(M);
  uint32_t ostart = 0;
  for (uint32_t p = 0; p < M; ++p) {
    h_info[p] = PartInfo{L.slot_base[p], L.n_owned[p], ostart, h_pb[p]};
    ostart += L.n_owned[p];
  }
  PartInfo* info = nullptr;
  TRY(tmp.get(&info, M));
  CK(cudaMemcpyAsync(info, h_info.data(), sizeof(PartInfo) * M, cudaMemcpyHostToDevice, s));
  DevGraph& g = ctx->g;
  uint32_t* slot_gid = const_cast<uint32_t*>(g.slot_gid);
  uint32_t* row_off = const_cast<uint32_t*>(g.row_off);
  CK(cudaMemsetAsync(slot_gid, 0xFF, sizeof(uint32_t) * S, s));
  k_lay_owned<<<grid_of(ctx, V), LT, 0, s>>>(sv, mir, V, info, ctx->st.own_slot, slot_gid);
  k_lay_proxy_slots<<<grid_of(ctx, W * M), LT, 0, s>>>(bm, pre, W, M, info, slot_gid);
  uint32_t* sdeg = nullptr;
  TRY(tmp.get(&sdeg, S));
  k_lay_slot_deg<<<grid_of(ctx, S), LT, 0, s>>>(slot_gid, ctx->st.own_slot, g.outdeg, S, sdeg);
  CK_LAUNCH();
  TRY(scan<OpAdd>(ctx, tmp, sdeg, row_off, S, false, true));
  {  // edges per partition: its owned rows are contiguous in the row offsets
    std::vector<uint32_t> ends(2 * M);
    for (uint32_t p = 0; p < M; ++p) {
      CK(cudaMemcpyAsync(&ends[2 * p], row_off + L.slot_base[p], sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&ends[2 * p + 1], row_off + L.slot_base[p] + L.n_owned[p], sizeof(uint32_t),
                         cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    std::vector<uint64_t> part_edges(M);
    for (uint32_t p = 0; p < M; ++p) part_edges[p] = ends[2 * p + 1] - ends[2 * p];
    if (first) {
      L.part_edges = part_edges;
    } else if (part_edges != L.part_edges) {
      ctx->err = "grd_ingest: the graph's partition sizes differ from the ctx's";
      return GRD_E_INVALID;
    }
  }
  k_lay_edges<<<grid_of(ctx, E), LT, 0, s>>>(in, mir, esrc, ctx->st.own_slot, row_off, bm, pre, W, info,
                                             const_cast<uint32_t*>(g.col), const_cast<uint32_t*>(g.wgt));
  CK_LAUNCH();
  // hubs
  uint32_t* hoff = nullptr;
  TRY(tmp.get(&hoff, S + 1));
  k_lay_hub_count<<<grid_of(ctx, S), LT, 0, s>>>(row_off, S, sdeg);
  CK_LAUNCH();
  TRY(scan<OpAdd>(ctx, tmp, sdeg, hoff, S, false, true));
  uint32_t nh = 0;
  CK(cudaMemcpyAsync(&nh, hoff + S, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (first) {
    void* p = nullptr;
    TRY(grd_dev_alloc_bytes(ctx, &p, sizeof(HubChunkD) * std::max<uint32_t>(nh, 1)));
    g.hubs = static_cast<const HubChunkD*>(p);
    g.num_hubs = nh;
  } else if (nh != g.num_hubs) {
    ctx->err = "grd_ingest: the graph's hub rows differ from the ctx's";
    return GRD_E_INVALID;
  }
  k_lay_hub_fill<<<grid_of(ctx, S), LT, 0, s>>>(row_off, hoff, S, const_cast<HubChunkD*>(g.hubs));
  CK_LAUNCH();
  ctx->upload_bytes = h2d;
  if (ctx->in_edges_alloc) TRY(grd_device_in_edges(ctx));  // a re-ingest rebuilds the pull view too
  CK(cudaStreamSynchronize(s));
  ctx->layout_valid = true;
  return GRD_OK;
}

// In-edge (CSC) view of the resident layout, on the device.
int grd_device_in_edges(grd_ctx* ctx) {
  const Layout& L = ctx->L;
  const uint64_t S = L.S, E = L.E;
  cudaStream_t s = ctx->stream;
  DevGraph& g = ctx->g;
  if (!ctx->in_edges_alloc) {
    TRY(grd_dev_alloc_bytes(ctx, (void**)&g.in_off, sizeof(uint32_t) * (S + 1)));
    TRY(grd_dev_alloc_bytes(ctx, (void**)&g.in_src, sizeof(uint32_t) * std::max<uint64_t>(E, 4)));
    if (L.weighted) TRY(grd_dev_alloc_bytes(ctx, (void**)&g.in_wgt, sizeof(uint32_t) * std::max<uint64_t>(E, 4)));
  }
  Scratch tmp(ctx);
  uint32_t *lsrc = nullptr, *keys = nullptr, *vals = nullptr;
  TRY(tmp.get(&lsrc, E));
  TRY(tmp.get(&keys, E));
  TRY(tmp.get(&vals, E));
  if (E) {
    CK(cudaMemsetAsync(lsrc, 0, sizeof(uint32_t) * E, s));
    CK(cudaMemcpyAsync(keys, g.col, sizeof(uint32_t) * E, cudaMemcpyDeviceToDevice, s));
  }
  k_lay_row_marks<<<grid_of(ctx, S), LT, 0, s>>>(g.row_off, S, lsrc);
  k_iota<<<grid_of(ctx, E), LT, 0, s>>>(vals, E);
  CK_LAUNCH();
  TRY(scan<OpMax>(ctx, tmp, lsrc, lsrc, E, true, false));
  TRY(radix_sort(ctx, tmp, keys, vals, E, bits_for(S - 1)));
  k_lay_in_gather<<<grid_of(ctx, E), LT, 0, s>>>(vals, E, lsrc, L.weighted ? g.wgt : nullptr,
                                                 const_cast<uint32_t*>(g.in_src),
                                                 L.weighted ? const_cast<uint32_t*>(g.in_wgt) : nullptr);
  k_lay_in_off<<<grid_of(ctx, E + 1), LT, 0, s>>>(keys, E, S, const_cast<uint32_t*>(g.in_off));
  CK_LAUNCH();
  uint32_t *ch = nullptr, *cm = nullptr, *oh = nullptr, *om = nullptr;
  TRY(tmp.get(&ch, S));
  TRY(tmp.get(&cm, S));
  TRY(tmp.get(&oh, S + 1));
  TRY(tmp.get(&om, S + 1));
  k_lay_in_class<<<grid_of(ctx, S), LT, 0, s>>>(g.in_off, S, ch, cm);
  CK_LAUNCH();
  TRY(scan<OpAdd>(ctx, tmp, ch, oh, S, false, true));
  TRY(scan<OpAdd>(ctx, tmp, cm, om, S, false, true));
  uint32_t n2[2] = {0, 0};
  CK(cudaMemcpyAsync(&n2[0], oh + S, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&n2[1], om + S, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  PullState& P = ctx->pull;
  if (!ctx->in_edges_alloc) {
    TRY(grd_dev_alloc_bytes(ctx, (void**)&P.in_hubs, sizeof(HubChunkD) * std::max<uint32_t>(n2[0], 1)));
    TRY(grd_dev_alloc_bytes(ctx, (void**)&P.in_meds, sizeof(HubChunkD) * std::max<uint32_t>(n2[1], 1)));
    P.num_in_hubs = n2[0];
    P.num_in_meds = n2[1];
  } else if (n2[0] != P.num_in_hubs || n2[1] != P.num_in_meds) {
    ctx->err = "grd_ingest: the graph's in-degree classes differ from the ctx's";
    return GRD_E_INVALID;
  }
  k_lay_in_class_fill<<<grid_of(ctx, S), LT, 0, s>>>(g.in_off, S, oh, om, P.in_hubs, P.in_meds);
  CK_LAUNCH();
  CK(cudaStreamSynchronize(s));
  ctx->in_edges_alloc = true;
  ctx->layout_gen++;
  return GRD_OK;
}
