// sm_103a kernels of the per-round graph operator.
//
// Data layout in HBM (one ctx):
//   compute side, gid-indexed [V]: prop (vertex_properties), upd
//     (vertex_updates), ranks (PageRank pr_vals), frontier bitmap F and the
//     vertex_updates dirty bitmap UD (u32 words, bit g&31 of word g>>5);
//   memory side, global-slot-indexed [S]: mprop, mupd, out-edge CSR
//     (row_off/col/wgt), the forward wire bitvector FB (= the memory-side
//     vertex_properties dirty set), the backward wire bitvector MD (= the
//     memory-side vertex_updates dirty set), packed value buffers FV/BV laid
//     out per partition at slot_base[p], and the compacted active list AL.
// Bitvectors are u32 words; on a little-endian device the u64 word w of a
// partition's wire bitvector is u32 words 2w,2w+1, so the layout is the
// reference's DynamicBitSet word layout.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace grd {

constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr uint32_t K_TILE_SLOTS = 32768;
constexpr uint32_t K_TILE_WORDS = K_TILE_SLOTS / 32;
constexpr uint32_t K_HUB_DEGREE = 2048;

enum Algo : int { A_PR_DELTA = 0, A_PR_PULL = 1, A_CC = 2, A_SSSP_HOP = 3, A_SSSP_W = 4 };

enum Counter : int {
  C_FRONTIER = 0,  // |frontier| after update
  C_ACTIVE = 1,    // actives unpacked by the last forward sync (all partitions)
  C_EDGES = 2,     // cumulative edges scanned
  C_BYTES = 3,     // cumulative wire bytes (true size)
  C_REFBYTES = 4,  // cumulative bytes by the reference's accounting
  C_TOTAL = 5,     // total set bits of the last compaction scan
  C_ERR = 6,       // first device-side error code (0 = none)
  C_PULL_EDGES = 7,
  NUM_COUNTERS = 16
};

struct HubChunkD {
  uint32_t slot, e0, e1;
};

struct DevGraph {
  uint32_t V, M;
  uint64_t S;
  uint32_t num_tiles, num_hubs;
  const uint32_t* slot_gid;
  const uint32_t* row_off;
  const uint32_t* col;
  const uint32_t* wgt;
  const uint32_t* outdeg;
  const uint32_t* in_off;
  const uint32_t* in_src;
  const uint32_t* in_wgt;
  const HubChunkD* hubs;
  const uint32_t* tile_part;
  const uint32_t* part_base;   // [M] slot base
  const uint32_t* part_T;      // [M] owned + proxy
  const uint32_t* part_owned;  // [M]
};

struct DevState {
  uint32_t* prop;
  uint32_t* upd;
  float* ranks;
  uint32_t* F;
  uint32_t* UD;
  uint32_t* mprop;
  uint32_t* mupd;
  uint32_t* FB;
  uint32_t* FV;
  uint32_t* MD;
  uint32_t* BV;
  uint32_t* AL;
  uint32_t* tile_cnt;
  uint32_t* tile_off;
  uint32_t* tile_goff;
  uint32_t* part_cnt;
  unsigned long long* counters;
};

// ---------------------------------------------------------------- helpers --
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const uint32_t lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t n = __shfl_up_sync(FULL, v, o);
    if (lane >= (uint32_t)o) v += n;
  }
  return v;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// Block-wide sum for blockDim.x <= 1024 (result valid in every thread).
__device__ __forceinline__ uint32_t block_sum(uint32_t v) {
  __shared__ uint32_t s_part[32];
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) s_part[w] = v;
  __syncthreads();
  const uint32_t nw = (blockDim.x + 31) >> 5;
  uint32_t r = lane < nw ? s_part[lane] : 0;
  r = warp_sum(r);
  return r;
}

__device__ __forceinline__ bool test_bit(const uint32_t* bm, uint32_t i) {
  return (bm[i >> 5] >> (i & 31)) & 1u;
}

__device__ __forceinline__ void set_dirty(uint32_t* bm, uint32_t i) {
  const uint32_t bit = 1u << (i & 31);
  uint32_t* w = bm + (i >> 5);
  if (!(__ldcg(w) & bit)) atomicOr(w, bit);
}

__device__ __forceinline__ uint32_t sat_add(uint32_t a, uint32_t b) {
  uint32_t s = a + b;
  return s < a ? 0xFFFFFFFFu : s;
}

// ------------------------------------------------------------------- init --
// Reference init(): pr.cpp:20-61, cc.cpp:18-40, sssp.cpp:18-47.
template <int A>
__global__ void __launch_bounds__(256) k_init(DevGraph g, DevState st, uint32_t source, double damping) {
  const uint64_t n = g.S > g.V ? g.S : g.V;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ((n + 31) & ~31ull);
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t fbit = 0;
    if (i < g.V) {
      const uint32_t v = (uint32_t)i;
      if (A == A_CC) {
        st.prop[v] = v;
        st.upd[v] = 0xFFFFFFFFu;
        fbit = 1;
      } else if (A == A_SSSP_HOP || A == A_SSSP_W) {
        const uint32_t x = (v == source) ? 0u : 0xFFFFFFFFu;
        st.prop[v] = x;
        st.upd[v] = x;
        fbit = (v == source);
      } else {  // PageRank (delta and pull share the initial state)
        const uint32_t deg = g.outdeg[v];
        if (deg != 0) {
          st.prop[v] = __float_as_uint((float)(damping * (1.0 - damping) / (double)deg));
          st.ranks[v] = (float)(1.0 - damping);
          fbit = 1;
        } else {
          st.prop[v] = 0;
          st.ranks[v] = 0.0f;
        }
        st.upd[v] = 0;
      }
    }
    const uint32_t m = __ballot_sync(FULL, fbit);
    if (lane_id() == 0 && i < g.V) {
      st.F[i >> 5] = m;
      st.UD[i >> 5] = 0;
    }
    if (i < g.S) {
      const uint32_t x = (A == A_PR_DELTA || A == A_PR_PULL) ? 0u : 0xFFFFFFFFu;
      st.mprop[i] = x;
      st.mupd[i] = x;
      if ((i & 31) == 0) {
        st.FB[i >> 5] = 0;
        st.MD[i >> 5] = 0;
      }
    }
  }
}

// ---------------------------------------------------- forward sync: bits --
// Compute side of src/GraphAlgorithm.cpp:199-246: every frontier vertex sets
// the bit of its owned slot in its mirror partition's bitvector.  One warp
// builds one 32-bit word by ballot over 32 consecutive slots; the per-tile
// popcount feeds the compaction scan.
static __global__ void __launch_bounds__(256) k_fwd_bits(DevGraph g, DevState st) {
  const uint32_t t = blockIdx.x;
  const uint32_t p = g.tile_part[t];
  const uint32_t base = g.part_base[p], nown = g.part_owned[p];
  const uint32_t t0 = t * K_TILE_SLOTS;
  uint32_t cnt = 0;
  for (uint32_t i = threadIdx.x; i < K_TILE_SLOTS; i += blockDim.x) {
    const uint32_t s = t0 + i;
    uint32_t bit = 0;
    if (s - base < nown) {
      const uint32_t gid = __ldg(&g.slot_gid[s]);
      bit = test_bit(st.F, gid);
    }
    const uint32_t m = __ballot_sync(FULL, bit);
    if (lane_id() == 0) {
      st.FB[s >> 5] = m;
      cnt += __popc(m);
    }
  }
  cnt = block_sum(cnt);
  if (threadIdx.x == 0) st.tile_cnt[t] = cnt;
}

// Per-tile set-bit count of a bitvector (backward sync).
static __global__ void __launch_bounds__(256) k_tile_count(const uint32_t* __restrict__ bits, uint32_t* tile_cnt) {
  const uint32_t t = blockIdx.x;
  const uint32_t* w = bits + (size_t)t * K_TILE_WORDS;
  uint32_t c = 0;
  for (uint32_t i = threadIdx.x; i < K_TILE_WORDS; i += blockDim.x) c += __popc(w[i]);
  c = block_sum(c);
  if (threadIdx.x == 0) tile_cnt[t] = c;
}

// Exclusive scan of tile counts, restarting per partition (packed value index
// j of the j-th set bit) and global (index into the active list).  Also
// accumulates the wire-size statistics of one sync direction.
static __global__ void __launch_bounds__(1024) k_scan_tiles(DevGraph g, DevState st, int set_active) {
  __shared__ uint32_t s_w[32];
  __shared__ uint32_t s_carry;
  const uint32_t tid = threadIdx.x, lane = lane_id(), w = tid >> 5;
  uint32_t gcarry = 0;
  unsigned long long bytes = 0, refbytes = 0;
  for (uint32_t p = 0; p < g.M; ++p) {
    const uint32_t t0 = g.part_base[p] / K_TILE_SLOTS;
    const uint32_t t1 = (p + 1 < g.M) ? g.part_base[p + 1] / K_TILE_SLOTS : g.num_tiles;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t c0 = t0; c0 < t1; c0 += blockDim.x) {
      const uint32_t t = c0 + tid;
      const uint32_t v = t < t1 ? st.tile_cnt[t] : 0;
      uint32_t incl = warp_incl_scan(v);
      if (lane == 31) s_w[w] = incl;
      __syncthreads();
      if (w == 0) {
        uint32_t x = s_w[lane];
        s_w[lane] = warp_incl_scan(x) - x;
      }
      __syncthreads();
      incl += s_w[w];
      const uint32_t carry = s_carry;
      if (t < t1) {
        st.tile_off[t] = carry + incl - v;
        st.tile_goff[t] = gcarry + carry + incl - v;
      }
      __syncthreads();
      if (tid == blockDim.x - 1) s_carry = carry + incl;
      __syncthreads();
    }
    const uint32_t kp = s_carry;
    if (tid == 0) {
      st.part_cnt[p] = kp;
      const unsigned long long words64 = ((unsigned long long)g.part_T[p] + 63ull) / 64ull;
      bytes += words64 * 8ull + (unsigned long long)kp * 4ull;
      refbytes += words64 * 64ull + (unsigned long long)kp * 4ull;
    }
    gcarry += kp;
    __syncthreads();
  }
  if (tid == 0) {
    st.counters[C_TOTAL] = gcarry;
    if (set_active) st.counters[C_ACTIVE] = gcarry;
    st.counters[C_BYTES] += bytes;
    st.counters[C_REFBYTES] += refbytes;
  }
}

// ------------------------------------------------------------- compaction --
// Visits every set bit of `bits` over the tiles [tile_begin, tile_begin +
// gridDim.x) in ascending slot order and calls op(p, slot, j, jg) where j is
// the bit's rank inside its partition (packed value index) and jg its rank
// over all partitions.  One warp owns 128 words; 32 words are loaded
// coalesced, warp-scanned by popcount, then expanded one word at a time so
// that lane l handles slot 32*word + l (coalesced value traffic).
template <class Op>
__global__ void __launch_bounds__(256)
    k_compact(const uint32_t* __restrict__ bits, uint32_t* clear_bits, uint32_t tile_begin, DevGraph g,
              DevState st, Op op) {
  __shared__ uint32_t s_wsum[8];
  const uint32_t t = tile_begin + blockIdx.x;
  const uint32_t p = g.tile_part[t];
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const size_t wbase = (size_t)t * K_TILE_WORDS + warp * 128;
  uint32_t x[4];
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    x[k] = __ldcg(&bits[wbase + k * 32 + lane]);
    c += __popc(x[k]);
  }
  c = warp_sum(c);
  if (lane == 0) s_wsum[warp] = c;
  __syncthreads();
  uint32_t wb = 0;
  for (uint32_t i = 0; i < warp; ++i) wb += s_wsum[i];
  uint32_t run = st.tile_off[t] + wb;
  uint32_t grun = st.tile_goff[t] + wb;
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t xc = __popc(x[k]);
    const uint32_t incl = warp_incl_scan(xc);
    const uint32_t excl = incl - xc;
    const uint32_t ctot = __shfl_sync(FULL, incl, 31);
    if (ctot) {
      for (int j = 0; j < 32; ++j) {
        const uint32_t wj = __shfl_sync(FULL, x[k], j);
        if (wj == 0) continue;
        const uint32_t ej = __shfl_sync(FULL, excl, j);
        if ((wj >> lane) & 1u) {
          const uint32_t r = ej + __popc(wj & lt);
          const uint32_t slot = t * K_TILE_SLOTS + (warp * 128 + k * 32 + j) * 32 + lane;
          op(g, st, p, slot, run + r, grun + r);
        }
      }
    }
    run += ctot;
    grun += ctot;
  }
  if (clear_bits) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (x[k]) clear_bits[wbase + k * 32 + lane] = 0;
  }
}

// Forward pack (compute side): packed value j of partition p is
// vertex_properties of the j-th set bit (src/GraphAlgorithm.cpp:233-235).
struct OpFwdPack {
  __device__ __forceinline__ void operator()(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                             uint32_t j, uint32_t) const {
    st.FV[g.part_base[p] + j] = st.prop[g.slot_gid[slot]];
  }
};
// Forward unpack (memory side, src/GraphAlgorithm.cpp:316-334): set() the
// slot's property (the bitvector itself is the dirty set) and append the
// slot to the active list.
struct OpFwdUnpack {
  __device__ __forceinline__ void operator()(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                             uint32_t j, uint32_t jg) const {
    st.mprop[slot] = st.FV[g.part_base[p] + j];
    st.AL[jg] = slot;
  }
};
// Fused forward pack + unpack (one pass; the wire buffer is still written).
struct OpFwdXfer {
  __device__ __forceinline__ void operator()(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                             uint32_t j, uint32_t jg) const {
    const uint32_t v = st.prop[g.slot_gid[slot]];
    st.FV[g.part_base[p] + j] = v;
    st.mprop[slot] = v;
    st.AL[jg] = slot;
  }
};
// Backward pack (memory side, src/GraphAlgorithm.cpp:388-393); PageRank
// zeroes the sent entry (vertex_updates.clear(), :674-677).
template <bool kClear>
struct OpBwdPack {
  __device__ __forceinline__ void operator()(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                             uint32_t j, uint32_t) const {
    st.BV[g.part_base[p] + j] = st.mupd[slot];
    if (kClear) st.mupd[slot] = 0;
  }
};

// Compute-side aggregate of one received value (plugin aggregate()).
template <int A>
__device__ __forceinline__ void aggregate_one(const DevState& st, uint32_t gid, uint32_t v) {
  if (A == A_PR_DELTA || A == A_PR_PULL) {
    // Partitions are aggregated by ordered launches and a gid occurs at most
    // once per partition, so this read-modify-write is race free and the
    // per-vertex summation order is partition 0, 1, ..., M-1.
    st.upd[gid] = __float_as_uint(__fadd_rn(__uint_as_float(st.upd[gid]), __uint_as_float(v)));
    set_dirty(st.UD, gid);
  } else {
    if (v < __ldcg(&st.upd[gid])) {
      const uint32_t old = atomicMin(&st.upd[gid], v);
      if (v < old) set_dirty(st.UD, gid);
    }
  }
}

template <int A>
struct OpAggregate {
  __device__ __forceinline__ void operator()(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                             uint32_t j, uint32_t) const {
    aggregate_one<A>(st, g.slot_gid[slot], st.BV[g.part_base[p] + j]);
  }
};
// Fused backward pack + aggregate.
template <int A>
struct OpBwdXfer {
  __device__ __forceinline__ void operator()(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                             uint32_t j, uint32_t) const {
    const uint32_t v = st.mupd[slot];
    st.BV[g.part_base[p] + j] = v;
    if (A == A_PR_DELTA) st.mupd[slot] = 0;
    aggregate_one<A>(st, g.slot_gid[slot], v);
  }
};

// -------------------------------------------------------------- edge map --
// One relaxation (PropertyList::minUpdate / addUpdate,
// include/DistributedGraph.hpp:103-130): the dirty bit is set when a min
// lowers the value, and always for an add.
template <int A>
__device__ __forceinline__ void relax(const DevState& st, uint32_t d, uint32_t sval, uint32_t w) {
  if (A == A_PR_DELTA) {
    atomicAdd(reinterpret_cast<float*>(st.mupd) + d, __uint_as_float(sval));
    set_dirty(st.MD, d);
  } else {
    const uint32_t cand = (A == A_SSSP_W) ? sat_add(sval, w) : sval;
    if (cand < __ldcg(&st.mupd[d])) {
      const uint32_t old = atomicMin(&st.mupd[d], cand);
      if (cand < old) set_dirty(st.MD, d);
    }
  }
}

// Source value after the per-source transform (sssp.cpp:69: prop + 1).
template <int A>
__device__ __forceinline__ uint32_t source_value(uint32_t v) {
  return A == A_SSSP_HOP ? v + 1u : v;
}

// Push edge-map over the compacted active list (gen_updates).  Each warp
// takes 32 actives, scans their degrees and walks the concatenation of their
// rows 32 edges at a time; a lane locates its source by a 5-step binary search
// over the scanned offsets, so consecutive lanes read consecutive edges.
// Rows longer than K_HUB_DEGREE are skipped here and run by k_hub_push.
template <int A>
__global__ void __launch_bounds__(256) k_push(DevGraph g, DevState st) {
  const uint64_t K = __ldcg(&st.counters[C_ACTIVE]);
  const uint32_t lane = lane_id();
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  unsigned long long scanned = 0;
  for (uint64_t c = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; c < K;
       c += warps * 32) {
    const uint64_t i = c + lane;
    uint32_t b = 0, deg = 0, sv = 0;
    if (i < K) {
      const uint32_t s = st.AL[i];
      b = __ldg(&g.row_off[s]);
      deg = __ldg(&g.row_off[s + 1]) - b;
      if (deg > K_HUB_DEGREE) deg = 0;
      sv = source_value<A>(st.mprop[s]);
    }
    const uint32_t incl = warp_incl_scan(deg);
    const uint32_t excl = incl - deg;
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    scanned += total;
    for (uint32_t e0 = 0; e0 < total; e0 += 32) {
      const uint32_t eid = e0 + lane;
      uint32_t lo = 0;
#pragma unroll
      for (uint32_t step = 16; step; step >>= 1) {
        const uint32_t cand = lo + step;
        const uint32_t xe = __shfl_sync(FULL, excl, cand & 31);
        if (cand < 32 && xe <= eid) lo = cand;
      }
      const uint32_t sb = __shfl_sync(FULL, b, lo);
      const uint32_t se = __shfl_sync(FULL, excl, lo);
      const uint32_t ssv = __shfl_sync(FULL, sv, lo);
      if (eid < total) {
        const uint32_t e = sb + (eid - se);
        const uint32_t d = __ldg(&g.col[e]);
        const uint32_t w = (A == A_SSSP_W) ? __ldg(&g.wgt[e]) : 0u;
        relax<A>(st, d, ssv, w);
      }
    }
  }
  if (lane == 0 && scanned) atomicAdd(&st.counters[C_EDGES], scanned);
}

// Hub rows: static work items of at most 4096 edges; a block runs an item
// when its row is active this round (bit set in the forward bitvector) and
// reads the aligned interior of the row with 128-bit loads.
template <int A>
__global__ void __launch_bounds__(256) k_hub_push(DevGraph g, DevState st) {
  unsigned long long scanned = 0;
  for (uint32_t c = blockIdx.x; c < g.num_hubs; c += gridDim.x) {
    const HubChunkD h = g.hubs[c];
    if (!test_bit(st.FB, h.slot)) continue;
    const uint32_t sv = source_value<A>(st.mprop[h.slot]);
    const uint32_t a0 = min(h.e1, (h.e0 + 3u) & ~3u);
    const uint32_t a1 = max(a0, h.e1 & ~3u);
    for (uint32_t e = h.e0 + threadIdx.x; e < a0; e += blockDim.x)
      relax<A>(st, __ldg(&g.col[e]), sv, A == A_SSSP_W ? __ldg(&g.wgt[e]) : 0u);
    const uint4* c4 = reinterpret_cast<const uint4*>(g.col);
    const uint4* w4 = reinterpret_cast<const uint4*>(g.wgt);
    for (uint32_t q = (a0 >> 2) + threadIdx.x; q < (a1 >> 2); q += blockDim.x) {
      const uint4 d = __ldg(&c4[q]);
      uint4 w = make_uint4(0, 0, 0, 0);
      if (A == A_SSSP_W) w = __ldg(&w4[q]);
      relax<A>(st, d.x, sv, w.x);
      relax<A>(st, d.y, sv, w.y);
      relax<A>(st, d.z, sv, w.z);
      relax<A>(st, d.w, sv, w.w);
    }
    for (uint32_t e = a1 + threadIdx.x; e < h.e1; e += blockDim.x)
      relax<A>(st, __ldg(&g.col[e]), sv, A == A_SSSP_W ? __ldg(&g.wgt[e]) : 0u);
    if (threadIdx.x == 0) scanned += h.e1 - h.e0;
  }
  if (threadIdx.x == 0 && scanned) atomicAdd(&st.counters[C_EDGES], scanned);
}

// ------------------------------------------------------------------ update --
// UpdateWorker::update = update_frontier() then apply_updates()
// (src/Workers.cpp:77-82), over the vertex_updates dirty set; rebuilds the
// frontier bitmap (frontier.reset() first, src/GraphAlgorithm.cpp:646),
// clears the dirty bits (clear_uv, :661) and counts |frontier|.
// PageRank: pr.cpp:123-147 then :63-88.  prev_updates is set and reset within
// the same round for every frontier vertex, so its test is always true and
// the array is not kept.  CC/SSSP: cc.cpp:86-107, sssp.cpp:92-113.
template <int A>
__global__ void __launch_bounds__(256) k_update(DevGraph g, DevState st, double tol, double damping) {
  uint32_t cnt = 0;
  for (uint32_t base = blockIdx.x * blockDim.x; base < g.V; base += gridDim.x * blockDim.x) {
    const uint32_t v = base + threadIdx.x;
    uint32_t nf = 0;
    if (v < g.V && test_bit(st.UD, v)) {
      if (A == A_PR_DELTA) {
        const float u = __uint_as_float(st.upd[v]);
        if ((double)u > tol) {
          nf = 1;
          st.ranks[v] = __fadd_rn(st.ranks[v], u);
          st.prop[v] = __float_as_uint((float)(damping * (double)u / (double)g.outdeg[v]));
          st.upd[v] = 0;
        }
      } else {
        const uint32_t u = st.upd[v];
        if (st.prop[v] > u) {
          st.prop[v] = u;
          nf = 1;
        }
      }
    }
    const uint32_t m = __ballot_sync(FULL, nf);
    if (lane_id() == 0 && v < g.V) {  // v is the first gid of this word
      st.F[v >> 5] = m;
      st.UD[v >> 5] = 0;
      cnt += __popc(m);
    }
  }
  cnt = block_sum(cnt);
  if (threadIdx.x == 0 && cnt) atomicAdd(&st.counters[C_FRONTIER], (unsigned long long)cnt);
}

}  // namespace grd
