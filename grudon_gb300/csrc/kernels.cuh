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
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace grd {

enum ListCounter : int { L_DL = 0, L_UL = 1, L_FL = 2, NUM_LIST_COUNTERS = 4 };

constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr uint32_t K_TILE_SLOTS = 8192;
constexpr uint32_t K_TILE_WORDS = K_TILE_SLOTS / 32;
constexpr uint32_t K_HUB_DEGREE = 2048;

enum Algo : int { A_PR_DELTA = 0, A_PR_PULL = 1, A_CC = 2, A_SSSP_HOP = 3, A_SSSP_W = 4 };

enum Counter : int {
  C_FRONTIER = 0,  // |frontier| after update
  C_ACTIVE = 1,    // actives unpacked by the last forward sync (all partitions)
  C_EDGES = 2,     // cumulative edges scanned
  C_BYTES = 3,     // cumulative wire bytes (true size)
  C_REFBYTES = 4,  // cumulative bytes by the reference's accounting
  C_RESID = 5,     // PR_PULL: L1 residual of the last iteration (FP64 bits)
  C_ERR = 6,       // first device-side error code (0 = none)
  C_PULL_EDGES = 7,
  C_MEDGES = 8,    // edges of the load-balanced push this round (non-hub rows)
  C_ROUNDS = 9,         // device-driven loop: rounds run
  C_PUSH_ROUNDS = 10,   // device-driven loop: rounds that pushed
  C_PULL_ROUNDS = 11,   // device-driven loop: rounds that pulled
  C_ACTIVE_TOTAL = 12,  // device-driven loop: sum of C_ACTIVE over rounds
  C_MODE = 13,          // edge-map mode chosen for the current round
  C_LAUNCHES = 14,      // device-driven loop: kernels launched
  C_PUSH_ACTIVES = 15,  // device-driven loop: C_ACTIVE summed over push rounds
  // Shape of the frontier left by the last update (round-policy inputs).
  C_FEDGES = 16,     // out-edges of the frontier (sum of global out-degrees)
  C_FMAXDEG = 17,    // largest out-degree in the frontier
  C_UNVISITED = 18,  // SSSP: out-edges of vertices not reached yet
  C_DONE = 19,       // finished-block count of k_update_list (last-block reset)
  C_VERIFY = 20,     // [4] grd_verify accumulators
  C_NOOFF_ROUNDS = 24,  // device-driven loop: rounds run NO_OFFLOAD
  NUM_COUNTERS = 26
};

struct HubChunkD {
  uint32_t slot, e0, e1;
};

struct DevGraph {
  uint32_t V, M;
  uint64_t S;
  uint64_t E;
  // Wire size of the bitvectors of one sync pass (one per memory partition):
  // true bytes, and the reference's count (MPI_UINT64_T elements x 8).
  unsigned long long bv_bytes, bv_refbytes;
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
  uint32_t* snap;  // [S] mupd as of its last send (dense-mode dirty detection)
  uint32_t* FB;
  uint32_t* FV;
  uint32_t* MD;
  uint32_t* BV;
  uint32_t* AL;
  uint32_t* tile_cnt;     // set bits per compaction tile of the bitvector being compacted
  uint32_t* tile_deg;     // [T] capped out-degrees of each tile's actives (push, bitvector form)
  uint32_t* warp_deg;     // [8T] the same per 1024-slot warp range
  uint32_t* DP;           // [S+1] exclusive degree prefix over the active list
  uint32_t* RB;           // [S] row start of each active (active-list order)
  uint32_t* SV;           // [S] property of each active (active-list order)
  uint32_t* chunk_start;  // [E/256+2] first active of each 256-edge chunk
  uint32_t* blk_sum;      // [LBS blocks]
  // Sparse-list sync (list-format rounds): the frontier as a gid list, the
  // memory-side dirty slots and the compute-side updated gids as lists.
  uint32_t* FL;           // [V] frontier gids (valid after every update)
  uint32_t* DL;           // [S] dirty slots of the current round
  uint32_t* UL;           // [V] gids whose vertex_updates changed this round
  uint32_t* own_slot;     // [V] gid -> its owned global slot
  uint32_t* lc;           // [4] list lengths: L_DL, L_UL, L_FL
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

// Appends value to list with one counter update per group of converged
// lanes (warp-aggregated atomic).
__device__ __forceinline__ void list_append(uint32_t* list, uint32_t* counter, uint32_t value) {
  namespace cg = cooperative_groups;
  cg::coalesced_group grp = cg::coalesced_threads();
  uint32_t base = 0;
  if (grp.thread_rank() == 0) base = atomicAdd(counter, grp.size());
  base = grp.shfl(base, 0);
  list[base + grp.thread_rank()] = value;
}

// Sets bit i of bm; the lane that sets it first appends i to list.
__device__ __forceinline__ void mark_listed(uint32_t* bm, uint32_t i, uint32_t* list, uint32_t* counter) {
  const uint32_t bit = 1u << (i & 31);
  uint32_t* w = bm + (i >> 5);
  if (__ldcg(w) & bit) return;
  if (atomicOr(w, bit) & bit) return;
  list_append(list, counter, i);
}

// Block-aggregated append of up to N flagged values per thread; every
// thread of the block calls it (block-uniform control flow).  One counter
// update per block and call.
template <int N>
__device__ __forceinline__ void block_append_n(uint32_t* list, uint32_t* counter, const bool (&flag)[N],
                                               const uint32_t (&value)[N]) {
  __shared__ uint32_t s_ws[32];
  __shared__ uint32_t s_b;
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  uint32_t cnt = 0;
#pragma unroll
  for (int k = 0; k < N; ++k) cnt += flag[k] ? 1u : 0u;
  const uint32_t incl = warp_incl_scan(cnt);
  if (lane == 31) s_ws[w] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t nw = (blockDim.x + 31) >> 5;
    uint32_t t = 0;
    for (uint32_t k = 0; k < nw; ++k) {
      const uint32_t c = s_ws[k];
      s_ws[k] = t;
      t += c;
    }
    s_b = t ? atomicAdd(counter, t) : 0u;
  }
  __syncthreads();
  uint32_t pos = s_b + s_ws[w] + incl - cnt;
#pragma unroll
  for (int k = 0; k < N; ++k)
    if (flag[k]) list[pos++] = value[k];
  __syncthreads();
}

// Sets bit i of bm; true for the thread that set it.
__device__ __forceinline__ bool claim_bit(uint32_t* bm, uint32_t i) {
  const uint32_t bit = 1u << (i & 31);
  uint32_t* w = bm + (i >> 5);
  if (__ldcg(w) & bit) return false;
  return !(atomicOr(w, bit) & bit);
}

__device__ __forceinline__ uint32_t block_max(uint32_t v) {
  __shared__ uint32_t s_mx[32];
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
#pragma unroll
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o));
  __syncthreads();
  if (lane == 0) s_mx[w] = v;
  __syncthreads();
  const uint32_t nw = (blockDim.x + 31) >> 5;
  uint32_t r = lane < nw ? s_mx[lane] : 0;
#pragma unroll
  for (int o = 16; o; o >>= 1) r = max(r, __shfl_xor_sync(FULL, r, o));
  return r;
}

// Block-aggregated append: every thread of the block calls it (block-uniform
// control flow); the threads whose flag is set append their value.  One
// counter update per block and call.
__device__ __forceinline__ void block_append(uint32_t* list, uint32_t* counter, bool flag, uint32_t value) {
  __shared__ uint32_t s_wc[32];
  __shared__ uint32_t s_base;
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  const uint32_t m = __ballot_sync(FULL, flag);
  if (lane == 0) s_wc[w] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t nw = (blockDim.x + 31) >> 5;
    uint32_t t = 0;
    for (uint32_t k = 0; k < nw; ++k) {
      const uint32_t c = s_wc[k];
      s_wc[k] = t;
      t += c;
    }
    s_base = t ? atomicAdd(counter, t) : 0u;
  }
  __syncthreads();
  if (flag) list[s_base + s_wc[w] + __popc(m & ((1u << lane) - 1u))] = value;
  __syncthreads();  // s_wc / s_base are reused by the next call
}

// Warp-aggregated append of up to N flagged values per lane; every lane of
// the warp calls it.  One counter update per warp and call.
template <int N>
__device__ __forceinline__ void warp_append_n(uint32_t* list, uint32_t* counter, const bool (&flag)[N],
                                              const uint32_t (&value)[N]) {
  uint32_t cnt = 0;
#pragma unroll
  for (int k = 0; k < N; ++k) cnt += flag[k] ? 1u : 0u;
  const uint32_t incl = warp_incl_scan(cnt);
  const uint32_t tot = __shfl_sync(FULL, incl, 31);
  if (tot == 0) return;
  uint32_t base = 0;
  if (lane_id() == 31) base = atomicAdd(counter, tot);
  uint32_t pos = __shfl_sync(FULL, base, 31) + incl - cnt;
#pragma unroll
  for (int k = 0; k < N; ++k)
    if (flag[k]) list[pos++] = value[k];
}

// ------------------------------------------------------------------- init --
// Reference init(): pr.cpp:20-61, cc.cpp:18-40, sssp.cpp:18-47.  Also lists
// the frontier and records its shape (count, out-edges, largest degree, and
// for SSSP the out-edges not reached yet).  Block-uniform loop: every thread
// of a block runs the same iterations (block-aggregated list appends).
template <int A>
__global__ void __launch_bounds__(256) k_init(DevGraph g, DevState st, uint32_t source, double damping) {
  constexpr int U = 4;  // elements per thread per step; one list append per block and step
  const uint64_t n = g.S > g.V ? g.S : g.V;
  uint32_t fcount = 0, fedges = 0, fmax = 0, unvis = 0;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x * U; b < n; b += (uint64_t)gridDim.x * blockDim.x * U) {
    bool fb[U];
    uint32_t ids[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t i = b + (uint64_t)u * blockDim.x + threadIdx.x;  // a warp takes 32 consecutive ids
      ids[u] = (uint32_t)i;
      uint32_t fbit = 0;
      if (i < g.V) {
        const uint32_t v = (uint32_t)i;
        const uint32_t deg = g.outdeg[v];
        if (A == A_CC) {
          st.prop[v] = v;
          st.upd[v] = 0xFFFFFFFFu;
          fbit = 1;
        } else if (A == A_SSSP_HOP || A == A_SSSP_W) {
          const uint32_t x = (v == source) ? 0u : 0xFFFFFFFFu;
          st.prop[v] = x;
          st.upd[v] = x;
          fbit = (v == source);
          if (!fbit) unvis += deg;
        } else {  // PageRank (delta and pull share the initial state)
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
        if (fbit) {
          fedges += deg;
          fmax = max(fmax, deg);
        }
      }
      fb[u] = fbit != 0;
      const uint32_t m = __ballot_sync(FULL, fbit);
      if (lane_id() == 0 && i < g.V) {  // i is the first gid of its word
        st.F[i >> 5] = m;
        st.UD[i >> 5] = 0;
        fcount += __popc(m);
      }
      if (i < g.S) {
        const uint32_t x = (A == A_PR_DELTA || A == A_PR_PULL) ? 0u : 0xFFFFFFFFu;
        st.mprop[i] = x;
        st.mupd[i] = x;
        st.snap[i] = x;
        if ((i & 31) == 0) {
          st.FB[i >> 5] = 0;
          st.MD[i >> 5] = 0;
        }
      }
    }
    block_append_n<U>(st.FL, st.lc + L_FL, fb, ids);
  }
  // one counter update per block
  fcount = block_sum(fcount);
  fedges = block_sum(fedges);
  unvis = block_sum(unvis);
  fmax = block_max(fmax);
  if (threadIdx.x == 0) {
    if (fcount) atomicAdd(&st.counters[C_FRONTIER], (unsigned long long)fcount);
    if (fedges) atomicAdd(&st.counters[C_FEDGES], (unsigned long long)fedges);
    if (unvis) atomicAdd(&st.counters[C_UNVISITED], (unsigned long long)unvis);
    if (fmax) atomicMax(&st.counters[C_FMAXDEG], (unsigned long long)fmax);
  }
}

// ---------------------------------------------------- forward sync: bits --
// Compute side of src/GraphAlgorithm.cpp:199-246: every frontier vertex sets
// the bit of its owned slot in its mirror partition's bitvector.  One warp
// builds one 32-bit word by ballot over 32 consecutive slots; the per-tile
// popcount feeds the compaction scan.  A round starts here (bitvector
// rounds), so block 0 also clears the per-round counters and the lists the
// update of this round rebuilds (nothing reads them before the update).
__device__ __forceinline__ void reset_round_counters(const DevState& st) {
  st.counters[C_FRONTIER] = 0;
  st.counters[C_FEDGES] = 0;
  st.counters[C_FMAXDEG] = 0;
}

//
// Warp w of the block builds the words of slots [w*1024, w*1024+1024) of its
// tile, the same split as the compaction's warps.  kDeg (push rounds in
// bitvector form): each warp also sums the hub-capped out-degrees of its
// actives (warp_deg) and the block those of the tile (tile_deg), so that the
// compaction can place every active's degree prefix directly.
constexpr uint32_t K_WARP_SLOTS = K_TILE_SLOTS / 8;  // slots per warp of a 256-thread tile block

// Out-degree of an owned slot as the load-balanced push counts it: rows longer
// than K_HUB_DEGREE count as 0 (they run in k_hub_push).
__device__ __forceinline__ uint32_t capped_degree(const DevGraph& g, uint32_t s) {
  const uint32_t d = __ldg(&g.row_off[s + 1]) - __ldg(&g.row_off[s]);
  return d > K_HUB_DEGREE ? 0u : d;
}

template <bool kDeg>
__global__ void __launch_bounds__(256) k_fwd_bits(DevGraph g, DevState st) {
  const uint32_t t = blockIdx.x;
  if (t == 0 && threadIdx.x == 0) {
    reset_round_counters(st);
    st.counters[C_ACTIVE] = 0;  // the compaction adds each tile's actives
    st.lc[L_FL] = 0;
    st.lc[L_UL] = 0;  // the bitvector update consumes every dirty bit
  }
  const uint32_t p = g.tile_part[t];
  const uint32_t base = g.part_base[p], nown = g.part_owned[p];
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  const uint32_t w0 = t * K_TILE_SLOTS + w * K_WARP_SLOTS;
  constexpr int U = 4;  // independent gathers in flight per thread
  uint32_t cnt = 0, deg = 0;
  for (uint32_t i = lane; i < K_WARP_SLOTS; i += 32 * U) {
    uint32_t gid[U], fw[U], bit[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t s = w0 + i + u * 32;
      gid[u] = (s - base < nown) ? __ldg(&g.slot_gid[s]) : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) fw[u] = gid[u] != 0xFFFFFFFFu ? st.F[gid[u] >> 5] : 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t s = w0 + i + u * 32;
      bit[u] = gid[u] != 0xFFFFFFFFu ? (fw[u] >> (gid[u] & 31)) & 1u : 0u;
      const uint32_t m = __ballot_sync(FULL, bit[u]);
      if (lane == 0) {
        st.FB[s >> 5] = m;
        cnt += __popc(m);
      }
    }
    if (kDeg) {
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (bit[u]) deg += capped_degree(g, w0 + i + u * 32);
    }
  }
  cnt = block_sum(cnt);
  if (threadIdx.x == 0) st.tile_cnt[t] = cnt;
  if (kDeg) {  // deg is still this lane's own sum: block_sum adds over all lanes
    const uint32_t wdeg = warp_sum(deg);
    if (lane == 0) st.warp_deg[t * 8 + w] = wdeg;
    deg = block_sum(deg);
    if (threadIdx.x == 0) st.tile_deg[t] = deg;
  }
}

// Per-tile set-bit count of a bitvector (backward sync).  `zero`, when
// given, is another bitvector whose words of this tile are cleared (the
// forward bitvector, no longer read once the edge-map has run).
static __global__ void __launch_bounds__(256) k_tile_count(const uint32_t* __restrict__ bits, uint32_t* tile_cnt,
                                                           uint32_t* zero = nullptr) {
  const uint32_t t = blockIdx.x;
  const uint32_t* w = bits + (size_t)t * K_TILE_WORDS;
  uint32_t c = 0;
  for (uint32_t i = threadIdx.x; i < K_TILE_WORDS; i += blockDim.x) {
    c += __popc(w[i]);
    if (zero) zero[(size_t)t * K_TILE_WORDS + i] = 0;
  }
  c = block_sum(c);
  if (threadIdx.x == 0) tile_cnt[t] = c;
}

// ------------------------------------------------------------- compaction --
// Fire-and-forget reductions (no returned value, so no round trip).
__device__ __forceinline__ void red_or(uint32_t* a, uint32_t v) {
  asm volatile("red.global.or.b32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void red_min(uint32_t* a, uint32_t v) {
  asm volatile("red.global.min.u32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void red_add_f32(float* a, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(a), "f"(v) : "memory");
}

// Visits every set bit of `bits` over the tiles [tile_begin, tile_begin +
// gridDim.x) in ascending slot order with j = the bit's rank inside its
// partition (packed value index) and jg = its rank over all partitions.
// Each block first sums the set-bit counts of the tiles before its own
// (st.tile_cnt, from the kernel that produced the bitvector): a few hundred
// L2 reads per block instead of a separate one-block scan launch.
// `count` adds this sync pass's wire bytes to the statistics (1), and also
// the actives of a forward pass to C_ACTIVE (2); 0 for the second half of a
// split pass.
// Phase A: each of the 8 warps loads its K_TILE_WORDS/8 words (coalesced),
// scans their popcounts and writes the slot of every set bit to a warp-private
// shared buffer in rank order (shuffles and shared stores only).  Phase B:
// lanes walk the buffer 32 apart, U = 4 items per lane at a time, issuing all
// loads of an item group (Op::gather) before any store (Op::scatter), so each
// lane keeps 4 independent memory chains in flight.
struct Payload {
  uint32_t v, gid, cur, cmp;
};

// Phase A's second half: the warp's words x[k] (word index wbase + 32k +
// lane) become the slots of their set bits in `buf`, in ascending order;
// returns how many.
template <int KW>
__device__ __forceinline__ uint32_t collect_set_bits(const uint32_t (&x)[KW], size_t wbase, uint32_t* buf) {
  const uint32_t lane = lane_id(), lt = (1u << lane) - 1u;
  uint32_t n = 0;
#pragma unroll
  for (int k = 0; k < KW; ++k) {
    const uint32_t xc = __popc(x[k]);
    const uint32_t incl = warp_incl_scan(xc);
    const uint32_t excl = incl - xc;
    const uint32_t ctot = __shfl_sync(FULL, incl, 31);
    if (ctot) {
      for (int j = 0; j < 32; ++j) {
        const uint32_t wj = __shfl_sync(FULL, x[k], j);
        if (wj == 0) continue;
        const uint32_t ej = __shfl_sync(FULL, excl, j);
        if ((wj >> lane) & 1u) buf[n + ej + __popc(wj & lt)] = (uint32_t)(wbase + k * 32 + j) * 32 + lane;
      }
    }
    n += ctot;
  }
  __syncwarp();
  return n;
}

template <class Op>
__global__ void __launch_bounds__(256)
    k_compact(const uint32_t* __restrict__ bits, uint32_t* clear_bits, uint32_t tile_begin, DevGraph g,
              DevState st, Op op, int count) {
  constexpr int KW = K_TILE_WORDS / 256;  // 32-word groups per warp
  constexpr int CAP = 32 * 32 * KW;       // slots owned by one warp
  constexpr int U = 4;
  __shared__ uint32_t s_wsum[8];
  __shared__ uint32_t s_slot[8][CAP];
  const uint32_t t = tile_begin + blockIdx.x;
  const uint32_t p = g.tile_part[t];
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  uint32_t pre_p = 0, pre_g = 0;  // set bits before this tile: in its partition, in all
  {
    const uint32_t t0 = g.part_base[p] / K_TILE_SLOTS;
    for (uint32_t i = threadIdx.x; i < t; i += blockDim.x) {
      const uint32_t c = __ldcg(&st.tile_cnt[i]);
      pre_g += c;
      if (i >= t0) pre_p += c;
    }
    pre_p = block_sum(pre_p);
    pre_g = block_sum(pre_g);
  }
  const size_t wbase = (size_t)t * K_TILE_WORDS + warp * (32 * KW);
  uint32_t x[KW];
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < KW; ++k) {
    x[k] = __ldcg(&bits[wbase + k * 32 + lane]);
    c += __popc(x[k]);
  }
  c = warp_sum(c);
  if (lane == 0) s_wsum[warp] = c;
  __syncthreads();
  uint32_t wb = 0;
  for (uint32_t i = 0; i < warp; ++i) wb += s_wsum[i];
  const uint32_t run = pre_p + wb;
  const uint32_t grun = pre_g + wb;
  if (count && threadIdx.x == 0) {
    uint32_t ct = 0;
    for (int i = 0; i < 8; ++i) ct += s_wsum[i];
    // every partition's bitvector once per pass, plus 4 B per packed value
    unsigned long long b = 4ull * ct, rb = 4ull * ct;
    if (t == 0) b += g.bv_bytes, rb += g.bv_refbytes;
    if (b) atomicAdd(&st.counters[C_BYTES], b);
    if (rb) atomicAdd(&st.counters[C_REFBYTES], rb);
    if (count == 2 && ct) atomicAdd(&st.counters[C_ACTIVE], (unsigned long long)ct);
  }
  uint32_t* buf = s_slot[warp];
  const uint32_t n = collect_set_bits(x, wbase, buf);
  for (uint32_t q0 = 0; q0 < n; q0 += 32 * U) {
    uint32_t sl[U];
    Payload pv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t q = q0 + u * 32 + lane;
      if (q < n) {
        sl[u] = buf[q];
        pv[u] = op.gather(g, st, p, sl[u], run + q);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t q = q0 + u * 32 + lane;
      if (q < n) op.scatter(g, st, p, sl[u], run + q, grun + q, pv[u]);
    }
  }
  if (clear_bits) {
#pragma unroll
    for (int k = 0; k < KW; ++k)
      if (x[k]) clear_bits[wbase + k * 32 + lane] = 0;
  }
}

// Forward pack (compute side): packed value j of partition p is
// vertex_properties of the j-th set bit (src/GraphAlgorithm.cpp:233-235).
struct OpFwdPack {
  __device__ __forceinline__ Payload gather(const DevGraph& g, const DevState& st, uint32_t, uint32_t slot,
                                            uint32_t) const {
    return Payload{st.prop[__ldg(&g.slot_gid[slot])], 0, 0};
  }
  __device__ __forceinline__ void scatter(const DevGraph& g, const DevState& st, uint32_t p, uint32_t, uint32_t j,
                                          uint32_t, const Payload& v) const {
    st.FV[g.part_base[p] + j] = v.v;
  }
};
// Forward unpack (memory side, src/GraphAlgorithm.cpp:316-334): set() the
// slot's property (the bitvector itself is the dirty set) and append the
// slot to the active list.
struct OpFwdUnpack {
  __device__ __forceinline__ Payload gather(const DevGraph& g, const DevState& st, uint32_t p, uint32_t,
                                            uint32_t j) const {
    return Payload{st.FV[g.part_base[p] + j], 0, 0};
  }
  __device__ __forceinline__ void scatter(const DevGraph&, const DevState& st, uint32_t, uint32_t slot, uint32_t,
                                          uint32_t jg, const Payload& v) const {
    st.mprop[slot] = v.v;
    st.AL[jg] = slot;
  }
};
// Fused forward pack + unpack (one pass): the value goes straight from the
// compute side to the memory-side slot; the packed wire buffer, which only
// carries values between the separate pack and unpack stages, is skipped.
struct OpFwdXfer {
  __device__ __forceinline__ Payload gather(const DevGraph& g, const DevState& st, uint32_t, uint32_t slot,
                                            uint32_t) const {
    return Payload{st.prop[__ldg(&g.slot_gid[slot])], 0, 0};
  }
  __device__ __forceinline__ void scatter(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                          uint32_t, uint32_t jg, const Payload& v) const {
    st.mprop[slot] = v.v;
    st.AL[jg] = slot;
  }
};

// Backward pack (memory side, src/GraphAlgorithm.cpp:388-393); PageRank
// zeroes the sent entry (vertex_updates.clear(), :674-677); the min
// algorithms record the sent value as the dirty-detection snapshot.
template <int A>
__device__ __forceinline__ void retire_update(const DevState& st, uint32_t slot, uint32_t v) {
  if (A == A_PR_DELTA)
    st.mupd[slot] = 0;
  else
    st.snap[slot] = v;
}

template <int A>
struct OpBwdPack {
  __device__ __forceinline__ Payload gather(const DevGraph&, const DevState& st, uint32_t, uint32_t slot,
                                            uint32_t) const {
    return Payload{st.mupd[slot], 0, 0};
  }
  __device__ __forceinline__ void scatter(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                          uint32_t j, uint32_t, const Payload& v) const {
    st.BV[g.part_base[p] + j] = v.v;
    retire_update<A>(st, slot, v.v);
  }
};

// Compute-side aggregate of one received value (plugin aggregate()) in a
// bitvector round: PageRank addUpdate, CC/SSSP minUpdate.  No dirty bit: the
// bitvector round's update (k_update) tests every vertex, and its test is
// false for every vertex whose entry this round left unchanged.
template <int A>
__device__ __forceinline__ void aggregate_one(const DevState& st, uint32_t gid, uint32_t v, uint32_t cur) {
  if (A == A_PR_DELTA || A == A_PR_PULL) {
    // Partitions are aggregated by ordered launches and a gid occurs at most
    // once per partition, so this read-modify-write is race free and the
    // per-vertex summation order is partition 0, 1, ..., M-1.
    st.upd[gid] = __float_as_uint(__fadd_rn(__uint_as_float(cur), __uint_as_float(v)));
  } else if (v < cur) {
    red_min(st.upd + gid, v);
  }
}

template <int A>
__device__ __forceinline__ uint32_t aggregate_peek(const DevState& st, uint32_t gid) {
  return (A == A_PR_DELTA || A == A_PR_PULL) ? st.upd[gid] : __ldcg(&st.upd[gid]);
}

template <int A>
struct OpAggregate {
  __device__ __forceinline__ Payload gather(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                            uint32_t j) const {
    const uint32_t gid = __ldg(&g.slot_gid[slot]);
    return Payload{st.BV[g.part_base[p] + j], gid, aggregate_peek<A>(st, gid)};
  }
  __device__ __forceinline__ void scatter(const DevGraph&, const DevState& st, uint32_t, uint32_t, uint32_t,
                                          uint32_t, const Payload& v) const {
    aggregate_one<A>(st, v.gid, v.v, v.cur);
  }
};
// Fused backward pack + aggregate (no wire buffer, as OpFwdXfer).
template <int A>
struct OpBwdXfer {
  __device__ __forceinline__ Payload gather(const DevGraph& g, const DevState& st, uint32_t, uint32_t slot,
                                            uint32_t) const {
    const uint32_t gid = __ldg(&g.slot_gid[slot]);
    return Payload{st.mupd[slot], gid, aggregate_peek<A>(st, gid)};
  }
  __device__ __forceinline__ void scatter(const DevGraph&, const DevState& st, uint32_t, uint32_t slot, uint32_t,
                                          uint32_t, const Payload& v) const {
    retire_update<A>(st, slot, v.v);
    aggregate_one<A>(st, v.gid, v.v, v.cur);
  }
};

// Host-supplied (gid, value) pairs (grd_aggregate_values).  A gid may repeat
// within one call, so PageRank adds atomically here.
template <int A>
__global__ void __launch_bounds__(256) k_aggregate_values(DevState st, const uint32_t* gids, const uint32_t* vals,
                                                          uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t gid = gids[i], v = vals[i];
    if (A == A_PR_DELTA || A == A_PR_PULL) {
      atomicAdd(reinterpret_cast<float*>(st.upd) + gid, __uint_as_float(v));
      mark_listed(st.UD, gid, st.UL, st.lc + L_UL);
    } else {
      const uint32_t old = atomicMin(&st.upd[gid], v);
      if (v < old) mark_listed(st.UD, gid, st.UL, st.lc + L_UL);
    }
  }
}

// -------------------------------------------------------------- edge map --
// Relaxation (PropertyList::minUpdate / addUpdate,
// include/DistributedGraph.hpp:103-130): the dirty bit is set when a min
// lowers the value, and always for an add.  `cur` is a prior read of
// mupd[d] (a stale read is only ever larger, values never grow in a round).
//
// Dense form (bitvector rounds): reductions only; the dirty set is rebuilt
// afterwards by k_diff_dirty.
template <int A>
__device__ __forceinline__ void relax_dense(const DevState& st, uint32_t d, uint32_t cand, uint32_t cur) {
  if (A == A_PR_DELTA)
    red_add_f32(reinterpret_cast<float*>(st.mupd) + d, __uint_as_float(cand));
  else if (cand < cur)
    red_min(st.mupd + d, cand);
}

// Sparse form (list rounds), N edges per lane (d = 0xFFFFFFFF: none): all N
// returning atomics are issued before any result is used, then every lowered
// slot (PageRank: every touched slot) claims its dirty bit; nd[k] is set for
// the one thread that claimed it, so each dirty slot is listed once.
template <int A, int N>
__device__ __forceinline__ void relax_sparse(const DevState& st, const uint32_t (&d)[N], const uint32_t (&cand)[N],
                                             const uint32_t (&cur)[N], bool (&nd)[N]) {
  bool low[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    low[k] = false;
    if (d[k] == 0xFFFFFFFFu) continue;
    if (A == A_PR_DELTA) {
      red_add_f32(reinterpret_cast<float*>(st.mupd) + d[k], __uint_as_float(cand[k]));
      low[k] = true;
    } else if (cand[k] < cur[k]) {
      low[k] = cand[k] < atomicMin(&st.mupd[d[k]], cand[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < N; ++k) nd[k] = low[k] && claim_bit(st.MD, d[k]);
}

template <int A>
__device__ __forceinline__ uint32_t relax_cand(uint32_t sval, uint32_t w) {
  return A == A_SSSP_W ? sat_add(sval, w) : sval;
}

template <int A>
__device__ __forceinline__ uint32_t relax_peek(const DevState& st, uint32_t d) {
  return A == A_PR_DELTA ? 0u : __ldcg(&st.mupd[d]);
}

// Source value after the per-source transform (sssp.cpp:69: prop + 1).
template <int A>
__device__ __forceinline__ uint32_t source_value(uint32_t v) {
  return A == A_SSSP_HOP ? v + 1u : v;
}

// NO_OFFLOAD relaxation (src/GraphAlgorithm.cpp:582-637): the compute
// partition applies the algorithm's own update for each shipped edge straight
// to its vertex_updates (gid index) — the minUpdate / addUpdate that the
// memory-side gen_updates and the compute-side aggregate would apply in two
// steps — so the dirty set is that of the aggregate: a gid whose entry
// lowered (PageRank: received anything).  d[k] holds gids (0xFFFFFFFF:
// none); nd[k] is set for the one thread that claimed the gid's dirty bit.
template <int A>
__device__ __forceinline__ uint32_t relax_peek_gid(const DevState& st, uint32_t v) {
  return A == A_PR_DELTA ? 0u : __ldcg(&st.upd[v]);
}

template <int A, int N>
__device__ __forceinline__ void relax_compute(const DevState& st, const uint32_t (&d)[N],
                                              const uint32_t (&cand)[N], const uint32_t (&cur)[N], bool (&nd)[N]) {
  bool low[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    low[k] = false;
    if (d[k] == 0xFFFFFFFFu) continue;
    if (A == A_PR_DELTA) {
      red_add_f32(reinterpret_cast<float*>(st.upd) + d[k], __uint_as_float(cand[k]));
      low[k] = true;
    } else if (cand[k] < cur[k]) {
      low[k] = cand[k] < atomicMin(&st.upd[d[k]], cand[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < N; ++k) nd[k] = low[k] && claim_bit(st.UD, d[k]);
}

// ---- load-balanced push (gen_updates over the compacted active list) ------
// The edge-map runs in two steps so that every warp gets the same number of
// edges whatever the degree skew: (1) per-block sums of the (hub-capped)
// degrees of the active list, (2) each block adds up the sums before its own
// and writes the exclusive degree prefix DP[i] of its actives and, for every
// 256-edge chunk boundary that falls inside a row, the chunk's first active
// (chunk_start).  k_push_lbs then hands one 256-edge chunk to a warp.
// Rows longer than K_HUB_DEGREE count as 0 here and run in k_hub_push.
constexpr uint32_t LBS_CHUNK = 256;

// Fixed grid: block b owns actives [b*seg, min(K,(b+1)*seg)), seg = ceil(K/B).
__device__ __forceinline__ void lbs_segment(uint64_t K, uint32_t& b0, uint32_t& b1) {
  const uint64_t seg = (K + gridDim.x - 1) / gridDim.x;
  const uint64_t a = (uint64_t)blockIdx.x * seg;
  b0 = (uint32_t)(a < K ? a : K);
  b1 = (uint32_t)(a + seg < K ? a + seg : K);
}

static __global__ void __launch_bounds__(256) k_deg_reduce(DevGraph g, DevState st) {
  const uint64_t K = __ldcg(&st.counters[C_ACTIVE]);
  uint32_t b0, b1;
  lbs_segment(K, b0, b1);
  uint32_t sum = 0;
  for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) sum += capped_degree(g, st.AL[i]);
  sum = block_sum(sum);
  if (threadIdx.x == 0) st.blk_sum[blockIdx.x] = sum;
}

// Push rounds in list form: the forward sync from the frontier list
// (k_fwd_list) and the first degree pass (k_deg_reduce) in one kernel over
// the same segments of the list (its length is known from the last update).
static __global__ void __launch_bounds__(256) k_fwd_list_deg(DevGraph g, DevState st) {
  const uint32_t K = __ldcg(&st.lc[L_FL]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st.counters[C_ACTIVE] = K;
    st.counters[C_BYTES] += g.bv_bytes + 4ull * K;
    st.counters[C_REFBYTES] += g.bv_refbytes + 4ull * K;
    reset_round_counters(st);
    st.lc[L_DL] = 0;
  }
  uint32_t b0, b1;
  lbs_segment(K, b0, b1);
  uint32_t sum = 0;
  for (uint32_t j = b0 + threadIdx.x; j < b1; j += blockDim.x) {
    const uint32_t gid = st.FL[j];
    const uint32_t s = st.own_slot[gid];
    st.AL[j] = s;
    st.mprop[s] = st.prop[gid];
    atomicOr(&st.FB[s >> 5], 1u << (s & 31));
    sum += capped_degree(g, s);
  }
  sum = block_sum(sum);
  if (threadIdx.x == 0) st.blk_sum[blockIdx.x] = sum;
}

// Each block first sums the degree totals of the blocks before it (a few
// hundred L2 reads: no separate scan launch); the last block records the
// round's edge total m (C_MEDGES, and DP[K]).
static __global__ void __launch_bounds__(256) k_deg_down(DevGraph g, DevState st) {
  __shared__ uint32_t s_w[8];
  const uint64_t K = __ldcg(&st.counters[C_ACTIVE]);
  uint32_t b0, b1;
  lbs_segment(K, b0, b1);
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  uint32_t run = 0;
  for (uint32_t i = threadIdx.x; i < blockIdx.x; i += blockDim.x) run += __ldcg(&st.blk_sum[i]);
  run = block_sum(run);
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    const uint32_t m = run + __ldcg(&st.blk_sum[blockIdx.x]);
    st.DP[K] = m;
    st.counters[C_MEDGES] = m;
    st.counters[C_EDGES] += m;
  }
  for (uint32_t base = b0; base < b1; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    uint32_t d = 0;
    if (i < b1) {
      const uint32_t s = st.AL[i];
      const uint32_t r0 = __ldg(&g.row_off[s]);
      d = __ldg(&g.row_off[s + 1]) - r0;
      if (d > K_HUB_DEGREE) d = 0;
      st.RB[i] = r0;                 // row start and source value in active
      st.SV[i] = st.mprop[s];        // order: one-level loads in k_push_lbs
    }
    const uint32_t incl = warp_incl_scan(d);
    if (lane == 31) s_w[w] = incl;
    __syncthreads();
    uint32_t wb = 0, tot = 0;
    for (uint32_t k = 0; k < 8; ++k) {
      const uint32_t x = s_w[k];
      if (k < w) wb += x;
      tot += x;
    }
    const uint32_t ex = run + wb + incl - d;
    if (i < b1) {
      st.DP[i] = ex;
      if (d) {
        const uint32_t c0 = (ex + LBS_CHUNK - 1) / LBS_CHUNK, c1 = (ex + d + LBS_CHUNK - 1) / LBS_CHUNK;
        for (uint32_t c = c0; c < c1; ++c) st.chunk_start[c] = i;
      }
    }
    run += tot;
    __syncthreads();
  }
}

// Forward transfer of a push round in bitvector form fused with both degree
// passes (k_deg_reduce, k_deg_down).  The active list is the compaction
// order, so the block of tile t knows where its actives start (tile_cnt of
// the tiles before it) and where their edges start (tile_deg), and warp w
// adds the warp_deg of the warps before it: every active's exclusive degree
// prefix DP, row start RB, source value SV and the chunks that start in its
// row are written here, with no scan launch and no second read of the list.
// The last tile's block records the round's edge total (DP[K], C_MEDGES).
static __global__ void __launch_bounds__(256) k_fwd_xfer_deg(DevGraph g, DevState st) {
  constexpr int KW = K_TILE_WORDS / 256;
  constexpr int CAP = 32 * 32 * KW;
  constexpr int U = 4;
  static_assert(CAP == K_WARP_SLOTS, "the compaction's warps own k_fwd_bits's warp ranges");
  __shared__ uint32_t s_wsum[8], s_wdeg[8];
  __shared__ uint32_t s_slot[8][CAP];
  const uint32_t t = blockIdx.x;
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  uint32_t pre_g = 0, pre_d = 0;  // actives and their capped edges before this tile
  for (uint32_t i = threadIdx.x; i < t; i += blockDim.x) {
    pre_g += __ldcg(&st.tile_cnt[i]);
    pre_d += __ldcg(&st.tile_deg[i]);
  }
  pre_g = block_sum(pre_g);
  pre_d = block_sum(pre_d);
  const size_t wbase = (size_t)t * K_TILE_WORDS + warp * (32 * KW);
  uint32_t x[KW];
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < KW; ++k) {
    x[k] = __ldcg(&st.FB[wbase + k * 32 + lane]);
    c += __popc(x[k]);
  }
  c = warp_sum(c);
  if (lane == 0) {
    s_wsum[warp] = c;
    s_wdeg[warp] = __ldcg(&st.warp_deg[t * 8 + warp]);
  }
  __syncthreads();
  uint32_t wb = 0, wd = 0, ct = 0, dt = 0;
  for (uint32_t i = 0; i < 8; ++i) {
    const uint32_t a = s_wsum[i], d = s_wdeg[i];
    if (i < warp) wb += a, wd += d;
    ct += a;
    dt += d;
  }
  if (threadIdx.x == 0) {
    // bitvectors once per pass, plus 4 B per packed value (k_compact's count 2)
    unsigned long long b = 4ull * ct, rb = 4ull * ct;
    if (t == 0) b += g.bv_bytes, rb += g.bv_refbytes;
    if (b) atomicAdd(&st.counters[C_BYTES], b);
    if (rb) atomicAdd(&st.counters[C_REFBYTES], rb);
    if (ct) atomicAdd(&st.counters[C_ACTIVE], (unsigned long long)ct);
    if (t == gridDim.x - 1) {
      const uint32_t m = pre_d + dt;
      st.DP[pre_g + ct] = m;
      st.counters[C_MEDGES] = m;
      st.counters[C_EDGES] += m;
    }
  }
  uint32_t* buf = s_slot[warp];
  const uint32_t n = collect_set_bits(x, wbase, buf);
  const uint32_t grun = pre_g + wb;
  uint32_t drun = pre_d + wd;  // capped edges of this warp's actives before the group
  for (uint32_t q0 = 0; q0 < n; q0 += 32 * U) {
    uint32_t sl[U], gid[U], r0[U], d[U], v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t q = q0 + u * 32 + lane;
      sl[u] = q < n ? buf[q] : 0u;
      gid[u] = q < n ? __ldg(&g.slot_gid[sl[u]]) : 0u;
      r0[u] = q < n ? __ldg(&g.row_off[sl[u]]) : 0u;
      d[u] = q < n ? __ldg(&g.row_off[sl[u] + 1]) - r0[u] : 0u;
      if (d[u] > K_HUB_DEGREE) d[u] = 0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = (q0 + u * 32 + lane) < n ? st.prop[gid[u]] : 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t q = q0 + u * 32 + lane;
      const uint32_t incl = warp_incl_scan(d[u]);
      const uint32_t ex = drun + incl - d[u];
      drun += __shfl_sync(FULL, incl, 31);
      if (q < n) {
        const uint32_t i = grun + q;
        st.mprop[sl[u]] = v[u];
        st.DP[i] = ex;
        st.RB[i] = r0[u];
        st.SV[i] = v[u];
        if (d[u]) {
          const uint32_t c0 = (ex + LBS_CHUNK - 1) / LBS_CHUNK, c1 = (ex + d[u] + LBS_CHUNK - 1) / LBS_CHUNK;
          for (uint32_t cc = c0; cc < c1; ++cc) st.chunk_start[cc] = i;
        }
      }
    }
  }
}

// One warp per 256-edge chunk.  The warp stages a window of up to LBS_WIN
// consecutive actives (their DP, and the pair row start minus DP / source
// value) in shared memory, 32 at a time with coalesced loads, only as many
// as the chunk's edges need (one group of 32 for a typical degree) — one
// window covers the whole chunk unless more than LBS_WIN actives fall inside
// it, and a chunk of that many low-degree rows takes a second window.
// The row of each of the window's edge positions comes from a mark-and-scan:
// every active with edges marks the position where its row starts, then a
// running max over the 256 positions.  Marks carry a per-warp generation
// number above the window index, so the mark array is never cleared: the
// current window always marks position 0, and its marks outrank every older
// one.  An edge then costs two shared loads (its row, then the row's edge
// base and source value as one 8-byte load), and lane l takes positions l,
// l+32, ...: one load instruction of the warp reads 32 consecutive edges,
// whose destinations (sorted within a row) share sectors.  All 8 edges of a
// lane are loaded (index, weight, current value) before any update is
// issued, keeping 8 independent memory chains in flight per lane.
// The kernel is bound by the latency of those chains, and the L1 that the
// shared memory leaves sets how many of them are in flight: 20 KB per block
// (5 blocks per SM) leaves most of the SM's 256 KB to L1; 34 KB per block
// (a 256-active window) ran 14-22 % slower, and 39-40 KB per block, which
// leaves only the minimum L1, ran 2x slower.
constexpr uint32_t LBS_WIN = 128;
constexpr int LBS_JBITS = 9;  // window index bits of a mark
static_assert(LBS_WIN <= (1u << LBS_JBITS), "window index fits its mark field");

template <int A, bool kDense, bool kCompute = false>
__global__ void __launch_bounds__(256, 5) k_push_lbs(DevGraph g, DevState st) {
  static_assert(!(kDense && kCompute), "NO_OFFLOAD rounds use the sparse form");
  constexpr int B = LBS_CHUNK / 32;
  constexpr int SW = LBS_WIN / 32;
  constexpr uint32_t GEN_MAX = (1u << (32 - LBS_JBITS)) - 1u;
  static_assert(LBS_CHUNK == 8 * 32, "each lane owns 8 consecutive edge positions");
  __shared__ uint32_t s_dp[8][LBS_WIN];   // DP of window active j
  __shared__ uint2 s_bs[8][LBS_WIN];     // its (row start - DP, source value): edge index = .x + position
  __shared__ uint32_t s_src[8][LBS_CHUNK];
  const uint32_t K = (uint32_t)__ldcg(&st.counters[C_ACTIVE]);
  const uint32_t m = (uint32_t)__ldcg(&st.counters[C_MEDGES]);
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t nchunks = (m + LBS_CHUNK - 1) / LBS_CHUNK;
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  uint32_t* dp = s_dp[w];
  uint2* bs = s_bs[w];
  uint32_t* srcs = s_src[w];
  uint32_t gen = GEN_MAX;  // the first step clears the marks
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + w; c < nchunks; c += nwarps) {
    uint32_t e = c * LBS_CHUNK;
    const uint32_t e_end = min(m, e + LBS_CHUNK);
    uint32_t i0 = st.chunk_start[c];
    while (e < e_end) {
      if (gen == GEN_MAX) {  // start (and, in principle, generation wrap): clear the marks
#pragma unroll
        for (int q = 0; q < B; ++q) srcs[B * lane + q] = 0;
        gen = 0;
      }
      ++gen;
      // Load the window 32 actives at a time, only as far as the chunk
      // needs: `cover` is the DP of the first active not loaded.
      uint32_t nw = 0, cover;
      do {
        const uint32_t idx = i0 + nw * 32 + lane;
        const uint32_t av = idx < K ? st.DP[idx] : m;
        const uint32_t bv = idx < K ? st.RB[idx] : 0u;
        const uint32_t vv = idx < K ? st.SV[idx] : 0u;
        const uint32_t nx = i0 + nw * 32 + 32;
        const uint32_t tl = (lane == 31) ? (nx < K ? st.DP[nx] : m) : 0u;
        dp[nw * 32 + lane] = av;
        bs[nw * 32 + lane] = make_uint2(bv - av, source_value<A>(vv));
        cover = __shfl_sync(FULL, tl, 31);
        ++nw;
      } while (nw < (uint32_t)SW && cover < e_end);
      const uint32_t wend = min(e_end, cover);
      __syncwarp();
      // mark: the row of window active j starts at position dp[j] - e (the
      // first active's row may start before the window: position 0).  Only
      // rows with edges mark, so no two actives share a position.
      const uint32_t tag = gen << LBS_JBITS;
#pragma unroll
      for (int k = 0; k < SW; ++k) {
        const uint32_t j = k * 32 + lane;
        if ((uint32_t)k < nw) {
          const uint32_t aj = dp[j];
          const uint32_t next = j + 1 < nw * 32 ? dp[j + 1] : cover;
          if (aj < wend && next > aj) srcs[(aj > e ? aj : e) - e] = tag | j;
        }
      }
      __syncwarp();
      // scan: running max over the positions (lane-local 8, then the warp),
      // written back as window indices
      {
        uint32_t loc[B], run = 0;
#pragma unroll
        for (int q = 0; q < B; ++q) {
          run = max(run, srcs[B * lane + q]);
          loc[q] = run;
        }
        uint32_t inc = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t n = __shfl_up_sync(FULL, inc, o);
          if (lane >= (uint32_t)o) inc = max(inc, n);
        }
        uint32_t ex = __shfl_up_sync(FULL, inc, 1);
        if (lane == 0) ex = 0;
#pragma unroll
        for (int q = 0; q < B; ++q) srcs[B * lane + q] = max(ex, loc[q]);  // the lane's own positions
      }
      __syncwarp();
      uint32_t dst[B], cand[B], cur[B];
#pragma unroll
      for (int k = 0; k < B; ++k) {
        const uint32_t eid = e + k * 32 + lane;
        dst[k] = 0xFFFFFFFFu;
        cand[k] = 0;
        if (eid < wend) {
          const uint32_t j = srcs[k * 32 + lane] & ((1u << LBS_JBITS) - 1u);
          const uint2 b = bs[j];
          const uint32_t ed = b.x + eid;
          dst[k] = __ldg(&g.col[ed]);
          cand[k] = b.y;
          if (A == A_SSSP_W) cand[k] = relax_cand<A>(cand[k], __ldg(&g.wgt[ed]));
        }
      }
      if (kCompute) {  // destination slot -> gid: the shipped adjacency holds gids
#pragma unroll
        for (int k = 0; k < B; ++k)
          if (dst[k] != 0xFFFFFFFFu) dst[k] = __ldg(&g.slot_gid[dst[k]]);
#pragma unroll
        for (int k = 0; k < B; ++k) cur[k] = dst[k] != 0xFFFFFFFFu ? relax_peek_gid<A>(st, dst[k]) : 0u;
        bool nd[B];
        relax_compute<A, B>(st, dst, cand, cur, nd);
        warp_append_n<B>(st.UL, st.lc + L_UL, nd, dst);
      } else {
#pragma unroll
        for (int k = 0; k < B; ++k) cur[k] = dst[k] != 0xFFFFFFFFu ? relax_peek<A>(st, dst[k]) : 0u;
        if (kDense) {
#pragma unroll
          for (int k = 0; k < B; ++k)
            if (dst[k] != 0xFFFFFFFFu) relax_dense<A>(st, dst[k], cand[k], cur[k]);
        } else {
          bool nd[B];
          relax_sparse<A, B>(st, dst, cand, cur, nd);
          warp_append_n<B>(st.DL, st.lc + L_DL, nd, dst);
        }
      }
      __syncwarp();
      e = wend;
      i0 += nw * 32;
    }
  }
}

// Hub rows: static work items of at most 4096 edges; a block runs an item
// when its row is active this round (bit set in the forward bitvector) and
// reads the aligned interior of the row with 128-bit loads.  All loops are
// block-uniform (the sparse form appends warp-aggregated).
template <int A, bool kDense, int N, bool kCompute = false>
__device__ __forceinline__ void hub_relax(const DevGraph& g, const DevState& st, const uint32_t (&d)[N],
                                          const uint32_t (&c)[N]) {
  uint32_t cur[N];
  if (kCompute) {
    uint32_t v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = d[k] != 0xFFFFFFFFu ? __ldg(&g.slot_gid[d[k]]) : 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < N; ++k) cur[k] = v[k] != 0xFFFFFFFFu ? relax_peek_gid<A>(st, v[k]) : 0u;
    bool nd[N];
    relax_compute<A, N>(st, v, c, cur, nd);
    warp_append_n<N>(st.UL, st.lc + L_UL, nd, v);
    return;
  }
#pragma unroll
  for (int k = 0; k < N; ++k) cur[k] = d[k] != 0xFFFFFFFFu ? relax_peek<A>(st, d[k]) : 0u;
  if (kDense) {
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (d[k] != 0xFFFFFFFFu) relax_dense<A>(st, d[k], c[k], cur[k]);
  } else {
    bool nd[N];
    relax_sparse<A, N>(st, d, c, cur, nd);
    warp_append_n<N>(st.DL, st.lc + L_DL, nd, d);
  }
}

template <int A, bool kDense, bool kCompute = false>
__global__ void __launch_bounds__(256) k_hub_push(DevGraph g, DevState st) {
  unsigned long long scanned = 0;
  for (uint32_t c = blockIdx.x; c < g.num_hubs; c += gridDim.x) {
    const HubChunkD h = g.hubs[c];
    if (!test_bit(st.FB, h.slot)) continue;
    const uint32_t sv = source_value<A>(st.mprop[h.slot]);
    const uint32_t a0 = min(h.e1, (h.e0 + 3u) & ~3u);
    const uint32_t a1 = max(a0, h.e1 & ~3u);
    {
      // unaligned head [e0, a0) and tail [a1, e1): at most 3 edges each
      const uint32_t t = threadIdx.x;
      uint32_t e = 0xFFFFFFFFu;
      if (t < a0 - h.e0) e = h.e0 + t;
      else if (t >= 4 && t - 4 < h.e1 - a1) e = a1 + (t - 4);
      uint32_t d[1] = {0xFFFFFFFFu}, cv[1] = {0u};
      if (e != 0xFFFFFFFFu) {
        d[0] = __ldg(&g.col[e]);
        cv[0] = relax_cand<A>(sv, A == A_SSSP_W ? __ldg(&g.wgt[e]) : 0u);
      }
      hub_relax<A, kDense, 1, kCompute>(g, st, d, cv);
    }
    const uint4* c4 = reinterpret_cast<const uint4*>(g.col);
    const uint4* w4 = reinterpret_cast<const uint4*>(g.wgt);
    for (uint32_t q0 = a0 >> 2; q0 < (a1 >> 2); q0 += blockDim.x) {
      const uint32_t q = q0 + threadIdx.x;
      uint32_t d[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, cv[4] = {0u, 0u, 0u, 0u};
      if (q < (a1 >> 2)) {
        const uint4 dv = __ldg(&c4[q]);
        uint4 w = make_uint4(0, 0, 0, 0);
        if (A == A_SSSP_W) w = __ldg(&w4[q]);
        d[0] = dv.x, d[1] = dv.y, d[2] = dv.z, d[3] = dv.w;
        cv[0] = relax_cand<A>(sv, w.x), cv[1] = relax_cand<A>(sv, w.y);
        cv[2] = relax_cand<A>(sv, w.z), cv[3] = relax_cand<A>(sv, w.w);
      }
      hub_relax<A, kDense, 4, kCompute>(g, st, d, cv);
    }
    if (threadIdx.x == 0) scanned += h.e1 - h.e0;
  }
  if (threadIdx.x == 0 && scanned) atomicAdd(&st.counters[C_EDGES], scanned);
}

// Dense-mode dirty set: a slot is dirty when its running min dropped below
// the snapshot taken at its last send (CC/SSSP), or when it received any
// PageRank contribution (the entry is zeroed after every send and every
// contribution is positive).  Rebuilds every word of MD.
// One block per compaction tile: it also writes the tile's dirty count (for
// the backward compaction) and clears the tile's forward bitvector words,
// which nothing reads once the edge-map has run.
template <int A>
__global__ void __launch_bounds__(256) k_diff_dirty(DevGraph g, DevState st) {
  constexpr int U = 8;  // slots in flight per thread
  static_assert(K_TILE_SLOTS % (256 * U) == 0, "whole steps per tile");
  const uint32_t t = blockIdx.x;
  const uint64_t s0 = (uint64_t)t * K_TILE_SLOTS;
  uint32_t c = 0;
  for (uint32_t i0 = 0; i0 < K_TILE_SLOTS; i0 += 256 * U) {
    uint32_t a[U], b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t s = s0 + i0 + u * 256 + threadIdx.x;
      a[u] = __ldcg(&st.mupd[s]);
      b[u] = A == A_PR_DELTA ? 0u : __ldcg(&st.snap[s]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t s = s0 + i0 + u * 256 + threadIdx.x;
      const bool dirty = A == A_PR_DELTA ? a[u] != 0u : a[u] < b[u];
      const uint32_t m = __ballot_sync(FULL, dirty);
      if (lane_id() == 0) {
        st.MD[s >> 5] = m;
        st.FB[s >> 5] = 0;
        c += __popc(m);
      }
    }
  }
  c = block_sum(c);
  if (threadIdx.x == 0) st.tile_cnt[t] = c;
}

// Push + bitvector rounds of the min algorithms: the dirty diff, the
// backward transfer and the aggregate in one pass over the slots.  The
// backward compaction only gives each dirty value its rank in the packed
// message, which the fused path never writes; a dirty slot needs nothing but
// its own gid.  So each thread retires its dirty slot (the snapshot becomes
// the sent value, as OpBwdXfer) and folds the value into vertex_updates with
// red.min.  The tile's words of MD (not needed: left clear, as the backward
// compaction leaves them) and of the forward bitvector are cleared, and the
// sync bytes counted as the backward compaction counts them.
template <int A>
__global__ void __launch_bounds__(256) k_diff_aggregate(DevGraph g, DevState st) {
  static_assert(A != A_PR_DELTA && A != A_PR_PULL, "PageRank aggregates partition by partition");
  constexpr int U = 4;  // slots in flight per thread (8: more registers, 3 blocks per SM, slower)
  static_assert(K_TILE_SLOTS % (256 * U) == 0, "whole steps per tile");
  const uint32_t t = blockIdx.x;
  const uint64_t s0 = (uint64_t)t * K_TILE_SLOTS;
  uint32_t c = 0;
  for (uint32_t i0 = 0; i0 < K_TILE_SLOTS; i0 += 256 * U) {
    uint32_t a[U], b[U], gid[U], cur[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t s = s0 + i0 + u * 256 + threadIdx.x;
      a[u] = __ldcg(&st.mupd[s]);
      b[u] = __ldcg(&st.snap[s]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t s = s0 + i0 + u * 256 + threadIdx.x;
      gid[u] = a[u] < b[u] ? __ldg(&g.slot_gid[s]) : 0u;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) cur[u] = a[u] < b[u] ? __ldcg(&st.upd[gid[u]]) : 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t s = s0 + i0 + u * 256 + threadIdx.x;
      const bool dirty = a[u] < b[u];
      if (dirty) {
        st.snap[s] = a[u];
        if (a[u] < cur[u]) red_min(st.upd + gid[u], a[u]);
      }
      const uint32_t m = __ballot_sync(FULL, dirty);
      if (lane_id() == 0) {
        st.FB[s >> 5] = 0;
        st.MD[s >> 5] = 0;
        c += __popc(m);
      }
    }
  }
  c = block_sum(c);
  if (threadIdx.x == 0) {
    unsigned long long bytes = 4ull * c, rbytes = 4ull * c;
    if (t == 0) bytes += g.bv_bytes, rbytes += g.bv_refbytes;
    if (bytes) atomicAdd(&st.counters[C_BYTES], bytes);
    if (rbytes) atomicAdd(&st.counters[C_REFBYTES], rbytes);
  }
}

// -------------------------------------------------------------- pull map --
// Pull edge-map over each partition's in-edge lists (sources in ascending
// slot order).  Min algorithms fold every in-edge: a source that is not in
// this round's frontier still holds the value it last sent, whose
// relaxation has already been applied, so it cannot lower anything — the
// values and the dirty set equal those of the push over the frontier, with no
// atomics.  Delta PageRank pulls with its fixed-order sums (k_pr_delta_pull
// below) and Jacobi PageRank with k_pr_pull (pr_pull.cu); kahan_add is the
// compensated step both PageRank sums use.
constexpr uint32_t K_PULL_HUB = 1024;  // = PULL_HUB of the layout
constexpr uint32_t K_PULL_MED = 64;    // = PULL_MED of the layout
constexpr uint32_t PULL_CH = 256;      // staged in-edges per warp step

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Value contributed by one in-edge (bit pattern), and the fold identity.
// The generic pull serves the min algorithms (CC, SSSP): delta PageRank pulls
// with its fixed-order sums (k_pr_delta_pull) and Jacobi PageRank with
// k_pr_pull (pr_pull.cu).
template <int A>
__device__ __forceinline__ uint32_t pull_value(const DevState& st, uint32_t src, uint32_t w) {
  static_assert(A == A_CC || A == A_SSSP_HOP || A == A_SSSP_W, "min algorithms only");
  const uint32_t v = st.mprop[src];
  if (A == A_SSSP_HOP) return v == 0xFFFFFFFFu ? v : v + 1u;
  if (A == A_SSSP_W) return sat_add(v, w);
  return v;  // CC
}

template <int A>
struct PullAcc {
  static_assert(A == A_CC || A == A_SSSP_HOP || A == A_SSSP_W, "min algorithms only");
  uint32_t best = 0xFFFFFFFFu;
  __device__ __forceinline__ void fold(uint32_t v) { best = min(best, v); }
};

// Writes the pulled value of destination slot d; returns its dirty bit.
template <int A>
__device__ __forceinline__ bool pull_commit(const DevState& st, uint32_t d, const PullAcc<A>& a, bool) {
  if (a.best < st.mupd[d]) {
    st.mupd[d] = a.best;
    return true;
  }
  return false;
}

// One warp per 32 consecutive destination slots.  Their in-edges are
// concatenated (warp scan of in-degrees) and staged 256 at a time: lanes load
// consecutive in_src entries (coalesced), gather the source values into
// shared memory, then every lane folds its own slot's part of the stage in
// ascending source order.  In-lists longer than K_PULL_MED go to k_pull_med
// (up to K_PULL_HUB) and k_pull_hub.
// The warp writes its 32 dirty bits as one word.
template <int A, bool kList = false>
__global__ void __launch_bounds__(256) k_pull(DevGraph g, DevState st) {
  __shared__ uint32_t s_val[8][PULL_CH];
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint64_t nwarps = (uint64_t)gridDim.x * 8;
  for (uint64_t base = ((uint64_t)blockIdx.x * 8 + warp) * 32; base < g.S; base += nwarps * 32) {
    const uint32_t d = (uint32_t)base + lane;
    const uint32_t b = __ldg(&g.in_off[d]);
    uint32_t deg = __ldg(&g.in_off[d + 1]) - b;
    const bool has = deg > 0;
    const bool hub = deg > K_PULL_MED;  // k_pull_med / k_pull_hub fold it
    if (hub) deg = 0;
    const uint32_t incl = warp_incl_scan(deg);
    const uint32_t excl = incl - deg;
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    PullAcc<A> acc;
    for (uint32_t c0 = 0; c0 < total; c0 += PULL_CH) {
      uint32_t src[PULL_CH / 32], wt[PULL_CH / 32];
#pragma unroll
      for (int k = 0; k < (int)(PULL_CH / 32); ++k) {
        const uint32_t q = c0 + k * 32 + lane;
        uint32_t lo = 0;
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1) {
          const uint32_t cand = lo + step;
          if (__shfl_sync(FULL, excl, cand) <= q) lo = cand;
        }
        const uint32_t sb = __shfl_sync(FULL, b, lo);
        const uint32_t se = __shfl_sync(FULL, excl, lo);
        const uint32_t e = sb + (q - se);
        src[k] = q < total ? __ldg(&g.in_src[e]) : 0xFFFFFFFFu;
        wt[k] = (A == A_SSSP_W && q < total) ? __ldg(&g.in_wgt[e]) : 0u;
      }
#pragma unroll
      for (int k = 0; k < (int)(PULL_CH / 32); ++k)
        s_val[warp][k * 32 + lane] = src[k] != 0xFFFFFFFFu ? pull_value<A>(st, src[k], wt[k]) : 0u;
      __syncwarp();
      const uint32_t q0 = max(excl, c0), q1 = min(excl + deg, c0 + PULL_CH);
      for (uint32_t q = q0; q < q1; ++q) acc.fold(s_val[warp][q - c0]);
      __syncwarp();
    }
    bool dirty = false;
    if (!hub) dirty = pull_commit<A>(st, d, acc, has);
    const uint32_t m = __ballot_sync(FULL, dirty);
    if (lane == 0) st.MD[d >> 5] = m;
    // S is a multiple of 256, so every warp of a block runs the same
    // iterations and the block-wide append is safe.
    if (kList) block_append(st.DL, st.lc + L_DL, dirty, d);
  }
}

// A fold's result (the value pull_commit stores).
template <int A>
__device__ __forceinline__ uint32_t pull_part(const PullAcc<A>& acc) {
  return acc.best;
}

// Medium in-lists (more than K_PULL_MED, at most K_PULL_HUB in-edges): one
// warp per destination; lane l folds the elements l, l+32, ... (coalesced),
// then the 32 partials combine by a butterfly of mins.  Keeps the per-lane
// fold of k_pull balanced: its longest
// list is K_PULL_MED.  Runs after k_pull, whose dirty word for the slot is
// already written: a dirty destination ORs its bit in.
template <int A, bool kList = false>
__global__ void __launch_bounds__(256) k_pull_med(DevGraph g, DevState st, const HubChunkD* meds, uint32_t n) {
  const uint32_t lane = lane_id();
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += nw) {
    const HubChunkD hc = meds[w];
    PullAcc<A> acc;
    uint32_t q = hc.e0 + lane;
    for (; q + 3 * 32 < hc.e1; q += 4 * 32) {
      uint32_t v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t e = q + u * 32;
        v[u] = pull_value<A>(st, __ldg(&g.in_src[e]), A == A_SSSP_W ? __ldg(&g.in_wgt[e]) : 0u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) acc.fold(v[u]);
    }
    for (; q < hc.e1; q += 32)
      acc.fold(pull_value<A>(st, __ldg(&g.in_src[q]), A == A_SSSP_W ? __ldg(&g.in_wgt[q]) : 0u));
    uint32_t part = pull_part<A>(acc);
#pragma unroll
    for (int o = 16; o; o >>= 1) part = min(part, __shfl_xor_sync(FULL, part, o));
    if (lane == 0) {
      PullAcc<A> tot;
      tot.fold(part);
      if (pull_commit<A>(st, hc.slot, tot, true)) {
        if (kList)
          mark_listed(st.MD, hc.slot, st.DL, st.lc + L_DL);
        else
          red_or(st.MD + (hc.slot >> 5), 1u << (hc.slot & 31));
      }
    }
  }
}

// Long in-lists: one block per destination; thread t folds the elements t,
// t+256, ... (coalesced), then thread 0 takes the min of the 256 partials.
// Runs after k_pull, whose
// dirty word for the slot is already written: a dirty hub ORs its bit in.
template <int A, bool kList = false>
__global__ void __launch_bounds__(256) k_pull_hub(DevGraph g, DevState st, const HubChunkD* hubs, uint32_t n) {
  __shared__ uint32_t s_part[256];
  for (uint32_t h = blockIdx.x; h < n; h += gridDim.x) {
    const HubChunkD hc = hubs[h];
    PullAcc<A> acc;
    uint32_t q = hc.e0 + threadIdx.x;
    for (; q + 3 * 256 < hc.e1; q += 4 * 256) {
      uint32_t v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t e = q + u * 256;
        v[u] = pull_value<A>(st, __ldg(&g.in_src[e]), A == A_SSSP_W ? __ldg(&g.in_wgt[e]) : 0u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) acc.fold(v[u]);
    }
    for (; q < hc.e1; q += 256)
      acc.fold(pull_value<A>(st, __ldg(&g.in_src[q]), A == A_SSSP_W ? __ldg(&g.in_wgt[q]) : 0u));
    s_part[threadIdx.x] = pull_part<A>(acc);
    __syncthreads();
    if (threadIdx.x == 0) {
      PullAcc<A> tot;
      for (int i = 0; i < 256; ++i) tot.fold(s_part[i]);
      if (pull_commit<A>(st, hc.slot, tot, true)) {
        if (kList)
          mark_listed(st.MD, hc.slot, st.DL, st.lc + L_DL);
        else
          red_or(st.MD + (hc.slot >> 5), 1u << (hc.slot & 31));
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------- delta PageRank: one fixed order --
// Every delta-PageRank edge-map (push or pull, bitvector or list sync, the
// one-CTA round) gives each memory-side destination slot the same value: its
// in-list (ascending source slot) is cut into 32-edge chunks from the list's
// start; a chunk's frontier contributions (0 for sources outside the
// frontier and past the list's end) are added by a halving tree -- x[i] +=
// x[i + o] for o = 16, 8, 4, 2, 1, which is the warp's xor butterfly -- and
// the chunk sums are added in chunk order.  So the value depends on the graph
// and the frontier only, not on the round mode or on thread timing, and the
// oracle restates the same order.  The push's reductions still find the
// slots it touches (the dirty set); their sums are then replaced by this one.
// Warp-wide: every lane returns the sum.
__device__ __forceinline__ float pr_delta_sum_warp(const DevGraph& g, const DevState& st, uint32_t d) {
  const uint32_t lane = lane_id();
  const uint32_t a = __ldg(&g.in_off[d]), b = __ldg(&g.in_off[d + 1]);
  float acc = 0.0f;
  for (uint32_t c = a; c < b; c += 4 * 32) {  // four chunks' loads in flight
    uint32_t src[4];
    float x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t e = c + 32u * q + lane;
      src[q] = e < b ? __ldg(&g.in_src[e]) : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      x[q] = (src[q] != 0xFFFFFFFFu && test_bit(st.FB, src[q])) ? __uint_as_float(st.mprop[src[q]]) : 0.0f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
      for (int o = 16; o; o >>= 1) x[q] = __fadd_rn(x[q], __shfl_xor_sync(FULL, x[q], o));
      if (c + 32u * q < b) acc = __fadd_rn(acc, x[q]);  // chunks past the list's end do not exist
    }
  }
  return acc;
}

// The same sum of a list of at most 32 in-edges by one lane: the halving
// tree run on registers gives the bits of the xor butterfly, and 0 + x = x.
__device__ __forceinline__ float pr_delta_sum_lane(const DevGraph& g, const DevState& st, uint32_t a, uint32_t n) {
  float x[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    x[i] = 0.0f;
    if ((uint32_t)i < n) {
      const uint32_t src = __ldg(&g.in_src[a + i]);
      if (test_bit(st.FB, src)) x[i] = __uint_as_float(st.mprop[src]);
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1)
#pragma unroll
    for (int i = 0; i < o; ++i) x[i] = __fadd_rn(x[i], x[i + o]);
  return __fadd_rn(0.0f, x[0]);
}

// Lists of more than 32 in-edges are summed grid-wide: every 32-edge chunk
// by its own warp into a scratch array, then each list's chunk sums in chunk
// order by one warp -- the same order, with the whole GPU on the chunks.
constexpr uint32_t K_PRD_SHORT = 32;

__device__ __forceinline__ bool pr_delta_long(const DevGraph& g, uint32_t d) {
  return __ldg(&g.in_off[d + 1]) - __ldg(&g.in_off[d]) > K_PRD_SHORT;
}

// Every lane with `want` gets the fixed-order sum of its slot d when the list
// is short (at most 32 in-edges, summed by the lane itself); *long_list tells
// the lanes whose list the grid-wide path sums.
__device__ __forceinline__ float pr_delta_sum_slots(const DevGraph& g, const DevState& st, uint32_t d, bool want,
                                                    bool* long_list) {
  uint32_t a = 0, n = 0;
  if (want) {
    a = __ldg(&g.in_off[d]);
    n = __ldg(&g.in_off[d + 1]) - a;
  }
  *long_list = want && n > K_PRD_SHORT;
  return (want && n <= K_PRD_SHORT) ? pr_delta_sum_lane(g, st, a, n) : 0.0f;
}

struct PrHubs {
  const HubChunkD* hubs;      // (slot, e0, e1) of every list of more than 32 in-edges
  const uint32_t* coff;       // [nh + 1] first chunk of each such list
  const uint32_t* chunk_hub;  // [nc] list of each chunk
  float* csum;                // [nc] chunk sums
  uint32_t nh, nc;
};

// kMode 0: pull (every hub), 1: push + bitvector (touched: mupd != 0),
// 2: push + list (touched: dirty bit claimed).
template <int kMode>
__device__ __forceinline__ bool pr_hub_needed(const DevState& st, uint32_t slot) {
  if (kMode == 0) return true;
  if (kMode == 1) return __ldcg(&st.mupd[slot]) != 0u;
  return (__ldcg(&st.MD[slot >> 5]) >> (slot & 31)) & 1u;
}

__device__ __forceinline__ float pr_delta_chunk(const DevState& st, const DevGraph& g, uint32_t e, uint32_t end) {
  float x = 0.0f;
  if (e < end) {
    const uint32_t src = __ldg(&g.in_src[e]);
    if (test_bit(st.FB, src)) x = __uint_as_float(st.mprop[src]);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) x = __fadd_rn(x, __shfl_xor_sync(FULL, x, o));
  return x;
}

template <int kMode>
__global__ void __launch_bounds__(256) k_pr_delta_hub_chunks(DevGraph g, DevState st, PrHubs h) {
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < h.nc; q += nw) {
    const uint32_t k = h.chunk_hub[q];
    const HubChunkD hc = h.hubs[k];
    if (!pr_hub_needed<kMode>(st, hc.slot)) continue;
    const float x = pr_delta_chunk(st, g, hc.e0 + 32u * (q - h.coff[k]) + lane_id(), hc.e1);
    if (lane_id() == 0) h.csum[q] = x;
  }
}

// One warp per long list: the chunk sums are loaded 128 at a time
// (coalesced) and added in chunk order through shuffles (every lane keeps the
// same sum).
template <int kMode, bool kList>
__global__ void __launch_bounds__(256) k_pr_delta_hub_sum(DevGraph g, DevState st, PrHubs h) {
  const uint32_t lane = lane_id();
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < h.nh; k += nw) {
    const uint32_t slot = h.hubs[k].slot;
    if (!pr_hub_needed<kMode>(st, slot)) continue;
    const uint32_t q0 = h.coff[k], q1 = h.coff[k + 1];
    float acc = 0.0f;
    for (uint32_t q = q0; q < q1; q += 128) {
      float x[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t idx = q + 32u * i + lane;
        x[i] = idx < q1 ? h.csum[idx] : 0.0f;  // past the end: adds nothing
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int l = 0; l < 32; ++l) acc = __fadd_rn(acc, __shfl_sync(FULL, x[i], l));
    }
    if (lane != 0) continue;
    if (kMode != 0) {
      st.mupd[slot] = __float_as_uint(acc);
    } else if (acc > 0.0f) {  // pull: the warp kernel wrote the slot's dirty word first
      st.mupd[slot] = __float_as_uint(acc);
      if (kList)
        mark_listed(st.MD, slot, st.DL, st.lc + L_DL);
      else
        red_or(st.MD + (slot >> 5), 1u << (slot & 31));
    }
  }
}

// Push + bitvector rounds: the slots the push touched (mupd != 0: every
// contribution is positive) get the fixed-order sum; runs before the dirty
// diff, which clears the forward bitvector.
static __global__ void __launch_bounds__(256) k_pr_delta_resum_bits(DevGraph g, DevState st) {
  const uint32_t lane = lane_id();
  const uint64_t nwords = g.S / 32;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t w = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nwords; w += nw) {
    const uint32_t s = (uint32_t)(w * 32) + lane;
    const bool touched = __ldcg(&st.mupd[s]) != 0u;
    bool lng;
    const float v = pr_delta_sum_slots(g, st, s, touched, &lng);
    if (touched && !lng) st.mupd[s] = __float_as_uint(v);
  }
}

// Push + list rounds: the listed dirty slots get the fixed-order sum.
static __global__ void __launch_bounds__(256) k_pr_delta_resum_list(DevGraph g, DevState st) {
  const uint32_t n = __ldcg(&st.lc[L_DL]);
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t j0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; j0 < n; j0 += nw * 32) {
    const uint32_t j = j0 + lane_id();
    const uint32_t d = j < n ? st.DL[j] : 0u;
    bool lng;
    const float v = pr_delta_sum_slots(g, st, d, j < n, &lng);
    if (j < n && !lng) st.mupd[d] = __float_as_uint(v);  // in-hubs: k_pr_delta_hub_*
  }
}

// Pull rounds: every slot with in-edges gets the fixed-order sum; a slot with
// a frontier in-neighbour (sum > 0) is dirty.  One warp per 32-slot word
// writes the word's dirty bits; kList also lists the dirty slots.
template <bool kList>
__global__ void __launch_bounds__(256) k_pr_delta_pull(DevGraph g, DevState st) {
  const uint32_t lane = lane_id();
  const uint64_t nwords = g.S / 32;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t w = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nwords; w += nw) {
    const uint32_t s = (uint32_t)(w * 32) + lane;
    bool lng;
    const float v = pr_delta_sum_slots(g, st, s, true, &lng);  // an empty list sums to 0: not dirty
    const bool dirty = !lng && v > 0.0f;
    if (dirty) st.mupd[s] = __float_as_uint(v);
    const uint32_t m = __ballot_sync(FULL, dirty);
    if (lane == 0) st.MD[w] = m;  // in-hubs OR their bits in afterwards (k_pr_delta_hub_sum)
    if (kList && dirty) list_append(st.DL, st.lc + L_DL, s);
  }
}

// -------------------------------------------------------- list-format sync --
// List rounds carry the same data as bitvector rounds — the frontier's values
// to their owning memory partitions, the dirty memory-side updates back — as
// (slot, value) lists, so a round costs O(frontier + dirty) instead of
// O(slots).  Values, dirty sets and round counts are identical to bitvector
// rounds.  The byte statistics keep the bitvector formula: every sync pass
// sends each partition's bitvector (a constant) plus 4 bytes per value.
//
// Between rounds: FB and MD are all-zero, F and FL hold the frontier, and UL
// lists exactly the gids whose vertex_updates dirty bit is set.

// Forward sync from the frontier list: the j-th entry's value goes to the
// owned slot of its gid, which joins the active list (j-th entry) and the
// forward bitvector (hub rows, PageRank pull).  A round starts here, so block
// 0 also clears the per-round counters and the dirty-slot list.
static __global__ void __launch_bounds__(256) k_fwd_list(DevGraph g, DevState st) {
  const uint32_t K = __ldcg(&st.lc[L_FL]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st.counters[C_ACTIVE] = K;
    st.counters[C_BYTES] += g.bv_bytes + 4ull * K;
    st.counters[C_REFBYTES] += g.bv_refbytes + 4ull * K;
    reset_round_counters(st);
    st.lc[L_DL] = 0;
  }
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < K; j += gridDim.x * blockDim.x) {
    const uint32_t gid = st.FL[j];
    const uint32_t s = st.own_slot[gid];
    st.AL[j] = s;
    st.mprop[s] = st.prop[gid];
    atomicOr(&st.FB[s >> 5], 1u << (s & 31));
  }
}

// Backward sync from the dirty list: send (retire) each dirty slot's value,
// clear its dirty bit, and aggregate it into the compute-side
// vertex_updates, listing every gid whose entry became dirty.  Also retires
// the old frontier (its FB and F bits), which nothing reads after the
// edge-map.
// PageRank runs it once per memory partition, in ascending order (part = p:
// only that partition's dirty slots; the first launch also retires the old
// frontier and counts the bytes), so every vertex receives its partitions'
// sums in partition order, as in bitvector rounds; part = ~0: all at once.
template <int A>
__global__ void __launch_bounds__(256) k_bwd_list(DevGraph g, DevState st, uint32_t part) {
  const uint32_t n = __ldcg(&st.lc[L_DL]);
  const uint32_t K = (uint32_t)__ldcg(&st.counters[C_ACTIVE]);
  const bool first = part == 0u || part == 0xFFFFFFFFu;
  if (first && blockIdx.x == 0 && threadIdx.x == 0) {
    st.counters[C_BYTES] += g.bv_bytes + 4ull * n;
    st.counters[C_REFBYTES] += g.bv_refbytes + 4ull * n;
    st.lc[L_FL] = 0;  // the update rebuilds it; entries below are read by index
  }
  if (first)
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < K; j += gridDim.x * blockDim.x) {
      const uint32_t s = st.AL[j], gid = st.FL[j];
      atomicAnd(&st.FB[s >> 5], ~(1u << (s & 31)));
      atomicAnd(&st.F[gid >> 5], ~(1u << (gid & 31)));
    }
  for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
    const uint32_t j = b + threadIdx.x;
    bool listed = false;
    uint32_t gid = 0;
    const uint32_t s = j < n ? st.DL[j] : 0u;
    if (j < n && (part == 0xFFFFFFFFu || g.tile_part[s / K_TILE_SLOTS] == part)) {
      const uint32_t v = st.mupd[s];
      gid = __ldg(&g.slot_gid[s]);
      retire_update<A>(st, s, v);
      atomicAnd(&st.MD[s >> 5], ~(1u << (s & 31)));
      if (A == A_PR_DELTA) {  // one slot per vertex in this launch
        st.upd[gid] = __float_as_uint(__fadd_rn(__uint_as_float(st.upd[gid]), __uint_as_float(v)));
        listed = claim_bit(st.UD, gid);
      } else if (v < __ldcg(&st.upd[gid])) {
        if (v < atomicMin(&st.upd[gid], v)) listed = claim_bit(st.UD, gid);
      }
    }
    block_append(st.UL, st.lc + L_UL, listed, gid);
  }
}

// NO_OFFLOAD round, after the compute-side edge-map: retires the old
// frontier (its FB and F bits; the update rebuilds the list) and counts the
// shipped adjacency.  Per frontier vertex the owning memory partition sends
// one message of its gid and its out-edges' destination gids (and, weighted
// SSSP, their weights), 4 bytes each (src/GraphAlgorithm.cpp:426-474); the
// reference's counter adds it at the send and again at the receive
// (include/MPI.hpp:40-54), the true size counts it once.
template <int A>
__global__ void __launch_bounds__(256) k_retire_list(DevGraph g, DevState st) {
  const uint32_t K = (uint32_t)__ldcg(&st.counters[C_ACTIVE]);
  if (blockIdx.x == 0 && threadIdx.x == 0) st.lc[L_FL] = 0;  // entries below are read by index
  unsigned long long words = 0;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < K; j += gridDim.x * blockDim.x) {
    const uint32_t s = st.AL[j], gid = st.FL[j];
    atomicAnd(&st.FB[s >> 5], ~(1u << (s & 31)));
    atomicAnd(&st.F[gid >> 5], ~(1u << (gid & 31)));
    words += 1ull + (unsigned long long)g.outdeg[gid] * (A == A_SSSP_W ? 2ull : 1ull);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) words += __shfl_xor_sync(FULL, words, o);
  if (lane_id() == 0 && words) {
    atomicAdd(&st.counters[C_BYTES], 4ull * words);
    atomicAdd(&st.counters[C_REFBYTES], 8ull * words);
  }
}

// ------------------------------------------------------------------ update --
// UpdateWorker::update = update_frontier() then apply_updates()
// (src/Workers.cpp:77-82) for one vertex whose vertex_updates entry is dirty.
// PageRank: pr.cpp:123-147 then :63-88.  prev_updates is set and reset
// within the same round for every frontier vertex, so its test is always
// true and the array is not kept.  CC/SSSP: cc.cpp:86-107, sssp.cpp:92-113.
// Returns true when v joins the frontier; `visited` collects the out-degree
// of SSSP vertices reached for the first time.
template <int A>
__device__ __forceinline__ bool update_one(const DevGraph& g, const DevState& st, uint32_t v, double tol,
                                           double damping, uint32_t& visited) {
  if (A == A_PR_DELTA) {
    const float u = __uint_as_float(st.upd[v]);
    if ((double)u > tol) {
      st.ranks[v] = __fadd_rn(st.ranks[v], u);
      st.prop[v] = __float_as_uint((float)(damping * (double)u / (double)g.outdeg[v]));
      st.upd[v] = 0;
      return true;
    }
    return false;
  }
  const uint32_t u = st.upd[v];
  const uint32_t p = st.prop[v];
  if (p > u) {
    st.prop[v] = u;
    if ((A == A_SSSP_HOP || A == A_SSSP_W) && p == 0xFFFFFFFFu) visited += g.outdeg[v];
    return true;
  }
  return false;
}

// Frontier shape of one block, one counter update each.
__device__ __forceinline__ void flush_frontier_shape(const DevState& st, uint32_t fcount, uint32_t fedges,
                                                     uint32_t fmax, uint32_t visited) {
  fcount = block_sum(fcount);
  fedges = block_sum(fedges);
  visited = block_sum(visited);
  fmax = block_max(fmax);
  if (threadIdx.x == 0) {
    if (fcount) atomicAdd(&st.counters[C_FRONTIER], (unsigned long long)fcount);
    if (fedges) atomicAdd(&st.counters[C_FEDGES], (unsigned long long)fedges);
    if (fmax) atomicMax(&st.counters[C_FMAXDEG], (unsigned long long)fmax);
    if (visited) atomicAdd(&st.counters[C_UNVISITED], 0ull - (unsigned long long)visited);
  }
}

// Update over the updated-gid list (list rounds).  The last block to finish
// empties the list.
template <int A>
__global__ void __launch_bounds__(256) k_update_list(DevGraph g, DevState st, double tol, double damping) {
  const uint32_t n = __ldcg(&st.lc[L_UL]);
  uint32_t fcount = 0, fedges = 0, fmax = 0, visited = 0;
  for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
    const uint32_t j = b + threadIdx.x;
    bool nf = false;
    uint32_t v = 0;
    if (j < n) {
      v = st.UL[j];
      atomicAnd(&st.UD[v >> 5], ~(1u << (v & 31)));
      nf = update_one<A>(g, st, v, tol, damping, visited);
      if (nf) {
        atomicOr(&st.F[v >> 5], 1u << (v & 31));
        const uint32_t d = g.outdeg[v];
        ++fcount;
        fedges += d;
        fmax = max(fmax, d);
      }
    }
    block_append(st.FL, st.lc + L_FL, nf, v);
  }
  flush_frontier_shape(st, fcount, fedges, fmax, visited);
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&st.counters[C_DONE], 1ull) == gridDim.x - 1) {
      st.lc[L_UL] = 0;  // every block has read n
      st.counters[C_DONE] = 0;
    }
  }
}

// ------------------------------------------------------------ tiny round --
// A whole push + list round in one CTA of 1024 threads, for frontiers of at
// most K_TINY_ACTIVE vertices and K_TINY_EDGES out-edges (every row of such a
// frontier, hub or not, runs here).  The phases are those of k_fwd_list,
// the push edge-map, k_bwd_list and k_update_list, separated by block
// barriers instead of kernel boundaries, so a small round costs one launch.
// Values, dirty sets, lists and statistics equal the multi-kernel round's.
// kCompute: the same for a NO_OFFLOAD round (compute-side push straight into
// vertex_updates, no backward sync), equal to the multi-kernel NO_OFFLOAD
// round (k_fwd_list, the degree scan, k_push_lbs/k_hub_push<.., true>,
// k_retire_list, k_update_list).
constexpr uint32_t K_TINY_ACTIVE = 2048;
constexpr uint32_t K_TINY_EDGES = 16384;
constexpr int K_TINY_THREADS = 1024;

// One whole round by one CTA of K_TINY_THREADS (k_round_tiny, and the
// in-kernel round loop of the device-driven loop).
template <int A, bool kCompute>
__device__ __forceinline__ void tiny_round(const DevGraph& g, const DevState& st, double tol, double damping) {
  __shared__ uint32_t s_dp[K_TINY_ACTIVE + 1];
  __shared__ uint32_t s_rb[K_TINY_ACTIVE];
  __shared__ uint32_t s_sv[K_TINY_ACTIVE];
  __shared__ uint32_t s_carry;
  const uint32_t tid = threadIdx.x;
  const uint32_t K = __ldcg(&st.lc[L_FL]);
  if (K > K_TINY_ACTIVE) {  // never chosen for such a frontier; refuse rather than drop actives
    if (tid == 0) atomicCAS(&st.counters[C_ERR], 0ull, 3ull);
    return;
  }
  // forward sync + per-round counters
  if (tid == 0) {
    st.counters[C_ACTIVE] = K;
    st.counters[C_BYTES] += g.bv_bytes + 4ull * K;
    st.counters[C_REFBYTES] += g.bv_refbytes + 4ull * K;
    reset_round_counters(st);
    st.lc[L_DL] = 0;
    s_carry = 0;
  }
  __syncthreads();
  // degree prefix of the actives (block scan, 1024 at a time)
  for (uint32_t b = 0; b < K; b += K_TINY_THREADS) {
    const uint32_t j = b + tid;
    uint32_t d = 0;
    if (j < K) {
      const uint32_t gid = st.FL[j];
      const uint32_t s = st.own_slot[gid];
      const uint32_t v = st.prop[gid];
      st.AL[j] = s;
      st.mprop[s] = v;
      if (A == A_PR_DELTA && !kCompute) atomicOr(&st.FB[s >> 5], 1u << (s & 31));  // the fixed-order sum reads it
      const uint32_t r0 = __ldg(&g.row_off[s]);
      d = __ldg(&g.row_off[s + 1]) - r0;
      s_rb[j] = r0;
      s_sv[j] = source_value<A>(v);
    }
    const uint32_t incl = warp_incl_scan(d);
    __shared__ uint32_t s_w[32];
    if (lane_id() == 31) s_w[tid >> 5] = incl;
    __syncthreads();
    if (tid < 32) {
      const uint32_t x = s_w[tid];
      s_w[tid] = warp_incl_scan(x) - x;
    }
    __syncthreads();
    const uint32_t carry = s_carry;
    if (j < K) s_dp[j] = carry + s_w[tid >> 5] + incl - d;
    __syncthreads();
    if (tid == K_TINY_THREADS - 1) s_carry = carry + s_w[tid >> 5] + incl;
    __syncthreads();
  }
  const uint32_t m = s_carry;  // frontier out-edges
  if (tid == 0) {
    s_dp[K] = m;
    st.counters[C_EDGES] += m;
  }
  __syncthreads();
  // push edge-map over the m edges, 4 per thread per step
  constexpr int N = 4;
  for (uint32_t e0 = 0; e0 < m; e0 += K_TINY_THREADS * N) {
    uint32_t dst[N], cand[N], cur[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const uint32_t e = e0 + k * K_TINY_THREADS + tid;
      dst[k] = 0xFFFFFFFFu;
      cand[k] = 0;
      if (e < m) {
        uint32_t lo = 0, hi = K;  // last i with s_dp[i] <= e
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (s_dp[mid] <= e) lo = mid; else hi = mid;
        }
        const uint32_t ed = s_rb[lo] + (e - s_dp[lo]);
        dst[k] = __ldg(&g.col[ed]);
        cand[k] = relax_cand<A>(s_sv[lo], A == A_SSSP_W ? __ldg(&g.wgt[ed]) : 0u);
      }
    }
    bool nd[N];
    if (kCompute) {  // NO_OFFLOAD: straight into the compute partition's vertex_updates
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (dst[k] != 0xFFFFFFFFu) dst[k] = __ldg(&g.slot_gid[dst[k]]);
#pragma unroll
      for (int k = 0; k < N; ++k) cur[k] = dst[k] != 0xFFFFFFFFu ? relax_peek_gid<A>(st, dst[k]) : 0u;
      relax_compute<A, N>(st, dst, cand, cur, nd);
      block_append_n<N>(st.UL, st.lc + L_UL, nd, dst);
    } else {
#pragma unroll
      for (int k = 0; k < N; ++k) cur[k] = dst[k] != 0xFFFFFFFFu ? relax_peek<A>(st, dst[k]) : 0u;
      relax_sparse<A, N>(st, dst, cand, cur, nd);
      block_append_n<N>(st.DL, st.lc + L_DL, nd, dst);
    }
  }
  __syncthreads();
  if (A == A_PR_DELTA && !kCompute) {  // the listed slots get the fixed-order sum
    const uint32_t nd = __ldcg(&st.lc[L_DL]);
    for (uint32_t j0 = (tid >> 5) * 32; j0 < nd; j0 += K_TINY_THREADS) {
      const uint32_t j = j0 + lane_id();
      const uint32_t d = j < nd ? st.DL[j] : 0u;
      bool lng;
      const float v = pr_delta_sum_slots(g, st, d, j < nd, &lng);
      if (j < nd && !lng) st.mupd[d] = __float_as_uint(v);
      // lists of 33..1024 in-edges: the whole warp, one after another
      uint32_t m = __ballot_sync(FULL, lng && __ldg(&g.in_off[d + 1]) - __ldg(&g.in_off[d]) <= K_PULL_HUB);
      while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t dl = __shfl_sync(FULL, d, l);
        const float x = pr_delta_sum_warp(g, st, dl);
        if (lane_id() == 0) st.mupd[dl] = __float_as_uint(x);
      }
    }
    // lists of more than 1024 in-edges: every warp sums chunks, thread 0 adds
    // them in order
    __shared__ uint32_t s_long[K_TINY_THREADS];
    __shared__ uint32_t s_nlong;
    __shared__ float s_cs[K_TINY_THREADS];
    __shared__ float s_acc;
    for (uint32_t b = 0; b < nd; b += K_TINY_THREADS) {
      __syncthreads();
      if (tid == 0) s_nlong = 0;
      __syncthreads();
      if (b + tid < nd) {
        const uint32_t d = st.DL[b + tid];
        if (__ldg(&g.in_off[d + 1]) - __ldg(&g.in_off[d]) > K_PULL_HUB) s_long[atomicAdd(&s_nlong, 1u)] = d;
      }
      __syncthreads();
      const uint32_t nl = s_nlong;
      for (uint32_t i = 0; i < nl; ++i) {
        const uint32_t d = s_long[i];
        const uint32_t a = __ldg(&g.in_off[d]), e = __ldg(&g.in_off[d + 1]);
        const uint32_t nch = (e - a + 31) / 32;
        if (tid == 0) s_acc = 0.0f;
        for (uint32_t c0 = 0; c0 < nch; c0 += K_TINY_THREADS) {
          const uint32_t c1 = min(nch, c0 + K_TINY_THREADS);
          for (uint32_t c = c0 + (tid >> 5); c < c1; c += K_TINY_THREADS / 32) {
            const float x = pr_delta_chunk(st, g, a + 32u * c + lane_id(), e);
            if (lane_id() == 0) s_cs[c - c0] = x;
          }
          __syncthreads();
          if (tid == 0) {
            float acc = s_acc;
            for (uint32_t c = c0; c < c1; ++c) acc = __fadd_rn(acc, s_cs[c - c0]);
            s_acc = acc;
          }
          __syncthreads();
        }
        if (tid == 0) st.mupd[d] = __float_as_uint(s_acc);
      }
    }
    __syncthreads();
  }
  // backward sync: retire the old frontier, send and aggregate the dirty
  // slots (NO_OFFLOAD: count the shipped adjacency instead, as k_retire_list)
  const uint32_t n = kCompute ? 0u : __ldcg(&st.lc[L_DL]);
  if (tid == 0) {
    if (kCompute) {
      const unsigned long long words = (unsigned long long)K + (unsigned long long)m * (A == A_SSSP_W ? 2ull : 1ull);
      st.counters[C_BYTES] += 4ull * words;
      st.counters[C_REFBYTES] += 8ull * words;
    } else {
      st.counters[C_BYTES] += g.bv_bytes + 4ull * n;
      st.counters[C_REFBYTES] += g.bv_refbytes + 4ull * n;
    }
  }
  for (uint32_t j = tid; j < K; j += K_TINY_THREADS) {
    const uint32_t gid = st.FL[j];
    atomicAnd(&st.F[gid >> 5], ~(1u << (gid & 31)));
    if (A == A_PR_DELTA && !kCompute) {
      const uint32_t s = st.AL[j];
      atomicAnd(&st.FB[s >> 5], ~(1u << (s & 31)));
    }
  }
  // PageRank aggregates partition by partition (ascending), as the
  // multi-kernel rounds do; min-aggregates in one pass
  const uint32_t groups = A == A_PR_DELTA ? g.M : 1u;
  for (uint32_t p = 0; p < groups; ++p) {
    for (uint32_t b = 0; b < n; b += K_TINY_THREADS) {
      const uint32_t j = b + tid;
      bool listed = false;
      uint32_t gid = 0;
      const uint32_t s = j < n ? st.DL[j] : 0u;
      if (j < n && (A != A_PR_DELTA || g.tile_part[s / K_TILE_SLOTS] == p)) {
        const uint32_t v = st.mupd[s];
        gid = __ldg(&g.slot_gid[s]);
        retire_update<A>(st, s, v);
        atomicAnd(&st.MD[s >> 5], ~(1u << (s & 31)));
        if (A == A_PR_DELTA) {  // one slot per vertex in this pass
          st.upd[gid] = __float_as_uint(__fadd_rn(__uint_as_float(st.upd[gid]), __uint_as_float(v)));
          listed = claim_bit(st.UD, gid);
        } else if (v < __ldcg(&st.upd[gid])) {
          if (v < atomicMin(&st.upd[gid], v)) listed = claim_bit(st.UD, gid);
        }
      }
      block_append(st.UL, st.lc + L_UL, listed, gid);
    }
    if (A == A_PR_DELTA) __syncthreads();
  }
  if (tid == 0) st.lc[L_FL] = 0;
  __syncthreads();
  // update over the updated-gid list
  const uint32_t nu = __ldcg(&st.lc[L_UL]);
  uint32_t fcount = 0, fedges = 0, fmax = 0, visited = 0;
  for (uint32_t b = 0; b < nu; b += K_TINY_THREADS) {
    const uint32_t j = b + tid;
    bool nf = false;
    uint32_t v = 0;
    if (j < nu) {
      v = st.UL[j];
      atomicAnd(&st.UD[v >> 5], ~(1u << (v & 31)));
      nf = update_one<A>(g, st, v, tol, damping, visited);
      if (nf) {
        atomicOr(&st.F[v >> 5], 1u << (v & 31));
        const uint32_t d = g.outdeg[v];
        ++fcount;
        fedges += d;
        fmax = max(fmax, d);
      }
    }
    block_append(st.FL, st.lc + L_FL, nf, v);
  }
  flush_frontier_shape(st, fcount, fedges, fmax, visited);
  __syncthreads();
  if (tid == 0) st.lc[L_UL] = 0;
}

template <int A, bool kCompute = false>
__global__ void __launch_bounds__(K_TINY_THREADS) k_round_tiny(DevGraph g, DevState st, double tol, double damping) {
  tiny_round<A, kCompute>(g, st, tol, damping);
}

// Update of a bitvector round: rebuilds the frontier bitmap
// (frontier.reset() first, src/GraphAlgorithm.cpp:646) and list, clears the
// dirty bits (clear_uv, :661) and records the frontier's shape.  The
// reference tests its dirty vertices; this tests every vertex, which selects
// the same ones: after each update, update_frontier's test (CC/SSSP
// prop > upd, PageRank upd > tol) is false for every vertex, and only an
// aggregate (this round's, or grd_aggregate_values) can make it true again.
// Block-uniform loop.
template <int A>
__global__ void __launch_bounds__(256) k_update(DevGraph g, DevState st, double tol, double damping) {
  constexpr int U = 4;  // vertices per thread per step; one list append per block and step
  uint32_t fcount = 0, fedges = 0, fmax = 0, visited = 0;
  for (uint32_t base = blockIdx.x * blockDim.x * U; base < g.V; base += gridDim.x * blockDim.x * U) {
    bool nf[U];
    uint32_t vs[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t v = base + u * blockDim.x + threadIdx.x;  // a warp takes 32 consecutive vertices
      vs[u] = v;
      nf[u] = false;
      if (v < g.V) {
        nf[u] = update_one<A>(g, st, v, tol, damping, visited);
        if (nf[u]) {
          const uint32_t d = g.outdeg[v];
          ++fcount;
          fedges += d;
          fmax = max(fmax, d);
        }
      }
      const uint32_t m = __ballot_sync(FULL, nf[u]);
      if (lane_id() == 0 && v < g.V) {  // v is the first gid of this word
        st.F[v >> 5] = m;
        st.UD[v >> 5] = 0;
      }
    }
    block_append_n<U>(st.FL, st.lc + L_FL, nf, vs);
  }
  flush_frontier_shape(st, fcount, fedges, fmax, visited);
}

}  // namespace grd
