// GRD_PR_PULL: Jacobi PageRank through the partitioned round structure.
//
// Fixed point (the one the reference's delta-push PageRank converges to,
// src/graph_algorithms/pr.cpp:20-88):
//   pr[v] = (1-d)*[outdeg(v) > 0] + sum_{u->v} d * pr[u] / outdeg(u)
// One iteration is one round of src/GraphAlgorithm.cpp:145-701 with every
// non-dangling vertex in the frontier:
//   forward sync   the compute partition's contributions c[u] = d*pr[u]/outdeg(u)
//                  are what the memory partitions read: all partitions share
//                  one HBM, so the pull gathers them straight from the compute
//                  partition's array (vertex_properties, written by
//                  k_pr_update as it forms the rank), and the send only copies
//                  the hot sources' values (k_pr_update; k_pr_fwd at init);
//   edge-map       every memory partition sums, per destination slot, its
//                  in-edges' contributions with a Kahan-compensated FP32 sum
//                  (k_pr_pull, k_pr_fix);
//   backward sync  the partial sums go back to the compute partition, which
//   + aggregate    merges them per vertex in partition order (Kahan), forms
//                  the new rank in FP32 and reduces the L1 residual across
//                  threads and blocks in FP64 (k_pr_update, k_pr_round_end).
// Every order is fixed by the layout, so ranks, residuals and iteration
// counts are reproducible run to run.
//
// The edge-map is edge-balanced: the in-edges of all partitions (in_src, each
// in-list in ascending source slot order) are cut into 512-edge tiles, one per
// warp, 16 consecutive edges per lane, whatever the in-degrees.  An in-list
// is summed in its stored order as a chain of pieces: each lane folds its
// edges of the list with Kahan, a list that crosses lanes continues the
// running sum lane by lane (in lane order), and one that crosses tiles
// continues tile by tile (k_pr_fix, in tile order).  The hottest sources (the
// highest out-degrees, up to PR_HOT_CAP of them) are staged in shared memory
// each iteration; their in-edges carry the hot index instead of the source
// vertex, so about a third of the gathers never leave the SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "ctx.hpp"
#include "kernels.cuh"

using namespace grd;

namespace {

constexpr uint32_t PR_TILE = 512;      // in-edges per warp tile
constexpr uint32_t PR_LANE = 16;       // consecutive in-edges per lane
constexpr uint32_t PR_THREADS = 1024;  // k_pr_pull: one block per SM
constexpr uint32_t PR_HOT_CAP = 32768; // hot sources in shared memory (128 KB)
constexpr uint32_t PR_HOT_BIT = 0x80000000u;
constexpr int PR_HIST = 128;           // out-degree histogram buckets (4 per octave)
constexpr uint32_t PR_FINE = 4096;     // exact-degree bins when the cap falls inside a bucket
static_assert(PR_TILE == 32 * PR_LANE, "a tile is one warp's lanes");

// Tile piece flags.
constexpr uint32_t F_HEAD = 1u;          // the tile's first in-edge continues a list from earlier tiles
constexpr uint32_t F_HEAD_THROUGH = 2u;  // ... and that list runs past the tile's end
constexpr uint32_t F_TAIL = 4u;          // a list opened in this tile runs past its end

struct PrArgs {
  const uint32_t* src;
  const uint32_t* start_bits;
  const uint32_t* tile_nz;
  const uint32_t* contrib;  // [V] contributions (FP32 bits) by vertex: the compute partition's array
  const float* hot_val;
  float* part;
  uint4* piece;
  uint32_t* pflags;
  uint64_t E, T;
  uint32_t H;
};

struct PrUpd {
  const float* part;
  const uint32_t* voff;  // [V+1] vertex v's in-lists are part[voff[v] .. voff[v+1])
  const uint32_t* hot_base;
  float* hot_val;
  double* resid_part;
  uint32_t H, hot_deg;
  float damping, base;
};

struct PrRound {
  const double* resid_part;
  uint32_t nparts;
  uint32_t V;
  uint32_t max_rounds;
  double tol;
  unsigned long long E, bytes, refbytes, actives, launches;
};

__device__ __forceinline__ uint4 ld_stream_v4(const uint32_t* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}

// ------------------------------------------------------------- edge-map --
// One source value: a hot source from the shared-memory copy, the others from
// global memory.  (One generic load for both kinds measured slower: 0.868 ms
// against 0.840 ms per RMAT-24 pull.)
__device__ __forceinline__ float pr_gather(const float* s_hot, const uint32_t* contrib, uint32_t code) {
  return (code & PR_HOT_BIT) ? s_hot[code & ~PR_HOT_BIT] : __uint_as_float(__ldg(contrib + code));
}

// One 512-edge tile (warp-wide).  kFull: all 512 in-edges exist (every tile
// but the last); the lane count n is then the constant 16.
template <bool kFull>
__device__ __forceinline__ void pr_tile(const PrArgs& a, const float* s_hot, uint64_t t) {
  const uint32_t lane = lane_id();
  const uint64_t e0 = t * PR_TILE;
  const uint64_t ea = e0 + (uint64_t)lane * PR_LANE;
  const uint32_t n = kFull ? PR_LANE : (ea < a.E ? (uint32_t)(a.E - ea < PR_LANE ? a.E - ea : PR_LANE) : 0u);
  // the lane's in-edges: hot index or source slot
  uint32_t code[PR_LANE];
  if (kFull) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint4 x = ld_stream_v4(a.src + ea + 4 * q);  // ea is a multiple of 16: 16-byte aligned
      code[4 * q] = x.x;
      code[4 * q + 1] = x.y;
      code[4 * q + 2] = x.z;
      code[4 * q + 3] = x.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < (int)PR_LANE; ++j) code[j] = (uint32_t)j < n ? __ldg(a.src + ea + j) : 0u;
  }
  // Start bits of the lane's edges (bit j: edge ea+j opens an in-list).  The
  // words of a tile are [e0/32, e0/32 + 16); the array is padded by one tile
  // of zero words, so the reads below stay in bounds for every tile.
  const uint32_t word = __ldg(a.start_bits + (e0 >> 5) + (lane >> 1));
  const uint32_t data_mask = n >= PR_LANE ? 0xFFFFu : ((1u << n) - 1u);
  const uint32_t sb = (word >> ((lane & 1u) * 16u)) & data_mask;
  const uint32_t sbv = sb | (~data_mask & 0xFFFFu);  // past the data counts as a start
  // index of the in-list holding the lane's first edge
  const uint32_t cnt = __popc(sb);
  const uint32_t incl = warp_incl_scan(cnt);
  const uint32_t k_first = __ldg(a.tile_nz + t) + (incl - cnt) + (sb & 1u) - 1u;
  // does the edge after the lane's last one open an in-list (or end the data)?
  uint32_t next_start = __shfl_down_sync(FULL, sbv, 1) & 1u;
  if (lane == 31) next_start = (e0 + PR_TILE >= a.E) ? 1u : (__ldg(a.start_bits + (e0 >> 5) + 16) & 1u);
  const uint32_t lane0_sb = __shfl_sync(FULL, sb, 0);
  float v[PR_LANE];
#pragma unroll
  for (int j = 0; j < (int)PR_LANE; ++j) v[j] = (kFull || (uint32_t)j < n) ? pr_gather(s_hot, a.contrib, code[j]) : 0.0f;
  // fold in stored order; a list that opens in this lane and closes in it is
  // complete
  uint32_t k = k_first;
  bool started = (sb & 1u) != 0;
  float s = 0.0f, c = 0.0f;
  bool has_left = false;
  float left = 0.0f;
#pragma unroll
  for (int j = 0; j < (int)PR_LANE; ++j) {
    if (kFull || (uint32_t)j < n) {
      if (j > 0 && ((sb >> j) & 1u)) {
        const float val = __fsub_rn(s, c);
        if (started)
          a.part[k] = val;
        else {
          has_left = true;  // closes a list that opened before this lane
          left = val;
        }
        ++k;
        s = 0.0f;
        c = 0.0f;
        started = true;
      }
      kahan_add(s, c, v[j]);
    }
  }
  bool through = false, has_right = false;
  if (n > 0) {
    if (next_start) {
      const float val = __fsub_rn(s, c);
      if (started)
        a.part[k] = val;
      else {
        has_left = true;
        left = val;
      }
    } else if (started) {
      has_right = true;  // opened here, continues in the next lane
    } else {
      through = true;  // the whole lane lies inside one list
    }
  }
  const float piece = has_left ? left : (through ? __fsub_rn(s, c) : 0.0f);
  const uint32_t thr_mask = __ballot_sync(FULL, through);
  if (thr_mask == FULL) {
    // The whole tile lies inside the list it starts in (an interior tile of
    // a long in-list): the head is the 32 lane pieces folded in lane order,
    // the same steps the walk below takes, with every lane folding the
    // broadcast pieces instead of one lane stepping through the warp.
    float hs = 0.0f, hc = 0.0f;
#pragma unroll
    for (int i = 0; i < 32; ++i) kahan_add(hs, hc, __shfl_sync(FULL, piece, i));
    if (lane == 31) {
      a.piece[t] = make_uint4(__float_as_uint(__fsub_rn(hs, hc)), __float_as_uint(s), __float_as_uint(c), k);
      a.pflags[t] = F_HEAD | F_HEAD_THROUGH;
    }
    return;
  }
  // Chains across lanes, walked in lane order: lanes 0..30 continue their open
  // list into the next lanes; lane 31 (whose open list, if any, is the tile's
  // tail) walks the tile's head: the list the tile starts inside.
  bool open;
  uint32_t cur;
  float ws, wc;
  if (lane < 31) {
    open = has_right;
    cur = lane + 1;
    ws = s;
    wc = c;
  } else {
    open = (lane0_sb & 1u) == 0;  // lane 0 always holds data
    cur = 0;
    ws = 0.0f;
    wc = 0.0f;
  }
  bool my_tail = lane == 31 && has_right;
  float ts = s, tc = c;
  uint32_t tk = k;
  float head_val = 0.0f;
  bool head_through = false;
  while (__any_sync(FULL, open)) {
    const float x = __shfl_sync(FULL, piece, cur & 31u);
    if (open) {
      kahan_add(ws, wc, x);
      const bool thr = (thr_mask >> (cur & 31u)) & 1u;
      if (!thr) {  // the list closes in lane `cur`
        if (lane < 31)
          a.part[k] = __fsub_rn(ws, wc);
        else
          head_val = __fsub_rn(ws, wc);
        open = false;
      } else if (cur == 31) {  // the list runs past the tile's end
        if (lane < 31) {
          my_tail = true;
          ts = ws;
          tc = wc;
          tk = k;
        } else {
          head_val = __fsub_rn(ws, wc);
          head_through = true;
        }
        open = false;
      } else {
        ++cur;
      }
    }
  }
  const uint32_t tail_mask = __ballot_sync(FULL, my_tail);
  const int tl = tail_mask ? __ffs(tail_mask) - 1 : 31;
  const float t_s = __shfl_sync(FULL, ts, tl), t_c = __shfl_sync(FULL, tc, tl);
  const uint32_t t_k = __shfl_sync(FULL, tk, tl);
  if (lane == 31) {
    const bool hc = (lane0_sb & 1u) == 0;
    a.piece[t] = make_uint4(__float_as_uint(head_val), __float_as_uint(t_s), __float_as_uint(t_c), t_k);
    a.pflags[t] = (hc ? F_HEAD : 0u) | (head_through ? F_HEAD_THROUGH : 0u) | (tail_mask ? F_TAIL : 0u);
  }
}

// One warp per 512-edge tile (static interleaved assignment), one block of
// 1024 threads per SM with the hot contributions in shared memory.
__global__ void __launch_bounds__(PR_THREADS, 1) k_pr_pull(PrArgs a) {
  extern __shared__ float s_hot[];
  for (uint32_t i = threadIdx.x; i < a.H; i += blockDim.x) s_hot[i] = a.hot_val[i];
  __syncthreads();
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t full = a.E / PR_TILE;  // tiles with 512 in-edges
  for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < a.T; t += nw) {
    if (t < full)
      pr_tile<true>(a, s_hot, t);
    else
      pr_tile<false>(a, s_hot, t);
  }
}

// Lists that cross tiles: the tile that opened the list holds the running
// Kahan state at its end; the heads of the following tiles are added in tile
// order until a tile where the list closes.  A warp takes 32 consecutive
// tiles; a list that closes in the next tile is finished by its own lane,
// longer ones by the whole warp, 32 tiles per step.
__global__ void __launch_bounds__(256) k_pr_fix(PrArgs a) {
  const uint32_t lane = lane_id();
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t g0 = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; g0 < a.T;
       g0 += nw * 32) {
    const uint64_t t = g0 + lane;
    bool open = false;
    float s = 0.0f, c = 0.0f;
    uint32_t k = 0;
    unsigned long long u = t + 1;
    if (t < a.T && (a.pflags[t] & F_TAIL)) {
      const uint4 pc = a.piece[t];
      s = __uint_as_float(pc.y);
      c = __uint_as_float(pc.z);
      k = pc.w;
      open = true;
      if (u < a.T) {  // always: an open tail is followed by a tile holding the rest
        const uint32_t fu = a.pflags[u];
        kahan_add(s, c, __uint_as_float(a.piece[u].x));
        if (!(fu & F_HEAD_THROUGH)) {
          a.part[k] = __fsub_rn(s, c);
          open = false;
        } else {
          ++u;
        }
      } else {
        a.part[k] = __fsub_rn(s, c);
        open = false;
      }
    }
    uint32_t longm = __ballot_sync(FULL, open);
    while (longm) {
      const int L = __ffs(longm) - 1;
      longm &= longm - 1;
      float ws = __shfl_sync(FULL, s, L), wc = __shfl_sync(FULL, c, L);
      const uint32_t wk = __shfl_sync(FULL, k, L);
      unsigned long long wu = __shfl_sync(FULL, u, L);
      for (;;) {
        const unsigned long long q = wu + lane;
        const bool in = q < a.T;
        const uint32_t fq = in ? a.pflags[q] : 0u;
        const float hq = in ? __uint_as_float(a.piece[q].x) : 0.0f;
        const uint32_t thr = __ballot_sync(FULL, in && (fq & F_HEAD_THROUGH));
        const int last = thr == FULL ? 31 : __ffs(~thr) - 1;
        const bool end_in_data = wu + (unsigned long long)last < a.T;
        for (int i = 0; i <= last; ++i) {
          const float x = __shfl_sync(FULL, hq, i);
          if (wu + (unsigned long long)i < a.T) kahan_add(ws, wc, x);
        }
        if (thr != FULL || !end_in_data) {
          if (lane == 0) a.part[wk] = __fsub_rn(ws, wc);
          break;
        }
        wu += 32;
      }
    }
  }
}

// -------------------------------------------------------- update / fwd --
// Per vertex: the partial sums of its slots' in-lists (stored contiguously,
// partition order) merged with Kahan (an exactly zero partial adds nothing and
// is skipped), the new rank, the L1 residual, and the new contribution in the
// vertex's entry of vertex_properties, which the next pull gathers from (and
// in the hot array when the vertex is hot).
// Warps take 32 consecutive vertices (the hot rank is a ballot prefix), two
// such words per step with every independent load issued before the partial
// sums, whose addresses depend on the list offsets.
// Residual: |new - old| of one vertex is exact in FP32 whenever the two ranks
// are within a factor of two (Sterbenz), so each thread sums its vertices'
// differences with a compensated FP32 sum, and the threads' sums are reduced in
// FP64 (block partials here, the blocks in k_pr_round_end), in a fixed order.
constexpr int UPD_WORDS = 2;

__global__ void __launch_bounds__(256) k_pr_update(DevGraph g, DevState st, PrUpd u) {
  __shared__ double s_red[8];
  float rs = 0.0f, rc = 0.0f;
  const uint32_t lane = lane_id();
  const uint32_t nwords = (g.V + 31) / 32;
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t w0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * UPD_WORDS; w0 < nwords;
       w0 += nw * UPD_WORDS) {
    uint32_t v[UPD_WORDS], deg[UPD_WORDS], b[UPD_WORDS], e[UPD_WORDS];
    float ov[UPD_WORDS];
    bool valid[UPD_WORDS];
#pragma unroll
    for (int q = 0; q < UPD_WORDS; ++q) {
      v[q] = (w0 + q) * 32 + lane;
      valid[q] = w0 + q < nwords && v[q] < g.V;
      deg[q] = valid[q] ? __ldg(&g.outdeg[v[q]]) : 0u;
      b[q] = valid[q] ? __ldg(&u.voff[v[q]]) : 0u;
      e[q] = valid[q] ? __ldg(&u.voff[v[q] + 1]) : 0u;
      ov[q] = valid[q] ? st.ranks[v[q]] : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < UPD_WORDS; ++q) {
      float s = 0.0f, c = 0.0f;
      for (uint32_t i = b[q]; i < e[q]; i += 4) {
        uint32_t x[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = i + k < e[q] ? __float_as_uint(u.part[i + k]) : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (x[k] != 0u) kahan_add(s, c, __uint_as_float(x[k]));
      }
      const bool hot = valid[q] && u.H != 0 && deg[q] != 0 && deg[q] >= u.hot_deg;
      const uint32_t hm = __ballot_sync(FULL, hot);
      if (valid[q]) {
        const float nv = __fadd_rn(deg[q] ? u.base : 0.0f, __fsub_rn(s, c));
        kahan_add(rs, rc, fabsf(__fsub_rn(nv, ov[q])));
        st.ranks[v[q]] = nv;
        const float contrib = deg[q] ? __fdiv_rn(__fmul_rn(u.damping, nv), (float)deg[q]) : 0.0f;
        const uint32_t cb = __float_as_uint(contrib);
        st.prop[v[q]] = cb;
        if (hot) u.hot_val[u.hot_base[w0 + q] + __popc(hm & ((1u << lane) - 1u))] = contrib;
      }
    }
  }
  double r = (double)rs - (double)rc;
#pragma unroll
  for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(FULL, r, o);
  if (lane == 0) s_red[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (uint32_t i = 0; i < (blockDim.x >> 5); ++i) t += s_red[i];
    u.resid_part[blockIdx.x] = t;
  }
}

// Initial contributions (init()'s vertex_properties) of the hot sources to
// the hot array.
__global__ void __launch_bounds__(256) k_pr_fwd(DevGraph g, DevState st, PrUpd u) {
  const uint32_t lane = lane_id();
  const uint32_t nwords = (g.V + 31) / 32;
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nwords; w += nw) {
    const uint32_t v = w * 32 + lane;
    const bool valid = v < g.V;
    const uint32_t deg = valid ? g.outdeg[v] : 0u;
    const bool hot = valid && u.H != 0 && deg != 0 && deg >= u.hot_deg;
    const uint32_t hm = __ballot_sync(FULL, hot);
    if (valid) {
      if (hot) u.hot_val[u.hot_base[w] + __popc(hm & ((1u << lane) - 1u))] = __uint_as_float(st.prop[v]);
    }
  }
}

// Residual (block partials summed in block order), round statistics and the
// loop condition: continue while the residual per vertex is at least the
// tolerance and the round cap is not reached.
__global__ void __launch_bounds__(256) k_pr_round_end(DevState st, PrRound pr, cudaGraphConditionalHandle h,
                                                      int use_cond) {
  __shared__ double s_sum[256];
  double x = 0.0;
  for (uint32_t i = threadIdx.x; i < pr.nparts; i += blockDim.x) x += pr.resid_part[i];
  s_sum[threadIdx.x] = x;
  __syncthreads();
  for (uint32_t o = blockDim.x / 2; o; o >>= 1) {
    if (threadIdx.x < o) s_sum[threadIdx.x] += s_sum[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double total = s_sum[0];
    st.counters[C_RESID] = (unsigned long long)__double_as_longlong(total);
    const unsigned long long r = st.counters[C_ROUNDS] + 1;
    st.counters[C_ROUNDS] = r;
    st.counters[C_PULL_ROUNDS] += 1;
    st.counters[C_EDGES] += pr.E;
    st.counters[C_BYTES] += pr.bytes;
    st.counters[C_REFBYTES] += pr.refbytes;
    st.counters[C_ACTIVE] = pr.actives;
    st.counters[C_ACTIVE_TOTAL] += pr.actives;
    st.counters[C_LAUNCHES] += pr.launches;
    const bool conv = total / (double)(pr.V ? pr.V : 1u) < pr.tol;
    st.counters[C_FRONTIER] = conv ? 0ull : pr.actives;
    if (use_cond) cudaGraphSetConditional(h, (!conv && r < pr.max_rounds) ? 1u : 0u);
  }
}

__global__ void k_pr_seed(DevState st, unsigned long long rounds, unsigned long long actives_total) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  st.counters[C_ROUNDS] = rounds;
  st.counters[C_PULL_ROUNDS] = rounds;
  st.counters[C_ACTIVE_TOTAL] = actives_total;
  st.counters[C_LAUNCHES] = 0;
}

// ----------------------------------------------------------------- set-up --
__device__ __forceinline__ uint32_t deg_bucket(uint32_t d) {
  const uint32_t m = 31u - __clz(d);
  const uint32_t f = m >= 2 ? (d >> (m - 2)) & 3u : (d << (2 - m)) & 3u;
  return 4u * m + f;
}

// Histogram of the out-degrees of non-dangling vertices (count and smallest
// degree per bucket; buckets grow with the degree).
__global__ void __launch_bounds__(256) k_pr_deg_hist(DevGraph g, uint32_t* cnt, uint32_t* dmin) {
  __shared__ uint32_t s_cnt[PR_HIST], s_min[PR_HIST];
  for (uint32_t i = threadIdx.x; i < PR_HIST; i += blockDim.x) {
    s_cnt[i] = 0;
    s_min[i] = 0xFFFFFFFFu;
  }
  __syncthreads();
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x) {
    const uint32_t d = g.outdeg[v];
    if (d) {
      const uint32_t b = deg_bucket(d);
      atomicAdd(&s_cnt[b], 1u);
      atomicMin(&s_min[b], d);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < PR_HIST; i += blockDim.x)
    if (s_cnt[i]) {
      atomicAdd(&cnt[i], s_cnt[i]);
      atomicMin(&dmin[i], s_min[i]);
    }
}

// Exact out-degree counts in [lo, lo + n): the histogram bucket that the hot
// set's cap falls in, split so that the cut lands on an exact degree.
__global__ void __launch_bounds__(256) k_pr_deg_fine(DevGraph g, uint32_t lo, uint32_t n, uint32_t* cnt) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x) {
    const uint32_t d = g.outdeg[v] - lo;  // wraps for degrees below lo
    if (d < n) atomicAdd(&cnt[d], 1u);
  }
}

__global__ void __launch_bounds__(256) k_pr_hot_words(DevGraph g, uint32_t hot_deg, uint32_t H, uint32_t* words) {
  const uint32_t lane = lane_id();
  const uint32_t nwords = (g.V + 31) / 32;
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nwords; w += nw) {
    const uint32_t v = w * 32 + lane;
    const uint32_t deg = v < g.V ? g.outdeg[v] : 0u;
    const uint32_t m = __ballot_sync(FULL, H != 0 && deg != 0 && deg >= hot_deg);
    if (lane == 0) words[w] = __popc(m);
  }
}

// Code of every owned slot: the hot rank with the top bit, or the slot's vertex
// (the pull gathers cold sources' contributions by vertex).
__global__ void __launch_bounds__(256) k_pr_slot_code(DevGraph g, DevState st, uint32_t hot_deg, uint32_t H,
                                                      const uint32_t* hot_base, uint32_t* code) {
  const uint32_t lane = lane_id();
  const uint32_t nwords = (g.V + 31) / 32;
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nwords; w += nw) {
    const uint32_t v = w * 32 + lane;
    const bool valid = v < g.V;
    const uint32_t deg = valid ? g.outdeg[v] : 0u;
    const bool hot = valid && H != 0 && deg != 0 && deg >= hot_deg;
    const uint32_t m = __ballot_sync(FULL, hot);
    if (valid) {
      const uint32_t s = st.own_slot[v];
      code[s] = hot ? (PR_HOT_BIT | (hot_base[w] + __popc(m & ((1u << lane) - 1u)))) : v;
    }
  }
}

// Per vertex: its non-empty in-lists (one per partition at most).
__global__ void __launch_bounds__(256) k_pr_list_count(DevGraph g, uint32_t* vcnt) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.S; s += (uint64_t)gridDim.x * blockDim.x)
    if (g.in_off[s + 1] > g.in_off[s]) atomicAdd(vcnt + g.slot_gid[s], 1u);
}

// Vertex-major position of partition p's non-empty in-lists (partitions run
// in order, so every vertex lists partition 0's first) and their lengths.
__global__ void __launch_bounds__(256) k_pr_list_pos(DevGraph g, uint64_t s0, uint64_t s1, const uint32_t* voff,
                                                     uint32_t* cur, uint32_t* lpos, uint32_t* llen) {
  for (uint64_t s = s0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < s1;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t d = g.in_off[s + 1] - g.in_off[s];
    if (!d) continue;
    const uint32_t gid = g.slot_gid[s];
    const uint32_t j = voff[gid] + cur[gid];
    cur[gid] += 1;  // a vertex has at most one slot per partition
    lpos[s] = j;
    llen[j] = d;
  }
}

// Shift of every edge from the slot-ordered in-edge view to the
// vertex-major list order: +shift at a list's first edge, -shift past its
// last (an add-scan then gives each edge its list's shift, mod 2^32).
__global__ void __launch_bounds__(256) k_pr_shift_marks(DevGraph g, const uint32_t* lpos, const uint32_t* loff,
                                                        uint32_t* marks) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.S; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = g.in_off[s], b = g.in_off[s + 1];
    if (b == a) continue;
    const uint32_t shift = loff[lpos[s]] - a;
    atomicAdd(marks + a, shift);
    atomicAdd(marks + b, 0u - shift);
  }
}

// Every in-edge to its vertex-major place, as its source's code.
__global__ void __launch_bounds__(256) k_pr_move(const uint32_t* __restrict__ in_src, uint64_t E,
                                                 const uint32_t* __restrict__ shift, const uint32_t* __restrict__ code,
                                                 uint32_t* out) {
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x)
    out[(uint32_t)e + shift[e]] = code[in_src[e]];
}

__global__ void __launch_bounds__(256) k_pr_start_bits(const uint32_t* loff, uint64_t n, uint32_t* start_bits) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = loff[j];
    atomicOr(start_bits + (a >> 5), 1u << (a & 31));
  }
}

__global__ void __launch_bounds__(256) k_pr_tile_count(const uint32_t* start_bits, uint64_t T, uint32_t* out) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t c = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) c += __popc(start_bits[t * 16 + i]);
    out[t] = c;
  }
}

// Set-up scratch: slices of one device buffer kept by the ctx (allocated at
// the first set-up, and again only if a layout ever needs more), so that a
// set-up after every upload allocates nothing.
struct Tmp {
  grd_ctx* ctx;
  char* base = nullptr;
  size_t cap = 0, used = 0;
  explicit Tmp(grd_ctx* c) : ctx(c) {}
  int reserve(size_t words) {
    const size_t bytes = words * sizeof(uint32_t) + 64 * 256;  // slices are 256-byte aligned
    PrPullState& P = ctx->pr;
    if (P.scratch_cap < bytes) {
      void* d = nullptr;
      TRY(grd_dev_alloc_bytes(ctx, &d, bytes));
      P.scratch = static_cast<char*>(d);
      P.scratch_cap = bytes;
    }
    base = P.scratch;
    cap = P.scratch_cap;
    used = 0;
    return GRD_OK;
  }
  template <class T>
  int get(T** p, size_t count) {
    const size_t bytes = ((sizeof(T) * std::max<size_t>(count, 1)) + 255) / 256 * 256;
    if (used + bytes > cap) {
      ctx->err = "PageRank set-up scratch too small";
      return GRD_E_INVALID;
    }
    *p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return GRD_OK;
  }
};

uint32_t grid(const grd_ctx* ctx, uint64_t n, uint32_t per_sm = 8) {
  const uint64_t b = (n + 255) / 256;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(b, (uint64_t)ctx->num_sms * per_sm));
}

// Builds the derived arrays when the resident layout changed since the last
// build (uploads, ingests and in-edge builds bump ctx->layout_gen).
int pr_prepare(grd_ctx* ctx) {
  PrPullState& P = ctx->pr;
  if (P.layout_gen == ctx->layout_gen) return GRD_OK;
  const Layout& L = ctx->L;
  const uint64_t V = L.V, S = L.S, E = L.E;
  const uint64_t T = (E + PR_TILE - 1) / PR_TILE;
  const uint64_t W = 16 * (T + 1);  // start-bit words, one zero tile of padding
  if (S >= PR_HOT_BIT) {
    ctx->err = "PR_PULL needs fewer than 2^31 slots";
    return GRD_E_INVALID;
  }
  cudaStream_t s = ctx->stream;
  DevGraph& g = ctx->g;
  // sizes are fixed for a ctx (an ingest keeps V, E, M and the slot counts);
  // allocate on first use, or again if they ever grow
  if (!P.src || E > P.cap_E || S > P.cap_S || V > P.cap_V || T > P.cap_T) {
    auto alloc = [&](auto** q, uint64_t count) -> int {
      void* d = nullptr;
      TRY(grd_dev_alloc_bytes(ctx, &d, sizeof(**q) * std::max<uint64_t>(count, 4)));
      *q = static_cast<std::remove_reference_t<decltype(*q)>>(d);
      return GRD_OK;
    };
    TRY(alloc(&P.src, E));
    TRY(alloc(&P.start_bits, W));
    TRY(alloc(&P.tile_nz, T + 1));
    TRY(alloc(&P.piece, T));
    TRY(alloc(&P.piece_flags, T));
    TRY(alloc(&P.part, S));
    TRY(alloc(&P.vmap_off, V + 1));
    TRY(alloc(&P.hot_base, V / 32 + 2));
    TRY(alloc(&P.hot_val, (uint64_t)PR_HOT_CAP));
    if (!P.resid_part) {
      P.update_blocks = (uint32_t)ctx->num_sms * 8;
      TRY(alloc(&P.resid_part, P.update_blocks));
    }
    P.cap_E = E;
    P.cap_S = S;
    P.cap_V = V;
    P.cap_T = T;
  }

  Tmp tmp(ctx);
  TRY(tmp.reserve(2 * PR_HIST + PR_FINE + (V / 32 + 2) + (V + 1) + V + 4 * S + 1 + (T + 1) + (E + 1)));
  // (1) hot set: the highest out-degrees, at most PR_HOT_CAP vertices, cut at
  // a histogram bucket boundary, then inside the next bucket at an exact
  // degree (RMAT's degree plateaus put tens of thousands of vertices in one
  // bucket: at RMAT-24 the bucket cut alone keeps 12 959 hot sources, the
  // exact cut about 32 700)
  uint32_t *hist = nullptr;
  TRY(tmp.get(&hist, 2 * PR_HIST));
  CK(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * PR_HIST, s));
  CK(cudaMemsetAsync(hist + PR_HIST, 0xFF, sizeof(uint32_t) * PR_HIST, s));
  k_pr_deg_hist<<<grid(ctx, V), 256, 0, s>>>(g, hist, hist + PR_HIST);
  CK_LAUNCH();
  uint32_t h_hist[2 * PR_HIST];
  CK(cudaMemcpyAsync(h_hist, hist, sizeof(h_hist), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  uint64_t nondangling = 0, cum = 0;
  uint32_t H = 0, hot_deg = 0;
  for (int b = 0; b < PR_HIST; ++b) nondangling += h_hist[b];
  int cut = -1;  // the bucket the cap falls in
  for (int b = PR_HIST - 1; b >= 0; --b) {
    if (!h_hist[b]) continue;
    if (cum + h_hist[b] > PR_HOT_CAP) {
      cut = b;
      break;
    }
    cum += h_hist[b];
    H = (uint32_t)cum;
    hot_deg = h_hist[PR_HIST + b];
  }
  if (cut >= 8) {  // bucket 4m + f holds the degrees [(4 + f) << (m - 2), (5 + f) << (m - 2))
    const uint32_t m = (uint32_t)cut / 4, f = (uint32_t)cut % 4;
    const uint32_t lo = (4u + f) << (m - 2), width = 1u << (m - 2);
    if (width > 1 && width <= PR_FINE) {
      uint32_t* fine = nullptr;
      TRY(tmp.get(&fine, PR_FINE));
      CK(cudaMemsetAsync(fine, 0, sizeof(uint32_t) * width, s));
      k_pr_deg_fine<<<grid(ctx, V), 256, 0, s>>>(g, lo, width, fine);
      CK_LAUNCH();
      std::vector<uint32_t> h_fine(width);
      CK(cudaMemcpyAsync(h_fine.data(), fine, sizeof(uint32_t) * width, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      for (int d = (int)width - 1; d >= 0; --d) {
        if (!h_fine[d]) continue;
        if (cum + h_fine[d] > PR_HOT_CAP) break;
        cum += h_fine[d];
        H = (uint32_t)cum;
        hot_deg = lo + (uint32_t)d;
      }
    }
  }
  if (H == 0) hot_deg = 0;
  // (2) hot ranks: per 32-vertex word, then its exclusive scan
  const uint64_t nwords = (V + 31) / 32;
  {
    uint32_t* words = nullptr;
    TRY(tmp.get(&words, nwords + 1));
    k_pr_hot_words<<<grid(ctx, V), 256, 0, s>>>(g, hot_deg, H, words);
    CK_LAUNCH();
    TRY(grd_scan_add_u32(ctx, words, P.hot_base, nwords, true));
  }
  // (3) non-empty in-lists in vertex-major order (each vertex's lists in
  // partition order): positions, lengths, edge offsets
  uint32_t *vcnt = nullptr, *cur = nullptr, *lpos = nullptr, *llen = nullptr, *loff = nullptr, *tcnt = nullptr;
  TRY(tmp.get(&vcnt, V + 1));
  TRY(tmp.get(&cur, V));
  TRY(tmp.get(&lpos, S));
  TRY(tmp.get(&llen, S));
  TRY(tmp.get(&loff, S + 1));
  TRY(tmp.get(&tcnt, T + 1));
  CK(cudaMemsetAsync(vcnt, 0, sizeof(uint32_t) * (V + 1), s));
  CK(cudaMemsetAsync(cur, 0, sizeof(uint32_t) * std::max<uint64_t>(V, 1), s));
  k_pr_list_count<<<grid(ctx, S), 256, 0, s>>>(g, vcnt);
  CK_LAUNCH();
  TRY(grd_scan_add_u32(ctx, vcnt, P.vmap_off, V, true));
  for (uint32_t p = 0; p < L.M; ++p) {
    const uint64_t s0 = L.slot_base[p], s1 = p + 1 < L.M ? L.slot_base[p + 1] : S;
    if (s1 > s0) k_pr_list_pos<<<grid(ctx, s1 - s0), 256, 0, s>>>(g, s0, s1, P.vmap_off, cur, lpos, llen);
  }
  CK_LAUNCH();
  uint32_t s_nz = 0;
  CK(cudaMemcpyAsync(&s_nz, P.vmap_off + V, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  TRY(grd_scan_add_u32(ctx, llen, loff, s_nz, true));
  // (4) the in-edges moved to that order, each as its source's code (hot rank
  // or slot), and the start bit of every list
  {
    uint32_t *code = nullptr, *marks = nullptr;
    TRY(tmp.get(&code, S));
    TRY(tmp.get(&marks, E + 1));
    k_pr_slot_code<<<grid(ctx, V), 256, 0, s>>>(g, ctx->st, hot_deg, H, P.hot_base, code);
    CK(cudaMemsetAsync(marks, 0, sizeof(uint32_t) * (E + 1), s));
    k_pr_shift_marks<<<grid(ctx, S), 256, 0, s>>>(g, lpos, loff, marks);
    CK_LAUNCH();
    TRY(grd_scan_u32(ctx, marks, marks, E, true, false));
    k_pr_move<<<grid(ctx, E, 16), 256, 0, s>>>(g.in_src, E, marks, code, P.src);
    CK(cudaMemsetAsync(P.start_bits, 0, sizeof(uint32_t) * W, s));
    k_pr_start_bits<<<grid(ctx, s_nz), 256, 0, s>>>(loff, s_nz, P.start_bits);
    CK_LAUNCH();
  }
  k_pr_tile_count<<<grid(ctx, T), 256, 0, s>>>(P.start_bits, T, tcnt);
  CK_LAUNCH();
  TRY(grd_scan_add_u32(ctx, tcnt, P.tile_nz, T, true));
  CK(cudaStreamSynchronize(s));
  P.E = E;
  P.T = T;
  P.S_nz = s_nz;
  P.H = H;
  P.hot_deg = hot_deg;
  P.nondangling = nondangling;
  P.layout_gen = ctx->layout_gen;
  return GRD_OK;
}

PrArgs pr_args(grd_ctx* ctx) {
  PrPullState& P = ctx->pr;
  return PrArgs{P.src, P.start_bits, P.tile_nz, ctx->st.prop, P.hot_val, P.part, P.piece, P.piece_flags,
                P.E, P.T, P.H};
}

PrUpd pr_upd(grd_ctx* ctx) {
  PrPullState& P = ctx->pr;
  const double d = ctx->params.damping;
  return PrUpd{P.part, P.vmap_off, P.hot_base, P.hot_val, P.resid_part, P.H, P.hot_deg, (float)d,
               (float)(1.0 - d)};
}

// Bytes of one round by the sync's wire format: each direction sends every
// partition's bitvector plus 4 bytes per value (the forward sync one per
// non-dangling vertex, the backward sync one per non-empty in-list).
PrRound pr_round(grd_ctx* ctx) {
  PrPullState& P = ctx->pr;
  const DevGraph& g = ctx->g;
  PrRound r{};
  r.resid_part = P.resid_part;
  r.nparts = P.update_blocks;
  r.V = ctx->L.V;
  r.max_rounds = ctx->params.max_rounds;
  r.tol = ctx->params.tolerance;
  r.E = P.E;
  r.bytes = 2ull * g.bv_bytes + 4ull * (P.nondangling + P.S_nz);
  r.refbytes = 2ull * g.bv_refbytes + 4ull * (P.nondangling + P.S_nz);
  r.actives = P.nondangling;
  r.launches = 4;
  return r;
}

size_t pull_smem(const grd_ctx* ctx) { return sizeof(float) * (size_t)ctx->pr.H; }

int set_pull_smem(grd_ctx* ctx) {
  CK(cudaFuncSetAttribute(k_pr_pull, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(float) * PR_HOT_CAP)));
  return GRD_OK;
}

int enqueue_fwd(grd_ctx* ctx) {
  k_pr_fwd<<<grid(ctx, ctx->L.V), 256, 0, ctx->stream>>>(ctx->g, ctx->st, pr_upd(ctx));
  CK_LAUNCH();
  return GRD_OK;
}

// timed: CUDA events around the pull kernel (profiled host-driven runs).
int enqueue_edge_map(grd_ctx* ctx, bool timed = false) {
  if (ctx->pr.T) {
    TRY(set_pull_smem(ctx));
    if (timed) CK(cudaEventRecord(ctx->ev[5], ctx->stream));
    k_pr_pull<<<ctx->num_sms, PR_THREADS, pull_smem(ctx), ctx->stream>>>(pr_args(ctx));
    if (timed) CK(cudaEventRecord(ctx->ev[6], ctx->stream));
    const uint64_t groups = (ctx->pr.T + 31) / 32;
    k_pr_fix<<<(uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((groups + 7) / 8, (uint64_t)ctx->num_sms * 8)),
               256, 0, ctx->stream>>>(pr_args(ctx));
    CK_LAUNCH();
  }
  ctx->stats.kernel_launches += 2;
  return GRD_OK;
}

int enqueue_update(grd_ctx* ctx, cudaGraphConditionalHandle h, int use_cond) {
  k_pr_update<<<ctx->pr.update_blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, pr_upd(ctx));
  k_pr_round_end<<<1, 256, 0, ctx->stream>>>(ctx->st, pr_round(ctx), h, use_cond);
  CK_LAUNCH();
  ctx->stats.kernel_launches += 2;
  return GRD_OK;
}

double resid_of(const grd_ctx* ctx) {
  double r;
  const unsigned long long bits = ctx->h_counters[C_RESID];
  std::memcpy(&r, &bits, sizeof(r));
  return r / (double)std::max<uint32_t>(ctx->L.V, 1);
}

// Host-driven iteration end: statistics from the counters.
int read_round(grd_ctx* ctx) {
  TRY(grd_read_counters(ctx));  // synchronises the stream
  ctx->stats.last_residual = resid_of(ctx);
  ctx->stats.pull_rounds++;
  return GRD_OK;
}

int build_graph(grd_ctx* ctx) {
  const grd_stats saved = ctx->stats;
  cudaGraph_t top = nullptr;
  CK(cudaGraphCreate(&top, 0));
  ctx->pr_graph = top;
  cudaGraphConditionalHandle wh;
  CK(cudaGraphConditionalHandleCreate(&wh, top, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = wh;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, top, nullptr, nullptr, 0, &p));
  cudaGraph_t body = p.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_edge_map(ctx);
  if (rc == GRD_OK) rc = enqueue_update(ctx, wh, 1);
  cudaGraph_t out = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &out);
  ctx->stats = saved;
  if (rc != GRD_OK) return rc;
  CK(e);
  CK(cudaGraphInstantiate(&ctx->pr_exec, top, 0));
  return GRD_OK;
}

}  // namespace

void grd_ctx_release_extras(grd_ctx* ctx) { grd_pull_graph_release(ctx); }

void grd_pull_graph_release(grd_ctx* ctx) {
  if (ctx->pr_exec) cudaGraphExecDestroy(ctx->pr_exec);
  if (ctx->pr_graph) cudaGraphDestroy(ctx->pr_graph);
  ctx->pr_exec = nullptr;
  ctx->pr_graph = nullptr;
}

int grd_pull_stage(grd_ctx* ctx, int stage) {
  switch (stage) {
    case -1: {  // init: derived arrays, then the initial contributions
      if (ctx->pr.layout_gen != ctx->layout_gen) grd_pull_graph_release(ctx);  // the graph holds the old sizes
      TRY(pr_prepare(ctx));
      return enqueue_fwd(ctx);
    }
    case 0: return enqueue_fwd(ctx);  // resends the contributions (the update already sent them)
    case 1: return enqueue_edge_map(ctx);
    case 2:
    case 3: return GRD_OK;  // the edge-map's partial sums are the message; the update merges them
    case 4: {
      TRY(enqueue_update(ctx, 0, 0));
      return read_round(ctx);
    }
    default: return GRD_E_INVALID;
  }
}

int grd_pull_run(grd_ctx* ctx) {
  ctx->stats.converged = 0;
  while (ctx->stats.rounds < ctx->params.max_rounds) {
    grd_prof_mark(ctx, 0);
    grd_prof_mark(ctx, 1);
    const bool timed = ctx->profiling && ctx->pr.T != 0;
    TRY(enqueue_edge_map(ctx, timed));
    grd_prof_mark(ctx, 2);
    grd_prof_mark(ctx, 3);
    TRY(enqueue_update(ctx, 0, 0));
    grd_prof_mark(ctx, 4);
    TRY(read_round(ctx));
    grd_prof_collect(ctx);
    if (timed) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]) == cudaSuccess) {
        ctx->stats.pull_ms += ms;
        ctx->stats.pull_launches += 1;
      }
      (void)cudaGetLastError();
    }
    ctx->stats.rounds++;
    if (ctx->stats.last_residual < ctx->params.tolerance) {
      ctx->stats.converged = 1;
      break;
    }
  }
  return GRD_OK;
}

int grd_pull_graph_run(grd_ctx* ctx, bool* used, bool async) {
  *used = false;
  if (ctx->graph_failed) return GRD_OK;
  if (!ctx->pr_exec) {
    CK(cudaStreamSynchronize(ctx->stream));  // capture starts on an idle stream
    const int rc = build_graph(ctx);
    if (rc != GRD_OK) {
      ctx->graph_failed = true;
      ctx->graph_error = ctx->err;
      ctx->err.clear();
      grd_pull_graph_release(ctx);
      cudaStreamCaptureStatus st;
      if (cudaStreamIsCapturing(ctx->stream, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
      }
      (void)cudaGetLastError();
      return GRD_OK;
    }
  }
  k_pr_seed<<<1, 32, 0, ctx->stream>>>(ctx->st, ctx->stats.rounds, ctx->stats.actives_total);
  CK_LAUNCH();
  CK(cudaGraphLaunch(ctx->pr_exec, ctx->stream));
  *used = true;
  if (async) {
    CK(cudaMemcpyAsync(ctx->h_counters, ctx->st.counters, sizeof(unsigned long long) * NUM_COUNTERS,
                       cudaMemcpyDeviceToHost, ctx->stream));
    ctx->run_pending = true;
    return GRD_OK;
  }
  TRY(grd_read_counters(ctx));
  return grd_pull_run_finish(ctx);
}

int grd_pull_run_finish(grd_ctx* ctx) {
  const unsigned long long* c = ctx->h_counters;
  ctx->stats.rounds = (uint32_t)c[C_ROUNDS];
  ctx->stats.pull_rounds = (uint32_t)c[C_PULL_ROUNDS];
  ctx->stats.actives_total = c[C_ACTIVE_TOTAL];
  ctx->stats.kernel_launches += c[C_LAUNCHES];
  ctx->stats.last_residual = resid_of(ctx);
  ctx->stats.converged = ctx->stats.last_residual < ctx->params.tolerance;
  return GRD_OK;
}
