// Device primitives of the on-GPU layout build: a three-pass scan over u32
// (add or max) and a stable LSD radix sort of (u32 key, u32 value) pairs.
// Both are deterministic: results never depend on scheduling.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace grd {
namespace prim {

constexpr uint32_t FULLMASK = 0xFFFFFFFFu;

struct OpAdd {
  __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
  static constexpr uint32_t identity = 0u;
};
struct OpMax {
  __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a > b ? a : b; }
  static constexpr uint32_t identity = 0u;
};

// ------------------------------------------------------------------ scan --
// Tiles of SCAN_TILE items: (1) each block reduces its tile, (2) one block
// scans the tile totals exclusively, (3) each block scans its tile from its
// carried prefix.  Items are staged through shared memory so that global
// loads and stores stay coalesced while each thread scans 8 consecutive
// items.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <class Op>
__device__ __forceinline__ uint32_t warp_incl(uint32_t v, Op op) {
  const uint32_t lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t n = __shfl_up_sync(FULLMASK, v, o);
    if (lane >= (uint32_t)o) v = op(v, n);
  }
  return v;
}

// Exclusive block scan of one value per thread (blockDim.x == SCAN_THREADS);
// *total gets the block's reduction.
template <class Op>
__device__ __forceinline__ uint32_t block_excl(uint32_t v, Op op, uint32_t* total) {
  __shared__ uint32_t s_w[32];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t incl = warp_incl(v, op);
  if (lane == 31) s_w[w] = incl;
  __syncthreads();
  if (w == 0) {
    const uint32_t x = s_w[lane];
    const uint32_t xi = warp_incl(x, op);
    s_w[lane] = xi;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t before = w ? s_w[w - 1] : Op::identity;
  const uint32_t ex_in_warp = __shfl_up_sync(FULLMASK, incl, 1);
  const uint32_t ex = op(before, lane ? ex_in_warp : Op::identity);
  *total = s_w[31];
  __syncthreads();
  return ex;
}

template <class Op>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in, uint64_t n,
                                                             uint32_t* tile_sums) {
  const Op op;
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
  uint32_t acc = Op::identity;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const uint64_t i = base + (uint64_t)k * SCAN_THREADS + threadIdx.x;
    if (i < n) acc = op(acc, in[i]);
  }
  uint32_t total;
  (void)block_excl(acc, op, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block: exclusive scan of the tile totals in place.
template <class Op>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(uint32_t* sums, uint64_t ntiles) {
  const Op op;
  __shared__ uint32_t s_carry;
  if (threadIdx.x == 0) s_carry = Op::identity;
  __syncthreads();
  for (uint64_t c0 = 0; c0 < ntiles; c0 += SCAN_THREADS) {
    const uint64_t i = c0 + threadIdx.x;
    const uint32_t v = i < ntiles ? sums[i] : Op::identity;
    uint32_t total;
    const uint32_t ex = block_excl(v, op, &total);
    const uint32_t carry = s_carry;
    if (i < ntiles) sums[i] = op(carry, ex);
    __syncthreads();
    if (threadIdx.x == 0) s_carry = op(carry, total);
    __syncthreads();
  }
}

// out may alias in.  inclusive = false: out[i] = op(in[0..i-1]); with
// total_at_n, out[n] also receives the reduction of all n items.
template <class Op>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const uint32_t* in, uint32_t* out, uint64_t n,
                                                           const uint32_t* __restrict__ tile_prefix, int inclusive,
                                                           int total_at_n) {
  const Op op;
  __shared__ uint32_t s_items[SCAN_TILE];
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const uint32_t j = k * SCAN_THREADS + threadIdx.x;
    const uint64_t i = base + j;
    s_items[j] = i < n ? in[i] : Op::identity;
  }
  __syncthreads();
  uint32_t loc[SCAN_ITEMS], acc = Op::identity;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    loc[k] = s_items[threadIdx.x * SCAN_ITEMS + k];
    acc = op(acc, loc[k]);
  }
  uint32_t total;
  uint32_t run = op(tile_prefix[blockIdx.x], block_excl(acc, op, &total));
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const uint32_t x = loc[k];
    if (inclusive) run = op(run, x);
    s_items[threadIdx.x * SCAN_ITEMS + k] = run;
    if (!inclusive) run = op(run, x);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const uint32_t j = k * SCAN_THREADS + threadIdx.x;
    const uint64_t i = base + j;
    if (i < n) out[i] = s_items[j];
  }
  if (total_at_n && base + SCAN_TILE >= n && threadIdx.x == SCAN_THREADS - 1)
    out[n] = op(tile_prefix[blockIdx.x], total);  // the last tile holds the end
}

// ------------------------------------------------------------ radix sort --
// One pass over 8 key bits, tiles of RS_TILE items: (1) per-tile digit
// histograms, stored digit-major, (2) their exclusive scan (digit, tile
// order), (3) a stable scatter.  In (3) warp w of a tile owns items
// [w*512, w*512+512) and walks them 32 at a time; lanes with the same digit
// rank themselves with __match_any_sync, so the rank of an item counts
// exactly the same-digit items before it in input order.
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr uint32_t RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_BINS = 256;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t* __restrict__ keys, uint64_t n, int shift,
                                                       uint32_t* hist, uint32_t ntiles) {
  __shared__ uint32_t s_cnt[RS_BINS];
  s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const uint64_t i = base + (uint64_t)r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&s_cnt[(keys[i] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = s_cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in, uint64_t n, int shift,
                                                          const uint32_t* __restrict__ offsets, uint32_t ntiles,
                                                          uint32_t* __restrict__ keys_out,
                                                          uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t s_wc[RS_THREADS / 32][RS_BINS];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = lane; d < RS_BINS; d += 32) s_wc[w][d] = 0;
  __syncwarp();
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE + (uint64_t)w * (32 * RS_ROUNDS);
  uint32_t k[RS_ROUNDS], v[RS_ROUNDS], rk[RS_ROUNDS];
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const uint64_t i = base + (uint64_t)r * 32 + lane;
    const bool valid = i < n;
    k[r] = valid ? keys_in[i] : 0u;
    v[r] = valid ? vals_in[i] : 0u;
    const uint32_t d = valid ? ((k[r] >> shift) & 0xFFu) : 0x100u;
    const uint32_t peers = __match_any_sync(FULLMASK, d);
    const uint32_t before = valid ? s_wc[w][d] : 0u;
    rk[r] = before + __popc(peers & lt);
    __syncwarp();
    if (valid && lane == 31u - __clz(peers)) s_wc[w][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {  // per digit: exclusive prefix over the warps of the tile, plus the tile's global offset
    const uint32_t d = threadIdx.x;
    uint32_t run = offsets[(uint64_t)d * ntiles + blockIdx.x];
#pragma unroll
    for (int ww = 0; ww < RS_THREADS / 32; ++ww) {
      const uint32_t c = s_wc[ww][d];
      s_wc[ww][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const uint64_t i = base + (uint64_t)r * 32 + lane;
    if (i < n) {
      const uint32_t d = (k[r] >> shift) & 0xFFu;
      const uint32_t pos = s_wc[w][d] + rk[r];
      keys_out[pos] = k[r];
      vals_out[pos] = v[r];
    }
  }
}

}  // namespace prim
}  // namespace grd
