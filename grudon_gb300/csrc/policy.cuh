// Per-round mode choice on the device: the offload decision (the reference's
// NDPEngine rule, include/offload_engine/NDPEngine.hpp:10-51, which its run()
// leaves disabled at src/GraphAlgorithm.cpp:189), then, for NDP_OFFLOAD
// rounds, the fixed threshold rule or the learned MLP (inference by one
// 64-thread block, fused into the round's policy kernel).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstddef>

#include "../../include/grudon_gpu.h"
#include "kernels.cuh"

namespace grd {

constexpr int P_IN = GRD_POLICY_IN, P_HID = GRD_POLICY_HID, P_OUT = GRD_POLICY_OUT;
static_assert(P_OUT == 4, "one output per round mode");

struct PolicyArgs {
  int direction, format, has_in;
  uint32_t dense_div, pull_div;
  int offload;              // GRD_OFFLOAD_*
  uint32_t launches[7];     // kernels of one round per branch (device loop stats)
  unsigned long long edges; // E
  uint32_t round;           // round index (host loop; the device loop counts)
};

// Offload decision of a round whose entering frontier has f vertices.
// NDPEngine (include/offload_engine/NDPEngine.hpp:17-50) returns NO_OFFLOAD
// when 0 < f <= V/20 (its threshold, src/GraphAlgorithm.cpp:172) and two
// tests pass that always pass with one compute partition: every frontier
// vertex is covered (coverage_vector[v]: all out-neighbours share v's master,
// src/DistributedGraph.cpp:333-343 — every vertex's master is partition 0),
// and the busiest memory partition holds at least the mean number of
// frontier vertices over the partitions it touches (a maximum is never below
// a mean).
__host__ __device__ inline bool policy_no_offload(int offload, unsigned long long f, uint32_t V) {
  if (offload == GRD_OFFLOAD_NONE) return true;
  if (offload != GRD_OFFLOAD_ENGINE) return false;
  return f != 0 && f <= (unsigned long long)(V / 20u);
}

// SWITCH branch of a round in `mode`: modes 0-3 and GRD_ROUND_NO_OFFLOAD are
// their own branch; a frontier small enough for one CTA runs its push + list
// round as branch 4 (k_round_tiny) and its NO_OFFLOAD round as branch 6.
constexpr int P_BRANCH_TINY = 4, P_BRANCH_NOOFF_TINY = 6;
__host__ __device__ inline int policy_branch(int mode, unsigned long long f, unsigned long long fe) {
  const bool small = f <= K_TINY_ACTIVE && fe <= K_TINY_EDGES;
  if (small && mode == GRD_ROUND_PUSH_LIST) return P_BRANCH_TINY;
  if (small && mode == GRD_ROUND_NO_OFFLOAD) return P_BRANCH_NOOFF_TINY;
  return mode;
}

// Raw policy features (grd_policy_features computes the same on the host).
// Sizes enter as log2 fractions of the graph (frontier of V, its edges and
// the unvisited edges of E, its largest degree of V) plus the graph's own
// log2 size and degree, so one model covers graphs of any scale.
__host__ __device__ inline void policy_features(double frontier, double fedges, double unvisited, double maxdeg,
                                                double round, double V, double E, float* f) {
  const double v = V > 1.0 ? V : 1.0;
  const float lv = log2f((float)v), le = log2f((float)(1.0 + E));
  f[0] = log2f((float)(1.0 + frontier)) - lv;
  f[1] = log2f((float)(1.0 + fedges)) - le;
  f[2] = log2f((float)(1.0 + unvisited)) - le;
  f[3] = log2f((float)(1.0 + fedges / (frontier > 1.0 ? frontier : 1.0)));
  f[4] = log2f((float)(1.0 + maxdeg)) - lv;
  f[5] = log2f((float)(1.0 + round));
  f[6] = lv;
  f[7] = log2f((float)(1.0 + E / v));
}

// Modes the round may use: forced direction / format, and pull only with
// the in-edge view.  Bit m = round mode m (0 push+bitvector, 1 push+list,
// 2 pull+bitvector, 3 pull+list).
__host__ __device__ inline uint32_t policy_allowed(int direction, int format, bool has_in) {
  uint32_t dir = 0x3u << 0 | 0x3u << 2;  // both directions
  if (direction == GRD_DIR_PUSH || !has_in) dir &= 0x3u;
  if (direction == GRD_DIR_PULL && has_in) dir &= 0xCu;
  uint32_t fmt = 0xFu;
  if (format == GRD_FMT_BITVEC) fmt = 0x5u;
  if (format == GRD_FMT_LIST) fmt = 0xAu;
  return dir & fmt;
}

__device__ __forceinline__ float h2f(uint16_t b) { return __half2float(__ushort_as_half(b)); }

// Normalised input i of the model from raw feature f (clamped to the
// training range).
__device__ __forceinline__ float policy_input(const grd_policy_model* m, int i, float f) {
  return (fminf(fmaxf(f, m->lo[i]), m->hi[i]) - m->mean[i]) * m->scale[i];
}

// Weights of hidden unit j (thread j) and, for threads below P_OUT, of
// output j, held in registers: every load is issued at once, so one memory
// latency covers the whole model (the struct keeps each row 16-byte aligned).
static_assert(offsetof(grd_policy_model, w1) % 16 == 0 && offsetof(grd_policy_model, w2) % 16 == 0 &&
                  offsetof(grd_policy_model, w3) % 16 == 0,
              "16-byte aligned weight rows");

struct MlpRegs {
  uint4 w1;     // 8 fp16
  uint4 w2[8];  // 64 fp16
  uint4 w3[8];  // 64 fp16 (threads < P_OUT)
  float b1, b2, b3;
};

__device__ __forceinline__ void mlp_load(const grd_policy_model* m, MlpRegs& r) {
  const int j = threadIdx.x;
  r.w1 = __ldg(reinterpret_cast<const uint4*>(m->w1 + j * P_IN));
  const uint4* w2 = reinterpret_cast<const uint4*>(m->w2 + j * P_HID);
#pragma unroll
  for (int q = 0; q < 8; ++q) r.w2[q] = __ldg(w2 + q);
  const uint4* w3 = reinterpret_cast<const uint4*>(m->w3 + (j < P_OUT ? j : 0) * P_HID);
#pragma unroll
  for (int q = 0; q < 8; ++q) r.w3[q] = __ldg(w3 + q);
  r.b1 = m->b1[j];
  r.b2 = m->b2[j];
  r.b3 = m->b3[j < P_OUT ? j : 0];
}

// acc += w[0..7] . x[0..7] as fmaf in index order.
__device__ __forceinline__ float dot8(uint4 w, const float* x, float acc) {
  const uint32_t u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    acc = fmaf(h2f((uint16_t)(u[q] & 0xFFFFu)), x[2 * q], acc);
    acc = fmaf(h2f((uint16_t)(u[q] >> 16)), x[2 * q + 1], acc);
  }
  return acc;
}

// MLP forward for one input by a block of exactly P_HID threads.  xs: the
// normalised input (shared), out: P_OUT predictions (shared).  Fixed
// summation order (fmaf chains in index order).
__device__ __forceinline__ void mlp_eval(const MlpRegs& r, const float* xs, float* h1, float* h2, float* out) {
  const int j = threadIdx.x;
  h1[j] = fmaxf(dot8(r.w1, xs, r.b1), 0.0f);
  __syncthreads();
  float a = r.b2;
#pragma unroll
  for (int q = 0; q < 8; ++q) a = dot8(r.w2[q], h1 + 8 * q, a);
  h2[j] = fmaxf(a, 0.0f);
  __syncthreads();
  if (j < P_OUT) {
    float o = r.b3;
#pragma unroll
    for (int q = 0; q < 8; ++q) o = dot8(r.w3[q], h2 + 8 * q, o);
    out[j] = o;
  }
  __syncthreads();
}

// Fixed rule (grd_choose_round_mode applies the same on the host).
__device__ __forceinline__ int policy_fixed(const DevGraph& g, const PolicyArgs& a, unsigned long long f,
                                            unsigned long long fe) {
  const bool pull =
      a.has_in && (a.direction == GRD_DIR_PULL || (a.direction == GRD_DIR_AUTO && f * a.pull_div >= g.V));
  const bool list = a.format == GRD_FMT_LIST ||
                    (a.format == GRD_FMT_AUTO && f * a.dense_div < g.S && fe * a.dense_div < a.edges);
  return pull ? (list ? GRD_ROUND_PULL_LIST : GRD_ROUND_PULL_BITVEC)
              : (list ? GRD_ROUND_PUSH_LIST : GRD_ROUND_PUSH_BITVEC);
}

// The model overrides the plain method's choice (the fixed rule without the
// in-edge view, i.e. push only, unless pull is forced) only when it predicts
// that round to be faster by more than this margin (log2 units, ~7 %).
constexpr float P_MARGIN = 0.1f;

// A frontier that fits one CTA runs as push + list (one kernel, k_round_tiny)
// whatever the model would say: no other mode comes close for it, and the
// round skips the inference.
__host__ __device__ inline bool policy_tiny(unsigned long long f, unsigned long long fe, uint32_t allowed) {
  return f <= K_TINY_ACTIVE && fe <= K_TINY_EDGES && ((allowed >> GRD_ROUND_PUSH_LIST) & 1u);
}

// Mode of the next round, by a block of P_HID threads (valid in thread 0).
__device__ __forceinline__ int policy_choose(const DevGraph& g, const DevState& st, const PolicyArgs& a,
                                             const grd_policy_model* model, uint32_t round) {
  __shared__ float s_x[P_IN], s_h1[P_HID], s_h2[P_HID], s_out[P_OUT];
  const unsigned long long f = st.counters[C_FRONTIER], fe = st.counters[C_FEDGES];
  if (policy_no_offload(a.offload, f, g.V)) return GRD_ROUND_NO_OFFLOAD;
  if (model == nullptr) return policy_fixed(g, a, f, fe);
  const uint32_t allowed = policy_allowed(a.direction, a.format, a.has_in != 0);
  if (policy_tiny(f, fe, allowed)) return GRD_ROUND_PUSH_LIST;
  MlpRegs r;
  mlp_load(model, r);
  if (threadIdx.x == 0) {
    float raw[P_IN];
    policy_features((double)f, (double)fe, (double)st.counters[C_UNVISITED], (double)st.counters[C_FMAXDEG],
                    (double)round, (double)g.V, (double)a.edges, raw);
    for (int i = 0; i < P_IN; ++i) s_x[i] = policy_input(model, i, raw[i]);
  }
  __syncthreads();
  mlp_eval(r, s_x, s_h1, s_h2, s_out);
  int best = -1;
  for (int m = 0; m < P_OUT; ++m)
    if (((allowed >> m) & 1u) && (best < 0 || s_out[m] < s_out[best])) best = m;
  PolicyArgs plain = a;
  if (a.direction != GRD_DIR_PULL) plain.has_in = 0;
  const int fm = policy_fixed(g, plain, f, fe);
  if (best < 0) return fm;
  return s_out[best] + P_MARGIN < s_out[fm] ? best : fm;
}

// In the device-driven loop, a one-CTA round is followed in the same kernel
// by the next one while the policy would choose one again: after each round
// thread 0 decides as k_policy would (offload rule, then the fixed rule or
// the tiny guard that precedes the model's inference, then the branch) and,
// to go on, records the device-loop statistics of the finished round and of
// the next one as k_round_end and k_policy would.  A high-diameter graph's
// long tail of small rounds then costs one launch instead of three per round.
template <bool kCompute>
__device__ __forceinline__ bool tiny_continue(const DevGraph& g, const DevState& st, const PolicyArgs& a,
                                              const grd_policy_model* model, uint32_t max_rounds) {
  if (st.counters[C_ERR]) return false;
  const unsigned long long f = st.counters[C_FRONTIER], fe = st.counters[C_FEDGES];
  const unsigned long long r = st.counters[C_ROUNDS] + 1;  // rounds finished, this one included
  if (f == 0 || r >= max_rounds) return false;
  int mode;
  if (policy_no_offload(a.offload, f, g.V))
    mode = GRD_ROUND_NO_OFFLOAD;
  else if (model == nullptr)
    mode = policy_fixed(g, a, f, fe);
  else if (policy_tiny(f, fe, policy_allowed(a.direction, a.format, a.has_in != 0)))
    mode = GRD_ROUND_PUSH_LIST;
  else
    return false;  // the model's inference decides: back to the loop graph
  if (policy_branch(mode, f, fe) != (kCompute ? P_BRANCH_NOOFF_TINY : P_BRANCH_TINY)) return false;
  st.counters[C_ROUNDS] = r;  // k_round_end of the finished round
  st.counters[C_ACTIVE_TOTAL] += st.counters[C_ACTIVE];
  st.counters[C_PUSH_ACTIVES] += st.counters[C_ACTIVE];
  st.counters[C_PUSH_ROUNDS] += 1;  // k_policy of the next (no launch)
  if (kCompute) st.counters[C_NOOFF_ROUNDS] += 1;
  st.counters[C_MODE] = (unsigned long long)mode;
  return true;
}

template <int A, bool kCompute>
__global__ void __launch_bounds__(K_TINY_THREADS) k_round_tiny_loop(DevGraph g, DevState st, double tol,
                                                                    double damping, PolicyArgs a,
                                                                    const grd_policy_model* model,
                                                                    uint32_t max_rounds) {
  __shared__ int s_go;
  for (;;) {
    tiny_round<A, kCompute>(g, st, tol, damping);
    __syncthreads();
    if (threadIdx.x == 0) s_go = tiny_continue<kCompute>(g, st, a, model, max_rounds) ? 1 : 0;
    __syncthreads();
    if (!s_go) break;
  }
}

// The round's policy kernel (one block of P_HID threads).  In the device
// loop (kGraph) it also counts the round's statistics and selects the SWITCH
// branch; in the host loop it only leaves the mode in C_MODE.
template <bool kGraph>
static __global__ void __launch_bounds__(P_HID) k_policy(DevGraph g, DevState st, cudaGraphConditionalHandle sw,
                                                         PolicyArgs a, const grd_policy_model* model) {
  const uint32_t round = kGraph ? (uint32_t)st.counters[C_ROUNDS] : a.round;
  const int mode = policy_choose(g, st, a, model, round);
  if (threadIdx.x != 0) return;
  st.counters[C_MODE] = (unsigned long long)mode;
  if (kGraph) {
    if (mode == GRD_ROUND_PULL_BITVEC || mode == GRD_ROUND_PULL_LIST) {
      st.counters[C_PULL_ROUNDS] += 1;
      st.counters[C_EDGES] += a.edges;
    } else {
      st.counters[C_PUSH_ROUNDS] += 1;
      if (mode == GRD_ROUND_NO_OFFLOAD) st.counters[C_NOOFF_ROUNDS] += 1;
    }
    const int branch = policy_branch(mode, st.counters[C_FRONTIER], st.counters[C_FEDGES]);
    st.counters[C_LAUNCHES] += a.launches[branch];
    cudaGraphSetConditional(sw, (unsigned)branch);
  }
}

}  // namespace grd
