// ORACLE — test infrastructure only.  CPU restatement of the Jacobi
// PageRank of the benchmark's PageRank workload, in the arithmetic that
// workload prescribes: FP32 ranks and contributions, a Kahan-compensated FP32
// sum per vertex over its in-edges in ascending source order, and the L1
// residual reduced in FP64.  Fixed point (the one the reference's delta-push
// PageRank converges to, src/graph_algorithms/pr.cpp:20-88 of the Grudon
// project):
//   pr[v] = (1-d)*[outdeg(v) > 0] + sum_{u->v} d * pr[u] / outdeg(u)
// from pr = (1-d) on non-dangling vertices (pr.cpp:30-49).
//
// A stateful object, so that the CPU baseline can transpose the graph once
// and then time bounded samples of iterations on all host threads.  Results
// do not depend on the thread count (each vertex's sum has a fixed order and
// the residual is reduced over fixed vertex blocks in block order).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

template <class F>
void run_threads(int n, F&& f) {
  std::vector<std::thread> ts;
  for (int t = 1; t < n; ++t) ts.emplace_back([&f, t] { f(t); });
  f(0);
  for (auto& th : ts) th.join();
}

struct PrJacobi {
  uint32_t V = 0;
  int nt = 1;
  double d = 0.85;
  std::vector<uint64_t> in_off;
  std::vector<uint32_t> in_src, outdeg;
  std::vector<float> ranks, contrib;
};

constexpr uint32_t BLOCK = 65536;  // vertices per residual block

inline void kahan(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

}  // namespace

extern "C" {

void* orc_prj_create(uint32_t V, const uint64_t* ro, const uint32_t* col, double damping, int threads) {
  PrJacobi* p = new PrJacobi;
  p->V = V;
  p->d = damping;
  p->nt = threads > 0 ? threads : std::max(1u, std::thread::hardware_concurrency());
  const int nt = p->nt;
  const uint64_t E = ro[V];
  p->outdeg.resize(V);
  for (uint32_t v = 0; v < V; ++v) p->outdeg[v] = (uint32_t)(ro[v + 1] - ro[v]);
  // in-lists in ascending source order: thread t owns the destinations of
  // [V*t/nt, V*(t+1)/nt) and scans every row in source order
  std::vector<uint64_t> cnt((size_t)V + 1, 0);
  run_threads(nt, [&](int t) {
    const uint32_t lo = (uint32_t)((uint64_t)V * t / nt), hi = (uint32_t)((uint64_t)V * (t + 1) / nt);
    for (uint64_t i = 0; i < E; ++i)
      if (col[i] >= lo && col[i] < hi) ++cnt[col[i] + 1];
  });
  p->in_off.resize((size_t)V + 1);
  p->in_off[0] = 0;
  for (uint32_t v = 0; v < V; ++v) p->in_off[v + 1] = p->in_off[v] + cnt[v + 1];
  p->in_src.resize(E ? E : 1);
  run_threads(nt, [&](int t) {
    const uint32_t lo = (uint32_t)((uint64_t)V * t / nt), hi = (uint32_t)((uint64_t)V * (t + 1) / nt);
    std::vector<uint64_t> cur(p->in_off.begin() + lo, p->in_off.begin() + hi);
    for (uint32_t u = 0; u < V; ++u)
      for (uint64_t i = ro[u]; i < ro[u + 1]; ++i) {
        const uint32_t v = col[i];
        if (v >= lo && v < hi) p->in_src[cur[v - lo]++] = u;
      }
  });
  p->ranks.assign(V, 0.0f);
  p->contrib.assign(V, 0.0f);
  return p;
}

// init(): ranks (1-d) on non-dangling vertices, their contributions.
void orc_prj_init(void* h) {
  PrJacobi* p = static_cast<PrJacobi*>(h);
  for (uint32_t v = 0; v < p->V; ++v) {
    const uint32_t deg = p->outdeg[v];
    p->ranks[v] = deg ? (float)(1.0 - p->d) : 0.0f;
    p->contrib[v] = deg ? (float)(p->d * (1.0 - p->d) / (double)deg) : 0.0f;
  }
}

// Runs up to `iters` iterations, stopping early once the L1 residual / V
// falls below tol (tol > 0).  Returns the iterations run; *residual gets the
// last residual / V.
uint32_t orc_prj_iterate(void* h, uint32_t iters, double tol, double* residual) {
  PrJacobi* p = static_cast<PrJacobi*>(h);
  const uint32_t V = p->V;
  const uint32_t nb = (V + BLOCK - 1) / BLOCK;
  const float df = (float)p->d, base = (float)(1.0 - p->d);
  std::vector<float> next(V);
  std::vector<double> part(nb ? nb : 1);
  uint32_t it = 0;
  double res = 0.0;
  while (it < iters) {
    run_threads(p->nt, [&](int t) {
      for (uint32_t b = (uint32_t)t; b < nb; b += (uint32_t)p->nt) {
        const uint32_t v0 = b * BLOCK, v1 = std::min(V, v0 + BLOCK);
        double r = 0.0;
        for (uint32_t v = v0; v < v1; ++v) {
          float s = 0.0f, c = 0.0f;
          for (uint64_t i = p->in_off[v]; i < p->in_off[v + 1]; ++i) kahan(s, c, p->contrib[p->in_src[i]]);
          const float nv = (p->outdeg[v] ? base : 0.0f) + (s - c);
          r += std::fabs((double)nv - (double)p->ranks[v]);
          next[v] = nv;
        }
        part[b] = r;
      }
    });
    res = 0.0;
    for (uint32_t b = 0; b < nb; ++b) res += part[b];
    res /= (double)(V ? V : 1);
    p->ranks.swap(next);
    run_threads(p->nt, [&](int t) {
      const uint32_t lo = (uint32_t)((uint64_t)V * t / p->nt), hi = (uint32_t)((uint64_t)V * (t + 1) / p->nt);
      for (uint32_t v = lo; v < hi; ++v) {
        const uint32_t deg = p->outdeg[v];
        p->contrib[v] = deg ? (df * p->ranks[v]) / (float)deg : 0.0f;
      }
    });
    ++it;
    if (tol > 0 && res < tol) break;
  }
  if (residual) *residual = res;
  return it;
}

void orc_prj_ranks(const void* h, float* out) {
  const PrJacobi* p = static_cast<const PrJacobi*>(h);
  std::memcpy(out, p->ranks.data(), sizeof(float) * p->V);
}

void orc_prj_free(void* h) { delete static_cast<PrJacobi*>(h); }

}  // extern "C"
