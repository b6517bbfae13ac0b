// ORACLE — test infrastructure only.  CPU restatement of Grudon's per-round
// graph operator (1 compute + M memory partitions, MPI replaced by memcpy
// between in-process partition objects) plus independent textbook oracles.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load this library; the product path never does.
//
// Parity status: UNPINNED against the reference's own outputs.  The
// reference (Kadle11/Grudon) has no tests, fixtures or golden vectors, and
// it cannot be compiled here (its Galois, cxxopts and spdlog submodules are
// empty; MPI, Boost and libnuma are absent).  This restatement is instead
// cross-checked against independent oracles (BFS, Dijkstra, union-find,
// FP64 power iteration), hand-computed tiny graphs and the reference's own
// verify() invariants.
//
// Third-party semantics restated (Galois, fork Kadle11/Galois branch
// "Grudon", commit not pinned in the reference): atomicMin/atomicAdd are CAS
// loops returning the previous value; DynamicBitSet is a u64-word bitset whose
// getOffsets() lists set bits in ascending order; LC_CSR_Graph keeps edges of
// a row in insertion order.
//
// Files followed (paths within the Grudon project):
//   src/GraphAlgorithm.cpp:145-701       round loop C1-C9
//   src/graph_algorithms/pr.cpp:20-160   PageRank (delta push, float)
//   src/graph_algorithms/cc.cpp:18-120   CC (min label)
//   src/graph_algorithms/sssp.cpp:18-126 SSSP (unit weight; weighted variant
//                                        substitutes prop+w at sssp.cpp:69)
//   include/DistributedGraph.hpp:91-214  PropertyList semantics
//   src/DistributedGraph.cpp:285-775     proxies, translation tables
//   include/partitioning_engine/Partitioner.hpp:11-205 master = gid % C
//   include/offload_engine/NDPEngine.hpp:10-51 offload decision, and the
//   NO_OFFLOAD round of src/GraphAlgorithm.cpp:426-474, 582-637
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <queue>
#include <thread>
#include <vector>

namespace {

enum { ORC_PR_DELTA = 0, ORC_PR_PULL = 1, ORC_CC = 2, ORC_SSSP_HOP = 3, ORC_SSSP_W = 4 };

// ------------------------------------------------------------ thread pool --
// Persistent pool standing in for the Galois do_all runtime (threads > 1 is
// the timed CPU baseline; threads == 1 is the deterministic checker).
class Pool {
 public:
  explicit Pool(int n) : n_(std::max(1, n)) {
    for (int i = 1; i < n_; ++i) ts_.emplace_back([this, i] { loop(i); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : ts_) t.join();
  }
  int size() const { return n_; }
  // fn(begin, end) over [0,n) in dynamic chunks.
  void run(uint64_t n, uint64_t grain, const std::function<void(uint64_t, uint64_t)>& fn) {
    if (n_ == 1 || n <= grain) {
      if (n) fn(0, n);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m_);
      fn_ = &fn;
      n_items_ = n;
      grain_ = grain;
      next_.store(0);
      pending_ = n_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(m_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  void work() {
    for (;;) {
      uint64_t b = next_.fetch_add(grain_);
      if (b >= n_items_) break;
      (*fn_)(b, std::min(n_items_, b + grain_));
    }
  }
  void loop(int) {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
      }
      work();
      {
        std::lock_guard<std::mutex> g(m_);
        if (--pending_ == 0) done_cv_.notify_all();
      }
    }
  }
  int n_;
  std::vector<std::thread> ts_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  uint64_t gen_ = 0;
  bool stop_ = false;
  const std::function<void(uint64_t, uint64_t)>* fn_ = nullptr;
  uint64_t n_items_ = 0, grain_ = 1;
  std::atomic<uint64_t> next_{0};
  int pending_ = 0;
};

// --------------------------------------------------- Galois-like helpers --
struct Bitset {  // DynamicBitSet
  std::vector<uint64_t> w;
  uint64_t n = 0;
  void resize(uint64_t bits) {
    n = bits;
    w.assign((bits + 63) / 64, 0);
  }
  void set(uint64_t i) {
    const uint64_t b = 1ull << (i & 63);
    if (!(__atomic_load_n(&w[i >> 6], __ATOMIC_RELAXED) & b)) __atomic_fetch_or(&w[i >> 6], b, __ATOMIC_RELAXED);
  }
  bool test(uint64_t i) const { return (w[i >> 6] >> (i & 63)) & 1; }
  void reset() { std::fill(w.begin(), w.end(), 0); }
  uint64_t count() const {
    uint64_t c = 0;
    for (uint64_t x : w) c += __builtin_popcountll(x);
    return c;
  }
  std::vector<uint32_t> offsets() const {  // getOffsets(): ascending
    std::vector<uint32_t> o;
    for (uint64_t k = 0; k < w.size(); ++k) {
      uint64_t x = w[k];
      while (x) {
        o.push_back((uint32_t)(k * 64 + __builtin_ctzll(x)));
        x &= x - 1;
      }
    }
    return o;
  }
  uint64_t size_bytes() const { return w.size() * sizeof(uint64_t); }
};

template <class T>
struct Bits;
template <>
struct Bits<uint32_t> {
  static uint32_t to(uint32_t v) { return v; }
  static uint32_t from(uint32_t b) { return b; }
};
template <>
struct Bits<float> {
  static uint32_t to(float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    return b;
  }
  static float from(uint32_t b) {
    float v;
    std::memcpy(&v, &b, 4);
    return v;
  }
};

// PropertyList<T> (include/DistributedGraph.hpp:91-214) over 32-bit values.
template <class T>
struct PropertyList {
  std::vector<uint32_t> v;  // value bits (atomically updated)
  Bitset dirty;
  void allocate(uint64_t n) {
    v.assign(n, 0);
    dirty.resize(n);
  }
  T get(uint64_t i) const { return Bits<T>::from(__atomic_load_n(&v[i], __ATOMIC_RELAXED)); }
  void put(uint64_t i, T x) { __atomic_store_n(&v[i], Bits<T>::to(x), __ATOMIC_RELAXED); }
  // galois::atomicMin: CAS loop, returns the previous value; dirty iff lowered.
  void minUpdate(uint64_t i, T val) {
    uint32_t old = __atomic_load_n(&v[i], __ATOMIC_RELAXED);
    while (Bits<T>::from(old) > val &&
           !__atomic_compare_exchange_n(&v[i], &old, Bits<T>::to(val), true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
    if (val < Bits<T>::from(old)) dirty.set(i);
  }
  // galois::atomicAdd: CAS loop; always dirty.
  void addUpdate(uint64_t i, T val) {
    dirty.set(i);
    uint32_t old = __atomic_load_n(&v[i], __ATOMIC_RELAXED);
    for (;;) {
      T nv = Bits<T>::from(old) + val;
      if (__atomic_compare_exchange_n(&v[i], &old, Bits<T>::to(nv), true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) break;
    }
  }
  void set(uint64_t i, T x) {
    dirty.set(i);
    put(i, x);
  }
  void clear() {  // zero dirty entries, reset bits
    for (uint32_t i : dirty.offsets()) v[i] = 0;
    dirty.reset();
  }
  void clear_uv() { dirty.reset(); }
};

// Memory partition p (a TraverseWorker rank) with C = 1.
struct MemPart {
  uint32_t n_owned = 0, n_proxy = 0;
  std::vector<uint32_t> lid_gid;   // lid -> gid (owned then proxies)
  std::vector<uint64_t> row_end;   // lgraph row ends over owned lids
  std::vector<uint32_t> dst;       // local lids
  std::vector<uint32_t> w;         // weights (weighted SSSP only)
  uint32_t T() const { return n_owned + n_proxy; }
};

// In-edge lists of one memory partition: for each destination lid its
// sources (owned lids) in ascending order.
struct InEdges {
  std::vector<uint64_t> off;
  std::vector<uint32_t> src;
};

InEdges build_in_edges(const MemPart& P) {
  InEdges IE;
  IE.off.assign((size_t)P.T() + 1, 0);
  const uint64_t E = P.dst.size();
  for (uint64_t i = 0; i < E; ++i) IE.off[P.dst[i] + 1]++;
  for (uint32_t d = 0; d < P.T(); ++d) IE.off[d + 1] += IE.off[d];
  IE.src.resize(E);
  std::vector<uint64_t> cur(IE.off.begin(), IE.off.end() - 1);
  for (uint32_t u = 0; u < P.n_owned; ++u) {
    const uint64_t r0 = u ? P.row_end[u - 1] : 0, r1 = P.row_end[u];
    for (uint64_t i = r0; i < r1; ++i) IE.src[cur[P.dst[i]]++] = u;
  }
  return IE;
}

struct Layout {
  uint32_t V = 0, M = 0;
  std::vector<uint32_t> mirror;       // compute-side mirror_partition (lid = gid)
  std::vector<uint64_t> outdeg;       // compute-side out_degrees
  std::vector<MemPart> parts;
  // compute-side translation: sTrans[p][gid] (owned slot of gid in its mirror
  // partition) and rTrans[p][slot] = gid.
  std::vector<std::vector<uint32_t>> rTrans;
  std::vector<uint32_t> sOwned;  // slot of gid in mirror[gid]
  std::vector<uint8_t> coverage;  // compute-side coverage_vector
};

// DistributedGraph ctor restated for C = 1 (src/DistributedGraph.cpp:13-785).
void build(Layout& L, uint32_t V, const uint64_t* ro, const uint32_t* col, const uint32_t* w,
           const uint32_t* mirror, uint32_t M) {
  L.V = V;
  L.M = M;
  L.mirror.resize(V);
  L.outdeg.resize(V);
  for (uint32_t g = 0; g < V; ++g) {
    // NaivePartitioner is gid % M (Partitioner.hpp:32-33, used when M == 1).
    // For M > 1 without a file the reference leaves every vertex in partition
    // 0 (zero-filled vector, Partitioner.hpp:87); callers pass an explicit
    // assignment in that case.
    L.mirror[g] = mirror ? mirror[g] : g % M;
    L.outdeg[g] = ro[g + 1] - ro[g];
  }
  // cross_node_mirrors[p]: dst of an edge from a p-owned vertex, mirrored
  // elsewhere (:345-349).
  std::vector<Bitset> cross(M);
  for (auto& b : cross) b.resize(V);
  for (uint32_t u = 0; u < V; ++u)
    for (uint64_t i = ro[u]; i < ro[u + 1]; ++i)
      if (L.mirror[col[i]] != L.mirror[u]) cross[L.mirror[u]].set(col[i]);
  // coverage_vector (:296-343): a vertex stays covered unless an out-edge
  // leads to a vertex with another master.  The master partition is
  // gid % C (Partitioner.hpp:11-205), i.e. 0 for every vertex with C = 1.
  auto master = [](uint32_t) { return 0u; };
  L.coverage.assign(V, 1);
  for (uint32_t u = 0; u < V; ++u)
    for (uint64_t i = ro[u]; i < ro[u + 1]; ++i)
      if (master(col[i]) != master(u)) L.coverage[u] = 0;
  L.parts.assign(M, MemPart());
  L.rTrans.assign(M, {});
  L.sOwned.assign(V, 0);
  // Compute side (:688-758): owned slots in ascending lid, then cross mirrors.
  for (uint32_t g = 0; g < V; ++g) {
    uint32_t p = L.mirror[g];
    L.sOwned[g] = (uint32_t)L.rTrans[p].size();
    L.rTrans[p].push_back(g);
  }
  for (uint32_t g = 0; g < V; ++g)
    for (uint32_t p = 0; p < M; ++p)
      if (p != L.mirror[g] && cross[p].test(g)) L.rTrans[p].push_back(g);
  // Memory side (:506-616): owned lids in gid order, then proxies in gid order.
  std::vector<uint32_t> g2l(V);
  for (uint32_t p = 0; p < M; ++p) {
    MemPart& P = L.parts[p];
    for (uint32_t g = 0; g < V; ++g)
      if (L.mirror[g] == p) P.lid_gid.push_back(g);
    P.n_owned = (uint32_t)P.lid_gid.size();
    for (uint32_t g = 0; g < V; ++g)
      if (cross[p].test(g)) P.lid_gid.push_back(g);
    P.n_proxy = (uint32_t)P.lid_gid.size() - P.n_owned;
    for (uint32_t l = 0; l < P.lid_gid.size(); ++l) g2l[P.lid_gid[l]] = l;
    P.row_end.resize(P.n_owned);
    uint64_t ec = 0;
    for (uint32_t l = 0; l < P.n_owned; ++l) {
      uint32_t g = P.lid_gid[l];
      for (uint64_t i = ro[g]; i < ro[g + 1]; ++i) {
        P.dst.push_back(g2l[col[i]]);
        if (w) P.w.push_back(w[i]);
      }
      ec += ro[g + 1] - ro[g];
      P.row_end[l] = ec;
    }
    // The memory-side slot of lid l towards compute 0 is l itself (:644-660).
  }
}

struct Stats {
  uint32_t rounds;
  uint32_t converged;
  uint64_t edges_scanned;
  uint64_t bytes_synced;
  uint64_t reference_bytes_moved;
  uint32_t no_offload_rounds;
};

enum Offload { OFF_NDP = 0, OFF_ENGINE = 1, OFF_NONE = 2 };

// NDPEngine (include/offload_engine/NDPEngine.hpp:10-51) on the compute
// rank, with its threshold total_vertices / 20 (src/GraphAlgorithm.cpp:172).
// True = NO_OFFLOAD.  The reference's call site (commented out at :189-190)
// sizes mirrorCoverage by num_compute while indexing it by memory partition;
// it is sized by M here.
bool ndp_engine_no_offload(const Layout& L, const std::vector<uint32_t>& fr) {
  const uint64_t threshold = L.V / 20;
  if (fr.empty() || fr.size() > threshold) return false;
  for (uint32_t v : fr)
    if (!L.coverage[v]) return false;
  std::vector<uint64_t> mc(L.M, 0);
  for (uint32_t lid : fr) mc[L.mirror[lid]]++;  // lid = gid on the compute rank (C = 1)
  uint64_t mx = 0, total = 0, touched = 0;
  for (uint64_t c : mc) {
    mx = std::max(mx, c);
    total += c;
    touched += c > 0;
  }
  if (touched == 0 || mx < total / touched) return false;
  return true;
}

template <class T, int A>
void run_protocol(const Layout& L, uint32_t source, uint32_t max_rounds, double damping, double tol, Pool& pool,
                  int offload, T* props_out, float* ranks_out, T* updates_out, Stats& st) {
  const uint32_t V = L.V, M = L.M;
  const T MAXV = std::numeric_limits<T>::max();
  // Compute rank state.
  PropertyList<T> cprop, cupd;
  PropertyList<float> pr_vals, prev_updates;
  cprop.allocate(V);
  cupd.allocate(V);
  Bitset frontier;
  frontier.resize(V);
  // Memory rank state.
  std::vector<PropertyList<T>> mprop(M), mupd(M);
  for (uint32_t p = 0; p < M; ++p) {
    mprop[p].allocate(L.parts[p].T());
    mupd[p].allocate(L.parts[p].T());
  }
  // init()
  if (A == ORC_PR_DELTA) {
    pr_vals.allocate(V);
    prev_updates.allocate(V);
    for (uint32_t n = 0; n < V; ++n) {
      if (L.outdeg[n] != 0) {
        cprop.put(n, (T)(damping * (1.0 - damping) / (double)L.outdeg[n]));
        pr_vals.put(n, (float)(1.0 - damping));
        frontier.set(n);
      } else {
        cprop.put(n, (T)0);
        pr_vals.put(n, 0.0f);
      }
      cupd.put(n, (T)0);
      prev_updates.put(n, 0.0f);
    }
    for (uint32_t p = 0; p < M; ++p)
      for (uint32_t l = 0; l < L.parts[p].T(); ++l) {
        mprop[p].put(l, (T)0);
        mupd[p].put(l, (T)0);
      }
  } else if (A == ORC_CC) {
    for (uint32_t n = 0; n < V; ++n) {
      cprop.put(n, (T)n);
      cupd.put(n, MAXV);
      frontier.set(n);
    }
    for (uint32_t p = 0; p < M; ++p)
      for (uint32_t l = 0; l < L.parts[p].T(); ++l) {
        mprop[p].put(l, MAXV);
        mupd[p].put(l, MAXV);
      }
  } else {
    for (uint32_t n = 0; n < V; ++n) {
      cprop.put(n, MAXV);
      cupd.put(n, MAXV);
    }
    for (uint32_t p = 0; p < M; ++p)
      for (uint32_t l = 0; l < L.parts[p].T(); ++l) {
        mprop[p].put(l, MAXV);
        mupd[p].put(l, MAXV);
      }
    cprop.put(source, (T)0);
    cupd.put(source, (T)0);
    frontier.set(source);
  }
  const bool clear_updates = (A == ORC_PR_DELTA);

  std::vector<InEdges> in_edges(A == ORC_PR_DELTA ? M : 0);
  for (uint32_t p = 0; p < in_edges.size(); ++p) in_edges[p] = build_in_edges(L.parts[p]);
  std::vector<Bitset> fwd_bv(M), bwd_bv(M);
  std::vector<std::vector<T>> fwd_buf(M), bwd_buf(M);
  for (uint32_t p = 0; p < M; ++p) {
    fwd_bv[p].resize(L.parts[p].T());
    bwd_bv[p].resize(L.parts[p].T());
  }
  uint64_t edges = 0, bytes = 0, refbytes = 0;
  uint32_t iteration = 0, no_offload_rounds = 0;
  bool done = false;
  const uint64_t msg_words_per_edge = (A == ORC_SSSP_W) ? 2 : 1;  // dst gid (+ weight)
  while (!done && iteration < max_rounds) {
    const std::vector<uint32_t> frontier_iter = frontier.offsets();
    // C1: offload decision (the reference's run() fixes NDP_OFFLOAD, :189).
    const bool no_off =
        offload == OFF_NONE || (offload == OFF_ENGINE && ndp_engine_no_offload(L, frontier_iter));
    no_offload_rounds += no_off;
    // C2: compute packs the frontier per mirror partition (ascending lid).
    for (uint32_t p = 0; p < M; ++p) fwd_buf[p].clear();
    for (uint32_t lid : frontier_iter) {
      uint32_t p = L.mirror[lid];
      fwd_bv[p].set(L.sOwned[lid]);
      fwd_buf[p].push_back(cprop.get(lid));
    }
    for (uint32_t p = 0; p < M; ++p) {
      bytes += fwd_bv[p].size_bytes() + fwd_buf[p].size() * sizeof(T);
      refbytes += fwd_bv[p].size_bytes() * 8 + fwd_buf[p].size() * sizeof(T);
    }
    // C3-C5 per memory partition.
    for (uint32_t p = 0; p < M; ++p) {
      const MemPart& P = L.parts[p];
      // C3 unpack: the j-th set bit's slot is the lid (C = 1).
      std::vector<uint32_t> bits = fwd_bv[p].offsets();
      for (size_t j = 0; j < bits.size(); ++j) mprop[p].set(bits[j], fwd_buf[p][j]);
      fwd_bv[p].reset();
      if (no_off) {
        // NO_OFFLOAD, memory side (:426-474): per updated vertex_properties
        // entry one message [gid, destination gids...] (weighted SSSP: and
        // the weights) to its compute rank; net.send counts it.
        for (uint32_t lid : mprop[p].dirty.offsets()) {
          const uint64_t r0 = lid ? P.row_end[lid - 1] : 0, r1 = P.row_end[lid];
          const uint64_t words = 1 + (r1 - r0) * msg_words_per_edge;
          bytes += words * 4;
          refbytes += words * 4;
        }
        mprop[p].clear_uv();
        continue;
      }
      // C4 gen_updates over dirty vertex_properties, ascending lid.
      std::vector<uint32_t> act = mprop[p].dirty.offsets();
      if (A == ORC_PR_DELTA) {
        // addUpdate's atomic adds leave each destination's sum in whatever
        // order the threads ran; this restatement fixes one order (the one
        // the GPU computes in every round mode): the destination's in-list
        // (ascending source lid) in 32-edge chunks from its start, each chunk
        // added by a halving tree (x[i] += x[i + o], o = 16 .. 1) over the
        // frontier sources' values (0 elsewhere), the chunk sums in order.
        // The destinations it touches, and so the dirty set, are unchanged.
        const InEdges& IE = in_edges[p];
        std::vector<uint8_t> active(P.T(), 0);
        uint64_t sc = 0;
        for (uint32_t lid : act) {
          active[lid] = 1;
          sc += (lid ? P.row_end[lid] - P.row_end[lid - 1] : P.row_end[lid]);
        }
        edges += sc;
        pool.run(P.T(), 4096, [&](uint64_t b, uint64_t e) {
          for (uint64_t d = b; d < e; ++d) {
            bool touched = false;
            float acc = 0.0f;
            for (uint64_t c = IE.off[d]; c < IE.off[d + 1]; c += 32) {
              float x[32];
              for (int i = 0; i < 32; ++i) {
                const uint64_t k = c + (uint64_t)i;
                x[i] = 0.0f;
                if (k < IE.off[d + 1] && active[IE.src[k]]) {
                  x[i] = Bits<float>::from(Bits<T>::to(mprop[p].get(IE.src[k])));
                  touched = true;
                }
              }
              for (int o = 16; o; o >>= 1)
                for (int i = 0; i < o; ++i) x[i] = x[i] + x[i + o];
              acc = acc + x[0];
            }
            if (touched) mupd[p].set(d, Bits<T>::from(Bits<float>::to(acc)));
          }
        });
      } else {
      std::atomic<uint64_t> scanned{0};
      pool.run(act.size(), 64, [&](uint64_t b, uint64_t e) {
        uint64_t sc = 0;
        for (uint64_t k = b; k < e; ++k) {
          const uint32_t lid = act[k];
          const uint64_t r0 = lid ? P.row_end[lid - 1] : 0, r1 = P.row_end[lid];
          sc += r1 - r0;
          const T pv = mprop[p].get(lid);
          for (uint64_t i = r0; i < r1; ++i) {
            const uint32_t d = P.dst[i];
            if (A == ORC_PR_DELTA) {
              mupd[p].addUpdate(d, pv);
            } else if (A == ORC_CC) {
              mupd[p].minUpdate(d, pv);
            } else if (A == ORC_SSSP_HOP) {
              mupd[p].minUpdate(d, (T)(pv + 1));
            } else {
              uint64_t c = (uint64_t)pv + P.w[i];
              mupd[p].minUpdate(d, (T)std::min<uint64_t>(c, 0xFFFFFFFFull));
            }
          }
        }
        scanned.fetch_add(sc);
      });
      edges += scanned.load();
      }
      // C5 pack dirty vertex_updates (master = compute 0 for every lid).
      bwd_buf[p].clear();
      for (uint32_t lid : mupd[p].dirty.offsets()) {
        bwd_bv[p].set(lid);
        bwd_buf[p].push_back(mupd[p].get(lid));
      }
      bytes += bwd_bv[p].size_bytes() + bwd_buf[p].size() * sizeof(T);
      refbytes += bwd_bv[p].size_bytes() * 8 + bwd_buf[p].size() * sizeof(T);
      // C8 (memory side end of round)
      if (clear_updates)
        mupd[p].clear();
      else
        mupd[p].clear_uv();
      mprop[p].clear_uv();
    }
    if (no_off) {
      // NO_OFFLOAD, compute side (:582-637): one message per frontier vertex
      // from its mirror partition (net.recv counts it again), then the
      // algorithm's update per shipped edge straight into vertex_updates.
      // The reference hard-codes addUpdate(l_dst, vertex_properties[src])
      // there (PageRank's gen_updates; :626 leaves "abstract this to the
      // graph algorithm" as a TODO with minUpdate commented out beside it);
      // each algorithm's own gen_updates relaxation is applied here.
      std::atomic<uint64_t> scanned{0}, words{0};
      pool.run(frontier_iter.size(), 64, [&](uint64_t b, uint64_t e) {
        uint64_t sc = 0, wd = 0;
        for (uint64_t k = b; k < e; ++k) {
          const uint32_t src = frontier_iter[k];
          const MemPart& P = L.parts[L.mirror[src]];
          const uint32_t lid = L.sOwned[src];
          const uint64_t r0 = lid ? P.row_end[lid - 1] : 0, r1 = P.row_end[lid];
          sc += r1 - r0;
          wd += 1 + (r1 - r0) * msg_words_per_edge;
          const T pv = cprop.get(src);
          for (uint64_t i = r0; i < r1; ++i) {
            const uint32_t d = P.lid_gid[P.dst[i]];
            if (A == ORC_PR_DELTA) {
              cupd.addUpdate(d, pv);
            } else if (A == ORC_CC) {
              cupd.minUpdate(d, pv);
            } else if (A == ORC_SSSP_HOP) {
              cupd.minUpdate(d, (T)(pv + 1));
            } else {
              uint64_t c = (uint64_t)pv + P.w[i];
              cupd.minUpdate(d, (T)std::min<uint64_t>(c, 0xFFFFFFFFull));
            }
          }
        }
        scanned.fetch_add(sc);
        words.fetch_add(wd);
      });
      edges += scanned.load();
      refbytes += words.load() * 4;
    }
    // C6 aggregate, partitions in ascending order (nothing was packed in a
    // NO_OFFLOAD round).
    for (uint32_t p = 0; p < M; ++p) {
      std::vector<uint32_t> bits = bwd_bv[p].offsets();
      for (size_t j = 0; j < bits.size(); ++j) {
        const uint32_t lid = L.rTrans[p][bits[j]];
        if (A == ORC_PR_DELTA)
          cupd.addUpdate(lid, bwd_buf[p][j]);
        else
          cupd.minUpdate(lid, bwd_buf[p][j]);
      }
      bwd_bv[p].reset();
    }
    // C7 frontier.reset(); update_frontier(); apply_updates();
    frontier.reset();
    for (uint32_t lid : cupd.dirty.offsets()) {
      if (A == ORC_PR_DELTA) {
        const float u = Bits<float>::from(Bits<T>::to(cupd.get(lid)));
        if ((double)u > tol && (double)prev_updates.get(lid) < tol) {
          frontier.set(lid);
          prev_updates.put(lid, u);
        }
      } else {
        const T u = cupd.get(lid);
        if (cprop.get(lid) > u) {
          cprop.put(lid, u);
          frontier.set(lid);
        }
      }
    }
    if (A == ORC_PR_DELTA) {
      for (uint32_t lid : frontier.offsets()) {
        const float u = Bits<float>::from(Bits<T>::to(cupd.get(lid)));
        if ((double)u > tol) {
          pr_vals.put(lid, pr_vals.get(lid) + u);
          cprop.put(lid, (T)(damping * (double)u / (double)L.outdeg[lid]));
          cupd.put(lid, (T)0);
          prev_updates.put(lid, 0.0f);
        }
      }
    }
    done = frontier.count() == 0;  // termination_check()
    cupd.clear_uv();
    cprop.clear_uv();
    ++iteration;
  }
  for (uint32_t n = 0; n < V; ++n) {
    if (props_out) props_out[n] = cprop.get(n);
    if (updates_out) updates_out[n] = cupd.get(n);
    if (ranks_out && A == ORC_PR_DELTA) ranks_out[n] = pr_vals.get(n);
  }
  st.rounds = iteration;
  st.converged = done;
  st.edges_scanned = edges;
  st.bytes_synced = bytes;
  st.reference_bytes_moved = refbytes;
  st.no_offload_rounds = no_offload_rounds;
}

}  // namespace

extern "C" {

struct orc_stats {
  uint32_t rounds;
  uint32_t converged;
  uint64_t edges_scanned;
  uint64_t bytes_synced;
  uint64_t reference_bytes_moved;
  uint32_t no_offload_rounds;
};

// Runs the restated round protocol.  props_out/updates_out receive V 32-bit
// values (u32 for CC/SSSP, float bits for PR); ranks_out receives pr_vals
// (PR only).  threads == 1 gives the deterministic order (ascending lids,
// edges in row order, partitions ascending); threads > 1 mirrors the
// reference's concurrent do_all with atomic CAS updates.
struct orc_layout {
  Layout L;
  bool weighted;
};

// Builds the partitioned layout once (the reference's setup, excluded from
// its run() timing); NULL on invalid arguments.
orc_layout* orc_layout_create(uint32_t V, const uint64_t* ro, const uint32_t* col, const uint32_t* w,
                              const uint32_t* mirror, uint32_t M) {
  if (M == 0 || !ro) return nullptr;
  for (uint32_t g = 0; mirror && g < V; ++g)
    if (mirror[g] >= M) return nullptr;
  orc_layout* h = new orc_layout();
  build(h->L, V, ro, col, w, mirror, M);
  h->weighted = w != nullptr;
  return h;
}

void orc_layout_free(orc_layout* h) { delete h; }

// Runs init() + run() of one algorithm on a prebuilt layout; offload: 0 every
// round NDP_OFFLOAD (the reference), 1 the NDPEngine rule, 2 every round
// NO_OFFLOAD.
int orc_run_layout_ex(const orc_layout* h, int algo, uint32_t source, uint32_t max_rounds, double damping, double tol,
                      int threads, int offload, void* props_out, float* ranks_out, void* updates_out, orc_stats* st) {
  if (!h || !st || offload < OFF_NDP || offload > OFF_NONE) return -1;
  const Layout& L = h->L;
  if ((algo == ORC_SSSP_W) && !h->weighted) return -1;
  if ((algo == ORC_SSSP_HOP || algo == ORC_SSSP_W) && source >= L.V) return -1;
  Pool pool(threads);
  Stats s{};
  switch (algo) {
    case ORC_PR_DELTA:
      run_protocol<float, ORC_PR_DELTA>(L, source, max_rounds, damping, tol, pool, offload, (float*)props_out,
                                        ranks_out, (float*)updates_out, s);
      break;
    case ORC_CC:
      run_protocol<uint32_t, ORC_CC>(L, source, max_rounds, damping, tol, pool, offload, (uint32_t*)props_out,
                                     nullptr, (uint32_t*)updates_out, s);
      break;
    case ORC_SSSP_HOP:
      run_protocol<uint32_t, ORC_SSSP_HOP>(L, source, max_rounds, damping, tol, pool, offload,
                                           (uint32_t*)props_out, nullptr, (uint32_t*)updates_out, s);
      break;
    case ORC_SSSP_W:
      run_protocol<uint32_t, ORC_SSSP_W>(L, source, max_rounds, damping, tol, pool, offload, (uint32_t*)props_out,
                                         nullptr, (uint32_t*)updates_out, s);
      break;
    default:
      return -1;
  }
  st->rounds = s.rounds;
  st->converged = s.converged;
  st->edges_scanned = s.edges_scanned;
  st->bytes_synced = s.bytes_synced;
  st->reference_bytes_moved = s.reference_bytes_moved;
  st->no_offload_rounds = s.no_offload_rounds;
  return 0;
}

int orc_run_layout(const orc_layout* h, int algo, uint32_t source, uint32_t max_rounds, double damping, double tol,
                   int threads, void* props_out, float* ranks_out, void* updates_out, orc_stats* st) {
  return orc_run_layout_ex(h, algo, source, max_rounds, damping, tol, threads, OFF_NDP, props_out, ranks_out,
                           updates_out, st);
}

int orc_run(int algo, uint32_t V, uint64_t E, const uint64_t* ro, const uint32_t* col, const uint32_t* w,
            const uint32_t* mirror, uint32_t M, uint32_t source, uint32_t max_rounds, double damping, double tol,
            int threads, void* props_out, float* ranks_out, void* updates_out, orc_stats* st) {
  (void)E;
  orc_layout* h = orc_layout_create(V, ro, col, w, mirror, M);
  if (!h) return -1;
  int rc = orc_run_layout(h, algo, source, max_rounds, damping, tol, threads, props_out, ranks_out, updates_out, st);
  orc_layout_free(h);
  return rc;
}

// Translation-slot order of memory partition p (owned gids ascending, then
// proxies ascending); returns T_p, writes up to cap gids.
uint32_t orc_layout_slots(uint32_t V, const uint64_t* ro, const uint32_t* col, const uint32_t* mirror, uint32_t M,
                          uint32_t p, uint32_t* out, uint32_t cap, uint32_t* n_owned) {
  Layout L;
  build(L, V, ro, col, nullptr, mirror, M);
  const MemPart& P = L.parts[p];
  for (uint32_t i = 0; i < P.T() && i < cap; ++i) out[i] = P.lid_gid[i];
  if (n_owned) *n_owned = P.n_owned;
  return P.T();
}

// ------------------------------------------------------ textbook oracles --
void orc_bfs(uint32_t V, const uint64_t* ro, const uint32_t* col, uint32_t src, uint32_t* dist) {
  std::fill(dist, dist + V, 0xFFFFFFFFu);
  std::vector<uint32_t> q;
  q.reserve(V);
  dist[src] = 0;
  q.push_back(src);
  for (size_t h = 0; h < q.size(); ++h) {
    uint32_t u = q[h];
    for (uint64_t i = ro[u]; i < ro[u + 1]; ++i)
      if (dist[col[i]] == 0xFFFFFFFFu) {
        dist[col[i]] = dist[u] + 1;
        q.push_back(col[i]);
      }
  }
}

void orc_dijkstra(uint32_t V, const uint64_t* ro, const uint32_t* col, const uint32_t* w, uint32_t src,
                  uint32_t* dist) {
  std::vector<uint64_t> d(V, ~0ull);
  using QE = std::pair<uint64_t, uint32_t>;
  std::priority_queue<QE, std::vector<QE>, std::greater<QE>> pq;
  d[src] = 0;
  pq.push({0, src});
  while (!pq.empty()) {
    auto [du, u] = pq.top();
    pq.pop();
    if (du != d[u]) continue;
    for (uint64_t i = ro[u]; i < ro[u + 1]; ++i) {
      uint64_t nd = du + w[i];
      if (nd < d[col[i]]) {
        d[col[i]] = nd;
        pq.push({nd, col[i]});
      }
    }
  }
  for (uint32_t v = 0; v < V; ++v) dist[v] = d[v] == ~0ull ? 0xFFFFFFFFu : (uint32_t)std::min<uint64_t>(d[v], 0xFFFFFFFEull);
}

// Min gid of each weakly connected component (equals min-label propagation
// on a symmetric graph).
void orc_cc_union_find(uint32_t V, const uint64_t* ro, const uint32_t* col, uint32_t* label) {
  std::vector<uint32_t> parent(V);
  for (uint32_t v = 0; v < V; ++v) parent[v] = v;
  std::function<uint32_t(uint32_t)> find = [&](uint32_t x) {
    while (parent[x] != x) {
      parent[x] = parent[parent[x]];
      x = parent[x];
    }
    return x;
  };
  for (uint32_t u = 0; u < V; ++u)
    for (uint64_t i = ro[u]; i < ro[u + 1]; ++i) {
      uint32_t a = find(u), b = find(col[i]);
      if (a != b) parent[std::max(a, b)] = std::min(a, b);
    }
  for (uint32_t v = 0; v < V; ++v) label[v] = find(v);
}

// FP64 Jacobi iteration on the reference's PageRank fixed point:
//   pr[v] = (1-d)*[outdeg(v) > 0] + d * sum_{u->v} pr[u] / outdeg(u)
// starting from the reference init (pr = 1-d on non-dangling vertices).
// Runs `iters` iterations (or until the L1 residual / V < tol when tol > 0)
// and returns the iteration count; residual_out gets the last residual / V.
uint32_t orc_pr_jacobi_fp64(uint32_t V, const uint64_t* ro, const uint32_t* col, double d, uint32_t iters,
                            double tol, double* pr, double* residual_out) {
  std::vector<double> contrib(V), acc(V);
  for (uint32_t v = 0; v < V; ++v) {
    uint64_t deg = ro[v + 1] - ro[v];
    pr[v] = deg ? (1.0 - d) : 0.0;
  }
  uint32_t it = 0;
  double res = 0;
  while (it < iters) {
    for (uint32_t v = 0; v < V; ++v) {
      uint64_t deg = ro[v + 1] - ro[v];
      contrib[v] = deg ? d * pr[v] / (double)deg : 0.0;
    }
    std::fill(acc.begin(), acc.end(), 0.0);
    for (uint32_t u = 0; u < V; ++u)
      for (uint64_t i = ro[u]; i < ro[u + 1]; ++i) acc[col[i]] += contrib[u];
    res = 0;
    for (uint32_t v = 0; v < V; ++v) {
      uint64_t deg = ro[v + 1] - ro[v];
      double nv = (deg ? (1.0 - d) : 0.0) + acc[v];
      res += std::fabs(nv - pr[v]);
      pr[v] = nv;
    }
    res /= (double)V;
    ++it;
    if (tol > 0 && res < tol) break;
  }
  if (residual_out) *residual_out = res;
  return it;
}

// Same iteration as orc_pr_jacobi_fp64, parallel over destinations (in-edge
// lists, each summed in ascending source order, so the result does not
// depend on the thread count).  Used as the FP64 reference at full size.
uint32_t orc_pr_jacobi_fp64_mt(uint32_t V, const uint64_t* ro, const uint32_t* col, double d, uint32_t iters,
                               double tol, int threads, double* pr, double* residual_out) {
  // in-lists in ascending source order; thread t fills the destinations of
  // [V*t/T, V*(t+1)/T) while scanning every row in source order
  const int T = std::max(1, threads);
  std::vector<uint64_t> in_off((size_t)V + 1, 0);
  {
    std::vector<std::thread> ts;
    for (int t = 0; t < T; ++t)
      ts.emplace_back([&, t] {
        const uint32_t lo = (uint32_t)((uint64_t)V * t / T), hi = (uint32_t)((uint64_t)V * (t + 1) / T);
        for (uint64_t i = 0; i < ro[V]; ++i)
          if (col[i] >= lo && col[i] < hi) in_off[col[i] + 1]++;
      });
    for (auto& th : ts) th.join();
  }
  for (uint32_t v = 0; v < V; ++v) in_off[v + 1] += in_off[v];
  std::vector<uint32_t> in_src(ro[V] ? ro[V] : 1);
  {
    std::vector<std::thread> ts;
    for (int t = 0; t < T; ++t)
      ts.emplace_back([&, t] {
        const uint32_t lo = (uint32_t)((uint64_t)V * t / T), hi = (uint32_t)((uint64_t)V * (t + 1) / T);
        std::vector<uint64_t> cur(in_off.begin() + lo, in_off.begin() + hi);
        for (uint32_t u = 0; u < V; ++u)
          for (uint64_t i = ro[u]; i < ro[u + 1]; ++i)
            if (col[i] >= lo && col[i] < hi) in_src[cur[col[i] - lo]++] = u;
      });
    for (auto& th : ts) th.join();
  }
  Pool pool(threads);
  std::vector<double> contrib(V);
  for (uint32_t v = 0; v < V; ++v) pr[v] = (ro[v + 1] > ro[v]) ? (1.0 - d) : 0.0;
  uint32_t it = 0;
  double res = 0;
  const int nt = pool.size();
  std::vector<double> part(nt > 0 ? 1024 : 1);
  while (it < iters) {
    pool.run(V, 65536, [&](uint64_t b, uint64_t e) {
      for (uint64_t v = b; v < e; ++v) {
        uint64_t deg = ro[v + 1] - ro[v];
        contrib[v] = deg ? d * pr[v] / (double)deg : 0.0;
      }
    });
    std::atomic<uint64_t> res_bits{0};
    std::mutex mu;
    double res_acc = 0;
    pool.run(V, 65536, [&](uint64_t b, uint64_t e) {
      double local = 0;
      for (uint64_t v = b; v < e; ++v) {
        double acc = 0;
        for (uint64_t i = in_off[v]; i < in_off[v + 1]; ++i) acc += contrib[in_src[i]];
        double nv = ((ro[v + 1] > ro[v]) ? (1.0 - d) : 0.0) + acc;
        local += std::fabs(nv - pr[v]);
        pr[v] = nv;
      }
      std::lock_guard<std::mutex> g(mu);
      res_acc += local;
    });
    (void)res_bits;
    res = res_acc / (double)V;
    ++it;
    if (tol > 0 && res < tol) break;
  }
  if (residual_out) *residual_out = res;
  return it;
}

}  // extern "C"
