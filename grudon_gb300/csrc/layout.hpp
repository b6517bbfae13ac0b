// Host-side partition layout: the 1-compute + M-memory-partition index space
// of the reference's DistributedGraph (src/DistributedGraph.cpp:13-785),
// flattened into one global slot space for single-GPU residency.
//
// Slot order per memory partition p follows the reference exactly
// (src/DistributedGraph.cpp:579-588, 630-758): p's owned vertices in
// ascending gid order, then p's proxies (remote destinations of p's edges)
// in ascending gid order.  With one compute partition the translation slot of
// a memory-side lid equals the lid, so sTranslationTable/rTranslationTable
// collapse to the slot -> gid array below.
//
// Partitions are concatenated; each starts on a TILE_SLOTS boundary so a
// compaction tile never spans two partitions and every partition's sync
// bitvector starts on a 64-bit word.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace grd {

constexpr uint32_t TILE_SLOTS = 8192;       // slots per compaction tile
constexpr uint32_t TILE_WORDS = TILE_SLOTS / 32;  // u32 bitvector words
constexpr uint32_t INVALID = 0xFFFFFFFFu;
constexpr uint32_t HUB_DEGREE = 2048;       // rows above this go to hub chunks
constexpr uint32_t HUB_CHUNK = 4096;        // edges per hub work item
constexpr uint32_t PULL_HUB = 1024;         // in-lists above this pull per block
constexpr uint32_t PULL_MED = 64;           // in-lists above this (up to PULL_HUB) pull per warp

struct HubChunk {
  uint32_t slot;   // global slot of the hub row
  uint32_t e0, e1; // edge range [e0, e1) of this work item
};

struct Layout {
  uint32_t V = 0;
  uint64_t E = 0;
  uint32_t M = 0;
  bool weighted = false;

  std::vector<uint32_t> n_owned, n_proxy, slot_base;  // per partition
  std::vector<uint64_t> part_edges;                   // per partition
  uint64_t S = 0;                                     // padded slot count

  std::vector<uint32_t> slot_gid;  // [S]  gid of slot, INVALID for padding
  std::vector<uint32_t> row_off;   // [S+1] out-edge offsets (proxies: empty)
  std::vector<uint32_t> col;       // [E]  destination global slot
  std::vector<uint32_t> wgt;       // [E]  edge weight (weighted graphs)
  std::vector<uint32_t> outdeg;    // [V]  global out-degree (compute side)
  std::vector<uint32_t> mirror;    // [V]  memory partition of each gid

  // In-edge (CSC) view of each partition, for pull traversal: for each
  // destination slot, the owned source slots in ascending order.
  std::vector<uint32_t> in_off;  // [S+1]
  std::vector<uint32_t> in_src;  // [E]
  std::vector<uint32_t> in_wgt;  // [E]
  std::vector<HubChunk> in_hubs; // destinations with more than PULL_HUB in-edges
  std::vector<HubChunk> in_meds; // destinations with PULL_MED+1 .. PULL_HUB in-edges

  std::vector<HubChunk> hubs;        // static hub work items (all partitions)
  std::vector<uint32_t> tile_part;   // [S/TILE_SLOTS] partition of each tile
  std::vector<uint32_t> tile_first;  // [S/TILE_SLOTS] first tile of that partition

  uint64_t num_tiles() const { return S / TILE_SLOTS; }
  uint32_t T(uint32_t p) const { return n_owned[p] + n_proxy[p]; }
  uint64_t bitvec_words64(uint32_t p) const { return ((uint64_t)T(p) + 63) / 64; }
};

// Builds the layout; returns an empty string on success, else the reason.
std::string build_layout(uint32_t V, uint64_t E, const uint64_t* row_offsets, const uint32_t* col,
                         const uint32_t* weights, const uint32_t* mirror_part, uint32_t M, Layout& out,
                         int threads = 0);

// Fills in_off/in_src/in_wgt (idempotent).
void build_in_edges(Layout& L);

}  // namespace grd
