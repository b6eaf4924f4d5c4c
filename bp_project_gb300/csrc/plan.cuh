// Host-side FFBP plan object (shared by the single-scene plan entry points and the
// scene batch, which reuses plans built by sarbp_ffbp_plan_create).
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

struct sarbp_ffbp_plan {
    int mode = SARBP_SPLIT;
    int n_nodes = 0;
    std::vector<sarbp::PolarDesc> nodes;
    std::vector<int> height;
    int max_height = 0;
    // Split: tile items; plain: 256-pixel blocks.  Stage h occupies [stage_begin[h], +stage_count[h]).
    std::vector<sarbp::TileItem> items;
    std::vector<int2> blocks;
    std::vector<int> stage_begin, stage_count;
    int leaf_chunk = 1, leaf_wb = 4;
    long long table_entries = 0;  // split: float4 row/column geometry entries of all nodes
    int max_dim = 1;
    std::vector<int> leaves;      // split: leaf node indices
    int max_pulse = 0;            // split: largest pulse index + 1 used by a leaf
    int leaf_span_bins = 4;       // split: range bins a 32-row leaf tile spans (before the pulse offsets)
    long long merge_items = 0;    // split: tile items of all merge levels (contiguous after the leaves)
    size_t node_bytes = 0, work_bytes = 0, leaf_list_bytes = 0, table_bytes = 0, table_offset = 0,
           prec_offset = 0, prec_bytes = 0, crec_offset = 0, crec_bytes = 0, arena_offset = 0, arena_bytes = 0,
           total_bytes = 0;
    void* bound = nullptr;
    size_t bound_bytes = 0;
    int launches = 0;
    int n_external = 0;           // leaves whose images the caller supplies (pulse range [-1, -1))
    // Split: all merge levels as one dependency-counting queue launch instead of one per height
    // (off by default: it measured 6-20% slower on the 4096-pulse plan).
    bool merge_queue = false;
    std::vector<int> q_remaining, q_pending, q_parent;  // per node: merge tiles, merge children, parent
    size_t queue_offset = 0, queue_bytes = 0;
    unsigned long long queue_limit_ns = 5000000000ull;  // wait limit per merge item
    int withheld = -1;            // a node that never becomes ready (tests of the wait limit), or -1
    // Split: merge tiles stage their children's footprints in shared memory by TMA, through one
    // tensor map per child image (encoded at bind).  staging: requested (default on); staged:
    // the tensor maps were encoded at the last bind.
    bool staging = true, staged = false;
    std::vector<size_t> merge_box_bytes;  // per height: a merge tile's footprint bytes (0: not staged)
    size_t tmap_offset = 0, tmap_bytes = 0;
};

// Range extent (m) of the tallest leaf tile of a split plan: the leaf kernel's range window per
// pulse covers it plus the pulse's offset from the leaf centre.
inline double ffbp_leaf_tile_span(const sarbp_ffbp_plan& p) {
    double span = 0.0;
    for (int i : p.leaves) {
        const sarbp::PolarDesc& d = p.nodes[i];
        span = std::max(span, (double)(sarbp::kSplitTilePixels >> d.tile_lc) * fabs(d.dr));
    }
    return span;
}
