// Scene batches: many independent scenes (direct lattice images and FFBP trees of
// uneven pulse and pixel counts) formed by persistent work-queue kernels.
//
// Host side: every FFBP scene is planned by sarbp_ffbp_plan_create (split mode);
// its nodes, tiles, tables, pulse records, child records and node images are then
// re-based into batch-wide arrays, so one set of launches covers all scenes:
//   memset(queue counters) -> tables -> leaf pulse records -> merge child records
//   -> one persistent launch over every direct tile (largest first, so the queue drains
//      evenly) and one over every FFBP leaf tile
//   -> one persistent merge launch per tree height over every scene's nodes of
//      that height.
// Items are independent within a launch, and heights are separated by launches, so
// no kernel waits on another CTA.  The result of each scene is bit-identical to the
// single-scene entry points with the same tile shape.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "plan.cuh"

using namespace sarbp;

struct sarbp_batch {
    int n_scenes = 0;
    std::vector<char> scenes;     // device form of every scene (split_batch_scene_bytes each)
    std::vector<PolarDesc> nodes;
    std::vector<int> leaves;
    std::vector<TileItem> bp_items, merge_items;
    std::vector<int> level_begin, level_count;  // merge heights 1..max_height at index h - 1
    int max_height = 0, max_dim = 1;
    long long table_entries = 0, pulse_records = 0;
    size_t direct_smem = 0, leaf_smem = 0;
    int n_direct = 0;             // bp_items[0, n_direct) are direct tiles, the rest leaf tiles
    int bp_blocks = 1, leaf_blocks = 1, merge_blocks = 1;
    int direct_scenes = 0, ffbp_scenes = 0;
    double pixel_pulses = 0.0;    // direct-equivalent work: pixels x pulses summed over scenes
    size_t scene_off = 0, node_off = 0, bp_off = 0, merge_off = 0, leaf_off = 0, counter_off = 0, table_off = 0,
           prec_off = 0, crec_off = 0, arena_off = 0, total = 0;
    void* bound = nullptr;
    unsigned long long* trace = nullptr;  // per-scene completion times (ns) + the start time, or none
    int launches = 0;
    // Concurrent mode: the FFBP chain (prologues, leaves, merges) runs on `side`, forked from and
    // joined back to the caller's stream with events, beside the direct queue on the caller's
    // stream.  A graph captured on the caller's stream records both branches.
    bool concurrent = false;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;

    ~sarbp_batch() {
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
    }
};

namespace {

constexpr size_t kAlign = 512;
size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

bool finite_value(double v) { return isfinite(v) != 0; }

int check_scene(const sarbp_batch_scene& s, int i) {
    if (!s.data || !s.pos || !s.weight || !s.phase || !s.out)
        return fail(SARBP_ERR_TYPE, "scene %d: data, pos, weight, phase and out must be device pointers", i);
    if (s.pulses < 1 || s.samples < 1) return fail(SARBP_ERR_VALUE, "scene %d: pulses and samples must be positive", i);
    if (!finite_value(s.data_dr) || s.data_dr == 0.0 || !finite_value(s.k) || !finite_value(s.range_start))
        return fail(SARBP_ERR_VALUE, "scene %d: range_start, data_dr and k must be finite, data_dr non-zero", i);
    if (s.kind == SARBP_BATCH_DIRECT) {
        const sarbp_lattice& L = s.lattice;
        if (L.rows <= 0 || L.cols <= 0) return fail(SARBP_ERR_VALUE, "scene %d: empty image grids are unsupported", i);
        for (int c = 0; c < 3; ++c)
            if (!finite_value(L.origin[c]) || !finite_value(L.step_row[c]) || !finite_value(L.step_col[c]))
                return fail(SARBP_ERR_VALUE, "scene %d: lattice geometry must be finite", i);
        if (L.step_row[2] != 0.0 || L.step_col[2] != 0.0)
            return fail(SARBP_ERR_VALUE, "scene %d: batched direct scenes need a flat (z-constant) lattice", i);
        if (s.tile_lc != 0 && (s.tile_lc < 2 || s.tile_lc > 5))
            return fail(SARBP_ERR_VALUE, "scene %d: tile_lc must be 0 (default) or 2..5", i);
    } else if (s.kind == SARBP_BATCH_FFBP) {
        if (!s.nodes || s.n_nodes < 1) return fail(SARBP_ERR_VALUE, "scene %d: an FFBP scene needs its plan nodes", i);
    } else {
        return fail(SARBP_ERR_VALUE, "scene %d: kind must be SARBP_BATCH_DIRECT or SARBP_BATCH_FFBP", i);
    }
    if (s.chunk_pulses < 0) return fail(SARBP_ERR_VALUE, "scene %d: chunk_pulses must be >= 0", i);
    return SARBP_OK;
}

PulseInputs scene_inputs(const sarbp_batch_scene& s) {
    PulseInputs in;
    in.data = reinterpret_cast<const float2*>(s.data);
    in.pulses = s.pulses;
    in.samples = s.samples;
    in.pos = s.pos;
    in.weight = s.weight;
    in.phase = s.phase;
    in.range_start = s.range_start;
    in.data_dr = s.data_dr;
    in.k = s.k;
    return in;
}

}  // namespace

extern "C" {

int sarbp_batch_create(const sarbp_batch_scene* scenes, int n_scenes, int blocks_per_sm, sarbp_batch** batch_out) {
    if (!batch_out) return fail(SARBP_ERR_TYPE, "batch pointer must not be NULL");
    *batch_out = nullptr;
    if (!scenes || n_scenes < 1) return fail(SARBP_ERR_VALUE, "a batch needs at least one scene");
    if (blocks_per_sm < 0 || blocks_per_sm > 8) return fail(SARBP_ERR_VALUE, "blocks_per_sm must be 0 (auto) to 8");
    for (int i = 0; i < n_scenes; ++i)
        if (int st = check_scene(scenes[i], i)) return st;
    auto* b = new sarbp_batch();
    b->n_scenes = n_scenes;
    const size_t scene_bytes = split_batch_scene_bytes();
    b->scenes.assign(scene_bytes * n_scenes, 0);
    size_t arena = 0;
    std::vector<double> bp_cost;
    std::vector<std::vector<TileItem>> merges_by_height;
    for (int i = 0; i < n_scenes; ++i) {
        const sarbp_batch_scene& s = scenes[i];
        BatchSceneDesc d{};
        d.in = scene_inputs(s);
        d.kind = s.kind;
        d.out = reinterpret_cast<float2*>(s.out);
        if (s.kind == SARBP_BATCH_DIRECT) {
            const int lc = s.tile_lc ? s.tile_lc : 5;
            d.lat = s.lattice;
            d.lc = lc;
            d.window_bins = split_window_bins(lattice_radius(s.lattice, lc), s.data_dr);
            d.chunk = split_chunk_for(d.window_bins, s.chunk_pulses ? s.chunk_pulses : 64);
            const int cols_t = 1 << lc, rows_t = kSplitTilePixels >> lc;
            for (int r = 0; r < s.lattice.rows; r += rows_t)
                for (int u = 0; u < s.lattice.cols; u += cols_t) {
                    b->bp_items.push_back(TileItem{-1, r, u, i});
                    bp_cost.push_back((double)kSplitTilePixels * s.pulses);
                }
            b->pixel_pulses += (double)s.lattice.rows * s.lattice.cols * s.pulses;
            ++b->direct_scenes;
        } else {
            sarbp_ffbp_plan* p = nullptr;
            if (int st = sarbp_ffbp_plan_create(s.nodes, s.n_nodes, s.crop_r0, s.crop_u0, s.crop_nr, s.crop_nu,
                                                SARBP_SPLIT, &p)) {
                delete b;
                return fail(st, "scene %d: %s", i, sarbp_last_error());
            }
            if (p->n_external) {
                sarbp_ffbp_plan_destroy(p);
                delete b;
                return fail(SARBP_ERR_PLAN, "scene %d: batched FFBP plans cannot have external nodes", i);
            }
            for (int n = 0; n < p->n_nodes; ++n)
                if (p->nodes[n].left < 0 && p->nodes[n].b > s.pulses) {
                    sarbp_ffbp_plan_destroy(p);
                    delete b;
                    return fail(SARBP_ERR_PLAN, "scene %d: leaf %d uses pulses beyond the %d supplied", i, n, s.pulses);
                }
            const int node0 = (int)b->nodes.size();
            for (int n = 0; n < p->n_nodes; ++n) {
                PolarDesc g = p->nodes[n];
                if (g.left >= 0) g.left += node0;
                if (g.right >= 0) g.right += node0;
                g.rows_off += b->table_entries;
                g.cols_off += b->table_entries;
                g.pad = i;
                if (n == 0)
                    g.dst = reinterpret_cast<float2*>(s.out);  // the root writes its crop window to the scene output
                else
                    g.out_offset += (long long)(arena / sizeof(float2));
                b->nodes.push_back(g);
            }
            for (int leaf : p->leaves) b->leaves.push_back(leaf + node0);
            // Leaf window and chunk exactly as sarbp_ffbp_execute chooses them.
            d.window_bins = (int)ceil(ffbp_leaf_tile_span(*p) / fabs(s.data_dr)) + 48;
            d.chunk = split_chunk_for(d.window_bins, s.chunk_pulses ? s.chunk_pulses : p->leaf_chunk, true);
            d.prec_offset = b->pulse_records;
            for (int t = p->stage_begin[0]; t < p->stage_begin[0] + p->stage_count[0]; ++t) {
                TileItem it = p->items[t];
                const PolarDesc& g = p->nodes[it.node];
                it.node += node0;
                it.pad = i;
                b->bp_items.push_back(it);
                bp_cost.push_back((double)kSplitTilePixels * (g.b - g.a));
            }
            if ((int)merges_by_height.size() < p->max_height) merges_by_height.resize(p->max_height);
            for (int h = 1; h <= p->max_height; ++h)
                for (int t = p->stage_begin[h]; t < p->stage_begin[h] + p->stage_count[h]; ++t) {
                    TileItem it = p->items[t];
                    it.node += node0;
                    it.pad = i;
                    merges_by_height[h - 1].push_back(it);
                }
            b->max_height = std::max(b->max_height, p->max_height);
            b->max_dim = std::max(b->max_dim, p->max_dim);
            b->table_entries += p->table_entries;
            b->pulse_records += p->max_pulse;
            arena += p->arena_bytes;
            b->pixel_pulses += (double)s.crop_nr * s.crop_nu * s.pulses;
            sarbp_ffbp_plan_destroy(p);
            ++b->ffbp_scenes;
        }
        const size_t smem = split_batch_pack_scene(d, b->scenes.data() + scene_bytes * i);
        if (s.kind == SARBP_BATCH_DIRECT)
            b->direct_smem = std::max(b->direct_smem, smem);
        else
            b->leaf_smem = std::max(b->leaf_smem, smem);
    }
    // Direct tiles first, largest first (stable: scenes and tiles keep their order among equals),
    // then the leaf tiles.
    std::vector<int> order(b->bp_items.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const bool dx = b->bp_items[x].node < 0, dy = b->bp_items[y].node < 0;
        if (dx != dy) return dx;
        return bp_cost[x] > bp_cost[y];
    });
    for (const TileItem& it : b->bp_items) b->n_direct += it.node < 0 ? 1 : 0;
    std::vector<TileItem> sorted(order.size());
    for (size_t t = 0; t < order.size(); ++t) sorted[t] = b->bp_items[order[t]];
    b->bp_items.swap(sorted);
    for (int h = 1; h <= b->max_height; ++h) {
        b->level_begin.push_back((int)b->merge_items.size());
        b->level_count.push_back((int)merges_by_height[h - 1].size());
        b->merge_items.insert(b->merge_items.end(), merges_by_height[h - 1].begin(), merges_by_height[h - 1].end());
    }
    if (b->bp_items.size() > (size_t)INT32_MAX || b->merge_items.size() > (size_t)INT32_MAX / 2) {
        delete b;
        return fail(SARBP_ERR_PLAN, "batch too large");
    }
    // Persistent grids: every resident CTA slot of the GPU (or blocks_per_sm per SM).
    int dev = 0, sms = 1, direct_occ = 1, leaf_occ = 1, merge_occ = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        delete b;
        return fail(SARBP_ERR_CUDA, "batch: %s", cudaGetErrorString(e));
    }
    const size_t min_smem = 1024;
    if (int st = split_batch_occupancy(std::max(b->direct_smem, min_smem), std::max(b->leaf_smem, min_smem),
                                       &direct_occ, &leaf_occ, &merge_occ)) {
        delete b;
        return st;
    }
    if (direct_occ < 1 || leaf_occ < 1) {
        delete b;
        return fail(SARBP_ERR_VALUE, "batch: %zu / %zu bytes of shared memory per CTA do not fit an SM",
                    b->direct_smem, b->leaf_smem);
    }
    const int n_leaf = (int)b->bp_items.size() - b->n_direct;
    const int per_sm = blocks_per_sm ? std::min(blocks_per_sm, direct_occ) : direct_occ;
    b->bp_blocks = std::max(1, std::min(b->n_direct, sms * per_sm));
    b->leaf_blocks = std::max(1, std::min(n_leaf, sms * leaf_occ));
    b->merge_blocks = std::max(1, sms * std::max(1, merge_occ));
    // Workspace layout.
    b->scene_off = 0;
    b->node_off = align_up(b->scenes.size());
    b->bp_off = b->node_off + align_up(sizeof(PolarDesc) * b->nodes.size());
    b->merge_off = b->bp_off + align_up(sizeof(TileItem) * b->bp_items.size());
    b->leaf_off = b->merge_off + align_up(sizeof(TileItem) * b->merge_items.size());
    b->counter_off = b->leaf_off + align_up(sizeof(int) * b->leaves.size());
    b->table_off = b->counter_off + align_up(sizeof(int) * (2 + b->max_height));
    b->prec_off = b->table_off + align_up(sizeof(float4) * (size_t)b->table_entries);
    b->crec_off = b->prec_off + align_up(split_ffbp_pulse_record_bytes() * (size_t)b->pulse_records);
    b->arena_off = b->crec_off + align_up(split_ffbp_child_record_bytes() * 2 * b->merge_items.size());
    b->total = b->arena_off + arena;
    b->launches = 1 + (b->ffbp_scenes ? 4 : 0) + (b->direct_scenes ? 1 : 0) + b->max_height;
    *batch_out = b;
    return SARBP_OK;
}

void sarbp_batch_destroy(sarbp_batch* batch) { delete batch; }

size_t sarbp_batch_workspace_bytes(const sarbp_batch* batch) { return batch ? batch->total : 0; }

int sarbp_batch_launch_count(const sarbp_batch* batch) { return batch ? batch->launches : 0; }

int sarbp_batch_set_trace(sarbp_batch* batch, unsigned long long* trace) {
    if (!batch) return fail(SARBP_ERR_TYPE, "batch must not be NULL");
    batch->trace = trace;
    return SARBP_OK;
}

int sarbp_batch_info(const sarbp_batch* batch, int* bp_items, int* merge_items, int* max_height, int* bp_blocks,
                     double* pixel_pulses) {
    if (!batch) return fail(SARBP_ERR_TYPE, "batch must not be NULL");
    if (bp_items) *bp_items = (int)batch->bp_items.size();
    if (merge_items) *merge_items = (int)batch->merge_items.size();
    if (max_height) *max_height = batch->max_height;
    if (bp_blocks) *bp_blocks = batch->bp_blocks;
    if (pixel_pulses) *pixel_pulses = batch->pixel_pulses;
    return SARBP_OK;
}

int sarbp_batch_bind(sarbp_batch* batch, void* workspace, size_t workspace_bytes, void* stream) {
    if (!batch) return fail(SARBP_ERR_TYPE, "batch must not be NULL");
    if (!workspace || workspace_bytes < batch->total)
        return fail(SARBP_ERR_WORKSPACE, "batch needs %zu workspace bytes", batch->total);
    if ((uintptr_t)workspace % 256) return fail(SARBP_ERR_TYPE, "workspace must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    char* base = reinterpret_cast<char*>(workspace);
    struct Copy {
        size_t off;
        const void* src;
        size_t bytes;
    } copies[] = {
        {batch->scene_off, batch->scenes.data(), batch->scenes.size()},
        {batch->node_off, batch->nodes.data(), sizeof(PolarDesc) * batch->nodes.size()},
        {batch->bp_off, batch->bp_items.data(), sizeof(TileItem) * batch->bp_items.size()},
        {batch->merge_off, batch->merge_items.data(), sizeof(TileItem) * batch->merge_items.size()},
        {batch->leaf_off, batch->leaves.data(), sizeof(int) * batch->leaves.size()},
    };
    cudaError_t e = cudaSuccess;
    for (const Copy& c : copies)
        if (c.bytes && e == cudaSuccess) e = cudaMemcpyAsync(base + c.off, c.src, c.bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "batch bind: %s", cudaGetErrorString(e));
    batch->bound = workspace;
    return SARBP_OK;
}

int sarbp_batch_set_concurrent(sarbp_batch* batch, int on) {
    if (!batch) return fail(SARBP_ERR_TYPE, "batch must not be NULL");
    if (on != 0 && on != 1) return fail(SARBP_ERR_VALUE, "on must be 0 or 1 (got %d)", on);
    if (on && !batch->side) {
        cudaError_t e = cudaStreamCreateWithFlags(&batch->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&batch->fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&batch->join, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "batch side stream: %s", cudaGetErrorString(e));
    }
    batch->concurrent = on != 0;
    return SARBP_OK;
}

int sarbp_batch_execute(const sarbp_batch* batch, void* stream) {
    if (!batch) return fail(SARBP_ERR_TYPE, "batch must not be NULL");
    if (!batch->bound) return fail(SARBP_ERR_PLAN, "sarbp_batch_bind must succeed before execute");
    cudaStream_t s = (cudaStream_t)stream;
    char* base = reinterpret_cast<char*>(batch->bound);
    const void* scenes = base + batch->scene_off;
    const PolarDesc* nodes = reinterpret_cast<const PolarDesc*>(base + batch->node_off);
    const TileItem* bp_items = reinterpret_cast<const TileItem*>(base + batch->bp_off);
    const TileItem* merge_items = reinterpret_cast<const TileItem*>(base + batch->merge_off);
    const int* leaves = reinterpret_cast<const int*>(base + batch->leaf_off);
    int* counters = reinterpret_cast<int*>(base + batch->counter_off);
    float4* tables = reinterpret_cast<float4*>(base + batch->table_off);
    void* precs = base + batch->prec_off;
    char* crecs = base + batch->crec_off;
    float2* arena = reinterpret_cast<float2*>(base + batch->arena_off);
    cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(int) * (2 + batch->max_height), s);
    unsigned long long* trace = batch->trace;
    if (trace && e == cudaSuccess) e = cudaMemsetAsync(trace, 0, sizeof(unsigned long long) * batch->n_scenes, s);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "batch counters: %s", cudaGetErrorString(e));
    int st = trace ? launch_split_batch_trace_start(trace + batch->n_scenes, s) : SARBP_OK;
    // The FFBP chain goes to the side stream when the batch runs concurrently and has both kinds.
    const bool fork = batch->concurrent && batch->ffbp_scenes && batch->direct_scenes;
    cudaStream_t fs = fork ? batch->side : s;
    if (st == SARBP_OK && fork) {
        e = cudaEventRecord(batch->fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(fs, batch->fork, 0);
        if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "batch fork: %s", cudaGetErrorString(e));
    }
    if (st == SARBP_OK && batch->ffbp_scenes)
        st = launch_split_batch_prologue(scenes, nodes, (int)batch->nodes.size(), batch->max_dim, leaves,
                                         (int)batch->leaves.size(), merge_items, (int)batch->merge_items.size(),
                                         tables, precs, crecs, arena, fs);
    const int n_leaf = (int)batch->bp_items.size() - batch->n_direct;
    if (st == SARBP_OK)
        st = launch_split_batch_direct(scenes, bp_items, batch->n_direct, counters, batch->bp_blocks,
                                       batch->direct_smem, trace, s);
    if (st == SARBP_OK)
        st = launch_split_batch_leaves(scenes, nodes, bp_items + batch->n_direct, n_leaf, tables, precs, arena,
                                       counters + 1, batch->leaf_blocks, batch->leaf_smem, trace, fs);
    const size_t crec_size = split_ffbp_child_record_bytes();
    for (int h = 1; h <= batch->max_height && st == SARBP_OK; ++h) {
        const int first = batch->level_begin[h - 1], count = batch->level_count[h - 1];
        st = launch_split_batch_merges(scenes, nodes, merge_items + first, count, tables,
                                       crecs + 2 * (size_t)first * crec_size, arena, counters + 1 + h,
                                       std::min(batch->merge_blocks, std::max(1, count)), trace, fs);
    }
    if (fork) {
        // Join even after a failed launch, so that a stream capture is never left forked.
        e = cudaEventRecord(batch->join, fs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, batch->join, 0);
        if (e != cudaSuccess && st == SARBP_OK) st = fail(SARBP_ERR_CUDA, "batch join: %s", cudaGetErrorString(e));
    }
    return st;
}

}  // extern "C"
