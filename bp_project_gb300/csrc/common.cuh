// Shared device helpers and internal launcher declarations for libsarbp.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sarbp.h"

namespace sarbp {

// x + kMagic - kMagic rounds |x| < 2^22 to the nearest integer in FP32, and
// the bit pattern of (x + kMagic) is kMagicBits + round(x).
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
constexpr double kInvTwoPi = 0.159154943091895335768883763372514362;
constexpr float kTwoPiF = 6.28318530717958647692f;

// ---- host-side bookkeeping (capi.cu) -----------------------------------------
int fail(int status, const char* fmt, ...);
int check_launch(const char* what);
void note_launches(int n);

inline int grid_blocks(int64_t count, int block) { return (int)((count + block - 1) / block); }

// ---- device helpers ------------------------------------------------------------
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float round_magic(float x) { return (x + kMagic) - kMagic; }

// Four-point Lagrange weights at taps i-1..i+2 for fraction t, written as in
// the reference (fast_bp/gpu/kernels.cu:8-20, ffbp.py:17-21).
template <class T>
__device__ __forceinline__ void lagrange_ref(T t, T w[4]) {
    w[0] = -t * (t - T(1)) * (t - T(2)) / T(6);
    w[1] = (t + T(1)) * (t - T(1)) * (t - T(2)) / T(2);
    w[2] = -(t + T(1)) * t * (t - T(2)) / T(2);
    w[3] = (t + T(1)) * t * (t - T(1)) / T(6);
}

// Lagrange weights in the centred variable s = t - 1/2 in [-1/2, 1/2]; the
// same cubic as lagrange_ref, with nine FP32 operations and no division.
__device__ __forceinline__ void lagrange_centred(float s, float w[4]) {
    const float a = fmaf(s, s, -0.25f);     // s^2 - 1/4
    const float a6 = a * (1.0f / 6.0f);
    const float b2 = fmaf(a, 0.5f, -1.0f);  // (s^2 - 9/4) / 2
    const float c1 = 1.5f * a6;
    const float c2 = 0.5f * b2;
    w[0] = fmaf(-a6, s, c1);
    w[3] = fmaf(a6, s, c1);
    w[1] = fmaf(b2, s, -c2);
    w[2] = fmaf(-b2, s, -c2);
}

// Horner coefficients of the interpolating cubic through taps x0..x3 (at
// t = -1, 0, 1, 2) in s = t - 1/2: v(s) = ((C3 s + C2) s + C1) s + C0.
__device__ __forceinline__ void cubic_coefficients(float2 x0, float2 x1, float2 x2, float2 x3, float a,
                                                   float4& c01, float4& c23) {
    const float s03r = x0.x + x3.x, s03i = x0.y + x3.y;
    const float s12r = x1.x + x2.x, s12i = x1.y + x2.y;
    const float d30r = x3.x - x0.x, d30i = x3.y - x0.y;
    const float d21r = x2.x - x1.x, d21i = x2.y - x1.y;
    c01.x = a * fmaf(9.0f / 16.0f, s12r, -(1.0f / 16.0f) * s03r);
    c01.y = a * fmaf(9.0f / 16.0f, s12i, -(1.0f / 16.0f) * s03i);
    c01.z = a * fmaf(9.0f / 8.0f, d21r, -(1.0f / 24.0f) * d30r);
    c01.w = a * fmaf(9.0f / 8.0f, d21i, -(1.0f / 24.0f) * d30i);
    c23.x = a * 0.25f * (s03r - s12r);
    c23.y = a * 0.25f * (s03i - s12i);
    c23.z = a * fmaf(1.0f / 6.0f, d30r, -0.5f * d21r);
    c23.w = a * fmaf(1.0f / 6.0f, d30i, -0.5f * d21i);
}

// Split a FP64 value into a multiple of 2^e (exact in FP32 when |v| < 2^(e+24))
// and a FP32 remainder.
__device__ __forceinline__ void quantize(double v, double scale, double inv_scale, float& hi, float& lo) {
    const double h = rint(v * inv_scale) * scale;
    hi = (float)h;
    lo = (float)(v - h);
}

// ---- descriptors shared by the split and plain FFBP paths ----------------------
struct PolarDesc {
    double ox, oy, oz;
    double r0, dr, u0, du;
    int nr, nu, side;
    int a, b;        // pulse range for leaves / direct jobs
    int left, right; // child nodes (-1 for leaves)
    int win_r0, win_u0, win_nr, win_nu;  // computed window of the grid
    long long out_offset;                // element offset of the output image in the image arena
    long long out_stride;                // row stride (elements) of the output image
    int tile_lc;                         // split kernels: log2 of tile columns (2..5); tile rows = 1024 >> tile_lc
    int pad;
    long long rows_off;                  // FFBP: first entry of this node's row table (float4 (g_hi, g_lo, psi, 0))
    long long cols_off;                  // FFBP: first entry of this node's column table (float4 (c_hi, c_lo, u_hi, u_lo))
    float2* dst;                         // if set: where the node's window is written (batched scene roots)
    // The FP64 geometry as two-float pairs (hi, lo), split on the host, so that per-tile set-up
    // on the GPU needs no FP64: origin x/y/z, r0, dr, u0, du, 1/dr, 1/du.
    float2 tf[9];
    // FFBP children in split mode: the rectangle of this node's image that a merge tile of its
    // parent reads, staged in shared memory by one TMA copy per tile.  It starts box_r rows and
    // box_u columns (then rounded down to an even column) before the stencil bin of the parent
    // tile's centre pixel and is box_h x box_w elements; box_w == 0: not staged.
    int box_r, box_u, box_h, box_w;
};

// Fills PolarDesc::tf from the FP64 fields (host).
inline void split_geometry(PolarDesc& d) {
    const double v[9] = {d.ox, d.oy, d.oz, d.r0, d.dr, d.u0, d.du, 1.0 / d.dr, 1.0 / d.du};
    for (int i = 0; i < 9; ++i) {
        const float h = (float)v[i];
        d.tf[i] = make_float2(h, (float)(v[i] - (double)h));
    }
}

struct TileItem {
    int node;
    int tile_r;  // first window row of the tile
    int tile_u;  // first window col of the tile
    int pad;
};

// ---- launchers (defined in plain.cu / split.cu) ------------------------------
struct PulseInputs {
    const float2* data;
    int pulses, samples;
    const double* pos;
    const double* weight;
    const double* phase;
    double range_start, data_dr, k;
};

// ---- argument checks and descriptors shared by the entry points (capi.cu) ------
// Each returns SARBP_OK or a status with the message recorded for sarbp_last_error.
int check_pulses(const float* data, int pulses, int samples, const double* pos, const double* weight,
                 const double* phase, double data_dr, double k);
int check_mode(int mode);
int check_grid(const sarbp_polar_grid* g);
PolarDesc desc_of(const sarbp_polar_grid& g);
PulseInputs inputs_of(const float* data, int pulses, int samples, const double* pos, const double* weight,
                      const double* phase, double range_start, double data_dr, double k);
// Split-precision direct BP onto a polar grid over all pulses: the tile shape, window and chunk
// choice of sarbp_direct_polar(mode = SARBP_SPLIT).  With pulse_split > 1 the partial images go to
// `parts` ([pulse_split, nr, nu]) and are summed in fixed order into `out`.
int split_direct_polar(const PulseInputs& in, const sarbp_polar_grid& grid, int chunk_pulses, int pulse_split,
                       float2* parts, float2* out, cudaStream_t s);

// Plain (reference-arithmetic) kernels.
int launch_plain_polar(int mode, const PulseInputs& in, const PolarDesc& g, int pulse_begin, int pulse_end,
                       int chunk, float2* out, long long out_stride, cudaStream_t s);
int launch_plain_points(int mode, const PulseInputs& in, const double* xyz, int npts, int chunk, float2* out,
                        cudaStream_t s);
int launch_plain_lattice(int mode, const PulseInputs& in, const sarbp_lattice& lat, int chunk, float2* out,
                         cudaStream_t s);
int launch_plain_regrid(int mode, const float2* img, const PolarDesc& src, const PolarDesc& dst, double k,
                        float2* out, cudaStream_t s);
int launch_plain_merge(int mode, const float2* left, const PolarDesc& lg, const float2* right,
                       const PolarDesc& rg, const PolarDesc& dst, double k, float2* out, cudaStream_t s);
int launch_plain_ffbp_leaves(int mode, const PulseInputs& in, const PolarDesc* nodes, const int2* blocks,
                             int nblocks, float2* arena, cudaStream_t s);
int launch_plain_ffbp_merges(int mode, double k, const PolarDesc* nodes, const int2* blocks, int nblocks,
                             float2* arena, float2* root_out, int root, cudaStream_t s);
int launch_evaluate(const float2* img, const PolarDesc& g, const double* xyz, int npts, double k, float2* out,
                    cudaStream_t s);
int launch_target_contrib(const PulseInputs& in, const double* xyz, int npts, float2* out, cudaStream_t s);
int launch_fill_lut(int samples, double range_start, double data_dr, double k, float2* lut, cudaStream_t s);
int launch_plain_polar_lut(const PulseInputs& in, const PolarDesc& g, const float2* lut, float2* out,
                           cudaStream_t s);
int launch_plain_polar_phase32(const PulseInputs& in, const PolarDesc& g, bool wrapped, float2* out,
                               cudaStream_t s);
int launch_add(float2* left, const float2* right, int64_t n, cudaStream_t s);
int launch_cast(const double2* in, float2* out, int64_t n, cudaStream_t s);
int launch_crop(const float2* in, int src_nu, int r_begin, int u_begin, int nr, int nu, float2* out,
                cudaStream_t s);
int launch_sum_parts(const float2* parts, int nparts, long long part_stride, long long n, float2* out,
                     cudaStream_t s);

// Split-precision kernels.
constexpr int kSplitThreads = 256;
constexpr int kSplitTilePixels = 1024;  // 256 threads x 4 pixels
// Bins each pulse window needs for tiles of at most `radius` metres (pixel offset from the tile centre).
int split_window_bins(double radius, double data_dr);
// Radius (m) of a lattice tile of 1024 >> lc rows by 1 << lc columns about its centre pixel.
double lattice_radius(const sarbp_lattice& lat, int lc);
// Pulses per shared-memory chunk that fit `window_bins` within the shared-memory budget.
int split_chunk_for(int window_bins, int requested, bool leaf = false);
int split_lattice_auto_split(const sarbp_lattice& lat, int pulses);
// Bounded waits in the kernels that ran out since the library was loaded (synchronises).
int split_wait_timeouts(int* count);
// Tile column exponent (2..5) that makes a polar tile of grid g closest to square in metres,
// and the largest pixel offset from the tile centre (metres) over the grid for that shape.
int split_polar_tile_lc(const PolarDesc& g, double* radius);
// The widest tile shape whose radius is within `slack` (>= 1) of the smallest (FFBP merge tiles).
int split_polar_tile_lc_slack(const PolarDesc& g, double slack, double* radius);
int launch_split_polar(const PulseInputs& in, const PolarDesc& g, int pulse_split, int chunk, int window_bins,
                       float2* out, long long out_stride, long long split_stride, cudaStream_t s);
int launch_split_lattice(const PulseInputs& in, const sarbp_lattice& lat, int pulse_split, int chunk,
                         int window_bins, float2* out, long long split_stride, cudaStream_t s);
int launch_split_points(const PulseInputs& in, const double* xyz, int npts, int pulse_split, int chunk,
                        int window_bins, float2* out, long long split_stride, cudaStream_t s);
// Adjoint of split-precision lattice BP: per-pulse gradients of a real image loss
// (grad = dl/dRe I + i dl/dIm I) with respect to position, phase and weight.
size_t split_adjoint_workspace(const sarbp_lattice& lat, int pulses);
int launch_split_lattice_adjoint(const PulseInputs& in, const sarbp_lattice& lat, int chunk, int window_bins,
                                 const float2* grad, float* partials, double* grad_pos, double* grad_phase,
                                 double* grad_weight, cudaStream_t s);

// Batched scenes (persistent work-queue kernels).  One descriptor per scene.
struct BatchSceneDesc {
    PulseInputs in;
    int kind;               // 0 direct lattice, 1 FFBP
    sarbp_lattice lat;      // direct scenes
    int lc;                 // direct: log2 of tile columns (2..5)
    int chunk;              // pulses per staged chunk
    int window_bins;        // range bins per pulse window
    float2* out;            // direct output image
    long long prec_offset;  // FFBP: first pulse record of the scene
};
size_t split_batch_scene_bytes();
// Writes the device form of `d` to dst; returns the dynamic shared memory its tiles need.
size_t split_batch_pack_scene(const BatchSceneDesc& d, void* dst);
int split_batch_occupancy(size_t direct_smem, size_t leaf_smem, int* direct_per_sm, int* leaf_per_sm,
                          int* merge_per_sm);
int launch_split_batch_prologue(const void* scenes, const PolarDesc* nodes, int n_nodes, int max_dim,
                                const int* leaves, int n_leaves, const TileItem* merge_items, int n_merge_items,
                                float4* tables, void* precs, void* crecs, float2* arena, cudaStream_t s);
int launch_split_batch_trace_start(unsigned long long* t0, cudaStream_t s);
int launch_split_batch_direct(const void* scenes, const TileItem* items, int nitems, int* counter, int blocks,
                              size_t smem, unsigned long long* trace, cudaStream_t s);
int launch_split_batch_leaves(const void* scenes, const PolarDesc* nodes, const TileItem* items, int nitems,
                              const float4* tables, const void* precs, float2* arena, int* counter, int blocks,
                              size_t smem, unsigned long long* trace, cudaStream_t s);
int launch_split_batch_merges(const void* scenes, const PolarDesc* nodes, const TileItem* items, int nitems,
                              const float4* tables, const void* crecs, float2* arena, int* counter, int blocks,
                              unsigned long long* trace, cudaStream_t s);

// Polar image -> flat ground lattice, split precision (evaluate_image on lattice points).
int launch_split_evaluate_lattice(const float2* image, const PolarDesc& grid, const sarbp_lattice& lattice, double k,
                                  float2* out, cudaStream_t s);

// Range compression around the FFTs (mean removal + padding, filter + Fourier interpolation, crop).
int launch_rc_prepare(const float2* raw, int pulses, int samples, int nfft, float2* out, cudaStream_t s);
int launch_rc_filter(const float2* spec, const float2* response, int pulses, int nfft, int length, float2* out,
                     cudaStream_t s);
int launch_rc_crop(const float2* corr, int pulses, int length, int offset, int samples, float scale, float2* out,
                   cudaStream_t s);
int launch_decode_iq(const unsigned char* frames, int n, long long frame_size, int iq_offset, int nr, float2* out,
                     cudaStream_t s);

// Zero-phase IIR smoothing along rows (autofocus phase-history filter).
size_t sosfiltfilt_workspace(int rows, int n, int padlen);
int launch_tile_argmax(const float* a, int nr, int nu, int nr_tiles, int nu_tiles, float* tmax, long long* first,
                       cudaStream_t s);
int launch_sosfiltfilt(const float* x, int rows, int n, const double* sos, const double* zi, int sections, int padlen,
                       double* y, double* ws, cudaStream_t s);

// FFBP split path: per-node row/column geometry tables (3 float4 per row, 1 per
// column), per-pulse leaf records and per-(merge tile, child) records, computed
// by three prologue launches per execute.
int launch_split_ffbp_tables(const PulseInputs& in, const PolarDesc* nodes, int n_nodes, int max_dim,
                             float4* tables, cudaStream_t s);
int launch_split_ffbp_leaf_pulses(const PulseInputs& in, const PolarDesc* nodes, const int* leaves, int n_leaves,
                                  void* recs, cudaStream_t s);
// tmaps: per node a 128-byte TMA tensor map of its image (used for children with box_w > 0), or
// NULL (no staging: the merge tiles gather from global memory).
int launch_split_ffbp_child_records(double k, const PolarDesc* nodes, const float4* tables, const TileItem* items,
                                    int n_items, float2* arena, const void* tmaps, void* recs, cudaStream_t s);
size_t split_ffbp_pulse_record_bytes();
size_t split_ffbp_child_record_bytes();
int launch_split_ffbp_leaves(const PulseInputs& in, const PolarDesc* nodes, const TileItem* items, int nitems,
                             int chunk, int window_bins, const float4* tables, const void* precs, float2* arena,
                             float2* root_out, int root, cudaStream_t s);
// Device state of the dependency-counting merge queue (all merge levels in one launch).
struct MergeQueue {
    int* next;                    // next item to claim
    int* remaining;               // per node: tiles not yet written
    int* pending;                 // per node: merge children not yet complete
    const int* parent;            // per node: parent index, -1 for the root
    int* status;                  // 0; 1 once a wait ran out (the image is then incomplete)
    unsigned long long limit_ns;  // wait limit per item
};
int launch_split_ffbp_merge_queue(double k, const PolarDesc* nodes, const TileItem* items, int nitems,
                                  const float4* tables, const void* crecs, float2* arena, float2* root_out, int root,
                                  const MergeQueue& Q, cudaStream_t s);
// box_bytes > 0: the level's child records carry tensor maps, and each merge tile stages its two
// children's footprints (at most box_bytes of shared memory together) by TMA, each warp waiting
// for them at most wait_ns; the tiles of node `withheld` (tests; -1 for none) declare 16 bytes more
// than their copies deliver, so that their waits run out.
int launch_split_ffbp_merges(double k, const PolarDesc* nodes, const TileItem* items, int nitems,
                             const float4* tables, const void* crecs, float2* arena, float2* root_out, int root,
                             size_t box_bytes, unsigned long long wait_ns, int withheld, cudaStream_t s);
// Shared-memory bytes of one staged child footprint (rows x cols complex64, 128-byte granules).
__host__ __device__ inline size_t split_box_bytes(int rows, int cols) { return ((size_t)rows * cols * 8 + 127) / 128 * 128; }
// Largest staged footprint per child, 13 KB: the 32 x 32 and 16 x 64 tiles of near-range plans need
// at most about 9.5 KB, so their merge CTAs stay within 28 KB and eight fit an SM's 228 KB; the 8 x 128
// tiles of far-range plans need up to 12.8 KB, and their levels run staged at six CTAs per SM, 4% faster
// per image than gathering at eight (7168 pulses onto 2048² at 5.8 km).
constexpr size_t kMaxChildBox = 13312;
// Tensor-map bytes per node.
constexpr size_t kTensorMapBytes = 128;

}  // namespace sarbp
