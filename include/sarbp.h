/*
 * sarbp.h - C ABI of the GB300 (sm_103a) SAR back-projection library.
 *
 * Direct back-projection (BP) and polar fast factorized back-projection
 * (FFBP): range-compressed complex64 pulses, per-pulse antenna positions and
 * an image grid go in, a complex64 image comes out.  This is the boundary the
 * Python host (bp_project_gb300) binds with ctypes; any other host can bind it
 * the same way.  No torch or CUDA C++ types appear in the signatures.
 *
 * Conventions (shared with the reference fast_bp path):
 *   - All array arguments are DEVICE pointers owned by the caller.  Complex
 *     arrays are interleaved float pairs (complex64) unless stated otherwise.
 *   - data is C-contiguous complex64 [pulses, samples]; pos is float64
 *     [pulses, 3] (x cross-track, y along-track, z height); weight and phase
 *     are float64 [pulses].  range_start (m) is the range of sample 0, data_dr
 *     (m) the sample spacing, k the signed two-way wavenumber 4*pi*fc/c.
 *   - Range interpolation is the reference's four-point Lagrange sample1
 *     (fast_bp/ffbp.py:17-29): zero unless every tap lies inside the row.
 *   - Polar grids: pixel (ir, iu) sits at r = r0 + ir*dr (slant range from the
 *     grid origin), u = u0 + iu*du (sine of the horizontal angle);
 *     x = ox + side*g*sqrt(1-u^2), y = oy + g*u, z = 0 with g = sqrt(r^2-oz^2).
 *     Polar images are demodulated by exp(-j*k*r) (fast_bp/ffbp.py:58-76).
 *   - Every call only enqueues work on `stream` (a cudaStream_t, NULL = the
 *     legacy default stream); none synchronises, allocates device memory or
 *     copies between host and device, except sarbp_ffbp_bind which uploads
 *     the plan tables.  Calls are safe to capture in a CUDA graph, except
 *     sarbp_ffbp_bind.
 *   - Return value: SARBP_OK or an error code; sarbp_last_error() returns a
 *     thread-local message for the most recent failure in the calling thread.
 *
 * Precision modes:
 *   SARBP_FP64  FP64 geometry, interpolation, phase and accumulation
 *   SARBP_FP32  FP32 everything (the reference's fp32 policy)
 *   SARBP_MIXED FP64 geometry and phase, FP32 interpolation and accumulation
 *   SARBP_SPLIT FP32 arithmetic with wide precision only per (pixel tile, pulse)
 *               and per tile: tile-centre ranges in two-float FP32 (~44 bits)
 *               from the FP64 inputs, per-pixel range offsets as exact split
 *               products, phase reduced in turns before a hardware sin/cos.
 *               Relative error vs FP64 is ~1e-6 (stated per image by the
 *               tests); this is the fast path.
 * The first three follow the reference's MODES (fast_bp/gpu_backend.py:57,
 * gpu/kernels.cu:1-6).
 */
#ifndef SARBP_H
#define SARBP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SARBP_ABI_VERSION 1

enum sarbp_status {
    SARBP_OK = 0,
    SARBP_ERR_VALUE = 1,       /* invalid argument value or shape (ValueError)        */
    SARBP_ERR_TYPE = 2,        /* null pointer / misaligned array (TypeError)         */
    SARBP_ERR_WORKSPACE = 3,   /* workspace missing or too small (ValueError)        */
    SARBP_ERR_CUDA = 4,        /* CUDA runtime error (RuntimeError)                  */
    SARBP_ERR_PLAN = 5,        /* FFBP plan inconsistent or not bound (RuntimeError) */
    SARBP_ERR_ENVELOPE = 6     /* geometry outside the split-precision envelope      */
};

enum sarbp_mode { SARBP_FP64 = 0, SARBP_FP32 = 1, SARBP_MIXED = 2, SARBP_SPLIT = 3 };

/* Polar image grid (fast_bp/gpu_backend.py:60-78 NodePlan geometry). */
typedef struct sarbp_polar_grid {
    double origin[3];
    double r0, dr;
    double u0, du;
    int32_t nr, nu;
    int32_t side;     /* +1 / -1 look side */
    int32_t reserved;
} sarbp_polar_grid;

/* Affine pixel lattice: pixel (i, j) at origin + i*step_row + j*step_col,
 * image [rows, cols].  Equivalent to backproject_points on the lattice points. */
typedef struct sarbp_lattice {
    double origin[3];
    double step_row[3];
    double step_col[3];
    int32_t rows, cols;
} sarbp_lattice;

/* One FFBP tree node (fast_bp/gpu_backend.py:60-78).  Nodes are given in
 * pre-order; left/right index children, -1 for leaves which back-project
 * pulses [a, b). */
typedef struct sarbp_ffbp_node {
    double origin[3];
    double r0, dr, u0, du;
    int32_t nr, nu;
    int32_t a, b;
    int32_t left, right;
    int32_t side;
    int32_t reserved;
} sarbp_ffbp_node;

typedef struct sarbp_ffbp_plan sarbp_ffbp_plan;

/* ---- library information -------------------------------------------------- */
const char* sarbp_version(void);
int sarbp_abi_version(void);
const char* sarbp_status_string(int status);
const char* sarbp_last_error(void);
/* Kernels this library launched since load (all entry points), for launch accounting. */
uint64_t sarbp_launch_count(void);

/* ---- direct back-projection ----------------------------------------------- */

/* Workspace bytes sarbp_direct_polar needs for these arguments (0 if none).
 * pulse_split > 1 splits the aperture over that many CTAs per pixel tile and
 * sums the partial images in fixed order (scratch: pulse_split images). */
size_t sarbp_direct_polar_workspace(int mode, const sarbp_polar_grid* grid, int pulses, int pulse_split);

/* Direct BP of all pulses onto a polar grid; out is complex64 [nr, nu].
 * Replaces CudaBaseline.run_direct (fast_bp/gpu_backend.py:471-555) and its
 * direct_chunk_{fp64,fp32,mixed} + cast_double2_to_float2 launches
 * (gpu/kernels.cu:240-339, :439-444); also the arithmetic of
 * bp_polar_{fp64,fp32,mixed} (gpu/kernels.cu:139-238) and ffbp.bp_polar
 * (ffbp.py:58-76).  chunk_pulses is the shared-memory pulse chunk (the
 * reference's --chunk-pulses, gpu_baseline.py:413); results do not depend on it. */
int sarbp_direct_polar(const float* data, int pulses, int samples, const double* pos,
                       const double* weight, const double* phase, const sarbp_polar_grid* grid,
                       double range_start, double data_dr, double k, int mode, int chunk_pulses,
                       int pulse_split, float* out, void* workspace, size_t workspace_bytes,
                       void* stream);

/* Allocation-free split-precision direct BP onto a polar grid: the same
 * result as sarbp_direct_polar(mode = SARBP_SPLIT, same pulse_split), with the
 * pulse-split partial images held in a fixed device array inside the library
 * instead of a caller workspace.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory where they image (hosts
 * that own all device memory through their own pool, real-time loops where
 * cudaMalloc would synchronise, cgo/JNI hosts that only see the buffers they
 * were handed).  Limit: pulse_split * nr * nu <= sarbp_static_scratch_elements()
 * (2^21 complex64, 16 MiB, held by every GPU that loads the library until
 * exit); larger requests fail with SARBP_ERR_VALUE.  Arguments are checked
 * exactly as sarbp_direct_polar checks them (alignment, finite geometry) before
 * anything reaches the GPU.  The first call on a device looks up the array's
 * device address and should come before any stream capture; the address is
 * kept for the life of the process, so a device that the process resets with
 * cudaDeviceReset must not be used with this entry point again.  All calls
 * share the array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  Nothing in the array
 * needs clearing: each call overwrites what it reads. */
size_t sarbp_static_scratch_elements(void);
int sarbp_direct_polar_static(const float* data, int pulses, int samples, const double* pos,
                              const double* weight, const double* phase, const sarbp_polar_grid* grid,
                              double range_start, double data_dr, double k, int chunk_pulses, int pulse_split,
                              float* out, void* stream);

/* Direct BP at arbitrary points xyz float64 [npts, 3]; out complex64 [npts].
 * Replaces ffbp.backproject_points (fast_bp/ffbp.py:43-55): phase k*r + phase[n],
 * not demodulated.  SPLIT mode groups consecutive points into tiles of 1024;
 * callers get the best speed with spatially coherent point order. */
size_t sarbp_backproject_points_workspace(int mode, int npts, int pulse_split);
int sarbp_backproject_points(const float* data, int pulses, int samples, const double* pos,
                             const double* weight, const double* phase, const double* xyz, int npts,
                             double range_start, double data_dr, double k, int mode, int pulse_split,
                             float* out, void* workspace, size_t workspace_bytes, void* stream);

/* Direct BP on an affine lattice (backproject_points semantics); out [rows, cols].
 * pulse_split as for sarbp_direct_polar; 0 (split mode) picks the split that fills the
 * GPU's CTA slots best for this lattice (the workspace query with 0 sizes for it). */
size_t sarbp_backproject_lattice_workspace(int mode, const sarbp_lattice* lattice, int pulse_split);
int sarbp_backproject_lattice(const float* data, int pulses, int samples, const double* pos,
                              const double* weight, const double* phase, const sarbp_lattice* lattice,
                              double range_start, double data_dr, double k, int mode, int pulse_split,
                              float* out, void* workspace, size_t workspace_bytes, void* stream);

/* ---- adjoint (differentiable BP) ------------------------------------------- */

/* Gradients of a real loss l(I) of the split-precision lattice image with
 * respect to the per-pulse inputs.  grad_image is complex64 [rows, cols] holding
 * dl/dRe I + i dl/dIm I (torch's gradient of a real loss of a complex tensor).
 * Outputs (any may be NULL, not all): grad_pos float64 [pulses, 3],
 * grad_phase float64 [pulses], grad_weight float64 [pulses].  The kernel
 * recomputes every pixel-pulse contribution (nothing is stored by the forward
 * pass) and sums per-tile partials in fixed order.  No counterpart in the
 * reference (its autofocus, fast_bp/autofocus.py:37-79, estimates phase
 * gradients from target contributions instead); it drives gradient-based
 * entropy autofocus. */
size_t sarbp_backproject_lattice_adjoint_workspace(const sarbp_lattice* lattice, int pulses);
int sarbp_backproject_lattice_adjoint(const float* data, int pulses, int samples, const double* pos,
                                      const double* weight, const double* phase, const sarbp_lattice* lattice,
                                      double range_start, double data_dr, double k, const float* grad_image,
                                      double* grad_pos, double* grad_phase, double* grad_weight, void* workspace,
                                      size_t workspace_bytes, void* stream);

/* ---- scene batches (persistent work-queue kernels) ------------------------- */

/* Many independent scenes of uneven pulse and pixel counts formed together:
 * direct split-precision BP onto a flat lattice, or split-precision FFBP of a
 * plan (the nodes sarbp_ffbp_plan_create takes).  All scenes' direct tiles run
 * in one persistent launch that takes work from a queue, largest items first,
 * and all FFBP leaf tiles in another; FFBP merges run as one persistent launch
 * per tree height across all scenes.  Each scene's output equals the single-scene entry
 * point's (sarbp_backproject_lattice / sarbp_ffbp_execute, split mode) bit for
 * bit when the tile shape is the same.  Inputs and outputs are bound at
 * creation; execute never synchronises or allocates and is graph-capturable.
 * No counterpart in the reference, which forms one scene at a time
 * (BatchedResidentProgram, batched_resident_backend.py:23-157, batches the
 * levels of one FFBP tree). */
enum sarbp_batch_kind { SARBP_BATCH_DIRECT = 0, SARBP_BATCH_FFBP = 1 };

typedef struct sarbp_batch_scene {
    const float* data;            /* complex64 [pulses, samples] */
    int pulses, samples;
    const double* pos;            /* float64 [pulses, 3] */
    const double* weight;         /* float64 [pulses] */
    const double* phase;          /* float64 [pulses] */
    double range_start, data_dr, k;
    int kind;                     /* sarbp_batch_kind */
    sarbp_lattice lattice;        /* DIRECT: the image lattice (step z components must be 0) */
    const sarbp_ffbp_node* nodes; /* FFBP: plan nodes in pre-order (copied at creation) */
    int n_nodes;
    int crop_r0, crop_u0, crop_nr, crop_nu;
    int tile_lc;                  /* DIRECT: log2 of tile columns, 2..5 (tile rows = 1024 >> tile_lc); 0 = 5 */
    int chunk_pulses;             /* pulses staged per chunk (DIRECT <= 64, FFBP leaves <= 32); 0 = default */
    float* out;                   /* DIRECT: complex64 [rows, cols]; FFBP: complex64 [crop_nr, crop_nu] */
} sarbp_batch_scene;

typedef struct sarbp_batch sarbp_batch;

/* blocks_per_sm: CTAs per SM of the persistent BP launch (0 = as many as fit). */
int sarbp_batch_create(const sarbp_batch_scene* scenes, int n_scenes, int blocks_per_sm, sarbp_batch** batch);
void sarbp_batch_destroy(sarbp_batch* batch);
size_t sarbp_batch_workspace_bytes(const sarbp_batch* batch);
int sarbp_batch_launch_count(const sarbp_batch* batch);
int sarbp_batch_info(const sarbp_batch* batch, int* bp_items, int* merge_items, int* max_height, int* bp_blocks,
                     double* pixel_pulses);
/* Uploads the scene, node and work tables into workspace (256-byte aligned); synchronises `stream`. */
int sarbp_batch_bind(sarbp_batch* batch, void* workspace, size_t workspace_bytes, void* stream);
int sarbp_batch_execute(const sarbp_batch* batch, void* stream);
/* Per-scene completion tracing for the following executes: trace is a device array of
 * n_scenes + 1 uint64; execute zeroes the first n_scenes, writes the GPU's nanosecond timer at its
 * start into trace[n_scenes] and, as each work item finishes, raises trace[scene] to the timer, so
 * trace[i] - trace[n_scenes] is scene i's latency within the batch.  NULL switches tracing off (a
 * captured graph keeps the setting it was captured with). */
int sarbp_batch_set_trace(sarbp_batch* batch, unsigned long long* trace);
/* on = 1: execute runs the FFBP scenes' chain (prologues, leaf queue, merge levels) on a stream of
 * the batch's own, forked from and joined back to the execute stream with events, so that it runs
 * beside the direct-scene queue and the GPU's CTA slots take work from both (a graph captured on
 * the execute stream records both branches).  on = 0 (the default): one stream, the direct queue
 * first.  The images do not depend on the setting. */
int sarbp_batch_set_concurrent(sarbp_batch* batch, int on);

/* ---- range compression (sar_io.range_compress, sar_io.py:116-139) --------- */

/* The matched filter that produces BP's input: y = crop(ifft(fft(pad(x - mean x))
 * * fft(h))) with h the conjugated, reversed, Hamming-weighted LFM reference.
 * The FFTs are library calls made by the host between these steps:
 *   sarbp_rc_prepare: out [pulses, nfft] = each pulse minus its mean, zero-padded;
 *   sarbp_rc_filter:  out [pulses, length] = spectrum * response (both [.., nfft]),
 *                     placed in a length = nfft * oversample spectrum for Fourier
 *                     interpolation with the even-length Nyquist bin split in half
 *                     (scipy.signal.resample); length == nfft multiplies in place
 *                     if out == spectrum;
 *   sarbp_rc_crop:    out [pulses, samples] = scale * corr[:, offset : offset + samples].
 * All arrays are complex64. */
int sarbp_rc_prepare(const float* raw, int pulses, int samples, int nfft, float* out, void* stream);
int sarbp_rc_filter(const float* spectrum, const float* response, int pulses, int nfft, int length, float* out,
                    void* stream);
int sarbp_rc_crop(const float* corr, int pulses, int length, int offset, int samples, float scale, float* out,
                  void* stream);

/* Raw capture frames -> complex64 pulses (sar_io.Capture.read, sar_io.py:79-81):
 * out [n, nr] = I + jQ from the little-endian int16 pairs that start iq_offset bytes
 * into each of n consecutive frames of frame_size bytes (device memory).  frames,
 * frame_size and iq_offset must be 4-byte aligned (the capture format's are). */
int sarbp_decode_iq(const void* frames, int n, long long frame_size, int iq_offset, int nr, float* out,
                    void* stream);

/* ---- autofocus helpers ---------------------------------------------------- */

/* Zero-phase IIR filtering of each row of x (complex64 [rows, n]) with a
 * cascade of `sections` second-order sections sos (float64 [sections, 6],
 * b0 b1 b2 a0 a1 a2 with a0 = 1) and steady-state initial conditions zi
 * (float64 [sections, 2]): odd extension by padlen samples, forward pass,
 * backward pass, extension removed; y is complex128 [rows, n].  Replaces
 * scipy.signal.sosfiltfilt(sos, xi, axis=1) in the phase-gradient autofocus
 * (fast_bp/autofocus.py:38-39).  sos_host (optional) is a host copy of sos
 * used only to check a0 == 1.  Requires n > padlen. */
size_t sarbp_sosfiltfilt_workspace(int rows, int n, int padlen);
int sarbp_sosfiltfilt(const float* x, int rows, int n, const double* sos, const double* zi, int sections,
                      const double* sos_host, int padlen, double* y, void* workspace, size_t workspace_bytes,
                      void* stream);

/* Brightest cell of every tile of a magnitude image (float32 [nr, nu]) split into
 * nr_tiles x nu_tiles tiles as numpy.array_split does: tile_max float32 and
 * tile_index int64 (row-major flat index; ties to the smallest) per tile,
 * tiles in row-major order.  The target picks of the autofocus
 * (fast_bp/autofocus.py:19-34, per-tile np.argmax). */
int sarbp_tile_argmax(const float* magnitude, int nr, int nu, int nr_tiles, int nu_tiles, float* tile_max,
                      long long* tile_index, void* stream);

/* ---- FFBP building blocks (eager schedule) -------------------------------- */

/* Child polar image -> parent polar grid with 4x4 Lagrange and exp(j k (rr-r)).
 * Replaces regrid_{fp64,fp32,mixed} (gpu/kernels.cu:341-429) / ffbp.regrid
 * (ffbp.py:79-95).  out complex64 [dst.nr, dst.nu]. */
int sarbp_regrid(const float* image, const sarbp_polar_grid* src, const sarbp_polar_grid* dst,
                 double k, int mode, float* out, void* stream);

/* Both child regrids rounded to complex64, then added: merge_regrid_*
 * (gpu/resident_kernels.cu:35-157). */
int sarbp_merge_regrid(const float* left, const sarbp_polar_grid* left_grid, const float* right,
                       const sarbp_polar_grid* right_grid, const sarbp_polar_grid* dst, double k,
                       int mode, float* out, void* stream);

/* left += right over n complex64 values: add_float2_inplace (gpu/kernels.cu:431-437). */
int sarbp_add_inplace(float* left, const float* right, int64_t n, void* stream);
/* complex128 -> complex64: cast_double2_to_float2 (gpu/kernels.cu:439-444). */
int sarbp_cast_c128_to_c64(const double* in, float* out, int64_t n, void* stream);
/* Root guard crop: crop_float2 (gpu/kernels.cu:446-454). out [nr, nu] = in[r_begin:, u_begin:]. */
int sarbp_crop(const float* in, int src_nu, int r_begin, int u_begin, int nr, int nu, float* out,
               void* stream);

/* ---- FFBP programs (level-batched, preallocated) -------------------------- */

/* Replaces ResidentProgram(algorithm='ffbp') / BatchedResidentProgram
 * (fast_bp/resident_backend.py:24-319, batched_resident_backend.py:23-157):
 * one launch for all leaves, one per tree height, the root crop fused into the
 * last merge.  create/destroy are host-only; bind uploads the tables into the
 * caller's workspace (synchronous w.r.t. stream); execute only launches.  A
 * leaf whose pulse range is [-1, -1) is an external node: the plan does no work
 * for it and merges the image the caller supplies with sarbp_ffbp_set_node_image. */
int sarbp_ffbp_plan_create(const sarbp_ffbp_node* nodes, int n_nodes, int crop_r0, int crop_u0,
                           int crop_nr, int crop_nu, int mode, sarbp_ffbp_plan** plan);
void sarbp_ffbp_plan_destroy(sarbp_ffbp_plan* plan);
size_t sarbp_ffbp_workspace_bytes(const sarbp_ffbp_plan* plan);
int sarbp_ffbp_launch_count(const sarbp_ffbp_plan* plan);
int sarbp_ffbp_bind(sarbp_ffbp_plan* plan, void* workspace, size_t workspace_bytes, void* stream);
/* Supplies the image (complex64 [nr, nu], device, row-major) of an external node: a leaf of the
 * plan whose pulse range is [-1, -1), formed elsewhere, e.g. a subtree root imaged on another GPU
 * (bp_project_gb300.shard).  The plan must be bound; the copy is enqueued on `stream` and the plan
 * never writes the node.  No counterpart in the reference (its trees are formed in one process). */
int sarbp_ffbp_set_node_image(const sarbp_ffbp_plan* plan, int node, const float* image, void* stream);
/* on = 1: a split plan runs all merge levels as one persistent launch, a dependency-counting queue
 * in which a parent's tiles start once both its children are complete (no barrier between tree
 * heights; child images read with coherent loads after an acquire).  on = 0 (the default): one
 * launch per tree height, which measured faster.  The images are the same bit for bit.  No
 * counterpart in the reference (its levels are separate launches). */
int sarbp_ffbp_set_merge_queue(sarbp_ffbp_plan* plan, int on);
/* on = 1 (the default): the merge tiles of a split plan stage each child's footprint (the child
 * stencil rows and columns the tile reads) in shared memory with one TMA tensor copy per child,
 * through a tensor map per child image that sarbp_ffbp_bind encodes; on = 0: the tiles gather
 * from the child images in global memory.  Set before sarbp_ffbp_bind.  The images are the same
 * bit for bit.  Replaces the global-memory stencil gathers of the reference's merges
 * (fast_bp/gpu/kernels.cu:70-137 sample2, gpu/resident_kernels.cu:35-55). */
int sarbp_ffbp_set_staging(sarbp_ffbp_plan* plan, int on);
/* *staged = 1 if the bound plan's merges stage their footprints (staging requested and the
 * driver's tensor-map encoder available at bind), else 0.  No counterpart in the reference. */
int sarbp_ffbp_staging(const sarbp_ffbp_plan* plan, int* staged);
/* The merges' wait limit per tile (default 5 s; (0, 60]) and, for tests of that limit, a merge node
 * whose waits run out (withheld_node >= 0; -1 for none).  Set before sarbp_ffbp_bind.  With the merge
 * queue, the withheld node's children are never counted complete; a wait that runs out stops the
 * launch and sets the status read by sarbp_ffbp_status, and the image is then incomplete.  With
 * staged merges (sarbp_ffbp_set_staging), the withheld node's tiles declare more bytes than their
 * TMA copies deliver; a warp whose wait runs out gathers from the child images instead, so the
 * image stays the same, and sarbp_wait_timeouts counts the wait. */
int sarbp_ffbp_set_wait_limit(sarbp_ffbp_plan* plan, double seconds, int withheld_node);
/* *status = 1 if a merge-queue wait ran out in the last execute, else 0 (synchronises the device). */
int sarbp_ffbp_status(const sarbp_ffbp_plan* plan, int* status);
int sarbp_ffbp_execute(const sarbp_ffbp_plan* plan, const float* data, int pulses, int samples,
                       const double* pos, const double* weight, const double* phase, double range_start,
                       double data_dr, double k, float* out, void* stream);

/* ---- polar -> Cartesian and autofocus helpers ------------------------------- */

/* ffbp.evaluate_image (ffbp.py:189-198): sample2 of a polar image at ground
 * points xyz [npts, 3] (z ignored) times exp(j k r).  FP64 geometry and phase. */
int sarbp_evaluate_image(const float* image, const sarbp_polar_grid* grid, const double* xyz, int npts,
                         double k, float* out, void* stream);

/* evaluate_image on the points of a ground lattice (z components ignored), out
 * complex64 [rows, cols], in split precision: two-float once per 32 x 32 pixel tile,
 * FP32 per pixel (offsets as exact split products, phase reduced in turns).
 * Same result as sarbp_evaluate_image on lattice points within ~1e-6 relative;
 * run.py's ground image (run.py:120-125) is this call on its lattice. */
int sarbp_evaluate_lattice(const float* image, const sarbp_polar_grid* grid, const sarbp_lattice* lattice, double k,
                           float* out, void* stream);

/* ffbp.target_contributions (ffbp.py:201-211): out[p, n] = sample1 * exp(j k r),
 * complex64 [npts, pulses]; FP64 geometry and phase. */
int sarbp_target_contributions(const float* data, int pulses, int samples, const double* pos,
                               const double* xyz, int npts, double range_start, double data_dr, double k,
                               float* out, void* stream);

/* ---- phase look-up-table probe (gpu/precision_probe.cu:106-164) ------------ */
int sarbp_fill_range_phase_lut(int samples, double range_start, double data_dr, double k, float* lut,
                               void* stream);
int sarbp_direct_polar_lut(const float* data, int pulses, int samples, const double* pos,
                           const double* weight, const double* phase, const sarbp_polar_grid* grid,
                           double range_start, double data_dr, double k, const float* lut, float* out,
                           void* stream);

/* ---- FP32-sincos phase probes (gpu/precision_probe.cu:19-79) ----------------
 * Replaces direct_chunk_mixed_phase32 (wrapped = 0) and
 * direct_chunk_mixed_phase32_wrapped (wrapped = 1): the mixed policy's FP64
 * geometry, sampling coordinate and phase k (d - r) + phase[n], with the phase
 * cast to FP32 for the library sincosf; wrapped = 1 first reduces it with FP64
 * remainder(phase, 2 pi).  All pulses in one launch; out complex64 [nr, nu]. */
int sarbp_direct_polar_phase32(const float* data, int pulses, int samples, const double* pos,
                               const double* weight, const double* phase, const sarbp_polar_grid* grid,
                               double range_start, double data_dr, double k, int wrapped, float* out,
                               void* stream);

/* ---- measurement ----------------------------------------------------------- */

/* FP32 issue-rate microbenchmark on the current device (no counterpart in the reference): eight
 * independent FMA chains per thread at full occupancy, scalar FFMA (packed = 0) or packed f32x2
 * FFMA2 (packed = 1), `iters` steps per chain; *tflops = flops (FMA = 2) per second over the
 * CUDA-event time of one launch after an untimed one.  Synchronises the device.  It is the
 * measured FP32 denominator of the back-projection kernels' roofline. */
int sarbp_fp32_peak(int packed, int iters, double* tflops);

/* Number of bounded waits on asynchronous copies in the library's kernels that ran out since it
 * was loaded (no counterpart in the reference); synchronises the device.  The waiting kernels are
 * the staged FFBP merges (a warp whose TMA footprints did not arrive in time gathers from the
 * child images instead: the image is still right) and those of the bulk-copy window staging build
 * (SARBP_BULK_WINDOWS: a tile whose range windows did not arrive in time stops early, so its image
 * is invalid). */
int sarbp_wait_timeouts(int* count);

#ifdef __cplusplus
}
#endif

#endif /* SARBP_H */
