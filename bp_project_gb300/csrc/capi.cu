// extern "C" entry points of libsarbp: argument validation, dispatch to the
// plain / split kernels, and the level-batched FFBP plan object.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "plan.cuh"

namespace sarbp {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

int fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int check_launch(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "%s launch failed: %s", what, cudaGetErrorString(e));
    return SARBP_OK;
}

void note_launches(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

namespace {

constexpr size_t kAlign = 512;

size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

bool is_finite_value(double v) { return isfinite(v) != 0; }

}  // namespace

// Argument checks and descriptor builders shared by every entry point (declared in common.cuh).
int check_pulses(const float* data, int pulses, int samples, const double* pos, const double* weight,
                 const double* phase, double data_dr, double k) {
    if (!data || !pos || !weight || !phase) return fail(SARBP_ERR_TYPE, "data, pos, weight and phase must be device pointers");
    if (((uintptr_t)data & 7) || ((uintptr_t)pos & 7) || ((uintptr_t)weight & 7) || ((uintptr_t)phase & 7))
        return fail(SARBP_ERR_TYPE, "arrays must be 8-byte aligned");
    if (pulses < 1) return fail(SARBP_ERR_VALUE, "at least one pulse is required (got %d)", pulses);
    if (samples < 1) return fail(SARBP_ERR_VALUE, "range-compressed data must have at least one sample per pulse");
    if (!is_finite_value(data_dr) || data_dr == 0.0) return fail(SARBP_ERR_VALUE, "data_dr must be finite and non-zero");
    if (!is_finite_value(k)) return fail(SARBP_ERR_VALUE, "k must be finite");
    return SARBP_OK;
}

int check_mode(int mode) {
    if (mode < SARBP_FP64 || mode > SARBP_SPLIT) return fail(SARBP_ERR_VALUE, "mode must be one of fp64, fp32, mixed, split (got %d)", mode);
    return SARBP_OK;
}

int check_grid(const sarbp_polar_grid* g) {
    if (!g) return fail(SARBP_ERR_TYPE, "grid must not be NULL");
    if (g->nr <= 0 || g->nu <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    if (!is_finite_value(g->r0) || !is_finite_value(g->dr) || !is_finite_value(g->u0) || !is_finite_value(g->du) || !is_finite_value(g->origin[0]) ||
        !is_finite_value(g->origin[1]) || !is_finite_value(g->origin[2]))
        return fail(SARBP_ERR_VALUE, "grid geometry must be finite");
    if (g->side != 1 && g->side != -1) return fail(SARBP_ERR_VALUE, "side must be +1 or -1");
    return SARBP_OK;
}

PolarDesc desc_of(const sarbp_polar_grid& g) {
    PolarDesc d{};
    d.ox = g.origin[0];
    d.oy = g.origin[1];
    d.oz = g.origin[2];
    d.r0 = g.r0;
    d.dr = g.dr;
    d.u0 = g.u0;
    d.du = g.du;
    d.nr = g.nr;
    d.nu = g.nu;
    d.side = g.side;
    d.left = d.right = -1;
    d.win_r0 = 0;
    d.win_u0 = 0;
    d.win_nr = g.nr;
    d.win_nu = g.nu;
    d.out_offset = 0;
    d.out_stride = g.nu;
    d.tile_lc = 5;
    split_geometry(d);
    return d;
}

PulseInputs inputs_of(const float* data, int pulses, int samples, const double* pos, const double* weight,
                      const double* phase, double range_start, double data_dr, double k) {
    PulseInputs in;
    in.data = reinterpret_cast<const float2*>(data);
    in.pulses = pulses;
    in.samples = samples;
    in.pos = pos;
    in.weight = weight;
    in.phase = phase;
    in.range_start = range_start;
    in.data_dr = data_dr;
    in.k = k;
    return in;
}

int split_direct_polar(const PulseInputs& in, const sarbp_polar_grid& grid, int chunk_pulses, int pulse_split,
                       float2* parts, float2* out, cudaStream_t s) {
    PolarDesc g = desc_of(grid);
    g.a = 0;
    g.b = in.pulses;
    const long long npix = (long long)grid.nr * grid.nu;
    double radius = 0.0;
    g.tile_lc = split_polar_tile_lc(g, &radius);
    const int wb = split_window_bins(radius, in.data_dr);
    const int ch = split_chunk_for(wb, chunk_pulses);
    int st = launch_split_polar(in, g, pulse_split, ch, wb, pulse_split > 1 ? parts : out, g.nu, npix, s);
    if (st == SARBP_OK && pulse_split > 1) st = launch_sum_parts(parts, pulse_split, npix, npix, out, s);
    return st;
}


namespace {

// Window radius assumed for point tiles: pulses of wider tiles run through the two-float fallback.
constexpr double kPointRadius = 24.0;
// Split-mode merge tiles may be up to this factor wider (in radius) than the squarest shape:
// a warp's pixels then span fewer rows, and its stencil gathers fewer sectors.
constexpr double kMergeTileSlack = 1.5;

// Child-image coordinates (range bin, angle bin; fractional) of pixel (i, j) of the parent grid
// p, in FP64: the child polar grid's r and u = dy / g of the pixel's ground point (the
// quantities the merge kernel computes in FP32 per pixel).
void child_bins(const PolarDesc& p, const PolarDesc& c, int i, int j, double& qr, double& qu) {
    const double r = p.r0 + i * p.dr, u = p.u0 + j * p.du;
    const double g = sqrt(fmax(r * r - p.oz * p.oz, 0.0));
    const double x = p.ox + p.side * g * sqrt(fmax(1.0 - u * u, 0.0)), y = p.oy + g * u;
    const double vx = x - c.ox, vy = y - c.oy;
    const double gc = sqrt(vx * vx + vy * vy), rr = sqrt(gc * gc + c.oz * c.oz);
    qr = (rr - c.r0) / c.dr;
    qu = (vy / gc - c.u0) / c.du;
}

// Footprint boxes of split-mode merges (PolarDesc::box_*, PolarDesc of each child): the child
// stencil rows and columns that a parent tile reads, relative to the stencil bin of the tile's
// centre pixel, over the corners and edge midpoints of up to 4 x 4 tiles of each parent (evenly
// spaced, the first and last included), plus one bin of margin on every side.  The mapping is
// smooth and the footprints grow monotonically towards the grid's edges, so the sampled extremes
// bound the rest up to that margin; a warp whose stencils fall outside the staged box reads the
// child image instead.  (Plans are rebuilt per autofocus iteration: this stays well under a
// millisecond for them.)  A box over 256 rows or columns (the TMA's limit) or kMaxChildBox bytes
// is not staged.  Also sets merge_box_bytes per height.
void child_footprints(sarbp_ffbp_plan& p) {
    p.merge_box_bytes.assign(p.max_height + 1, 0);
    for (int n = 0; n < p.n_nodes; ++n) {
        const PolarDesc& d = p.nodes[n];
        if (d.left < 0) continue;
        const int cols_t = 1 << d.tile_lc, rows_t = kSplitTilePixels >> d.tile_lc;
        const int ntr = (d.win_nr + rows_t - 1) / rows_t, ntu = (d.win_nu + cols_t - 1) / cols_t;
        const int sr = std::min(ntr, 4), su = std::min(ntu, 4);
        size_t bytes = 0;
        for (int ch : {d.left, d.right}) {
            PolarDesc& c = p.nodes[ch];
            double lo_r = 0, hi_r = 0, lo_u = 0, hi_u = 0;
            bool finite = true;
            for (int a = 0; a < sr; ++a) {
                const int tr = sr > 1 ? (int)((long long)a * (ntr - 1) / (sr - 1)) : 0;
                const int r_first = d.win_r0 + tr * rows_t, r_last = std::min(r_first + rows_t - 1, d.nr - 1);
                const int i0 = std::min(r_first + (rows_t >> 1), d.nr - 1);
                for (int b = 0; b < su; ++b) {
                    const int tu = su > 1 ? (int)((long long)b * (ntu - 1) / (su - 1)) : 0;
                    const int u_first = d.win_u0 + tu * cols_t, u_last = std::min(u_first + cols_t - 1, d.nu - 1);
                    const int j0 = std::min(u_first + (cols_t >> 1), d.nu - 1);
                    double qr, qu;
                    child_bins(d, c, i0, j0, qr, qu);
                    const double ir = floor(qr), iu = floor(qu);
                    const int is[3] = {r_first, (r_first + r_last) / 2, r_last};
                    const int js[3] = {u_first, (u_first + u_last) / 2, u_last};
                    for (int i : is)
                        for (int j : js) {
                            child_bins(d, c, i, j, qr, qu);
                            if (!std::isfinite(qr) || !std::isfinite(qu) || !std::isfinite(ir) || !std::isfinite(iu)) {
                                finite = false;
                                continue;
                            }
                            const double fr = floor(qr), fu = floor(qu);
                            lo_r = fmax(lo_r, ir - (fr - 1.0));
                            hi_r = fmax(hi_r, fr + 2.0 - ir);
                            lo_u = fmax(lo_u, iu - (fu - 1.0));
                            hi_u = fmax(hi_u, fu + 2.0 - iu);
                        }
                }
            }
            c.box_w = 0;
            if (!finite || lo_r + hi_r > 250.0 || lo_u + hi_u > 250.0) continue;
            const int br = (int)lo_r + 1, bu = (int)lo_u + 1;
            // At least 8 x 8 (the kernel's block test needs 5 x 4); one more column because the
            // first one is rounded down to an even column.
            const int bh = std::max(br + (int)hi_r + 1 + 1, 8);
            int bw = std::max(bu + (int)hi_u + 1 + 2, 8);
            bw += bw & 1;
            if (bh > 256 || bw > 256 || split_box_bytes(bh, bw) > kMaxChildBox) continue;
            c.box_r = br;
            c.box_u = bu;
            c.box_h = bh;
            c.box_w = bw;
            bytes += split_box_bytes(bh, bw);
        }
        const int h = p.height[n];
        p.merge_box_bytes[h] = std::max(p.merge_box_bytes[h], bytes);
    }
}

// The driver's tensor-map encoder, through the runtime's entry-point query (no link against
// the driver library); NULL where the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// One 2-D tensor map per child image with a footprint box (8-byte elements, nu x nr, row pitch
// out_stride elements, box box_w x box_h, zero fill outside the image); the others stay zero.
bool encode_child_maps(const sarbp_ffbp_plan& p, float2* arena, std::vector<CUtensorMap>& maps) {
    static_assert(sizeof(CUtensorMap) == kTensorMapBytes, "tensor map size");
    const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return false;
    maps.assign(p.n_nodes, CUtensorMap{});
    for (int n = 0; n < p.n_nodes; ++n) {
        const PolarDesc& c = p.nodes[n];
        if (n == 0 || c.box_w <= 0) continue;
        const cuuint64_t dims[2] = {(cuuint64_t)c.nu, (cuuint64_t)c.nr};
        const cuuint64_t pitch[1] = {(cuuint64_t)c.out_stride * sizeof(float2)};
        const cuuint32_t box[2] = {(cuuint32_t)c.box_w, (cuuint32_t)c.box_h};
        const cuuint32_t unit[2] = {1, 1};
        if (encode(&maps[n], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, arena + c.out_offset, dims, pitch, box, unit,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

}  // namespace

double lattice_radius(const sarbp_lattice& lat, int lc) {
    const double hr = (double)((kSplitTilePixels >> lc) >> 1), hc = (double)((1 << lc) >> 1);
    double s = 0.0;
    for (int c = 0; c < 3; ++c) {
        const double b = hr * fabs(lat.step_row[c]) + hc * fabs(lat.step_col[c]);
        s += b * b;
    }
    return sqrt(s) * 1.0001 + 1e-6;
}

}  // namespace sarbp

using namespace sarbp;

// ---- FFBP plan object -------------------------------------------------------------------

extern "C" {

const char* sarbp_version(void) { return "libsarbp 0.1.0 (sm_103a)"; }
int sarbp_abi_version(void) { return SARBP_ABI_VERSION; }

const char* sarbp_status_string(int status) {
    switch (status) {
        case SARBP_OK: return "ok";
        case SARBP_ERR_VALUE: return "invalid value";
        case SARBP_ERR_TYPE: return "invalid pointer or type";
        case SARBP_ERR_WORKSPACE: return "workspace missing or too small";
        case SARBP_ERR_CUDA: return "CUDA error";
        case SARBP_ERR_PLAN: return "FFBP plan error";
        case SARBP_ERR_ENVELOPE: return "outside the split-precision envelope";
        default: return "unknown status";
    }
}

const char* sarbp_last_error(void) { return g_last_error.c_str(); }

int sarbp_wait_timeouts(int* count) {
    if (!count) return fail(SARBP_ERR_TYPE, "count must not be NULL");
    return split_wait_timeouts(count);
}
uint64_t sarbp_launch_count(void) { return g_launches.load(); }

// ---- direct BP ---------------------------------------------------------------------------
size_t sarbp_direct_polar_workspace(int mode, const sarbp_polar_grid* grid, int pulses, int pulse_split) {
    (void)mode;
    (void)pulses;
    if (!grid || pulse_split <= 1) return 0;
    return (size_t)pulse_split * (size_t)grid->nr * (size_t)grid->nu * sizeof(float2);
}

int sarbp_direct_polar(const float* data, int pulses, int samples, const double* pos, const double* weight,
                       const double* phase, const sarbp_polar_grid* grid, double range_start, double data_dr,
                       double k, int mode, int chunk_pulses, int pulse_split, float* out, void* workspace,
                       size_t workspace_bytes, void* stream) {
    if (int st = check_mode(mode)) return st;
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (int st = check_grid(grid)) return st;
    if (!out) return fail(SARBP_ERR_TYPE, "out must not be NULL");
    if (chunk_pulses <= 0) return fail(SARBP_ERR_VALUE, "chunk_pulses must be positive");
    if (pulse_split < 1 || pulse_split > pulses) return fail(SARBP_ERR_VALUE, "pulse_split must be in [1, pulses]");
    const size_t need = sarbp_direct_polar_workspace(mode, grid, pulses, pulse_split);
    if (need && (!workspace || workspace_bytes < need))
        return fail(SARBP_ERR_WORKSPACE, "direct_polar needs %zu workspace bytes", need);
    cudaStream_t s = (cudaStream_t)stream;
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    float2* dst = reinterpret_cast<float2*>(out);
    float2* parts = pulse_split > 1 ? reinterpret_cast<float2*>(workspace) : dst;
    if (mode == SARBP_SPLIT) return split_direct_polar(in, *grid, chunk_pulses, pulse_split, parts, dst, s);
    PolarDesc g = desc_of(*grid);
    g.a = 0;
    g.b = pulses;
    const long long npix = (long long)grid->nr * grid->nu;
    int st = SARBP_OK;
    for (int part = 0; part < pulse_split && st == SARBP_OK; ++part) {
        const int p0 = (int)((long long)pulses * part / pulse_split);
        const int p1 = (int)((long long)pulses * (part + 1) / pulse_split);
        st = launch_plain_polar(mode, in, g, p0, p1, chunk_pulses, parts + part * npix, g.nu, s);
    }
    if (st == SARBP_OK && pulse_split > 1) st = launch_sum_parts(parts, pulse_split, npix, npix, dst, s);
    return st;
}

size_t sarbp_backproject_points_workspace(int mode, int npts, int pulse_split) {
    (void)mode;
    if (pulse_split <= 1 || npts <= 0) return 0;
    return (size_t)pulse_split * (size_t)npts * sizeof(float2);
}

int sarbp_backproject_points(const float* data, int pulses, int samples, const double* pos, const double* weight,
                             const double* phase, const double* xyz, int npts, double range_start, double data_dr,
                             double k, int mode, int pulse_split, float* out, void* workspace,
                             size_t workspace_bytes, void* stream) {
    if (int st = check_mode(mode)) return st;
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (!xyz || !out) return fail(SARBP_ERR_TYPE, "xyz and out must not be NULL");
    if (npts <= 0) return fail(SARBP_ERR_VALUE, "at least one point is required");
    if (pulse_split < 1 || pulse_split > pulses) return fail(SARBP_ERR_VALUE, "pulse_split must be in [1, pulses]");
    if (mode != SARBP_SPLIT && pulse_split != 1) return fail(SARBP_ERR_VALUE, "pulse_split applies to split mode only");
    const size_t need = sarbp_backproject_points_workspace(mode, npts, pulse_split);
    if (need && (!workspace || workspace_bytes < need))
        return fail(SARBP_ERR_WORKSPACE, "backproject_points needs %zu workspace bytes", need);
    cudaStream_t s = (cudaStream_t)stream;
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    float2* dst = reinterpret_cast<float2*>(out);
    if (mode != SARBP_SPLIT) return launch_plain_points(mode, in, xyz, npts, 0, dst, s);
    float2* parts = pulse_split > 1 ? reinterpret_cast<float2*>(workspace) : dst;
    const int wb = split_window_bins(kPointRadius, data_dr);
    const int ch = split_chunk_for(wb, 64);
    int st = launch_split_points(in, xyz, npts, pulse_split, ch, wb, parts, npts, s);
    if (st == SARBP_OK && pulse_split > 1) st = launch_sum_parts(parts, pulse_split, npts, npts, dst, s);
    return st;
}

size_t sarbp_backproject_lattice_workspace(int mode, const sarbp_lattice* lattice, int pulse_split) {
    if (!lattice || lattice->rows <= 0 || lattice->cols <= 0) return 0;
    if (pulse_split == 0) pulse_split = mode == SARBP_SPLIT ? split_lattice_auto_split(*lattice, 8) : 1;
    if (pulse_split <= 1) return 0;
    return (size_t)pulse_split * (size_t)lattice->rows * (size_t)lattice->cols * sizeof(float2);
}

int sarbp_backproject_lattice(const float* data, int pulses, int samples, const double* pos, const double* weight,
                              const double* phase, const sarbp_lattice* lattice, double range_start,
                              double data_dr, double k, int mode, int pulse_split, float* out, void* workspace,
                              size_t workspace_bytes, void* stream) {
    if (int st = check_mode(mode)) return st;
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (!lattice || !out) return fail(SARBP_ERR_TYPE, "lattice and out must not be NULL");
    if (lattice->rows <= 0 || lattice->cols <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    for (int c = 0; c < 3; ++c)
        if (!is_finite_value(lattice->origin[c]) || !is_finite_value(lattice->step_row[c]) || !is_finite_value(lattice->step_col[c]))
            return fail(SARBP_ERR_VALUE, "lattice geometry must be finite");
    if (pulse_split < 0 || pulse_split > pulses)
        return fail(SARBP_ERR_VALUE, "pulse_split must be 0 (automatic) or in [1, pulses]");
    if (mode != SARBP_SPLIT && pulse_split > 1) return fail(SARBP_ERR_VALUE, "pulse_split applies to split mode only");
    if (pulse_split == 0) pulse_split = mode == SARBP_SPLIT ? split_lattice_auto_split(*lattice, pulses) : 1;
    const size_t need = sarbp_backproject_lattice_workspace(mode, lattice, pulse_split);
    if (need && (!workspace || workspace_bytes < need))
        return fail(SARBP_ERR_WORKSPACE, "backproject_lattice needs %zu workspace bytes", need);
    cudaStream_t s = (cudaStream_t)stream;
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    float2* dst = reinterpret_cast<float2*>(out);
    if (mode != SARBP_SPLIT) return launch_plain_lattice(mode, in, *lattice, 0, dst, s);
    const long long npix = (long long)lattice->rows * lattice->cols;
    float2* parts = pulse_split > 1 ? reinterpret_cast<float2*>(workspace) : dst;
    const int wb = split_window_bins(lattice_radius(*lattice, 5), data_dr);
    const int ch = split_chunk_for(wb, 64);
    int st = launch_split_lattice(in, *lattice, pulse_split, ch, wb, parts, npix, s);
    if (st == SARBP_OK && pulse_split > 1) st = launch_sum_parts(parts, pulse_split, npix, npix, dst, s);
    return st;
}

size_t sarbp_backproject_lattice_adjoint_workspace(const sarbp_lattice* lattice, int pulses) {
    if (!lattice || lattice->rows <= 0 || lattice->cols <= 0 || pulses <= 0) return 0;
    return split_adjoint_workspace(*lattice, pulses);
}

int sarbp_backproject_lattice_adjoint(const float* data, int pulses, int samples, const double* pos,
                                      const double* weight, const double* phase, const sarbp_lattice* lattice,
                                      double range_start, double data_dr, double k, const float* grad_image,
                                      double* grad_pos, double* grad_phase, double* grad_weight, void* workspace,
                                      size_t workspace_bytes, void* stream) {
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (!lattice || !grad_image) return fail(SARBP_ERR_TYPE, "lattice and grad_image must not be NULL");
    if (!grad_pos && !grad_phase && !grad_weight) return fail(SARBP_ERR_VALUE, "no gradient requested");
    if (lattice->rows <= 0 || lattice->cols <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    for (int c = 0; c < 3; ++c)
        if (!is_finite_value(lattice->origin[c]) || !is_finite_value(lattice->step_row[c]) ||
            !is_finite_value(lattice->step_col[c]))
            return fail(SARBP_ERR_VALUE, "lattice geometry must be finite");
    const size_t need = sarbp_backproject_lattice_adjoint_workspace(lattice, pulses);
    if (!workspace || workspace_bytes < need)
        return fail(SARBP_ERR_WORKSPACE, "backproject_lattice_adjoint needs %zu workspace bytes", need);
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    const int wb = split_window_bins(lattice_radius(*lattice, 5), data_dr);
    const int ch = split_chunk_for(wb, 64);
    return launch_split_lattice_adjoint(in, *lattice, ch, wb, reinterpret_cast<const float2*>(grad_image),
                                        reinterpret_cast<float*>(workspace), grad_pos, grad_phase, grad_weight,
                                        (cudaStream_t)stream);
}

int sarbp_rc_prepare(const float* raw, int pulses, int samples, int nfft, float* out, void* stream) {
    if (!raw || !out) return fail(SARBP_ERR_TYPE, "raw and out must be device pointers");
    if (pulses < 1 || samples < 1) return fail(SARBP_ERR_VALUE, "raw data must have at least one pulse and sample");
    if (nfft < samples) return fail(SARBP_ERR_VALUE, "nfft (%d) must be >= samples (%d)", nfft, samples);
    return launch_rc_prepare(reinterpret_cast<const float2*>(raw), pulses, samples, nfft, reinterpret_cast<float2*>(out),
                             (cudaStream_t)stream);
}

int sarbp_rc_filter(const float* spectrum, const float* response, int pulses, int nfft, int length, float* out,
                    void* stream) {
    if (!spectrum || !response || !out) return fail(SARBP_ERR_TYPE, "spectrum, response and out must be device pointers");
    if (pulses < 1 || nfft < 1) return fail(SARBP_ERR_VALUE, "pulses and nfft must be positive");
    if (length < nfft) return fail(SARBP_ERR_VALUE, "length (%d) must be >= nfft (%d)", length, nfft);
    if (length > nfft && (void*)spectrum == (void*)out) return fail(SARBP_ERR_VALUE, "oversampling cannot run in place");
    return launch_rc_filter(reinterpret_cast<const float2*>(spectrum), reinterpret_cast<const float2*>(response),
                            pulses, nfft, length, reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_rc_crop(const float* corr, int pulses, int length, int offset, int samples, float scale, float* out,
                  void* stream) {
    if (!corr || !out) return fail(SARBP_ERR_TYPE, "corr and out must be device pointers");
    if (pulses < 1 || samples < 1 || offset < 0 || offset + samples > length)
        return fail(SARBP_ERR_VALUE, "crop window [%d, %d) outside the %d-sample correlation", offset, offset + samples,
                    length);
    return launch_rc_crop(reinterpret_cast<const float2*>(corr), pulses, length, offset, samples, scale,
                          reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_decode_iq(const void* frames, int n, long long frame_size, int iq_offset, int nr, float* out,
                    void* stream) {
    if (!frames || !out) return fail(SARBP_ERR_TYPE, "frames and out must be device pointers");
    if (n < 1 || nr < 1) return fail(SARBP_ERR_VALUE, "at least one frame and one sample are required");
    if (iq_offset < 0 || (long long)iq_offset + 4LL * nr > frame_size)
        return fail(SARBP_ERR_VALUE, "I/Q block [%d, %lld) outside the %lld-byte frame", iq_offset,
                    (long long)iq_offset + 4LL * nr, frame_size);
    if (((uintptr_t)frames & 3) || (frame_size & 3) || (iq_offset & 3))
        return fail(SARBP_ERR_TYPE, "frames, frame_size and iq_offset must be 4-byte aligned");
    return launch_decode_iq(reinterpret_cast<const unsigned char*>(frames), n, frame_size, iq_offset, nr,
                            reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

size_t sarbp_sosfiltfilt_workspace(int rows, int n, int padlen) {
    if (rows <= 0 || n <= 0 || padlen < 0) return 0;
    return sosfiltfilt_workspace(rows, n, padlen);
}

int sarbp_sosfiltfilt(const float* x, int rows, int n, const double* sos, const double* zi, int sections,
                      const double* sos_host, int padlen, double* y, void* workspace, size_t workspace_bytes,
                      void* stream) {
    if (!x || !sos || !zi || !y) return fail(SARBP_ERR_TYPE, "x, sos, zi and y must be device pointers");
    if (rows < 1 || n < 1) return fail(SARBP_ERR_VALUE, "x must have at least one row and one sample");
    if (sections < 1 || sections > 8) return fail(SARBP_ERR_VALUE, "1 to 8 second-order sections are supported (got %d)", sections);
    if (padlen < 0 || n <= padlen)
        return fail(SARBP_ERR_VALUE, "the length of the input vector x must be greater than padlen, which is %d", padlen);
    if (sos_host)
        for (int s = 0; s < sections; ++s)
            if (sos_host[6 * s + 3] != 1.0) return fail(SARBP_ERR_VALUE, "sos[:, 3] should be all ones");
    const size_t need = sarbp_sosfiltfilt_workspace(rows, n, padlen);
    if (!workspace || workspace_bytes < need) return fail(SARBP_ERR_WORKSPACE, "sosfiltfilt needs %zu workspace bytes", need);
    return launch_sosfiltfilt(x, rows, n, sos, zi, sections, padlen, y, reinterpret_cast<double*>(workspace),
                              (cudaStream_t)stream);
}

int sarbp_tile_argmax(const float* magnitude, int nr, int nu, int nr_tiles, int nu_tiles, float* tile_max,
                      long long* tile_index, void* stream) {
    if (!magnitude || !tile_max || !tile_index) return fail(SARBP_ERR_TYPE, "magnitude, tile_max and tile_index must be device pointers");
    if (nr_tiles < 1 || nu_tiles < 1) return fail(SARBP_ERR_VALUE, "at least one tile per axis is required");
    if (nr < nr_tiles || nu < nu_tiles) return fail(SARBP_ERR_VALUE, "the image has fewer rows or columns than tiles");
    if ((long long)nr_tiles * nu_tiles > INT32_MAX) return fail(SARBP_ERR_VALUE, "too many tiles");
    return launch_tile_argmax(magnitude, nr, nu, nr_tiles, nu_tiles, tile_max, tile_index, (cudaStream_t)stream);
}

// ---- FFBP building blocks ---------------------------------------------------------------
int sarbp_regrid(const float* image, const sarbp_polar_grid* src, const sarbp_polar_grid* dst, double k, int mode,
                 float* out, void* stream) {
    if (int st = check_mode(mode)) return st;
    if (!image || !out) return fail(SARBP_ERR_TYPE, "image and out must not be NULL");
    if (int st = check_grid(src)) return st;
    if (int st = check_grid(dst)) return st;
    if (!is_finite_value(k)) return fail(SARBP_ERR_VALUE, "k must be finite");
    const int m = mode == SARBP_SPLIT ? SARBP_MIXED : mode;
    return launch_plain_regrid(m, reinterpret_cast<const float2*>(image), desc_of(*src), desc_of(*dst), k,
                               reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_merge_regrid(const float* left, const sarbp_polar_grid* left_grid, const float* right,
                       const sarbp_polar_grid* right_grid, const sarbp_polar_grid* dst, double k, int mode, float* out,
                       void* stream) {
    if (int st = check_mode(mode)) return st;
    if (!left || !right || !out) return fail(SARBP_ERR_TYPE, "images and out must not be NULL");
    if (int st = check_grid(left_grid)) return st;
    if (int st = check_grid(right_grid)) return st;
    if (int st = check_grid(dst)) return st;
    if (!is_finite_value(k)) return fail(SARBP_ERR_VALUE, "k must be finite");
    const int m = mode == SARBP_SPLIT ? SARBP_MIXED : mode;
    return launch_plain_merge(m, reinterpret_cast<const float2*>(left), desc_of(*left_grid),
                              reinterpret_cast<const float2*>(right), desc_of(*right_grid), desc_of(*dst), k,
                              reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_add_inplace(float* left, const float* right, int64_t n, void* stream) {
    if (!left || !right) return fail(SARBP_ERR_TYPE, "left and right must not be NULL");
    if (n <= 0) return fail(SARBP_ERR_VALUE, "n must be positive");
    return launch_add(reinterpret_cast<float2*>(left), reinterpret_cast<const float2*>(right), n, (cudaStream_t)stream);
}

int sarbp_cast_c128_to_c64(const double* in, float* out, int64_t n, void* stream) {
    if (!in || !out) return fail(SARBP_ERR_TYPE, "in and out must not be NULL");
    if (n <= 0) return fail(SARBP_ERR_VALUE, "n must be positive");
    return launch_cast(reinterpret_cast<const double2*>(in), reinterpret_cast<float2*>(out), n, (cudaStream_t)stream);
}

int sarbp_crop(const float* in, int src_nu, int r_begin, int u_begin, int nr, int nu, float* out, void* stream) {
    if (!in || !out) return fail(SARBP_ERR_TYPE, "in and out must not be NULL");
    if (nr <= 0 || nu <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    if (r_begin < 0 || u_begin < 0 || u_begin + nu > src_nu)
        return fail(SARBP_ERR_VALUE, "crop window outside the source image");
    return launch_crop(reinterpret_cast<const float2*>(in), src_nu, r_begin, u_begin, nr, nu,
                       reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

// ---- FFBP plan -------------------------------------------------------------------------
int sarbp_ffbp_plan_create(const sarbp_ffbp_node* nodes, int n_nodes, int crop_r0, int crop_u0, int crop_nr,
                           int crop_nu, int mode, sarbp_ffbp_plan** plan_out) {
    if (!plan_out) return fail(SARBP_ERR_TYPE, "plan pointer must not be NULL");
    *plan_out = nullptr;
    if (int st = check_mode(mode)) return st;
    if (!nodes || n_nodes < 1) return fail(SARBP_ERR_VALUE, "an FFBP plan needs at least one node");
    const sarbp_ffbp_node& root = nodes[0];
    if (crop_nr <= 0 || crop_nu <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    if (crop_r0 < 0 || crop_u0 < 0 || crop_r0 + crop_nr > root.nr || crop_u0 + crop_nu > root.nu)
        return fail(SARBP_ERR_VALUE, "crop window outside the root grid");
    auto* p = new sarbp_ffbp_plan();
    p->mode = mode;
    p->n_nodes = n_nodes;
    p->nodes.resize(n_nodes);
    p->height.assign(n_nodes, -1);
    for (int i = 0; i < n_nodes; ++i) {
        const sarbp_ffbp_node& n = nodes[i];
        sarbp_polar_grid g{};
        for (int c = 0; c < 3; ++c) g.origin[c] = n.origin[c];
        g.r0 = n.r0;
        g.dr = n.dr;
        g.u0 = n.u0;
        g.du = n.du;
        g.nr = n.nr;
        g.nu = n.nu;
        g.side = n.side;
        if (int st = check_grid(&g)) {
            delete p;
            return fail(st, "node %d: %s", i, g_last_error.c_str());
        }
        const bool leaf = n.left < 0 && n.right < 0;
        if (!leaf && (n.left <= i || n.right <= i || n.left >= n_nodes || n.right >= n_nodes)) {
            delete p;
            return fail(SARBP_ERR_PLAN, "node %d: children must follow their parent in pre-order", i);
        }
        // A leaf with the pulse range [-1, -1) is external: its image comes from the caller
        // (sarbp_ffbp_set_node_image), e.g. a subtree formed on another GPU.
        const bool external = leaf && n.a == -1 && n.b == -1;
        if (external && i == 0) {
            delete p;
            return fail(SARBP_ERR_PLAN, "the root cannot be an external node");
        }
        if (leaf && !external && (n.a < 0 || n.b <= n.a)) {
            delete p;
            return fail(SARBP_ERR_PLAN, "leaf %d: invalid pulse range [%d, %d)", i, n.a, n.b);
        }
        p->n_external += external ? 1 : 0;
        PolarDesc d = desc_of(g);
        d.a = n.a;
        d.b = n.b;
        d.left = leaf ? -1 : n.left;
        d.right = leaf ? -1 : n.right;
        p->nodes[i] = d;
    }
    // Heights (children follow parents, so a reverse sweep sees children first).
    for (int i = n_nodes - 1; i >= 0; --i) {
        const PolarDesc& d = p->nodes[i];
        p->height[i] = d.left < 0 ? 0 : 1 + std::max(p->height[d.left], p->height[d.right]);
    }
    p->max_height = p->height[0];
    // Windows, arena offsets, tile shapes.
    size_t arena = 0;
    double leaf_radius = 0.0;
    int leaf_pulses = 1;
    for (int i = 0; i < n_nodes; ++i) {
        PolarDesc& d = p->nodes[i];
        if (i == 0) {
            d.win_r0 = crop_r0;
            d.win_u0 = crop_u0;
            d.win_nr = crop_nr;
            d.win_nu = crop_nu;
            d.out_offset = 0;
            d.out_stride = crop_nu;
        } else {
            // Split mode: rows of an even number of elements, so that every row starts on a
            // 16-byte boundary (the TMA copies of the merge tiles' footprints need that).
            d.out_offset = (long long)(arena / sizeof(float2));
            d.out_stride = mode == SARBP_SPLIT ? d.nu + (d.nu & 1) : d.nu;
            arena += align_up((size_t)d.nr * d.out_stride * sizeof(float2));
        }
        d.rows_off = p->table_entries;
        d.cols_off = p->table_entries + 3LL * d.nr;
        p->table_entries += 3LL * d.nr + d.nu;
        p->max_dim = std::max(p->max_dim, std::max(d.nr, d.nu));
        double radius = 0.0;
        d.tile_lc = split_polar_tile_lc(d, &radius);
        if (d.left >= 0 && mode == SARBP_SPLIT) d.tile_lc = split_polar_tile_lc_slack(d, kMergeTileSlack, nullptr);
        const bool external = d.left < 0 && d.a < 0;
        if (d.left < 0 && mode == SARBP_SPLIT && !external) {
            // Leaves use the origin formulation: precision does not depend on the tile shape.  Of the
            // 32x32, 16x64 and 8x128 shapes the one with the fewest tiles over the leaf grid wastes the
            // least work on pixels past its edge (ties: the shorter tile, whose range windows are shorter).
            d.tile_lc = 5;
            long long fewest = -1;
            for (int lc = 5; lc >= 3; --lc) {
                const long long rows_t = kSplitTilePixels >> lc, cols_t = 1LL << lc;
                const long long t = ((d.win_nr + rows_t - 1) / rows_t) * ((d.win_nu + cols_t - 1) / cols_t);
                if (fewest < 0 || t < fewest) {
                    fewest = t;
                    d.tile_lc = lc;
                }
            }
            p->leaves.push_back(i);
            p->max_pulse = std::max(p->max_pulse, d.b);
        }
        if (d.left < 0 && !external) {
            leaf_radius = std::max(leaf_radius, radius);
            leaf_pulses = std::max(leaf_pulses, d.b - d.a);
        }
    }
    p->leaf_wb = std::max(4, split_window_bins(leaf_radius, 1.0));  // rescaled at execute for data_dr
    // Work lists per stage.
    p->stage_begin.assign(p->max_height + 1, 0);
    p->stage_count.assign(p->max_height + 1, 0);
    for (int h = 0; h <= p->max_height; ++h) {
        p->stage_begin[h] = mode == SARBP_SPLIT ? (int)p->items.size() : (int)p->blocks.size();
        for (int i = 0; i < n_nodes; ++i) {
            if (p->height[i] != h) continue;
            const PolarDesc& d = p->nodes[i];
            if (d.left < 0 && d.a < 0) continue;  // external: no work, its image is supplied
            if (mode == SARBP_SPLIT) {
                const int cols_t = 1 << d.tile_lc, rows_t = kSplitTilePixels >> d.tile_lc;
                for (int r = 0; r < d.win_nr; r += rows_t)
                    for (int u = 0; u < d.win_nu; u += cols_t) p->items.push_back(TileItem{i, r, u, 0});
            } else {
                const long long npix = (long long)d.win_nr * d.win_nu;
                for (long long s = 0; s < npix; s += 256) p->blocks.push_back(make_int2(i, (int)s));
            }
        }
        p->stage_count[h] = (mode == SARBP_SPLIT ? (int)p->items.size() : (int)p->blocks.size()) - p->stage_begin[h];
    }
    if ((mode == SARBP_SPLIT ? p->items.size() : p->blocks.size()) > (size_t)INT32_MAX) {
        delete p;
        return fail(SARBP_ERR_PLAN, "plan too large");
    }
    p->leaf_chunk = leaf_pulses;
    p->node_bytes = align_up(sizeof(PolarDesc) * n_nodes);
    p->work_bytes = align_up(mode == SARBP_SPLIT ? sizeof(TileItem) * p->items.size() : sizeof(int2) * p->blocks.size());
    if (mode == SARBP_SPLIT) {
        p->merge_items = (long long)p->items.size() - p->stage_count[0];
        p->leaf_list_bytes = align_up(sizeof(int) * p->leaves.size());
        p->table_bytes = align_up(sizeof(float4) * (size_t)p->table_entries);
        p->prec_bytes = align_up(split_ffbp_pulse_record_bytes() * (size_t)p->max_pulse);
        p->crec_bytes = align_up(split_ffbp_child_record_bytes() * 2 * (size_t)p->merge_items);
    }
    if (mode == SARBP_SPLIT) {
        // Merge queue: per node its merge tiles, its merge children (leaves and external nodes are
        // complete before the queue starts) and its parent.
        p->q_remaining.assign(n_nodes, 0);
        p->q_pending.assign(n_nodes, 0);
        p->q_parent.assign(n_nodes, -1);
        for (int i = 0; i < n_nodes; ++i) {
            const PolarDesc& d = p->nodes[i];
            if (d.left < 0) continue;
            for (int c : {d.left, d.right}) {
                p->q_parent[c] = i;
                if (p->nodes[c].left >= 0) ++p->q_pending[i];
            }
        }
        for (size_t t = (size_t)p->stage_begin[0] + p->stage_count[0]; t < p->items.size(); ++t)
            ++p->q_remaining[p->items[t].node];
        // [next, status] then live remaining, live pending, parent, initial remaining, initial pending
        p->queue_bytes = align_up(sizeof(int) * (2 + 5 * (size_t)n_nodes));
    }
    if (mode == SARBP_SPLIT) {
        child_footprints(*p);
        p->tmap_bytes = align_up(kTensorMapBytes * (size_t)n_nodes);
    }
    p->table_offset = p->node_bytes + p->work_bytes + p->leaf_list_bytes;
    p->prec_offset = p->table_offset + p->table_bytes;
    p->crec_offset = p->prec_offset + p->prec_bytes;
    p->queue_offset = p->crec_offset + p->crec_bytes;
    p->tmap_offset = p->queue_offset + p->queue_bytes;
    p->arena_offset = p->tmap_offset + p->tmap_bytes;
    p->arena_bytes = arena;
    p->total_bytes = p->arena_offset + arena;
    p->launches = p->max_height + 1 + (mode == SARBP_SPLIT ? 3 : 0);
    *plan_out = p;
    return SARBP_OK;
}

void sarbp_ffbp_plan_destroy(sarbp_ffbp_plan* plan) { delete plan; }

size_t sarbp_ffbp_workspace_bytes(const sarbp_ffbp_plan* plan) { return plan ? plan->total_bytes : 0; }

int sarbp_ffbp_launch_count(const sarbp_ffbp_plan* plan) { return plan ? plan->launches : 0; }

int sarbp_ffbp_bind(sarbp_ffbp_plan* plan, void* workspace, size_t workspace_bytes, void* stream) {
    if (!plan) return fail(SARBP_ERR_TYPE, "plan must not be NULL");
    if (!workspace || workspace_bytes < plan->total_bytes)
        return fail(SARBP_ERR_WORKSPACE, "FFBP plan needs %zu workspace bytes", plan->total_bytes);
    if ((uintptr_t)workspace % 256) return fail(SARBP_ERR_TYPE, "workspace must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    char* base = reinterpret_cast<char*>(workspace);
    cudaError_t e = cudaMemcpyAsync(base, plan->nodes.data(), sizeof(PolarDesc) * plan->n_nodes,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        if (plan->mode == SARBP_SPLIT)
            e = cudaMemcpyAsync(base + plan->node_bytes, plan->items.data(), sizeof(TileItem) * plan->items.size(),
                                cudaMemcpyHostToDevice, s);
        else
            e = cudaMemcpyAsync(base + plan->node_bytes, plan->blocks.data(), sizeof(int2) * plan->blocks.size(),
                                cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess && !plan->leaves.empty())
        e = cudaMemcpyAsync(base + plan->node_bytes + plan->work_bytes, plan->leaves.data(),
                            sizeof(int) * plan->leaves.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && plan->queue_bytes) {
        const size_t n = (size_t)plan->n_nodes;
        int* q = reinterpret_cast<int*>(base + plan->queue_offset);
        e = cudaMemcpyAsync(q + 2 + 2 * n, plan->q_parent.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(q + 2 + 3 * n, plan->q_remaining.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            std::vector<int> pending = plan->q_pending;
            if (plan->withheld >= 0) ++pending[plan->withheld];  // never reaches zero
            e = cudaMemcpyAsync(q + 2 + 4 * n, pending.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // `pending` is a host temporary
        }
    }
    // Tensor maps of the child images (merge tiles stage their footprints by TMA); without the
    // driver's encoder the merges gather from the child images instead (the same image).
    std::vector<CUtensorMap> maps;
    plan->staged = false;
    if (e == cudaSuccess && plan->mode == SARBP_SPLIT && plan->staging && plan->tmap_bytes) {
        float2* arena = reinterpret_cast<float2*>(base + plan->arena_offset);
        plan->staged = encode_child_maps(*plan, arena, maps);
        if (plan->staged)
            e = cudaMemcpyAsync(base + plan->tmap_offset, maps.data(), sizeof(CUtensorMap) * maps.size(),
                                cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // also keeps `maps` alive until its copy is done
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "FFBP bind: %s", cudaGetErrorString(e));
    plan->bound = workspace;
    plan->bound_bytes = workspace_bytes;
    return SARBP_OK;
}

int sarbp_ffbp_set_node_image(const sarbp_ffbp_plan* plan, int node, const float* image, void* stream) {
    if (!plan) return fail(SARBP_ERR_TYPE, "plan must not be NULL");
    if (!plan->bound) return fail(SARBP_ERR_PLAN, "sarbp_ffbp_bind must succeed before set_node_image");
    if (!image) return fail(SARBP_ERR_TYPE, "image must not be NULL");
    if (node <= 0 || node >= plan->n_nodes) return fail(SARBP_ERR_VALUE, "node %d is not a non-root node", node);
    const PolarDesc& d = plan->nodes[node];
    if (!(d.left < 0 && d.a < 0)) return fail(SARBP_ERR_PLAN, "node %d is not an external node", node);
    if ((uintptr_t)image & 7) return fail(SARBP_ERR_TYPE, "image must be 8-byte aligned");
    float2* arena = reinterpret_cast<float2*>(reinterpret_cast<char*>(plan->bound) + plan->arena_offset);
    const cudaError_t e = cudaMemcpy2DAsync(arena + d.out_offset, (size_t)d.out_stride * sizeof(float2), image,
                                            (size_t)d.nu * sizeof(float2), (size_t)d.nu * sizeof(float2), (size_t)d.nr,
                                            cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "set_node_image: %s", cudaGetErrorString(e));
    return SARBP_OK;
}

int sarbp_ffbp_set_merge_queue(sarbp_ffbp_plan* plan, int on) {
    if (!plan) return fail(SARBP_ERR_TYPE, "plan must not be NULL");
    if (on != 0 && on != 1) return fail(SARBP_ERR_VALUE, "on must be 0 or 1 (got %d)", on);
    if (on && plan->mode != SARBP_SPLIT) return fail(SARBP_ERR_VALUE, "the merge queue is a split-mode path");
    plan->merge_queue = on != 0;
    plan->launches = plan->mode == SARBP_SPLIT
                         ? 3 + 1 + (plan->max_height > 0 ? (plan->merge_queue ? 1 : plan->max_height) : 0)
                         : plan->max_height + 1;
    return SARBP_OK;
}

int sarbp_ffbp_set_staging(sarbp_ffbp_plan* plan, int on) {
    if (!plan) return fail(SARBP_ERR_TYPE, "plan must not be NULL");
    if (on != 0 && on != 1) return fail(SARBP_ERR_VALUE, "on must be 0 or 1 (got %d)", on);
    if (plan->bound) return fail(SARBP_ERR_PLAN, "set staging before sarbp_ffbp_bind");
    plan->staging = on != 0;
    return SARBP_OK;
}

int sarbp_ffbp_staging(const sarbp_ffbp_plan* plan, int* staged) {
    if (!plan || !staged) return fail(SARBP_ERR_TYPE, "plan and staged must not be NULL");
    *staged = plan->staged ? 1 : 0;
    return SARBP_OK;
}

int sarbp_ffbp_set_wait_limit(sarbp_ffbp_plan* plan, double seconds, int withheld_node) {
    if (!plan) return fail(SARBP_ERR_TYPE, "plan must not be NULL");
    if (!(seconds > 0.0 && seconds <= 60.0)) return fail(SARBP_ERR_VALUE, "the wait limit must be in (0, 60] s");
    if (withheld_node < -1 || withheld_node >= plan->n_nodes || (withheld_node >= 0 && plan->nodes[withheld_node].left < 0))
        return fail(SARBP_ERR_VALUE, "withheld_node must be -1 or a merge node");
    if (plan->bound) return fail(SARBP_ERR_PLAN, "set the wait limit before sarbp_ffbp_bind");
    plan->queue_limit_ns = (unsigned long long)(seconds * 1e9);
    plan->withheld = withheld_node;
    return SARBP_OK;
}

int sarbp_ffbp_status(const sarbp_ffbp_plan* plan, int* status) {
    if (!plan || !status) return fail(SARBP_ERR_TYPE, "plan and status must not be NULL");
    if (!plan->bound) return fail(SARBP_ERR_PLAN, "sarbp_ffbp_bind must succeed before status");
    *status = 0;
    if (!plan->queue_bytes) return SARBP_OK;
    const int* q = reinterpret_cast<const int*>(reinterpret_cast<const char*>(plan->bound) + plan->queue_offset);
    const cudaError_t e = cudaMemcpy(status, q + 1, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "status: %s", cudaGetErrorString(e));
    return SARBP_OK;
}

int sarbp_ffbp_execute(const sarbp_ffbp_plan* plan, const float* data, int pulses, int samples, const double* pos,
                       const double* weight, const double* phase, double range_start, double data_dr, double k,
                       float* out, void* stream) {
    if (!plan) return fail(SARBP_ERR_TYPE, "plan must not be NULL");
    if (!plan->bound) return fail(SARBP_ERR_PLAN, "sarbp_ffbp_bind must succeed before execute");
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (!out) return fail(SARBP_ERR_TYPE, "out must not be NULL");
    for (int i = 0; i < plan->n_nodes; ++i)
        if (plan->nodes[i].left < 0 && plan->nodes[i].b > pulses)
            return fail(SARBP_ERR_PLAN, "leaf %d uses pulses beyond the %d supplied", i, pulses);
    cudaStream_t s = (cudaStream_t)stream;
    char* base = reinterpret_cast<char*>(plan->bound);
    const PolarDesc* nodes = reinterpret_cast<const PolarDesc*>(base);
    float2* arena = reinterpret_cast<float2*>(base + plan->arena_offset);
    float2* root_out = reinterpret_cast<float2*>(out);
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    int st = SARBP_OK;
    if (plan->mode == SARBP_SPLIT) {
        const TileItem* items = reinterpret_cast<const TileItem*>(base + plan->node_bytes);
        const int* leaves = reinterpret_cast<const int*>(base + plan->node_bytes + plan->work_bytes);
        float4* tables = reinterpret_cast<float4*>(base + plan->table_offset);
        void* precs = base + plan->prec_offset;
        void* crecs = base + plan->crec_offset;
        // A leaf tile spans rows_t dr of range; pulses add their offset from the leaf centre.
        const int wb = (int)ceil(ffbp_leaf_tile_span(*plan) / fabs(data_dr)) + 48;
        const int ch = split_chunk_for(wb, plan->leaf_chunk, true);
        st = launch_split_ffbp_tables(in, nodes, plan->n_nodes, plan->max_dim, tables, s);
        if (st == SARBP_OK)
            st = launch_split_ffbp_leaf_pulses(in, nodes, leaves, (int)plan->leaves.size(), precs, s);
        if (st == SARBP_OK)
            st = launch_split_ffbp_child_records(k, nodes, tables, items + plan->stage_begin[0] + plan->stage_count[0],
                                                 (int)plan->merge_items, arena,
                                                 plan->staged && !plan->merge_queue ? base + plan->tmap_offset : nullptr,
                                                 crecs, s);
        if (st == SARBP_OK)
            st = launch_split_ffbp_leaves(in, nodes, items + plan->stage_begin[0], plan->stage_count[0], ch, wb,
                                          tables, precs, arena, root_out, 0, s);
        const size_t crec_size = split_ffbp_child_record_bytes();
        if (plan->merge_queue && plan->max_height > 0 && st == SARBP_OK) {
            const size_t n = (size_t)plan->n_nodes;
            int* q = reinterpret_cast<int*>(base + plan->queue_offset);
            cudaError_t e = cudaMemsetAsync(q, 0, 2 * sizeof(int), s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(q + 2, q + 2 + 3 * n, 2 * n * sizeof(int), cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "merge queue reset: %s", cudaGetErrorString(e));
            MergeQueue Q;
            Q.next = q;
            Q.status = q + 1;
            Q.remaining = q + 2;
            Q.pending = q + 2 + n;
            Q.parent = q + 2 + 2 * n;
            Q.limit_ns = plan->queue_limit_ns;
            st = launch_split_ffbp_merge_queue(k, nodes, items + plan->stage_begin[1], (int)plan->merge_items, tables,
                                               crecs, arena, root_out, 0, Q, s);
        }
        for (int h = 1; h <= plan->max_height && st == SARBP_OK && !plan->merge_queue; ++h) {
            const size_t first = (size_t)(plan->stage_begin[h] - plan->stage_begin[1]);
            st = launch_split_ffbp_merges(k, nodes, items + plan->stage_begin[h], plan->stage_count[h], tables,
                                          reinterpret_cast<char*>(crecs) + 2 * first * crec_size, arena, root_out, 0,
                                          plan->staged ? plan->merge_box_bytes[h] : 0, plan->queue_limit_ns,
                                          plan->withheld, s);
        }
    } else {
        const int2* blocks = reinterpret_cast<const int2*>(base + plan->node_bytes);
        st = launch_plain_ffbp_leaves(plan->mode, in, nodes, blocks + plan->stage_begin[0], plan->stage_count[0],
                                      arena, s);
        for (int h = 1; h <= plan->max_height && st == SARBP_OK; ++h)
            st = launch_plain_ffbp_merges(plan->mode, k, nodes, blocks + plan->stage_begin[h], plan->stage_count[h],
                                          arena, root_out, 0, s);
    }
    return st;
}

// ---- polar -> Cartesian, autofocus helpers, LUT probe ---------------------------------------
int sarbp_evaluate_image(const float* image, const sarbp_polar_grid* grid, const double* xyz, int npts, double k,
                         float* out, void* stream) {
    if (!image || !xyz || !out) return fail(SARBP_ERR_TYPE, "image, xyz and out must not be NULL");
    if (int st = check_grid(grid)) return st;
    if (npts <= 0) return fail(SARBP_ERR_VALUE, "at least one point is required");
    if (!is_finite_value(k)) return fail(SARBP_ERR_VALUE, "k must be finite");
    return launch_evaluate(reinterpret_cast<const float2*>(image), desc_of(*grid), xyz, npts, k,
                           reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_evaluate_lattice(const float* image, const sarbp_polar_grid* grid, const sarbp_lattice* lattice, double k,
                           float* out, void* stream) {
    if (!image || !lattice || !out) return fail(SARBP_ERR_TYPE, "image, lattice and out must not be NULL");
    if (int st = check_grid(grid)) return st;
    if (lattice->rows <= 0 || lattice->cols <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    for (int c = 0; c < 3; ++c)
        if (!is_finite_value(lattice->origin[c]) || !is_finite_value(lattice->step_row[c]) ||
            !is_finite_value(lattice->step_col[c]))
            return fail(SARBP_ERR_VALUE, "lattice geometry must be finite");
    if (!is_finite_value(k)) return fail(SARBP_ERR_VALUE, "k must be finite");
    return launch_split_evaluate_lattice(reinterpret_cast<const float2*>(image), desc_of(*grid), *lattice, k,
                                         reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_target_contributions(const float* data, int pulses, int samples, const double* pos, const double* xyz,
                               int npts, double range_start, double data_dr, double k, float* out, void* stream) {
    if (!data || !pos || !xyz || !out) return fail(SARBP_ERR_TYPE, "data, pos, xyz and out must not be NULL");
    if (pulses < 1 || samples < 1 || npts < 1) return fail(SARBP_ERR_VALUE, "pulses, samples and npts must be positive");
    if (!is_finite_value(data_dr) || data_dr == 0.0 || !is_finite_value(k)) return fail(SARBP_ERR_VALUE, "data_dr and k must be finite, data_dr non-zero");
    const PulseInputs in = inputs_of(data, pulses, samples, pos, nullptr, nullptr, range_start, data_dr, k);
    return launch_target_contrib(in, xyz, npts, reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_fill_range_phase_lut(int samples, double range_start, double data_dr, double k, float* lut, void* stream) {
    if (!lut) return fail(SARBP_ERR_TYPE, "lut must not be NULL");
    if (samples < 1) return fail(SARBP_ERR_VALUE, "samples must be positive");
    return launch_fill_lut(samples, range_start, data_dr, k, reinterpret_cast<float2*>(lut), (cudaStream_t)stream);
}

int sarbp_direct_polar_lut(const float* data, int pulses, int samples, const double* pos, const double* weight,
                           const double* phase, const sarbp_polar_grid* grid, double range_start, double data_dr,
                           double k, const float* lut, float* out, void* stream) {
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (int st = check_grid(grid)) return st;
    if (!lut || !out) return fail(SARBP_ERR_TYPE, "lut and out must not be NULL");
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    return launch_plain_polar_lut(in, desc_of(*grid), reinterpret_cast<const float2*>(lut),
                                  reinterpret_cast<float2*>(out), (cudaStream_t)stream);
}

int sarbp_direct_polar_phase32(const float* data, int pulses, int samples, const double* pos, const double* weight,
                               const double* phase, const sarbp_polar_grid* grid, double range_start, double data_dr,
                               double k, int wrapped, float* out, void* stream) {
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (int st = check_grid(grid)) return st;
    if (!out) return fail(SARBP_ERR_TYPE, "out must not be NULL");
    if (wrapped != 0 && wrapped != 1) return fail(SARBP_ERR_VALUE, "wrapped must be 0 or 1 (got %d)", wrapped);
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    return launch_plain_polar_phase32(in, desc_of(*grid), wrapped != 0, reinterpret_cast<float2*>(out),
                                      (cudaStream_t)stream);
}

}  // extern "C"
