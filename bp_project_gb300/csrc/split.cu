// Split-precision back-projection kernels (the fast path).
//
// Work unit: one CTA = one tile of 1024 output pixels (256 threads x 4 pixels),
// looping over its pulses in shared-memory chunks.  Precision plan (per pixel p,
// pulse n, tile centre c; the wide-precision work is per tile or per (tile, pulse), in
// two-float FP32 from the FP64 inputs split once into hi + lo):
//
//   d(p,n) = R + L + eps,    R = |c - pos_n| (two-float, per tile-pulse)
//                            L = u . delta_p  (u = (c - pos_n)/R, delta_p = p - c)
//                            eps = |delta_p x u|^2 / (R + L + d)   (<= ~1 cm, FP32)
//   phase turns = frac(K R + phase_n / 2pi)            two-float -> FP32, per tile-pulse
//               + frac(K u . delta_p)                  exact: W_hi . delta_hi
//               + W_hi . delta_lo + W_lo . delta_p     FP32, tiny terms
//               + K eps - K r_p (polar demodulation, per pixel)
//
// with K = k / 2pi, W = K u.  W_hi is a multiple of 2^eW with <= 10 significant
// bits and delta_hi a multiple of 2^ed with <= 12 (2-D) / 11 (3-D) bits, so each
// product and their sum are exact in FP32 and the large linear phase term is
// reduced modulo one turn without rounding.  The reduced phase feeds the
// hardware sin/cos (MUFU) on [-pi, pi).
//
// Lattice tiles go further: delta_p = i s_row + j s_col, so u . delta_p and W . delta_p are
// sums of a row and a column term.  The records carry the two terms per pulse (the phase
// ones split exactly as above), each thread forms them once per pulse at a reference pixel,
// and its four pixels, m rows apart, step from there: per pixel-pulse only the eps term,
// the window gather and the rotation remain.
//
// Range interpolation: for each (tile, pulse) the chunk stages the range bins
// the tile can touch as Horner coefficients of the reference's four-point
// Lagrange cubic (weight folded in), 32 bytes per bin; a pixel-pulse is then
// two 16-byte shared loads and six FMAs.  Bins whose taps leave the row are
// stored as zero, which reproduces the reference's support rule
// (fast_bp/ffbp.py:27).  A pulse whose window would not fit the staged bins, or that lies
// outside the precision envelope, runs through a two-float per-sample fallback instead.
#include <limits.h>
#include <math.h>

#include "common.cuh"

namespace sarbp {
namespace {

constexpr int kThreads = kSplitThreads;
constexpr int kPX = 4;
// Threads of the single-scene merge kernel: four column pairs of parent pixels per thread (more
// gathers in flight per warp than two pairs at 256 threads).
constexpr int kMergeThreads = 128;
constexpr int kMaxRows = kSplitTilePixels >> 2;  // tile_lc >= 2
constexpr int kMaxCols = 32;                     // tile_lc <= 5
constexpr int kMaxChunk = 64;      // pulses per chunk of the direct kernels: two warps compute the records
constexpr int kMaxLeafChunk = 32;  // pulses per chunk of the FFBP leaf kernels: one warp computes the records
// Window bytes per CTA: with kMaxChunk records this keeps three CTAs per SM within 227 KB.
constexpr int kWindowBudget = 68 * 1024;
// Lattice tiles (64 registers): four CTAs per SM.  Per CTA, 49 KB of windows, 5 KB of 80-byte
// records, up to 1.25 KB of static shared memory (the batch kernel) and the 1 KB the runtime
// reserves: 4 x 56.25 KB fits the SM's 228 KB.  The packed windows of a 32 x 32 tile at the
// usual geometries need 15-25 bins per pulse, so 64-pulse chunks mostly fit; wider windows
// just fit fewer pulses per chunk (the image does not depend on the chunking).
constexpr int kLatticeWindowBudget = 49 * 1024;
#ifndef SARBP_BULK_WINDOWS
#define SARBP_BULK_WINDOWS 0
#endif
// Bulk-copy window staging (SARBP_BULK_WINDOWS = 1): each pulse's raw samples arrive in shared
// memory by one cp.async.bulk copy (completion on an mbarrier) before the Horner transform,
// instead of the transform's own global loads.  The raw samples need room beside the windows:
// per window bin 8 bytes plus five samples of margin per pulse, so the window budgets shrink to
// keep the same CTAs per SM.
constexpr int kBulkMargin = 5;
__host__ __device__ constexpr int raw_bytes_for(int cap, int chunk) {
    return SARBP_BULK_WINDOWS ? (cap + kBulkMargin * chunk) * 8 + 16 : 0;
}
// K rho^2 / R limits (turns) for the FP32 eps term: direct BP targets 1e-5 relative
// error, FFBP leaves 1e-4.
constexpr double kDirectEnvelope = 8.0;

struct Rec {
    float4 a;  // W_hi.x, W_hi.y, W_lo.x, W_lo.y   (lattice: B_row hi, lo, B_col hi, lo)
    float4 b;  // u.x, u.y, 2R, frac(Q) - 1/2       (lattice: u.s_row, u.s_col, 2R, frac(Q) - 1/2)
    float4 c;  // Phi, window bias bits, window offset bits, window count - 1 bits
    float4 d;  // u.z, W_hi.z, W_lo.z                (lattice: 2 pi frac(m B_row), m u.s_row or u.x, u.y, u.z)
    float4 e;  // lattice forward: the pairs (2R, 2R), (frac(Q) - 1/2, frac(Q) - 1/2) of packed-FP32 operands
};

struct Pix {
    float dx, dy, dz;
    float dxh, dyh, dzh;
    float dxl, dyl, dzl;
    float d2, psi;
    float ar, ai;
};

struct TileShared {
    double cx, cy, cz;
    float ch[3], cl[3];         // the centre as two-float (hi + lo), for the FP32 records
    float rhof;
    double rho;                 // bound on |delta_p| (m)
    double scale_d, inv_scale_d;
    double sum[4];
    float bnd[3];               // bounds on |delta_x|, |delta_y|, |delta_z| (m)
    float scale_f, inv_scale_f; // FP32 offset quantum of polar merge tiles
    float red[8][8];
    int base[kMaxChunk];        // global bin of window entry 0, per pulse of the chunk
    float wt[kMaxChunk];
    int nfit;
    int nfit_w[2];              // fitting pulses among each record warp's 32
    unsigned miss_w[2];         // pulses of each record warp that cannot be staged (bit per lane)
    int wsum;                   // window entries of record warp 0's pulses
    float sth[6], stl[6];       // lattice tiles: step_row (0-2) and step_col (3-5) as two-float
    int row_step;               // lattice tiles: rows between a thread's successive pixels
#if SARBP_BULK_WINDOWS
    int roff[kMaxChunk];        // bulk staging: first raw sample of each pulse in shared memory
    long long raw0[kMaxChunk];  // bulk staging: data-array index of that sample
#endif
};

// Row/column tables of a polar tile; aliased onto the window region during set-up.
struct PolarTables {
    double rx[kMaxRows], ry[kMaxRows];
    float rxh[kMaxRows], rxl[kMaxRows], ryh[kMaxRows], ryl[kMaxRows], dg[kMaxRows], psi[kMaxRows];
    double cxd[kMaxCols], cyd[kMaxCols];
    float cxh[kMaxCols], cxl[kMaxCols], cyh[kMaxCols], cyl[kMaxCols], dcs[kMaxCols], duu[kMaxCols];
};

struct SplitParams {
    PulseInputs in;
    float2* out;           // direct jobs: output image (pulse split s writes out + s * split_stride)
    long long out_stride;
    double K;              // k / 2pi (turns per metre)
    double inv_dr;         // 1 / data_dr
    double scale_w, inv_scale_w;
    float Kf, inv_drf;
    int chunk;             // pulses per chunk (<= kMaxChunk)
    int cap;               // window entries (32 bytes each) available per chunk
    int pulse_split;
    long long split_stride;
    // Precision envelope of the FP32 eps term: the fast path needs K rho^2 / R <= envelope
    // (the FP32 error of eps is ~2.5e-7 * rho^2 / R metres, i.e. ~2.5e-7 * envelope turns).
    double envelope;
    // Two-float (hi + lo) copies for the FP32 fallback of pulses outside the envelope.
    float Kh, Kl, rsh, rsl, idrh, idrl;
};

struct Job {
    PolarDesc g;          // polar grids
    sarbp_lattice lat;    // lattices
    const double* xyz;    // point lists
    int npts;
    int tile_r, tile_u, lc;
    int p0, p1;
};

// (v, v): an operand of the packed FP32 (f32x2) instructions.
__device__ __forceinline__ float2 pair(float v) { return make_float2(v, v); }

// ---- block reductions (256 threads) ---------------------------------------------
template <int N>
__device__ __forceinline__ void block_max(TileShared& S, float v[N]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[i] = fmaxf(v[i], __shfl_xor_sync(0xffffffffu, v[i], o));
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < N; ++i) S.red[warp][i] = v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float m = S.red[0][i];
#pragma unroll
        for (int w = 1; w < 8; ++w) m = fmaxf(m, S.red[w][i]);
        v[i] = m;
    }
    __syncthreads();
}

__device__ __forceinline__ void block_sum4(TileShared& S, double v[4]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double part[8][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) part[warp][i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < 4; ++i) {
            double s = 0.0;
            for (int w = 0; w < 8; ++w) s += part[w][i];
            S.sum[i] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = S.sum[i];
    __syncthreads();
}

// v as an unevaluated sum h + l of two FP32 numbers.
__device__ __forceinline__ void split2(double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

__device__ __forceinline__ void set_quantum(TileShared& S, float bound, int bits) {
    int e;
    frexp((double)bound, &e);
    S.scale_d = ldexp(1.0, e - bits);
    S.inv_scale_d = ldexp(1.0, bits - e);
}

__device__ __forceinline__ void pixel_from_offsets(const TileShared& S, double ox, double oy, double oz, Pix& P) {
    quantize(ox, S.scale_d, S.inv_scale_d, P.dxh, P.dxl);
    quantize(oy, S.scale_d, S.inv_scale_d, P.dyh, P.dyl);
    quantize(oz, S.scale_d, S.inv_scale_d, P.dzh, P.dzl);
    P.dx = (float)ox;
    P.dy = (float)oy;
    P.dz = (float)oz;
    P.d2 = P.dx * P.dx + P.dy * P.dy + P.dz * P.dz;
}

// ---- per-tile set-up: tile centre, quantum, per-pixel offsets -------------------
// Polar tile: rows/cols of a polar grid window; separable FP64 row and column
// tables give each pixel offset as an exact hi part plus an FP32 remainder.
__device__ void setup_polar(const SplitParams& P, const Job& J, TileShared& S, PolarTables& T, Pix px[kPX],
                            bool demodulate) {
    const PolarDesc& g = J.g;
    const int tid = threadIdx.x;
    const int cols_t = 1 << J.lc, rows_t = kSplitTilePixels >> J.lc;
    const double oz = g.oz, side = (double)g.side;
    const int i0 = g.win_r0 + J.tile_r + (rows_t >> 1);
    const int j0 = g.win_u0 + J.tile_u + (cols_t >> 1);
    const double rc = g.r0 + (double)i0 * g.dr;
    const double gc = sqrt(fmax(0.0, rc * rc - oz * oz));
    const double uc = g.u0 + (double)j0 * g.du;
    const double cc = sqrt(fmax(0.0, 1.0 - uc * uc));
    float m[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (tid < rows_t) {
        const double r = g.r0 + (double)(g.win_r0 + J.tile_r + tid) * g.dr;
        const double dg = sqrt(fmax(0.0, r * r - oz * oz)) - gc;
        const double rx = side * dg * cc, ry = dg * uc;
        T.rx[tid] = rx;
        T.ry[tid] = ry;
        T.dg[tid] = (float)dg;
        const double t = -P.K * r;
        T.psi[tid] = demodulate ? (float)(t - rint(t)) : 0.0f;
        m[0] = (float)fabs(rx);
        m[1] = (float)fabs(ry);
        m[2] = (float)fabs(dg);
    }
    if (tid < cols_t) {
        const double u = g.u0 + (double)(g.win_u0 + J.tile_u + tid) * g.du;
        const double dc = sqrt(fmax(0.0, 1.0 - u * u)) - cc, du = u - uc;
        const double cx = side * gc * dc, cy = gc * du;
        T.cxd[tid] = cx;
        T.cyd[tid] = cy;
        T.dcs[tid] = (float)(side * dc);
        T.duu[tid] = (float)du;
        m[3] = (float)fabs(cx);
        m[4] = (float)fabs(cy);
        m[5] = (float)fabs(dc);
        m[6] = (float)fabs(du);
    }
    block_max<7>(S, m);
    // Bounds on |delta_x|, |delta_y| (slightly enlarged for the FP32 maxima).
    const float bx = (m[0] + m[3] + m[2] * m[5]) * 1.0001f + 1e-6f;
    const float by = (m[1] + m[4] + m[2] * m[6]) * 1.0001f + 1e-6f;
    if (tid == 0) {
        S.cx = g.ox + side * gc * cc;
        S.cy = g.oy + gc * uc;
        S.cz = 0.0;
        S.rho = sqrt((double)bx * bx + (double)by * by);
        S.bnd[0] = bx;
        S.bnd[1] = by;
        S.bnd[2] = 0.0f;
        set_quantum(S, fmaxf(bx, by), 12);
    }
    __syncthreads();
    if (tid < rows_t) {
        quantize(T.rx[tid], S.scale_d, S.inv_scale_d, T.rxh[tid], T.rxl[tid]);
        quantize(T.ry[tid], S.scale_d, S.inv_scale_d, T.ryh[tid], T.ryl[tid]);
    }
    if (tid < cols_t) {
        quantize(T.cxd[tid], S.scale_d, S.inv_scale_d, T.cxh[tid], T.cxl[tid]);
        quantize(T.cyd[tid], S.scale_d, S.inv_scale_d, T.cyh[tid], T.cyl[tid]);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int p = tid + kThreads * k;
        const int row = p >> J.lc, col = p & (cols_t - 1);
        Pix& q = px[k];
        q.dxh = T.rxh[row] + T.cxh[col];  // exact: both multiples of the quantum
        q.dyh = T.ryh[row] + T.cyh[col];
        q.dxl = fmaf(T.dg[row], T.dcs[col], T.rxl[row] + T.cxl[col]);
        q.dyl = fmaf(T.dg[row], T.duu[col], T.ryl[row] + T.cyl[col]);
        q.dzh = q.dzl = q.dz = 0.0f;
        q.dx = q.dxh + q.dxl;
        q.dy = q.dyh + q.dyl;
        q.d2 = q.dx * q.dx + q.dy * q.dy;
        q.psi = T.psi[row];
        q.ar = q.ai = 0.0f;
    }
    __syncthreads();  // the tables alias the window region
}

// Polar tile set-up from per-node tables of float pairs (FFBP):
// FP32 two-float arithmetic only, no block reductions.  Row i holds three
// float4: (g hi, g lo, psi, 0), (g/r hi, g/r lo, -oz/r hi, -oz/r lo) and
// (2r, frac(Q) - 1/2, floor(Q) bits, 0) with g = sqrt(r^2 - oz^2),
// psi = frac(-K r) and Q = (r - range_start) / data_dr; column j holds
// (c hi, c lo, u hi, u lo) with c = sqrt(1 - u^2).
struct TabF {
    float rxh[kMaxRows], rxl[kMaxRows], ryh[kMaxRows], ryl[kMaxRows], dg[kMaxRows], psi[kMaxRows];
    float cxh[kMaxCols], cxl[kMaxCols], cyh[kMaxCols], cyl[kMaxCols], dcs[kMaxCols], duu[kMaxCols];
};

// (ah + al) * (bh + bl) as an unevaluated pair p + e.
__device__ __forceinline__ void two_prod(float ah, float al, float bh, float bl, float& p, float& e) {
    p = ah * bh;
    e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
}

__device__ __forceinline__ void quantize_pair(float& p, float& e, float q, float iq) {
    const float h = rintf(p * iq) * q;  // exact: q is a power of two and |p / q| < 2^14
    e = (p - h) + e;                    // p - h is exact
    p = h;
}

// One row (i) and one column (j) of a merge tile's tables, before quantization; r0v and c0v are
// the tile centre's row and column (i0, j0).
struct TabRow {
    float rxh, rxl, ryh, ryl, dg, psi;
};
struct TabCol {
    float cxh, cxl, cyh, cyl, dcs, duu;
};

__device__ __forceinline__ TabRow tab_row(const PolarDesc& g, const float4* __restrict__ tables, float4 r0v,
                                          float4 c0v, int i) {
    const float4 rv = __ldg(tables + g.rows_off + 3 * (long long)i);
    const float side = (float)g.side;
    const float dh = rv.x - r0v.x, dl = rv.y - r0v.y;  // g values of one node: dh is exact
    TabRow R;
    float p, e;
    two_prod(dh, dl, c0v.x, c0v.y, p, e);
    R.rxh = side * p;
    R.rxl = side * e;
    two_prod(dh, dl, c0v.z, c0v.w, p, e);
    R.ryh = p;
    R.ryl = e;
    R.dg = dh + dl;
    R.psi = rv.z;
    return R;
}

__device__ __forceinline__ TabCol tab_col(const PolarDesc& g, const float4* __restrict__ tables, float4 r0v,
                                          float4 c0v, int j, int j0) {
    const float4 cv = __ldg(tables + g.cols_off + j);
    const float side = (float)g.side;
    const float ch = cv.x - c0v.x, cl = cv.y - c0v.y;  // c in (0, 1] within a factor 2: exact
    // u_j - u_0 = (j - j0) du, formed from the integer offset (no cancellation).
    const float kj = (float)(j - j0);
    const float duh = (float)g.du, dul = (float)(g.du - (double)duh);
    const float uh = kj * duh;
    const float ul = fmaf(kj, duh, -uh) + kj * dul;
    TabCol C;
    float p, e;
    two_prod(r0v.x, r0v.y, ch, cl, p, e);
    C.cxh = side * p;
    C.cxl = side * e;
    two_prod(r0v.x, r0v.y, uh, ul, p, e);
    C.cyh = p;
    C.cyl = e;
    C.dcs = side * (ch + cl);
    C.duu = uh + ul;
    return C;
}

// Tile centre row and column of a merge tile (rows_t x cols_t pixels at (tile_r, tile_u)).
__device__ __forceinline__ void tab_centre(const PolarDesc& g, int lc, int tile_r, int tile_u,
                                           const float4* __restrict__ tables, float4& r0v, float4& c0v, int& j0) {
    const int cols_t = 1 << lc, rows_t = kSplitTilePixels >> lc;
    const int i0 = min(g.win_r0 + tile_r + (rows_t >> 1), g.nr - 1);
    j0 = min(g.win_u0 + tile_u + (cols_t >> 1), g.nu - 1);
    r0v = __ldg(tables + g.rows_off + 3 * (long long)i0);
    c0v = __ldg(tables + g.cols_off + j0);
}

// Power-of-two quantum of a merge tile's pixel offsets, 2^(e - 12) with the bound on |delta_x|,
// |delta_y| = m 2^e, m in [0.5, 1): row terms are monotone in i and column terms extreme at the
// tile edges, so the bound comes from the first and last row and column.  FP32 bit arithmetic;
// computed once per tile in the child-record prologue.
__device__ __forceinline__ void tab_quantum(const PolarDesc& g, int lc, int tile_r, int tile_u,
                                            const float4* __restrict__ tables, float& q, float& iq) {
    const int cols_t = 1 << lc, rows_t = kSplitTilePixels >> lc;
    float4 r0v, c0v;
    int j0;
    tab_centre(g, lc, tile_r, tile_u, tables, r0v, c0v, j0);
    const TabRow ra = tab_row(g, tables, r0v, c0v, min(g.win_r0 + tile_r, g.nr - 1));
    const TabRow rb = tab_row(g, tables, r0v, c0v, min(g.win_r0 + tile_r + rows_t - 1, g.nr - 1));
    const TabCol ca = tab_col(g, tables, r0v, c0v, min(g.win_u0 + tile_u, g.nu - 1), j0);
    const TabCol cb = tab_col(g, tables, r0v, c0v, min(g.win_u0 + tile_u + cols_t - 1, g.nu - 1), j0);
    const float mrx = fmaxf(fabsf(ra.rxh), fabsf(rb.rxh)), mry = fmaxf(fabsf(ra.ryh), fabsf(rb.ryh));
    const float mdg = fmaxf(fabsf(ra.dg), fabsf(rb.dg));
    const float mcx = fmaxf(fabsf(ca.cxh), fabsf(cb.cxh)), mcy = fmaxf(fabsf(ca.cyh), fabsf(cb.cyh));
    const float mdc = fmaxf(fabsf(ca.dcs), fabsf(cb.dcs)), mdu = fmaxf(fabsf(ca.duu), fabsf(cb.duu));
    const float bx = fmaf(fmaf(mdg, mdc, mrx + mcx), 1.0001f, 1e-6f);
    const float by = fmaf(fmaf(mdg, mdu, mry + mcy), 1.0001f, 1e-6f);
    const int e = ((__float_as_int(fmaxf(bx, by)) >> 23) & 0xff) - 126;
    q = __int_as_float((e - 12 + 127) << 23);
    iq = __int_as_float((12 - e + 127) << 23);
}

// Polar merge-tile set-up from per-node tables of float pairs (FFBP): FP32 two-float arithmetic
// only, one barrier.  The offsets are quantized on the tile's quantum (q, iq) from its child
// record, so each table entry is final when it is written.
template <int THREADS>
__device__ void setup_polar_tab(const Job& J, TabF& T, const float4* __restrict__ tables, float q, float iq) {
    const PolarDesc& g = J.g;
    const int tid = threadIdx.x;
    const int cols_t = 1 << J.lc, rows_t = kSplitTilePixels >> J.lc;
    float4 r0v, c0v;
    int j0;
    tab_centre(g, J.lc, J.tile_r, J.tile_u, tables, r0v, c0v, j0);
    // rows_t <= 256: one row per thread, or a loop when the block is narrower.
    const auto row = [&](int t) {
        TabRow R = tab_row(g, tables, r0v, c0v, min(g.win_r0 + J.tile_r + t, g.nr - 1));
        quantize_pair(R.rxh, R.rxl, q, iq);
        quantize_pair(R.ryh, R.ryl, q, iq);
        T.rxh[t] = R.rxh;
        T.rxl[t] = R.rxl;
        T.ryh[t] = R.ryh;
        T.ryl[t] = R.ryl;
        T.dg[t] = R.dg;
        T.psi[t] = R.psi;
    };
    if (THREADS >= kMaxRows) {
        if (tid < rows_t) row(tid);
    } else {
        for (int t = tid; t < rows_t; t += THREADS) row(t);
    }
    if (tid < cols_t) {  // cols_t <= 32
        TabCol C = tab_col(g, tables, r0v, c0v, min(g.win_u0 + J.tile_u + tid, g.nu - 1), j0);
        quantize_pair(C.cxh, C.cxl, q, iq);
        quantize_pair(C.cyh, C.cyl, q, iq);
        T.cxh[tid] = C.cxh;
        T.cxl[tid] = C.cxl;
        T.cyh[tid] = C.cyh;
        T.cyl[tid] = C.cyl;
        T.dcs[tid] = C.dcs;
        T.duu[tid] = C.duu;
    }
    __syncthreads();
}

template <bool HAS_Z>
__device__ void setup_lattice(const Job& J, TileShared& S, Pix px[kPX]) {
    const sarbp_lattice& L = J.lat;
    const int tid = threadIdx.x;
    const int cols_t = 1 << J.lc, rows_t = kSplitTilePixels >> J.lc;
    const int hr = rows_t >> 1, hc = cols_t >> 1;
    if (tid == 0) {
        const double i0 = (double)(J.tile_r + hr), j0 = (double)(J.tile_u + hc);
        S.cx = L.origin[0] + i0 * L.step_row[0] + j0 * L.step_col[0];
        S.cy = L.origin[1] + i0 * L.step_row[1] + j0 * L.step_col[1];
        S.cz = L.origin[2] + i0 * L.step_row[2] + j0 * L.step_col[2];
        double b[3];
        for (int c = 0; c < 3; ++c) b[c] = hr * fabs(L.step_row[c]) + hc * fabs(L.step_col[c]);
        S.rho = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) * 1.0001 + 1e-6;
        for (int c = 0; c < 3; ++c) S.bnd[c] = (float)(b[c] * 1.0001 + 1e-6);
        set_quantum(S, (float)(fmax(b[0], fmax(b[1], b[2])) * 1.0001 + 1e-6), HAS_Z ? 11 : 12);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int p = tid + kThreads * k;
        const double di = (double)((p >> J.lc) - hr), dj = (double)((p & (cols_t - 1)) - hc);
        Pix& q = px[k];
        pixel_from_offsets(S, di * L.step_row[0] + dj * L.step_col[0], di * L.step_row[1] + dj * L.step_col[1],
                           HAS_Z ? di * L.step_row[2] + dj * L.step_col[2] : 0.0, q);
        q.psi = 0.0f;
        q.ar = q.ai = 0.0f;
    }
}

// Lattice tile set-up for the separable pulse loop: the tile centre, bounds and quantum as
// setup_lattice, the steps as two-float, and per pixel only |delta|^2 (FP32).  Thread t holds
// pixels (row (t >> lc) + k m, column t & (cols - 1)), k = 0..3, m = kThreads >> lc.
__device__ void setup_lattice_sep(const Job& J, TileShared& S, float d2[kPX]) {
    const sarbp_lattice& L = J.lat;
    const int tid = threadIdx.x;
    const int cols_t = 1 << J.lc, rows_t = kSplitTilePixels >> J.lc;
    const int hr = rows_t >> 1, hc = cols_t >> 1;
    if (tid == 0) {
        const double i0 = (double)(J.tile_r + hr), j0 = (double)(J.tile_u + hc);
        S.cx = L.origin[0] + i0 * L.step_row[0] + j0 * L.step_col[0];
        S.cy = L.origin[1] + i0 * L.step_row[1] + j0 * L.step_col[1];
        S.cz = L.origin[2] + i0 * L.step_row[2] + j0 * L.step_col[2];
        double b[3];
        for (int c = 0; c < 3; ++c) {
            b[c] = hr * fabs(L.step_row[c]) + hc * fabs(L.step_col[c]);
            split2(L.step_row[c], S.sth[c], S.stl[c]);
            split2(L.step_col[c], S.sth[3 + c], S.stl[3 + c]);
        }
        S.rho = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) * 1.0001 + 1e-6;
        for (int c = 0; c < 3; ++c) S.bnd[c] = (float)(b[c] * 1.0001 + 1e-6);
        const bool has_z = L.step_row[2] != 0.0 || L.step_col[2] != 0.0;
        set_quantum(S, (float)(fmax(b[0], fmax(b[1], b[2])) * 1.0001 + 1e-6), has_z ? 11 : 12);
        S.row_step = kThreads >> J.lc;
    }
    __syncthreads();
    const float dj = (float)((tid & (cols_t - 1)) - hc);
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const float di = (float)(((tid + kThreads * k) >> J.lc) - hr);
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float x = fmaf(di, S.sth[c], dj * S.sth[3 + c]);
            v = fmaf(x, x, v);
        }
        d2[k] = v;
    }
}

__device__ void setup_points(const Job& J, TileShared& S, Pix px[kPX]) {
    const int tid = threadIdx.x;
    double p3[kPX][3];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int idx = J.tile_r + tid + kThreads * k;
        const bool ok = idx < J.npts;
        const int q = ok ? idx : J.tile_r;
        p3[k][0] = J.xyz[3 * q];
        p3[k][1] = J.xyz[3 * q + 1];
        p3[k][2] = J.xyz[3 * q + 2];
        if (ok) {
            v[0] += p3[k][0];
            v[1] += p3[k][1];
            v[2] += p3[k][2];
            v[3] += 1.0;
        }
    }
    block_sum4(S, v);
    const double cx = v[0] / v[3], cy = v[1] / v[3], cz = v[2] / v[3];
    float m[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        m[0] = fmaxf(m[0], (float)fabs(p3[k][0] - cx));
        m[1] = fmaxf(m[1], (float)fabs(p3[k][1] - cy));
        m[2] = fmaxf(m[2], (float)fabs(p3[k][2] - cz));
    }
    block_max<3>(S, m);
    if (tid == 0) {
        S.cx = cx;
        S.cy = cy;
        S.cz = cz;
        const double b0 = m[0] * 1.0001 + 1e-6, b1 = m[1] * 1.0001 + 1e-6, b2 = m[2] * 1.0001 + 1e-6;
        S.rho = sqrt(b0 * b0 + b1 * b1 + b2 * b2);
        S.bnd[0] = (float)b0;
        S.bnd[1] = (float)b1;
        S.bnd[2] = (float)b2;
        set_quantum(S, (float)fmax(b0, fmax(b1, b2)), 11);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        Pix& q = px[k];
        pixel_from_offsets(S, p3[k][0] - cx, p3[k][1] - cy, p3[k][2] - cz, q);
        q.psi = 0.0f;
        q.ar = q.ai = 0.0f;
    }
}

// ---- the pulse loop ---------------------------------------------------------------
template <bool HAS_Z, bool DEMOD>
__device__ __forceinline__ void fast_chunk(const SplitParams& P, const Rec* __restrict__ rec,
                                           const float4* __restrict__ win, int chn, Pix px[kPX]) {
    const float inv_dr = P.inv_drf, Kf = P.Kf;
#pragma unroll 1
    for (int nl = 0; nl < chn; ++nl) {
        const float4 ra = rec[nl].a, rb = rec[nl].b, rc = rec[nl].c;
        float4 rd = make_float4(0.f, 0.f, 0.f, 0.f);
        if (HAS_Z) rd = rec[nl].d;
        const int bias = __float_as_int(rc.y);
        const unsigned last = (unsigned)__float_as_int(rc.w);
        const float4* wrow = win + 2 * __float_as_int(rc.z);
#pragma unroll
        for (int k = 0; k < kPX; ++k) {
            Pix& q = px[k];
            float L = fmaf(rb.x, q.dx, rb.y * q.dy);
            if (HAS_Z) L = fmaf(rd.x, q.dz, L);
            const float q2 = fmaf(-L, L, q.d2);
            const float B = rcp_approx(fmaf(2.0f, L, rb.z));
            const float e0 = q2 * B;
            const float eps = fmaf(-e0 * e0, B, e0);
            const float qp = fmaf(L + eps, inv_dr, rb.w);
            const float tq = qp + kMagic;
            const float s = qp - (tq - kMagic);
            const unsigned j = min((unsigned)(__float_as_int(tq) - bias), last);
            const float4 c01 = wrow[2 * j], c23 = wrow[2 * j + 1];
            const float vr = fmaf(fmaf(fmaf(c23.z, s, c23.x), s, c01.z), s, c01.x);
            const float vi = fmaf(fmaf(fmaf(c23.w, s, c23.y), s, c01.w), s, c01.y);
            float tb = ra.y * q.dyh;
            if (HAS_Z) tb = fmaf(rd.y, q.dzh, tb);
            tb = fmaf(ra.x, q.dxh, tb);
            float sm = fmaf(Kf, eps, rc.x);
            sm = fmaf(ra.x, q.dxl, sm);
            sm = fmaf(ra.y, q.dyl, sm);
            sm = fmaf(ra.z, q.dx, sm);
            sm = fmaf(ra.w, q.dy, sm);
            if (HAS_Z) {
                sm = fmaf(rd.y, q.dzl, sm);
                sm = fmaf(rd.z, q.dz, sm);
            }
            if (DEMOD) sm += q.psi;
            // The reduced large term is in [-1/2, 1/2] turn and |sm| <= 1 + K eps <= 1 + envelope / 2
            // turns (5 turns for direct tiles), so the angle stays within +-40 rad: the hardware
            // sin/cos reduce it themselves with an absolute error below 3e-6 rad, and a second
            // reduction in turns is not needed.
            const float ang = ((tb - round_magic(tb)) + sm) * kTwoPiF;
            float sn, cs;
            __sincosf(ang, &sn, &cs);
            q.ar = fmaf(vr, cs, q.ar);
            q.ar = fmaf(-vi, sn, q.ar);
            q.ai = fmaf(vr, sn, q.ai);
            q.ai = fmaf(vi, cs, q.ai);
        }
    }
}

// fast_chunk for 2-D demodulated tiles (polar grids) with the thread's pixels k = 2h, 2h + 1
// as packed FP32 (f32x2) pairs through the range, fraction, window-index and phase steps; the
// complex cubic evaluates (re, im) as one pair and the accumulation stays scalar.  Every half
// rounds like fast_chunk's scalar operation, and the chain carries -L, -q2, -e0 and -eps
// (negation is exact), so the image is fast_chunk<false, true>'s bit for bit:
//   -L = (-u) . delta,  -q2 = (-L)^2 - d2,  2L + 2R = -2 (-L) + 2R,  -e0 = -q2 B,
//   -eps = (-e0)^2 B + (-e0),  qp = ((-L) + (-eps)) (-1/dr) + Fm,  sm = -K (-eps) + Phi + ...
__device__ __forceinline__ void polar_chunk(const SplitParams& P, const Rec* __restrict__ rec,
                                            const float4* __restrict__ win, int chn, Pix px[kPX]) {
    static_assert(kPX == 4, "two pixel pairs per thread");
    const float2 ninv = pair(-P.inv_drf), nKf = pair(-P.Kf), mone = pair(-1.0f), mtwo = pair(-2.0f);
    const float2 magic = pair(kMagic), nmagic = pair(-kMagic), twopi = pair(kTwoPiF);
#pragma unroll
    for (int k = 0; k < kPX; ++k) px[k].d2 = -px[k].d2;  // carried as -d2 through the chunk
#pragma unroll 1
    for (int nl = 0; nl < chn; ++nl) {
        const float4 ra = rec[nl].a, rb = rec[nl].b, rc = rec[nl].c;
        const int bias = __float_as_int(rc.y);
        const unsigned last = (unsigned)__float_as_int(rc.w);
        const float4* wrow = win + 2 * __float_as_int(rc.z);
        const float2 nux = pair(-rb.x), nuy = pair(-rb.y), twoR = pair(rb.z), fm = pair(rb.w);
        const float2 Wx = pair(ra.x), Wy = pair(ra.y), Wlx = pair(ra.z), Wly = pair(ra.w), phi = pair(rc.x);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const Pix &pa = px[2 * h], &pb = px[2 * h + 1];
            const float2 dx = make_float2(pa.dx, pb.dx), dy = make_float2(pa.dy, pb.dy);
            const float2 nL = __ffma2_rn(nux, dx, __fmul2_rn(nuy, dy));
            const float2 nq2 = __ffma2_rn(nL, nL, make_float2(pa.d2, pb.d2));
            const float2 den = __ffma2_rn(mtwo, nL, twoR);
            const float2 B = make_float2(rcp_approx(den.x), rcp_approx(den.y));
            const float2 ne0 = __fmul2_rn(nq2, B);
            const float2 neps = __ffma2_rn(__fmul2_rn(ne0, ne0), B, ne0);
            const float2 qp = __ffma2_rn(__fadd2_rn(nL, neps), ninv, fm);
            const float2 tq = __fadd2_rn(qp, magic);
            const float2 sv = __ffma2_rn(__fadd2_rn(tq, nmagic), mone, qp);
            const float2 tb = __ffma2_rn(Wx, make_float2(pa.dxh, pb.dxh), __fmul2_rn(Wy, make_float2(pa.dyh, pb.dyh)));
            float2 sm = __ffma2_rn(nKf, neps, phi);
            sm = __ffma2_rn(Wx, make_float2(pa.dxl, pb.dxl), sm);
            sm = __ffma2_rn(Wy, make_float2(pa.dyl, pb.dyl), sm);
            sm = __ffma2_rn(Wlx, dx, sm);
            sm = __ffma2_rn(Wly, dy, sm);
            sm = __fadd2_rn(sm, make_float2(pa.psi, pb.psi));
            // The reduced large term is in [-1/2, 1/2] turn and |sm| <= 1 + K eps <= 1 + envelope / 2
            // turns, so the angle stays within +-40 rad, which the hardware sin/cos reduce themselves.
            const float2 rtb = __fadd2_rn(__fadd2_rn(tb, magic), nmagic);
            const float2 ang = __fmul2_rn(__fadd2_rn(__ffma2_rn(rtb, mone, tb), sm), twopi);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                Pix& q = px[2 * h + c];
                const unsigned j = min((unsigned)(__float_as_int(c ? tq.y : tq.x) - bias), last);
                const float4 c01 = wrow[2 * j], c23 = wrow[2 * j + 1];
                const float2 ss = pair(c ? sv.y : sv.x);
                const float2 v = __ffma2_rn(
                    __ffma2_rn(__ffma2_rn(make_float2(c23.z, c23.w), ss, make_float2(c23.x, c23.y)), ss,
                               make_float2(c01.z, c01.w)),
                    ss, make_float2(c01.x, c01.y));
                float sn, cs;
                __sincosf(c ? ang.y : ang.x, &sn, &cs);
                q.ar = fmaf(v.x, cs, q.ar);
                q.ar = fmaf(-v.y, sn, q.ar);
                q.ai = fmaf(v.x, sn, q.ai);
                q.ai = fmaf(v.y, cs, q.ai);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kPX; ++k) px[k].d2 = -px[k].d2;
}

// ---- two-float arithmetic (unevaluated sums hi + lo of two FP32 numbers) ----------------
//
// Error-free transformations (Knuth's two-sum, the FMA form of Dekker's product) give about
// 44 significant bits in FP32 arithmetic, which runs at full rate where GB300's FP64 does not.
// They carry pulses that fall outside the split path's precision envelope.
struct FF {
    float h, l;
};

__device__ __forceinline__ FF ff_norm(float s, float e) {  // |s| >= |e|
    const float h = s + e;
    return FF{h, e - (h - s)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb);
    return ff_norm(s, e + (a.l + b.l));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p);
    return ff_norm(p, fmaf(a.h, b.l, fmaf(a.l, b.h, e)));
}
__device__ __forceinline__ FF ff_sqr(FF a) {
    const float p = a.h * a.h;
    const float e = fmaf(a.h, a.h, -p);
    return ff_norm(p, fmaf(2.0f * a.h, a.l, e));
}
// sqrt by one Newton step on the FP32 root: s + (a - s^2) / (2 s).
__device__ __forceinline__ FF ff_sqrt(FF a) {
    const float s = __fsqrt_rn(a.h);
    const float p = s * s;
    const float e = fmaf(s, s, -p);
    const float r = ((a.h - p) - e) + a.l;
    return ff_norm(s, r * (0.5f / s));
}
__device__ __forceinline__ FF ff_of(float2 v) { return FF{v.x, v.y}; }
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.h, -a.l}; }
// 1/a: the FP32 reciprocal refined by one Newton step in two-float.
__device__ __forceinline__ FF ff_rcp(FF a) {
    const float i0 = __frcp_rn(a.h);
    const FF e = ff_mul(a, FF{i0, 0.0f});
    return ff_norm(i0, i0 * ((1.0f - e.h) - e.l));
}
// Splits a two-float value q into floor and centred fraction: q = I + F + 1/2, F in [-1/2, 1/2).
__device__ __forceinline__ float ff_floor_frac(FF q, float& F) {
    float I = floorf(q.h);
    float f = (q.h - I) + q.l;  // q.h - I is exact
    if (f < 0.0f) {
        f += 1.0f;
        I -= 1.0f;
    } else if (f >= 1.0f) {
        f -= 1.0f;
        I += 1.0f;
    }
    F = f - 0.5f;
    return I;
}


// Per (tile, pulse) data of a pulse the fast path cannot stage: the FP64 vector from the
// antenna to the tile centre as two-float components, the pulse phase in turns, the weight.
struct SlowRec {
    float4 a;  // w.x hi, w.x lo, w.y hi, w.y lo
    float4 b;  // w.z hi, w.z lo, phase / 2pi reduced to [-1/2, 1/2], weight
};

// Sum over pulses [c0, c0 + n) of one pixel's contributions in two-float geometry.  Out of
// line (and the pixel by value) so that the rarely taken fallback does not add registers
// to the kernels' fast path.
__device__ __noinline__ float2 slow_pixel(const SplitParams& P, const SlowRec* srec, int n, int c0, float dxh,
                                          float dxl, float dyh, float dyl, float dzh, float dzl, float psi);

// Dynamic shared memory of the chunk kernels: [records | windows]; the two-float records of
// a chunk that stages no window live at the start of the window space.
__host__ __device__ constexpr size_t window_offset() { return (size_t)kMaxChunk * sizeof(Rec); }

// Range-sample value and its derivative for a pixel at offset delta from the tile centre,
// pulse record sr, in two-float geometry: returns false when the taps leave the row.
struct SlowSample {
    float vr, vi, dvr, dvi;  // sample1 value and d/dq
    float ang;               // phase (radians, reduced)
    float ex, ey, ez;        // unit vector pulse -> pixel
    float d;                 // range (m, FP32)
};

template <bool DERIV>
__device__ __forceinline__ bool slow_sample(const SplitParams& P, const SlowRec& sr, const float2* __restrict__ row,
                                            const Pix& q, float psi, SlowSample& o) {
    const FF vx = ff_add(FF{sr.a.x, sr.a.y}, FF{q.dxh, q.dxl});
    const FF vy = ff_add(FF{sr.a.z, sr.a.w}, FF{q.dyh, q.dyl});
    const FF vz = ff_add(FF{sr.b.x, sr.b.y}, FF{q.dzh, q.dzl});
    const FF d = ff_sqrt(ff_add(ff_add(ff_sqr(vx), ff_sqr(vy)), ff_sqr(vz)));
    const FF t = ff_mul(FF{P.Kh, P.Kl}, d);
    float tot = ((t.h - rintf(t.h)) + t.l) + (sr.b.z + psi);
    tot -= rintf(tot);
    o.ang = tot * kTwoPiF;
    const FF qq = ff_mul(ff_add(d, FF{-P.rsh, -P.rsl}), FF{P.idrh, P.idrl});
    float fl = floorf(qq.h);
    float f = (qq.h - fl) + qq.l;
    if (f < 0.0f) {
        f += 1.0f;
        fl -= 1.0f;
    } else if (f >= 1.0f) {
        f -= 1.0f;
        fl += 1.0f;
    }
    if (!(fl >= 1.0f && fl <= (float)(P.in.samples - 3))) return false;
    const int i = (int)fl;
    const float2 x0 = __ldg(row + i - 1), x1 = __ldg(row + i), x2 = __ldg(row + i + 1), x3 = __ldg(row + i + 2);
    float4 c01, c23;
    cubic_coefficients(x0, x1, x2, x3, 1.0f, c01, c23);
    const float s = f - 0.5f;
    o.vr = fmaf(fmaf(fmaf(c23.z, s, c23.x), s, c01.z), s, c01.x);
    o.vi = fmaf(fmaf(fmaf(c23.w, s, c23.y), s, c01.w), s, c01.y);
    if (DERIV) {
        o.dvr = fmaf(fmaf(3.0f * c23.z, s, 2.0f * c23.x), s, c01.z);
        o.dvi = fmaf(fmaf(3.0f * c23.w, s, 2.0f * c23.y), s, c01.w);
        const float inv = 1.0f / d.h;
        o.ex = (vx.h + vx.l) * inv;
        o.ey = (vy.h + vy.l) * inv;
        o.ez = (vz.h + vz.l) * inv;
        o.d = d.h;
    }
    return true;
}


// Two-float record of a pulse the fast path cannot stage (out of line: it is rare, and its
// FP64 temporaries would otherwise add to the registers of every chunk kernel).
__device__ __noinline__ void slow_record(const SplitParams& P, const TileShared& S, int n, SlowRec* out) {
    const PulseInputs& in = P.in;
    SlowRec sr;
    split2(S.cx - in.pos[3 * n], sr.a.x, sr.a.y);
    split2(S.cy - in.pos[3 * n + 1], sr.a.z, sr.a.w);
    split2(S.cz - in.pos[3 * n + 2], sr.b.x, sr.b.y);
    const double ph = in.phase[n] * kInvTwoPi;
    sr.b.z = (float)(ph - rint(ph));
    sr.b.w = (float)in.weight[n];
    *out = sr;
}

// Per (tile, pulse) record, computed by lane `lane` of the record warps in two-float FP32
// arithmetic (about 44 bits; GB300's FP64 rate would make these records the barrier-bound
// part of every chunk).  Returns the number of window entries the pulse needs (cap + 1 if
// it cannot be staged).
// MODE 0: per-pixel offsets (polar, points); 1: lattice tiles; 2: lattice tiles, adjoint.
template <int MODE>
__device__ __forceinline__ int make_record(const SplitParams& P, TileShared& S, Rec* rec, int lane, int n) {
    const PulseInputs& in = P.in;
    float ph_, pl_;
    split2(in.pos[3 * n], ph_, pl_);
    const FF vx = ff_add(FF{S.ch[0], S.cl[0]}, FF{-ph_, -pl_});
    split2(in.pos[3 * n + 1], ph_, pl_);
    const FF vy = ff_add(FF{S.ch[1], S.cl[1]}, FF{-ph_, -pl_});
    split2(in.pos[3 * n + 2], ph_, pl_);
    const FF vz = ff_add(FF{S.ch[2], S.cl[2]}, FF{-ph_, -pl_});
    const FF R = ff_sqrt(ff_add(ff_add(ff_sqr(vx), ff_sqr(vy)), ff_sqr(vz)));
    // 1/R: the FP32 reciprocal refined by one Newton step in two-float.
    const float i0 = __frcp_rn(R.h);
    const FF e = ff_mul(R, FF{i0, 0.0f});
    const FF iR = ff_norm(i0, i0 * ((1.0f - e.h) - e.l));
    const FF ux = ff_mul(vx, iR), uy = ff_mul(vy, iR), uz = ff_mul(vz, iR);
    const FF Kk{P.Kh, P.Kl};
    const FF t = ff_mul(Kk, R);
    const double ph = in.phase[n] * kInvTwoPi;
    float t1 = ((t.h - rintf(t.h)) + t.l) + (float)(ph - rint(ph));
    t1 -= rintf(t1);
    const FF Q = ff_mul(ff_add(R, FF{-P.rsh, -P.rsl}), FF{P.idrh, P.idrl});
    float I = floorf(Q.h);
    float fq = (Q.h - I) + Q.l;
    if (fq < 0.0f) {
        fq += 1.0f;
        I -= 1.0f;
    } else if (fq >= 1.0f) {
        fq -= 1.0f;
        I += 1.0f;
    }
    const float Fm = fq - 0.5f;
    const float Rf = R.h, uxf = ux.h + ux.l, uyf = uy.h + uy.l, uzf = uz.h + uz.l;
    // |L| <= sum_c |u_c| bound_c and 0 <= eps <= rho^2 / (2 (R - rho)), in bins.
    const float lin = fabsf(uxf) * S.bnd[0] + fabsf(uyf) * S.bnd[1] + fabsf(uzf) * S.bnd[2];
    const float eps = S.rhof * S.rhof / (2.0f * fmaxf(Rf - S.rhof, 1.0f));
    const float hw = (lin + eps) * fabsf(P.inv_drf) + 1e-3f;
    const float lo = floorf(Fm - hw), hi = ceilf(Fm + hw);
    const bool ok = Rf > 0.0f && fabsf(Q.h) < 1.0e7f && hi - lo + 1.0f <= (float)P.cap &&
                    fabsf(P.Kf) * S.rhof * S.rhof <= (float)P.envelope * Rf && S.rhof < 0.25f * Rf;
    const int bo = ok ? (int)lo : 0;
    S.base[lane] = ok ? (int)I + bo : 0;
    S.wt[lane] = (float)in.weight[n];
    Rec r;
    const FF Wx = ff_mul(Kk, ux), Wy = ff_mul(Kk, uy), Wz = ff_mul(Kk, uz);
    if (MODE != 0) {
        // Lattice tile: the linear phase W . delta of pixel (i, j) is i B_row + j B_col with
        // B = W . step.  Both are split on one power-of-two quantum with <= 10 significant
        // bits, so i B_row_hi + j B_col_hi is exact in FP32 for |i|, |j| < 2^12.
        const FF Br = ff_add(ff_add(ff_mul(Wx, FF{S.sth[0], S.stl[0]}), ff_mul(Wy, FF{S.sth[1], S.stl[1]})),
                             ff_mul(Wz, FF{S.sth[2], S.stl[2]}));
        const FF Bc = ff_add(ff_add(ff_mul(Wx, FF{S.sth[3], S.stl[3]}), ff_mul(Wy, FF{S.sth[4], S.stl[4]})),
                             ff_mul(Wz, FF{S.sth[5], S.stl[5]}));
        const int e = ((__float_as_int(fmaxf(fmaxf(fabsf(Br.h), fabsf(Bc.h)), 1e-30f)) >> 23) & 0xff) - 126;
        const float q = __int_as_float((e - 10 + 127) << 23), iq = __int_as_float((10 - e + 127) << 23);
        r.a.x = rintf(Br.h * iq) * q;
        r.a.y = (Br.h - r.a.x) + Br.l;
        r.a.z = rintf(Bc.h * iq) * q;
        r.a.w = (Bc.h - r.a.z) + Bc.l;
        // Phase and range steps between a thread's successive pixels (m = kThreads >> lc rows).
        const float m = (float)S.row_step;
        const float mh = m * Br.h;  // exact: m is a power of two
        float sp = (mh - rintf(mh)) + m * Br.l;
        sp -= rintf(sp);
        const float Ar = fmaf(uxf, S.sth[0], fmaf(uyf, S.sth[1], uzf * S.sth[2]));
        const float Ac = fmaf(uxf, S.sth[3], fmaf(uyf, S.sth[4], uzf * S.sth[5]));
        r.b = make_float4(Ar, Ac, 2.0f * Rf, Fm);
        // The phase step in radians; the range step (forward) or u (adjoint).
        // The forward holds its per-pulse operands as float2 pairs: (phase step, phase step),
        // (-range step, -range step) in d and (2R, 2R), (Fm, Fm) in e.
        const float spr = sp * kTwoPiF, nstep = -(m * Ar);
        r.d = MODE == 1 ? make_float4(spr, spr, nstep, nstep) : make_float4(spr, uxf, uyf, uzf);
        r.e = make_float4(2.0f * Rf, 2.0f * Rf, Fm, Fm);
    } else {
        const float sw = (float)P.scale_w, isw = (float)P.inv_scale_w;  // powers of two: exact
        r.a.x = rintf(Wx.h * isw) * sw;
        r.a.z = (Wx.h - r.a.x) + Wx.l;
        r.a.y = rintf(Wy.h * isw) * sw;
        r.a.w = (Wy.h - r.a.y) + Wy.l;
        r.d.y = rintf(Wz.h * isw) * sw;
        r.d.z = (Wz.h - r.d.y) + Wz.l;
        r.b = make_float4(uxf, uyf, 2.0f * Rf, Fm);
        r.d.x = uzf;
        r.d.w = 0.0f;
        r.e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    r.c.x = t1;
    r.c.y = __int_as_float(kMagicBits + bo);
    const int count = ok ? (int)(hi - lo) + 1 : P.cap + 1;
    r.c.z = 0.0f;
    r.c.w = __int_as_float(count - 1);
    rec[lane] = r;
    return count;
}

__device__ __noinline__ float2 slow_pixel(const SplitParams& P, const SlowRec* srec, int n, int c0, float dxh,
                                          float dxl, float dyh, float dyl, float dzh, float dzl, float psi) {
    Pix q;
    q.dxh = dxh;
    q.dxl = dxl;
    q.dyh = dyh;
    q.dyl = dyl;
    q.dzh = dzh;
    q.dzl = dzl;
    float ar = 0.0f, ai = 0.0f;
    for (int j = 0; j < n; ++j) {
        const SlowRec sr = srec[j];
        SlowSample o;
        if (!slow_sample<false>(P, sr, P.in.data + (size_t)(c0 + j) * P.in.samples, q, psi, o)) continue;
        float sn, cs;
        __sincosf(o.ang, &sn, &cs);
        const float a = sr.b.w;
        ar = fmaf(a * o.vr, cs, fmaf(-a * o.vi, sn, ar));
        ai = fmaf(a * o.vr, sn, fmaf(a * o.vi, cs, ai));
    }
    return make_float2(ar, ai);
}

__device__ int g_wait_timeouts;  // bounded waits on asynchronous copies that ran out

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `phase` of the mbarrier at shared address bar, for at most limit_ns of the GPU's
// timer (and at most 2^24 polls); true once the phase completed.
__device__ __forceinline__ bool timed_wait(unsigned bar, unsigned phase, unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    for (int it = 0; it < (1 << 24); ++it) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Bounded wait for the phase `phase` of the mbarrier at shared address bar; true once it completed.
__device__ __forceinline__ bool bulk_wait(unsigned bar, unsigned phase) {
    unsigned done = 0;
    for (int it = 0; it < (1 << 22) && !done; ++it)
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
    return done != 0;
}

#if SARBP_BULK_WINDOWS
// Raw samples [b - 1, b + cnt + 2) of each fitting pulse's row (clipped to the row) arrive in
// shared memory by one 1-D cp.async.bulk copy per pulse, issued by warp 0 after lane 0 has set
// the transaction count on the mbarrier; every thread waits for the phase (a bounded wait that
// records a timeout), then the Horner transform reads shared memory.  A copy must start and end
// on 16-byte boundaries of the data array, so the copied range is widened to even elements.
// Returns false (the same in every thread) if the copies did not arrive within the bounded wait;
// the caller then stops staging and waits once more before leaving.
__device__ __forceinline__ bool bulk_stage_windows(const SplitParams& P, TileShared& S, const Rec* rec, float4* win,
                                                   float2* raw, unsigned long long& mbar, unsigned phase, int c0,
                                                   int nfit, bool weighted) {
    const PulseInputs& in = P.in;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bar = (unsigned)__cvta_generic_to_shared(&mbar);
    if (warp == 0) {
        long long a0[2];
        int len[2];
        int mine = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int nl = lane + 32 * h;
            a0[h] = 0;
            len[h] = 0;
            if (nl < nfit) {
                const long long row0 = (long long)(c0 + nl) * in.samples;
                const long long b0 = S.base[nl];
                const int cnt = __float_as_int(rec[nl].c.w) + 1;
                // [g0, g1) within the row; rows start on even elements (samples is even), so
                // widening to even bounds stays inside the row.
                const long long g0 = min(max(b0 - 1, 0ll), (long long)in.samples);
                const long long g1 = max(min(b0 + cnt + 2, (long long)in.samples), g0);
                const long long e0 = (row0 + g0) & ~1ll, e1 = (row0 + g1 + 1) & ~1ll;
                a0[h] = e0;
                len[h] = (int)max(e1 - e0, 0ll);
                mine += len[h];
            }
        }
        // Exclusive prefix of the raw lengths (even, so every destination stays 16-byte aligned).
        int inc = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        const int total = __shfl_sync(0xffffffffu, inc, 31);
        int off = inc - mine;
        if (lane == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(total * 8)
                         : "memory");
        }
        __syncwarp();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the last chunk's reads precede these writes
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int nl = lane + 32 * h;
            if (nl < nfit) {
                S.roff[nl] = off;
                S.raw0[nl] = a0[h];
                if (len[h] > 0) {
                    const unsigned dst = (unsigned)__cvta_generic_to_shared(raw + off);
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            dst),
                        "l"(in.data + a0[h]), "r"(len[h] * 8), "r"(bar)
                        : "memory");
                }
                off += len[h];
            }
        }
    }
    // Bounded wait for the copies of this chunk's phase.
    const bool done = __syncthreads_and(bulk_wait(bar, phase)) != 0;  // also orders roff / raw0 of warp 0
    if (!done) {
        if (threadIdx.x == 0) atomicAdd(&g_wait_timeouts, 1);
        return false;
    }
    for (int nl = warp; nl < nfit; nl += kThreads / 32) {
        const int woff = __float_as_int(rec[nl].c.z);
        const int cnt = __float_as_int(rec[nl].c.w) + 1;
        const long long b0 = S.base[nl];
        const float a = weighted ? S.wt[nl] : 1.0f;
        const float2* r = raw + S.roff[nl] + ((long long)(c0 + nl) * in.samples - S.raw0[nl]);  // row-relative
        for (int j = lane; j < cnt; j += 32) {
            const long long g = b0 + j;
            float4 c01 = make_float4(0.f, 0.f, 0.f, 0.f), c23 = c01;
            if (g >= 1 && g <= (long long)in.samples - 3)
                cubic_coefficients(r[g - 1], r[g], r[g + 1], r[g + 2], a, c01, c23);
            win[2 * (woff + j)] = c01;
            win[2 * (woff + j) + 1] = c23;
        }
    }
    return true;
}
#endif

// Horner windows of one pulse (cnt entries from bin b0) staged by one warp with one global load
// per lane and step: lane l loads sample b0 + j0 + l - 1, and entry j0 + l (l < 29) takes its four
// taps from lanes l .. l + 3 by shuffles (the FFBP leaves and polar-grid direct BP).
__device__ __forceinline__ void stage_window_shfl(const float2* __restrict__ row, long long samples, long long b0,
                                                  int cnt, float a, float4* __restrict__ wentry, int lane) {
    for (int j0 = 0; j0 < cnt; j0 += 29) {
        const long long gi = b0 + j0 + lane - 1;
        float2 x = make_float2(0.0f, 0.0f);
        if (gi >= 0 && gi < samples) x = __ldg(row + gi);
        float2 x1, x2, x3;
        x1.x = __shfl_down_sync(0xffffffffu, x.x, 1);
        x1.y = __shfl_down_sync(0xffffffffu, x.y, 1);
        x2.x = __shfl_down_sync(0xffffffffu, x.x, 2);
        x2.y = __shfl_down_sync(0xffffffffu, x.y, 2);
        x3.x = __shfl_down_sync(0xffffffffu, x.x, 3);
        x3.y = __shfl_down_sync(0xffffffffu, x.y, 3);
        const int j = j0 + lane;
        if (lane < 29 && j < cnt) {
            const long long g = b0 + j;
            float4 c01 = make_float4(0.f, 0.f, 0.f, 0.f), c23 = c01;
            if (g >= 1 && g <= samples - 3) cubic_coefficients(x, x1, x2, x3, a, c01, c23);
            wentry[2 * j] = c01;
            wentry[2 * j + 1] = c23;
        }
    }
}

// Chunk driver shared by the forward and adjoint kernels: per chunk of up to 64
// pulses, warps 0 and 1 compute the (tile, pulse) records (one pulse per lane, two-float,
// on two SM sub-partitions at once) and pack the pulses' range windows, all warps
// stage the windows (Horner coefficients, times the pulse weight when `weighted`),
// then `body.fast(rec, win, nfit, c0)` consumes them; a pulse whose window cannot be
// staged goes through `body.slow(c0, n, slow)` with its two-float record.
template <class Body>
__device__ void chunk_loop(const SplitParams& P, const Job& J, TileShared& S, char* smem, bool weighted, Body& body) {
    const PulseInputs& in = P.in;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Rec* rec = reinterpret_cast<Rec*>(smem);
    float4* win = reinterpret_cast<float4*>(smem + window_offset());
    SlowRec* slow = reinterpret_cast<SlowRec*>(win);  // a chunk that stages nothing reuses the window space
#if SARBP_BULK_WINDOWS
    float2* raw = reinterpret_cast<float2*>(smem + window_offset() + (size_t)P.cap * 32);
    __shared__ __align__(8) unsigned long long mbar;
    unsigned phase = 0;
    // Bulk copies need 16-byte aligned rows: an even sample count on a 16-byte aligned array.
    const bool bulk = ((reinterpret_cast<uintptr_t>(in.data) & 15) == 0) && (in.samples % 2 == 0);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((unsigned)__cvta_generic_to_shared(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
#endif
    if (threadIdx.x == 0) {  // the tile centre as two-float for the records (ordered by the loop's barrier)
        split2(S.cx, S.ch[0], S.cl[0]);
        split2(S.cy, S.ch[1], S.cl[1]);
        split2(S.cz, S.ch[2], S.cl[2]);
        S.rhof = (float)S.rho;
    }
    for (int c0 = J.p0; c0 < J.p1;) {
        const int want = min(P.chunk, J.p1 - c0);
        __syncthreads();  // the previous chunk's records and windows are consumed
        if (warp < 2) {
            const int idx = 32 * warp + lane;
            const int count = idx < want ? make_record<Body::kRecMode>(P, S, rec, idx, c0 + idx) : 0;
            int inc = count;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (warp == 0 && lane == 31) S.wsum = inc;
            asm volatile("bar.sync 2, 64;" ::: "memory");  // warps 0 and 1 only
            if (warp == 1) inc += S.wsum;
            // Counts are >= 1, so the pulses that fit form a prefix of the chunk.
            const unsigned fits = __ballot_sync(0xffffffffu, idx < want && inc <= P.cap);
            if (idx < want) rec[idx].c.z = __int_as_float(inc - count);
            if (lane == 0) S.nfit_w[warp] = __popc(fits);
        }
        __syncthreads();
        const int nfit = S.nfit_w[0] + S.nfit_w[1];
        if (nfit > 0) {
#if SARBP_BULK_WINDOWS
            if (bulk) {
                if (!bulk_stage_windows(P, S, rec, win, raw, mbar, phase, c0, nfit, weighted)) {
                    // The copies did not arrive: the tile's image is invalid (g_wait_timeouts counts it).
                    // Wait once more, bounded, for the copies still in flight, then leave.
                    bulk_wait((unsigned)__cvta_generic_to_shared(&mbar), phase);
                    break;
                }
                phase ^= 1u;
            } else
#endif
            for (int nl = warp; nl < nfit; nl += kThreads / 32) {
                const int off = __float_as_int(rec[nl].c.z);
                const int cnt = __float_as_int(rec[nl].c.w) + 1;
                const long long b0 = S.base[nl];
                const float a = weighted ? S.wt[nl] : 1.0f;
                const float2* row = in.data + (size_t)(c0 + nl) * in.samples;
                if (Body::kShflWindows) {
                    stage_window_shfl(row, in.samples, b0, cnt, a, win + 2 * off, lane);
                    continue;
                }
                for (int j = lane; j < cnt; j += 32) {
                    const long long g = b0 + j;
                    float4 c01 = make_float4(0.f, 0.f, 0.f, 0.f), c23 = c01;
                    if (g >= 1 && g <= (long long)in.samples - 3)
                        cubic_coefficients(__ldg(row + g - 1), __ldg(row + g), __ldg(row + g + 1), __ldg(row + g + 2),
                                           a, c01, c23);
                    win[2 * (off + j)] = c01;
                    win[2 * (off + j) + 1] = c23;
                }
            }
            __syncthreads();
            body.fast(rec, win, nfit, c0);
            c0 += nfit;
        } else {
            // The leading pulses that cannot be staged (outside the precision envelope or with
            // windows too wide): two-float geometry per pixel, [c0, c0 + nslow).
            // (the records mark them with a window count of cap + 1)
            if (warp < 2) {
                const int idx = 32 * warp + lane;
                const unsigned misses =
                    __ballot_sync(0xffffffffu, idx < want && __float_as_int(rec[idx].c.w) + 1 > P.cap);
                if (lane == 0) S.miss_w[warp] = misses;
            }
            __syncthreads();
            const unsigned long long m = (unsigned long long)S.miss_w[0] | ((unsigned long long)S.miss_w[1] << 32);
            const int nslow = ~m == 0ull ? kMaxChunk : __ffsll((long long)~m) - 1;
            if (threadIdx.x < nslow) slow_record(P, S, c0 + threadIdx.x, slow + threadIdx.x);
            __syncthreads();
            body.slow(c0, nslow, slow);
            c0 += nslow;
        }
    }
#if SARBP_BULK_WINDOWS
    __syncthreads();  // every wait on the barrier is over: it can be invalidated (and initialised again)
    if (threadIdx.x == 0)
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"((unsigned)__cvta_generic_to_shared(&mbar)) : "memory");
#endif
}

template <bool HAS_Z, bool DEMOD>
struct ForwardBody {
    static constexpr int kRecMode = 0;
    // Polar grids stage their windows with one load per lane and shuffled neighbours (751 against
    // 744 Gpixel-pulses/s on the 4096-pulse root grid); the lattice loop measured 0.5% slower with it.
    static constexpr bool kShflWindows = !HAS_Z && DEMOD;
    const SplitParams& P;
    const TileShared& S;
    Pix* px;
    __device__ void fast(const Rec* rec, const float4* win, int nfit, int) {
        if (!HAS_Z && DEMOD)
            polar_chunk(P, rec, win, nfit, px);
        else
            fast_chunk<HAS_Z, DEMOD>(P, rec, win, nfit, px);
    }
    __device__ void slow(int c0, int nslow, const SlowRec* srec) {
#pragma unroll
        for (int k = 0; k < kPX; ++k) {
            const Pix& q = px[k];
            const float2 v = slow_pixel(P, srec, nslow, c0, q.dxh, q.dxl, q.dyh, q.dyl, q.dzh, q.dzl,
                                        DEMOD ? q.psi : 0.0f);
            px[k].ar += v.x;
            px[k].ai += v.y;
        }
    }
};

template <bool HAS_Z, bool DEMOD>
__device__ void pulse_loop(const SplitParams& P, const Job& J, TileShared& S, char* smem, Pix px[kPX]) {
    ForwardBody<HAS_Z, DEMOD> body{P, S, px};
    chunk_loop(P, J, S, smem, true, body);
}

// ---- lattice tiles: separable pulse loop ------------------------------------------------
//
// On a lattice the pixel offset is delta = i s_row + j s_col, so u . delta and W . delta
// split into row and column terms.  Per (thread, pulse) the record gives the terms at the
// thread's reference pixel (row (t >> lc) + 2m, its column): L0 = u . delta, and the phase
// r0 = frac(Phi + W . delta) from the exact hi products; its other pixels are kc = -2..1
// steps of m rows away, L = L0 + kc (m u . s_row) and phase r0 + kc frac(m W . s_row).
// Per pixel-pulse this leaves the eps term, the window gather and the rotation.

// The forward's per-pixel geometry runs on packed FP32 (f32x2): pixels k = 2h and 2h + 1 of
// a thread form one float2 lane pair through the range, fraction, index and angle steps, so
// one instruction issues both pixels' operation.  Each half rounds exactly like the scalar
// operation, and the chain is carried with the sign of L, q2, e0 and eps flipped (negation
// is exact, so every value equals the scalar formulation's bit for bit):
//   -L = kc (-m u.s_row) + (-L0),  -q2 = (-L)^2 - d2,  2L + 2R = -2 (-L) + 2R,
//   -e0 = -q2 B,  -eps = (-e0)^2 B + (-e0),  qp = ((-L) + (-eps)) (-1/dr) + Fm,
//   s = qp - (tq - M) = (tq - M) (-1) + qp,  ang = (-kr) (-eps) + (kc sp + r0).
// The complex cubic evaluates (re, im) as one pair; the accumulation stays scalar.
__device__ __forceinline__ void lattice_chunk(const SplitParams& P, const Rec* __restrict__ rec,
                                              const float4* __restrict__ win, int chn, int lc, const float d2[kPX],
                                              float ar[kPX], float ai[kPX]) {
    static_assert(kPX == 4, "two pixel pairs per thread");
    const float inv_dr = P.inv_drf, kr = P.Kf * kTwoPiF;
    const int m = kThreads >> lc, hr = (kSplitTilePixels >> lc) >> 1, cols_t = 1 << lc;
    const int tid = threadIdx.x;
    const float di = (float)((tid >> lc) + 2 * m - hr);
    const float dj = (float)((tid & (cols_t - 1)) - (cols_t >> 1));
    const float2 nd2[2] = {make_float2(-d2[0], -d2[1]), make_float2(-d2[2], -d2[3])};
    const float2 kcs[2] = {make_float2(-2.0f, -1.0f), make_float2(0.0f, 1.0f)};
    const float2 ninv = pair(-inv_dr), nkr = pair(-kr), magic = pair(kMagic), nmagic = pair(-kMagic);
    const float2 mone = pair(-1.0f), mtwo = pair(-2.0f);
#pragma unroll 1
    for (int nl = 0; nl < chn; ++nl) {
        const float4 ra = rec[nl].a, rb = rec[nl].b, rc = rec[nl].c, rd = rec[nl].d, re = rec[nl].e;
        const int bias = __float_as_int(rc.y);
        const unsigned last = (unsigned)__float_as_int(rc.w);
        const float4* wrow = win + 2 * __float_as_int(rc.z);
        const float nL0 = fmaf(-dj, rb.y, -di * rb.x);  // -L0, exactly
        const float t = fmaf(dj, ra.z, di * ra.x);       // exact
        const float r0 = ((t - round_magic(t)) + fmaf(dj, ra.w, fmaf(di, ra.y, rc.x))) * kTwoPiF;  // radians
        const float2 sp = make_float2(rd.x, rd.y), nstep = make_float2(rd.z, rd.w);
        const float2 twoR = make_float2(re.x, re.y), fm = make_float2(re.z, re.w);
        const float2 nL02 = pair(nL0), r02 = pair(r0);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2 nL = __ffma2_rn(kcs[h], nstep, nL02);
            const float2 nq2 = __ffma2_rn(nL, nL, nd2[h]);
            const float2 den = __ffma2_rn(mtwo, nL, twoR);
            const float2 B = make_float2(rcp_approx(den.x), rcp_approx(den.y));
            const float2 ne0 = __fmul2_rn(nq2, B);
            const float2 neps = __ffma2_rn(__fmul2_rn(ne0, ne0), B, ne0);
            const float2 qp = __ffma2_rn(__fadd2_rn(nL, neps), ninv, fm);
            const float2 tq = __fadd2_rn(qp, magic);
            const float2 s = __ffma2_rn(__fadd2_rn(tq, nmagic), mone, qp);
            // |r0| <= 1/2 + small, |kc frac| <= 1 and K eps <= envelope / 2 turns: the angle
            // stays within +-40 rad, which the hardware sin/cos reduce themselves.
            const float2 ang = __ffma2_rn(nkr, neps, __ffma2_rn(kcs[h], sp, r02));
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int k = 2 * h + c;
                const float tqc = c ? tq.y : tq.x, sc = c ? s.y : s.x;
                const unsigned j = min((unsigned)(__float_as_int(tqc) - bias), last);
                const float4 c01 = wrow[2 * j], c23 = wrow[2 * j + 1];
                const float2 ss = pair(sc);
                const float2 v = __ffma2_rn(
                    __ffma2_rn(__ffma2_rn(make_float2(c23.z, c23.w), ss, make_float2(c23.x, c23.y)), ss,
                               make_float2(c01.z, c01.w)),
                    ss, make_float2(c01.x, c01.y));
                float sn, cs;
                __sincosf(c ? ang.y : ang.x, &sn, &cs);
                ar[k] = fmaf(v.x, cs, ar[k]);
                ar[k] = fmaf(-v.y, sn, ar[k]);
                ai[k] = fmaf(v.x, sn, ai[k]);
                ai[k] = fmaf(v.y, cs, ai[k]);
            }
        }
    }
}

struct LatticeBody {
    static constexpr int kRecMode = 1;
    static constexpr bool kShflWindows = false;
    const SplitParams& P;
    const TileShared& S;
    const Job& J;
    const float* d2;
    float* ar;
    float* ai;
    __device__ void fast(const Rec* rec, const float4* win, int nfit, int) {
        lattice_chunk(P, rec, win, nfit, J.lc, d2, ar, ai);
    }
    // Pulses the fast path cannot stage: the pixel offsets in two-float from FP64 (rare).
    __device__ void slow(int c0, int nslow, const SlowRec* srec) {
        const sarbp_lattice& L = J.lat;
        const int tid = threadIdx.x, cols_t = 1 << J.lc, hr = (kSplitTilePixels >> J.lc) >> 1;
        const double dj = (double)((tid & (cols_t - 1)) - (cols_t >> 1));
#pragma unroll 1
        for (int k = 0; k < kPX; ++k) {
            const double di = (double)(((tid + kThreads * k) >> J.lc) - hr);
            Pix q;
            pixel_from_offsets(S, di * L.step_row[0] + dj * L.step_col[0], di * L.step_row[1] + dj * L.step_col[1],
                               di * L.step_row[2] + dj * L.step_col[2], q);
            const float2 v = slow_pixel(P, srec, nslow, c0, q.dxh, q.dxl, q.dyh, q.dyl, q.dzh, q.dzl, 0.0f);
            ar[k] += v.x;
            ai[k] += v.y;
        }
    }
};

// ---- adjoint (gradients of a real image loss) -------------------------------------------
//
// With G_p = dl/dRe I_p + i dl/dIm I_p and c_pn = w_n v_pn exp(i phi_pn), the
// per-pulse sums U_n = sum_p conj(G_p) v_pn exp(i phi_pn) and
// A_n = sum_p Re(conj(G_p) (v'_pn / data_dr + i k v_pn) exp(i phi_pn)) e_pn
// (e_pn the unit vector from pos_n to pixel p, v' = d sample1 / dq) give
// dl/dpos_n = -w_n A_n, dl/dphase_n = -w_n Im U_n, dl/dweight_n = Re U_n.
// Each CTA recomputes its tile's contributions and writes per-pulse partial
// sums; adjoint_sum_kernel adds the tiles in fixed order.
constexpr int kAdjVals = 5;  // Re U, Im U, A.x, A.y, A.z

template <bool HAS_Z, bool DEMOD>
struct AdjointBody {
    static constexpr int kRecMode = 0;
    static constexpr bool kShflWindows = false;
    const SplitParams& P;
    const TileShared& S;
    Pix* px;
    const float* gre;
    const float* gim;
    float (*red)[kMaxChunk][kAdjVals];  // [warp][pulse][value]
    float* part;                        // this tile's partial sums, [pulse][kAdjVals]
    int pixels;                         // pixels of the tile that exist (the rest have G = 0)

    __device__ void flush(int n0, int cnt) {
        __syncthreads();
        for (int t = threadIdx.x; t < cnt * kAdjVals; t += kThreads) {
            const int nl = t / kAdjVals, v = t - nl * kAdjVals;
            float acc = 0.0f;
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) acc += red[w][nl][v];
            part[(size_t)(n0 + nl) * kAdjVals + v] = acc;
        }
    }

    __device__ void fast(const Rec* rec, const float4* win, int nfit, int c0) {
        const float inv_dr = P.inv_drf, Kf = P.Kf, kr = P.Kf * kTwoPiF;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 1
        for (int nl = 0; nl < nfit; ++nl) {
            // rd.x (the unit vector's z) is needed for the z gradient even on a flat lattice.
            const float4 ra = rec[nl].a, rb = rec[nl].b, rc = rec[nl].c, rd = rec[nl].d;
            const int bias = __float_as_int(rc.y);
            const unsigned last = (unsigned)__float_as_int(rc.w);
            const float4* wrow = win + 2 * __float_as_int(rc.z);
            const float R = 0.5f * rb.z;
            float v5[kAdjVals] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < kPX; ++k) {
                const Pix& q = px[k];
                float L = fmaf(rb.x, q.dx, rb.y * q.dy);
                if (HAS_Z) L = fmaf(rd.x, q.dz, L);
                const float q2 = fmaf(-L, L, q.d2);
                const float B = rcp_approx(fmaf(2.0f, L, rb.z));
                const float e0 = q2 * B;
                const float eps = fmaf(-e0 * e0, B, e0);
                const float qp = fmaf(L + eps, inv_dr, rb.w);
                const float tq = qp + kMagic;
                const float s = qp - (tq - kMagic);
                const unsigned j = min((unsigned)(__float_as_int(tq) - bias), last);
                const float4 c01 = wrow[2 * j], c23 = wrow[2 * j + 1];
                const float vr = fmaf(fmaf(fmaf(c23.z, s, c23.x), s, c01.z), s, c01.x);
                const float vi = fmaf(fmaf(fmaf(c23.w, s, c23.y), s, c01.w), s, c01.y);
                const float dvr = fmaf(fmaf(3.0f * c23.z, s, 2.0f * c23.x), s, c01.z);
                const float dvi = fmaf(fmaf(3.0f * c23.w, s, 2.0f * c23.y), s, c01.w);
                float tb = ra.y * q.dyh;
                if (HAS_Z) tb = fmaf(rd.y, q.dzh, tb);
                tb = fmaf(ra.x, q.dxh, tb);
                float sm = fmaf(Kf, eps, rc.x);
                sm = fmaf(ra.x, q.dxl, sm);
                sm = fmaf(ra.y, q.dyl, sm);
                sm = fmaf(ra.z, q.dx, sm);
                sm = fmaf(ra.w, q.dy, sm);
                if (HAS_Z) {
                    sm = fmaf(rd.y, q.dzl, sm);
                    sm = fmaf(rd.z, q.dz, sm);
                }
                if (DEMOD) sm += q.psi;
                const float tot = (tb - round_magic(tb)) + sm;
                const float ang = (tot - round_magic(tot)) * kTwoPiF;
                float sn, cs;
                __sincosf(ang, &sn, &cs);
                const float gr = gre[k], gi = gim[k];
                const float er = vr * cs - vi * sn, ei = vr * sn + vi * cs;  // v exp(i phi)
                v5[0] = fmaf(gr, er, fmaf(gi, ei, v5[0]));
                v5[1] = fmaf(gr, ei, fmaf(-gi, er, v5[1]));
                const float zr = fmaf(dvr, inv_dr, -kr * vi), zi = fmaf(dvi, inv_dr, kr * vr);
                const float fr = zr * cs - zi * sn, fi = zr * sn + zi * cs;
                const float t = fmaf(gr, fr, gi * fi) * rcp_approx(R + L + eps);
                v5[2] = fmaf(t, fmaf(R, rb.x, q.dx), v5[2]);
                v5[3] = fmaf(t, fmaf(R, rb.y, q.dy), v5[3]);
                v5[4] = fmaf(t, fmaf(R, rd.x, q.dz), v5[4]);
            }
#pragma unroll
            for (int v = 0; v < kAdjVals; ++v) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v5[v] += __shfl_xor_sync(0xffffffffu, v5[v], o);
            }
            if (lane == 0) {
#pragma unroll
                for (int v = 0; v < kAdjVals; ++v) red[warp][nl][v] = v5[v];
            }
        }
        flush(c0, nfit);
    }

    // Pulses the fast path cannot stage: two-float geometry per pixel, FP32 interpolation.
    __device__ void slow(int c0, int nslow, const SlowRec* srec) {
        const PulseInputs& in = P.in;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const float kr = P.Kf * kTwoPiF, inv_dr = P.inv_drf;
#pragma unroll 1
        for (int j = 0; j < nslow; ++j) {
            const SlowRec sr = srec[j];
            const float2* row = in.data + (size_t)(c0 + j) * in.samples;
            float v5[kAdjVals] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < kPX; ++k) {
                SlowSample o;
                if (!slow_sample<true>(P, sr, row, px[k], DEMOD ? px[k].psi : 0.0f, o)) continue;
                float sn, cs;
                __sincosf(o.ang, &sn, &cs);
                const float gr = gre[k], gi = gim[k];
                const float er = o.vr * cs - o.vi * sn, ei = o.vr * sn + o.vi * cs;
                v5[0] = fmaf(gr, er, fmaf(gi, ei, v5[0]));
                v5[1] = fmaf(gr, ei, fmaf(-gi, er, v5[1]));
                const float zr = fmaf(o.dvr, inv_dr, -kr * o.vi), zi = fmaf(o.dvi, inv_dr, kr * o.vr);
                const float fr = zr * cs - zi * sn, fi = zr * sn + zi * cs;
                const float t = fmaf(gr, fr, gi * fi);
                v5[2] = fmaf(t, o.ex, v5[2]);
                v5[3] = fmaf(t, o.ey, v5[3]);
                v5[4] = fmaf(t, o.ez, v5[4]);
            }
#pragma unroll
            for (int v = 0; v < kAdjVals; ++v) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v5[v] += __shfl_xor_sync(0xffffffffu, v5[v], o);
            }
            if (lane == 0) {
#pragma unroll
                for (int v = 0; v < kAdjVals; ++v) red[warp][j][v] = v5[v];
            }
        }
        flush(c0, nslow);
    }
};

// Adjoint on lattice tiles, with the forward's separable row/column terms.  Per pulse a
// thread sums its pixels' t_p = Re(conj(G_p) z_p e^{i phi}) / d_p as T0 = sum t_p and
// S1 = sum kc_p t_p; with delta_p = di_p s_row + dj_p s_col the position sum is
// A = sum t_p (R u + delta_p) = R u T0 + s_row Ti + s_col Tj, Ti = sum t_p di_p = di T0 + m S1,
// Tj = dj T0 (a thread's pixels share the column).  The warps reduce (Re U, Im U, T0, Ti, Tj)
// and the flush turns them into A with the chunk's records.
__device__ __noinline__ void lattice_adjoint_slow(const SplitParams& P, const TileShared& S, const Job& J, float g0,
                                                  float g1, float g2, float g3, float h0, float h1, float h2,
                                                  float h3, float (*red)[kMaxChunk][kAdjVals], float* part, int c0,
                                                  int nslow, const SlowRec* srec) {
    const sarbp_lattice& L = J.lat;
    const int tid = threadIdx.x, cols_t = 1 << J.lc, hr = (kSplitTilePixels >> J.lc) >> 1;
    const double dj = (double)((tid & (cols_t - 1)) - (cols_t >> 1));
    Pix px[kPX];
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const double di = (double)(((tid + kThreads * k) >> J.lc) - hr);
        pixel_from_offsets(S, di * L.step_row[0] + dj * L.step_col[0], di * L.step_row[1] + dj * L.step_col[1],
                           di * L.step_row[2] + dj * L.step_col[2], px[k]);
        px[k].psi = 0.0f;
    }
    const float gre[kPX] = {g0, g1, g2, g3}, gim[kPX] = {h0, h1, h2, h3};
    static_assert(AdjointBody<true, false>::kRecMode == 0, "the fallback works from per-pixel offsets");
    AdjointBody<true, false> body{P, S, px, gre, gim, red, part, kSplitTilePixels};
    body.slow(c0, nslow, srec);  // writes A directly
}

// Warp sums of five values in 28 instructions instead of 50: the first two butterfly levels halve
// the values each lane carries (a lane keeps one of each pair and trades the other with its
// partner), the last three are plain.  Lane l ends with the sum of value (l >> 4) + 2 ((l >> 3) & 1)
// of v0..v3 in sq and of v4 in s4.
__device__ __forceinline__ void warp_sum5(float v0, float v1, float v2, float v3, float v4, float& sq, float& s4) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    float a = h16 ? v1 : v0;
    a += __shfl_xor_sync(full, h16 ? v0 : v1, 16);
    float b = h16 ? v3 : v2;
    b += __shfl_xor_sync(full, h16 ? v2 : v3, 16);
    float e = v4 + __shfl_xor_sync(full, v4, 16);
    float c = h8 ? b : a;
    c += __shfl_xor_sync(full, h8 ? a : b, 8);
    e += __shfl_xor_sync(full, e, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
        c += __shfl_xor_sync(full, c, o);
        e += __shfl_xor_sync(full, e, o);
    }
    sq = c;
    s4 = e;
}

struct LatticeAdjointBody {
    static constexpr int kRecMode = 2;
    static constexpr bool kShflWindows = false;
    const SplitParams& P;
    const TileShared& S;
    const Job& J;
    const float* d2;
    const float* gre;
    const float* gim;
    float (*red)[kMaxChunk][kAdjVals];
    float* part;

    __device__ void flush(int n0, int cnt, const Rec* rec) {
        __syncthreads();
        for (int nl = threadIdx.x; nl < cnt; nl += kThreads) {
            float v[kAdjVals];
#pragma unroll
            for (int c = 0; c < kAdjVals; ++c) {
                float acc = 0.0f;
#pragma unroll
                for (int w = 0; w < kThreads / 32; ++w) acc += red[w][nl][c];
                v[c] = acc;
            }
            const float4 rd = rec[nl].d;
            const float R = 0.5f * rec[nl].b.z, t0 = v[2], ti = v[3], tj = v[4];
            const float u[3] = {rd.y, rd.z, rd.w};
            float* out = part + (size_t)(n0 + nl) * kAdjVals;
            out[0] = v[0];
            out[1] = v[1];
#pragma unroll
            for (int c = 0; c < 3; ++c) out[2 + c] = fmaf(R * u[c], t0, fmaf(S.sth[c], ti, S.sth[3 + c] * tj));
        }
    }

    __device__ void fast(const Rec* rec, const float4* win, int nfit, int c0) {
        const float inv_dr = P.inv_drf, kr = P.Kf * kTwoPiF;
        const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, lc = J.lc;
        const int m = kThreads >> lc, hr = (kSplitTilePixels >> lc) >> 1, cols_t = 1 << lc;
        const float di = (float)((tid >> lc) + 2 * m - hr);
        const float dj = (float)((tid & (cols_t - 1)) - (cols_t >> 1));
        const float mf = (float)m;
        // The forward's packed pixel pairs (see lattice_chunk), plus R + (L + eps) as a pair.
        const float2 nd2[2] = {make_float2(-d2[0], -d2[1]), make_float2(-d2[2], -d2[3])};
        const float2 kcs[2] = {make_float2(-2.0f, -1.0f), make_float2(0.0f, 1.0f)};
        const float2 ninv = pair(-inv_dr), nkr = pair(-kr), magic = pair(kMagic), nmagic = pair(-kMagic);
        const float2 mone = pair(-1.0f), mtwo = pair(-2.0f), half = pair(0.5f);
#pragma unroll 1
        for (int nl = 0; nl < nfit; ++nl) {
            const float4 ra = rec[nl].a, rb = rec[nl].b, rc = rec[nl].c, rd = rec[nl].d, re = rec[nl].e;
            const int bias = __float_as_int(rc.y);
            const unsigned last = (unsigned)__float_as_int(rc.w);
            const float4* wrow = win + 2 * __float_as_int(rc.z);
            const float nL0 = fmaf(-dj, rb.y, -di * rb.x), nmA = -(mf * rb.x);  // -L0, -m u.s_row: exact
            const float t = fmaf(dj, ra.z, di * ra.x);                           // exact
            const float r0 = ((t - round_magic(t)) + fmaf(dj, ra.w, fmaf(di, ra.y, rc.x))) * kTwoPiF;
            const float2 twoR = make_float2(re.x, re.y), fm = make_float2(re.z, re.w);
            const float2 R2 = __fmul2_rn(twoR, half);
            const float2 nL02 = pair(nL0), nstep = pair(nmA), sp = pair(rd.x), r02 = pair(r0);
            float u0 = 0.f, u1 = 0.f, t0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float2 nL = __ffma2_rn(kcs[h], nstep, nL02);
                const float2 nq2 = __ffma2_rn(nL, nL, nd2[h]);
                const float2 den = __ffma2_rn(mtwo, nL, twoR);
                const float2 B = make_float2(rcp_approx(den.x), rcp_approx(den.y));
                const float2 ne0 = __fmul2_rn(nq2, B);
                const float2 neps = __ffma2_rn(__fmul2_rn(ne0, ne0), B, ne0);
                const float2 nLe = __fadd2_rn(nL, neps);  // -(L + eps)
                const float2 qp = __ffma2_rn(nLe, ninv, fm);
                const float2 tq = __fadd2_rn(qp, magic);
                const float2 s = __ffma2_rn(__fadd2_rn(tq, nmagic), mone, qp);
                const float2 ang = __ffma2_rn(nkr, neps, __ffma2_rn(kcs[h], sp, r02));
                const float2 dist = __ffma2_rn(nLe, mone, R2);  // R + (L + eps)
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const int k = 2 * h + c;
                    const float kc = (float)(k - 2);
                    const float tqc = c ? tq.y : tq.x;
                    const unsigned j = min((unsigned)(__float_as_int(tqc) - bias), last);
                    const float4 c01 = wrow[2 * j], c23 = wrow[2 * j + 1];
                    // Horner for the value as (re, im) pairs; the derivative c1 + 2 c2 s + 3 c3 s^2 =
                    // p2 + s (p1 + c3 s) reuses its partial results p1 = c3 s + c2, p2 = p1 s + c1.
                    const float2 ss = pair(c ? s.y : s.x), c3 = make_float2(c23.z, c23.w);
                    const float2 p1 = __ffma2_rn(c3, ss, make_float2(c23.x, c23.y));
                    const float2 p2 = __ffma2_rn(p1, ss, make_float2(c01.z, c01.w));
                    const float2 v = __ffma2_rn(p2, ss, make_float2(c01.x, c01.y));
                    const float2 dv = __ffma2_rn(ss, __ffma2_rn(c3, ss, p1), p2);
                    float sn, cs;
                    __sincosf(c ? ang.y : ang.x, &sn, &cs);
                    // h = conj(G) exp(i phi): U += v h, and the position weight
                    // Re(conj(G) (v'/dr + i k v) exp(i phi)) / d = (Re(v' h) / dr - k Im(v h)) / d.
                    const float gr = gre[k], gi = gim[k];
                    const float hr = fmaf(gr, cs, gi * sn), hi = fmaf(gr, sn, -gi * cs);
                    u0 = fmaf(v.x, hr, fmaf(-v.y, hi, u0));
                    const float w1 = fmaf(v.x, hi, v.y * hr);
                    u1 += w1;
                    const float q = fmaf(dv.x, hr, -dv.y * hi);
                    const float tt = fmaf(q, inv_dr, -kr * w1) * rcp_approx(c ? dist.y : dist.x);
                    t0 += tt;
                    s1 = fmaf(kc, tt, s1);
                }
            }
            float sq, s4;
            warp_sum5(u0, u1, t0, fmaf(di, t0, mf * s1), dj * t0, sq, s4);
            if ((lane & 7) == 0) red[warp][nl][(lane >> 4) | ((lane >> 2) & 2)] = sq;
            if (lane == 0) red[warp][nl][4] = s4;
        }
        flush(c0, nfit, rec);
    }

    __device__ void slow(int c0, int nslow, const SlowRec* srec) {
        lattice_adjoint_slow(P, S, J, gre[0], gre[1], gre[2], gre[3], gim[0], gim[1], gim[2], gim[3], red, part, c0,
                             nslow, srec);
    }
};

// ---- output ----------------------------------------------------------------------
__device__ __forceinline__ void store_window(const Job& J, int win_nr, int win_nu, const Pix px[kPX], float2* out,
                                             long long stride) {
    const int cols_t = 1 << J.lc;
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int p = threadIdx.x + kThreads * k;
        const int wr = J.tile_r + (p >> J.lc), wu = J.tile_u + (p & (cols_t - 1));
        if (wr < win_nr && wu < win_nu) out[(long long)wr * stride + wu] = make_float2(px[k].ar, px[k].ai);
    }
}

__device__ __forceinline__ void split_range(int p0, int p1, int parts, int part, int& b, int& e) {
    const long long len = (long long)p1 - p0;
    b = p0 + (int)(len * part / parts);
    e = p0 + (int)(len * (part + 1) / parts);
}

__device__ __forceinline__ void tile_of(int index, int win_nu, int lc, int& tile_r, int& tile_u) {
    const int cols_t = 1 << lc, rows_t = kSplitTilePixels >> lc;
    const int tiles_u = (win_nu + cols_t - 1) / cols_t;
    tile_r = (index / tiles_u) * rows_t;
    tile_u = (index % tiles_u) * cols_t;
}

// ---- direct BP kernels --------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 3) split_polar_kernel(SplitParams P, PolarDesc g) {
    extern __shared__ __align__(16) char smem[];
    __shared__ TileShared S;
    Job J;
    J.g = g;
    J.lc = g.tile_lc;
    tile_of(blockIdx.x, g.win_nu, J.lc, J.tile_r, J.tile_u);
    split_range(g.a, g.b, P.pulse_split, blockIdx.y, J.p0, J.p1);
    Pix px[kPX];
    PolarTables& T = *reinterpret_cast<PolarTables*>(smem + window_offset());
    setup_polar(P, J, S, T, px, true);
    pulse_loop<false, true>(P, J, S, smem, px);
    store_window(J, g.win_nr, g.win_nu, px, P.out + blockIdx.y * P.split_stride, P.out_stride);
}

// One lattice tile over pulses [p0, p1): the per-item body shared by the one-tile-per-CTA
// kernel and the persistent batch kernel.
__device__ __forceinline__ void lattice_tile(const SplitParams& P, const sarbp_lattice& lat, int lc, int tile_r,
                                             int tile_u, int p0, int p1, float2* out, TileShared& S, char* smem) {
    Job J;
    J.lat = lat;
    J.lc = lc;
    J.tile_r = tile_r;
    J.tile_u = tile_u;
    J.p0 = p0;
    J.p1 = p1;
    float d2[kPX], ar[kPX], ai[kPX];
    setup_lattice_sep(J, S, d2);
#pragma unroll
    for (int k = 0; k < kPX; ++k) ar[k] = ai[k] = 0.0f;
    LatticeBody body{P, S, J, d2, ar, ai};
    chunk_loop(P, J, S, smem, true, body);
    const int cols_t = 1 << lc;
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int p = threadIdx.x + kThreads * k;
        const int wr = tile_r + (p >> lc), wu = tile_u + (p & (cols_t - 1));
        if (wr < lat.rows && wu < lat.cols) out[(long long)wr * lat.cols + wu] = make_float2(ar[k], ai[k]);
    }
}

__global__ void __launch_bounds__(kThreads, 4) split_lattice_kernel(SplitParams P, sarbp_lattice lat, int lc) {
    extern __shared__ __align__(16) char smem[];
    __shared__ TileShared S;
    int tile_r, tile_u, p0, p1;
    tile_of(blockIdx.x, lat.cols, lc, tile_r, tile_u);
    split_range(0, P.in.pulses, P.pulse_split, blockIdx.y, p0, p1);
    lattice_tile(P, lat, lc, tile_r, tile_u, p0, p1, P.out + blockIdx.y * P.split_stride, S, smem);
}

__global__ void __launch_bounds__(kThreads, 3) split_points_kernel(SplitParams P, const double* __restrict__ xyz,
                                                                   int npts) {
    extern __shared__ __align__(16) char smem[];
    __shared__ TileShared S;
    Job J;
    J.xyz = xyz;
    J.npts = npts;
    J.lc = 0;
    J.tile_r = blockIdx.x * kSplitTilePixels;
    J.tile_u = 0;
    split_range(0, P.in.pulses, P.pulse_split, blockIdx.y, J.p0, J.p1);
    Pix px[kPX];
    setup_points(J, S, px);
    pulse_loop<true, false>(P, J, S, smem, px);
    float2* out = P.out + blockIdx.y * P.split_stride;
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int idx = J.tile_r + threadIdx.x + kThreads * k;
        if (idx < npts) out[idx] = make_float2(px[k].ar, px[k].ai);
    }
}

// ---- adjoint kernels ----------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 3) split_lattice_adjoint_kernel(SplitParams P, sarbp_lattice lat, int lc,
                                                                            const float2* __restrict__ grad,
                                                                            float* __restrict__ partials) {
    extern __shared__ __align__(16) char smem[];
    __shared__ TileShared S;
    __shared__ float red[kThreads / 32][kMaxChunk][kAdjVals];
    Job J;
    J.lat = lat;
    J.lc = lc;
    tile_of(blockIdx.x, lat.cols, lc, J.tile_r, J.tile_u);
    split_range(0, P.in.pulses, gridDim.y, blockIdx.y, J.p0, J.p1);  // the splits write disjoint partials
    float d2[kPX], gre[kPX], gim[kPX];
    setup_lattice_sep(J, S, d2);
    const int cols_t = 1 << lc;
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const int p = threadIdx.x + kThreads * k;
        const int i = J.tile_r + (p >> lc), j = J.tile_u + (p & (cols_t - 1));
        float2 g = make_float2(0.0f, 0.0f);
        if (i < lat.rows && j < lat.cols) g = grad[(size_t)i * lat.cols + j];
        gre[k] = g.x;
        gim[k] = g.y;
    }
    LatticeAdjointBody body{P, S, J, d2, gre, gim, red, partials + (size_t)blockIdx.x * P.in.pulses * kAdjVals};
    chunk_loop(P, J, S, smem, false, body);
}

// Per-pulse gradients from the tiles' partial sums, in a fixed order (deterministic): each
// block takes 32 pulses; its 8 thread groups sum every 8th tile (coalesced: for one tile the
// 32 pulses' values are contiguous), then the 8 group sums are added in group order.
constexpr int kSumPulses = 32, kSumGroups = kThreads / kSumPulses;

__global__ void __launch_bounds__(kThreads) adjoint_sum_kernel(const float* __restrict__ partials, int ntiles,
                                                               int pulses, const double* __restrict__ weight,
                                                               double* grad_pos, double* grad_phase,
                                                               double* grad_weight) {
    __shared__ double part[kSumGroups][kSumPulses][kAdjVals];
    const int pl = threadIdx.x % kSumPulses, grp = threadIdx.x / kSumPulses;
    const int n = blockIdx.x * kSumPulses + pl;
    double acc[kAdjVals] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (n < pulses) {
        for (int t = grp; t < ntiles; t += kSumGroups) {
            const float* p = partials + ((size_t)t * pulses + n) * kAdjVals;
#pragma unroll
            for (int v = 0; v < kAdjVals; ++v) acc[v] += (double)p[v];
        }
    }
#pragma unroll
    for (int v = 0; v < kAdjVals; ++v) part[grp][pl][v] = acc[v];
    __syncthreads();
    if (grp != 0 || n >= pulses) return;
#pragma unroll
    for (int v = 0; v < kAdjVals; ++v) {
        double s = part[0][pl][v];
        for (int g = 1; g < kSumGroups; ++g) s += part[g][pl][v];
        acc[v] = s;
    }
    const double w = weight[n];
    if (grad_pos) {
        grad_pos[3 * n] = -w * acc[2];
        grad_pos[3 * n + 1] = -w * acc[3];
        grad_pos[3 * n + 2] = -w * acc[4];
    }
    if (grad_phase) grad_phase[n] = -w * acc[1];
    if (grad_weight) grad_weight[n] = acc[0];
}

// ---- FFBP: per-node tables and per-pulse leaf records (prologue kernels) ------------------
// Two-float constants of the table entries: K (turns/m), range_start, 1 / data_dr.
struct TableConsts {
    float Kh, Kl, rsh, rsl, idrh, idrl;
};

__host__ __device__ inline TableConsts table_consts(const SplitParams& P) {
    return TableConsts{P.Kh, P.Kl, P.rsh, P.rsl, P.idrh, P.idrl};
}

__device__ __forceinline__ FF ff_sqrt0(FF a) { return a.h > 0.0f ? ff_sqrt(a) : FF{0.0f, 0.0f}; }

// Row t and column t of node g's tables in two-float FP32 arithmetic from the node geometry
// split on the host (PolarDesc::tf).
__device__ __forceinline__ void table_entries(const TableConsts& C, const PolarDesc& g, int t,
                                              float4* __restrict__ tables) {
    const FF ft{(float)t, 0.0f};  // exact: node dimensions are far below 2^24
    if (t < g.nr) {
        const FF r = ff_add(ff_of(g.tf[3]), ff_mul(ft, ff_of(g.tf[4])));
        const FF oz = ff_of(g.tf[2]);
        const FF gg = ff_sqrt0(ff_add(ff_sqr(r), ff_neg(ff_sqr(oz))));
        const FF ph = ff_mul(FF{-C.Kh, -C.Kl}, r);
        float psi = (ph.h - rintf(ph.h)) + ph.l;
        psi -= rintf(psi);
        const FF ir = ff_rcp(r);
        const FF gr = ff_mul(gg, ir), ez = ff_mul(ff_neg(oz), ir);
        float F;
        const float I = fminf(fmaxf(ff_floor_frac(ff_mul(ff_add(r, FF{-C.rsh, -C.rsl}), FF{C.idrh, C.idrl}), F),
                                    -1.0e9f), 1.0e9f);
        float4* row = tables + g.rows_off + 3 * (long long)t;
        row[0] = make_float4(gg.h, gg.l, psi, 0.0f);
        row[1] = make_float4(gr.h, gr.l, ez.h, ez.l);
        row[2] = make_float4(2.0f * (r.h + r.l), F, __int_as_float((int)I), 0.0f);
    }
    if (t < g.nu) {
        const FF u = ff_add(ff_of(g.tf[5]), ff_mul(ft, ff_of(g.tf[6])));
        const FF c = ff_sqrt0(ff_add(FF{1.0f, 0.0f}, ff_neg(ff_sqr(u))));
        tables[g.cols_off + t] = make_float4(c.h, c.l, u.h, u.l);
    }
}

__global__ void ffbp_tables_kernel(TableConsts C, const PolarDesc* __restrict__ nodes, float4* __restrict__ tables) {
    table_entries(C, nodes[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x, tables);
}

// Leaf pulses relative to the leaf's phase centre O (origin formulation).
// A = -K (pos - O) is split into a multiple of a per-leaf power-of-two
// quantum with <= 10 significant bits plus an FP32 remainder.
struct PulseRec {
    float4 a;  // A_hi.x, A_hi.y, A_hi.z, frac(phase / 2pi)
    float4 b;  // A_lo.x, A_lo.y, A_lo.z, |pos - O|^2
    float4 c;  // (pos - O).x, .y, .z, weight
    float4 d;  // the leaf's A quantum (a power of two), its inverse
};

__device__ __forceinline__ void leaf_pulses(double K, const double* __restrict__ pos, const double* __restrict__ weight,
                                            const double* __restrict__ phase, const PolarDesc& g,
                                            PulseRec* __restrict__ recs, int& amax) {
    if (threadIdx.x == 0) amax = 0;
    __syncthreads();
    float m = 0.0f;
    for (int n = g.a + threadIdx.x; n < g.b; n += blockDim.x) {
        const double ax = pos[3 * n] - g.ox, ay = pos[3 * n + 1] - g.oy, az = pos[3 * n + 2] - g.oz;
        m = fmaxf(m, (float)(fabs(K) * fmax(fabs(ax), fmax(fabs(ay), fabs(az)))));
    }
    atomicMax(&amax, __float_as_int(m));  // non-negative floats order like their bit patterns
    __syncthreads();
    int e = 0;
    frexp((double)__int_as_float(amax) * 1.0001 + 1e-30, &e);
    const double scale = ldexp(1.0, e - 10), inv_scale = ldexp(1.0, 10 - e);
    for (int n = g.a + threadIdx.x; n < g.b; n += blockDim.x) {
        const double ax = pos[3 * n] - g.ox, ay = pos[3 * n + 1] - g.oy, az = pos[3 * n + 2] - g.oz;
        PulseRec r;
        quantize(-K * ax, scale, inv_scale, r.a.x, r.b.x);
        quantize(-K * ay, scale, inv_scale, r.a.y, r.b.y);
        quantize(-K * az, scale, inv_scale, r.a.z, r.b.z);
        const double t = phase[n] * kInvTwoPi;
        r.a.w = (float)(t - rint(t));
        r.b.w = (float)(ax * ax + ay * ay + az * az);
        r.c = make_float4((float)ax, (float)ay, (float)az, (float)weight[n]);
        r.d = make_float4((float)scale, (float)inv_scale, 0.0f, 0.0f);
        recs[n] = r;
    }
}

__global__ void ffbp_leaf_pulses_kernel(double K, const double* __restrict__ pos, const double* __restrict__ weight,
                                        const double* __restrict__ phase, const PolarDesc* __restrict__ nodes,
                                        const int* __restrict__ leaves, PulseRec* __restrict__ recs) {
    __shared__ int amax;
    leaf_pulses(K, pos, weight, phase, nodes[leaves[blockIdx.x]], recs, amax);
}

// ---- FFBP: leaves (origin formulation) ---------------------------------------------------
//
// With O the leaf's phase centre and a = pos_n - O (|a| ~ the leaf aperture),
// a pixel at slant range r from O in unit direction e satisfies exactly
//   d = |r e - a| = r - L + eps,  L = e . a,  eps = (|a|^2 - L^2) / (2 (r - L) + eps),
// so the demodulated phase k (d - r) + phase_n is -K e . a + K eps + phase_n / 2pi
// (turns): no large term, no per-tile FP64.  On a polar grid e = (alpha s, alpha u, beta) with
// alpha = g / r and beta = -oz / r per row and s = side sqrt(1 - u^2), u per column, so
//   e . a = alpha C + beta a.z,       C = s a.x + u a.y,
//   -K e . a = alpha D + beta A.z,    D = s A.x + u A.y   (A = -K a),
// with C and D once per (pulse, tile column).  The phase's large part alpha_hi D_hi + beta_hi
// A_hi.z is exact in FP32: alpha_hi and beta_hi are multiples of 2^-11 (11 bits), D_hi and
// A_hi.z multiples of the leaf's A quantum below 2^10.5 quanta, so each product has at most 22
// bits and their sum 23.  A thread's four pixels share the tile column and run as two pairs
// of f32x2 lanes.
struct LeafRec {
    float4 p0;  // (a.z, a.z), (-|a|^2, -|a|^2)
    float4 p1;  // (A_hi.z, A_hi.z), (A_lo.z, A_lo.z)
    float4 p2;  // (A.z, A.z), (Phi, Phi)
    int4 w;     // window bias bits, window offset, window count - 1, unused
};

struct LeafCol {
    float4 p0;  // (C, C), (D_hi, D_hi)
    float4 p1;  // (D_lo, D_lo), (D, D)
};

constexpr int kLeafColStride = 32;  // LeafCol entries per pulse: the widest leaf tile

__host__ __device__ constexpr size_t leaf_col_offset() { return (size_t)kMaxLeafChunk * sizeof(LeafRec); }
__host__ __device__ constexpr size_t leaf_window_offset(int chunk) {
    return leaf_col_offset() + (size_t)chunk * kLeafColStride * sizeof(LeafCol);
}

// Two pixels of one tile column (the lanes), rows (row0, row1).
struct LPair {
    float2 na, nb;  // -alpha, -beta
    float2 ah, al;  // alpha = ah + al, ah a multiple of 2^-11
    float2 bh, bl;  // beta = bh + bl
    float2 r2, fm;  // 2 r, frac(Q) - 1/2 with Q = (r - range_start) / data_dr
    float2 ar, ai;  // accumulated image, real and imaginary parts
    int o0, o1;     // floor(Q) - I_first
};

constexpr float kUnitQ = 1.0f / 2048.0f;  // quantum of unit-vector components (11 bits)

__device__ __forceinline__ void unit_split(float p, float e, float& h, float& l, float& full) {
    h = rintf(p * 2048.0f) * kUnitQ;
    l = (p - h) + e;
    full = p + e;
}

// The row values of pixel row i (tables: (g/r, -oz/r) as float pairs, (2r, frac(Q) - 1/2, floor(Q))).
__device__ __forceinline__ void leaf_row(const PolarDesc& g, const float4* __restrict__ tables, int i, int I_first,
                                         float& na, float& nb, float& ah, float& al, float& bh, float& bl, float& r2,
                                         float& fm, int& o) {
    const float4 r1 = __ldg(tables + g.rows_off + 3 * (long long)i + 1);
    const float4 rq = __ldg(tables + g.rows_off + 3 * (long long)i + 2);
    float a, b;
    unit_split(r1.x, r1.y, ah, al, a);
    unit_split(r1.z, r1.w, bh, bl, b);
    na = -a;
    nb = -b;
    r2 = rq.x;
    fm = rq.y;
    o = __float_as_int(rq.z) - I_first;
}

// One pixel's windowed sample (the reference's cubic, weight folded in) at bin index bits tq and
// centred fraction s; with no fitting window the taps come straight from the pulse row.
template <bool STAGED>
__device__ __forceinline__ float2 leaf_sample(const float4* wrow, unsigned last, int bias, float tq,
                                              float s, int o, const float2* drow, int I_first, int samples, float wt) {
    float2 v;
    if (STAGED) {
        const unsigned j = min((unsigned)(__float_as_int(tq) + o - bias), last);
        const float4 c01 = wrow[2 * j], c23 = wrow[2 * j + 1];
        const float2 sp = pair(s);
        v = __ffma2_rn(make_float2(c23.z, c23.w), sp, make_float2(c23.x, c23.y));
        v = __ffma2_rn(v, sp, make_float2(c01.z, c01.w));
        v = __ffma2_rn(v, sp, make_float2(c01.x, c01.y));
    } else {  // the pulse's window does not fit: gather its taps directly
        const long long gb = (long long)(__float_as_int(tq) - kMagicBits) + o + I_first;
        v = make_float2(0.0f, 0.0f);
        if (gb >= 1 && gb <= (long long)samples - 3) {
            float w[4];
            lagrange_centred(s, w);
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const float2 x = __ldg(drow + gb + b - 1);
                v.x = fmaf(w[b], x.x, v.x);
                v.y = fmaf(w[b], x.y, v.y);
            }
            v.x *= wt;
            v.y *= wt;
        }
    }
    return v;
}

// One pulse on one pixel pair: range, window sample, phase and the accumulation.
template <bool STAGED>
__device__ __forceinline__ void leaf_pair_pulse(LPair& q, const LeafRec& R, const LeafCol& Cc, const float4* wrow, unsigned last, int bias, const float2* drow,
                                                int I_first, int samples, float wt, float2 nKf, float2 ninv_dr) {
    const float2 magic = pair(kMagic), nmagic = pair(-kMagic), mone = pair(-1.0f);
    const float2 az = make_float2(R.p0.x, R.p0.y), naa = make_float2(R.p0.z, R.p0.w);
    const float2 C = make_float2(Cc.p0.x, Cc.p0.y);
    const float2 nL = __ffma2_rn(q.na, C, __fmul2_rn(q.nb, az));  // -L
    const float2 nq2 = __ffma2_rn(nL, nL, naa);                    // -(|a|^2 - L^2)
    const float2 den = __ffma2_rn(pair(2.0f), nL, q.r2);           // 2 (r - L)
    const float2 B = make_float2(rcp_approx(den.x), rcp_approx(den.y));
    const float2 ne0 = __fmul2_rn(nq2, B);
    const float2 neps = __ffma2_rn(__fmul2_rn(ne0, ne0), B, ne0);  // -eps (second order: leaves are wide)
    const float2 qp = __ffma2_rn(__ffma2_rn(nL, mone, neps), ninv_dr, q.fm);
    const float2 tq = __fadd2_rn(qp, magic);
    const float2 s = __ffma2_rn(__fadd2_rn(tq, nmagic), mone, qp);
    // Phase (turns): the exact part, then the small terms.
    const float2 tb = __ffma2_rn(q.ah, make_float2(Cc.p0.z, Cc.p0.w), __fmul2_rn(q.bh, make_float2(R.p1.x, R.p1.y)));
    float2 sm = __ffma2_rn(nKf, neps, make_float2(R.p2.z, R.p2.w));
    sm = __ffma2_rn(q.ah, make_float2(Cc.p1.x, Cc.p1.y), sm);
    sm = __ffma2_rn(q.al, make_float2(Cc.p1.z, Cc.p1.w), sm);
    sm = __ffma2_rn(q.bh, make_float2(R.p1.z, R.p1.w), sm);
    sm = __ffma2_rn(q.bl, make_float2(R.p2.x, R.p2.y), sm);
    // The reduced exact term is in [-1/2, 1/2] turn and |sm| <= 1 + K eps (eps is second order in
    // the pulse's offset from the leaf centre), so the angle stays within a few turns, which the
    // hardware sin/cos reduce themselves.
    const float2 rtb = __fadd2_rn(__fadd2_rn(tb, magic), nmagic);
    const float2 ang = __fmul2_rn(__fadd2_rn(__ffma2_rn(rtb, mone, tb), sm), pair(kTwoPiF));
    float sn0, cs0, sn1, cs1;
    __sincosf(ang.x, &sn0, &cs0);
    __sincosf(ang.y, &sn1, &cs1);
    const float2 v0 = leaf_sample<STAGED>(wrow, last, bias, tq.x, s.x, q.o0, drow, I_first, samples, wt);
    const float2 v1 = leaf_sample<STAGED>(wrow, last, bias, tq.y, s.y, q.o1, drow, I_first, samples, wt);
    q.ar.x = fmaf(v0.x, cs0, q.ar.x);
    q.ar.x = fmaf(-v0.y, sn0, q.ar.x);
    q.ai.x = fmaf(v0.x, sn0, q.ai.x);
    q.ai.x = fmaf(v0.y, cs0, q.ai.x);
    q.ar.y = fmaf(v1.x, cs1, q.ar.y);
    q.ar.y = fmaf(-v1.y, sn1, q.ar.y);
    q.ai.y = fmaf(v1.x, sn1, q.ai.y);
    q.ai.y = fmaf(v1.y, cs1, q.ai.y);
}

// C and D of one (pulse, tile column) from the pulse record and the column table (c, u pairs):
// D in two-float, split on the leaf's A quantum.
__device__ __forceinline__ LeafCol leaf_col(const PulseRec& pr, float4 cv, float side) {
    const float sh = side * cv.x, sl = side * cv.y, uh = cv.z, ul = cv.w;
    const float C = fmaf(sh, pr.c.x, uh * pr.c.y);
    const float p1 = sh * pr.a.x, e1 = fmaf(sh, pr.a.x, -p1);
    const float p2 = uh * pr.a.y, e2 = fmaf(uh, pr.a.y, -p2);
    const float S = p1 + p2, bb = S - p1;
    float rest = (p1 - (S - bb)) + (p2 - bb);
    rest += e1 + e2;
    rest = fmaf(sh, pr.b.x, rest);
    rest = fmaf(sl, pr.a.x, rest);
    rest = fmaf(uh, pr.b.y, rest);
    rest = fmaf(ul, pr.a.y, rest);
    const float Dh = rintf(S * pr.d.y) * pr.d.x;  // the A quantum is a power of two: exact
    const float Dl = (S - Dh) + rest;             // S - Dh is exact (|S - Dh| <= quantum / 2)
    LeafCol L;
    L.p0 = make_float4(C, C, Dh, Dh);
    L.p1 = make_float4(Dl, Dl, S + rest, S + rest);
    return L;
}

// One leaf tile: the per-item body of the leaf kernels.  precs holds the pulse records of
// the leaf's scene (indexed by pulse); a node with a destination pointer writes there.
__device__ __forceinline__ void leaf_tile(const SplitParams& P, const PolarDesc* __restrict__ nodes, const TileItem it,
                                          const float4* __restrict__ tables, const PulseRec* __restrict__ precs,
                                          float2* __restrict__ arena, float2* root_out, int root, char* smem,
                                          int* s_base, float* s_wt, int& s_nfit) {
    const PolarDesc g = nodes[it.node];
    const int lc = g.tile_lc, cols_t = 1 << lc, rows_t = kSplitTilePixels >> lc;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int col = tid & (cols_t - 1);
    const int ifirst = min(g.win_r0 + it.tile_r, g.nr - 1);
    const int ilast = min(g.win_r0 + it.tile_r + rows_t - 1, g.nr - 1);
    const float4 rfirst = __ldg(tables + g.rows_off + 3 * (long long)ifirst + 2);
    const int I_first = __float_as_int(rfirst.z);
    const int I_span = __float_as_int(__ldg(tables + g.rows_off + 3 * (long long)ilast + 2).z) - I_first;
    const float r_min = 0.5f * rfirst.x;
    // Pixel k of this thread is row (tid >> lc) + k (256 >> lc) of its column; pairs (0, 1), (2, 3).
    LPair px[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        LPair& q = px[h];
        const int i0 = min(g.win_r0 + it.tile_r + (tid >> lc) + (kThreads >> lc) * (2 * h), g.nr - 1);
        const int i1 = min(g.win_r0 + it.tile_r + (tid >> lc) + (kThreads >> lc) * (2 * h + 1), g.nr - 1);
        leaf_row(g, tables, i0, I_first, q.na.x, q.nb.x, q.ah.x, q.al.x, q.bh.x, q.bl.x, q.r2.x, q.fm.x, q.o0);
        leaf_row(g, tables, i1, I_first, q.na.y, q.nb.y, q.ah.y, q.al.y, q.bh.y, q.bl.y, q.r2.y, q.fm.y, q.o1);
        q.ar = q.ai = make_float2(0.0f, 0.0f);
    }
    LeafRec* rec = reinterpret_cast<LeafRec*>(smem);
    LeafCol* cols = reinterpret_cast<LeafCol*>(smem + leaf_col_offset());
    float4* win = reinterpret_cast<float4*>(smem + leaf_window_offset(P.chunk));
    const PulseInputs& in = P.in;
    const float2 nKf = pair(-P.Kf), ninv_dr = pair(-P.inv_drf);
    const float side = (float)g.side;
    for (int c0 = g.a; c0 < g.b;) {
        const int want = min(P.chunk, g.b - c0);
        __syncthreads();
        if (warp == 0) {
            int count = 0;
            if (lane < want) {
                const PulseRec pr = precs[c0 + lane];
                const float amag = sqrtf(pr.b.w);
                const float eps_max = pr.b.w / (2.0f * fmaxf(r_min - amag, 1.0f));
                const float hw = (amag + eps_max) * fabsf(P.inv_drf) + 1e-3f;
                const int bo = (int)floorf(-0.5f - hw), top = (int)ceilf(0.5f + hw);
                const long long cnt = (long long)I_span + top - bo + 1;
                count = cnt <= P.cap ? (int)cnt : P.cap + 1;
                s_base[lane] = I_first + bo;
                s_wt[lane] = pr.c.w;
                LeafRec r;
                r.p0 = make_float4(pr.c.z, pr.c.z, -pr.b.w, -pr.b.w);
                r.p1 = make_float4(pr.a.z, pr.a.z, pr.b.z, pr.b.z);
                const float Az = pr.a.z + pr.b.z;
                r.p2 = make_float4(Az, Az, pr.a.w, pr.a.w);
                r.w = make_int4(kMagicBits + bo, 0, count - 1, 0);
                rec[lane] = r;
            }
            int inc = count;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            const unsigned fits = __ballot_sync(0xffffffffu, lane < want && inc <= P.cap);
            if (lane < want) rec[lane].w.y = inc - count;
            if (lane == 0) s_nfit = __popc(fits);
        }
        __syncthreads();
        const int nfit = s_nfit;
        const int chn = nfit > 0 ? nfit : 1;
        for (int e = tid; e < (chn << lc); e += kThreads) {  // C, D per (pulse, column)
            const int nl = e >> lc, cc = e & (cols_t - 1);
            const float4 cv = __ldg(tables + g.cols_off + min(g.win_u0 + it.tile_u + cc, g.nu - 1));
            cols[nl * kLeafColStride + cc] = leaf_col(precs[c0 + nl], cv, side);
        }
        if (nfit > 0) {
            for (int nl = warp; nl < nfit; nl += kThreads / 32) {
                const int off = rec[nl].w.y;
                const int cnt = rec[nl].w.z + 1;
                const long long b0 = s_base[nl];
                const float a = s_wt[nl];
                const float2* row = in.data + (size_t)(c0 + nl) * in.samples;
                stage_window_shfl(row, in.samples, b0, cnt, a, win + 2 * off, lane);
            }
        }
        __syncthreads();
        if (nfit > 0) {
#pragma unroll 1
            for (int nl = 0; nl < nfit; ++nl) {
                const LeafRec R = rec[nl];
                const LeafCol Cc = cols[nl * kLeafColStride + col];
                const float4* wrow = win + 2 * R.w.y;
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    leaf_pair_pulse<true>(px[h], R, Cc, wrow, (unsigned)R.w.z, R.w.x, nullptr, I_first, in.samples, 0.0f,
                                          nKf, ninv_dr);
            }
        } else {  // one pulse whose window does not fit: its taps come straight from the pulse row
            const LeafRec R = rec[0];
            const LeafCol Cc = cols[col];
            const float2* drow = in.data + (size_t)c0 * in.samples;
#pragma unroll
            for (int h = 0; h < 2; ++h)
                leaf_pair_pulse<false>(px[h], R, Cc, nullptr, 0u, 0, drow, I_first, in.samples, s_wt[0], nKf, ninv_dr);
        }
        c0 += chn;
    }
    float2* dst = g.dst ? g.dst : (it.node == root ? root_out : arena + g.out_offset);
    const int wu = it.tile_u + col;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int wr0 = it.tile_r + (tid >> lc) + (kThreads >> lc) * (2 * h);
        const int wr1 = wr0 + (kThreads >> lc);
        if (wu < g.win_nu) {
            if (wr0 < g.win_nr) dst[(long long)wr0 * g.out_stride + wu] = make_float2(px[h].ar.x, px[h].ai.x);
            if (wr1 < g.win_nr) dst[(long long)wr1 * g.out_stride + wu] = make_float2(px[h].ar.y, px[h].ai.y);
        }
    }
}

__global__ void __launch_bounds__(kThreads, 3) split_leaf_kernel(SplitParams P, const PolarDesc* __restrict__ nodes,
                                                                 const TileItem* __restrict__ items,
                                                                 const float4* __restrict__ tables,
                                                                 const PulseRec* __restrict__ precs,
                                                                 float2* __restrict__ arena, float2* root_out,
                                                                 int root) {
    extern __shared__ __align__(16) char smem[];
    __shared__ int s_base[kMaxLeafChunk];
    __shared__ float s_wt[kMaxLeafChunk];
    __shared__ int s_nfit;
    leaf_tile(P, nodes, items[blockIdx.x], tables, precs, arena, root_out, root, smem, s_base, s_wt, s_nfit);
}

// ---- FFBP: merges (both child regrids of one parent tile) --------------------------------
struct ChildRec {
    float4 a;  // W_hi.x, W_hi.y, W_lo.x, W_lo.y
    float4 b;  // u.x, u.y, 2 RR, frac(Qr) - 1/2
    float4 c;  // Phi, h.x, h.y, 2 G
    float4 d;  // G, frac(Qu) - 1/2
    float inv_sdr, inv_sdu;
    int ir0, iu0, snr, snu;
    const float2* img;
    int sstr;           // row stride of the child image (elements)
    int br0, bu0;       // staged footprint: first row and (even) first column in the child image
    int bh, bw;         // footprint rows and columns; bw == 0: not staged
    const void* tmap;   // TMA tensor map of the child image (staged footprints only)
};

// Record of a polar image c seen from the ground point (px, py, 0), in two-float FP32
// arithmetic from the node geometry split on the host (PolarDesc::tf): the FP32 quantities
// child_value needs for points near it (a parent tile, or a lattice tile).  K in turns/m.
__device__ __forceinline__ ChildRec child_rec_at(FF K, float scale_w, float inv_scale_w, const PolarDesc& c, FF px,
                                                 FF py, const float2* img) {
    const FF vx = ff_add(px, ff_neg(ff_of(c.tf[0])));
    const FF vy = ff_add(py, ff_neg(ff_of(c.tf[1])));
    const FF vz = ff_neg(ff_of(c.tf[2]));
    const FF g2 = ff_add(ff_sqr(vx), ff_sqr(vy));
    const FF G = ff_sqrt(g2);
    const FF RR = ff_sqrt(ff_add(g2, ff_sqr(vz)));
    const FF iR = ff_rcp(RR), iG = ff_rcp(G);
    const FF ux = ff_mul(vx, iR), uy = ff_mul(vy, iR);
    const FF hy = ff_mul(vy, iG);
    const FF t = ff_mul(K, RR);
    float phi = (t.h - rintf(t.h)) + t.l;
    phi -= rintf(phi);
    float fr, fu;
    const FF Qr = ff_mul(ff_add(RR, ff_neg(ff_of(c.tf[3]))), ff_of(c.tf[7]));
    const FF Qu = ff_mul(ff_add(hy, ff_neg(ff_of(c.tf[5]))), ff_of(c.tf[8]));
    const float ir = ff_floor_frac(Qr, fr), iu = ff_floor_frac(Qu, fu);
    const FF Wx = ff_mul(K, ux), Wy = ff_mul(K, uy);
    ChildRec R;
    R.a.x = rintf(Wx.h * inv_scale_w) * scale_w;  // scale_w is a power of two: exact
    R.a.z = (Wx.h - R.a.x) + Wx.l;
    R.a.y = rintf(Wy.h * inv_scale_w) * scale_w;
    R.a.w = (Wy.h - R.a.y) + Wy.l;
    const float Gf = G.h + G.l;
    R.b = make_float4(ux.h + ux.l, uy.h + uy.l, 2.0f * (RR.h + RR.l), fr);
    R.c = make_float4(phi, ff_mul(vx, iG).h, hy.h + hy.l, 2.0f * Gf);
    R.d = make_float4(Gf, fu, 0.0f, 0.0f);
    R.inv_sdr = c.tf[7].x;
    R.inv_sdu = c.tf[8].x;
    const bool ok = fabsf(Qr.h) < 1.0e7f && fabsf(Qu.h) < 1.0e7f && G.h > 0.0f;  // false for NaN
    R.ir0 = ok ? (int)ir : -(1 << 30);
    R.iu0 = ok ? (int)iu : -(1 << 30);
    R.snr = c.nr;
    R.snu = c.nu;
    R.img = img;
    R.sstr = (int)c.out_stride;
    R.br0 = R.bu0 = R.bh = R.bw = 0;
    R.tmap = nullptr;
    return R;
}

// One thread per (merge tile, child).  The tile centre is the centre pixel's position from
// the node's row and column tables (two-float g and c, u), the same point setup_polar_tab
// measures the pixel offsets from.  With tensor maps (tmaps != NULL) a child whose node has a
// footprint box gets the box's origin in its image: box_r rows and box_u columns (rounded down
// to an even column, the TMA's 16-byte rule for 8-byte elements) before the centre's bin.
__device__ __forceinline__ void child_record(FF K, float scale_w, float inv_scale_w,
                                             const PolarDesc* __restrict__ nodes, const float4* __restrict__ tables,
                                             const TileItem it, int t, float2* __restrict__ arena,
                                             const void* tmaps, ChildRec* __restrict__ out) {
    const PolarDesc& g = nodes[it.node];
    const int ci = (t & 1) ? g.right : g.left;
    const PolarDesc& c = nodes[ci];
    const int cols_t = 1 << g.tile_lc, rows_t = kSplitTilePixels >> g.tile_lc;
    const int i0 = min(g.win_r0 + it.tile_r + (rows_t >> 1), g.nr - 1);
    const int j0 = min(g.win_u0 + it.tile_u + (cols_t >> 1), g.nu - 1);
    const float4 rv = __ldg(tables + g.rows_off + 3 * (long long)i0);
    const float4 cv = __ldg(tables + g.cols_off + j0);
    const FF g0{rv.x, rv.y};
    const FF gc = ff_mul(g0, FF{cv.x, cv.y});
    const FF px = ff_add(ff_of(g.tf[0]), g.side < 0 ? ff_neg(gc) : gc);
    const FF py = ff_add(ff_of(g.tf[1]), ff_mul(g0, FF{cv.z, cv.w}));
    ChildRec R = child_rec_at(K, scale_w, inv_scale_w, c, px, py, arena + c.out_offset);
    if (!(t & 1)) tab_quantum(g, g.tile_lc, it.tile_r, it.tile_u, tables, R.d.z, R.d.w);
    if (tmaps != nullptr && c.box_w > 0 && R.ir0 > -(1 << 30)) {
        R.br0 = R.ir0 - c.box_r;
        R.bu0 = (R.iu0 - c.box_u) & ~1;
        R.bh = c.box_h;
        R.bw = c.box_w;
        R.tmap = static_cast<const char*>(tmaps) + kTensorMapBytes * (size_t)ci;
    }
    out[t] = R;
}

__global__ void ffbp_child_records_kernel(float Kh, float Kl, float scale_w, float inv_scale_w,
                                          const PolarDesc* __restrict__ nodes, const float4* __restrict__ tables,
                                          const TileItem* __restrict__ items, int n_items,
                                          float2* __restrict__ arena, const void* tmaps, ChildRec* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n_items) return;
    child_record(FF{Kh, Kl}, scale_w, inv_scale_w, nodes, tables, items[t >> 1], t, arena, tmaps, out);
}

// Child-image coordinates of a parent pixel: bin indices (ir, iu), centred fractions
// (sr, su) and the second-order range term eps.  ok: the 4x4 stencil lies inside the child.
struct ChildCoord {
    int ir, iu;
    float sr, su, eps;
    bool ok;
};

__device__ __forceinline__ ChildCoord child_coords(const ChildRec& R, const Pix& q) {
    ChildCoord c;
    const float L = fmaf(R.b.x, q.dx, R.b.y * q.dy);
    const float q2 = fmaf(-L, L, q.d2);
    const float B = rcp_approx(fmaf(2.0f, L, R.b.z));
    const float e0 = q2 * B;
    c.eps = fmaf(-e0 * e0, B, e0);
    const float qr = fmaf(L + c.eps, R.inv_sdr, R.b.w);
    const float tr = qr + kMagic;
    c.sr = qr - (tr - kMagic);
    c.ir = R.ir0 + (__float_as_int(tr) - kMagicBits);
    const float Lh = fmaf(R.c.y, q.dx, R.c.z * q.dy);
    const float q2h = fmaf(-Lh, Lh, q.d2);
    const float Bh = rcp_approx(fmaf(2.0f, Lh, R.c.w));
    const float eh = q2h * Bh;
    const float dG = Lh + fmaf(-eh * eh, Bh, eh);
    const float gp = R.d.x + dG;
    const float duu = fmaf(-R.c.z, dG, q.dy) * rcp_approx(gp);
    const float qu = fmaf(duu, R.inv_sdu, R.d.y);
    const float tu = qu + kMagic;
    c.su = qu - (tu - kMagic);
    c.iu = R.iu0 + (__float_as_int(tu) - kMagicBits);
    c.ok = c.ir >= 1 && c.ir <= R.snr - 3 && c.iu >= 1 && c.iu <= R.snu - 3 && gp > 0.0f;
    return c;
}

__device__ __forceinline__ float2 child_value(float Kf, const ChildRec& R, const Pix& q) {
    const ChildCoord c = child_coords(R, q);
    float vr = 0.0f, vi = 0.0f;
    if (c.ok) {
        float wr[4], wu[4];
        lagrange_centred(c.sr, wr);
        lagrange_centred(c.su, wu);
        const float2* base = R.img + (size_t)(c.ir - 1) * R.sstr + (c.iu - 1);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const float2* row = base + (size_t)a * R.sstr;
            const float2 x0 = __ldg(row), x1 = __ldg(row + 1), x2 = __ldg(row + 2), x3 = __ldg(row + 3);
            float rr = wu[0] * x0.x, ri = wu[0] * x0.y;
            rr = fmaf(wu[1], x1.x, rr);
            ri = fmaf(wu[1], x1.y, ri);
            rr = fmaf(wu[2], x2.x, rr);
            ri = fmaf(wu[2], x2.y, ri);
            rr = fmaf(wu[3], x3.x, rr);
            ri = fmaf(wu[3], x3.y, ri);
            vr = fmaf(wr[a], rr, vr);
            vi = fmaf(wr[a], ri, vi);
        }
    }
    const float tb = fmaf(R.a.x, q.dxh, R.a.y * q.dyh);
    float sm = fmaf(Kf, c.eps, R.c.x);
    sm = fmaf(R.a.x, q.dxl, sm);
    sm = fmaf(R.a.y, q.dyl, sm);
    sm = fmaf(R.a.z, q.dx, sm);
    sm = fmaf(R.a.w, q.dy, sm);
    const float tot = (tb - round_magic(tb)) + (sm + q.psi);
    const float ang = (tot - round_magic(tot)) * kTwoPiF;
    float sn, cs;
    __sincosf(ang, &sn, &cs);
    return make_float2(vr * cs - vi * sn, vr * sn + vi * cs);
}

// Child records of a merge tile for the packed merge: every field of one child as a duplicated
// (x, x) pair, so that a chain over two parent pixels (the two lanes of f32x2 operations) takes
// each operand with one 8-byte shared load.  Negated copies stand in for the scalar code's
// subtractions (negation is exact), so every lane equals child_value's arithmetic bit for bit.
struct __align__(16) ChildDup {
    float2 nbx, nby;   // -u.x, -u.y
    float2 bz, bw;     // 2 RR, frac(Qr) - 1/2
    float2 ncy, ncz;   // -h.x, -h.y
    float2 cz, cw;     // h.y, 2 G
    float2 dx, dy;     // G, frac(Qu) - 1/2
    float2 nisr, isu;  // -1/sdr, 1/sdu
    float2 ax, ay;     // W_hi.x, W_hi.y
    float2 az, aw;     // W_lo.x, W_lo.y
    float2 cx;         // Phi
    int ir0, iu0, snr, snu;
    const float2* img;
    int sstr;          // row stride of the child image
    int xr0, xu0, xh, xw;  // staged footprint: first row, first column, rows, columns (xw == 0: not staged)
};

__device__ __forceinline__ void child_dup_store(const ChildRec& R, ChildDup& P) {
    P.nbx = pair(-R.b.x);
    P.nby = pair(-R.b.y);
    P.bz = pair(R.b.z);
    P.bw = pair(R.b.w);
    P.ncy = pair(-R.c.y);
    P.ncz = pair(-R.c.z);
    P.cz = pair(R.c.z);
    P.cw = pair(R.c.w);
    P.dx = pair(R.d.x);
    P.dy = pair(R.d.y);
    P.nisr = pair(-R.inv_sdr);
    P.isu = pair(R.inv_sdu);
    P.ax = pair(R.a.x);
    P.ay = pair(R.a.y);
    P.az = pair(R.a.z);
    P.aw = pair(R.a.w);
    P.cx = pair(R.c.x);
    P.ir0 = R.ir0;
    P.iu0 = R.iu0;
    P.snr = R.snr;
    P.snu = R.snu;
    P.img = R.img;
    P.sstr = R.sstr;
    P.xr0 = R.br0;
    P.xu0 = R.bu0;
    P.xh = R.bh;
    P.xw = R.bw;
}

// Offsets of the parent pixels (row, col) and (row + 1, col) from the tile centre as (upper,
// lower) lane pairs, row even: tab_pixel's arithmetic lane by lane, with d2 negated (exact).
struct VPix {
    float2 dx, dy, dxh, dyh, dxl, dyl, nd2, psi;
};

__device__ __forceinline__ float2 ld_pair(const float* p) { return *reinterpret_cast<const float2*>(p); }

__device__ __forceinline__ VPix tab_vpair(const TabF& T, int row, int col) {
    VPix v;
    v.dxh = __fadd2_rn(ld_pair(T.rxh + row), pair(T.cxh[col]));  // exact: both multiples of the quantum
    v.dyh = __fadd2_rn(ld_pair(T.ryh + row), pair(T.cyh[col]));
    const float2 dg = ld_pair(T.dg + row);
    v.dxl = __ffma2_rn(dg, pair(T.dcs[col]), __fadd2_rn(ld_pair(T.rxl + row), pair(T.cxl[col])));
    v.dyl = __ffma2_rn(dg, pair(T.duu[col]), __fadd2_rn(ld_pair(T.ryl + row), pair(T.cyl[col])));
    v.dx = __fadd2_rn(v.dxh, v.dxl);
    v.dy = __fadd2_rn(v.dyh, v.dyl);
    v.nd2 = __fmul2_rn(__ffma2_rn(v.dx, v.dx, __fmul2_rn(v.dy, v.dy)), pair(-1.0f));
    v.psi = ld_pair(T.psi + row);
    return v;
}

// lagrange_centred for two fractions at once (the lanes of f32x2 operations), per lane the same
// operations and roundings: -a/6, -c2 and -s are the scalar code's a/6, c2 and s negated (exact).
__device__ __forceinline__ void lagrange_centred2(float2 s, float2 w[4]) {
    const float2 a = __ffma2_rn(s, s, pair(-0.25f));
    const float2 na6 = __fmul2_rn(a, pair(-1.0f / 6.0f));
    const float2 b2 = __ffma2_rn(a, pair(0.5f), pair(-1.0f));
    const float2 c1 = __fmul2_rn(pair(-1.5f), na6);
    const float2 nc2 = __fmul2_rn(pair(-0.5f), b2);
    const float2 ns = __fmul2_rn(s, pair(-1.0f));
    w[0] = __ffma2_rn(na6, s, c1);
    w[3] = __ffma2_rn(na6, ns, c1);
    w[1] = __ffma2_rn(b2, s, nc2);
    w[2] = __ffma2_rn(b2, ns, nc2);
}

// Where a stencil's taps come from: the child image through the read-only path (kLdg), the
// child image with weak coherent loads (kCoherent: the merge queue, whose child images were
// written by other CTAs of the same launch; L1-cached, ordered by the acquire that made the
// node ready), or the tile's staged footprint in shared memory (kShared).
enum TapSource { kLdg = 0, kCoherent = 1, kShared = 2 };

// The coherent asm has no memory clobber, so the compiler schedules it as freely as __ldg; its
// address comes from values read after the CTA barrier that follows the acquire.
template <int SRC>
__device__ __forceinline__ void ld_child_row(const float2* p, float2& x0, float2& x1, float2& x2, float2& x3) {
    if (SRC == kCoherent) {
        asm("ld.global.v2.f32 {%0, %1}, [%8];\n\t"
            "ld.global.v2.f32 {%2, %3}, [%8+8];\n\t"
            "ld.global.v2.f32 {%4, %5}, [%8+16];\n\t"
            "ld.global.v2.f32 {%6, %7}, [%8+24];"
            : "=f"(x0.x), "=f"(x0.y), "=f"(x1.x), "=f"(x1.y), "=f"(x2.x), "=f"(x2.y), "=f"(x3.x), "=f"(x3.y)
            : "l"(p));
    } else if (SRC == kShared) {
        x0 = p[0];
        x1 = p[1];
        x2 = p[2];
        x3 = p[3];
    } else {
        x0 = __ldg(p);
        x1 = __ldg(p + 1);
        x2 = __ldg(p + 2);
        x3 = __ldg(p + 3);
    }
}

// 4x4 Lagrange stencil whose first tap is base (rows `stride` elements apart) with weights wr
// (range) and wu (angle); (re, im) run as one f32x2 pair.
template <int SRC>
__device__ __forceinline__ float2 child_stencil(const float2* base, int stride, const float wr[4], const float wu[4]) {
    float2 v = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        float2 x0, x1, x2, x3;
        ld_child_row<SRC>(base + (size_t)a * stride, x0, x1, x2, x3);
        float2 r = __fmul2_rn(pair(wu[0]), x0);
        r = __ffma2_rn(pair(wu[1]), x1, r);
        r = __ffma2_rn(pair(wu[2]), x2, r);
        r = __ffma2_rn(pair(wu[3]), x3, r);
        v = __ffma2_rn(pair(wr[a]), r, v);
    }
    return v;
}

// The two stencils of a vertical pair that share three rows: one 5x4 block from row (base),
// the upper pixel's stencil in rows 0-3, the lower one's in rows 1-4 (the same sums as
// child_stencil per pixel).
template <int SRC>
__device__ __forceinline__ void child_pair_block(const float2* base, int stride, const float wrA[4],
                                                 const float wuA[4], const float wrB[4], const float wuB[4],
                                                 float2& vA, float2& vB) {
#pragma unroll
    for (int a = 0; a < 5; ++a) {
        float2 x0, x1, x2, x3;
        ld_child_row<SRC>(base + (size_t)a * stride, x0, x1, x2, x3);
        if (a < 4) {
            float2 r = __fmul2_rn(pair(wuA[0]), x0);
            r = __ffma2_rn(pair(wuA[1]), x1, r);
            r = __ffma2_rn(pair(wuA[2]), x2, r);
            r = __ffma2_rn(pair(wuA[3]), x3, r);
            vA = __ffma2_rn(pair(wrA[a]), r, vA);
        }
        if (a > 0) {
            float2 r = __fmul2_rn(pair(wuB[0]), x0);
            r = __ffma2_rn(pair(wuB[1]), x1, r);
            r = __ffma2_rn(pair(wuB[2]), x2, r);
            r = __ffma2_rn(pair(wuB[3]), x3, r);
            vB = __ffma2_rn(pair(wrB[a - 1]), r, vB);
        }
    }
}

// Child C at the column pair q (lanes: the upper and the lower parent pixel), rotated: per lane
// child_value's arithmetic (the Lagrange weights, the stencil's sum order and the rotation are
// the same).  Two vertically adjacent parent pixels nearly always fall one child range bin apart
// in the same angle column (a parent range step is one child range step, shortened by the
// cosine of the angle between the two phase centres' lines of sight), so their 4x4 stencils
// share three rows: when that holds for every lane of the warp, the pair gathers one 5x4 block
// (20 loads instead of 32).  Otherwise each pixel gathers its own stencil.
// sbox (STAGED, not NULL): the child's footprint staged in shared memory (C.xh x C.xw elements
// from row C.xr0, column C.xu0); a warp whose pairs all share a block inside it reads the blocks
// from shared memory, any other warp gathers each pixel's stencil from the child image (staged
// kernels have no other paths: fewer code paths keep their loop in the instruction cache).  The
// taps are the same values either way.
template <bool COHERENT, bool STAGED>
__device__ __forceinline__ void child_vpair(float Kf, const ChildDup& C, const VPix& q, float2& oA, float2& oB,
                                            const float2* sbox) {
    constexpr int SRC = COHERENT ? kCoherent : kLdg;
    const float2 magic = pair(kMagic), nmagic = pair(-kMagic), mone = pair(-1.0f);
    const float2 nL = __ffma2_rn(C.nbx, q.dx, __fmul2_rn(C.nby, q.dy));
    const float2 nq2 = __ffma2_rn(nL, nL, q.nd2);
    const float2 den = __ffma2_rn(pair(-2.0f), nL, C.bz);
    const float2 B = make_float2(rcp_approx(den.x), rcp_approx(den.y));
    const float2 ne0 = __fmul2_rn(nq2, B);
    const float2 neps = __ffma2_rn(__fmul2_rn(ne0, ne0), B, ne0);
    const float2 tb = __ffma2_rn(C.ax, q.dxh, __fmul2_rn(C.ay, q.dyh));
    float2 sm = __ffma2_rn(pair(-Kf), neps, C.cx);
    sm = __ffma2_rn(C.ax, q.dxl, sm);
    sm = __ffma2_rn(C.ay, q.dyl, sm);
    sm = __ffma2_rn(C.az, q.dx, sm);
    sm = __ffma2_rn(C.aw, q.dy, sm);
    const float2 rtb = __fadd2_rn(__fadd2_rn(tb, magic), nmagic);
    const float2 tot = __fadd2_rn(__ffma2_rn(rtb, mone, tb), __fadd2_rn(sm, q.psi));
    const float2 rtot = __fadd2_rn(__fadd2_rn(tot, magic), nmagic);
    const float2 ang = __fmul2_rn(__ffma2_rn(rtot, mone, tot), pair(kTwoPiF));
    float snA, csA, snB, csB;
    __sincosf(ang.x, &snA, &csA);
    __sincosf(ang.y, &snB, &csB);
    const float2 qr = __ffma2_rn(__fadd2_rn(nL, neps), C.nisr, C.bw);
    const float2 tr = __fadd2_rn(qr, magic);
    const float2 sr = __ffma2_rn(__fadd2_rn(tr, nmagic), mone, qr);
    const float2 nLh = __ffma2_rn(C.ncy, q.dx, __fmul2_rn(C.ncz, q.dy));
    const float2 nq2h = __ffma2_rn(nLh, nLh, q.nd2);
    const float2 denh = __ffma2_rn(pair(-2.0f), nLh, C.cw);
    const float2 Bh = make_float2(rcp_approx(denh.x), rcp_approx(denh.y));
    const float2 neh = __fmul2_rn(nq2h, Bh);
    const float2 ndG = __fadd2_rn(nLh, __ffma2_rn(__fmul2_rn(neh, neh), Bh, neh));
    const float2 gp = __ffma2_rn(ndG, mone, C.dx);
    const float2 num = __ffma2_rn(C.cz, ndG, q.dy);
    const float2 duu = __fmul2_rn(num, make_float2(rcp_approx(gp.x), rcp_approx(gp.y)));
    const float2 qu = __ffma2_rn(duu, C.isu, C.dy);
    const float2 tu = __fadd2_rn(qu, magic);
    const float2 su = __ffma2_rn(__fadd2_rn(tu, nmagic), mone, qu);
    const int irA = C.ir0 + (__float_as_int(tr.x) - kMagicBits), irB = C.ir0 + (__float_as_int(tr.y) - kMagicBits);
    const int iuA = C.iu0 + (__float_as_int(tu.x) - kMagicBits), iuB = C.iu0 + (__float_as_int(tu.y) - kMagicBits);
    const bool okA = irA >= 1 && irA <= C.snr - 3 && iuA >= 1 && iuA <= C.snu - 3 && gp.x > 0.0f;
    const bool okB = irB >= 1 && irB <= C.snr - 3 && iuB >= 1 && iuB <= C.snu - 3 && gp.y > 0.0f;
    const bool share = okA && okB && irB == irA + 1 && iuB == iuA;
    float2 vA = make_float2(0.0f, 0.0f), vB = vA;
    // The pair's block origin relative to the staged footprint (at least 8 x 8 elements when staged).
    const int rA = irA - 1 - C.xr0, uA = iuA - 1 - C.xu0;
    if (STAGED && sbox != nullptr && __all_sync(0xffffffffu, share && (unsigned)rA <= (unsigned)(C.xh - 5) &&
                                              (unsigned)uA <= (unsigned)(C.xw - 4))) {
        float wrA[4], wuA[4], wrB[4], wuB[4];
        float2 wr2[4], wu2[4];
        lagrange_centred2(sr, wr2);  // both pixels' weights as lane pairs
        lagrange_centred2(su, wu2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            wrA[k] = wr2[k].x;
            wrB[k] = wr2[k].y;
            wuA[k] = wu2[k].x;
            wuB[k] = wu2[k].y;
        }
        child_pair_block<kShared>(sbox + rA * C.xw + uA, C.xw, wrA, wuA, wrB, wuB, vA, vB);
    } else if (!STAGED && __all_sync(0xffffffffu, share)) {
        float wrA[4], wuA[4], wrB[4], wuB[4];
        lagrange_centred(sr.x, wrA);
        lagrange_centred(su.x, wuA);
        lagrange_centred(sr.y, wrB);
        lagrange_centred(su.y, wuB);
        child_pair_block<SRC>(C.img + (size_t)(irA - 1) * C.sstr + (iuA - 1), C.sstr, wrA, wuA, wrB, wuB, vA, vB);
    } else {
        if (okA) {
            float wr[4], wu[4];
            lagrange_centred(sr.x, wr);
            lagrange_centred(su.x, wu);
            vA = child_stencil<SRC>(C.img + (size_t)(irA - 1) * C.sstr + (iuA - 1), C.sstr, wr, wu);
        }
        if (okB) {
            float wr[4], wu[4];
            lagrange_centred(sr.y, wr);
            lagrange_centred(su.y, wu);
            vB = child_stencil<SRC>(C.img + (size_t)(irB - 1) * C.sstr + (iuB - 1), C.sstr, wr, wu);
        }
    }
    // (vr cs - vi sn, vr sn + vi cs)
    oA = __ffma2_rn(pair(vA.x), make_float2(csA, snA), __fmul2_rn(pair(vA.y), make_float2(-snA, csA)));
    oB = __ffma2_rn(pair(vB.x), make_float2(csB, snB), __fmul2_rn(pair(vB.y), make_float2(-snB, csB)));
}

// Bytes of a merge tile's tables in dynamic shared memory (the staged footprints follow them).
constexpr int kTabBytes = (int)((sizeof(TabF) + 127) / 128 * 128);

// Staged merge tiles: one thread starts the TMA copies of both children's footprints (2-D tiles
// of the child images, the box's first column even so that it starts on a 16-byte boundary;
// rows or columns outside the image arrive as zeros and are never read, since such stencils
// fail the bounds test) with completion on one mbarrier.  Child 1's footprint follows child 0's
// at the next 128-byte boundary.  withhold: bytes declared on the mbarrier beyond those the copies
// deliver (0; 16 in tests of the wait limit, whose phase then never completes).
__device__ __forceinline__ void stage_children(const ChildRec* __restrict__ crec, unsigned box0, unsigned bar,
                                               unsigned withhold) {
    const int bw0 = crec[0].bw, bw1 = crec[1].bw;
    const unsigned b0 = bw0 > 0 ? (unsigned)(crec[0].bh * bw0 * 8) : 0u;
    const unsigned b1 = bw1 > 0 ? (unsigned)(crec[1].bh * bw1 * 8) : 0u;
    if (b0 + b1 == 0) return;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(b0 + b1 + withhold)
                 : "memory");
    if (b0)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
            ::"r"(box0), "l"(crec[0].tmap), "r"(crec[0].bu0), "r"(crec[0].br0), "r"(bar)
            : "memory");
    if (b1)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
            ::"r"(box0 + (b0 + 127u) / 128u * 128u), "l"(crec[1].tmap), "r"(crec[1].bu0), "r"(crec[1].br0), "r"(bar)
            : "memory");
}

// One merge tile: both children regridded onto the parent tile, each rounded to complex64,
// then added (the reference's rounding points).  crec points at the tile's two child records.
// Thread t of THREADS forms the column pairs (rows 2 m and 2 m + 1 of column t mod cols) for
// m = t / cols + i THREADS / cols; its offsets come back from the shared tables per pair, which
// keeps the live state small.
// STAGED: smem is 128-byte aligned and holds [tables | child 0's footprint | child 1's], which
// stage_children's copies fill (completion on the mbarrier at shared address bar).  Each warp
// waits for them, at most wait_ns; a warp whose wait runs out counts a timeout and gathers from
// the child images instead (the same values), and waits once more, as long, before the CTA ends,
// so that no copy into its shared memory is still in flight when it exits.
template <bool COHERENT = false, int THREADS = kThreads, bool STAGED = false>
__device__ __forceinline__ void merge_tile(float Kf, const PolarDesc* __restrict__ nodes, const TileItem it,
                                           const float4* __restrict__ tables, const ChildRec* __restrict__ crec,
                                           ChildDup* C, float2* __restrict__ arena, float2* root_out, int root,
                                           char* smem, unsigned bar = 0, unsigned long long wait_ns = 0) {
    Job J;
    J.g = nodes[it.node];
    J.lc = J.g.tile_lc;
    J.tile_r = it.tile_r;
    J.tile_u = it.tile_u;
    if (threadIdx.x < 2) child_dup_store(crec[threadIdx.x], C[threadIdx.x]);
    const float4 d0 = __ldg(&crec[0].d);  // (G, frac(Qu) - 1/2, tile quantum, its inverse)
    TabF& T = *reinterpret_cast<TabF*>(smem);
    setup_polar_tab<THREADS>(J, T, tables, d0.z, d0.w);
    const float2* sbox[2] = {nullptr, nullptr};
    bool waited = true;
    if (STAGED && (C[0].xw > 0 || C[1].xw > 0)) {
        waited = __all_sync(0xffffffffu, timed_wait(bar, 0, wait_ns));
        if (!waited) {
            if ((threadIdx.x & 31) == 0) atomicAdd(&g_wait_timeouts, 1);
        } else {
            const float2* b0 = reinterpret_cast<const float2*>(smem + kTabBytes);
            if (C[0].xw > 0) sbox[0] = b0;
            if (C[1].xw > 0)
                sbox[1] = b0 + (C[0].xw > 0 ? (int)split_box_bytes(C[0].xh, C[0].xw) / 8 : 0);
        }
    }
    float2* dst = J.g.dst ? J.g.dst : (it.node == root ? root_out : arena + J.g.out_offset);
    const int col = threadIdx.x & ((1 << J.lc) - 1), wu = J.tile_u + col;
    constexpr int kPairs = kSplitTilePixels / (2 * THREADS);  // column pairs per thread
    float2 m[2 * kPairs];
    // Gathering tiles keep all their pairs' gathers in flight (unrolled); staged tiles read shared
    // memory with short latency, and the smaller loop body keeps their instruction cache warm.
    constexpr int kUnroll = STAGED ? 1 : kPairs;
#pragma unroll kUnroll
    for (int k = 0; k < kPairs; ++k) {
        const int row = 2 * ((threadIdx.x >> J.lc) + (THREADS >> J.lc) * k);
        const VPix v = tab_vpair(T, row, col);
        float2 a0, b0, a1, b1;
        child_vpair<COHERENT, STAGED>(Kf, C[0], v, a0, b0, sbox[0]);
        child_vpair<COHERENT, STAGED>(Kf, C[1], v, a1, b1, sbox[1]);
        const float2 mA = __fadd2_rn(a0, a1), mB = __fadd2_rn(b0, b1);
        if (!COHERENT) {
            const int wr = J.tile_r + row;
            if (wu < J.g.win_nu) {
                if (wr < J.g.win_nr) dst[(long long)wr * J.g.out_stride + wu] = mA;
                if (wr + 1 < J.g.win_nr) dst[(long long)(wr + 1) * J.g.out_stride + wu] = mB;
            }
        } else {
            // Coherent child loads may not pass this thread's earlier image stores, so the
            // results are stored after the last gather.
            m[2 * k] = mA;
            m[2 * k + 1] = mB;
        }
    }
    if (COHERENT) {
#pragma unroll
        for (int k = 0; k < kPairs; ++k) {
            const int wr = J.tile_r + 2 * ((threadIdx.x >> J.lc) + (THREADS >> J.lc) * k);
            if (wu < J.g.win_nu) {
                if (wr < J.g.win_nr) dst[(long long)wr * J.g.out_stride + wu] = m[2 * k];
                if (wr + 1 < J.g.win_nr) dst[(long long)(wr + 1) * J.g.out_stride + wu] = m[2 * k + 1];
            }
        }
    }
    if (STAGED && !waited) timed_wait(bar, 0, wait_ns);  // the copies may still land: not past the CTA's end
}

__global__ void __launch_bounds__(kMergeThreads, 8) split_merge_kernel(SplitParams P, const PolarDesc* __restrict__ nodes,
                                                                  const TileItem* __restrict__ items,
                                                                  const float4* __restrict__ tables,
                                                                  const ChildRec* __restrict__ crecs,
                                                                  float2* __restrict__ arena, float2* root_out,
                                                                  int root) {
    extern __shared__ __align__(16) char smem[];
    __shared__ ChildDup C[2];
    merge_tile<false, kMergeThreads>(P.Kf, nodes, items[blockIdx.x], tables, crecs + 2 * (long long)blockIdx.x, C, arena,
                                     root_out, root, smem);
}

// The merge with both children's footprints staged in shared memory by TMA (tiles whose child
// records carry tensor maps; any other child gathers from its image as in split_merge_kernel).
// The dynamic shared memory is 128 bytes of alignment slack, the tables and the footprints.
__global__ void __launch_bounds__(kMergeThreads, 8) split_merge_staged_kernel(SplitParams P,
                                                                         const PolarDesc* __restrict__ nodes,
                                                                         const TileItem* __restrict__ items,
                                                                         const float4* __restrict__ tables,
                                                                         const ChildRec* __restrict__ crecs,
                                                                         float2* __restrict__ arena,
                                                                         float2* root_out, int root,
                                                                         unsigned long long wait_ns, int withheld) {
    extern __shared__ __align__(128) char smem_raw[];
    __shared__ ChildDup C[2];
    __shared__ __align__(8) unsigned long long mbar;
    const unsigned raw = (unsigned)__cvta_generic_to_shared(smem_raw);
    char* smem = smem_raw + (((raw + 127u) & ~127u) - raw);
    const unsigned bar = (unsigned)__cvta_generic_to_shared(&mbar);
    const ChildRec* crec = crecs + 2 * (long long)blockIdx.x;
    const TileItem it = items[blockIdx.x];
    if (threadIdx.x == 0)
        stage_children(crec, (unsigned)__cvta_generic_to_shared(smem + kTabBytes), bar, it.node == withheld ? 16u : 0u);
    merge_tile<false, kMergeThreads, true>(P.Kf, nodes, it, tables, crec, C, arena, root_out, root, smem, bar, wait_ns);
}

// All merge levels in one persistent launch.  Items are in height order; a CTA claims the next
// item and waits (bounded) until the item's node has no unfinished merge children.  Every
// dependency of an item has a lower index, so it is held by a running CTA (or finished) and the
// wait ends.  A finished tile counts down its node's tiles; the node's last tile counts down its
// parent's pending children.  A wait that runs out sets *status and every CTA stops.
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}


__global__ void __launch_bounds__(kThreads, 4) split_merge_queue_kernel(SplitParams P, const PolarDesc* __restrict__ nodes,
                                                                        const TileItem* __restrict__ items, int nitems,
                                                                        const float4* __restrict__ tables,
                                                                        const ChildRec* __restrict__ crecs,
                                                                        float2* arena, float2* root_out, int root,
                                                                        MergeQueue Q) {
    extern __shared__ __align__(16) char smem[];
    __shared__ ChildDup C[2];
    __shared__ int s_item, s_ok;
    for (;;) {
        if (threadIdx.x == 0) {
            const int idx = atomicAdd(Q.next, 1);
            int ok = 1;
            if (idx < nitems) {
                const int node = items[idx].node;
                const unsigned long long t0 = global_ns();
                while (ld_acquire_gpu(Q.pending + node) > 0) {
                    if (ld_acquire_gpu(Q.status) != 0) {  // another CTA gave up: stop too
                        ok = 0;
                        break;
                    }
                    if (global_ns() - t0 > Q.limit_ns) {
                        atomicExch(Q.status, 1);
                        ok = 0;
                        break;
                    }
                    __nanosleep(200);
                }
            }
            s_item = idx;
            s_ok = ok;
        }
        __syncthreads();
        const int idx = s_item;
        if (idx >= nitems || !s_ok) return;
        const TileItem it = items[idx];
        merge_tile<true>(P.Kf, nodes, it, tables, crecs + 2 * (long long)idx, C, arena, root_out, root, smem);
        __syncthreads();  // every thread's writes of this tile are issued
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicSub(Q.remaining + it.node, 1) == 1) {
                __threadfence();
                const int parent = Q.parent[it.node];
                if (parent >= 0) atomicSub(Q.pending + parent, 1);
            }
        }
    }
}

SplitParams make_params(const PulseInputs& in, int chunk, int cap, int pulse_split) {
    SplitParams P;
    P.in = in;
    P.out = nullptr;
    P.out_stride = 0;
    P.K = in.k * kInvTwoPi;
    P.inv_dr = in.data_dr != 0.0 ? 1.0 / in.data_dr : 0.0;
    int e = 0;
    frexp(fabs(P.K) > 0.0 ? fabs(P.K) : 1e-30, &e);
    P.scale_w = ldexp(1.0, e - 10);
    P.inv_scale_w = ldexp(1.0, 10 - e);
    P.Kf = (float)P.K;
    P.inv_drf = (float)P.inv_dr;
    P.chunk = chunk < 1 ? 1 : (chunk > kMaxChunk ? kMaxChunk : chunk);
    P.cap = cap < 64 ? 64 : cap;  // >= kMaxChunk two-float records (32 bytes each) fit the window space
    P.pulse_split = pulse_split;
    P.split_stride = 0;
    P.envelope = kDirectEnvelope;
    P.Kh = (float)P.K;
    P.Kl = (float)(P.K - (double)P.Kh);
    P.rsh = (float)in.range_start;
    P.rsl = (float)(in.range_start - (double)P.rsh);
    P.idrh = (float)P.inv_dr;
    P.idrl = (float)(P.inv_dr - (double)P.idrh);
    return P;
}

size_t merge_smem() { return sizeof(TabF); }

size_t dynamic_smem(int cap, bool polar) {
    size_t win = (size_t)cap * 32;
    if (polar && win < sizeof(PolarTables)) win = sizeof(PolarTables);
    return window_offset() + win + raw_bytes_for(cap, kMaxChunk);
}

template <class K>
int prepare(K kernel, size_t smem) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    }
    return SARBP_OK;
}

// Pulse split that fills the GPU's CTA slots best: the fewest waves ceil(tiles s / slots) / s over
// s <= 8 (and <= pulses), ties to the smaller split.  A tile's pulse ranges are independent
// work, so a small image with few tiles still keeps every SM busy to the end.
template <class K>
int best_pulse_split(K kernel, size_t smem, long long tiles, int pulses) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem) != cudaSuccess || per_sm <= 0 ||
        sms <= 0 || tiles <= 0) {
        cudaGetLastError();
        return 1;
    }
    const long long slots = (long long)sms * per_sm;
    int best = 1;
    double best_waves = 1e300;
    for (int sp = 1; sp <= 8 && sp <= pulses; ++sp) {
        const double waves = (double)((tiles * sp + slots - 1) / slots) / sp;
        if (waves < best_waves - 1e-9) {
            best_waves = waves;
            best = sp;
        }
    }
    return best;
}

int tiles_of(int nr, int nu, int lc) {
    const int cols_t = 1 << lc, rows_t = kSplitTilePixels >> lc;
    return ((nr + rows_t - 1) / rows_t) * ((nu + cols_t - 1) / cols_t);
}

// Window entries for one chunk: `chunk` pulses whose windows span at most
// `window_bins` bins each (the kernel packs the actual, usually smaller, windows).
int capacity_for(int chunk, int window_bins, int budget_bytes = kWindowBudget) {
    long long cap = (long long)chunk * window_bins;
    // With bulk staging a window bin also needs 8 bytes of raw samples (plus a fixed margin).
    // (2 KB more are left for the bulk path's larger static shared memory.)
    const long long budget =
        SARBP_BULK_WINDOWS ? (budget_bytes - raw_bytes_for(0, kMaxChunk) - 2048) / 40 : budget_bytes / 32;
    return (int)(cap > budget ? budget : cap);
}

// Leaf window entries: the windows share the CTA's shared memory with the chunk's pulse and
// (pulse, column) records, within the same per-CTA total as the direct kernels' windows.
int leaf_capacity(int chunk, int window_bins) {
    return capacity_for(chunk, window_bins, kWindowBudget - (int)leaf_window_offset(chunk));
}

}  // namespace

int split_window_bins(double radius, double data_dr) {
    // Worst case: the pixel offset lies along the line of sight; eps <= radius^2/(2(R - radius)) is
    // small at any range used here (R >= 100 m gives the bound below).
    const double wing = (radius + radius * radius / 200.0) / fabs(data_dr) + 0.01;
    return (int)ceil(2.0 * wing) + 4;
}

int split_chunk_for(int window_bins, int requested, bool leaf) {
    const int most = leaf ? kMaxLeafChunk : kMaxChunk;
    int ch = requested > 0 ? requested : most;
    if (ch > most) ch = most;
    const int fit = kWindowBudget / (window_bins * 32 > 0 ? window_bins * 32 : 32);
    if (ch > fit) ch = fit;
    return ch < 1 ? 1 : ch;
}

int split_polar_tile_lc(const PolarDesc& g, double* radius) { return split_polar_tile_lc_slack(g, 1.0, radius); }

int split_polar_tile_lc_slack(const PolarDesc& g, double slack, double* radius) {
    // Ground displacement per range row <= dr * r / g; per angle column <= du * g / sqrt(1 - u^2).
    const double rmin = g.r0 + g.win_r0 * g.dr, rmax = g.r0 + (g.win_r0 + g.win_nr - 1) * g.dr;
    const double gmin = sqrt(fmax(1e-6, rmin * rmin - g.oz * g.oz));
    const double gmax = sqrt(fmax(1e-6, rmax * rmax - g.oz * g.oz));
    const double ua = fabs(g.u0 + g.win_u0 * g.du), ub = fabs(g.u0 + (g.win_u0 + g.win_nu - 1) * g.du);
    const double cmin = sqrt(fmax(1e-6, 1.0 - fmax(ua, ub) * fmax(ua, ub)));
    const double per_row = fabs(g.dr) * fmax(rmin, rmax) / gmin;
    const double per_col = fabs(g.du) * gmax / cmin;
    double rads[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int best = 5;
    double best_r = 1e300;
    for (int lc = 2; lc <= 5; ++lc) {
        const double er = (kSplitTilePixels >> lc) * per_row, eu = (1 << lc) * per_col;
        rads[lc] = 0.5 * sqrt(er * er + eu * eu) * 1.05;
        if (rads[lc] < best_r) {
            best_r = rads[lc];
            best = lc;
        }
    }
    // The widest shape within `slack` of the smallest radius (wider tiles keep a warp's pixels in
    // fewer rows).
    for (int lc = 5; lc > best; --lc)
        if (rads[lc] <= slack * best_r) {
            best = lc;
            break;
        }
    if (radius) *radius = rads[best];
    return best;
}

int launch_split_polar(const PulseInputs& in, const PolarDesc& g, int pulse_split, int chunk, int window_bins,
                       float2* out, long long out_stride, long long split_stride, cudaStream_t s) {
    SplitParams P = make_params(in, chunk, capacity_for(chunk, window_bins), pulse_split);
    P.out = out;
    P.out_stride = out_stride;
    P.split_stride = split_stride;
    const size_t smem = dynamic_smem(P.cap, true);
    if (int st = prepare(split_polar_kernel, smem)) return st;
    dim3 grid(tiles_of(g.win_nr, g.win_nu, g.tile_lc), pulse_split);
    split_polar_kernel<<<grid, kThreads, smem, s>>>(P, g);
    note_launches(1);
    return check_launch("split_polar");
}

int split_wait_timeouts(int* count) {
    const cudaError_t e = cudaMemcpyFromSymbol(count, g_wait_timeouts, sizeof(int));
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "wait timeouts: %s", cudaGetErrorString(e));
    return SARBP_OK;
}

// The pulse split of a direct lattice launch that asks for the automatic one: sized for the
// largest window budget, so that it depends on the lattice only and the workspace query and the
// launch agree (fewer pulses only lower it).
int split_lattice_auto_split(const sarbp_lattice& lat, int pulses) {
    const size_t smem = dynamic_smem(capacity_for(kMaxChunk, 1 << 20, kLatticeWindowBudget), false);
    if (prepare(split_lattice_kernel, smem) != SARBP_OK) return 1;
    return best_pulse_split(split_lattice_kernel, smem, tiles_of(lat.rows, lat.cols, 5), pulses);
}

int launch_split_lattice(const PulseInputs& in, const sarbp_lattice& lat, int pulse_split, int chunk, int window_bins,
                         float2* out, long long split_stride, cudaStream_t s) {
    SplitParams P = make_params(in, chunk, capacity_for(chunk, window_bins, kLatticeWindowBudget), pulse_split);
    P.out = out;
    P.split_stride = split_stride;
    const int lc = 5;
    const size_t smem = dynamic_smem(P.cap, false);
    dim3 grid(tiles_of(lat.rows, lat.cols, lc), pulse_split);
    if (int st = prepare(split_lattice_kernel, smem)) return st;
    split_lattice_kernel<<<grid, kThreads, smem, s>>>(P, lat, lc);
    note_launches(1);
    return check_launch("split_lattice");
}

int launch_split_points(const PulseInputs& in, const double* xyz, int npts, int pulse_split, int chunk,
                        int window_bins, float2* out, long long split_stride, cudaStream_t s) {
    SplitParams P = make_params(in, chunk, capacity_for(chunk, window_bins), pulse_split);
    P.out = out;
    P.split_stride = split_stride;
    const size_t smem = dynamic_smem(P.cap, false);
    if (int st = prepare(split_points_kernel, smem)) return st;
    dim3 grid((npts + kSplitTilePixels - 1) / kSplitTilePixels, pulse_split);
    split_points_kernel<<<grid, kThreads, smem, s>>>(P, xyz, npts);
    note_launches(1);
    return check_launch("split_points");
}

size_t split_adjoint_workspace(const sarbp_lattice& lat, int pulses) {
    return (size_t)tiles_of(lat.rows, lat.cols, 5) * (size_t)pulses * kAdjVals * sizeof(float);
}

int launch_split_lattice_adjoint(const PulseInputs& in, const sarbp_lattice& lat, int chunk, int window_bins,
                                 const float2* grad, float* partials, double* grad_pos, double* grad_phase,
                                 double* grad_weight, cudaStream_t s) {
    SplitParams P = make_params(in, chunk, capacity_for(chunk, window_bins, kLatticeWindowBudget), 1);
    const int lc = 5;
    const size_t smem = dynamic_smem(P.cap, false);
    const int ntiles = tiles_of(lat.rows, lat.cols, lc);
    if (int st = prepare(split_lattice_adjoint_kernel, smem)) return st;
    const dim3 grid(ntiles, best_pulse_split(split_lattice_adjoint_kernel, smem, ntiles, in.pulses));
    split_lattice_adjoint_kernel<<<grid, kThreads, smem, s>>>(P, lat, lc, grad, partials);
    note_launches(1);
    if (int st = check_launch("split_lattice_adjoint")) return st;
    adjoint_sum_kernel<<<grid_blocks(in.pulses, kSumPulses), kThreads, 0, s>>>(partials, ntiles, in.pulses, in.weight,
                                                                              grad_pos, grad_phase, grad_weight);
    note_launches(1);
    return check_launch("adjoint_sum");
}

int launch_split_ffbp_tables(const PulseInputs& in, const PolarDesc* nodes, int n_nodes, int max_dim,
                             float4* tables, cudaStream_t s) {
    if (n_nodes <= 0) return SARBP_OK;
    dim3 grid((max_dim + kThreads - 1) / kThreads, n_nodes);
    ffbp_tables_kernel<<<grid, kThreads, 0, s>>>(table_consts(make_params(in, 1, 4, 1)), nodes, tables);
    note_launches(1);
    return check_launch("split_ffbp_tables");
}

int launch_split_ffbp_leaf_pulses(const PulseInputs& in, const PolarDesc* nodes, const int* leaves, int n_leaves,
                                  void* recs, cudaStream_t s) {
    if (n_leaves <= 0) return SARBP_OK;
    ffbp_leaf_pulses_kernel<<<n_leaves, 128, 0, s>>>(in.k * kInvTwoPi, in.pos, in.weight, in.phase, nodes, leaves,
                                                     reinterpret_cast<PulseRec*>(recs));
    note_launches(1);
    return check_launch("split_ffbp_leaf_pulses");
}

int launch_split_ffbp_child_records(double k, const PolarDesc* nodes, const float4* tables, const TileItem* items,
                                    int n_items, float2* arena, const void* tmaps, void* recs, cudaStream_t s) {
    if (n_items <= 0) return SARBP_OK;
    PulseInputs none{};
    none.k = k;
    none.data_dr = 1.0;
    const SplitParams P = make_params(none, 1, 4, 1);
    ffbp_child_records_kernel<<<grid_blocks(2LL * n_items, kThreads), kThreads, 0, s>>>(
        P.Kh, P.Kl, (float)P.scale_w, (float)P.inv_scale_w, nodes, tables, items, n_items, arena, tmaps,
        reinterpret_cast<ChildRec*>(recs));
    note_launches(1);
    return check_launch("split_ffbp_child_records");
}

size_t split_ffbp_pulse_record_bytes() { return sizeof(PulseRec); }
size_t split_ffbp_child_record_bytes() { return sizeof(ChildRec); }

int launch_split_ffbp_leaves(const PulseInputs& in, const PolarDesc* nodes, const TileItem* items, int nitems,
                             int chunk, int window_bins, const float4* tables, const void* precs, float2* arena,
                             float2* root_out, int root, cudaStream_t s) {
    if (nitems <= 0) return SARBP_OK;
    SplitParams P = make_params(in, chunk, leaf_capacity(chunk, window_bins), 1);
    const size_t smem = leaf_window_offset(chunk) + (size_t)P.cap * 32;
    if (int st = prepare(split_leaf_kernel, smem)) return st;
    split_leaf_kernel<<<nitems, kThreads, smem, s>>>(P, nodes, items, tables, reinterpret_cast<const PulseRec*>(precs),
                                                     arena, root_out, root);
    note_launches(1);
    return check_launch("split_ffbp_leaves");
}

int launch_split_ffbp_merges(double k, const PolarDesc* nodes, const TileItem* items, int nitems,
                             const float4* tables, const void* crecs, float2* arena, float2* root_out, int root,
                             size_t box_bytes, unsigned long long wait_ns, int withheld, cudaStream_t s) {
    if (nitems <= 0) return SARBP_OK;
    PulseInputs none{};
    none.k = k;
    none.data_dr = 1.0;
    SplitParams P = make_params(none, 1, 4, 1);
    if (box_bytes > 0) {
        const size_t smem = 128 + kTabBytes + box_bytes;
        if (int st = prepare(split_merge_staged_kernel, smem)) return st;
        split_merge_staged_kernel<<<nitems, kMergeThreads, smem, s>>>(
            P, nodes, items, tables, reinterpret_cast<const ChildRec*>(crecs), arena, root_out, root, wait_ns, withheld);
        note_launches(1);
        return check_launch("split_ffbp_merges (staged)");
    }
    const size_t smem = merge_smem();
    if (int st = prepare(split_merge_kernel, smem)) return st;
    split_merge_kernel<<<nitems, kMergeThreads, smem, s>>>(P, nodes, items, tables, reinterpret_cast<const ChildRec*>(crecs),
                                                      arena, root_out, root);
    note_launches(1);
    return check_launch("split_ffbp_merges");
}

int launch_split_ffbp_merge_queue(double k, const PolarDesc* nodes, const TileItem* items, int nitems,
                                  const float4* tables, const void* crecs, float2* arena, float2* root_out, int root,
                                  const MergeQueue& Q, cudaStream_t s) {
    if (nitems <= 0) return SARBP_OK;
    PulseInputs none{};
    none.k = k;
    none.data_dr = 1.0;
    SplitParams P = make_params(none, 1, 4, 1);
    const size_t smem = merge_smem();
    if (int st = prepare(split_merge_queue_kernel, smem)) return st;
    int dev = 0, sms = 1, per_sm = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, split_merge_queue_kernel, kThreads, smem);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "merge queue: %s", cudaGetErrorString(e));
    const int blocks = std::max(1, std::min(nitems, sms * std::max(1, per_sm)));
    split_merge_queue_kernel<<<blocks, kThreads, smem, s>>>(P, nodes, items, nitems, tables,
                                                            reinterpret_cast<const ChildRec*>(crecs), arena,
                                                            root_out, root, Q);
    note_launches(1);
    return check_launch("split_ffbp_merge_queue");
}

// ---- polar image -> ground lattice (evaluate_image on a lattice, split precision) -----------
//
// A lattice tile is a parent tile whose pixels lie on the ground lattice, and the polar
// image is its only child: one two-float record per tile (child_rec_at at the tile centre),
// then per pixel the merge kernel's FP32 child coordinates, 4x4 stencil and phase.  The
// phase restores exp(j k r) (r: the point's range to the image origin); no demodulation.
__global__ void __launch_bounds__(kThreads, 3) split_evaluate_lattice_kernel(float Kh, float Kl, float scale_w,
                                                                             float inv_scale_w, PolarDesc c,
                                                                             const float2* __restrict__ img,
                                                                             sarbp_lattice lat, int lc,
                                                                             float2* __restrict__ out) {
    __shared__ TileShared S;
    __shared__ ChildRec C;
    Job J;
    J.lat = lat;
    J.lc = lc;
    tile_of(blockIdx.x, lat.cols, lc, J.tile_r, J.tile_u);
    Pix px[kPX];
    setup_lattice<false>(J, S, px);
    if (threadIdx.x == 0) {
        FF x, y;
        split2(S.cx, x.h, x.l);
        split2(S.cy, y.h, y.l);
        C = child_rec_at(FF{Kh, Kl}, scale_w, inv_scale_w, c, x, y, img);
    }
    __syncthreads();
    const float Kf = Kh;
    const int cols_t = 1 << lc;
#pragma unroll
    for (int k = 0; k < kPX; ++k) {
        const float2 v = child_value(Kf, C, px[k]);
        const int p = threadIdx.x + kThreads * k;
        const int wr = J.tile_r + (p >> lc), wu = J.tile_u + (p & (cols_t - 1));
        if (wr < lat.rows && wu < lat.cols) out[(long long)wr * lat.cols + wu] = v;
    }
}

// ---- batched scenes: persistent work-queue kernels ------------------------------------------
//
// Many independent scenes (direct lattice images and FFBP trees) run as one work list.
// Each scene's parameters live in a device array; tile items carry their scene in
// TileItem::pad and FFBP nodes in PolarDesc::pad.  The BP kernel is persistent: every
// CTA takes the next item from a global counter until the list is exhausted, so scenes
// of very different sizes share the GPU without per-scene launches or idle tails.  Items
// are independent (no item waits for another), so the persistent grid needs no
// co-residency guarantee.  Merge levels run as one persistent launch per tree height
// over the nodes of that height in every FFBP scene.
namespace {

struct BatchScene {
    SplitParams P;          // pulse inputs, constants, chunk / window capacity; P.out = direct output
    sarbp_lattice lat;      // direct scenes
    int kind;               // 0 direct lattice, 1 FFBP
    int lc;                 // direct: log2 of tile columns
    int pad[2];
    long long prec_offset;  // FFBP: first pulse record of the scene
};

// Completion time of an item for the scene's trace slot (max over the scene's items): the
// GPU's nanosecond global timer, after every thread of the block is done with the item.
__device__ __forceinline__ void trace_item(unsigned long long* trace, int scene) {
    if (!trace) return;  // uniform
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        atomicMax(trace + scene, t);
    }
}

__global__ void batch_trace_start_kernel(unsigned long long* t0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *t0 = t;
}

__device__ __forceinline__ int next_item(int* counter, int& s_item) {
    __syncthreads();  // every thread is done with the previous item's shared state
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    return s_item;
}

__device__ __forceinline__ void load_scene(const BatchScene* __restrict__ scenes, int scene, BatchScene& sc) {
    const int* src = reinterpret_cast<const int*>(scenes + scene);
    int* dst = reinterpret_cast<int*>(&sc);
    for (int w = threadIdx.x; w < (int)(sizeof(BatchScene) / sizeof(int)); w += kThreads) dst[w] = src[w];
    __syncthreads();
}

// Direct tiles of every direct scene (flat lattices only, checked when the batch is created).
__global__ void __launch_bounds__(kThreads, 4) batch_direct_kernel(const BatchScene* __restrict__ scenes,
                                                                   const TileItem* __restrict__ items, int nitems,
                                                                   int* counter, unsigned long long* trace) {
    extern __shared__ __align__(16) char smem[];
    __shared__ TileShared S;
    __shared__ int s_item, s_scene;
    __shared__ __align__(16) BatchScene sc;
    if (threadIdx.x == 0) s_scene = -1;
    for (;;) {
        const int idx = next_item(counter, s_item);
        if (idx >= nitems) return;
        const TileItem it = items[idx];
        if (it.pad != s_scene) {  // uniform across the block
            load_scene(scenes, it.pad, sc);
            if (threadIdx.x == 0) s_scene = it.pad;
        }
        lattice_tile(sc.P, sc.lat, sc.lc, it.tile_r, it.tile_u, 0, sc.P.in.pulses, sc.P.out, S, smem);
        trace_item(trace, it.pad);
    }
}

// Leaf tiles of every FFBP scene.
__global__ void __launch_bounds__(kThreads, 3) batch_leaf_kernel(const BatchScene* __restrict__ scenes,
                                                                 const PolarDesc* __restrict__ nodes,
                                                                 const TileItem* __restrict__ items, int nitems,
                                                                 const float4* __restrict__ tables,
                                                                 const PulseRec* __restrict__ precs,
                                                                 float2* __restrict__ arena, int* counter,
                                                                 unsigned long long* trace) {
    extern __shared__ __align__(16) char smem[];
    __shared__ int s_base[kMaxLeafChunk];
    __shared__ float s_wt[kMaxLeafChunk];
    __shared__ int s_nfit, s_item, s_scene;
    __shared__ __align__(16) BatchScene sc;
    if (threadIdx.x == 0) s_scene = -1;
    for (;;) {
        const int idx = next_item(counter, s_item);
        if (idx >= nitems) return;
        const TileItem it = items[idx];
        if (it.pad != s_scene) {
            load_scene(scenes, it.pad, sc);
            if (threadIdx.x == 0) s_scene = it.pad;
        }
        leaf_tile(sc.P, nodes, it, tables, precs + sc.prec_offset, arena, nullptr, -1, smem, s_base, s_wt, s_nfit);
        trace_item(trace, it.pad);
    }
}

__global__ void __launch_bounds__(kMergeThreads, 8) batch_merge_kernel(const BatchScene* __restrict__ scenes,
                                                                  const PolarDesc* __restrict__ nodes,
                                                                  const TileItem* __restrict__ items, int nitems,
                                                                  const float4* __restrict__ tables,
                                                                  const ChildRec* __restrict__ crecs,
                                                                  float2* __restrict__ arena, int* counter,
                                                                  unsigned long long* trace) {
    extern __shared__ __align__(16) char smem[];
    __shared__ ChildDup C[2];
    __shared__ int s_item;
    for (;;) {
        const int idx = next_item(counter, s_item);
        if (idx >= nitems) return;
        const TileItem it = items[idx];
        merge_tile<false, kMergeThreads>(scenes[it.pad].P.Kf, nodes, it, tables, crecs + 2 * (long long)idx, C, arena,
                                         nullptr, -1, smem);
        trace_item(trace, it.pad);
    }
}

__global__ void batch_tables_kernel(const BatchScene* __restrict__ scenes, const PolarDesc* __restrict__ nodes,
                                    float4* __restrict__ tables) {
    const PolarDesc& g = nodes[blockIdx.y];
    const SplitParams& P = scenes[g.pad].P;
    table_entries(table_consts(P), g, blockIdx.x * blockDim.x + threadIdx.x, tables);
}

__global__ void batch_leaf_pulses_kernel(const BatchScene* __restrict__ scenes, const PolarDesc* __restrict__ nodes,
                                         const int* __restrict__ leaves, PulseRec* __restrict__ recs) {
    __shared__ int amax;
    const PolarDesc& g = nodes[leaves[blockIdx.x]];
    const BatchScene& sc = scenes[g.pad];
    leaf_pulses(sc.P.K, sc.P.in.pos, sc.P.in.weight, sc.P.in.phase, g, recs + sc.prec_offset, amax);
}

__global__ void batch_child_records_kernel(const BatchScene* __restrict__ scenes, const PolarDesc* __restrict__ nodes,
                                           const float4* __restrict__ tables, const TileItem* __restrict__ items,
                                           int n_items, float2* __restrict__ arena, ChildRec* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n_items) return;
    const TileItem it = items[t >> 1];
    const SplitParams& P = scenes[it.pad].P;
    child_record(FF{P.Kh, P.Kl}, (float)P.scale_w, (float)P.inv_scale_w, nodes, tables, it, t, arena, nullptr, out);
}

}  // namespace

size_t split_batch_scene_bytes() { return sizeof(BatchScene); }

size_t split_batch_pack_scene(const BatchSceneDesc& d, void* dst) {
    BatchScene b{};
    b.P = make_params(d.in, d.chunk,
                      d.kind == 0 ? capacity_for(d.chunk, d.window_bins, kLatticeWindowBudget)
                                  : leaf_capacity(d.chunk, d.window_bins),
                      1);
    b.P.out = d.out;
    b.lat = d.lat;
    b.kind = d.kind;
    b.lc = d.lc;
    b.prec_offset = d.prec_offset;
    memcpy(dst, &b, sizeof(b));
    return (d.kind == 0 ? window_offset() + raw_bytes_for(b.P.cap, kMaxChunk) : leaf_window_offset(d.chunk)) +
           (size_t)b.P.cap * 32;
}

int split_batch_occupancy(size_t direct_smem, size_t leaf_smem, int* direct_per_sm, int* leaf_per_sm,
                          int* merge_per_sm) {
    if (int st = prepare(batch_direct_kernel, direct_smem)) return st;
    if (int st = prepare(batch_leaf_kernel, leaf_smem)) return st;
    if (int st = prepare(batch_merge_kernel, merge_smem())) return st;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(direct_per_sm, batch_direct_kernel, kThreads,
                                                                  direct_smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(leaf_per_sm, batch_leaf_kernel, kThreads, leaf_smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(merge_per_sm, batch_merge_kernel, kMergeThreads, merge_smem());
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
    return SARBP_OK;
}

int launch_split_batch_prologue(const void* scenes, const PolarDesc* nodes, int n_nodes, int max_dim,
                                const int* leaves, int n_leaves, const TileItem* merge_items, int n_merge_items,
                                float4* tables, void* precs, void* crecs, float2* arena, cudaStream_t s) {
    const BatchScene* sc = reinterpret_cast<const BatchScene*>(scenes);
    if (n_nodes > 0) {
        dim3 grid((max_dim + kThreads - 1) / kThreads, n_nodes);
        batch_tables_kernel<<<grid, kThreads, 0, s>>>(sc, nodes, tables);
        note_launches(1);
        if (int st = check_launch("batch_tables")) return st;
    }
    if (n_leaves > 0) {
        batch_leaf_pulses_kernel<<<n_leaves, 128, 0, s>>>(sc, nodes, leaves, reinterpret_cast<PulseRec*>(precs));
        note_launches(1);
        if (int st = check_launch("batch_leaf_pulses")) return st;
    }
    if (n_merge_items > 0) {
        batch_child_records_kernel<<<grid_blocks(2LL * n_merge_items, kThreads), kThreads, 0, s>>>(
            sc, nodes, tables, merge_items, n_merge_items, arena, reinterpret_cast<ChildRec*>(crecs));
        note_launches(1);
        if (int st = check_launch("batch_child_records")) return st;
    }
    return SARBP_OK;
}

int launch_split_batch_trace_start(unsigned long long* t0, cudaStream_t s) {
    batch_trace_start_kernel<<<1, 1, 0, s>>>(t0);
    note_launches(1);
    return check_launch("batch_trace_start");
}

int launch_split_batch_direct(const void* scenes, const TileItem* items, int nitems, int* counter, int blocks,
                              size_t smem, unsigned long long* trace, cudaStream_t s) {
    if (nitems <= 0) return SARBP_OK;
    if (int st = prepare(batch_direct_kernel, smem)) return st;
    batch_direct_kernel<<<blocks, kThreads, smem, s>>>(reinterpret_cast<const BatchScene*>(scenes), items, nitems,
                                                       counter, trace);
    note_launches(1);
    return check_launch("batch_direct");
}

int launch_split_batch_leaves(const void* scenes, const PolarDesc* nodes, const TileItem* items, int nitems,
                              const float4* tables, const void* precs, float2* arena, int* counter, int blocks,
                              size_t smem, unsigned long long* trace, cudaStream_t s) {
    if (nitems <= 0) return SARBP_OK;
    if (int st = prepare(batch_leaf_kernel, smem)) return st;
    batch_leaf_kernel<<<blocks, kThreads, smem, s>>>(reinterpret_cast<const BatchScene*>(scenes), nodes, items, nitems,
                                                     tables, reinterpret_cast<const PulseRec*>(precs), arena, counter,
                                                     trace);
    note_launches(1);
    return check_launch("batch_leaves");
}

int launch_split_batch_merges(const void* scenes, const PolarDesc* nodes, const TileItem* items, int nitems,
                              const float4* tables, const void* crecs, float2* arena, int* counter, int blocks,
                              unsigned long long* trace, cudaStream_t s) {
    if (nitems <= 0) return SARBP_OK;
    if (int st = prepare(batch_merge_kernel, merge_smem())) return st;
    batch_merge_kernel<<<blocks, kMergeThreads, merge_smem(), s>>>(reinterpret_cast<const BatchScene*>(scenes), nodes,
                                                              items, nitems, tables,
                                                              reinterpret_cast<const ChildRec*>(crecs), arena,
                                                              counter, trace);
    note_launches(1);
    return check_launch("batch_merges");
}

int launch_split_evaluate_lattice(const float2* image, const PolarDesc& grid, const sarbp_lattice& lattice, double k,
                                  float2* out, cudaStream_t s) {
    PulseInputs none{};
    none.k = k;
    none.data_dr = 1.0;
    const SplitParams P = make_params(none, 1, 4, 1);
    sarbp_lattice flat = lattice;  // ground points: z is not used
    flat.origin[2] = flat.step_row[2] = flat.step_col[2] = 0.0;
    const int lc = 5;
    split_evaluate_lattice_kernel<<<tiles_of(lattice.rows, lattice.cols, lc), kThreads, 0, s>>>(
        P.Kh, P.Kl, (float)P.scale_w, (float)P.inv_scale_w, grid, image, flat, lc, out);
    note_launches(1);
    return check_launch("split_evaluate_lattice");
}

}  // namespace sarbp
