// Reference-arithmetic kernels for the three precision policies of the
// reference (fp64 / fp32 / mixed, fast_bp/gpu/kernels.cu:1-6): one thread per
// output pixel, per-pulse inputs staged through shared memory in chunks, the
// whole aperture in one launch.  They reproduce the reference's rounding
// points (sample1/sample2 weights, per-child complex64 rounding in merges) and
// are the "plain FP64-phase" baseline the split-precision kernels are
// measured against.
#include <math.h>

#include "common.cuh"

namespace sarbp {
namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 128;

template <int M>
struct Policy;
template <>
struct Policy<SARBP_FP64> {
    using G = double;  // geometry and phase
    using A = double;  // interpolation and accumulation
    using W = double;  // weight
};
template <>
struct Policy<SARBP_FP32> {
    using G = float;
    using A = float;
    using W = float;
};
template <>
struct Policy<SARBP_MIXED> {
    using G = double;
    using A = float;
    using W = float;
};

__device__ __forceinline__ void sin_cos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sin_cos(float x, float* s, float* c) { sincosf(x, s, c); }

// sample1 (ffbp.py:24-29, gpu/kernels.cu:22-68).  The support test is written
// on q itself (equivalent to 1 <= floor(q) <= samples-3) so that NaN or huge
// coordinates can never form an out-of-row index.
template <int M>
__device__ __forceinline__ void sample1(const float2* __restrict__ row, int samples, typename Policy<M>::G q,
                                        typename Policy<M>::A& zr, typename Policy<M>::A& zi) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    zr = A(0);
    zi = A(0);
    if (!(q >= G(1) && q < G(samples - 2))) return;
    const int i = (int)floor(q);
    A w[4];
    lagrange_ref<A>((A)(q - (G)i), w);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const float2 v = __ldg(row + i + a - 1);
        zr += w[a] * (A)v.x;
        zi += w[a] * (A)v.y;
    }
}

// sample2 (gpu/kernels.cu:70-137): 4x4 Lagrange with w = wr[a]*wu[b].
template <int M>
__device__ __forceinline__ void sample2(const float2* __restrict__ img, int nr, int nu, typename Policy<M>::G qr,
                                        typename Policy<M>::G qu, typename Policy<M>::A& zr,
                                        typename Policy<M>::A& zi) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    zr = A(0);
    zi = A(0);
    if (!(qr >= G(1) && qr < G(nr - 2) && qu >= G(1) && qu < G(nu - 2))) return;
    const int ir = (int)floor(qr);
    const int iu = (int)floor(qu);
    A wr[4], wu[4];
    lagrange_ref<A>((A)(qr - (G)ir), wr);
    lagrange_ref<A>((A)(qu - (G)iu), wu);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const float2 v = __ldg(img + (size_t)(ir + a - 1) * nu + iu + b - 1);
            const A w = wr[a] * wu[b];
            zr += w * (A)v.x;
            zi += w * (A)v.y;
        }
    }
}

// Per-pulse inputs converted to the policy's types and staged in shared memory.
template <int M>
struct PulseStage {
    typename Policy<M>::G pos[3 * kChunk];
    typename Policy<M>::W w[kChunk];
    typename Policy<M>::G ph[kChunk];
};

template <int M>
__device__ __forceinline__ void stage_pulses(PulseStage<M>& st, const PulseInputs& in, int c0, int count) {
    using G = typename Policy<M>::G;
    using W = typename Policy<M>::W;
    for (int t = threadIdx.x; t < count; t += blockDim.x) {
        const int n = c0 + t;
        st.pos[3 * t] = (G)in.pos[3 * n];
        st.pos[3 * t + 1] = (G)in.pos[3 * n + 1];
        st.pos[3 * t + 2] = (G)in.pos[3 * n + 2];
        st.w[t] = (W)in.weight[n];
        st.ph[t] = (G)in.phase[n];
    }
}

// Accumulate pulses [p0, p1) for one point (x, y, z) with phase k*(d - r_demod) + phase[n].
template <int M>
__device__ __forceinline__ void accumulate(PulseStage<M>& st, const PulseInputs& in, int p0, int p1, bool active,
                                           typename Policy<M>::G x, typename Policy<M>::G y,
                                           typename Policy<M>::G z, typename Policy<M>::G r_demod,
                                           typename Policy<M>::A& accr, typename Policy<M>::A& acci) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    const G rs = (G)in.range_start, ddr = (G)in.data_dr, kk = (G)in.k;
    for (int c0 = p0; c0 < p1; c0 += kChunk) {
        const int count = min(kChunk, p1 - c0);
        __syncthreads();
        stage_pulses<M>(st, in, c0, count);
        __syncthreads();
        if (!active) continue;
        for (int t = 0; t < count; ++t) {
            const G dx = x - st.pos[3 * t];
            const G dy = y - st.pos[3 * t + 1];
            const G dz = z - st.pos[3 * t + 2];
            const G d = sqrt(dx * dx + dy * dy + dz * dz);
            A vr, vi;
            sample1<M>(in.data + (size_t)(c0 + t) * in.samples, in.samples, (d - rs) / ddr, vr, vi);
            G sg, cg;
            sin_cos(kk * (d - r_demod) + st.ph[t], &sg, &cg);
            const A s = (A)sg, c = (A)cg;
            const A a = (A)st.w[t];
            accr += a * (vr * c - vi * s);
            acci += a * (vr * s + vi * c);
        }
    }
}

// Polar pixel (ir, iu) of grid g -> ground point and slant radius (gpu/kernels.cu:148-154).
template <class G>
__device__ __forceinline__ void polar_point(const PolarDesc& g, int ir, int iu, G& x, G& y, G& r) {
    const G oz = (G)g.oz;
    r = (G)g.r0 + (G)ir * (G)g.dr;
    const G u = (G)g.u0 + (G)iu * (G)g.du;
    const G ground = sqrt(fmax(G(0), r * r - oz * oz));
    x = (G)g.ox + (G)g.side * ground * sqrt(fmax(G(0), G(1) - u * u));
    y = (G)g.oy + ground * u;
}

template <class A>
__device__ __forceinline__ float2 to_c64(A r, A i) {
    return make_float2((float)r, (float)i);
}

// ---- direct BP ----------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(kThreads) plain_polar_kernel(PulseInputs in, PolarDesc g, int p0, int p1,
                                                                float2* __restrict__ out, long long out_stride) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    __shared__ PulseStage<M> st;
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    const long long npix = (long long)g.win_nr * g.win_nu;
    const bool active = p < npix;
    const int wr = active ? (int)(p / g.win_nu) : 0;
    const int wu = active ? (int)(p - (long long)wr * g.win_nu) : 0;
    G x, y, r;
    polar_point<G>(g, g.win_r0 + wr, g.win_u0 + wu, x, y, r);
    A accr = A(0), acci = A(0);
    accumulate<M>(st, in, p0, p1, active, x, y, G(0), r, accr, acci);
    if (active) out[(long long)wr * out_stride + wu] = to_c64(accr, acci);
}

template <int M>
__global__ void __launch_bounds__(kThreads) plain_points_kernel(PulseInputs in, const double* __restrict__ xyz,
                                                                 int npts, float2* __restrict__ out) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    __shared__ PulseStage<M> st;
    const int p = blockIdx.x * kThreads + threadIdx.x;
    const bool active = p < npts;
    const int q = active ? p : 0;
    const G x = (G)xyz[3 * q], y = (G)xyz[3 * q + 1], z = (G)xyz[3 * q + 2];
    A accr = A(0), acci = A(0);
    accumulate<M>(st, in, 0, in.pulses, active, x, y, z, G(0), accr, acci);
    if (active) out[p] = to_c64(accr, acci);
}

template <int M>
__global__ void __launch_bounds__(kThreads) plain_lattice_kernel(PulseInputs in, sarbp_lattice lat,
                                                                  float2* __restrict__ out) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    __shared__ PulseStage<M> st;
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    const long long npix = (long long)lat.rows * lat.cols;
    const bool active = p < npix;
    const double i = active ? (double)(p / lat.cols) : 0.0;
    const double j = active ? (double)(p % lat.cols) : 0.0;
    const G x = (G)(lat.origin[0] + i * lat.step_row[0] + j * lat.step_col[0]);
    const G y = (G)(lat.origin[1] + i * lat.step_row[1] + j * lat.step_col[1]);
    const G z = (G)(lat.origin[2] + i * lat.step_row[2] + j * lat.step_col[2]);
    A accr = A(0), acci = A(0);
    accumulate<M>(st, in, 0, in.pulses, active, x, y, z, G(0), accr, acci);
    if (active) out[p] = to_c64(accr, acci);
}

// ---- regrid / merge (gpu/kernels.cu:341-429, gpu/resident_kernels.cu:6-157) ---
template <int M>
__device__ __forceinline__ float2 regrid_pixel(const float2* __restrict__ img, const PolarDesc& src,
                                               const PolarDesc& dst, double k, int ir, int iu) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    G x, y, r;
    polar_point<G>(dst, ir, iu, x, y, r);
    const G dx = x - (G)src.ox, dy = y - (G)src.oy;
    const G g = sqrt(dx * dx + dy * dy);
    if (g == G(0)) return make_float2(0.0f, 0.0f);
    const G soz = (G)src.oz;
    const G rr = sqrt(g * g + soz * soz);
    const G uu = dy / g;
    A vr, vi;
    sample2<M>(img, src.nr, src.nu, (rr - (G)src.r0) / (G)src.dr, (uu - (G)src.u0) / (G)src.du, vr, vi);
    G sg, cg;
    sin_cos((G)k * (rr - r), &sg, &cg);
    const A s = (A)sg, c = (A)cg;
    return to_c64(vr * c - vi * s, vr * s + vi * c);
}

template <int M>
__global__ void __launch_bounds__(kThreads) plain_regrid_kernel(const float2* __restrict__ img, PolarDesc src,
                                                                 PolarDesc dst, double k, float2* __restrict__ out) {
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (p >= (long long)dst.win_nr * dst.win_nu) return;
    const int wr = (int)(p / dst.win_nu), wu = (int)(p % dst.win_nu);
    out[p] = regrid_pixel<M>(img, src, dst, k, dst.win_r0 + wr, dst.win_u0 + wu);
}

template <int M>
__global__ void __launch_bounds__(kThreads) plain_merge_kernel(const float2* __restrict__ left, PolarDesc lg,
                                                                const float2* __restrict__ right, PolarDesc rg,
                                                                PolarDesc dst, double k, float2* __restrict__ out) {
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (p >= (long long)dst.win_nr * dst.win_nu) return;
    const int ir = dst.win_r0 + (int)(p / dst.win_nu), iu = dst.win_u0 + (int)(p % dst.win_nu);
    const float2 a = regrid_pixel<M>(left, lg, dst, k, ir, iu);
    const float2 b = regrid_pixel<M>(right, rg, dst, k, ir, iu);
    out[p] = make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}

// ---- level-batched FFBP: block table entries are (node, first window pixel) ----
template <int M>
__global__ void __launch_bounds__(kThreads) plain_ffbp_leaf_kernel(PulseInputs in,
                                                                    const PolarDesc* __restrict__ nodes,
                                                                    const int2* __restrict__ blocks,
                                                                    float2* __restrict__ arena) {
    using G = typename Policy<M>::G;
    using A = typename Policy<M>::A;
    __shared__ PulseStage<M> st;
    const int2 blk = blocks[blockIdx.x];
    const PolarDesc g = nodes[blk.x];
    const long long p = (long long)blk.y + threadIdx.x;
    const long long npix = (long long)g.win_nr * g.win_nu;
    const bool active = p < npix;
    const int wr = active ? (int)(p / g.win_nu) : 0;
    const int wu = active ? (int)(p - (long long)wr * g.win_nu) : 0;
    G x, y, r;
    polar_point<G>(g, g.win_r0 + wr, g.win_u0 + wu, x, y, r);
    A accr = A(0), acci = A(0);
    accumulate<M>(st, in, g.a, g.b, active, x, y, G(0), r, accr, acci);
    if (active) arena[g.out_offset + (long long)wr * g.out_stride + wu] = to_c64(accr, acci);
}

template <int M>
__global__ void __launch_bounds__(kThreads) plain_ffbp_merge_kernel(double k, const PolarDesc* __restrict__ nodes,
                                                                     const int2* __restrict__ blocks,
                                                                     float2* __restrict__ arena,
                                                                     float2* __restrict__ root_out, int root) {
    const int2 blk = blocks[blockIdx.x];
    const PolarDesc g = nodes[blk.x];
    const long long p = (long long)blk.y + threadIdx.x;
    if (p >= (long long)g.win_nr * g.win_nu) return;
    const int wr = (int)(p / g.win_nu), wu = (int)(p % g.win_nu);
    const PolarDesc lg = nodes[g.left], rg = nodes[g.right];
    const float2 a = regrid_pixel<M>(arena + lg.out_offset, lg, g, k, g.win_r0 + wr, g.win_u0 + wu);
    const float2 b = regrid_pixel<M>(arena + rg.out_offset, rg, g, k, g.win_r0 + wr, g.win_u0 + wu);
    float2* dst = blk.x == root ? root_out : arena + g.out_offset;
    dst[(long long)wr * g.out_stride + wu] = make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}

// ---- evaluate_image / target_contributions (FP64 geometry and phase) -------------
__global__ void __launch_bounds__(kThreads) evaluate_kernel(const float2* __restrict__ img, PolarDesc g,
                                                             const double* __restrict__ xyz, int npts, double k,
                                                             float2* __restrict__ out) {
    const int p = blockIdx.x * kThreads + threadIdx.x;
    if (p >= npts) return;
    // ffbp.py:192-197: the points' z is not used.
    const double dx = xyz[3 * p] - g.ox, dy = xyz[3 * p + 1] - g.oy;
    const double gd = sqrt(dx * dx + dy * dy);
    const double r = sqrt(gd * gd + g.oz * g.oz);
    const double u = dy / gd;
    float vr, vi;
    sample2<SARBP_MIXED>(img, g.nr, g.nu, (r - g.r0) / g.dr, (u - g.u0) / g.du, vr, vi);
    double sd, cd;
    sincos(k * r, &sd, &cd);
    const float s = (float)sd, c = (float)cd;
    out[p] = make_float2(vr * c - vi * s, vr * s + vi * c);
}

__global__ void __launch_bounds__(kThreads) target_contrib_kernel(PulseInputs in, const double* __restrict__ xyz,
                                                                   int npts, float2* __restrict__ out) {
    const long long e = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (e >= (long long)npts * in.pulses) return;
    const int p = (int)(e / in.pulses), n = (int)(e % in.pulses);
    const double dx = xyz[3 * p] - in.pos[3 * n];
    const double dy = xyz[3 * p + 1] - in.pos[3 * n + 1];
    const double dz = xyz[3 * p + 2] - in.pos[3 * n + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    float vr, vi;
    sample1<SARBP_MIXED>(in.data + (size_t)n * in.samples, in.samples, (r - in.range_start) / in.data_dr, vr, vi);
    double sd, cd;
    sincos(in.k * r, &sd, &cd);
    const float s = (float)sd, c = (float)cd;
    out[e] = make_float2(vr * c - vi * s, vr * s + vi * c);
}

// ---- range-bin phase LUT probe (gpu/precision_probe.cu:106-164) -----------------
__global__ void fill_lut_kernel(int samples, double range_start, double data_dr, double k, float2* lut) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= samples) return;
    double s, c;
    sincos(k * (range_start + (double)i * data_dr), &s, &c);
    lut[i] = make_float2((float)c, (float)s);
}

__global__ void __launch_bounds__(kThreads) plain_polar_lut_kernel(PulseInputs in, PolarDesc g,
                                                                    const float2* __restrict__ lut,
                                                                    float2* __restrict__ out) {
    __shared__ PulseStage<SARBP_MIXED> st;
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    const long long npix = (long long)g.win_nr * g.win_nu;
    const bool active = p < npix;
    const int wr = active ? (int)(p / g.win_nu) : 0;
    const int wu = active ? (int)(p - (long long)wr * g.win_nu) : 0;
    double x, y, r;
    polar_point<double>(g, g.win_r0 + wr, g.win_u0 + wu, x, y, r);
    double rsd, rcd;
    sincos(-in.k * r, &rsd, &rcd);
    const float ref_s = (float)rsd, ref_c = (float)rcd;
    float accr = 0.0f, acci = 0.0f;
    for (int c0 = 0; c0 < in.pulses; c0 += kChunk) {
        const int count = min(kChunk, in.pulses - c0);
        __syncthreads();
        stage_pulses<SARBP_MIXED>(st, in, c0, count);
        __syncthreads();
        if (!active) continue;
        for (int t = 0; t < count; ++t) {
            const double dx = x - st.pos[3 * t], dy = y - st.pos[3 * t + 1], dz = -st.pos[3 * t + 2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            const double q = (d - in.range_start) / in.data_dr;
            if (!(q >= 1.0 && q < (double)(in.samples - 2))) continue;
            const int i = (int)floor(q);
            float vr, vi;
            sample1<SARBP_MIXED>(in.data + (size_t)(c0 + t) * in.samples, in.samples, q, vr, vi);
            float is, ic;
            sincosf((float)(in.k * in.data_dr * (q - (double)i) + st.ph[t]), &is, &ic);
            const float2 base = __ldg(lut + i);
            const float bc = base.x * ic - base.y * is;
            const float bs = base.x * is + base.y * ic;
            const float c = bc * ref_c - bs * ref_s;
            const float s = bc * ref_s + bs * ref_c;
            const float a = st.w[t];
            accr += a * (vr * c - vi * s);
            acci += a * (vr * s + vi * c);
        }
    }
    if (active) out[(long long)wr * g.win_nu + wu] = make_float2(accr, acci);
}

// ---- FP32-sincos phase probes (gpu/precision_probe.cu:19-79) ----------------------
// The mixed policy's FP64 geometry, sampling coordinate and phase k (d - r) + phase[n];
// the finished phase is cast to FP32 and goes to the library sincosf (not the fast
// intrinsic).  WRAP first reduces it with FP64 remainder(phi, 2 pi), which separates the
// quantisation of a large angle in FP32 from the sincosf evaluation error.
template <bool WRAP>
__global__ void __launch_bounds__(kThreads) plain_polar_phase32_kernel(PulseInputs in, PolarDesc g,
                                                                        float2* __restrict__ out) {
    __shared__ PulseStage<SARBP_MIXED> st;
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    const long long npix = (long long)g.win_nr * g.win_nu;
    const bool active = p < npix;
    const int wr = active ? (int)(p / g.win_nu) : 0;
    const int wu = active ? (int)(p - (long long)wr * g.win_nu) : 0;
    double x, y, r;
    polar_point<double>(g, g.win_r0 + wr, g.win_u0 + wu, x, y, r);
    float accr = 0.0f, acci = 0.0f;
    for (int c0 = 0; c0 < in.pulses; c0 += kChunk) {
        const int count = min(kChunk, in.pulses - c0);
        __syncthreads();
        stage_pulses<SARBP_MIXED>(st, in, c0, count);
        __syncthreads();
        if (!active) continue;
        for (int t = 0; t < count; ++t) {
            const double dx = x - st.pos[3 * t], dy = y - st.pos[3 * t + 1], dz = -st.pos[3 * t + 2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            float vr, vi;
            sample1<SARBP_MIXED>(in.data + (size_t)(c0 + t) * in.samples, in.samples, (d - in.range_start) / in.data_dr,
                                 vr, vi);
            double phi = in.k * (d - r) + st.ph[t];
            if (WRAP) phi = remainder(phi, 6.283185307179586476925286766559);
            float sn, cs;
            sincosf((float)phi, &sn, &cs);
            const float a = st.w[t];
            accr += a * (vr * cs - vi * sn);
            acci += a * (vr * sn + vi * cs);
        }
    }
    if (active) out[(long long)wr * g.win_nu + wu] = make_float2(accr, acci);
}

// ---- elementwise ----------------------------------------------------------------
__global__ void add_kernel(float2* __restrict__ left, const float2* __restrict__ right, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (p >= n) return;
    const float2 a = left[p], b = right[p];
    left[p] = make_float2(a.x + b.x, a.y + b.y);
}

__global__ void cast_kernel(const double2* __restrict__ in, float2* __restrict__ out, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (p >= n) return;
    const double2 z = in[p];
    out[p] = make_float2((float)z.x, (float)z.y);
}

__global__ void crop_kernel(const float2* __restrict__ in, int src_nu, int r_begin, int u_begin, int nr, int nu,
                            float2* __restrict__ out) {
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (p >= (int64_t)nr * nu) return;
    const int64_t ir = p / nu, iu = p - ir * nu;
    out[p] = in[(ir + r_begin) * src_nu + iu + u_begin];
}

// Fixed-order sum of pulse-split partial images.
__global__ void sum_parts_kernel(const float2* __restrict__ parts, int nparts, long long part_stride, long long n,
                                 float2* __restrict__ out) {
    const long long p = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (p >= n) return;
    float2 acc = parts[p];
    for (int s = 1; s < nparts; ++s) {
        const float2 v = parts[(long long)s * part_stride + p];
        acc.x += v.x;
        acc.y += v.y;
    }
    out[p] = acc;
}

template <template <int> class K>
struct ByMode {};

}  // namespace

#define SARBP_DISPATCH(mode, CALL)                                    \
    switch (mode) {                                                   \
        case SARBP_FP64: { constexpr int M = SARBP_FP64; CALL; break; } \
        case SARBP_FP32: { constexpr int M = SARBP_FP32; CALL; break; } \
        case SARBP_MIXED: { constexpr int M = SARBP_MIXED; CALL; break; } \
        default: return fail(SARBP_ERR_VALUE, "plain kernels support fp64, fp32 and mixed only (mode %d)", mode); \
    }

int launch_plain_polar(int mode, const PulseInputs& in, const PolarDesc& g, int p0, int p1, int chunk,
                       float2* out, long long out_stride, cudaStream_t s) {
    (void)chunk;
    const long long npix = (long long)g.win_nr * g.win_nu;
    SARBP_DISPATCH(mode, (plain_polar_kernel<M><<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(in, g, p0, p1, out,
                                                                                               out_stride)));
    note_launches(1);
    return check_launch("plain_polar");
}

int launch_plain_points(int mode, const PulseInputs& in, const double* xyz, int npts, int chunk, float2* out,
                        cudaStream_t s) {
    (void)chunk;
    SARBP_DISPATCH(mode, (plain_points_kernel<M><<<grid_blocks(npts, kThreads), kThreads, 0, s>>>(in, xyz, npts, out)));
    note_launches(1);
    return check_launch("plain_points");
}

int launch_plain_lattice(int mode, const PulseInputs& in, const sarbp_lattice& lat, int chunk, float2* out,
                         cudaStream_t s) {
    (void)chunk;
    const long long npix = (long long)lat.rows * lat.cols;
    SARBP_DISPATCH(mode, (plain_lattice_kernel<M><<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(in, lat, out)));
    note_launches(1);
    return check_launch("plain_lattice");
}

int launch_plain_regrid(int mode, const float2* img, const PolarDesc& src, const PolarDesc& dst, double k,
                        float2* out, cudaStream_t s) {
    const long long npix = (long long)dst.win_nr * dst.win_nu;
    SARBP_DISPATCH(mode, (plain_regrid_kernel<M><<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(img, src, dst, k, out)));
    note_launches(1);
    return check_launch("plain_regrid");
}

int launch_plain_merge(int mode, const float2* left, const PolarDesc& lg, const float2* right, const PolarDesc& rg,
                       const PolarDesc& dst, double k, float2* out, cudaStream_t s) {
    const long long npix = (long long)dst.win_nr * dst.win_nu;
    SARBP_DISPATCH(mode, (plain_merge_kernel<M><<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(left, lg, right, rg,
                                                                                               dst, k, out)));
    note_launches(1);
    return check_launch("plain_merge");
}

int launch_plain_ffbp_leaves(int mode, const PulseInputs& in, const PolarDesc* nodes, const int2* blocks,
                             int nblocks, float2* arena, cudaStream_t s) {
    if (nblocks <= 0) return SARBP_OK;
    SARBP_DISPATCH(mode, (plain_ffbp_leaf_kernel<M><<<nblocks, kThreads, 0, s>>>(in, nodes, blocks, arena)));
    note_launches(1);
    return check_launch("plain_ffbp_leaves");
}

int launch_plain_ffbp_merges(int mode, double k, const PolarDesc* nodes, const int2* blocks, int nblocks,
                             float2* arena, float2* root_out, int root, cudaStream_t s) {
    if (nblocks <= 0) return SARBP_OK;
    SARBP_DISPATCH(mode, (plain_ffbp_merge_kernel<M><<<nblocks, kThreads, 0, s>>>(k, nodes, blocks, arena, root_out,
                                                                                 root)));
    note_launches(1);
    return check_launch("plain_ffbp_merges");
}

int launch_evaluate(const float2* img, const PolarDesc& g, const double* xyz, int npts, double k, float2* out,
                    cudaStream_t s) {
    evaluate_kernel<<<grid_blocks(npts, kThreads), kThreads, 0, s>>>(img, g, xyz, npts, k, out);
    note_launches(1);
    return check_launch("evaluate_image");
}

int launch_target_contrib(const PulseInputs& in, const double* xyz, int npts, float2* out, cudaStream_t s) {
    const long long n = (long long)npts * in.pulses;
    target_contrib_kernel<<<grid_blocks(n, kThreads), kThreads, 0, s>>>(in, xyz, npts, out);
    note_launches(1);
    return check_launch("target_contributions");
}

int launch_fill_lut(int samples, double range_start, double data_dr, double k, float2* lut, cudaStream_t s) {
    fill_lut_kernel<<<grid_blocks(samples, kThreads), kThreads, 0, s>>>(samples, range_start, data_dr, k, lut);
    note_launches(1);
    return check_launch("fill_range_phase_lut");
}

int launch_plain_polar_lut(const PulseInputs& in, const PolarDesc& g, const float2* lut, float2* out,
                           cudaStream_t s) {
    const long long npix = (long long)g.win_nr * g.win_nu;
    plain_polar_lut_kernel<<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(in, g, lut, out);
    note_launches(1);
    return check_launch("direct_polar_lut");
}

int launch_plain_polar_phase32(const PulseInputs& in, const PolarDesc& g, bool wrapped, float2* out,
                               cudaStream_t s) {
    const long long npix = (long long)g.win_nr * g.win_nu;
    if (wrapped)
        plain_polar_phase32_kernel<true><<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(in, g, out);
    else
        plain_polar_phase32_kernel<false><<<grid_blocks(npix, kThreads), kThreads, 0, s>>>(in, g, out);
    note_launches(1);
    return check_launch("direct_polar_phase32");
}

int launch_add(float2* left, const float2* right, int64_t n, cudaStream_t s) {
    add_kernel<<<grid_blocks(n, kThreads), kThreads, 0, s>>>(left, right, n);
    note_launches(1);
    return check_launch("add_inplace");
}

int launch_cast(const double2* in, float2* out, int64_t n, cudaStream_t s) {
    cast_kernel<<<grid_blocks(n, kThreads), kThreads, 0, s>>>(in, out, n);
    note_launches(1);
    return check_launch("cast_c128_to_c64");
}

int launch_crop(const float2* in, int src_nu, int r_begin, int u_begin, int nr, int nu, float2* out,
                cudaStream_t s) {
    crop_kernel<<<grid_blocks((int64_t)nr * nu, kThreads), kThreads, 0, s>>>(in, src_nu, r_begin, u_begin, nr, nu,
                                                                               out);
    note_launches(1);
    return check_launch("crop");
}

int launch_sum_parts(const float2* parts, int nparts, long long part_stride, long long n, float2* out,
                     cudaStream_t s) {
    sum_parts_kernel<<<grid_blocks(n, kThreads), kThreads, 0, s>>>(parts, nparts, part_stride, n, out);
    note_launches(1);
    return check_launch("sum_parts");
}

}  // namespace sarbp
