// CPU oracle for the SAR back-projection path.  TEST INFRASTRUCTURE ONLY:
// the product (bp_project_gb300) never links, loads or calls this file; only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
// FP64 result the GPU path is compared with and as the timed CPU baseline.
//
// This is a plain FP64 restatement of the reference's Numba kernels
// (fast_bp/ffbp.py).  Every function below names the reference lines it
// follows.  Arithmetic is kept in the same order as the reference (left to
// right products, IEEE divisions, libm sin/cos) and the build disables FMA
// contraction (-ffp-contract=off) so that results agree with the reference to
// the last few ulps on both x86-64 and aarch64.
//
// Complex arrays are interleaved float pairs (numpy complex64 layout) or
// interleaved double pairs (complex128).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct cd {
    double re, im;
};

// ffbp.py:17-21 cubic_weights: four-point Lagrange weights at taps i-1..i+2.
inline void cubic_weights(double t, double w[4]) {
    w[0] = -t * (t - 1) * (t - 2) / 6;
    w[1] = (t + 1) * (t - 1) * (t - 2) / 2;
    w[2] = -(t + 1) * t * (t - 2) / 2;
    w[3] = (t + 1) * t * (t - 1) / 6;
}

// ffbp.py:24-29 sample1: zero unless all four taps lie inside the row.
inline cd sample1(const float* row, int64_t len, double q) {
    const double fl = std::floor(q);
    // int(math.floor(q)); values far outside the row are rejected below.
    if (!(fl >= -1.0e15 && fl <= 1.0e15)) return {0.0, 0.0};
    const int64_t i = (int64_t)fl;
    const double t = q - (double)i;
    if (i < 1 || i + 2 >= len) return {0.0, 0.0};
    double w[4];
    cubic_weights(t, w);
    cd z{0.0, 0.0};
    for (int a = 0; a < 4; ++a) {
        const float* v = row + 2 * (i + a - 1);
        // w[a]*row[...] promotes complex64 to complex128; the sum runs left to right.
        z.re += w[a] * (double)v[0];
        z.im += w[a] * (double)v[1];
    }
    return z;
}

// ffbp.py:32-40 sample2: 4x4 Lagrange on a complex64 image [nr, nu].
inline cd sample2(const float* img, int64_t nr, int64_t nu, double r, double u) {
    const double fr = std::floor(r), fu = std::floor(u);
    if (!(fr >= -1.0e15 && fr <= 1.0e15 && fu >= -1.0e15 && fu <= 1.0e15)) return {0.0, 0.0};
    const int64_t ir = (int64_t)fr, iu = (int64_t)fu;
    if (ir < 1 || iu < 1 || ir + 2 >= nr || iu + 2 >= nu) return {0.0, 0.0};
    double wr[4], wu[4];
    cubic_weights(r - (double)ir, wr);
    cubic_weights(u - (double)iu, wu);
    cd z{0.0, 0.0};
    for (int a = 0; a < 4; ++a) {
        for (int b = 0; b < 4; ++b) {
            const float* v = img + 2 * ((ir + a - 1) * nu + iu + b - 1);
            // img[..]*wr[a]*wu[b] evaluates (img*wr[a])*wu[b].
            const double pr = (double)v[0] * wr[a];
            const double pi = (double)v[1] * wr[a];
            z.re += pr * wu[b];
            z.im += pi * wu[b];
        }
    }
    return z;
}

// complex128 multiply (a+bi)(c+di) as numpy/Numba evaluate it.
inline cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

inline void store(float* out64, double* out128, int64_t idx, cd v) {
    if (out64) {
        out64[2 * idx] = (float)v.re;
        out64[2 * idx + 1] = (float)v.im;
    }
    if (out128) {
        out128[2 * idx] = v.re;
        out128[2 * idx + 1] = v.im;
    }
}

}  // namespace

extern "C" {

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// ffbp.py:58-76 bp_polar (also the arithmetic of CudaBaseline fp64 direct BP,
// gpu/kernels.cu:139-170 and :240-271, which accumulates pulses in the same order).
void oracle_bp_polar(const float* data, int64_t pulses, int64_t samples, const double* pos,
                     const double* origin, double r0, double dr, int64_t nr, double u0, double du,
                     int64_t nu, double r_start, double data_dr, double k, const double* weight,
                     const double* phase, int side, float* out64, double* out128) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ir = 0; ir < nr; ++ir) {
        const double r = r0 + (double)ir * dr;
        const double ground = std::sqrt(std::fmax(0.0, r * r - origin[2] * origin[2]));
        for (int64_t iu = 0; iu < nu; ++iu) {
            const double u = u0 + (double)iu * du;
            const double x = origin[0] + (double)side * ground * std::sqrt(std::fmax(0.0, 1 - u * u));
            const double y = origin[1] + ground * u;
            cd total{0.0, 0.0};
            for (int64_t n = 0; n < pulses; ++n) {
                const double dx = x - pos[3 * n], dy = y - pos[3 * n + 1];
                const double d = std::sqrt(dx * dx + dy * dy + pos[3 * n + 2] * pos[3 * n + 2]);
                const cd v = sample1(data + 2 * n * samples, samples, (d - r_start) / data_dr);
                const double a = k * (d - r) + phase[n];
                const cd wv{weight[n] * v.re, weight[n] * v.im};
                const cd c = cmul(wv, cd{std::cos(a), std::sin(a)});
                total.re += c.re;
                total.im += c.im;
            }
            store(out64, out128, ir * nu + iu, total);
        }
    }
}

// ffbp.py:43-55 backproject_points: direct BP at arbitrary xyz, phase k*r (not demodulated).
void oracle_backproject_points(const float* data, int64_t pulses, int64_t samples,
                               const double* pos, const double* xyz, int64_t npts, double r_start,
                               double dr, double k, const double* weight, const double* phase,
                               float* out64, double* out128) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t p = 0; p < npts; ++p) {
        cd total{0.0, 0.0};
        for (int64_t n = 0; n < pulses; ++n) {
            const double dx = xyz[3 * p] - pos[3 * n];
            const double dy = xyz[3 * p + 1] - pos[3 * n + 1];
            const double dz = xyz[3 * p + 2] - pos[3 * n + 2];
            const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            const cd v = sample1(data + 2 * n * samples, samples, (r - r_start) / dr);
            const double a = k * r + phase[n];
            const cd wv{weight[n] * v.re, weight[n] * v.im};
            const cd c = cmul(wv, cd{std::cos(a), std::sin(a)});
            total.re += c.re;
            total.im += c.im;
        }
        store(out64, out128, p, total);
    }
}

// ffbp.py:79-95 regrid (child polar image -> parent polar grid).  A zero
// horizontal distance returns zero, as the GPU kernels do (gpu/kernels.cu:359).
void oracle_regrid(const float* img, int64_t snr, int64_t snu, const double* so, double sr0,
                   double sdr, double su0, double sdu, const double* dstv, double r0, double dr,
                   int64_t nr, double u0, double du, int64_t nu, double k, int side, float* out64,
                   double* out128) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ir = 0; ir < nr; ++ir) {
        const double r = r0 + (double)ir * dr;
        const double gr = std::sqrt(std::fmax(0.0, r * r - dstv[2] * dstv[2]));
        for (int64_t iu = 0; iu < nu; ++iu) {
            const double u = u0 + (double)iu * du;
            const double x = dstv[0] + (double)side * gr * std::sqrt(std::fmax(0.0, 1 - u * u));
            const double y = dstv[1] + gr * u;
            const double dx = x - so[0], dy = y - so[1];
            const double g = std::sqrt(dx * dx + dy * dy);
            cd res{0.0, 0.0};
            if (g != 0.0) {
                const double rr = std::sqrt(g * g + so[2] * so[2]);
                const double uu = dy / g;
                const cd v = sample2(img, snr, snu, (rr - sr0) / sdr, (uu - su0) / sdu);
                const double a = k * (rr - r);
                res = cmul(v, cd{std::cos(a), std::sin(a)});
            }
            store(out64, out128, ir * nu + iu, res);
        }
    }
}

// ffbp.py:189-198 evaluate_image (polar image -> arbitrary ground points; z of the points is ignored).
void oracle_evaluate_image(const float* img, int64_t nr, int64_t nu, const double* origin, double r0,
                           double dr, double u0, double du, const double* xyz, int64_t npts,
                           double k, float* out64, double* out128) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npts; ++p) {
        const double dx = xyz[3 * p] - origin[0], dy = xyz[3 * p + 1] - origin[1];
        const double g = std::sqrt(dx * dx + dy * dy);
        const double r = std::sqrt(g * g + origin[2] * origin[2]);
        const double u = dy / g;
        const cd v = sample2(img, nr, nu, (r - r0) / dr, (u - u0) / du);
        store(out64, out128, p, cmul(v, cd{std::cos(k * r), std::sin(k * r)}));
    }
}

// ffbp.py:201-211 target_contributions: out[p, n] = sample1 * exp(j k r) (no weight, no phase).
void oracle_target_contributions(const float* data, int64_t pulses, int64_t samples,
                                 const double* pos, const double* xyz, int64_t npts, double r_start,
                                 double dr, double k, float* out64) {
#pragma omp parallel for schedule(static) collapse(2)
    for (int64_t p = 0; p < npts; ++p) {
        for (int64_t n = 0; n < pulses; ++n) {
            const double dx = xyz[3 * p] - pos[3 * n];
            const double dy = xyz[3 * p + 1] - pos[3 * n + 1];
            const double dz = xyz[3 * p + 2] - pos[3 * n + 2];
            const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            const cd v = sample1(data + 2 * n * samples, samples, (r - r_start) / dr);
            const double a = k * r;
            store(out64, nullptr, p * pulses + n, cmul(v, cd{std::cos(a), std::sin(a)}));
        }
    }
}

// Polar FFBP over a flattened node tree (ffbp.py:141-170).  Node i has
// geometry geom[8*i .. 8*i+7] = (ox, oy, oz, r0, dr, u0, du, side) and
// integers idx[6*i .. 6*i+5] = (a, b, nr, nu, left, right), left/right = -1
// for leaves.  Leaves run bp_polar over pulses [a, b); inner nodes regrid the
// left child, then add the regridded right child with complex64 rounding of
// both terms (numpy complex64 in-place add).  The root image (uncropped) is
// written to root_out; counts[0..3] receive leaves, merges,
// leaf pixel-pulse products and merged pixels.
static void ffbp_node(int64_t node, const float* data, int64_t samples, const double* pos,
                      const double* geom, const int64_t* idx, double r_start, double data_dr,
                      double k, const double* weight, const double* phase,
                      std::vector<float>& out, int64_t* counts) {
    const double* g = geom + 8 * node;
    const int64_t* d = idx + 6 * node;
    const int64_t a = d[0], b = d[1], nr = d[2], nu = d[3], left = d[4], right = d[5];
    const int side = (int)g[7];
    out.assign((size_t)(2 * nr * nu), 0.0f);
    if (left < 0) {
        oracle_bp_polar(data + 2 * a * samples, b - a, samples, pos + 3 * a, g, g[3], g[4], nr, g[5],
                        g[6], nu, r_start, data_dr, k, weight + a, phase + a, side, out.data(),
                        nullptr);
        counts[0] += 1;
        counts[2] += nr * nu * (b - a);
        return;
    }
    std::vector<float> child;
    ffbp_node(left, data, samples, pos, geom, idx, r_start, data_dr, k, weight, phase, child, counts);
    {
        const double* cg = geom + 8 * left;
        const int64_t* cd_ = idx + 6 * left;
        oracle_regrid(child.data(), cd_[2], cd_[3], cg, cg[3], cg[4], cg[5], cg[6], g, g[3], g[4], nr,
                      g[5], g[6], nu, k, side, out.data(), nullptr);
    }
    ffbp_node(right, data, samples, pos, geom, idx, r_start, data_dr, k, weight, phase, child, counts);
    {
        const double* cg = geom + 8 * right;
        const int64_t* cd_ = idx + 6 * right;
        std::vector<float> tmp((size_t)(2 * nr * nu));
        oracle_regrid(child.data(), cd_[2], cd_[3], cg, cg[3], cg[4], cg[5], cg[6], g, g[3], g[4], nr,
                      g[5], g[6], nu, k, side, tmp.data(), nullptr);
        for (size_t i = 0; i < tmp.size(); ++i) out[i] = out[i] + tmp[i];
    }
    counts[1] += 1;
    counts[3] += 2 * nr * nu;
}

void oracle_ffbp_execute(const float* data, int64_t pulses, int64_t samples, const double* pos,
                         const double* geom, const int64_t* idx, int64_t root, double r_start,
                         double data_dr, double k, const double* weight, const double* phase,
                         float* root_out, int64_t* counts) {
    (void)pulses;
    std::vector<float> out;
    counts[0] = counts[1] = counts[2] = counts[3] = 0;
    ffbp_node(root, data, samples, pos, geom, idx, r_start, data_dr, k, weight, phase, out, counts);
    std::memcpy(root_out, out.data(), out.size() * sizeof(float));
}

}  // extern "C"
