// Zero-phase IIR smoothing of per-target pulse histories for the phase-gradient
// autofocus (fast_bp/autofocus.py:38-39: butter(4, cutoff) as second-order
// sections, then sosfiltfilt along the pulse axis).
//
// Method: forward-backward filtering of an odd-extended signal with
// steady-state initial conditions (Gustafsson's filtfilt, as published with
// scipy.signal.sosfiltfilt): the row is extended by `padlen` samples at each
// end with 2*x[end] - mirror, filtered forward through the cascade of
// direct-form-II-transposed biquads starting from zi * first sample, then
// filtered again over the reversed output starting from zi * its first
// sample, and the extension is cut off.  The extension is formed in complex64
// arithmetic like the reference's (its input is complex64); the filter runs
// in FP64 with explicit roundings (no contraction; on GB300 separate FP64
// multiplies and adds also run faster than fused ones here).
//
// The recursion is serial along the pulses and the rows are independent.  One warp
// per row: its lanes build the odd-extended row in shared memory with coalesced
// loads, then 2 x sections lanes (one per channel and section) run the forward pass
// into shared memory and the backward pass out to the result, each section one
// sample behind the one before it, so every step of the recursion reads shared
// memory or a register instead of waiting on a global load.  Rows too long for
// shared memory use one thread per channel with the forward pass in a time-major
// global workspace.
#include "common.cuh"

namespace sarbp {
namespace {

constexpr int kMaxSections = 8;

__device__ __forceinline__ float extended(const float* x, int n, int padlen, int i, int comp) {
    if (i < padlen) return __fsub_rn(2.0f * x[comp], x[2 * (padlen - i) + comp]);
    const int j = i - padlen;
    if (j < n) return x[2 * j + comp];
    const int m = j - n;  // 0 .. padlen-1
    return __fsub_rn(2.0f * x[2 * (n - 1) + comp], x[2 * (n - 2 - m) + comp]);
}

struct Biquads {
    double b0[kMaxSections], b1[kMaxSections], b2[kMaxSections], a1[kMaxSections], a2[kMaxSections];
    double z0[kMaxSections], z1[kMaxSections];
    int sections;

    __device__ double step(double v) {
#pragma unroll
        for (int s = 0; s < kMaxSections; ++s) {
            if (s < sections) {
                const double y = __dadd_rn(__dmul_rn(b0[s], v), z0[s]);
                z0[s] = __dadd_rn(__dsub_rn(__dmul_rn(b1[s], v), __dmul_rn(a1[s], y)), z1[s]);
                z1[s] = __dsub_rn(__dmul_rn(b2[s], v), __dmul_rn(a2[s], y));
                v = y;
            }
        }
        return v;
    }
};

__global__ void sosfiltfilt_kernel(const float* __restrict__ x, int rows, int n, const double* __restrict__ sos,
                                   const double* __restrict__ zi, int sections, int padlen, double* __restrict__ y,
                                   double* __restrict__ ws) {
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    const int channels = 2 * rows;
    if (ch >= channels) return;
    const int row = ch >> 1, comp = ch & 1;
    const float* xr = x + (size_t)row * n * 2;
    const int m = n + 2 * padlen;
    Biquads f;
    f.sections = sections;
    double zs0[kMaxSections], zs1[kMaxSections];
#pragma unroll
    for (int s = 0; s < kMaxSections; ++s) {
        if (s < sections) {
            f.b0[s] = sos[6 * s];
            f.b1[s] = sos[6 * s + 1];
            f.b2[s] = sos[6 * s + 2];
            f.a1[s] = sos[6 * s + 4];  // a0 == 1 (checked by the caller)
            f.a2[s] = sos[6 * s + 5];
            zs0[s] = zi[2 * s];
            zs1[s] = zi[2 * s + 1];
        }
    }
    const double first = (double)extended(xr, n, padlen, 0, comp);
#pragma unroll
    for (int s = 0; s < kMaxSections; ++s) {
        if (s < sections) {
            f.z0[s] = __dmul_rn(zs0[s], first);
            f.z1[s] = __dmul_rn(zs1[s], first);
        }
    }
    for (int i = 0; i < m; ++i) ws[(size_t)i * channels + ch] = f.step((double)extended(xr, n, padlen, i, comp));
    const double last = ws[(size_t)(m - 1) * channels + ch];
#pragma unroll
    for (int s = 0; s < kMaxSections; ++s) {
        if (s < sections) {
            f.z0[s] = __dmul_rn(zs0[s], last);
            f.z1[s] = __dmul_rn(zs1[s], last);
        }
    }
    double* yr = y + (size_t)row * n * 2;
    for (int i = m - 1; i >= 0; --i) {
        const double v = f.step(ws[(size_t)i * channels + ch]);
        const int j = i - padlen;
        if (j >= 0 && j < n) yr[2 * j + comp] = v;
    }
}

constexpr size_t kRowSmemLimit = 200 * 1024;

size_t row_smem(int n, int padlen) { return (size_t)(n + 2 * padlen) * (sizeof(double2) + sizeof(float2)); }

// One warp per row with the cascade pipelined across lanes: lane comp * S + s (S sections, comp =
// real / imaginary) runs section s and hands its output to lane s + 1 by a shuffle, one sample
// behind.  A step's critical path is one section plus a shuffle instead of the whole cascade;
// every section performs the same roundings in the same order as Biquads::step, so the result
// is bit-identical to the one-thread-per-channel kernel.  The extended row and the forward pass
// stay in shared memory.
__global__ void __launch_bounds__(32) sosfiltfilt_pipe_kernel(const float* __restrict__ x, int n,
                                                              const double* __restrict__ sos,
                                                              const double* __restrict__ zi, int sections,
                                                              int padlen, double* __restrict__ y) {
    extern __shared__ __align__(16) char smem[];
    const int row = blockIdx.x, lane = threadIdx.x;
    const int m = n + 2 * padlen;
    double2* fwd = reinterpret_cast<double2*>(smem);
    float2* ext = reinterpret_cast<float2*>(smem + (size_t)m * sizeof(double2));
    const float* xr = x + (size_t)row * n * 2;
    for (int i = lane; i < m; i += 32) ext[i] = make_float2(extended(xr, n, padlen, i, 0), extended(xr, n, padlen, i, 1));
    __syncwarp();
    const int S = sections;
    const bool active = lane < 2 * S;
    const int comp = active ? lane / S : 0, sec = active ? lane - comp * S : 0;
    const unsigned mask = 2 * S >= 32 ? 0xffffffffu : (1u << (2 * S)) - 1u;
    double b0 = 0.0, b1 = 0.0, b2 = 0.0, a1 = 0.0, a2 = 0.0, zs0 = 0.0, zs1 = 0.0, z0 = 0.0, z1 = 0.0;
    double* fw = reinterpret_cast<double*>(fwd) + comp;
    if (active) {
        b0 = sos[6 * sec];
        b1 = sos[6 * sec + 1];
        b2 = sos[6 * sec + 2];
        a1 = sos[6 * sec + 4];  // a0 == 1 (checked by the caller)
        a2 = sos[6 * sec + 5];
        zs0 = zi[2 * sec];
        zs1 = zi[2 * sec + 1];
        const float* e = reinterpret_cast<const float*>(ext) + comp;
        const double first = (double)e[0];
        z0 = __dmul_rn(zs0, first);
        z1 = __dmul_rn(zs1, first);
        double carry = 0.0;
        for (int t = 0; t < m + S - 1; ++t) {
            const int i = t - sec;
            double out = 0.0;
            if (i >= 0 && i < m) {
                const double v = sec == 0 ? (double)e[2 * i] : carry;
                out = __dadd_rn(__dmul_rn(b0, v), z0);
                z0 = __dadd_rn(__dsub_rn(__dmul_rn(b1, v), __dmul_rn(a1, out)), z1);
                z1 = __dsub_rn(__dmul_rn(b2, v), __dmul_rn(a2, out));
                if (sec == S - 1) fw[2 * i] = out;
            }
            carry = __shfl_up_sync(mask, out, 1);
        }
    }
    __syncwarp();
    if (active) {
        const double last = fw[2 * (m - 1)];
        z0 = __dmul_rn(zs0, last);
        z1 = __dmul_rn(zs1, last);
        double* yr = y + (size_t)row * n * 2 + comp;
        double carry = 0.0;
        for (int t = 0; t < m + S - 1; ++t) {
            const int i = m - 1 - (t - sec);
            double out = 0.0;
            if (t - sec >= 0 && i >= 0) {
                const double v = sec == 0 ? fw[2 * i] : carry;
                out = __dadd_rn(__dmul_rn(b0, v), z0);
                z0 = __dadd_rn(__dsub_rn(__dmul_rn(b1, v), __dmul_rn(a1, out)), z1);
                z1 = __dsub_rn(__dmul_rn(b2, v), __dmul_rn(a2, out));
                const int j = i - padlen;
                if (sec == S - 1 && j >= 0 && j < n) yr[2 * j] = out;
            }
            carry = __shfl_up_sync(mask, out, 1);
        }
    }
}

// np.array_split bounds: part t of n items over k parts starts at t (n / k) + min(t, n % k).
__device__ __forceinline__ int split_start(int n, int k, int t) { return t * (n / k) + min(t, n % k); }

// Brightest cell of each tile of an nr x nu image of magnitudes (the autofocus target picks):
// one block per tile; ties go to the smallest row-major index, as numpy's argmax over the tile.
constexpr int kArgmaxThreads = 256;

__global__ void __launch_bounds__(kArgmaxThreads) tile_argmax_kernel(const float* __restrict__ a, int nr, int nu,
                                                                     int nr_tiles, int nu_tiles, float* tmax,
                                                                     long long* first) {
    const int tr = blockIdx.x / nu_tiles, tc = blockIdx.x - tr * nu_tiles;
    const int r0 = split_start(nr, nr_tiles, tr), r1 = split_start(nr, nr_tiles, tr + 1);
    const int c0 = split_start(nu, nu_tiles, tc), c1 = split_start(nu, nu_tiles, tc + 1);
    const int w = c1 - c0, cells = (r1 - r0) * w;
    float best = -1.0f;
    long long at = (long long)nr * nu;
    for (int q = threadIdx.x; q < cells; q += kArgmaxThreads) {  // increasing row-major order per thread
        const int r = r0 + q / w, c = c0 + q - (q / w) * w;
        const long long idx = (long long)r * nu + c;
        const float v = a[idx];
        if (v > best) {
            best = v;
            at = idx;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float bv = __shfl_xor_sync(0xffffffffu, best, o);
        const long long ba = __shfl_xor_sync(0xffffffffu, at, o);
        if (bv > best || (bv == best && ba < at)) {
            best = bv;
            at = ba;
        }
    }
    __shared__ float sv[kArgmaxThreads / 32];
    __shared__ long long sa[kArgmaxThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sv[warp] = best;
        sa[warp] = at;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < kArgmaxThreads / 32; ++i)
            if (sv[i] > best || (sv[i] == best && sa[i] < at)) {
                best = sv[i];
                at = sa[i];
            }
        tmax[blockIdx.x] = best;
        first[blockIdx.x] = at;
    }
}

}  // namespace

int launch_tile_argmax(const float* a, int nr, int nu, int nr_tiles, int nu_tiles, float* tmax, long long* first,
                       cudaStream_t s) {
    tile_argmax_kernel<<<nr_tiles * nu_tiles, kArgmaxThreads, 0, s>>>(a, nr, nu, nr_tiles, nu_tiles, tmax, first);
    note_launches(1);
    return check_launch("tile_argmax");
}

template <class K>
int set_smem(K kernel, size_t smem) {
    if (smem <= 48 * 1024) return SARBP_OK;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e == cudaSuccess ? SARBP_OK : fail(SARBP_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
}

size_t sosfiltfilt_workspace(int rows, int n, int padlen) {
    return (size_t)(n + 2 * padlen) * (size_t)rows * 2 * sizeof(double);
}

int launch_sosfiltfilt(const float* x, int rows, int n, const double* sos, const double* zi, int sections, int padlen,
                       double* y, double* ws, cudaStream_t s) {
    const size_t smem = row_smem(n, padlen);
    if (smem <= kRowSmemLimit) {
        if (int st = set_smem(sosfiltfilt_pipe_kernel, smem)) return st;
        sosfiltfilt_pipe_kernel<<<rows, 32, smem, s>>>(x, n, sos, zi, sections, padlen, y);
        note_launches(1);
        return check_launch("sosfiltfilt");
    }
    const int channels = 2 * rows;
    const int block = 64;
    sosfiltfilt_kernel<<<grid_blocks(channels, block), block, 0, s>>>(x, rows, n, sos, zi, sections, padlen, y, ws);
    note_launches(1);
    return check_launch("sosfiltfilt");
}

}  // namespace sarbp
