// Range compression: the FFT matched filter that turns raw LFM echoes into the
// range-compressed pulses the back-projection kernels consume (sar_io.range_compress,
// fast_bp/sar_io.py:116-139).  The FFTs are library calls (cuFFT through the host);
// these kernels are the memory-bound steps around them:
//   rc_prepare  - remove each pulse's mean and zero-pad it to the FFT length,
//   rc_filter   - multiply by the filter response and, when oversampling, place the
//                 product in the longer spectrum (Fourier interpolation with the
//                 Nyquist bin split in half, as scipy.signal.resample does),
//   rc_crop     - cut the exact-lag window out of the correlation and scale it.
// Each is one pass over its data: grid-stride loops, coalesced complex64 accesses.
// decode_iq turns raw capture frames (int16 I/Q after a header) into complex64 pulses.
#include "common.cuh"

namespace sarbp {
namespace {

constexpr int kRowThreads = 256;

// One block per pulse: the row's mean (FP32 partial sums per thread, FP64 across threads),
// then the centred, zero-padded row.  Rows are read as float4 pairs when 16-byte aligned.
__global__ void rc_prepare_kernel(const float2* __restrict__ raw, int samples, int nfft, float2* __restrict__ out) {
    const int row = blockIdx.x;
    const float2* x = raw + (size_t)row * samples;
    float pr = 0.0f, pi = 0.0f;
    const bool vec = ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
    const int pairs = vec ? samples / 2 : 0;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    for (int j = threadIdx.x; j < pairs; j += kRowThreads) {
        const float4 v = x4[j];
        pr += v.x + v.z;
        pi += v.y + v.w;
    }
    for (int j = 2 * pairs + threadIdx.x; j < samples; j += kRowThreads) {
        const float2 v = x[j];
        pr += v.x;
        pi += v.y;
    }
    double sr = pr, si = pi;
    __shared__ double red[2][kRowThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][warp] = sr;
        red[1][warp] = si;
    }
    __syncthreads();
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < kRowThreads / 32; ++w) {
        tr += red[0][w];
        ti += red[1][w];
    }
    const float mr = (float)(tr / samples), mi = (float)(ti / samples);  // complex64 mean, as the reference
    float2* y = out + (size_t)row * nfft;
    for (int j = threadIdx.x; j < nfft; j += kRowThreads) {
        float2 v = make_float2(0.0f, 0.0f);
        if (j < samples) {
            const float2 a = x[j];
            v = make_float2(a.x - mr, a.y - mi);
        }
        y[j] = v;
    }
}

// The same computation with the row held in registers between the mean and the write (one HBM
// read instead of two): P float4 (two samples each) per thread, rows of an even number of up to
// 2 * 256 * P samples starting on a 16-byte boundary.  Partial sums, their order and the FP64
// reduction are those of rc_prepare_kernel, so the output is bit-identical.
template <int P>
__global__ void __launch_bounds__(kRowThreads) rc_prepare_reg_kernel(const float2* __restrict__ raw, int samples,
                                                                     int nfft, float2* __restrict__ out) {
    const int row = blockIdx.x;
    const float2* x = raw + (size_t)row * samples;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const int pairs = samples / 2;
    float4 v[P];
    float pr = 0.0f, pi = 0.0f;
#pragma unroll
    for (int i = 0; i < P; ++i) {
        const int j = threadIdx.x + kRowThreads * i;
        v[i] = j < pairs ? x4[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < pairs) {
            pr += v[i].x + v[i].z;
            pi += v[i].y + v[i].w;
        }
    }
    double sr = pr, si = pi;
    __shared__ double red[2][kRowThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][warp] = sr;
        red[1][warp] = si;
    }
    __syncthreads();
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < kRowThreads / 32; ++w) {
        tr += red[0][w];
        ti += red[1][w];
    }
    const float mr = (float)(tr / samples), mi = (float)(ti / samples);  // complex64 mean, as the reference
    float2* y = out + (size_t)row * nfft;
#pragma unroll
    for (int i = 0; i < P; ++i) {
        const int j = threadIdx.x + kRowThreads * i;
        if (j < pairs) {
            y[2 * j] = make_float2(v[i].x - mr, v[i].y - mi);
            y[2 * j + 1] = make_float2(v[i].z - mr, v[i].w - mi);
        }
    }
    for (int j = samples + threadIdx.x; j < nfft; j += kRowThreads) y[j] = make_float2(0.0f, 0.0f);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// out[p, m] for m in [0, length): length == nfft multiplies in place order; a longer
// length places bins [0, nfft/2] at the front and the negative frequencies at the back,
// halving the positive Nyquist bin and copying it to the negative one (even nfft).
// spec and out may be the same array (length == nfft): no __restrict__ on either.
__global__ void rc_filter_kernel(const float2* spec, const float2* __restrict__ response, int pulses, int nfft,
                                 int length, float2* out) {
    const long long total = (long long)pulses * length;
    const int half = nfft / 2, nyq = nfft / 2 + 1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(t / length);
        const int m = (int)(t - (long long)p * length);
        const float2* s = spec + (size_t)p * nfft;
        float2 v = make_float2(0.0f, 0.0f);
        if (length == nfft) {
            v = cmul(s[m], response[m]);
        } else if (m < nyq) {
            v = cmul(s[m], response[m]);
            if ((nfft & 1) == 0 && m == half) v = make_float2(0.5f * v.x, 0.5f * v.y);
        } else if (m >= length - (nfft - nyq)) {
            const int k = m - length + nfft;  // negative frequency bin of the short spectrum
            v = cmul(s[k], response[k]);
        } else if ((nfft & 1) == 0 && m == length - half) {
            v = cmul(s[half], response[half]);
            v = make_float2(0.5f * v.x, 0.5f * v.y);
        }
        out[t] = v;
    }
}

// Row-per-blockIdx.y forms of the filter and the crop: column index from the x grid, no 64-bit
// division per element (grids with up to 65535 rows).
__global__ void rc_filter_rows_kernel(const float2* spec, const float2* __restrict__ response, int nfft, int length,
                                      float2* out) {
    const int p = blockIdx.y;
    const int half = nfft / 2, nyq = nfft / 2 + 1;
    const float2* s = spec + (size_t)p * nfft;
    float2* o = out + (size_t)p * length;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < length; m += gridDim.x * blockDim.x) {
        float2 v = make_float2(0.0f, 0.0f);
        if (length == nfft) {
            v = cmul(s[m], response[m]);
        } else if (m < nyq) {
            v = cmul(s[m], response[m]);
            if ((nfft & 1) == 0 && m == half) v = make_float2(0.5f * v.x, 0.5f * v.y);
        } else if (m >= length - (nfft - nyq)) {
            const int k = m - length + nfft;  // negative frequency bin of the short spectrum
            v = cmul(s[k], response[k]);
        } else if ((nfft & 1) == 0 && m == length - half) {
            v = cmul(s[half], response[half]);
            v = make_float2(0.5f * v.x, 0.5f * v.y);
        }
        o[m] = v;
    }
}

__global__ void rc_crop_rows_kernel(const float2* __restrict__ corr, int length, int offset, int samples, float scale,
                                    float2* __restrict__ out) {
    const int p = blockIdx.y;
    const float2* c = corr + (size_t)p * length + offset;
    float2* o = out + (size_t)p * samples;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < samples; j += gridDim.x * blockDim.x) {
        const float2 v = c[j];
        o[j] = make_float2(v.x * scale, v.y * scale);
    }
}

// Columns per block of the row kernels: enough blocks for every SM, a few columns per thread.
dim3 row_grid(int rows, int cols) {
    int bx = (cols + 4 * kRowThreads - 1) / (4 * kRowThreads);
    return dim3(bx > 0 ? bx : 1, rows);
}

__global__ void rc_crop_kernel(const float2* __restrict__ corr, int pulses, int length, int offset, int samples,
                               float scale, float2* __restrict__ out) {
    const long long total = (long long)pulses * samples;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(t / samples);
        const int j = (int)(t - (long long)p * samples);
        const float2 v = corr[(size_t)p * length + offset + j];
        out[t] = make_float2(v.x * scale, v.y * scale);
    }
}

// Raw frames -> complex64: frame i's I/Q pairs start iq_offset bytes into the frame.
__global__ void decode_iq_kernel(const unsigned char* __restrict__ frames, int n, long long frame_size, int iq_offset,
                                 int nr, float2* __restrict__ out) {
    const long long total = (long long)n * nr;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = t / nr, j = t - i * nr;
        const short2 v = *reinterpret_cast<const short2*>(frames + i * frame_size + iq_offset + 4 * j);
        out[t] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void decode_iq_rows_kernel(const unsigned char* __restrict__ frames, long long frame_size, int iq_offset,
                                      int nr, float2* __restrict__ out) {
    const long long i = blockIdx.y;
    const unsigned char* f = frames + i * frame_size + iq_offset;
    float2* o = out + i * nr;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nr; j += gridDim.x * blockDim.x) {
        const short2 v = *reinterpret_cast<const short2*>(f + 4 * (long long)j);
        o[j] = make_float2((float)v.x, (float)v.y);
    }
}

int stream_grid(long long n) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = (n + kRowThreads - 1) / kRowThreads;
    return (int)(blocks < 8LL * sms ? (blocks > 0 ? blocks : 1) : 8LL * sms);
}

}  // namespace

int launch_rc_prepare(const float2* raw, int pulses, int samples, int nfft, float2* out, cudaStream_t s) {
    const long long pairs = samples / 2;
    const bool aligned = (reinterpret_cast<uintptr_t>(raw) & 15) == 0 && (samples & 1) == 0;
    if (aligned && pairs <= 4LL * kRowThreads)
        rc_prepare_reg_kernel<4><<<pulses, kRowThreads, 0, s>>>(raw, samples, nfft, out);
    else if (aligned && pairs <= 8LL * kRowThreads)
        rc_prepare_reg_kernel<8><<<pulses, kRowThreads, 0, s>>>(raw, samples, nfft, out);
    else if (aligned && pairs <= 16LL * kRowThreads)
        rc_prepare_reg_kernel<16><<<pulses, kRowThreads, 0, s>>>(raw, samples, nfft, out);
    else
        rc_prepare_kernel<<<pulses, kRowThreads, 0, s>>>(raw, samples, nfft, out);
    note_launches(1);
    return check_launch("rc_prepare");
}

int launch_rc_filter(const float2* spec, const float2* response, int pulses, int nfft, int length, float2* out,
                     cudaStream_t s) {
    if (pulses <= 65535)
        rc_filter_rows_kernel<<<row_grid(pulses, length), kRowThreads, 0, s>>>(spec, response, nfft, length, out);
    else
        rc_filter_kernel<<<stream_grid((long long)pulses * length), kRowThreads, 0, s>>>(spec, response, pulses, nfft,
                                                                                        length, out);
    note_launches(1);
    return check_launch("rc_filter");
}

int launch_decode_iq(const unsigned char* frames, int n, long long frame_size, int iq_offset, int nr, float2* out,
                     cudaStream_t s) {
    if (n <= 65535)
        decode_iq_rows_kernel<<<row_grid(n, nr), kRowThreads, 0, s>>>(frames, frame_size, iq_offset, nr, out);
    else
        decode_iq_kernel<<<stream_grid((long long)n * nr), kRowThreads, 0, s>>>(frames, n, frame_size, iq_offset, nr,
                                                                               out);
    note_launches(1);
    return check_launch("decode_iq");
}

int launch_rc_crop(const float2* corr, int pulses, int length, int offset, int samples, float scale, float2* out,
                   cudaStream_t s) {
    if (pulses <= 65535)
        rc_crop_rows_kernel<<<row_grid(pulses, samples), kRowThreads, 0, s>>>(corr, length, offset, samples, scale,
                                                                               out);
    else
        rc_crop_kernel<<<stream_grid((long long)pulses * samples), kRowThreads, 0, s>>>(corr, pulses, length, offset,
                                                                                       samples, scale, out);
    note_launches(1);
    return check_launch("rc_crop");
}

}  // namespace sarbp
