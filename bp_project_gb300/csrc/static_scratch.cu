// Allocation-free variant of pulse-split direct BP (sarbp_direct_polar_static).
//
// sarbp_direct_polar with pulse_split > 1 needs a scratch buffer for the
// partial images, which the caller allocates and passes as `workspace`.  Some
// callers cannot allocate device memory at the point where they image: hosts
// that own all device memory through their own pool and forbid cudaMalloc
// after start-up, real-time processing loops where cudaMalloc/cudaFree would
// synchronise the device, and foreign-language hosts (cgo, JNI) that only see
// the buffers handed to them.  For them this file keeps the scratch in a fixed
// device array, sized once for all calls.
#include <mutex>

#include "common.cuh"

namespace sarbp {
namespace {

// 2^21 complex64 values = 16 MiB: room for pulse_split * nr * nu <= 2,097,152
// (e.g. 8 partial images of 512 x 512).  Every GPU that loads this library
// holds the array until the process exits.
constexpr size_t kStaticScratchElems = size_t(1) << 21;
static __device__ __align__(256) float2 g_static_scratch[kStaticScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
float2* g_scratch_address[kMaxDevices] = {};

// Device address of g_static_scratch on the current device, looked up once per device.
int static_scratch(float2** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(SARBP_ERR_CUDA, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_address[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(SARBP_ERR_CUDA, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
        g_scratch_address[dev] = reinterpret_cast<float2*>(ptr);
    }
    *out = g_scratch_address[dev];
    return SARBP_OK;
}

}  // namespace
}  // namespace sarbp

using namespace sarbp;

extern "C" {

size_t sarbp_static_scratch_elements(void) { return kStaticScratchElems; }

int sarbp_direct_polar_static(const float* data, int pulses, int samples, const double* pos, const double* weight,
                              const double* phase, const sarbp_polar_grid* grid, double range_start, double data_dr,
                              double k, int chunk_pulses, int pulse_split, float* out, void* stream) {
    if (!data || !pos || !weight || !phase || !grid || !out)
        return fail(SARBP_ERR_TYPE, "data, pos, weight, phase, grid and out must not be NULL");
    if (pulses < 1 || samples < 1) return fail(SARBP_ERR_VALUE, "pulses and samples must be positive");
    if (grid->nr <= 0 || grid->nu <= 0) return fail(SARBP_ERR_VALUE, "empty image grids are unsupported");
    if (grid->side != 1 && grid->side != -1) return fail(SARBP_ERR_VALUE, "side must be +1 or -1");
    if (!isfinite(data_dr) || data_dr == 0.0 || !isfinite(k)) return fail(SARBP_ERR_VALUE, "data_dr and k must be finite, data_dr non-zero");
    if (chunk_pulses <= 0) return fail(SARBP_ERR_VALUE, "chunk_pulses must be positive");
    if (pulse_split < 1 || pulse_split > pulses) return fail(SARBP_ERR_VALUE, "pulse_split must be in [1, pulses]");
    const long long npix = (long long)grid->nr * grid->nu;
    if (pulse_split > 1 && (unsigned long long)npix * (unsigned long long)pulse_split > kStaticScratchElems)
        return fail(SARBP_ERR_VALUE,
                    "pulse_split * nr * nu = %lld exceeds the static scratch of %zu complex64 values; "
                    "use sarbp_direct_polar with a workspace",
                    npix * pulse_split, kStaticScratchElems);
    float2* scratch = nullptr;
    if (pulse_split > 1) {
        if (int st = static_scratch(&scratch)) return st;
    }
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
    PolarDesc g{};
    g.ox = grid->origin[0];
    g.oy = grid->origin[1];
    g.oz = grid->origin[2];
    g.r0 = grid->r0;
    g.dr = grid->dr;
    g.u0 = grid->u0;
    g.du = grid->du;
    g.nr = grid->nr;
    g.nu = grid->nu;
    g.side = grid->side;
    g.a = 0;
    g.b = pulses;
    g.left = g.right = -1;
    g.win_nr = grid->nr;
    g.win_nu = grid->nu;
    g.out_stride = grid->nu;
    split_geometry(g);
    double radius = 0.0;
    g.tile_lc = split_polar_tile_lc(g, &radius);
    const int wb = split_window_bins(radius, data_dr);
    const int ch = split_chunk_for(wb, chunk_pulses);
    cudaStream_t s = (cudaStream_t)stream;
    float2* dst = reinterpret_cast<float2*>(out);
    // Every partial image is fully overwritten by the split kernel, so the
    // scratch needs no clearing between calls.
    int st = launch_split_polar(in, g, pulse_split, ch, wb, pulse_split > 1 ? scratch : dst, g.nu, npix, s);
    if (st == SARBP_OK && pulse_split > 1) st = launch_sum_parts(scratch, pulse_split, npix, npix, dst, s);
    return st;
}

}  // extern "C"
