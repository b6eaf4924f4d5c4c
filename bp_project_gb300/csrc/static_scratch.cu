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

// Device address of g_static_scratch on the current device, looked up once per device.  The
// cached address does not survive cudaDeviceReset (the module, and with it the array, is loaded
// again afterwards); a process that resets a device must not call the static entry point on it
// again.
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
    // The same checks, in the same order, as sarbp_direct_polar(mode = SARBP_SPLIT).
    if (int st = check_pulses(data, pulses, samples, pos, weight, phase, data_dr, k)) return st;
    if (int st = check_grid(grid)) return st;
    if (!out) return fail(SARBP_ERR_TYPE, "out must not be NULL");
    if (chunk_pulses <= 0) return fail(SARBP_ERR_VALUE, "chunk_pulses must be positive");
    if (pulse_split < 1 || pulse_split > pulses) return fail(SARBP_ERR_VALUE, "pulse_split must be in [1, pulses]");
    // nr * nu fits 63 bits (both are positive ints); compare against the capacity divided by the
    // split so that no product can wrap.
    const long long npix = (long long)grid->nr * grid->nu;
    if (pulse_split > 1 && npix > (long long)(kStaticScratchElems / (size_t)pulse_split))
        return fail(SARBP_ERR_VALUE,
                    "pulse_split * nr * nu = %d * %lld exceeds the static scratch of %zu complex64 values; "
                    "use sarbp_direct_polar with a workspace",
                    pulse_split, npix, kStaticScratchElems);
    float2* scratch = nullptr;
    if (pulse_split > 1) {
        if (int st = static_scratch(&scratch)) return st;
    }
    // Every partial image is fully overwritten by the split kernel, so the scratch needs no
    // clearing between calls.
    const PulseInputs in = inputs_of(data, pulses, samples, pos, weight, phase, range_start, data_dr, k);
    return split_direct_polar(in, *grid, chunk_pulses, pulse_split, scratch, reinterpret_cast<float2*>(out),
                              (cudaStream_t)stream);
}

}  // extern "C"
