// rsg_air_noalloc.cu -- the air-phase adjoint for callers that cannot allocate device memory.
//
// rsg_air_backward needs a tape workspace (152 bytes per instance and tick) that the caller
// allocates.  Some callers cannot do that: a plugin inside a host program whose device memory
// belongs to another allocator that has already reserved most of the GPU (a game engine, or a
// framework with its own caching pool), or a control loop that cannot afford the device-wide
// synchronisation that cudaMalloc and cudaFree may cause.  rsg_air_backward_noalloc serves them:
// its tape lives in the fixed-size array below, which the CUDA driver places in device memory
// when it loads this file's module, so the call itself allocates nothing.
//
// Limits and rules for callers:
//  * the array holds AIR_NOALLOC_TAPE_BYTES (16 MiB): n * ticks may be at most
//    AIR_NOALLOC_TAPE_BYTES / 152 = 110376 (e.g. 1839 instances x 60 ticks); larger requests
//    are rejected with RSG_ERR_ARG and a message, and launch nothing;
//  * every call on a device shares the one array, so calls whose kernels overlap on the GPU
//    (different streams, or different host threads without ordering) race on it and produce
//    garbage; order them on one stream or synchronise between them;
//  * nothing in the array needs to start at zero: the tape kernel writes every word the sweep
//    kernel reads, for the call's own n and ticks, before the sweep starts;
//  * the first call on each device looks up the array's device address (cudaGetSymbolAddress,
//    with that device current) and keeps it; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/rocketsim_gb300.h"
#include "rsg_kernels.h"

namespace {

constexpr size_t AIR_NOALLOC_TAPE_BYTES = size_t(16) << 20;
constexpr size_t AIR_TAPE_BYTES_PER_TICK = 152;  // 38 floats per instance and tick
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_air_tape[AIR_NOALLOC_TAPE_BYTES];

std::mutex g_setup_mutex;
void* g_tape_ptr[MAX_DEVICES] = {};

// The array's address on the current device, looked up once per device.
int tape_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return rsg::report_error(RSG_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES)
        return rsg::report_error(RSG_ERR_STATE, "rsg_air_backward_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_tape_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_air_tape);
        if (e != cudaSuccess) {
            std::string msg = std::string("rsg_air_backward_noalloc: cudaGetSymbolAddress failed: ") +
                              cudaGetErrorString(e);
            return rsg::report_error(RSG_ERR_CUDA, msg.c_str());
        }
        g_tape_ptr[dev] = p;
    }
    *out = g_tape_ptr[dev];
    return RSG_OK;
}

}  // namespace

extern "C" int rsg_air_backward_noalloc(const rsg_car_config* car, float tick_rate, int n, int ticks,
                                        const float* d_controls, const float* d_ckpt, int ckpt_every,
                                        const float* d_grad_final, float* d_grad_controls, float* d_grad_state0,
                                        void* stream) {
    if (n < 0 || ticks < 0)
        return rsg::report_error(RSG_ERR_ARG, "rsg_air_backward_noalloc: negative size");
    const size_t need = AIR_TAPE_BYTES_PER_TICK * (size_t)n * (size_t)ticks;
    if (need > AIR_NOALLOC_TAPE_BYTES) {
        std::string msg = "rsg_air_backward_noalloc: n * ticks = " + std::to_string((size_t)n * (size_t)ticks) +
                          " needs " + std::to_string(need) + " bytes of tape, above the " +
                          std::to_string(AIR_NOALLOC_TAPE_BYTES) + "-byte static scratch (n * ticks <= " +
                          std::to_string(AIR_NOALLOC_TAPE_BYTES / AIR_TAPE_BYTES_PER_TICK) +
                          "); use rsg_air_backward with a workspace";
        return rsg::report_error(RSG_ERR_ARG, msg.c_str());
    }
    void* tape = nullptr;
    int rc = tape_address(&tape);
    if (rc != RSG_OK) return rc;
    return rsg_air_backward(car, tick_rate, n, ticks, d_controls, d_ckpt, ckpt_every, d_grad_final, d_grad_controls,
                            d_grad_state0, tape, AIR_NOALLOC_TAPE_BYTES, stream);
}
