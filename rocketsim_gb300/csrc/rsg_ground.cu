// rsg_ground.cu -- differentiable driving rollouts of one car on the arena floor: the forward and
// tape kernels and the C ABI (the model and the reverse tick are in rsg_ground.cuh, the reverse
// sweep in rsg_ground_sweep.cu).
#include "rsg_ground.cuh"

namespace rsg {
namespace ground {

// ---------------------------------------------------------------- kernels
// 128 registers: 4 warps per SM sub-partition (16K registers each), 512 threads per SM, so 65536
// instances run in one wave on 152 SMs.
__global__ void __maxnreg__(128) ground_forward_kernel(int n, int ticks, const float* __restrict__ state0,
                                                       const float4* __restrict__ controls,
                                                       float* __restrict__ final_state, float* __restrict__ ckpt,
                                                       int ckpt_every, int* __restrict__ flags, Cfg k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fill_damping(k);
    GS x = load_state(state0 + (size_t)i * STATE);
    unsigned fl = 0;
    float4 un = ticks > 0 ? controls[i] : make_float4(0, 0, 0, 0);
    for (int t = 0; t < ticks; t++) {
        const float4 u = un;
        if (t + 1 < ticks) un = controls[(size_t)(t + 1) * n + i];  // a tick ahead
        if (ckpt && t % ckpt_every == 0) store_state(ckpt + ((size_t)(t / ckpt_every) * n + i) * STATE, x);
        fl |= car_tick(x, u, k, nullptr);
        ball_tick(x, k);
    }
    store_state(final_state + (size_t)i * STATE, x);
    if (flags) flags[i] = (int)fl;
}

// One thread per (segment, instance): recompute the segment from its checkpoint and write the
// tape, word w of tick t at tape[(t * TAPE_WORDS + w) * n + i].
__global__ void __maxnreg__(128) ground_tape_kernel(int n, int ticks, const float4* __restrict__ controls,
                                                    const float* __restrict__ ckpt, int ckpt_every, int nseg,
                                                    float* __restrict__ tape, Cfg k) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nseg * n) return;
    const int sgi = (int)(idx / n), i = (int)(idx % n);
    fill_damping(k);
    const int t0 = sgi * ckpt_every;
    const int t1 = t0 + ckpt_every < ticks ? t0 + ckpt_every : ticks;
    GS x = load_state(ckpt + ((size_t)sgi * n + i) * STATE);
    float4 un = controls[(size_t)t0 * n + i];
    for (int t = t0; t < t1; t++) {
        const float4 u = un;
        if (t + 1 < t1) un = controls[(size_t)(t + 1) * n + i];
        const Strided out{tape + (size_t)t * TAPE_WORDS * n + i, (size_t)n};
        store_state(out, x);
        adj::IntTape it;
        car_tick(x, u, k, &it);
        ball_tick(x, k);
        out[STATE + 0] = it.v1u.x;
        out[STATE + 1] = it.v1u.y;
        out[STATE + 2] = it.v1u.z;
        out[STATE + 3] = it.w1u.x;
        out[STATE + 4] = it.w1u.y;
        out[STATE + 5] = it.w1u.z;
    }
}

static Cfg make_cfg(const rsg_car_config* c, float tick_rate) {
    const CarCfgDev d = car_config_derived(*c);
    Cfg k;
    k.iinv = V3(d.inv_inertia[0], d.inv_inertia[1], d.inv_inertia[2]);
    k.dt = 1.f / tick_rate;
    for (int i = 0; i < 4; i++) k.conn[i] = V3(d.conn[i][0], d.conn[i][1], d.conn[i][2]);
    for (int f = 0; f < 2; f++) {
        k.rest[f] = d.rest[f];
        k.radius[f] = d.radius[f];
    }
    k.car_damp = k.ball_damp = 0.f;  // set by fill_damping on the device
    return k;
}

}  // namespace ground
}  // namespace rsg

using namespace rsg;

static size_t ground_tape_bytes(int n, int ticks) {
    return sizeof(float) * ground::TAPE_WORDS * (size_t)n * (size_t)ticks;
}

extern "C" int rsg_ground_forward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_state0,
                                  const float* d_controls, float* d_final, float* d_ckpt, int ckpt_every, int* d_flags,
                                  void* stream) {
    if (!car || n < 0 || ticks < 0 || !d_state0 || !d_controls || !d_final || !(tick_rate > 0.f))
        return report_error(RSG_ERR_ARG, "rsg_ground_forward: null pointer, negative size or tick_rate <= 0");
    if (d_ckpt && ckpt_every < 1) return report_error(RSG_ERR_ARG, "rsg_ground_forward: ckpt_every must be >= 1");
    if (n == 0) return RSG_OK;
    ground::Cfg k = ground::make_cfg(car, tick_rate);
    ground::ground_forward_kernel<<<(n + 63) / 64, 64, 0, (cudaStream_t)stream>>>(
        n, ticks, d_state0, reinterpret_cast<const float4*>(d_controls), d_final, d_ckpt, d_ckpt ? ckpt_every : 1,
        d_flags, k);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RSG_OK : report_error(RSG_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int rsg_ground_backward_workspace_size(int n, int ticks, size_t* bytes) {
    if (n < 0 || ticks < 0 || !bytes)
        return report_error(RSG_ERR_ARG, "rsg_ground_backward_workspace_size: negative size or null pointer");
    *bytes = ground_tape_bytes(n, ticks);
    return RSG_OK;
}

extern "C" int rsg_ground_backward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_controls,
                                   const float* d_ckpt, int ckpt_every, const float* d_grad_final,
                                   float* d_grad_controls, float* d_grad_state0, void* d_workspace,
                                   size_t workspace_bytes, void* stream) {
    if (!car || n < 0 || ticks < 0 || !d_controls || !d_ckpt || !d_grad_final || !d_grad_controls ||
        !(tick_rate > 0.f))
        return report_error(RSG_ERR_ARG, "rsg_ground_backward: null pointer, negative size or tick_rate <= 0");
    if (ckpt_every < 1) return report_error(RSG_ERR_ARG, "rsg_ground_backward: ckpt_every must be >= 1");
    if (n == 0) return RSG_OK;
    if (ticks == 0) {  // the gradient passes straight through
        if (d_grad_state0)
            if (cudaMemcpyAsync(d_grad_state0, d_grad_final, sizeof(float) * ground::STATE * (size_t)n,
                                cudaMemcpyDeviceToDevice, (cudaStream_t)stream) != cudaSuccess)
                return report_error(RSG_ERR_CUDA, "rsg_ground_backward: copy of the gradient failed");
        return RSG_OK;
    }
    if (!d_workspace || workspace_bytes < ground_tape_bytes(n, ticks))
        return report_error(RSG_ERR_ARG, "rsg_ground_backward: workspace missing or smaller than "
                                         "rsg_ground_backward_workspace_size");
    ground::Cfg k = ground::make_cfg(car, tick_rate);
    const int nseg = (ticks + ckpt_every - 1) / ckpt_every;
    const long long tape_threads = (long long)nseg * n;
    float* tape = static_cast<float*>(d_workspace);
    ground::ground_tape_kernel<<<(unsigned)((tape_threads + 63) / 64), 64, 0, (cudaStream_t)stream>>>(
        n, ticks, reinterpret_cast<const float4*>(d_controls), d_ckpt, ckpt_every, nseg, tape, k);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = ground::launch_ground_sweep(n, ticks, reinterpret_cast<const float4*>(d_controls), tape, d_grad_final,
                                        reinterpret_cast<float4*>(d_grad_controls), d_grad_state0, k,
                                        (cudaStream_t)stream);
    return e == cudaSuccess ? RSG_OK : report_error(RSG_ERR_CUDA, cudaGetErrorString(e));
}
