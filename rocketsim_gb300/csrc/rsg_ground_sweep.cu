// rsg_ground_sweep.cu -- the reverse sweep of the ground-driving adjoint (model and reverse tick in
// rsg_ground.cuh).
//
// This translation unit is compiled with -prec-div=false -prec-sqrt=false: the sweep recomputes
// each tick's intermediates only to linearise around them, from the exact start state on the
// tape, so divisions and square roots correct to about 2 ulp serve as well as correctly rounded
// ones and shrink the instruction stream and the code that the instruction cache must hold.  The
// forward and tape kernels, whose states must equal the arena tick's, are compiled with IEEE
// division and square root (rsg_ground.cu).
#include "rsg_ground.cuh"

namespace rsg {
namespace ground {

// One thread per instance: the reverse pass over all ticks.  The tape entry of a tick is read when
// the tick starts (its loads are independent of one another and mostly L2 hits; a reverse tick is
// tens of thousands of cycles, so keeping 45 registers for a prefetch would cost more in spills).
__global__ void __maxnreg__(128) ground_sweep_kernel(int n, int ticks, const float4* __restrict__ controls,
                                                     const float* __restrict__ tape,
                                                     const float* __restrict__ grad_final,
                                                     float4* __restrict__ grad_controls,
                                                     float* __restrict__ grad_state0, Cfg k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fill_damping(k);
    GS g = load_state(grad_final + (size_t)i * STATE);
    for (int t = ticks - 1; t >= 0; t--) {
        const Strided src{const_cast<float*>(tape) + (size_t)t * TAPE_WORDS * n + i, (size_t)n};
        const GS x0 = load_state(src);
        const V3 v1u(src[STATE + 0], src[STATE + 1], src[STATE + 2]);
        const V3 w1u(src[STATE + 3], src[STATE + 4], src[STATE + 5]);
        grad_controls[(size_t)t * n + i] = tick_bwd(x0, controls[(size_t)t * n + i], v1u, w1u, k, g);
    }
    if (grad_state0) store_state(grad_state0 + (size_t)i * STATE, g);
}

cudaError_t launch_ground_sweep(int n, int ticks, const float4* controls, const float* tape, const float* grad_final,
                                float4* grad_controls, float* grad_state0, const Cfg& k, cudaStream_t st) {
    ground_sweep_kernel<<<(n + 63) / 64, 64, 0, st>>>(n, ticks, controls, tape, grad_final, grad_controls, grad_state0,
                                                       k);
    return cudaGetLastError();
}

}  // namespace ground
}  // namespace rsg
