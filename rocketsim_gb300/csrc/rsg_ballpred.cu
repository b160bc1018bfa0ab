// rsg_ballpred.cu -- BallPredTracker (src/Sim/BallPredTracker/BallPredTracker.cpp:5-79) for every
// arena of a batch at once.
//
// Each source arena has a ball-only arena in a tracker batch (the reference's ballPredArena: same
// game mode, arena config and tick rate, default mutators, no cars) and a ring of `T` predicted ball
// states in HBM ([A][T] rsg_ball_state, `head[a]` = predData[0]).  An update runs in two launches:
//
//   plan   one thread per arena: UpdatePredManual's decision.  With k ticks since the last update,
//          0 <= k < T and predData[k].Matches(current) the ring's front advances by k and k new
//          states are due, simulated from predData.back(); otherwise predData[0] = current and T - 1
//          states are due.  The arena's ball is set to the start state and the arena is appended to
//          a run list with its step count and first ring slot.
//   run    the arena tick (rsg_tick.cuh, one warp per arena as in the main tick kernel) over the run
//          list, each block for the largest step count among its arenas; after each tick an arena
//          still within its own count writes its ball state into its next ring slot.  Ticks past an
//          arena's count change only its own ball, which the next plan sets again before use.
//
// The run list is built with an atomic counter, so which arenas share a block varies from call to
// call; arenas are independent, so the results do not.  The tracker batch holds no cars, so the
// tick's car-car code (and the EPA work pool of the main translation unit) is never reached here.
#include "rsg_kernels.h"
#include "rsg_tick.cuh"
#include "rsg_view.cuh"

namespace rsg {

// BallState::Matches (src/Sim/Ball/Ball.cpp:12-17) with its default margins (Ball.h:53): squared
// distances of position, velocity and angular velocity below 0.8^2, 0.4^2 and 0.02^2, each summed
// x, y, z in that order (Vec::LengthSq, MathTypes.h:36-38; the fourth component is 0).
RSG_D float dist_sq(const rsg_vec3& a, const rsg_vec3& b) {
    const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}
RSG_D bool ball_matches(const rsg_ball_state& s, const rsg_ball_state& o) {
    const float mp = 0.8f, mv = 0.4f, ma = 0.02f;
    return dist_sq(s.pos, o.pos) < __fmul_rn(mp, mp) && dist_sq(s.vel, o.vel) < __fmul_rn(mv, mv) &&
           dist_sq(s.ang_vel, o.ang_vel) < __fmul_rn(ma, ma);
}

// mode 0: UpdatePredFromArena (current state and tick count read from the source batch);
// mode 1: UpdatePredManual (cur[a], ticks[a]); mode 2: ForceUpdateAllPred (cur[a]).
// mask (may be null): arenas with mask[a] == 0 are left alone.
__global__ void rsg_ball_pred_plan_kernel(BatchView pv, BallPredDev d, BatchView src, int mode,
                                          const rsg_ball_state* __restrict__ cur, const int32_t* __restrict__ ticks,
                                          const uint8_t* __restrict__ mask) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= pv.A) return;
    if (mask && !mask[a]) return;
    const int T = d.T;
    rsg_ball_state now;
    int k = 0;
    if (mode == 0) {
        SoA s{src, a};
        now = ball_get(s);
        // int ticksSinceLastUpdate = arena->tickCount - lastUpdateTickCount (BallPredTracker.cpp:20)
        k = (int)((uint32_t)s.au(AU_TICK_LO) - (uint32_t)d.last_update[a]);
    } else {
        now = cur[a];
        k = mode == 1 ? ticks[a] : 0;
    }
    rsg_ball_state* ring = d.pred + (size_t)a * T;
    const uint32_t head = d.head[a];
    const bool reuse = mode != 2 && d.valid[a] && k >= 0 && k < T && ball_matches(ring[(head + (uint32_t)k) % T], now);
    int steps = 0;
    uint32_t base = 0;
    if (reuse) {
        if (k > 0) {  // drop the k oldest states, simulate k more from the last one
            ball_set(SoA{pv, a}, ring[(head + T - 1) % T]);
            steps = k;
            base = head;  // the freed slots, in order
            d.head[a] = (head + (uint32_t)k) % T;
        }
    } else {  // ForceUpdateAllPred (BallPredTracker.cpp:64-72)
        ball_set(SoA{pv, a}, now);
        ring[0] = now;
        d.head[a] = 0;
        steps = T - 1;
        base = 1;
        d.valid[a] = 1;
    }
    if (mode != 2) d.last_update[a] = (int32_t)((uint32_t)d.last_update[a] + (uint32_t)k);
    if (steps > 0) {
        d.steps[a] = steps;
        d.base[a] = base;
        const int at = atomicAdd(d.count, 1);
        d.list[at] = a;
    }
}

RSG_D rsg_ball_state ball_from_ctx(const Ctx& a) {
    rsg_ball_state o;
    const Body& b = a.ball;
    o.pos = to_rv(b.xf.o * RL::BT_TO_UU);
    o.rot_mat = basis_to_rot(b.xf.b);
    o.vel = to_rv(b.lin_vel * RL::BT_TO_UU);
    o.ang_vel = to_rv(b.ang_vel);
    o.tick_count_since_update = a.ball_ticks;
    return o;
}

// The arena tick of rsg_tick_kernel (rsg_kernels.cu) over the run list, recording the ball.
__global__ void __launch_bounds__(256, 2) rsg_ball_pred_run_kernel(BatchView bv, BallPredDev d, int hdr_cache) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int count = *d.count;
    const int first = blockIdx.x * wpb;
    if (first >= count) return;  // block-uniform, before any barrier
    const int nact = count - first < wpb ? count - first : wpb;
    const bool active = warp < nact;
    const int ar = active ? d.list[first + warp] : 0;
    const SmemLayout L = smem_layout(bv.MC);
    Ctx& a = bind_ctx(smem + (size_t)warp * L.bytes, L, lane);
    const Subtree* sub = bv.mesh.sub;
    if (hdr_cache) {
        uint32_t* dst = reinterpret_cast<uint32_t*>(smem + (size_t)wpb * L.bytes);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(bv.mesh.sub);
        for (int i = threadIdx.x; i < bv.mesh.nsub * 5; i += blockDim.x) dst[i] = __ldg(src + i);
        sub = reinterpret_cast<const Subtree*>(dst);
    }
    __shared__ int s_ticks;
    if (threadIdx.x == 0) s_ticks = 0;
    __syncthreads();
    int my_steps = 0;
    uint32_t slot = 0;
    if (active) {
        my_steps = d.steps[ar];
        slot = d.base[ar];
        if (lane == 0) {
            load_arena(bv, ar, a);
            a.sub = sub;
            atomicMax(&s_ticks, my_steps);
        }
        __syncwarp();
        load_pads(bv, ar, a, lane);
        __syncwarp();
    }
    __syncthreads();
    const int ticks = s_ticks;
    const BlockArenas B{smem, L.bytes, nact};
    rsg_ball_state* ring = d.pred + (size_t)ar * d.T;
    for (int t = 0; t < ticks; t++) {
        __syncthreads();
        block_tick_pre(bv, B, threadIdx.x, blockDim.x);
        if (active) step_bodies_pre(bv, a, lane);
        __syncthreads();
        step_collide_block(bv, a, lane, active, false);
        __syncthreads();
        block_tick_post(bv, B, threadIdx.x, blockDim.x);
        if (active && lane == 0 && t < my_steps) {
            ring[slot] = ball_from_ctx(a);
            slot = slot + 1 == (uint32_t)d.T ? 0 : slot + 1;
        }
    }
    if (active) {
        if (lane == 0) store_arena(bv, ar, a);
        store_pads(bv, ar, a, lane);
    }
}

cudaError_t launch_ball_pred(const BatchBuffers& pred, const BallPredDev& d, const BatchBuffers* src, int mode,
                             const rsg_ball_state* cur, const int32_t* ticks, const uint8_t* mask, cudaStream_t st) {
    if (pred.A <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d.count, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    const BatchView pv = make_view(pred);
    const BatchView sv = src ? make_view(*src) : pv;
    rsg_ball_pred_plan_kernel<<<(pred.A + 127) / 128, 128, 0, st>>>(pv, d, sv, mode, cur, ticks, mask);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (d.T <= 1) return cudaSuccess;
    const int wpb = 8;
    const int per_arena = smem_layout(pred.MC).bytes;
    int smem = per_arena * wpb;
    const int hdr_bytes = pred.mesh.sub ? pred.mesh.nsub * (int)sizeof(Subtree) : 0;
    // two blocks per SM (128 registers a thread): the header copy only where both still fit
    const int hdr_cache = (hdr_bytes > 0 && 2 * (smem + hdr_bytes + 1024) <= 228 * 1024) ? 1 : 0;
    if (hdr_cache) smem += hdr_bytes;
    if ((e = cudaFuncSetAttribute(rsg_ball_pred_run_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) !=
        cudaSuccess)
        return e;
    rsg_ball_pred_run_kernel<<<(pred.A + wpb - 1) / wpb, 32 * wpb, smem, st>>>(pv, d, hdr_cache);
    return cudaGetLastError();
}

}  // namespace rsg
