// rsg_kernels.cu -- kernels of the batched arena tick and the state gather /
// scatter kernels behind the C ABI.
//
// rsg_tick_kernel: one warp advances one arena by `ticks` ticks (its record is
// loaded into the warp's shared-memory region, the ticks run there in block-wide
// parts, and the record is stored back).  Arenas are independent; a block advances
// one group of arenas per block of the grid, or, in a persistent launch, groups
// taken from a counter until none is left.
#include <map>
#include <mutex>
#include <tuple>

#include "rsg_kernels.h"
#include "rsg_tick.cuh"
#include "rsg_view.cuh"

namespace rsg {

static_assert(sizeof(DevEvent) == DEV_EVENT_BYTES, "event record size");

// The tick kernel keeps the parts of an arena's working set that live only within a tick's collision
// work — manifold points, solver rows, solver bodies, candidate and island lists — in a global scratch
// per warp slot (L1-cached; only what a tick uses is touched), so that more arenas fit an SM's shared
// memory.
constexpr bool kRowsInSmem = false;
constexpr bool kPtsInSmem = false;
constexpr bool kMoreInSmem = false;

RSG_D void apply_controls(Car& c, const rsg_car_controls& k) {
    c.ctrl[0] = k.throttle;
    c.ctrl[1] = k.steer;
    c.ctrl[2] = k.pitch;
    c.ctrl[3] = k.yaw;
    c.ctrl[4] = k.roll;
    c.setf(F_CTRL_JUMP, k.jump != 0);
    c.setf(F_CTRL_BOOST, k.boost != 0);
    c.setf(F_CTRL_HB, k.handbrake != 0);
}

// One warp per arena: the arena's working set is carved out of dynamic shared memory
// (smem_layout), loaded from its record, advanced `ticks` ticks and stored back.  The warps of a
// block step through the parts of a tick together (block-wide barriers between parts), which keeps
// the instruction working set of an SM to one part of the tick at a time.  Group g of the launch
// (warp slots g * wpb ...) advances arenas place[g * wpb + warp]; lane 0 adds up the cycles of the
// arena's own collision work into cost[].  Block b takes group b; a persistent launch (as many blocks
// as are resident at once) then takes the next groups from the counter *group_next, in group order,
// so that the dearest groups (placed first) start first and the cheapest fill in at the end.
__global__ void __launch_bounds__(32 * TICK_MAX_ARENAS_PER_BLOCK, 1) rsg_tick_kernel(BatchView bv, const rsg_car_controls* __restrict__ controls,
                                                          int ticks, int hdr_cache, int collide_sync,
                                                          const uint32_t* __restrict__ place, uint32_t* __restrict__ cost,
                                                          uint32_t* group_next) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int ngroups = (bv.A + wpb - 1) / wpb;
    if ((long long)(blockIdx.x + 1) * wpb > bv.scratch_slots) {  // launch_tick keeps the grid within the slots
        for (int g = blockIdx.x; g < ngroups; g += gridDim.x)
            if (threadIdx.x < wpb && g * wpb + (int)threadIdx.x < bv.A)
                atomicOr(&bv.au[(size_t)AU_ERR * bv.A + place[g * wpb + threadIdx.x]], (uint32_t)ERR_LAUNCH);
        return;
    }
    const SmemLayout L = smem_layout(bv.MC, kRowsInSmem, kPtsInSmem, kMoreInSmem);
    unsigned char* const gscr = bv.tick_scratch + ((size_t)blockIdx.x * wpb + warp) * L.g_bytes;
    // the BVH subtree headers, read by every narrow-phase query, copied once into the block's
    // shared memory behind the arenas when they fit
    const size_t hdr_off = (size_t)wpb * L.bytes;
    const Subtree* sub = bv.mesh.sub;
    if (hdr_cache) {
        uint32_t* dst = reinterpret_cast<uint32_t*>(smem + hdr_off);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(bv.mesh.sub);
        for (int i = threadIdx.x; i < bv.mesh.nsub * 5; i += blockDim.x) dst[i] = __ldg(src + i);
        sub = reinterpret_cast<const Subtree*>(dst);
        __syncthreads();
    }
    // the next group's number, broadcast to the block through the word behind the arenas and headers
    volatile int* next_slot =
        reinterpret_cast<volatile int*>(smem + hdr_off + (hdr_cache ? (size_t)bv.mesh.nsub * sizeof(Subtree) : 0));
    for (int grp = blockIdx.x; grp < ngroups;) {
    const int slot0 = grp * wpb;
    const bool active = slot0 + warp < bv.A;  // warp-uniform; idle warps still take part in the barriers
    const int ar = active ? (int)place[slot0 + warp] : 0;
    Ctx& a = bind_ctx(smem + (size_t)warp * L.bytes, L, lane, gscr);
    if (active) {
        if (lane == 0) {
            load_arena(bv, ar, a);
            a.sub = sub;
        }
        __syncwarp();
        if (lane < a.ncars) load_car(bv, ar, a, lane);
        load_pads(bv, ar, a, lane);
    }
    // every warp's arena loaded (and its working-set pointers bound) before any thread of the block
    // touches another warp's arena (the controls below, the block-wide parts of the tick)
    __syncthreads();
    int nact = bv.A - slot0;
    nact = nact < wpb ? nact : wpb;
    const BlockArenas B{smem, L.bytes, nact};
    unsigned long long busy = 0;
    RSG_PHASE_BEGIN;
    for (int t = 0; t < ticks; t++) {
        if (controls)
            for (int u = threadIdx.x; u < nact * bv.MC; u += blockDim.x) {
                const int w = u / bv.MC, k = u % bv.MC;
                Ctx& aw = B(w);
                if (k < aw.ncars) apply_controls(aw.cars[k], controls[((size_t)t * bv.A + place[slot0 + w]) * bv.MC + k]);
            }
        __syncthreads();
        block_tick_pre(bv, B, threadIdx.x, blockDim.x);
        RSG_PHASE(0);
        if (active) step_bodies_pre(bv, a, lane);
        __syncthreads();
        RSG_PHASE(1);
        const long long c0 = clock64();
        step_collide_block(bv, a, lane, active, collide_sync != 0);
        busy += (unsigned long long)(clock64() - c0);
        __syncthreads();
        RSG_PHASE(2);
        block_tick_post(bv, B, threadIdx.x, blockDim.x);
        RSG_PHASE(3);
    }
    if (active) {
        if (lane == 0) {
            store_arena(bv, ar, a);
            cost[ar] = busy > 0xffffffffull ? 0xffffffffu : (uint32_t)busy;
        }
        if (lane < a.ncars) store_car(bv, ar, a, lane);
        store_pads(bv, ar, a, lane);
    }
    if (!group_next) break;
    __syncthreads();  // every warp is done with its working set (and has read next_slot)
    if (threadIdx.x == 0) *next_slot = (int)gridDim.x + (int)atomicAdd(group_next, 1u);
    __syncthreads();
    grp = *next_slot;
    }
}

// Placement order of the arenas: a counting sort by the cost of their collision work in the last
// launch, on a log scale with eight steps per octave, most expensive first.  Any order gives the same
// results (arenas are independent); this one makes the arenas of a block cost about the same.
__global__ void rsg_place_arenas_kernel(int A, const uint32_t* __restrict__ cost, uint32_t* __restrict__ place) {
    __shared__ uint32_t start[256];
    auto key = [](uint32_t c) {
        c |= 1u;
        const int l = 31 - __clz(c);
        const int frac = l >= 3 ? (int)((c >> (l - 3)) & 7u) : 0;
        return 255 - (l * 8 + frac);
    };
    for (int i = threadIdx.x; i < 256; i += blockDim.x) start[i] = 0;
    __syncthreads();
    for (int a = threadIdx.x; a < A; a += blockDim.x) atomicAdd(&start[key(cost[a])], 1u);
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive prefix sum of the 256 bucket sizes, 8 per lane
        uint32_t v[8], s = 0;
        for (int j = 0; j < 8; j++) { v[j] = start[threadIdx.x * 8 + j]; s += v[j]; }
        uint32_t incl = s;
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
            if ((int)threadIdx.x >= d) incl += o;
        }
        uint32_t run = incl - s;
        for (int j = 0; j < 8; j++) { start[threadIdx.x * 8 + j] = run; run += v[j]; }
    }
    __syncthreads();
    for (int a = threadIdx.x; a < A; a += blockDim.x) place[atomicAdd(&start[key(cost[a])], 1u)] = (uint32_t)a;
}

cudaError_t launch_place_arenas(const BatchBuffers& b, cudaStream_t st) {
    if (b.A <= 1) return cudaSuccess;
    rsg_place_arenas_kernel<<<1, 1024, 0, st>>>(b.A, b.cost, b.place);
    return cudaGetLastError();
}

int tick_smem_per_arena(int max_cars) { return smem_layout(max_cars, kRowsInSmem, kPtsInSmem, kMoreInSmem).bytes; }
int tick_scratch_slots(int A, int sms) {
    const long long per_grid = (long long)A + TICK_MAX_ARENAS_PER_BLOCK;  // ngroups * arenas per block < A + that
    const long long cap = 2LL * (sms > 0 ? sms : 1) * TICK_MAX_ARENAS_PER_BLOCK;
    return (int)(per_grid < cap ? per_grid : cap);
}
size_t tick_scratch_bytes(int slots, int max_cars) {
    return (size_t)slots * smem_layout(max_cars, kRowsInSmem, kPtsInSmem, kMoreInSmem).g_bytes;
}

// The EPA work-slot pool of the current device, made once per device for the process.
cudaError_t ensure_epa_pool() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return cudaSuccess;
    const int nslots = 1024;
    uint32_t* locks = nullptr;
    epa::Slot* slots = nullptr;
    if ((e = cudaMalloc((void**)&locks, sizeof(uint32_t) * nslots)) != cudaSuccess) return e;
    if ((e = cudaMemset(locks, 0, sizeof(uint32_t) * nslots)) != cudaSuccess) return e;
    if ((e = cudaMalloc((void**)&slots, sizeof(epa::Slot) * nslots)) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(epa::g_epa_lock, &locks, sizeof(locks))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(epa::g_epa_slots, &slots, sizeof(slots))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(epa::g_epa_nslots, &nslots, sizeof(nslots))) != cudaSuccess) return e;
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
    done[dev] = true;
    return cudaSuccess;
}

// Per device: the tick kernel's shared-memory limit raised once, and the blocks an SM holds for each
// (arenas per block, shared memory) a persistent launch asks about.
struct TickLaunchCache {
    std::mutex mu;
    std::map<int, bool> smem_set;
    std::map<std::tuple<int, int, int>, int> resident;
};
TickLaunchCache& tick_launch_cache() {
    static TickLaunchCache c;
    return c;
}

cudaError_t launch_tick(const BatchBuffers& b, const rsg_car_controls* controls, int ticks, const TickShape& shape,
                        cudaStream_t st) {
    if (b.A <= 0 || ticks <= 0) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    TickLaunchCache& tc = tick_launch_cache();
    int wpb = shape.arenas_per_block;
    if (wpb <= 0 || wpb > TICK_MAX_ARENAS_PER_BLOCK) wpb = TICK_MAX_ARENAS_PER_BLOCK;
    // the block must fit in shared memory
    const int per_arena = tick_smem_per_arena(b.MC);
    while (wpb > 1 && per_arena * wpb + 16 > 227 * 1024) wpb--;
    int smem = per_arena * wpb;
    // the header copy: on request, or (automatic) only when it costs no block per SM (228 KB of
    // shared memory per SM, 1 KB of it reserved per block)
    const int hdr_bytes = b.mesh.sub ? b.mesh.nsub * (int)sizeof(Subtree) : 0;
    const int sm_smem = 228 * 1024;
    const int blocks_without = sm_smem / (smem + 1024), blocks_with = sm_smem / (smem + hdr_bytes + 1024);
    const bool fits = hdr_bytes > 0 && smem + hdr_bytes + 16 <= 227 * 1024;
    const int hdr_cache = shape.header_cache < 0 ? ((fits && blocks_with >= blocks_without) ? 1 : 0)
                                                 : ((fits && shape.header_cache) ? 1 : 0);
    if (hdr_cache) smem += hdr_bytes;
    BatchView v = make_view(b);
    v.lanes_per_car = (shape.lanes_per_car == 1 || shape.lanes_per_car == 2) ? shape.lanes_per_car : 4;
    if (!shape.leaf_grid) {
        v.mesh.lg_block = nullptr;
        v.mesh.lg_over = nullptr;
    }
    smem += 16;  // the next group's number (persistent launches)
    {
        std::lock_guard<std::mutex> lock(tc.mu);
        if (!tc.smem_set[dev]) {
            e = cudaFuncSetAttribute(rsg_tick_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
            if (e != cudaSuccess) return e;
            tc.smem_set[dev] = true;
        }
    }
    const int ngroups = (b.A + wpb - 1) / wpb;
    int grid = ngroups;
    uint32_t* group_next = nullptr;
    // a grid wider than the scratch's slots runs as a persistent launch of resident blocks
    if ((shape.persistent || (long long)ngroups * wpb > b.scratch_slots) && b.group_next) {
        int resident = 0;
        {
            std::lock_guard<std::mutex> lock(tc.mu);
            auto it = tc.resident.find(std::make_tuple(dev, wpb, smem));
            if (it != tc.resident.end()) resident = it->second;
        }
        if (resident == 0) {
            int nsm = 0, per_sm = 0;
            if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rsg_tick_kernel, 32 * wpb, smem)) !=
                cudaSuccess)
                return e;
            resident = nsm * (per_sm > 0 ? per_sm : 1);
            std::lock_guard<std::mutex> lock(tc.mu);
            tc.resident[std::make_tuple(dev, wpb, smem)] = resident;
        }
        if (resident < ngroups) {
            grid = resident;
            group_next = b.group_next;
            if ((e = cudaMemsetAsync(group_next, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
        }
    }
    rsg_tick_kernel<<<grid, 32 * wpb, smem, st>>>(v, controls, ticks, hdr_cache, shape.collide_sync ? 1 : 0, b.place,
                                                   b.cost, group_next);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- state gather / scatter
// Car::GetState (src/Sim/Car/Car.cpp:10-20)
RSG_D void car_get(const SoA& s, int i, rsg_car_state& o) {
    uint32_t fl = s.cu(CU_FLAGS, i);
    auto F = [&](uint32_t m) -> uint8_t { return (fl & m) ? 1 : 0; };
    o.pos = to_rv(s.v3(CF_POS, i) * RL::BT_TO_UU);
    o.rot_mat = basis_to_rot(s.m3(CF_ROT, i));
    o.vel = to_rv(s.v3(CF_VEL, i) * RL::BT_TO_UU);
    o.ang_vel = to_rv(s.v3(CF_ANG, i));
    o.tick_count_since_update = u64(s.cu(CU_TICKS_LO, i), s.cu(CU_TICKS_HI, i));
    o.is_on_ground = F(F_ON_GROUND);
    for (int w = 0; w < 4; w++) o.wheels_with_contact[w] = F(F_WHEEL0 << w);
    o.has_jumped = F(F_HAS_JUMPED);
    o.has_double_jumped = F(F_HAS_DJ);
    o.has_flipped = F(F_HAS_FLIPPED);
    o.flip_rel_torque = to_rv(s.v3(CF_FLIP_REL, i));
    o.jump_time = s.cf(CF_JUMP_TIME, i);
    o.flip_time = s.cf(CF_FLIP_TIME, i);
    o.is_flipping = F(F_FLIPPING);
    o.is_jumping = F(F_JUMPING);
    o._pad0[0] = o._pad0[1] = 0;
    o.air_time = s.cf(CF_AIR_TIME, i);
    o.air_time_since_jump = s.cf(CF_AIR_TIME_SJ, i);
    o.boost = s.cf(CF_BOOST, i);
    o.time_since_boosted = s.cf(CF_TIME_SINCE_BOOST, i);
    o.is_boosting = F(F_BOOSTING);
    o._pad1[0] = o._pad1[1] = o._pad1[2] = 0;
    o.boosting_time = s.cf(CF_BOOSTING_TIME, i);
    o.is_supersonic = F(F_SUPERSONIC);
    o._pad2[0] = o._pad2[1] = o._pad2[2] = 0;
    o.supersonic_time = s.cf(CF_SUPERSONIC_TIME, i);
    o.handbrake_val = s.cf(CF_HANDBRAKE, i);
    o.is_auto_flipping = F(F_AUTOFLIPPING);
    o._pad3[0] = o._pad3[1] = o._pad3[2] = 0;
    o.auto_flip_timer = s.cf(CF_AUTOFLIP_TIMER, i);
    o.auto_flip_torque_scale = s.cf(CF_AUTOFLIP_SCALE, i);
    o.world_contact_has_contact = F(F_WC_CONTACT);
    o._pad4[0] = o._pad4[1] = o._pad4[2] = 0;
    o.world_contact_normal = to_rv(s.v3(CF_WC_NORMAL, i));
    o.car_contact_other_car_id = s.cu(CU_CC_OTHER, i);
    o.car_contact_cooldown_timer = s.cf(CF_CC_COOLDOWN, i);
    o.is_demoed = F(F_DEMOED);
    o._pad5[0] = o._pad5[1] = o._pad5[2] = 0;
    o.demo_respawn_timer = s.cf(CF_DEMO_TIMER, i);
    o.ball_hit_info.is_valid = F(F_BHI_VALID);
    o.ball_hit_info._pad0[0] = o.ball_hit_info._pad0[1] = o.ball_hit_info._pad0[2] = 0;
    o.ball_hit_info.relative_pos_on_ball = to_rv(s.v3(CF_BHI_REL, i));
    o.ball_hit_info.ball_pos = to_rv(s.v3(CF_BHI_BALLPOS, i));
    o.ball_hit_info.extra_hit_vel = to_rv(s.v3(CF_BHI_EXTRA, i));
    o.ball_hit_info.tick_count_when_hit = u64(s.cu(CU_BHI_HIT_LO, i), s.cu(CU_BHI_HIT_HI, i));
    o.ball_hit_info.tick_count_when_extra_impulse_applied = u64(s.cu(CU_BHI_EXTRA_LO, i), s.cu(CU_BHI_EXTRA_HI, i));
    o.last_controls.throttle = s.cf(CF_LAST_CTRL + 0, i);
    o.last_controls.steer = s.cf(CF_LAST_CTRL + 1, i);
    o.last_controls.pitch = s.cf(CF_LAST_CTRL + 2, i);
    o.last_controls.yaw = s.cf(CF_LAST_CTRL + 3, i);
    o.last_controls.roll = s.cf(CF_LAST_CTRL + 4, i);
    o.last_controls.jump = F(F_LAST_JUMP);
    o.last_controls.boost = F(F_LAST_BOOST);
    o.last_controls.handbrake = F(F_LAST_HB);
    o.last_controls._pad0 = 0;
}

// Car::SetState (src/Sim/Car/Car.cpp:23-36)
RSG_D void car_set(const SoA& s, int i, const rsg_car_state& st) {
    uint32_t fl = s.cu(CU_FLAGS, i) & (F_PRESENT | F_TEAM_ORANGE | F_CTRL_JUMP | F_CTRL_BOOST | F_CTRL_HB | F_NO_RESPONSE);
    auto S = [&](uint32_t m, uint8_t v) { if (v) fl |= m; };
    M3 basis = rot_to_basis(st.rot_mat);
    s.set_v3(CF_POS, i, from_rv(st.pos) * RL::UU_TO_BT);
    s.set_m3(CF_BASIS, i, basis);
    s.set_m3(CF_ROT, i, basis);
    s.set_v3(CF_VEL, i, from_rv(st.vel) * RL::UU_TO_BT);
    s.set_v3(CF_ANG, i, from_rv(st.ang_vel));
    s.set_v3(CF_VEL_CACHE, i, V3(0, 0, 0));
    s.cu(CU_TICKS_LO, i) = 0;
    s.cu(CU_TICKS_HI, i) = 0;
    S(F_ON_GROUND, st.is_on_ground);
    for (int w = 0; w < 4; w++) S(F_WHEEL0 << w, st.wheels_with_contact[w]);
    S(F_HAS_JUMPED, st.has_jumped);
    S(F_HAS_DJ, st.has_double_jumped);
    S(F_HAS_FLIPPED, st.has_flipped);
    s.set_v3(CF_FLIP_REL, i, from_rv(st.flip_rel_torque));
    s.cf(CF_JUMP_TIME, i) = st.jump_time;
    s.cf(CF_FLIP_TIME, i) = st.flip_time;
    S(F_FLIPPING, st.is_flipping);
    S(F_JUMPING, st.is_jumping);
    s.cf(CF_AIR_TIME, i) = st.air_time;
    s.cf(CF_AIR_TIME_SJ, i) = st.air_time_since_jump;
    s.cf(CF_BOOST, i) = st.boost;
    s.cf(CF_TIME_SINCE_BOOST, i) = st.time_since_boosted;
    S(F_BOOSTING, st.is_boosting);
    s.cf(CF_BOOSTING_TIME, i) = st.boosting_time;
    S(F_SUPERSONIC, st.is_supersonic);
    s.cf(CF_SUPERSONIC_TIME, i) = st.supersonic_time;
    s.cf(CF_HANDBRAKE, i) = st.handbrake_val;
    S(F_AUTOFLIPPING, st.is_auto_flipping);
    s.cf(CF_AUTOFLIP_TIMER, i) = st.auto_flip_timer;
    s.cf(CF_AUTOFLIP_SCALE, i) = st.auto_flip_torque_scale;
    S(F_WC_CONTACT, st.world_contact_has_contact);
    s.set_v3(CF_WC_NORMAL, i, from_rv(st.world_contact_normal));
    s.cu(CU_CC_OTHER, i) = st.car_contact_other_car_id;
    s.cf(CF_CC_COOLDOWN, i) = st.car_contact_cooldown_timer;
    S(F_DEMOED, st.is_demoed);
    s.cf(CF_DEMO_TIMER, i) = st.demo_respawn_timer;
    S(F_BHI_VALID, st.ball_hit_info.is_valid);
    s.set_v3(CF_BHI_REL, i, from_rv(st.ball_hit_info.relative_pos_on_ball));
    s.set_v3(CF_BHI_BALLPOS, i, from_rv(st.ball_hit_info.ball_pos));
    s.set_v3(CF_BHI_EXTRA, i, from_rv(st.ball_hit_info.extra_hit_vel));
    uint64_t th = st.ball_hit_info.tick_count_when_hit, te = st.ball_hit_info.tick_count_when_extra_impulse_applied;
    s.cu(CU_BHI_HIT_LO, i) = (uint32_t)th;
    s.cu(CU_BHI_HIT_HI, i) = (uint32_t)(th >> 32);
    s.cu(CU_BHI_EXTRA_LO, i) = (uint32_t)te;
    s.cu(CU_BHI_EXTRA_HI, i) = (uint32_t)(te >> 32);
    s.cf(CF_LAST_CTRL + 0, i) = st.last_controls.throttle;
    s.cf(CF_LAST_CTRL + 1, i) = st.last_controls.steer;
    s.cf(CF_LAST_CTRL + 2, i) = st.last_controls.pitch;
    s.cf(CF_LAST_CTRL + 3, i) = st.last_controls.yaw;
    s.cf(CF_LAST_CTRL + 4, i) = st.last_controls.roll;
    S(F_LAST_JUMP, st.last_controls.jump);
    S(F_LAST_BOOST, st.last_controls.boost);
    S(F_LAST_HB, st.last_controls.handbrake);
    s.cu(CU_FLAGS, i) = fl;
}

__global__ void rsg_get_cars_kernel(BatchView bv, const uint32_t* __restrict__ idx, int n, rsg_car_state* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int ar, slot;
    if (idx) { ar = (int)idx[2 * k]; slot = (int)idx[2 * k + 1]; }
    else { ar = k / bv.MC; slot = k % bv.MC; }
    if (ar < 0 || ar >= bv.A || slot < 0 || slot >= bv.MC) return;
    SoA s{bv, ar};
    if (slot >= (int)s.au(AU_NCARS)) return;
    rsg_car_state o;
    car_get(s, slot, o);
    out[k] = o;
}
__global__ void rsg_set_cars_kernel(BatchView bv, const uint32_t* __restrict__ idx, int n, const rsg_car_state* __restrict__ in) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int ar, slot;
    if (idx) { ar = (int)idx[2 * k]; slot = (int)idx[2 * k + 1]; }
    else { ar = k / bv.MC; slot = k % bv.MC; }
    if (ar < 0 || ar >= bv.A || slot < 0 || slot >= bv.MC) return;
    SoA s{bv, ar};
    if (slot >= (int)s.au(AU_NCARS)) return;
    rsg_car_state st = in[k];
    car_set(s, slot, st);
}

// Ball::GetState / SetState (src/Sim/Ball/Ball.cpp:27-51)
__global__ void rsg_get_balls_kernel(BatchView bv, const uint32_t* __restrict__ arenas, int n, rsg_ball_state* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int ar = arenas ? (int)arenas[k] : k;
    if (ar < 0 || ar >= bv.A) return;
    out[k] = ball_get(SoA{bv, ar});
}
__global__ void rsg_set_balls_kernel(BatchView bv, const uint32_t* __restrict__ arenas, int n, const rsg_ball_state* __restrict__ in) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int ar = arenas ? (int)arenas[k] : k;
    if (ar < 0 || ar >= bv.A) return;
    ball_set(SoA{bv, ar}, in[k]);
}

// BoostPad::GetState / SetState (src/Sim/BoostPad/BoostPad.h:44-45)
__global__ void rsg_get_pads_kernel(BatchView bv, const uint32_t* __restrict__ arenas, int n, rsg_pad_state* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n * bv.npads) return;
    int q = k / bv.npads, p = k % bv.npads;
    int ar = arenas ? (int)arenas[q] : q;
    if (ar < 0 || ar >= bv.A) return;
    SoA s{bv, ar};
    rsg_pad_state o;
    o.is_active = s.pu(PU_ACTIVE, p) ? 1 : 0;
    o._pad0[0] = o._pad0[1] = o._pad0[2] = 0;
    o.cooldown = s.pf(PF_COOLDOWN, p);
    uint32_t cur = s.pu(PU_CUR_LOCKED, p);
    o.cur_locked_car_id = (cur > 0 && (int)cur <= bv.MC) ? s.cu(CU_ID, (int)cur - 1) : 0u;
    o.prev_locked_car_id = s.pu(PU_PREV_LOCKED, p);
    out[k] = o;
}
__global__ void rsg_set_pads_kernel(BatchView bv, const uint32_t* __restrict__ arenas, int n, const rsg_pad_state* __restrict__ in) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n * bv.npads) return;
    int q = k / bv.npads, p = k % bv.npads;
    int ar = arenas ? (int)arenas[q] : q;
    if (ar < 0 || ar >= bv.A) return;
    SoA s{bv, ar};
    rsg_pad_state st = in[k];
    s.pu(PU_ACTIVE, p) = st.is_active ? 1u : 0u;
    s.pf(PF_COOLDOWN, p) = st.cooldown;
    s.pu(PU_CUR_LOCKED, p) = 0;
    s.pu(PU_PREV_LOCKED, p) = st.prev_locked_car_id;
}

__global__ void rsg_set_controls_kernel(BatchView bv, const rsg_car_controls* __restrict__ in) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= bv.A * bv.MC) return;
    int ar = k / bv.MC, slot = k % bv.MC;
    SoA s{bv, ar};
    rsg_car_controls c = in[k];
    s.cf(CF_CTRL + 0, slot) = c.throttle;
    s.cf(CF_CTRL + 1, slot) = c.steer;
    s.cf(CF_CTRL + 2, slot) = c.pitch;
    s.cf(CF_CTRL + 3, slot) = c.yaw;
    s.cf(CF_CTRL + 4, slot) = c.roll;
    uint32_t fl = s.cu(CU_FLAGS, slot) & ~(F_CTRL_JUMP | F_CTRL_BOOST | F_CTRL_HB);
    if (c.jump) fl |= F_CTRL_JUMP;
    if (c.boost) fl |= F_CTRL_BOOST;
    if (c.handbrake) fl |= F_CTRL_HB;
    s.cu(CU_FLAGS, slot) = fl;
}

__global__ void rsg_is_scored_kernel(BatchView bv, int* __restrict__ out) {
    int ar = blockIdx.x * blockDim.x + threadIdx.x;
    if (ar >= bv.A) return;
    SoA s{bv, ar};
    float y = s.bf(BF_POS + 1) * RL::BT_TO_UU;
    out[ar] = fabsf(y) > (bv.mut.goal_threshold_y + bv.mut.ball_radius_uu) ? 1 : 0;
}

// Arena::IsBallProbablyGoingIn (src/Sim/Arena/Arena.cpp:770-806), the soccar branch: the ball's
// time to the goal line along y, the point it would cross at under gravity, and the approximate
// goal mouth (half width 892.755, height 642.775) widened by a tenth of the ball radius plus the
// caller's margin.  gravity in uu/s^2 as the mutator config holds it.
RSG_D bool going_in(const SoA& s, const BatchView& bv, float max_time, float extra_margin, float gx, float gz,
                    int& team) {
    const float px = s.bf(BF_POS) * RL::BT_TO_UU, py = s.bf(BF_POS + 1) * RL::BT_TO_UU, pz = s.bf(BF_POS + 2) * RL::BT_TO_UU;
    const float vx = s.bf(BF_VEL) * RL::BT_TO_UU, vy = s.bf(BF_VEL + 1) * RL::BT_TO_UU, vz = s.bf(BF_VEL + 2) * RL::BT_TO_UU;
    team = -1;
    if (fabsf(vy) < 1.1920928955078125e-7f) return false;  // FLT_EPSILON
    const float sgn = (float)((vy > 0) - (vy < 0));
    const float goal_y = bv.mut.goal_threshold_y * sgn;
    const float t = fabsf(py - goal_y) / fabsf(vy);
    if (t > max_time) return false;
    const float ex = (px + vx * t) + ((gx * t) * t) / 2.f;
    const float ez = (pz + vz * t) + ((gz * t) * t) / 2.f;
    const float margin = bv.mut.ball_radius_uu * 0.1f + extra_margin;
    if (ez > 642.775f + margin || fabsf(ex) > 892.755f + margin) return false;
    team = sgn < 0 ? RSG_TEAM_BLUE : RSG_TEAM_ORANGE;
    return true;
}

__global__ void rsg_going_in_kernel(BatchView bv, float max_time, float extra_margin, float gx, float gz,
                                    int* __restrict__ out, int* __restrict__ team) {
    int ar = blockIdx.x * blockDim.x + threadIdx.x;
    if (ar >= bv.A) return;
    int tm = -1;
    out[ar] = going_in(SoA{bv, ar}, bv, max_time, extra_margin, gx, gz, tm) ? 1 : 0;
    if (team) team[ar] = tm;
}

// GetShooterPasser (src/Sim/GameEventTracker/GameEventTracker.cpp:5-46): the car of `team` (cars in
// update order) that touched the ball last within max_shooter ticks, and the teammate that touched it
// last within max_passer ticks before that; ids, 0 for none.
RSG_D bool shooter_passer(const SoA& s, uint64_t tick, int team, bool find_passer, uint64_t max_shooter,
                          uint64_t max_passer, uint32_t& shooter, uint32_t& passer) {
    const int n = (int)s.au(AU_NCARS);
    const uint32_t ord = s.au(AU_ORDER);
    int sh = -1, pa = -1;
    uint64_t sh_tick = 0, pa_tick = 0;
    for (int k = 0; k < n; k++) {
        const int slot = (int)((ord >> (4 * k)) & 0xf);
        const uint32_t fl = s.cu(CU_FLAGS, slot);
        if (((fl & F_TEAM_ORANGE) ? 1 : 0) != team || !(fl & F_BHI_VALID)) continue;
        const uint64_t hit = u64(s.cu(CU_BHI_HIT_LO, slot), s.cu(CU_BHI_HIT_HI, slot));
        if (hit + max_shooter >= tick && (sh < 0 || hit > sh_tick)) { sh = slot; sh_tick = hit; }
    }
    if (sh >= 0 && find_passer) {
        for (int k = 0; k < n; k++) {
            const int slot = (int)((ord >> (4 * k)) & 0xf);
            const uint32_t fl = s.cu(CU_FLAGS, slot);
            if (((fl & F_TEAM_ORANGE) ? 1 : 0) != team || !(fl & F_BHI_VALID) || slot == sh) continue;
            const uint64_t hit = u64(s.cu(CU_BHI_HIT_LO, slot), s.cu(CU_BHI_HIT_HI, slot));
            if (hit + max_passer >= sh_tick && (pa < 0 || hit > pa_tick)) { pa = slot; pa_tick = hit; }
        }
    }
    shooter = sh >= 0 ? s.cu(CU_ID, sh) : 0;
    passer = pa >= 0 ? s.cu(CU_ID, pa) : 0;
    return sh >= 0;
}

// GameEventTracker::Update (GameEventTracker.cpp:48-158) of every arena, one thread each; the
// tracker's persistent fields live in `st`, the event of this update (if any) goes to ev[ar].
__global__ void rsg_game_events_kernel(BatchView bv, GameEventDev st, GameEventCfgDev c, float gx, float gz,
                                       rsg_game_event* __restrict__ ev) {
    const int ar = blockIdx.x * blockDim.x + threadIdx.x;
    if (ar >= bv.A) return;
    SoA s{bv, ar};
    rsg_game_event e{0, 0, 0};
    const float py = s.bf(BF_POS + 1) * RL::BT_TO_UU;
    const bool scored = fabsf(py) > (bv.mut.goal_threshold_y + bv.mut.ball_radius_uu);
    const float tick_time = bv.dt, tickrate = 1.f / bv.dt;
    const uint64_t tick = u64(s.au(AU_TICK_LO), s.au(AU_TICK_HI));
    const uint64_t upd = u64(s.bu(BU_TICKS_LO), s.bu(BU_TICKS_HI));
    const uint64_t last = st.last_update[ar];
    if (upd > last || !c.auto_state_set_detection) {
        const uint64_t dticks = upd - last;
        const float dt = (float)dticks * tick_time;
        if (scored && !st.scored_last[ar]) {
            uint32_t a = 0, b = 0;
            const int team = -py < 0 ? RSG_TEAM_BLUE : RSG_TEAM_ORANGE;
            if (shooter_passer(s, tick, team, true, (uint64_t)(c.goal_max_touch_time * tickrate),
                               (uint64_t)(c.pass_max_touch_time * tickrate), a, b))
                e = rsg_game_event{RSG_GAME_EVENT_GOAL, a, b};
        } else if (!st.ball_shot[ar]) {
            if (st.shot_cooldown[ar] > 0) {
                const float v = st.shot_cooldown[ar] - dt;
                st.shot_cooldown[ar] = v > 0 ? v : 0.f;
            } else {
                const float vx = s.bf(BF_VEL) * RL::BT_TO_UU, vy = s.bf(BF_VEL + 1) * RL::BT_TO_UU,
                            vz = s.bf(BF_VEL + 2) * RL::BT_TO_UU;
                const float speed_sq = (vx * vx + vy * vy) + vz * vz;
                int goal_team = -1;
                if (speed_sq >= c.shot_min_speed * c.shot_min_speed &&
                    going_in(s, bv, c.shot_min_score_time, c.pred_score_extra_margin, gx, gz, goal_team)) {
                    const int shooter_team = 1 - goal_team;
                    const uint64_t min_delay = (uint64_t)(c.shot_touch_min_delay * tickrate);
                    uint32_t a = 0, b = 0;
                    if (shooter_passer(s, tick, shooter_team, true, dticks + min_delay,
                                       (uint64_t)(c.pass_max_touch_time * tickrate), a, b)) {
                        int slot = -1;
                        for (int k = 0; k < (int)s.au(AU_NCARS); k++)
                            if (s.cu(CU_ID, k) == a) slot = k;
                        const uint64_t since =
                            slot < 0 ? 0 : tick - u64(s.cu(CU_BHI_HIT_LO, slot), s.cu(CU_BHI_HIT_HI, slot));
                        if (slot >= 0 && since >= min_delay) {
                            st.ball_shot[ar] = 1;
                            st.shot_goal_team[ar] = goal_team;
                            st.shot_cooldown[ar] = c.shot_event_cooldown;
                            e = rsg_game_event{RSG_GAME_EVENT_SHOT, a, b};
                        }
                    }
                }
            }
        } else {
            int t_unused = -1;
            if (!going_in(s, bv, c.shot_min_score_time, c.pred_score_extra_margin, gx, gz, t_unused)) {
                uint32_t a = 0, b = 0;
                if (shooter_passer(s, tick, st.shot_goal_team[ar], false, dticks, 0, a, b))
                    e = rsg_game_event{RSG_GAME_EVENT_SAVE, a, 0};
                st.ball_shot[ar] = 0;
            }
        }
    } else if (upd == last) {
        ev[ar] = e;
        return;
    } else {  // ResetPersistentInfo
        st.scored_last[ar] = 0;
        st.ball_shot[ar] = 0;
        st.shot_cooldown[ar] = 0;
    }
    st.scored_last[ar] = scored ? 1 : 0;
    st.last_update[ar] = upd;
    ev[ar] = e;
}

static int blocks_for(int n, int bs) { return (n + bs - 1) / bs; }

cudaError_t launch_game_events(const BatchBuffers& b, const GameEventDev& st, const GameEventCfgDev& c, float gx,
                               float gz, rsg_game_event* ev, cudaStream_t s) {
    if (b.A <= 0) return cudaSuccess;
    rsg_game_events_kernel<<<blocks_for(b.A, 128), 128, 0, s>>>(make_view(b), st, c, gx, gz, ev);
    return cudaGetLastError();
}

cudaError_t launch_going_in(const BatchBuffers& b, float max_time, float extra_margin, float gx, float gz, int* out,
                            int* team, cudaStream_t st) {
    if (b.A <= 0) return cudaSuccess;
    rsg_going_in_kernel<<<blocks_for(b.A, 128), 128, 0, st>>>(make_view(b), max_time, extra_margin, gx, gz, out, team);
    return cudaGetLastError();
}

cudaError_t launch_get_cars(const BatchBuffers& b, const uint32_t* idx, int n, rsg_car_state* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    rsg_get_cars_kernel<<<blocks_for(n, 128), 128, 0, st>>>(make_view(b), idx, n, out);
    return cudaGetLastError();
}
cudaError_t launch_set_cars(const BatchBuffers& b, const uint32_t* idx, int n, const rsg_car_state* in, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    rsg_set_cars_kernel<<<blocks_for(n, 128), 128, 0, st>>>(make_view(b), idx, n, in);
    return cudaGetLastError();
}
cudaError_t launch_get_balls(const BatchBuffers& b, const uint32_t* arenas, int n, rsg_ball_state* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    rsg_get_balls_kernel<<<blocks_for(n, 128), 128, 0, st>>>(make_view(b), arenas, n, out);
    return cudaGetLastError();
}
cudaError_t launch_set_balls(const BatchBuffers& b, const uint32_t* arenas, int n, const rsg_ball_state* in, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    rsg_set_balls_kernel<<<blocks_for(n, 128), 128, 0, st>>>(make_view(b), arenas, n, in);
    return cudaGetLastError();
}
cudaError_t launch_get_pads(const BatchBuffers& b, const uint32_t* arenas, int n, rsg_pad_state* out, cudaStream_t st) {
    if (n <= 0 || b.npads <= 0) return cudaSuccess;
    rsg_get_pads_kernel<<<blocks_for(n * b.npads, 128), 128, 0, st>>>(make_view(b), arenas, n, out);
    return cudaGetLastError();
}
cudaError_t launch_set_pads(const BatchBuffers& b, const uint32_t* arenas, int n, const rsg_pad_state* in, cudaStream_t st) {
    if (n <= 0 || b.npads <= 0) return cudaSuccess;
    rsg_set_pads_kernel<<<blocks_for(n * b.npads, 128), 128, 0, st>>>(make_view(b), arenas, n, in);
    return cudaGetLastError();
}
cudaError_t launch_set_controls(const BatchBuffers& b, const rsg_car_controls* in, cudaStream_t st) {
    int n = b.A * b.MC;
    if (n <= 0) return cudaSuccess;
    rsg_set_controls_kernel<<<blocks_for(n, 128), 128, 0, st>>>(make_view(b), in);
    return cudaGetLastError();
}
cudaError_t launch_is_scored(const BatchBuffers& b, int* out, cudaStream_t st) {
    if (b.A <= 0) return cudaSuccess;
    rsg_is_scored_kernel<<<blocks_for(b.A, 128), 128, 0, st>>>(make_view(b), out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- batch bookkeeping kernels
// Arena::Arena's initial ball, pads and counters (src/Sim/Arena/Arena.cpp:416-540)
__global__ void rsg_init_arenas_kernel(BatchView bv, uint32_t ball_cell, uint32_t* place, uint32_t* cost) {
    int ar = blockIdx.x * blockDim.x + threadIdx.x;
    if (ar >= bv.A) return;
    place[ar] = (uint32_t)ar;
    cost[ar] = 0;
    SoA s{bv, ar};
    V3 p = V3(0, 0, RL::BALL_REST_Z) * RL::UU_TO_BT;
    for (int f = 0; f < BF_COUNT; f++) s.bf(f) = 0.f;
    s.bf(BF_HS_SPEED) = RL::HS::INITIAL_TARGET_SPEED;
    s.bf(BF_POS) = p.x; s.bf(BF_POS + 1) = p.y; s.bf(BF_POS + 2) = p.z;
    s.bf(BF_BASIS + 0) = 1.f; s.bf(BF_BASIS + 4) = 1.f; s.bf(BF_BASIS + 8) = 1.f;
    s.bu(BU_CELL) = ball_cell;
    s.bu(BU_CELL_SEQ) = 2;  // the ball proxy is the first dynamic proxy created
    s.bu(BU_TICKS_LO) = 0;
    s.bu(BU_TICKS_HI) = 0;
    for (int k = 0; k < NUM_PADS; k++) {
        s.pu(PU_ACTIVE, k) = 1;
        s.pf(PF_COOLDOWN, k) = 0.f;
        s.pu(PU_PREV_LOCKED, k) = 0;
        s.pu(PU_CUR_LOCKED, k) = 0;
    }
    for (int f = 0; f < AU_COUNT; f++) s.au(f) = 0;
    s.au(AU_SEQ) = 3;
}

// Arena::AddCar bookkeeping (src/Sim/Arena/Arena.cpp:50-62): clears the slot and registers the
// broadphase proxy; the respawn state is written afterwards by the state scatter kernel.
__global__ void rsg_add_car_kernel(BatchView bv, uint32_t ar, uint32_t slot, uint32_t id, uint32_t cfg, uint32_t flags,
                                   uint32_t cell, uint32_t ncars, uint32_t order) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (ar >= (uint32_t)bv.A || slot >= (uint32_t)bv.MC) return;
    SoA s{bv, (int)ar};
    for (int f = 0; f < CF_COUNT; f++) s.cf(f, slot) = 0.f;
    for (int f = 0; f < CU_COUNT; f++) s.cu(f, slot) = 0u;
    s.cu(CU_FLAGS, slot) = flags;
    s.cu(CU_ID, slot) = id;
    s.cu(CU_CFG, slot) = cfg;
    s.cu(CU_CELL, slot) = cell;
    uint32_t seq = s.au(AU_SEQ);
    s.cu(CU_CELL_SEQ, slot) = seq;
    s.au(AU_SEQ) = seq + 1;
    s.au(AU_NCARS) = ncars;
    s.au(AU_ORDER) = order;
}

// Arena::RemoveCar (src/Sim/Arena/Arena.cpp:80-94): the slots behind the removed one move down,
// keeping the relative order of the remaining cars' collision objects.
__global__ void rsg_remove_car_kernel(BatchView bv, uint32_t ar, uint32_t slot, uint32_t ncars, uint32_t order) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (ar >= (uint32_t)bv.A || slot >= (uint32_t)bv.MC || ncars >= (uint32_t)bv.MC) return;
    SoA s{bv, (int)ar};
    for (uint32_t t = slot; t < ncars; t++) {
        for (int f = 0; f < CF_COUNT; f++) s.cf(f, t) = s.cf(f, t + 1);
        for (int f = 0; f < CU_COUNT; f++) s.cu(f, t) = s.cu(f, t + 1);
    }
    for (int f = 0; f < CF_COUNT; f++) s.cf(f, ncars) = 0.f;
    for (int f = 0; f < CU_COUNT; f++) s.cu(f, ncars) = 0u;
    for (int k = 0; k < NUM_PADS; k++) {
        uint32_t cur = s.pu(PU_CUR_LOCKED, k);
        if (cur == slot + 1) s.pu(PU_CUR_LOCKED, k) = 0;
        else if (cur > slot + 1) s.pu(PU_CUR_LOCKED, k) = cur - 1;
    }
    s.au(AU_NCARS) = ncars;
    s.au(AU_ORDER) = order;
}

// Car::Demolish (src/Sim/Car/Car.cpp:38-41)
__global__ void rsg_demolish_kernel(BatchView bv, uint32_t ar, uint32_t slot, float delay) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (ar >= (uint32_t)bv.A || slot >= (uint32_t)bv.MC) return;
    SoA s{bv, (int)ar};
    s.cu(CU_FLAGS, slot) |= F_DEMOED;
    s.cf(CF_DEMO_TIMER, slot) = delay;
}

cudaError_t launch_init_arenas(const BatchBuffers& b, uint32_t ball_cell, cudaStream_t st) {
    rsg_init_arenas_kernel<<<blocks_for(b.A, 128), 128, 0, st>>>(make_view(b), ball_cell, b.place, b.cost);
    return cudaGetLastError();
}
cudaError_t launch_add_car(const BatchBuffers& b, uint32_t arena, uint32_t slot, uint32_t id, uint32_t cfg, uint32_t flags,
                           uint32_t cell, uint32_t ncars, uint32_t order, cudaStream_t st) {
    rsg_add_car_kernel<<<1, 1, 0, st>>>(make_view(b), arena, slot, id, cfg, flags, cell, ncars, order);
    return cudaGetLastError();
}
cudaError_t launch_remove_car(const BatchBuffers& b, uint32_t arena, uint32_t slot, uint32_t ncars, uint32_t order,
                              cudaStream_t st) {
    rsg_remove_car_kernel<<<1, 1, 0, st>>>(make_view(b), arena, slot, ncars, order);
    return cudaGetLastError();
}
cudaError_t launch_demolish(const BatchBuffers& b, uint32_t arena, uint32_t slot, float delay, cudaStream_t st) {
    rsg_demolish_kernel<<<1, 1, 0, st>>>(make_view(b), arena, slot, delay);
    return cudaGetLastError();
}

}  // namespace rsg

#if defined(RSG_PHASE_TIMERS)
extern "C" int rsg_phase_read(unsigned long long* out) {
    return (int)cudaMemcpyFromSymbol(out, rsg::g_phase_cycles, sizeof(unsigned long long) * 64);
}
extern "C" int rsg_phase_reset() {
    unsigned long long z[64] = {0};
    return (int)cudaMemcpyToSymbol(rsg::g_phase_cycles, z, sizeof(z));
}
#endif
