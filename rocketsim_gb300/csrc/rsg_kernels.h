// rsg_kernels.h -- host-side launchers of the device tick and of the state
// gather / scatter kernels (implemented in rsg_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/rocketsim_gb300.h"
#include "rsg_layout.h"
#include "rsg_mesh.h"

namespace rsg {

struct DevMeshPtrs {
    const float* tv;
    const QNode* nodes;
    const Subtree* sub;
    const TriInfo* info;
    const uint8_t* cells;
    const QNode* lg_block;
    const QNode* lg_over;
    const QNode* sub_grp;
    int nsub_grp;
    int lg_shift[3], lg_n[3];
    int ntri, nnodes, nsub;
    V3 bvh_min, bvh_max, quant, aabb_min, aabb_max;
};

// Device buffers of one batch (all SoA arrays as described in rsg_layout.h)
struct BatchBuffers {
    int A, MC, has_arena;
    float dt;
    MutatorsDev mut;
    const float4* pad_cfg;  // [npads] position (uu), is_big
    int npads, custom_pads, no_ball_rot;
    int heatseeker;  // GameMode::HEATSEEKER: the ball seeks a goal (Ball::_PreTickUpdate)
    uint32_t* rec;  // A records of rec_words(MC) 32-bit words
    uint32_t* au;   // [AU_COUNT][A]
    const CarCfgDev* cfgs;
    void* events;  // DevEvent[A * MAX_EVENTS_PER_ARENA]
    uint32_t event_mask;
    DevMeshPtrs mesh;
    GridSpec grid;
    uint32_t* place;  // [A] arena advanced by each warp slot of the tick kernel (a permutation of 0..A-1)
    uint32_t* cost;   // [A] cycles each arena's own collision work took in the last tick launch
    uint32_t* group_next;  // [1] groups taken so far by the blocks of a persistent tick launch
    unsigned char* tick_scratch;  // tick_scratch_bytes: per warp slot, the working set kept out of shared memory
    int scratch_slots;            // warp slots in tick_scratch: a launch's grid * arenas per block stays within
};

constexpr int DEV_EVENT_BYTES = 24;

// Launch shape of the tick kernel.  Every shape gives the same results (arenas never depend on the
// block they share or on how their units are spread); they differ in speed.
#ifndef RSG_TICK_MAX_WARPS
#define RSG_TICK_MAX_WARPS 16
#endif
// Most arenas (warps) per block of the tick kernel; its register budget per thread follows from it
// (16 warps: 128 registers, so that 16 warps of one or more blocks fit an SM's register file).
constexpr int TICK_MAX_ARENAS_PER_BLOCK = RSG_TICK_MAX_WARPS;

struct TickShape {
    int arenas_per_block = TICK_MAX_ARENAS_PER_BLOCK;  // one warp per arena (as many as shared memory holds)
    int lanes_per_car = 4;     // threads per car in the vehicle update after the rays: 1, 2 or 4
    int header_cache = -1;     // BVH subtree headers in shared memory: 1 yes, 0 no, -1 when it costs no block per SM
    int leaf_grid = 1;         // wheel rays scan the leaf grid (1) or walk the quantized BVH (0)
    int collide_sync = 1;      // block-wide barriers between the parts of the collision work (1) or not (0)
    int persistent = 0;        // one block per resident slot taking arena groups from a counter (1), or a block per group (0)
};

// Advances every arena by `ticks` ticks, one warp per arena, arenas placed in blocks by b.place.
// `controls` (device, may be null) holds [ticks][A][MC] rsg_car_controls applied before each tick.
cudaError_t launch_tick(const BatchBuffers& b, const rsg_car_controls* controls, int ticks, const TickShape& shape,
                        cudaStream_t st);
// Re-places the arenas for the next launch: b.place lists them by the cost of their collision work
// in the last launch, most expensive first, so that the arenas sharing a block (and waiting for each
// other at its barriers) cost about the same and the cheap blocks fill the last wave.
cudaError_t launch_place_arenas(const BatchBuffers& b, cudaStream_t st);
// Shared memory one arena needs in the tick kernel.
int tick_smem_per_arena(int max_cars);
// Warp slots of the tick kernel's global scratch for a batch of A arenas on a GPU of `sms` SMs: a slot
// per warp of a grid of a block per arena group, at most 2 slots per warp an SM holds (larger batches
// run persistent launches of resident blocks), and the scratch's bytes.
int tick_scratch_slots(int A, int sms);
size_t tick_scratch_bytes(int slots, int max_cars);

// Allocates the current device's pool of EPA work slots (once per device; about 14 MB).
cudaError_t ensure_epa_pool();

// The constants Car::_BulletSetup derives from a car configuration (src/Sim/Car/Car.cpp:195-292).
CarCfgDev car_config_derived(const rsg_car_config& c);

// Records `msg` as the calling thread's last error (rsg_get_last_error) and returns `code`.
int report_error(int code, const char* msg);

// Gathers states of `n` (arena, slot) pairs (idx[2k], idx[2k+1]); idx == null means
// all arenas x all slots in [arena][slot] order.  Slots beyond the arena's car count
// are not written.  Cars/balls/pads outputs are device arrays; any may be null.
cudaError_t launch_get_cars(const BatchBuffers& b, const uint32_t* idx, int n, rsg_car_state* out, cudaStream_t st);
cudaError_t launch_set_cars(const BatchBuffers& b, const uint32_t* idx, int n, const rsg_car_state* in, cudaStream_t st);
cudaError_t launch_get_balls(const BatchBuffers& b, const uint32_t* arenas, int n, rsg_ball_state* out, cudaStream_t st);
cudaError_t launch_set_balls(const BatchBuffers& b, const uint32_t* arenas, int n, const rsg_ball_state* in, cudaStream_t st);
cudaError_t launch_get_pads(const BatchBuffers& b, const uint32_t* arenas, int n, rsg_pad_state* out, cudaStream_t st);
cudaError_t launch_set_pads(const BatchBuffers& b, const uint32_t* arenas, int n, const rsg_pad_state* in, cudaStream_t st);
// Writes controls [A][MC] into the per-car control fields.
cudaError_t launch_set_controls(const BatchBuffers& b, const rsg_car_controls* in, cudaStream_t st);
// Arena::IsBallProbablyGoingIn (soccar) of every arena into out[A] (0/1) and team[A] (may be null;
// the scoring goal's team, -1 where no goal is coming); gravity components in uu/s^2.
cudaError_t launch_going_in(const BatchBuffers& b, float max_time, float extra_margin, float gx, float gz, int* out,
                            int* team, cudaStream_t st);
// GameEventTracker's persistent fields for every arena (device arrays [A]) and its config.
struct GameEventDev {
    float* shot_cooldown;
    int* ball_shot;
    int* shot_goal_team;
    int* scored_last;
    uint64_t* last_update;
};
struct GameEventCfgDev {
    float shot_min_speed, shot_touch_min_delay, pred_score_extra_margin, shot_event_cooldown, shot_min_score_time,
        goal_max_touch_time, pass_max_touch_time;
    int auto_state_set_detection;
};
// GameEventTracker::Update of every arena; ev[A] (device) receives each arena's event.
cudaError_t launch_game_events(const BatchBuffers& b, const GameEventDev& st, const GameEventCfgDev& c, float gx,
                               float gz, rsg_game_event* ev, cudaStream_t s);
// Ball-scored test of every arena into out[A] (0/1).
cudaError_t launch_is_scored(const BatchBuffers& b, int* out, cudaStream_t st);

// Device side of a ball prediction tracker (rsg_ballpred.cu): per arena a ring of T ball states
// ([A][T], head = predData[0]), lastUpdateTickCount and whether predData is filled; the run list
// of one update (arena, step count, first ring slot) and its length.
struct BallPredDev {
    int T;
    rsg_ball_state* pred;
    uint32_t* head;
    int32_t* last_update;
    uint8_t* valid;
    int* list;
    int* count;
    int* steps;
    uint32_t* base;
};

// One BallPredTracker update of every arena (mask[a] != 0, or all with mask null) of the tracker
// batch `pred`: mode 0 UpdatePredFromArena from `src`, 1 UpdatePredManual (cur, ticks: device
// arrays [A]), 2 ForceUpdateAllPred (cur).
cudaError_t launch_ball_pred(const BatchBuffers& pred, const BallPredDev& d, const BatchBuffers* src, int mode,
                             const rsg_ball_state* cur, const int32_t* ticks, const uint8_t* mask, cudaStream_t st);

}  // namespace rsg
