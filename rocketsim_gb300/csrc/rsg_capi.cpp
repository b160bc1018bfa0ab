// rsg_capi.cpp -- host side of the C ABI declared in include/rocketsim_gb300.h.
//
// A batch owns the structure-of-arrays state of many arenas in device memory
// (layout in rsg_layout.h) and one CUDA stream.  Host-side bookkeeping that the
// reference keeps in its Arena object (car ids, update order, the last id
// handed out) is mirrored here so that id lookups need no device round trip.
// Everything that changes during a tick lives only on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/rocketsim_gb300.h"
#include "rsg_consts.cuh"
#include "rsg_kernels.h"
#include "rsg_layout.h"
#include "rsg_mesh.h"

using namespace rsg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
}  // namespace

namespace rsg {
int report_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace rsg

namespace {
int cuda_fail(cudaError_t e, const char* what) {
    return fail(RSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define RSG_CUDA(call)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// ---------------------------------------------------------------- shared arena mesh
struct MeshStore {
    bool ready = false;
    int device = -1;
    HostMesh host;
    float* tv = nullptr;
    QNode* nodes = nullptr;
    Subtree* sub = nullptr;
    TriInfo* info = nullptr;
    uint8_t* cells = nullptr;
    QNode* lg_block = nullptr;
    QNode* lg_over = nullptr;
    QNode* sub_grp = nullptr;
};
std::mutex g_mesh_mutex;
MeshStore g_soccar;

DevMeshPtrs mesh_ptrs(const MeshStore& m) {
    DevMeshPtrs p{};
    if (!m.ready) return p;
    p.tv = m.tv;
    p.nodes = m.nodes;
    p.sub = m.sub;
    p.info = m.info;
    p.cells = m.cells;
    p.lg_block = m.host.lg_block.empty() ? nullptr : m.lg_block;
    p.lg_over = m.lg_over;
    p.sub_grp = m.sub_grp;
    p.nsub_grp = (int)m.host.sub_groups.size();
    for (int k = 0; k < 3; k++) {
        p.lg_shift[k] = m.host.lg_shift[k];
        p.lg_n[k] = m.host.lg_n[k];
    }
    p.ntri = m.host.ntri;
    p.nnodes = m.host.cur_node;
    p.nsub = (int)m.host.subtrees.size();
    p.bvh_min = m.host.bvh_min;
    p.bvh_max = m.host.bvh_max;
    p.quant = m.host.quant;
    p.aabb_min = m.host.aabb_min;
    p.aabb_max = m.host.aabb_max;
    return p;
}

template <class T>
int upload(T*& dst, const std::vector<T>& src, const char* what) {
    size_t bytes = src.size() * sizeof(T);
    if (bytes == 0) bytes = sizeof(T);
    cudaError_t e = cudaMalloc((void**)&dst, bytes);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (!src.empty()) {
        e = cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, what);
    }
    return RSG_OK;
}

// Car::_BulletSetup derived constants (src/Sim/Car/Car.cpp:195-292)
CarCfgDev derive_config(const rsg_car_config& c) {
    const float U = RL::UU_TO_BT;
    CarCfgDev d;
    std::memset(&d, 0, sizeof(d));
    V3 size(c.hitbox_size.x, c.hitbox_size.y, c.hitbox_size.z);
    V3 he = (size * U) / 2.f;
    // btBoxShape: implicit dimensions keep the default 0.04 margin while setSafeMargin shrinks the
    // margin itself (B/BulletCollision/CollisionShapes/btBoxShape.cpp:17-25, btConvexInternalShape.h:63-90)
    float margin = 0.04f;
    V3 implicit = he - V3(margin, margin, margin);
    int minax = he.x < he.y ? (he.x < he.z ? 0 : 2) : (he.y < he.z ? 1 : 2);
    float safe = 0.1f * he[minax];
    if (safe < margin) margin = safe;
    V3 off = V3(c.hitbox_pos_offset.x, c.hitbox_pos_offset.y, c.hitbox_pos_offset.z) * U;
    V3 hm = implicit + V3(margin, margin, margin);
    V3 cmin = off - hm, cmax = off + hm;
    float lx = 2.f * hm.x, ly = 2.f * hm.y, lz = 2.f * hm.z;
    float m = RL::CAR_MASS_BT;
    V3 inertia(m / 12.f * (ly * ly + lz * lz), m / 12.f * (lx * lx + lz * lz), m / 12.f * (lx * lx + ly * ly));
    V3 lhe = 0.5f * (cmax - cmin), lc = 0.5f * (cmax + cmin);
    V3 amin = lc - lhe, amax = lc + lhe;
    float rad = len(amax - amin) * 0.5f;
    V3 cen = (amin + amax) * 0.5f;
    for (int k = 0; k < 3; k++) {
        d.he[k] = implicit[k];
        d.off[k] = off[k];
        d.comp_min[k] = cmin[k];
        d.comp_max[k] = cmax[k];
        d.inv_inertia[k] = inertia[k] != 0 ? 1.f / inertia[k] : 0.f;
    }
    d.margin = margin;
    d.breaking = (rad + len(cen)) * 0.02f;
    for (int i = 0; i < 4; i++) {
        bool front = i < 2, left = (i % 2) != 0;
        const rsg_wheel_pair_config& wp = front ? c.front_wheels : c.back_wheels;
        V3 o(wp.connection_point_offset.x, wp.connection_point_offset.y, wp.connection_point_offset.z);
        if (left) o.y *= -1;
        o = o * U;
        d.conn[i][0] = o.x;
        d.conn[i][1] = o.y;
        d.conn[i][2] = o.z;
    }
    d.rest[0] = (c.front_wheels.suspension_rest_length - RL::MAX_SUSPENSION_TRAVEL) * U;
    d.rest[1] = (c.back_wheels.suspension_rest_length - RL::MAX_SUSPENSION_TRAVEL) * U;
    d.radius[0] = c.front_wheels.wheel_radius * U;
    d.radius[1] = c.back_wheels.wheel_radius * U;
    d.dodge_deadzone = c.dodge_deadzone;
    d.three_wheels = c.three_wheels ? 1 : 0;
    return d;
}

// Car::Respawn's state (src/Sim/Car/Car.cpp:43-56) with CarState's defaults (Car.h:17-120)
rsg_car_state respawn_state(int team, int idx, float boost) {
    rsg_car_state s;
    std::memset(&s, 0, sizeof(s));
    const float xs[4] = {-2304, -2688, 2304, 2688};
    const float ys[4] = {-4608, -4608, -4608, -4608};
    float yaw0 = (float)(3.14159265358979323846 / 2);
    s.pos.x = xs[idx];
    s.pos.y = ys[idx] * (team == RSG_TEAM_BLUE ? 1 : -1);
    s.pos.z = RL::CAR_RESPAWN_Z;
    float yaw = (float)((double)yaw0 + (team == RSG_TEAM_BLUE ? 0 : 3.14159265358979323846));
    M3 m = m_euler_ypr(yaw, -0.f, -0.f);
    V3 f = m.col(0), r = m.col(1), u = m.col(2);
    s.rot_mat.forward = {f.x, f.y, f.z};
    s.rot_mat.right = {r.x, r.y, r.z};
    s.rot_mat.up = {u.x, u.y, u.z};
    s.boost = boost;
    s.is_on_ground = 1;
    s.ball_hit_info.tick_count_when_hit = ~0ULL;
    s.ball_hit_info.tick_count_when_extra_impulse_applied = ~0ULL;
    return s;
}

}  // namespace

// ---------------------------------------------------------------- batch
struct DevEventHost {  // mirror of the device event record
    uint32_t kind, tick_lo, tick_hi, a, b, flag;
};
static_assert(sizeof(DevEventHost) == DEV_EVENT_BYTES, "event record");

struct rsg_batch {
    int game_mode = 0;
    int device = 0;
    // launch shape of the tick kernel: tuned on the batch's first launch and again once it has run
    // RETUNE_TICKS ticks (identical states for every trial), cached per (device, arenas, car slots,
    // game mode, round), or fixed by the environment
    TickShape shape;
    bool tune_pending = true;
    bool shape_fixed = false;
    int tune_round = 0;
    uint64_t ticks_launched = 0;
    std::string tune_log;
    BatchBuffers buf{};
    cudaStream_t stream = nullptr;
    std::vector<CarCfgDev> cfgs;
    CarCfgDev* d_cfgs = nullptr;
    int cfg_cap = 0;
    // host mirror of per-arena bookkeeping
    std::vector<uint32_t> ncars, last_id;
    std::vector<uint32_t> ids;     // [A][MC] car id by slot
    std::vector<uint8_t> order;    // [A][MC] slot by update position
    std::vector<rsg_car_config> car_cfg;  // [A][MC] configuration by slot (for Arena::Serialize)
    std::vector<uint8_t> car_team;        // [A][MC] team by slot
    // staging
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
    void* d_ctl = nullptr;  // rsg_step_controls' per-tick controls (apart from d_stage: callbacks may use that)
    size_t ctl_bytes = 0;
    void* h_bounce = nullptr;  // pinned host buffer of the bulk getter (batches with empty car slots)
    size_t bounce_bytes = 0;
    std::vector<uint32_t> h_counts;
    std::vector<DevEventHost> h_events;
    rsg_goal_fn goal_fn = nullptr;
    void* goal_user = nullptr;
    rsg_bump_fn bump_fn = nullptr;
    void* bump_user = nullptr;
    rsg_ball_hit_fn hit_fn = nullptr;
    void* hit_user = nullptr;
    rsg_mutator_config mutators{};
    std::vector<float4> pads;  // per pad: position (uu), is_big
    rsg_arena_config arena_cfg{};                  // as given at creation (custom pads copied below)
    std::vector<rsg_boost_pad_config> custom_pads;
    float4* d_pads = nullptr;
};

namespace {

int ensure_stage(rsg_batch* b, size_t bytes) {
    if (b->stage_bytes >= bytes) return RSG_OK;
    if (b->d_stage) cudaFree(b->d_stage);
    b->d_stage = nullptr;
    b->stage_bytes = 0;
    RSG_CUDA(cudaMalloc(&b->d_stage, bytes));
    b->stage_bytes = bytes;
    return RSG_OK;
}

int ensure_host_bounce(rsg_batch* b, size_t bytes) {
    if (b->bounce_bytes >= bytes) return RSG_OK;
    if (b->h_bounce) cudaFreeHost(b->h_bounce);
    b->h_bounce = nullptr;
    b->bounce_bytes = 0;
    RSG_CUDA(cudaMallocHost(&b->h_bounce, bytes));
    b->bounce_bytes = bytes;
    return RSG_OK;
}

int set_device(rsg_batch* b) {
    RSG_CUDA(cudaSetDevice(b->device));
    return RSG_OK;
}

int check_arena(const rsg_batch* b, uint32_t arena) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    if (arena >= (uint32_t)b->buf.A) return fail(RSG_ERR_ARG, "arena index out of range");
    return RSG_OK;
}

int find_slot(const rsg_batch* b, uint32_t arena, uint32_t car_id) {
    int MC = b->buf.MC;
    for (uint32_t s = 0; s < b->ncars[arena]; s++)
        if (b->ids[(size_t)arena * MC + s] == car_id) return (int)s;
    return -1;
}

uint32_t pack_order(const rsg_batch* b, uint32_t arena) {
    uint32_t v = 0;
    for (uint32_t k = 0; k < b->ncars[arena]; k++) v |= (uint32_t)b->order[(size_t)arena * b->buf.MC + k] << (4 * k);
    return v;
}

// index of an arena-scalar word in the au array
size_t au_index(const rsg_batch* b, int field, uint32_t arena) { return (size_t)field * b->buf.A + arena; }

int write_au(rsg_batch* b, int field, uint32_t arena, uint32_t v) {
    RSG_CUDA(cudaMemcpyAsync(b->buf.au + au_index(b, field, arena), &v, 4, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}
int read_au(rsg_batch* b, int field, uint32_t arena, uint32_t* v) {
    RSG_CUDA(cudaMemcpyAsync(v, b->buf.au + au_index(b, field, arena), 4, cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int cfg_index(rsg_batch* b, const CarCfgDev& d) {
    for (size_t i = 0; i < b->cfgs.size(); i++)
        if (std::memcmp(&b->cfgs[i], &d, sizeof(d)) == 0) return (int)i;
    b->cfgs.push_back(d);
    if ((int)b->cfgs.size() > b->cfg_cap) {
        int cap = b->cfg_cap ? b->cfg_cap * 2 : 16;
        CarCfgDev* nd = nullptr;
        cudaError_t e = cudaMalloc((void**)&nd, sizeof(CarCfgDev) * cap);
        if (e != cudaSuccess) { b->cfgs.pop_back(); return cuda_fail(e, "cudaMalloc(car configs)"); }
        cudaStreamSynchronize(b->stream);
        if (b->d_cfgs) cudaFree(b->d_cfgs);
        b->d_cfgs = nd;
        b->cfg_cap = cap;
        b->buf.cfgs = nd;
    }
    cudaError_t e = cudaMemcpyAsync(b->d_cfgs, b->cfgs.data(), sizeof(CarCfgDev) * b->cfgs.size(), cudaMemcpyHostToDevice,
                                    b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(car configs)");
    return (int)b->cfgs.size() - 1;
}

// Delivers queued events to the callbacks and clears the device queues.
int drain_events(rsg_batch* b) {
    if (!b->buf.event_mask) return RSG_OK;
    int A = b->buf.A;
    b->h_counts.resize(A);
    RSG_CUDA(cudaMemcpyAsync(b->h_counts.data(), b->buf.au + au_index(b, AU_EVENTS, 0), 4 * (size_t)A,
                             cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    bool any = false;
    for (int a = 0; a < A; a++) any |= b->h_counts[a] != 0;
    if (!any) return RSG_OK;
    b->h_events.resize((size_t)A * MAX_EVENTS_PER_ARENA);
    RSG_CUDA(cudaMemcpyAsync(b->h_events.data(), b->buf.events, sizeof(DevEventHost) * b->h_events.size(),
                             cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaMemsetAsync(b->buf.au + au_index(b, AU_EVENTS, 0), 0, 4 * (size_t)A, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    for (int a = 0; a < A; a++) {
        uint32_t n = b->h_counts[a];
        if (n > (uint32_t)MAX_EVENTS_PER_ARENA) n = MAX_EVENTS_PER_ARENA;
        for (uint32_t k = 0; k < n; k++) {
            const DevEventHost& e = b->h_events[(size_t)a * MAX_EVENTS_PER_ARENA + k];
            uint64_t tick = (uint64_t)e.tick_lo | ((uint64_t)e.tick_hi << 32);
            if (e.kind == RSG_EVENT_GOAL && b->goal_fn) b->goal_fn(b, (uint32_t)a, (int)e.a, b->goal_user);
            else if (e.kind == RSG_EVENT_BUMP && b->bump_fn) b->bump_fn(b, (uint32_t)a, e.a, e.b, (int)e.flag, b->bump_user);
            else if (e.kind == RSG_EVENT_BALL_HIT && b->hit_fn) b->hit_fn(b, (uint32_t)a, e.a, tick, b->hit_user);
        }
    }
    return RSG_OK;
}

void update_event_mask(rsg_batch* b) {
    uint32_t m = 0;
    if (b->goal_fn) m |= 1u << RSG_EVENT_GOAL;
    if (b->bump_fn) m |= 1u << RSG_EVENT_BUMP;
    if (b->hit_fn) m |= 1u << RSG_EVENT_BALL_HIT;
    b->buf.event_mask = m;
}

// Reads the device error words; warnings (bits >= 8) are not failures.
int check_device_errors(rsg_batch* b) {
    int A = b->buf.A;
    b->h_counts.resize(A);
    RSG_CUDA(cudaMemcpyAsync(b->h_counts.data(), b->buf.au + au_index(b, AU_ERR, 0), 4 * (size_t)A, cudaMemcpyDeviceToHost,
                             b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    for (int a = 0; a < A; a++) {
        uint32_t e = b->h_counts[a] & 0xffu;
        if (e) {
            char msg[160];
            std::snprintf(msg, sizeof(msg), "arena %d reported device error flags 0x%x (capacity overflow or launch error)", a, e);
            return fail(RSG_ERR_DEVICE, msg);
        }
    }
    return RSG_OK;
}

}  // namespace

// ---------------------------------------------------------------- kernels used only here
namespace rsg {
cudaError_t launch_add_car(const BatchBuffers& b, uint32_t arena, uint32_t slot, uint32_t id, uint32_t cfg, uint32_t flags,
                           uint32_t cell, uint32_t ncars, uint32_t order, cudaStream_t st);
cudaError_t launch_remove_car(const BatchBuffers& b, uint32_t arena, uint32_t slot, uint32_t ncars, uint32_t order,
                              cudaStream_t st);
cudaError_t launch_init_arenas(const BatchBuffers& b, uint32_t ball_cell, cudaStream_t st);
cudaError_t launch_demolish(const BatchBuffers& b, uint32_t arena, uint32_t slot, float delay, cudaStream_t st);
CarCfgDev car_config_derived(const rsg_car_config& c) { return derive_config(c); }

// MutatorConfig(GameMode) (src/Sim/MutatorConfig/MutatorConfig.cpp:5-40, defaults in MutatorConfig.h:16-79)
// for the game modes the batch supports (soccar and THE_VOID share them).
// MutatorConfig(gameMode) (src/Sim/MutatorConfig/MutatorConfig.cpp:5-40)
rsg_mutator_config default_mutators(int game_mode) {
    rsg_mutator_config m;
    std::memset(&m, 0, sizeof(m));
    m.gravity = rsg_vec3{0, 0, RL::GRAVITY_Z};
    m.car_mass = RL::CAR_MASS_BT;
    m.car_world_friction = RL::CARWORLD_COLLISION_FRICTION;
    m.car_world_restitution = RL::CARWORLD_COLLISION_RESTITUTION;
    m.ball_mass = RL::BALL_MASS_BT;
    m.ball_max_speed = RL::BALL_MAX_SPEED;
    m.ball_drag = RL::BALL_DRAG;
    m.ball_world_friction = RL::BALL_FRICTION;
    m.ball_world_restitution = RL::BALL_RESTITUTION;
    m.jump_accel = RL::JUMP_ACCEL;
    m.jump_immediate_force = RL::JUMP_IMMEDIATE_FORCE;
    m.boost_accel_ground = RL::BOOST_ACCEL_GROUND;
    m.boost_accel_air = RL::BOOST_ACCEL_AIR;
    m.boost_used_per_second = RL::BOOST_USED_PER_SECOND;
    m.respawn_delay = RL::DEMO_RESPAWN_TIME;
    m.bump_cooldown_time = RL::BUMP_COOLDOWN_TIME;
    m.boost_pad_cooldown_big = RL::PAD_COOLDOWN_BIG;
    m.boost_pad_cooldown_small = RL::PAD_COOLDOWN_SMALL;
    m.car_spawn_boost_amount = RL::BOOST_SPAWN_AMOUNT;
    m.ball_hit_extra_force_scale = 1;
    m.bump_force_scale = 1;
    m.ball_radius = RL::BALL_COLLISION_RADIUS_SOCCAR;
    m.recharge_boost_per_second = RL::RECHARGE_BOOST_PER_SECOND;
    m.recharge_boost_delay = RL::RECHARGE_BOOST_DELAY;
    m.demo_mode = 0;
    m.goal_base_threshold_y = RL::SOCCAR_GOAL_SCORE_BASE_THRESHOLD_Y;
    if (game_mode == RSG_GAMEMODE_HEATSEEKER) {  // infinite boost
        m.car_spawn_boost_amount = 100;
        m.boost_used_per_second = 0;
    }
    return m;
}

// The device copy the tick reads: gravity as btDiscreteDynamicsWorld::setGravity receives it
// (gravity * UU_TO_BT, Arena.cpp:26), the ball radius as Ball::_BulletSetup sizes the sphere
// (ballRadius * UU_TO_BT, Ball.cpp:79).
MutatorsDev mutators_dev(const rsg_mutator_config& m) {
    MutatorsDev d;
    d.grav_bt[0] = m.gravity.x * RL::UU_TO_BT;
    d.grav_bt[1] = m.gravity.y * RL::UU_TO_BT;
    d.grav_bt[2] = m.gravity.z * RL::UU_TO_BT;
    d.car_world_friction = m.car_world_friction;
    d.car_world_restitution = m.car_world_restitution;
    d.ball_mass = m.ball_mass;
    d.ball_max_speed = m.ball_max_speed;
    d.ball_drag = m.ball_drag;
    d.ball_world_friction = m.ball_world_friction;
    d.ball_world_restitution = m.ball_world_restitution;
    d.jump_accel = m.jump_accel;
    d.jump_immediate_force = m.jump_immediate_force;
    d.boost_accel_ground = m.boost_accel_ground;
    d.boost_accel_air = m.boost_accel_air;
    d.boost_used_per_second = m.boost_used_per_second;
    d.respawn_delay = m.respawn_delay;
    d.bump_cooldown_time = m.bump_cooldown_time;
    d.pad_cooldown_big = m.boost_pad_cooldown_big;
    d.pad_cooldown_small = m.boost_pad_cooldown_small;
    d.car_spawn_boost = m.car_spawn_boost_amount;
    d.ball_hit_scale = m.ball_hit_extra_force_scale;
    d.bump_force_scale = m.bump_force_scale;
    d.ball_radius_uu = m.ball_radius;
    d.ball_radius_bt = m.ball_radius * RL::UU_TO_BT;
    d.unlimited_flips = m.unlimited_flips != 0;
    d.unlimited_double_jumps = m.unlimited_double_jumps != 0;
    d.recharge_boost = m.recharge_boost_enabled != 0;
    d.recharge_per_second = m.recharge_boost_per_second;
    d.recharge_delay = m.recharge_boost_delay;
    d.demo_mode = m.demo_mode;
    d.team_demos = m.enable_team_demos != 0;
    d.goal_threshold_y = m.goal_base_threshold_y;
    return d;
}
}  // namespace rsg

extern "C" {

int rsg_get_last_error(char* buf, uint64_t buf_len) {
    if (!buf || buf_len == 0) return RSG_ERR_ARG;
    std::snprintf(buf, (size_t)buf_len, "%s", g_last_error.c_str());
    return RSG_OK;
}

int rsg_init_from_mem(int game_mode, const uint8_t* const* mesh_files, const uint64_t* mesh_sizes, int n_files) {
    if (game_mode != RSG_GAMEMODE_SOCCAR) return fail(RSG_ERR_ARG, "only soccar meshes are loaded");
    if (!mesh_files || !mesh_sizes || n_files <= 0) return fail(RSG_ERR_ARG, "no mesh files");
    std::lock_guard<std::mutex> lock(g_mesh_mutex);
    if (g_soccar.ready) return RSG_OK;  // idempotent like RocketSim::InitFromMem (RocketSim.cpp:100-105)
    if (n_files != 1) return fail(RSG_ERR_MESH, "exactly one soccar collision mesh is supported");
    MeshStore m;
    std::string err;
    if (!build_mesh(mesh_files[0], mesh_sizes[0], m.host, err)) return fail(RSG_ERR_MESH, "mesh rejected: " + err);
    RSG_CUDA(cudaGetDevice(&m.device));
    std::vector<float> tv(m.host.tri_verts.size() * 3);
    for (size_t i = 0; i < m.host.tri_verts.size(); i++) {
        tv[i * 3 + 0] = m.host.tri_verts[i].x;
        tv[i * 3 + 1] = m.host.tri_verts[i].y;
        tv[i * 3 + 2] = m.host.tri_verts[i].z;
    }
    int rc;
    if ((rc = upload(m.tv, tv, "mesh vertices")) != RSG_OK) return rc;
    if ((rc = upload(m.nodes, m.host.nodes, "mesh nodes")) != RSG_OK) return rc;
    if ((rc = upload(m.sub, m.host.subtrees, "mesh subtrees")) != RSG_OK) return rc;
    if ((rc = upload(m.info, m.host.info, "mesh edge info")) != RSG_OK) return rc;
    if ((rc = upload(m.cells, m.host.mesh_cells, "mesh cells")) != RSG_OK) return rc;
    if ((rc = upload(m.lg_block, m.host.lg_block, "mesh leaf grid")) != RSG_OK) return rc;
    if ((rc = upload(m.lg_over, m.host.lg_over, "mesh leaf grid")) != RSG_OK) return rc;
    if ((rc = upload(m.sub_grp, m.host.sub_groups, "mesh subtree groups")) != RSG_OK) return rc;
    m.ready = true;
    g_soccar = std::move(m);
    return RSG_OK;
}

int rsg_get_car_config_preset(int preset, rsg_car_config* out) {
    if (!out || preset < 0 || preset > 5) return fail(RSG_ERR_ARG, "preset out of range");
    const PresetData& p = PRESETS[preset];
    std::memset(out, 0, sizeof(*out));
    out->hitbox_size = {p.size[0], p.size[1], p.size[2]};
    out->hitbox_pos_offset = {p.off[0], p.off[1], p.off[2]};
    out->front_wheels.wheel_radius = p.frad;
    out->front_wheels.suspension_rest_length = p.fsus;
    out->front_wheels.connection_point_offset = {p.fwo[0], p.fwo[1], p.fwo[2]};
    out->back_wheels.wheel_radius = p.brad;
    out->back_wheels.suspension_rest_length = p.bsus;
    out->back_wheels.connection_point_offset = {p.bwo[0], p.bwo[1], p.bwo[2]};
    out->three_wheels = 0;
    out->dodge_deadzone = 0.5f;
    return RSG_OK;
}

namespace {

// Block-shape tuner.  Every launch shape gives the same results, so the shapes can be timed on the
// batch itself: a tuning launch saves the arena records, runs each candidate shape from the saved
// state (launch, wait, time), restores the records and launches for real with the fastest.  The
// candidates are searched one parameter at a time: barriers in the collision work (not in the first
// round), arenas per block (16 to 4, as shared memory allows), threads per car in the vehicle update
// (1, 2, 4), the BVH subtree headers in shared memory or read through L2, wheel rays on the leaf grid
// or walking the BVH, a persistent launch.  It runs on the batch's first launch and again, from the
// default shape and with a second look at the barriers and the arenas per block, on the first launch
// after RETUNE_TICKS ticks, when the arenas have left the start of the game (cars landed, on walls, in
// contact: the collision work that decides the best shape has grown).  The choice of each round is cached per
// (device, arenas, car slots, game mode).
constexpr uint64_t RETUNE_TICKS = 1024;
struct TuneKey {
    int dev, A, MC, arena, round;
    bool operator<(const TuneKey& o) const {
        return std::tie(dev, A, MC, arena, round) < std::tie(o.dev, o.A, o.MC, o.arena, o.round);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<TickShape, std::string>> g_tune_cache;

std::string shape_str(const TickShape& s) {
    char buf[160];
    std::snprintf(buf, sizeof(buf),
                  "arenas_per_block=%d lanes_per_car=%d header_cache=%d leaf_grid=%d collide_sync=%d persistent=%d",
                  s.arenas_per_block, s.lanes_per_car, s.header_cache, s.leaf_grid, s.collide_sync, s.persistent);
    return buf;
}

cudaError_t run_tuner(rsg_batch* b, const rsg_car_controls* controls, int ticks) {
    b->tune_pending = false;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(b->stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return cudaSuccess;  // no synchronous trials inside a capture: keep the current shape
    const int round = b->tune_round++;
    const std::string prefix = round == 0 ? "" : b->tune_log + " | after " + std::to_string(RETUNE_TICKS) + " ticks: ";
    const TuneKey key{b->device, b->buf.A, b->buf.MC, b->buf.has_arena, round};
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            b->shape = it->second.first;
            b->tune_log = prefix + it->second.second + " (cached)";
            return cudaSuccess;
        }
    }
    const BatchBuffers& B = b->buf;
    const size_t rec_b = sizeof(uint32_t) * (size_t)rec_words(B.MC) * B.A, au_b = sizeof(uint32_t) * AU_COUNT * B.A;
    const size_t pl_b = sizeof(uint32_t) * B.A;
    char* snap = nullptr;
    cudaError_t e = cudaMalloc(&snap, rec_b + au_b + 2 * pl_b);
    if (e != cudaSuccess) return e;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    auto copy_all = [&](bool save) -> cudaError_t {
        void* dev[4] = {B.rec, B.au, B.place, B.cost};
        size_t sz[4] = {rec_b, au_b, pl_b, pl_b}, off = 0;
        for (int i = 0; i < 4; i++) {
            cudaError_t r = save ? cudaMemcpyAsync(snap + off, dev[i], sz[i], cudaMemcpyDeviceToDevice, b->stream)
                                 : cudaMemcpyAsync(dev[i], snap + off, sz[i], cudaMemcpyDeviceToDevice, b->stream);
            if (r != cudaSuccess) return r;
            off += sz[i];
        }
        return cudaSuccess;
    };
    auto trial = [&](const TickShape& s, double& ms) -> cudaError_t {  // the faster of two launches
        cudaError_t r = cudaSuccess;
        ms = 1e30;
        for (int rep = 0; rep < 2 && r == cudaSuccess; rep++) {
            r = copy_all(false);
            if (r == cudaSuccess) r = cudaEventRecord(ev[0], b->stream);
            if (r == cudaSuccess) r = launch_tick(B, controls, ticks, s, b->stream);
            if (r == cudaSuccess) r = cudaEventRecord(ev[1], b->stream);
            if (r == cudaSuccess) r = cudaEventSynchronize(ev[1]);
            float f = 0;
            if (r == cudaSuccess) r = cudaEventElapsedTime(&f, ev[0], ev[1]);
            if (r == cudaSuccess && f < ms) ms = f;
        }
        return r;
    };
    std::string log;
    const int per_arena = tick_smem_per_arena(B.MC);
    // round 0 starts from the batch's shape, later rounds from the default one (the first round's
    // choice was made for the start of a game)
    TickShape best = round == 0 ? b->shape : TickShape{};
    while (best.arenas_per_block > 1 && per_arena * best.arenas_per_block + 16 > 227 * 1024) best.arenas_per_block--;
    do {
        if ((e = cudaEventCreate(&ev[0])) != cudaSuccess || (e = cudaEventCreate(&ev[1])) != cudaSuccess) break;
        if ((e = copy_all(true)) != cudaSuccess) break;
        double ms = 0, best_ms = 0;
        if ((e = trial(best, ms)) != cudaSuccess) break;  // loads the module and warms the caches
        if ((e = trial(best, best_ms)) != cudaSuccess) break;
        log = shape_str(best) + ": " + std::to_string(best_ms / ticks) + " ms/tick";
        auto consider = [&](TickShape s) -> cudaError_t {
            double t = 0;
            cudaError_t r = trial(s, t);
            if (r != cudaSuccess) return r;
            log += "; " + shape_str(s) + ": " + std::to_string(t / ticks) + " ms/tick";
            if (t < best_ms) { best_ms = t; best = s; }
            return cudaSuccess;
        };
        auto toggle_sync = [&]() -> cudaError_t {
            TickShape s = best;
            s.collide_sync = best.collide_sync ? 0 : 1;
            return consider(s);
        };
        auto widths = [&]() -> cudaError_t {
            const TickShape base = best;
            for (int w = TICK_MAX_ARENAS_PER_BLOCK; w >= 4; w--) {
                if (w == base.arenas_per_block || per_arena * w + 16 > 227 * 1024) continue;
                TickShape s = base;
                s.arenas_per_block = w;
                cudaError_t r = consider(s);
                if (r != cudaSuccess) return r;
            }
            return cudaSuccess;
        };
        // one parameter at a time from the best shape so far; the collision barriers first (at a
        // game's steady state they change the cost of everything else).  The first round keeps them:
        // at a batch's first launch the arenas have barely any collision work to measure them on.
        if (round > 0 && (e = toggle_sync()) != cudaSuccess) break;
        if ((e = widths()) != cudaSuccess) break;
        const TickShape base = best;
        for (int l : {1, 2, 4}) {
            if (e != cudaSuccess || l == base.lanes_per_car) continue;
            TickShape s = base;
            s.lanes_per_car = l;
            e = consider(s);
        }
        const TickShape base2 = best;
        for (int h : {0, 1}) {
            if (e != cudaSuccess || !B.mesh.sub || h == base2.header_cache) continue;
            TickShape s = base2;
            s.header_cache = h;
            e = consider(s);
        }
        if (e == cudaSuccess && B.mesh.lg_block) {
            TickShape s = best;
            s.leaf_grid = best.leaf_grid ? 0 : 1;
            e = consider(s);
        }
        if (e == cudaSuccess) {
            TickShape s = best;
            s.persistent = best.persistent ? 0 : 1;
            e = consider(s);
        }
        // after the start of a game, a second look at the two parameters that matter most
        if (e == cudaSuccess && round > 0) e = toggle_sync();
        if (e == cudaSuccess && round > 0) e = widths();
        if (e == cudaSuccess) e = copy_all(false);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    } while (false);
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    cudaFree(snap);
    if (e != cudaSuccess) return e;
    b->shape = best;
    const std::string mine = "chose " + shape_str(best) + " from " + log;
    b->tune_log = prefix + mine;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = {best, mine};
    return cudaSuccess;
}

// Launches `ticks` ticks (tuning the shape first on the batch's first launch and on its first launch
// after RETUNE_TICKS ticks), then re-places the arenas in blocks by the cost of their collision work
// in that launch.
cudaError_t tuned_launch(rsg_batch* b, const rsg_car_controls* controls, int ticks) {
    cudaError_t e = cudaSuccess;
    if (!b->shape_fixed && b->tune_round == 1 && b->ticks_launched >= RETUNE_TICKS) b->tune_pending = true;
    b->ticks_launched += (uint64_t)ticks;
    if (b->tune_pending) e = run_tuner(b, controls, ticks);
    if (e == cudaSuccess) e = launch_tick(b->buf, controls, ticks, b->shape, b->stream);
    if (e == cudaSuccess) e = launch_place_arenas(b->buf, b->stream);
    return e;
}

}  // namespace

int rsg_get_default_arena_config(rsg_arena_config* out) {
    if (!out) return fail(RSG_ERR_ARG, "null output");
    std::memset(out, 0, sizeof(*out));
    out->mem_weight_mode = 0;  // HEAVY
    out->no_ball_rot = 1;
    out->use_custom_broadphase = 1;
    out->use_custom_boost_pads = 0;
    out->min_pos = rsg_vec3{-5600, -6000, 0};
    out->max_pos = rsg_vec3{5600, 6000, 2200};
    out->max_aabb_len = 370;
    out->max_objects = 512;
    return RSG_OK;
}

rsg_batch* rsg_batch_create(int game_mode, uint32_t n_arenas, uint32_t max_cars_per_arena, float tick_rate) {
    return rsg_batch_create_ex(game_mode, n_arenas, max_cars_per_arena, tick_rate, nullptr);
}

rsg_batch* rsg_batch_create_ex(int game_mode, uint32_t n_arenas, uint32_t max_cars_per_arena, float tick_rate,
                               const rsg_arena_config* config) {
    rsg_arena_config cfg;
    rsg_get_default_arena_config(&cfg);
    if (config) {
        const rsg_arena_config& c = *config;
        if (c.min_pos.x != cfg.min_pos.x || c.min_pos.y != cfg.min_pos.y || c.min_pos.z != cfg.min_pos.z ||
            c.max_pos.x != cfg.max_pos.x || c.max_pos.y != cfg.max_pos.y || c.max_pos.z != cfg.max_pos.z ||
            c.max_aabb_len != cfg.max_aabb_len || !c.use_custom_broadphase) {
            fail(RSG_ERR_ARG, "only the default broadphase bounds, cell size and custom broadphase are supported");
            return nullptr;
        }
        if (c.use_custom_boost_pads && (c.num_custom_boost_pads > (uint32_t)NUM_PADS ||
                                        (c.num_custom_boost_pads && !c.custom_boost_pads))) {
            fail(RSG_ERR_ARG, "custom boost pads: at most 34, given as a host array");
            return nullptr;
        }
        cfg = c;
    }
    if (game_mode != RSG_GAMEMODE_SOCCAR && game_mode != RSG_GAMEMODE_HEATSEEKER && game_mode != RSG_GAMEMODE_THE_VOID) {
        fail(RSG_ERR_ARG, "game mode not supported (soccar, heatseeker and the void only)");
        return nullptr;
    }
    if (n_arenas == 0 || n_arenas > (1u << 24)) { fail(RSG_ERR_ARG, "n_arenas out of range"); return nullptr; }
    if (max_cars_per_arena == 0 || max_cars_per_arena > (uint32_t)MAX_CARS) {
        fail(RSG_ERR_ARG, "max_cars_per_arena must be 1..8");
        return nullptr;
    }
    if (!(tick_rate >= 15.f && tick_rate <= 120.f)) {  // Arena.cpp:419
        fail(RSG_ERR_ARG, "tick rate must be 15..120");
        return nullptr;
    }
    // heatseeker plays in the soccar arena (the same collision meshes, pads and goals)
    bool arena = game_mode == RSG_GAMEMODE_SOCCAR || game_mode == RSG_GAMEMODE_HEATSEEKER;
    if (arena && !g_soccar.ready) {
        fail(RSG_ERR_STATE, "no soccar mesh loaded (rsg_init_from_mem)");
        return nullptr;
    }
    rsg_batch* b = new rsg_batch();
    b->game_mode = game_mode;
    cudaError_t de = cudaGetDevice(&b->device);
    if (de != cudaSuccess) {
        delete b;
        cuda_fail(de, "cudaGetDevice");
        return nullptr;
    }
    if (arena && g_soccar.device != b->device) {
        delete b;
        fail(RSG_ERR_STATE, "the mesh was loaded on another device");
        return nullptr;
    }
    if (const char* w = std::getenv("RSG_TICK_SHAPE")) {  // fixed shape "w,lanes,header,leafgrid[,sync[,persistent]]"
        int v[6] = {TICK_MAX_ARENAS_PER_BLOCK, 4, -1, 1, 1, 0};
        std::sscanf(w, "%d,%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]);
        b->shape.arenas_per_block = v[0];
        b->shape.lanes_per_car = v[1];
        b->shape.header_cache = v[2];
        b->shape.leaf_grid = v[3];
        b->shape.collide_sync = v[4];
        b->shape.persistent = v[5] ? 1 : 0;
        b->tune_pending = false;
        b->shape_fixed = true;
    }
    {  // at most as many arenas per block as shared memory holds (launch_tick clamps the same way)
        const int per_arena = tick_smem_per_arena((int)max_cars_per_arena);
        int& w = b->shape.arenas_per_block;
        if (w < 1 || w > TICK_MAX_ARENAS_PER_BLOCK) w = TICK_MAX_ARENAS_PER_BLOCK;
        while (w > 1 && per_arena * w + 16 > 227 * 1024) w--;
    }
    if (!b->tune_pending) b->tune_log = "fixed by RSG_TICK_SHAPE: " + shape_str(b->shape);
    BatchBuffers& B = b->buf;
    B.A = (int)n_arenas;
    B.MC = (int)max_cars_per_arena;
    B.has_arena = arena ? 1 : 0;
    B.heatseeker = game_mode == RSG_GAMEMODE_HEATSEEKER ? 1 : 0;
    B.dt = 1.f / tick_rate;
    b->mutators = default_mutators(game_mode);
    B.mut = mutators_dev(b->mutators);
    // boost pads: ArenaConfig's custom list or the soccar pads (Arena.cpp:498-533)
    b->pads.clear();
    if (cfg.use_custom_boost_pads) {
        for (uint32_t i = 0; i < cfg.num_custom_boost_pads; i++) {
            const rsg_boost_pad_config& pc = cfg.custom_boost_pads[i];
            b->pads.push_back(float4{pc.pos.x, pc.pos.y, pc.pos.z, pc.is_big ? 1.f : 0.f});
        }
    } else {
        for (int i = 0; i < NUM_PADS; i++)
            b->pads.push_back(float4{PAD_LOCS[i][0], PAD_LOCS[i][1], PAD_LOCS[i][2], i < 6 ? 1.f : 0.f});
    }
    B.npads = (int)b->pads.size();
    b->arena_cfg = cfg;
    b->custom_pads.assign(cfg.custom_boost_pads, cfg.custom_boost_pads + (cfg.use_custom_boost_pads ? cfg.num_custom_boost_pads : 0));
    b->arena_cfg.custom_boost_pads = b->custom_pads.empty() ? nullptr : b->custom_pads.data();
    B.custom_pads = cfg.use_custom_boost_pads ? 1 : 0;
    B.no_ball_rot = cfg.no_ball_rot ? 1 : 0;
    B.mesh = mesh_ptrs(g_soccar);
    B.grid = default_grid();
    size_t A = n_arenas, MC = max_cars_per_arena;
    auto alloc = [&](void** p, size_t bytes) -> bool {  // zeroed on the batch's stream, ahead of its kernels
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, b->stream);
        if (e != cudaSuccess) { cuda_fail(e, "cudaMalloc(batch)"); return false; }
        return true;
    };
    if (cudaError_t pe = ensure_epa_pool(); pe != cudaSuccess) {
        delete b;
        cuda_fail(pe, "EPA work pool");
        return nullptr;
    }
    cudaError_t se = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (se != cudaSuccess) {
        cuda_fail(se, "cudaStreamCreateWithFlags");
        b->stream = nullptr;
        rsg_batch_destroy(b);
        return nullptr;
    }
    bool ok = alloc((void**)&b->d_pads, sizeof(float4) * NUM_PADS);
    if (ok && !b->pads.empty())
        ok = cudaMemcpyAsync(b->d_pads, b->pads.data(), sizeof(float4) * b->pads.size(), cudaMemcpyHostToDevice,
                             b->stream) == cudaSuccess &&
             cudaStreamSynchronize(b->stream) == cudaSuccess;  // after the buffer's zeroing, on the same stream
    B.pad_cfg = b->d_pads;
    ok = ok && alloc((void**)&B.rec, sizeof(uint32_t) * (size_t)rec_words((int)MC) * A);
    ok = ok && alloc((void**)&B.au, sizeof(uint32_t) * AU_COUNT * A);
    ok = ok && alloc(&B.events, (size_t)DEV_EVENT_BYTES * MAX_EVENTS_PER_ARENA * A);
    ok = ok && alloc((void**)&B.place, sizeof(uint32_t) * A);
    ok = ok && alloc((void**)&B.cost, sizeof(uint32_t) * A);
    ok = ok && alloc((void**)&B.group_next, sizeof(uint32_t));
    {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess) sms = 0;
        B.scratch_slots = tick_scratch_slots((int)A, sms);
        if (const size_t ts = tick_scratch_bytes(B.scratch_slots, (int)MC)) ok = ok && alloc((void**)&B.tick_scratch, ts);
    }
    if (!ok) {
        rsg_batch_destroy(b);
        return nullptr;
    }
    b->ncars.assign(A, 0);
    b->last_id.assign(A, 0);
    b->ids.assign(A * MC, 0);
    b->order.assign(A * MC, 0);
    b->car_cfg.assign(A * MC, rsg_car_config{});
    b->car_team.assign(A * MC, 0);
    // ball at rest (Arena.cpp:491-496) and its broadphase proxy created before any car
    {
        V3 p(0, 0, RL::BALL_REST_Z * RL::UU_TO_BT);
        float m = RL::BALL_COLLISION_RADIUS_SOCCAR * RL::UU_TO_BT + 0.08f;
        V3 mn = p - V3(m, m, m) - V3(0.02f, 0.02f, 0.02f);
        V3 f = (mn - B.grid.mn) / B.grid.cell;
        int i = std::min(std::max((int)f.x, 0), B.grid.nx - 1);
        int j = std::min(std::max((int)f.y, 0), B.grid.ny - 1);
        int k = std::min(std::max((int)f.z, 0), B.grid.nz - 1);
        uint32_t cell = (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16);
        cudaError_t e = launch_init_arenas(B, cell, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) {
            cuda_fail(e, "init arenas");
            rsg_batch_destroy(b);
            return nullptr;
        }
    }
    return b;
}

void rsg_batch_destroy(rsg_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    BatchBuffers& B = b->buf;
    void* ptrs[] = {B.rec, B.au, B.events, B.place, B.cost, B.group_next, B.tick_scratch, b->d_cfgs, b->d_stage,
                    b->d_pads, b->d_ctl};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->h_bounce) cudaFreeHost(b->h_bounce);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int rsg_batch_num_arenas(const rsg_batch* b, uint32_t* out) {
    if (!b || !out) return fail(RSG_ERR_ARG, "null argument");
    *out = (uint32_t)b->buf.A;
    return RSG_OK;
}

int rsg_batch_num_pads(const rsg_batch* b, uint32_t* out) {
    if (!b || !out) return fail(RSG_ERR_ARG, "null argument");
    *out = b->buf.has_arena ? (uint32_t)b->buf.npads : 0u;
    return RSG_OK;
}

static_assert(sizeof(rsg_mutator_config) == 116, "rsg_mutator_config layout");

int rsg_get_default_mutator_config(int game_mode, rsg_mutator_config* out) {
    if (!out) return fail(RSG_ERR_ARG, "null output");
    if (game_mode != RSG_GAMEMODE_SOCCAR && game_mode != RSG_GAMEMODE_HEATSEEKER && game_mode != RSG_GAMEMODE_THE_VOID)
        return fail(RSG_ERR_ARG, "game mode not supported (soccar and THE_VOID are)");
    *out = default_mutators(game_mode);
    return RSG_OK;
}

int rsg_get_mutator_config(const rsg_batch* b, rsg_mutator_config* out) {
    if (!b || !out) return fail(RSG_ERR_ARG, "null argument");
    *out = b->mutators;
    return RSG_OK;
}

// Arena::SetMutatorConfig (src/Sim/Arena/Arena.cpp:17-48) for every arena of the batch.
int rsg_set_mutator_config(rsg_batch* b, const rsg_mutator_config* c) {
    if (!b || !c) return fail(RSG_ERR_ARG, "null argument");
    if (c->car_mass != RL::CAR_MASS_BT)
        return fail(RSG_ERR_ARG, "car_mass other than CAR_MASS_BT is not supported (RocketSim applies it only to "
                                 "existing cars, with the ball's mass: Arena.cpp:35-41)");
    if (!(c->ball_radius > 0) || !(c->ball_mass > 0) || c->demo_mode > 2)
        return fail(RSG_ERR_ARG, "ball_radius and ball_mass must be > 0 and demo_mode 0..2");
    {  // btRSBroadphase::createProxy rejects a dynamic AABB whose diagonal exceeds the cell size
       // (libsrc/bullet3-3.24/BulletCollision/BroadphaseCollision/btRSBroadphase.cpp:228-229)
        const float side = 2.f * (c->ball_radius * RL::UU_TO_BT + 0.08f);
        if (3.f * side * side > b->buf.grid.cell * b->buf.grid.cell)
            return fail(RSG_ERR_ARG, "ball_radius too large: the ball's bounding box must fit a broadphase cell");
    }
    const bool ball_changed = c->ball_radius != b->mutators.ball_radius || c->ball_mass != b->mutators.ball_mass;
    if (ball_changed)
        for (uint32_t n : b->ncars)
            if (n) return fail(RSG_ERR_STATE, "ball_radius / ball_mass can change only while the batch holds no car "
                                              "(RocketSim re-creates its ball, after the cars in Bullet's object "
                                              "order: Arena.cpp:28-33)");
    int rc;
    if ((rc = set_device(b))) return rc;
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    b->mutators = *c;
    b->buf.mut = mutators_dev(*c);
    if (ball_changed) {  // the new ball starts at rest at (0, 0, radius) (Ball::_BulletSetup, Ball.cpp:85-115)
        const size_t A = (size_t)b->buf.A;
        std::vector<rsg_ball_state> balls(A);
        rsg_ball_state s;
        std::memset(&s, 0, sizeof(s));
        s.pos = rsg_vec3{0, 0, c->ball_radius};
        s.rot_mat.forward = rsg_vec3{1, 0, 0};
        s.rot_mat.right = rsg_vec3{0, 1, 0};
        s.rot_mat.up = rsg_vec3{0, 0, 1};
        for (auto& x : balls) x = s;
        if ((rc = ensure_stage(b, sizeof(rsg_ball_state) * A))) return rc;
        RSG_CUDA(cudaMemcpyAsync(b->d_stage, balls.data(), sizeof(rsg_ball_state) * A, cudaMemcpyHostToDevice,
                                 b->stream));
        RSG_CUDA(launch_set_balls(b->buf, nullptr, (int)A, (const rsg_ball_state*)b->d_stage, b->stream));
        RSG_CUDA(cudaStreamSynchronize(b->stream));
    }
    return RSG_OK;
}

// Arena::AddCar with the next car id, or with `forced_id` (Arena::DeserializeNew keeps ids)
static int add_car_impl(rsg_batch* b, uint32_t arena, int team, const rsg_car_config* config, int respawn_index,
                        uint32_t forced_id, uint32_t* out_car_id) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!config) return fail(RSG_ERR_ARG, "null car config");
    if (team != RSG_TEAM_BLUE && team != RSG_TEAM_ORANGE) return fail(RSG_ERR_ARG, "team must be 0 or 1");
    if (respawn_index < -1 || respawn_index > 3) return fail(RSG_ERR_ARG, "respawn index must be -1..3");
    if (b->ncars[arena] >= (uint32_t)b->buf.MC) return fail(RSG_ERR_STATE, "arena is full (max_cars_per_arena)");
    if ((rc = set_device(b))) return rc;
    CarCfgDev d = derive_config(*config);
    int ci = cfg_index(b, d);
    if (ci < 0) return ci;
    uint32_t slot = b->ncars[arena];
    uint32_t id = forced_id ? forced_id : ++b->last_id[arena];
    size_t MC = b->buf.MC;
    b->ids[arena * MC + slot] = id;
    b->car_cfg[arena * MC + slot] = *config;
    b->car_team[arena * MC + slot] = (uint8_t)team;
    b->order[arena * MC + slot] = (uint8_t)slot;
    b->ncars[arena] = slot + 1;
    // broadphase proxy at the AddCar-time transform (identity): cell of the compound AABB minimum
    V3 cmin(d.comp_min[0], d.comp_min[1], d.comp_min[2]), cmax(d.comp_max[0], d.comp_max[1], d.comp_max[2]);
    V3 lhe = 0.5f * (cmax - cmin), lc = 0.5f * (cmax + cmin);
    V3 mn = lc - lhe;
    const GridSpec& g = b->buf.grid;
    V3 f = (mn - g.mn) / g.cell;
    int i = std::min(std::max((int)f.x, 0), g.nx - 1);
    int j = std::min(std::max((int)f.y, 0), g.ny - 1);
    int k = std::min(std::max((int)f.z, 0), g.nz - 1);
    uint32_t cell = (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16);
    uint32_t flags = F_PRESENT | (team == RSG_TEAM_ORANGE ? F_TEAM_ORANGE : 0u);
    RSG_CUDA(launch_add_car(b->buf, arena, slot, id, (uint32_t)ci, flags, cell, slot + 1, pack_order(b, arena), b->stream));
    rsg_car_state s = respawn_state(team, respawn_index < 0 ? 0 : respawn_index, b->mutators.car_spawn_boost_amount);
    if ((rc = ensure_stage(b, sizeof(rsg_car_state) + 8))) return rc;
    uint32_t idx[2] = {arena, slot};
    char* st = (char*)b->d_stage;
    RSG_CUDA(cudaMemcpyAsync(st, &s, sizeof(s), cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaMemcpyAsync(st + sizeof(s), idx, 8, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_set_cars(b->buf, (const uint32_t*)(st + sizeof(s)), 1, (const rsg_car_state*)st, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    if (out_car_id) *out_car_id = id;
    return RSG_OK;
}

int rsg_add_car(rsg_batch* b, uint32_t arena, int team, const rsg_car_config* config, int respawn_index,
                uint32_t* out_car_id) {
    return add_car_impl(b, arena, team, config, respawn_index, 0, out_car_id);
}

int rsg_remove_car(rsg_batch* b, uint32_t arena, uint32_t car_id) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    int slot = find_slot(b, arena, car_id);
    if (slot < 0) return fail(RSG_ERR_ARG, "no car with that id");
    if ((rc = set_device(b))) return rc;
    size_t MC = b->buf.MC;
    uint32_t n = b->ncars[arena];
    for (uint32_t s = (uint32_t)slot; s + 1 < n; s++) {
        b->ids[arena * MC + s] = b->ids[arena * MC + s + 1];
        b->car_cfg[arena * MC + s] = b->car_cfg[arena * MC + s + 1];
        b->car_team[arena * MC + s] = b->car_team[arena * MC + s + 1];
    }
    // drop the slot from the update order and renumber the slots behind it
    std::vector<uint8_t> ord;
    for (uint32_t k = 0; k < n; k++) {
        uint8_t v = b->order[arena * MC + k];
        if (v == (uint8_t)slot) continue;
        ord.push_back(v > slot ? (uint8_t)(v - 1) : v);
    }
    for (size_t k = 0; k < ord.size(); k++) b->order[arena * MC + k] = ord[k];
    b->ncars[arena] = n - 1;
    RSG_CUDA(launch_remove_car(b->buf, arena, (uint32_t)slot, n - 1, pack_order(b, arena), b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_car_ids(const rsg_batch* b, uint32_t arena, uint32_t* out_ids, uint32_t cap, uint32_t* out_n) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    uint32_t n = b->ncars[arena];
    for (uint32_t k = 0; k < n && k < cap; k++)
        if (out_ids) out_ids[k] = b->ids[(size_t)arena * b->buf.MC + b->order[(size_t)arena * b->buf.MC + k]];
    if (out_n) *out_n = n;
    return RSG_OK;
}

int rsg_set_car_update_order(rsg_batch* b, uint32_t arena, const uint32_t* ids, uint32_t n) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!ids || n != b->ncars[arena]) return fail(RSG_ERR_ARG, "order must list every car of the arena once");
    std::vector<uint8_t> ord;
    uint32_t seen = 0;
    for (uint32_t k = 0; k < n; k++) {
        int s = find_slot(b, arena, ids[k]);
        if (s < 0 || (seen >> s) & 1u) return fail(RSG_ERR_ARG, "order must list every car of the arena once");
        seen |= 1u << s;
        ord.push_back((uint8_t)s);
    }
    for (uint32_t k = 0; k < n; k++) b->order[(size_t)arena * b->buf.MC + k] = ord[k];
    if ((rc = set_device(b))) return rc;
    return write_au(b, AU_ORDER, arena, pack_order(b, arena));
}

int rsg_set_car_controls(rsg_batch* b, uint32_t arena, uint32_t car_id, const rsg_car_controls* c) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!c) return fail(RSG_ERR_ARG, "null controls");
    int slot = find_slot(b, arena, car_id);
    if (slot < 0) return fail(RSG_ERR_ARG, "no car with that id");
    if ((rc = set_device(b))) return rc;
    // controls of one car: five floats and three flag bits in the car's SoA columns
    float v[5] = {c->throttle, c->steer, c->pitch, c->yaw, c->roll};
    uint32_t* rec = b->buf.rec + (size_t)arena * rec_words(b->buf.MC);
    RSG_CUDA(cudaMemcpyAsync(rec + rec_car_f(CF_CTRL, slot), v, sizeof(v), cudaMemcpyHostToDevice, b->stream));
    uint32_t* fl = rec + rec_car_u(CU_FLAGS, slot);
    uint32_t flags = 0;
    RSG_CUDA(cudaMemcpyAsync(&flags, fl, 4, cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    flags &= ~(uint32_t)(F_CTRL_JUMP | F_CTRL_BOOST | F_CTRL_HB);
    if (c->jump) flags |= F_CTRL_JUMP;
    if (c->boost) flags |= F_CTRL_BOOST;
    if (c->handbrake) flags |= F_CTRL_HB;
    RSG_CUDA(cudaMemcpyAsync(fl, &flags, 4, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_set_controls_all(rsg_batch* b, const rsg_car_controls* controls, uint64_t count) {
    if (!b || !controls) return fail(RSG_ERR_ARG, "null argument");
    size_t n = (size_t)b->buf.A * b->buf.MC;
    if (count != n) return fail(RSG_ERR_ARG, "controls count must be n_arenas * max_cars_per_arena");
    int rc;
    if ((rc = set_device(b))) return rc;
    if ((rc = ensure_stage(b, n * sizeof(rsg_car_controls)))) return rc;
    RSG_CUDA(cudaMemcpyAsync(b->d_stage, controls, n * sizeof(rsg_car_controls), cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_set_controls(b->buf, (const rsg_car_controls*)b->d_stage, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_car_state(rsg_batch* b, uint32_t arena, uint32_t car_id, rsg_car_state* out) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!out) return fail(RSG_ERR_ARG, "null output");
    int slot = find_slot(b, arena, car_id);
    if (slot < 0) return fail(RSG_ERR_ARG, "no car with that id");
    if ((rc = set_device(b))) return rc;
    if ((rc = ensure_stage(b, sizeof(rsg_car_state) + 8))) return rc;
    uint32_t idx[2] = {arena, (uint32_t)slot};
    char* st = (char*)b->d_stage;
    RSG_CUDA(cudaMemcpyAsync(st + sizeof(rsg_car_state), idx, 8, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_get_cars(b->buf, (const uint32_t*)(st + sizeof(rsg_car_state)), 1, (rsg_car_state*)st, b->stream));
    RSG_CUDA(cudaMemcpyAsync(out, st, sizeof(rsg_car_state), cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_set_car_state(rsg_batch* b, uint32_t arena, uint32_t car_id, const rsg_car_state* in) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!in) return fail(RSG_ERR_ARG, "null state");
    int slot = find_slot(b, arena, car_id);
    if (slot < 0) return fail(RSG_ERR_ARG, "no car with that id");
    if ((rc = set_device(b))) return rc;
    if ((rc = ensure_stage(b, sizeof(rsg_car_state) + 8))) return rc;
    uint32_t idx[2] = {arena, (uint32_t)slot};
    char* st = (char*)b->d_stage;
    RSG_CUDA(cudaMemcpyAsync(st, in, sizeof(rsg_car_state), cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaMemcpyAsync(st + sizeof(rsg_car_state), idx, 8, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_set_cars(b->buf, (const uint32_t*)(st + sizeof(rsg_car_state)), 1, (const rsg_car_state*)st, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_demolish_car(rsg_batch* b, uint32_t arena, uint32_t car_id, float respawn_delay) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    int slot = find_slot(b, arena, car_id);
    if (slot < 0) return fail(RSG_ERR_ARG, "no car with that id");
    if ((rc = set_device(b))) return rc;
    RSG_CUDA(launch_demolish(b->buf, arena, (uint32_t)slot, respawn_delay, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_ball_state(rsg_batch* b, uint32_t arena, rsg_ball_state* out) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!out) return fail(RSG_ERR_ARG, "null output");
    if ((rc = set_device(b))) return rc;
    if ((rc = ensure_stage(b, sizeof(rsg_ball_state) + 8))) return rc;
    char* st = (char*)b->d_stage;
    RSG_CUDA(cudaMemcpyAsync(st + sizeof(rsg_ball_state), &arena, 4, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_get_balls(b->buf, (const uint32_t*)(st + sizeof(rsg_ball_state)), 1, (rsg_ball_state*)st, b->stream));
    RSG_CUDA(cudaMemcpyAsync(out, st, sizeof(rsg_ball_state), cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_set_ball_state(rsg_batch* b, uint32_t arena, const rsg_ball_state* in) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!in) return fail(RSG_ERR_ARG, "null state");
    if ((rc = set_device(b))) return rc;
    if ((rc = ensure_stage(b, sizeof(rsg_ball_state) + 8))) return rc;
    char* st = (char*)b->d_stage;
    RSG_CUDA(cudaMemcpyAsync(st, in, sizeof(rsg_ball_state), cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaMemcpyAsync(st + sizeof(rsg_ball_state), &arena, 4, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_set_balls(b->buf, (const uint32_t*)(st + sizeof(rsg_ball_state)), 1, (const rsg_ball_state*)st,
                              b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

// BallState::hsInfo (src/Sim/Ball/Ball.h:24-32) of one arena: the three floats of its record.
int rsg_get_ball_heatseeker(rsg_batch* b, uint32_t arena, rsg_heatseeker_info* out) {
    int rc;
    if ((rc = check_arena(b, arena))) return rc;
    if (!out) return fail(RSG_ERR_ARG, "null output");
    if ((rc = set_device(b))) return rc;
    const uint32_t* src = b->buf.rec + (size_t)arena * rec_words(b->buf.MC) + rec_ball_f(BF_HS_DIR);
    float v[3];
    RSG_CUDA(cudaMemcpyAsync(v, src, sizeof(v), cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    out->y_target_dir = v[0];
    out->cur_target_speed = v[1];
    out->time_since_hit = v[2];
    return RSG_OK;
}

int rsg_set_ball_heatseeker(rsg_batch* b, uint32_t arena, const rsg_heatseeker_info* in) {
    int rc;
    if ((rc = check_arena(b, arena))) return rc;
    if (!in) return fail(RSG_ERR_ARG, "null input");
    if ((rc = set_device(b))) return rc;
    uint32_t* dst = b->buf.rec + (size_t)arena * rec_words(b->buf.MC) + rec_ball_f(BF_HS_DIR);
    const float v[3] = {in->y_target_dir, in->cur_target_speed, in->time_since_hit};
    RSG_CUDA(cudaMemcpyAsync(dst, v, sizeof(v), cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_pad_state(rsg_batch* b, uint32_t arena, uint32_t pad, rsg_pad_state* out) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!out || pad >= (uint32_t)b->buf.npads) return fail(RSG_ERR_ARG, "pad index out of range");
    if (!b->buf.has_arena) return fail(RSG_ERR_STATE, "this game mode has no boost pads");
    if ((rc = set_device(b))) return rc;
    size_t bytes = sizeof(rsg_pad_state) * b->buf.npads;
    if ((rc = ensure_stage(b, bytes + 8))) return rc;
    char* st = (char*)b->d_stage;
    RSG_CUDA(cudaMemcpyAsync(st + bytes, &arena, 4, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_get_pads(b->buf, (const uint32_t*)(st + bytes), 1, (rsg_pad_state*)st, b->stream));
    RSG_CUDA(cudaMemcpyAsync(out, st + sizeof(rsg_pad_state) * pad, sizeof(rsg_pad_state), cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_set_pad_state(rsg_batch* b, uint32_t arena, uint32_t pad, const rsg_pad_state* in) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!in || pad >= (uint32_t)b->buf.npads) return fail(RSG_ERR_ARG, "pad index out of range");
    if (!b->buf.has_arena) return fail(RSG_ERR_STATE, "this game mode has no boost pads");
    if ((rc = set_device(b))) return rc;
    // one pad block of the arena record: cooldown, active, previous and current locked car
    uint32_t words[PAD_WORDS];
    std::memcpy(&words[PF_COOLDOWN], &in->cooldown, 4);
    words[PF_COUNT + PU_ACTIVE] = in->is_active ? 1u : 0u;
    words[PF_COUNT + PU_PREV_LOCKED] = in->prev_locked_car_id;
    words[PF_COUNT + PU_CUR_LOCKED] = 0;
    uint32_t* rec = b->buf.rec + (size_t)arena * rec_words(b->buf.MC);
    RSG_CUDA(cudaMemcpyAsync(rec + rec_pad_f(0, (int)pad), words, sizeof(words), cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_pad_config(const rsg_batch* b, uint32_t pad, rsg_vec3* pos, int* is_big) {
    if (!b || !pos || !is_big) return fail(RSG_ERR_ARG, "bad argument");
    if (!b->buf.has_arena) return fail(RSG_ERR_STATE, "this game mode has no boost pads");
    if (pad >= (uint32_t)b->buf.npads) return fail(RSG_ERR_ARG, "pad index out of range");
    pos->x = b->pads[pad].x;
    pos->y = b->pads[pad].y;
    pos->z = b->pads[pad].z;
    *is_big = b->pads[pad].w != 0.f ? 1 : 0;
    return RSG_OK;
}

int rsg_get_tick_count(rsg_batch* b, uint32_t arena, uint64_t* out) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!out) return fail(RSG_ERR_ARG, "null output");
    if ((rc = set_device(b))) return rc;
    uint32_t lo = 0, hi = 0;
    if ((rc = read_au(b, AU_TICK_LO, arena, &lo))) return rc;
    if ((rc = read_au(b, AU_TICK_HI, arena, &hi))) return rc;
    *out = (uint64_t)lo | ((uint64_t)hi << 32);
    return RSG_OK;
}

int rsg_set_tick_count(rsg_batch* b, uint32_t arena, uint64_t tick) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if ((rc = set_device(b))) return rc;
    if ((rc = write_au(b, AU_TICK_LO, arena, (uint32_t)tick))) return rc;
    return write_au(b, AU_TICK_HI, arena, (uint32_t)(tick >> 32));
}

int rsg_is_ball_scored(rsg_batch* b, uint32_t arena, int* out) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!out) return fail(RSG_ERR_ARG, "null output");
    if (!b->buf.has_arena) { *out = 0; return RSG_OK; }
    rsg_ball_state s;
    if ((rc = rsg_get_ball_state(b, arena, &s))) return rc;
    // Arena::IsBallScored, soccar (Arena.cpp:893-901), on the state in uu
    *out = std::fabs(s.pos.y) > (b->mutators.goal_base_threshold_y + b->mutators.ball_radius) ? 1 : 0;
    return RSG_OK;
}

int rsg_is_ball_probably_going_in(rsg_batch* b, float max_time, float extra_margin, int* out, int* goal_team) {
    if (!b || !out) return fail(RSG_ERR_ARG, "null batch or output");
    if (b->game_mode != RSG_GAMEMODE_SOCCAR)
        return fail(RSG_ERR_STATE, "IsBallProbablyGoingIn is not supported for this game mode");
    int rc;
    if ((rc = set_device(b))) return rc;
    const size_t A = b->buf.A;
    if ((rc = ensure_stage(b, 2 * sizeof(int) * A))) return rc;
    int* d = (int*)b->d_stage;
    RSG_CUDA(launch_going_in(b->buf, max_time, extra_margin, b->mutators.gravity.x, b->mutators.gravity.z, d, d + A,
                             b->stream));
    RSG_CUDA(cudaMemcpyAsync(out, d, sizeof(int) * A, cudaMemcpyDeviceToHost, b->stream));
    if (goal_team) RSG_CUDA(cudaMemcpyAsync(goal_team, d + A, sizeof(int) * A, cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_all_states(rsg_batch* b, rsg_car_state* cars, rsg_ball_state* balls, rsg_pad_state* pads) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    int rc;
    if ((rc = set_device(b))) return rc;
    size_t A = b->buf.A, MC = b->buf.MC;
    size_t cb = cars ? sizeof(rsg_car_state) * A * MC : 0, bb = balls ? sizeof(rsg_ball_state) * A : 0;
    size_t pb = (pads && b->buf.has_arena) ? sizeof(rsg_pad_state) * A * b->buf.npads : 0;
    if ((rc = ensure_stage(b, cb + bb + pb + 16))) return rc;
    char* st = (char*)b->d_stage;
    // Occupied car slots are a prefix of each arena's slots.  When every slot of the batch holds a
    // car the gathered array goes straight to the caller; otherwise it lands in a host bounce
    // buffer and only each arena's occupied prefix is copied out, so empty slots keep the caller's
    // contents without any host-to-device traffic.
    bool full = true;
    for (size_t a = 0; a < A && full; a++) full = b->ncars[a] == MC;
    if (cars) {
        RSG_CUDA(launch_get_cars(b->buf, nullptr, (int)(A * MC), (rsg_car_state*)st, b->stream));
        if (full) {
            RSG_CUDA(cudaMemcpyAsync(cars, st, cb, cudaMemcpyDeviceToHost, b->stream));
        } else {
            if ((rc = ensure_host_bounce(b, cb))) return rc;
            RSG_CUDA(cudaMemcpyAsync(b->h_bounce, st, cb, cudaMemcpyDeviceToHost, b->stream));
        }
    }
    if (balls) {
        RSG_CUDA(launch_get_balls(b->buf, nullptr, (int)A, (rsg_ball_state*)(st + cb), b->stream));
        RSG_CUDA(cudaMemcpyAsync(balls, st + cb, bb, cudaMemcpyDeviceToHost, b->stream));
    }
    if (pb) {
        RSG_CUDA(launch_get_pads(b->buf, nullptr, (int)A, (rsg_pad_state*)(st + cb + bb), b->stream));
        RSG_CUDA(cudaMemcpyAsync(pads, st + cb + bb, pb, cudaMemcpyDeviceToHost, b->stream));
    }
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    if (cars && !full) {
        const rsg_car_state* src = (const rsg_car_state*)b->h_bounce;
        for (size_t a = 0; a < A; a++)
            if (b->ncars[a]) std::memcpy(cars + a * MC, src + a * MC, sizeof(rsg_car_state) * b->ncars[a]);
    }
    return RSG_OK;
}

int rsg_set_all_states(rsg_batch* b, const rsg_car_state* cars, const rsg_ball_state* balls, const rsg_pad_state* pads) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    int rc;
    if ((rc = set_device(b))) return rc;
    size_t A = b->buf.A, MC = b->buf.MC;
    size_t cb = cars ? sizeof(rsg_car_state) * A * MC : 0, bb = balls ? sizeof(rsg_ball_state) * A : 0;
    size_t pb = (pads && b->buf.has_arena) ? sizeof(rsg_pad_state) * A * b->buf.npads : 0;
    if ((rc = ensure_stage(b, cb + bb + pb + 16))) return rc;
    char* st = (char*)b->d_stage;
    if (cars) {
        RSG_CUDA(cudaMemcpyAsync(st, cars, cb, cudaMemcpyHostToDevice, b->stream));
        RSG_CUDA(launch_set_cars(b->buf, nullptr, (int)(A * MC), (const rsg_car_state*)st, b->stream));
    }
    if (balls) {
        RSG_CUDA(cudaMemcpyAsync(st + cb, balls, bb, cudaMemcpyHostToDevice, b->stream));
        RSG_CUDA(launch_set_balls(b->buf, nullptr, (int)A, (const rsg_ball_state*)(st + cb), b->stream));
    }
    if (pb) {
        RSG_CUDA(cudaMemcpyAsync(st + cb + bb, pads, pb, cudaMemcpyHostToDevice, b->stream));
        RSG_CUDA(launch_set_pads(b->buf, nullptr, (int)A, (const rsg_pad_state*)(st + cb + bb), b->stream));
    }
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_step(rsg_batch* b, int ticks) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    if (ticks < 0) return fail(RSG_ERR_ARG, "negative tick count");
    int rc;
    if ((rc = set_device(b))) return rc;
    // with callbacks registered, events are drained at least every 32 ticks so the
    // per-arena queues (64 entries) cannot overflow from goal events alone
    int chunk = b->buf.event_mask ? 32 : ticks;
    RSG_CUDA(cudaMemsetAsync(b->buf.au + au_index(b, AU_ERR, 0), 0, 4 * (size_t)b->buf.A, b->stream));
    for (int done = 0; done < ticks;) {
        int n = std::min(chunk, ticks - done);
        RSG_CUDA(tuned_launch(b, nullptr, n));
        done += n;
        if (b->buf.event_mask && (rc = drain_events(b))) return rc;
    }
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return check_device_errors(b);
}

int rsg_step_controls(rsg_batch* b, const rsg_car_controls* controls, int ticks) {
    if (!b || !controls) return fail(RSG_ERR_ARG, "null argument");
    if (ticks < 0) return fail(RSG_ERR_ARG, "negative tick count");
    int rc;
    if ((rc = set_device(b))) return rc;
    if (ticks == 0) return RSG_OK;
    const size_t per_tick = (size_t)b->buf.A * b->buf.MC, bytes = per_tick * sizeof(rsg_car_controls) * (size_t)ticks;
    if (b->ctl_bytes < bytes) {
        if (b->d_ctl) {
            RSG_CUDA(cudaStreamSynchronize(b->stream));
            cudaFree(b->d_ctl);
        }
        b->d_ctl = nullptr;
        b->ctl_bytes = 0;
        RSG_CUDA(cudaMalloc(&b->d_ctl, bytes));
        b->ctl_bytes = bytes;
    }
    const rsg_car_controls* d = (const rsg_car_controls*)b->d_ctl;
    RSG_CUDA(cudaMemcpyAsync(b->d_ctl, controls, bytes, cudaMemcpyHostToDevice, b->stream));
    int chunk = b->buf.event_mask ? 32 : ticks;  // as rsg_step: events drained at least every 32 ticks
    RSG_CUDA(cudaMemsetAsync(b->buf.au + au_index(b, AU_ERR, 0), 0, 4 * (size_t)b->buf.A, b->stream));
    for (int done = 0; done < ticks;) {
        int n = std::min(chunk, ticks - done);
        RSG_CUDA(tuned_launch(b, d + (size_t)done * per_tick, n));
        done += n;
        if (b->buf.event_mask && (rc = drain_events(b))) return rc;
    }
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return check_device_errors(b);
}

int rsg_step_async(rsg_batch* b, const rsg_car_controls* d_controls, int ticks) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    if (ticks < 0) return fail(RSG_ERR_ARG, "negative tick count");
    int rc;
    if ((rc = set_device(b))) return rc;
    RSG_CUDA(cudaMemsetAsync(b->buf.au + au_index(b, AU_ERR, 0), 0, 4 * (size_t)b->buf.A, b->stream));
    RSG_CUDA(tuned_launch(b, d_controls, ticks));
    return RSG_OK;
}

int rsg_sync(rsg_batch* b) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    int rc;
    if ((rc = set_device(b))) return rc;
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    if ((rc = drain_events(b))) return rc;
    return check_device_errors(b);
}

void* rsg_batch_stream(rsg_batch* b) { return b ? (void*)b->stream : nullptr; }

int rsg_set_goal_callback(rsg_batch* b, rsg_goal_fn fn, void* user) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    if (fn && !b->buf.has_arena) return fail(RSG_ERR_STATE, "no goal callback in THE_VOID (Arena.cpp:101-102)");
    b->goal_fn = fn;
    b->goal_user = user;
    update_event_mask(b);
    return RSG_OK;
}
int rsg_set_bump_callback(rsg_batch* b, rsg_bump_fn fn, void* user) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    b->bump_fn = fn;
    b->bump_user = user;
    update_event_mask(b);
    return RSG_OK;
}
int rsg_set_ball_hit_callback(rsg_batch* b, rsg_ball_hit_fn fn, void* user) {
    if (!b) return fail(RSG_ERR_ARG, "null batch");
    b->hit_fn = fn;
    b->hit_user = user;
    update_event_mask(b);
    return RSG_OK;
}

int rsg_get_device_flags(rsg_batch* b, uint32_t* out) {
    if (!b || !out) return fail(RSG_ERR_ARG, "null argument");
    int rc;
    if ((rc = set_device(b))) return rc;
    RSG_CUDA(cudaMemcpyAsync(out, b->buf.au + au_index(b, AU_ERR, 0), 4 * (size_t)b->buf.A, cudaMemcpyDeviceToHost, b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_get_tick_shape(const rsg_batch* b, int32_t out[6]) {
    if (!b || !out) return fail(RSG_ERR_ARG, "null argument");
    out[0] = b->shape.arenas_per_block;
    out[1] = b->shape.lanes_per_car;
    out[2] = b->shape.header_cache;
    out[3] = b->shape.leaf_grid;
    out[4] = b->shape.collide_sync;
    out[5] = b->shape.persistent;
    return RSG_OK;
}

int rsg_get_tuning_log(const rsg_batch* b, char* buf, uint64_t buf_len) {
    if (!b || !buf || buf_len == 0) return fail(RSG_ERR_ARG, "null argument");
    const std::string& s = b->tune_log.empty() ? std::string("not tuned yet") : b->tune_log;
    size_t n = std::min<size_t>(s.size(), (size_t)buf_len - 1);
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
    return RSG_OK;
}

// ---------------------------------------------------------------- Arena::Serialize / DeserializeNew / Clone
// RocketSim's byte format (src/DataStream/DataStreamOut.h, DataStreamIn.h): fields little-endian and
// raw; every WriteMultiple group starts with its field count (uint32); Vec is four floats (the
// fourth written 0), RotMat three Vec, bool one byte, enums one byte, CarControls its 24-byte struct.
}  // extern "C"

namespace {

struct StreamOut {
    std::vector<uint8_t> d;
    template <class T>
    void w(T v) {
        const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
        d.insert(d.end(), p, p + sizeof(T));
    }
    void u8(uint32_t v) { w<uint8_t>((uint8_t)v); }
    void vec(rsg_vec3 v) { w(v.x); w(v.y); w(v.z); w(0.f); }
    void rot(const rsg_rotmat& m) { vec(m.forward); vec(m.right); vec(m.up); }
    void group(uint32_t n) { w<uint32_t>(n); }
};

struct StreamIn {
    const uint8_t* p;
    size_t n, pos = 0;
    bool ok = true;
    template <class T>
    T r() {
        T v{};
        if (pos + sizeof(T) > n) { ok = false; pos = n; return v; }
        std::memcpy(&v, p + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    uint8_t u8() { return r<uint8_t>(); }
    rsg_vec3 vec() { rsg_vec3 v{r<float>(), r<float>(), r<float>()}; r<float>(); return v; }
    rsg_rotmat rot() { rsg_rotmat m; m.forward = vec(); m.right = vec(); m.up = vec(); return m; }
    bool group(uint32_t expect) { uint32_t g = r<uint32_t>(); ok = ok && g == expect; return ok; }
};

void put_controls_raw(StreamOut& o, const rsg_car_controls& c) {  // the CarControls struct, 24 bytes
    o.w(c.throttle); o.w(c.steer); o.w(c.pitch); o.w(c.yaw); o.w(c.roll);
    o.u8(c.jump); o.u8(c.boost); o.u8(c.handbrake); o.u8(0);
}
rsg_car_controls get_controls_raw(StreamIn& in) {
    rsg_car_controls c{};
    c.throttle = in.r<float>(); c.steer = in.r<float>(); c.pitch = in.r<float>(); c.yaw = in.r<float>();
    c.roll = in.r<float>();
    c.jump = in.u8(); c.boost = in.u8(); c.handbrake = in.u8(); in.u8();
    return c;
}

// The current controls of slot `slot` (what Car::controls holds), read from the arena record.
rsg_car_controls record_controls(const std::vector<uint32_t>& rec, int slot) {
    rsg_car_controls c{};
    auto f = [&](int k) { float v; std::memcpy(&v, &rec[rec_car_f(CF_CTRL + k, slot)], 4); return v; };
    c.throttle = f(0); c.steer = f(1); c.pitch = f(2); c.yaw = f(3); c.roll = f(4);
    const uint32_t fl = rec[rec_car_u(CU_FLAGS, slot)];
    c.jump = (fl & F_CTRL_JUMP) ? 1 : 0;
    c.boost = (fl & F_CTRL_BOOST) ? 1 : 0;
    c.handbrake = (fl & F_CTRL_HB) ? 1 : 0;
    return c;
}

void put_mutators(StreamOut& o, const rsg_mutator_config& m) {  // MutatorConfig::Serialize (MutatorConfig.cpp:42-45)
    o.w<uint16_t>(30);
    o.group(30);
    o.vec(m.gravity);
    o.w(m.car_mass); o.w(m.car_world_friction); o.w(m.car_world_restitution); o.w(m.ball_mass);
    o.w(m.ball_max_speed); o.w(m.ball_drag); o.w(m.ball_world_friction); o.w(m.ball_world_restitution);
    o.w(m.jump_accel); o.w(m.jump_immediate_force); o.w(m.boost_accel_ground); o.w(m.boost_accel_air);
    o.w(m.boost_used_per_second); o.w(m.respawn_delay); o.w(m.car_spawn_boost_amount); o.w(m.bump_cooldown_time);
    o.w(m.boost_pad_cooldown_big); o.w(m.boost_pad_cooldown_small); o.w(m.ball_hit_extra_force_scale);
    o.w(m.bump_force_scale); o.w(m.ball_radius);
    o.u8(m.unlimited_flips); o.u8(m.unlimited_double_jumps); o.u8(m.recharge_boost_enabled);
    o.w(m.recharge_boost_per_second); o.w(m.recharge_boost_delay);
    o.u8(m.demo_mode); o.u8(m.enable_team_demos);
    o.w(m.goal_base_threshold_y);
}
bool get_mutators(StreamIn& in, rsg_mutator_config& m) {
    std::memset(&m, 0, sizeof(m));
    if (in.r<uint16_t>() != 30 || !in.group(30)) return false;
    m.gravity = in.vec();
    m.car_mass = in.r<float>(); m.car_world_friction = in.r<float>(); m.car_world_restitution = in.r<float>();
    m.ball_mass = in.r<float>(); m.ball_max_speed = in.r<float>(); m.ball_drag = in.r<float>();
    m.ball_world_friction = in.r<float>(); m.ball_world_restitution = in.r<float>(); m.jump_accel = in.r<float>();
    m.jump_immediate_force = in.r<float>(); m.boost_accel_ground = in.r<float>(); m.boost_accel_air = in.r<float>();
    m.boost_used_per_second = in.r<float>(); m.respawn_delay = in.r<float>(); m.car_spawn_boost_amount = in.r<float>();
    m.bump_cooldown_time = in.r<float>(); m.boost_pad_cooldown_big = in.r<float>();
    m.boost_pad_cooldown_small = in.r<float>(); m.ball_hit_extra_force_scale = in.r<float>();
    m.bump_force_scale = in.r<float>(); m.ball_radius = in.r<float>();
    m.unlimited_flips = in.u8(); m.unlimited_double_jumps = in.u8(); m.recharge_boost_enabled = in.u8();
    m.recharge_boost_per_second = in.r<float>(); m.recharge_boost_delay = in.r<float>();
    m.demo_mode = in.u8(); m.enable_team_demos = in.u8();
    m.goal_base_threshold_y = in.r<float>();
    return in.ok;
}

}  // namespace

extern "C" {

// Arena::Serialize (src/Sim/Arena/Arena.cpp:546-574) of one arena.  With `out` NULL or `cap` too
// small, only *len is set (and RSG_OK returned when out is NULL).
int rsg_serialize_arena(rsg_batch* b, uint32_t arena, uint8_t* out, uint64_t cap, uint64_t* len) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!len) return fail(RSG_ERR_ARG, "null length");
    if ((rc = set_device(b))) return rc;
    const size_t MC = b->buf.MC;
    const size_t words = rec_words((int)MC);
    std::vector<uint32_t> rec(words);
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    RSG_CUDA(cudaMemcpy(rec.data(), b->buf.rec + words * arena, 4 * words, cudaMemcpyDeviceToHost));
    uint64_t tick = 0;
    if ((rc = rsg_get_tick_count(b, arena, &tick))) return rc;
    StreamOut o;
    o.group(4);  // gameMode, tickTime, tickCount, _lastCarID
    o.u8((uint32_t)b->game_mode);
    o.w(b->buf.dt);
    o.w<uint64_t>(tick);
    o.w<uint32_t>(b->last_id[arena]);
    const rsg_arena_config& ac = b->arena_cfg;  // ArenaConfig::Serialize (ArenaConfig.cpp:5-14)
    o.group(5);
    o.vec(ac.min_pos); o.vec(ac.max_pos); o.w(ac.max_aabb_len); o.u8(ac.no_ball_rot); o.u8(ac.use_custom_broadphase);
    o.u8(ac.use_custom_boost_pads);
    if (ac.use_custom_boost_pads) {
        o.w<uint32_t>((uint32_t)b->custom_pads.size());
        for (const auto& pc : b->custom_pads) {  // BoostPadConfig::Serialize
            o.group(2);
            o.vec(pc.pos);
            o.u8(pc.is_big);
        }
    }
    const uint32_t n = b->ncars[arena];
    o.w<uint32_t>(n);
    // cars by ascending id: Arena::DeserializeNew gives each car read the next id before forcing
    // the written one (Arena.cpp:590-606), and loses cars whose written ids collide with those
    std::vector<int> slots(n);
    for (uint32_t k = 0; k < n; k++) slots[k] = (int)k;
    std::sort(slots.begin(), slots.end(), [&](int x, int y) { return b->ids[arena * MC + x] < b->ids[arena * MC + y]; });
    for (uint32_t k = 0; k < n; k++) {
        const int slot = slots[k];
        const uint32_t id = b->ids[arena * MC + slot];
        const rsg_car_config& cc = b->car_cfg[arena * MC + slot];
        rsg_car_state st;
        if ((rc = rsg_get_car_state(b, arena, id, &st))) return rc;
        o.u8(b->car_team[arena * MC + slot]);
        o.w<uint32_t>(id);
        const rsg_car_controls c = record_controls(rec, slot);  // Car::Serialize (Car.cpp:325-329)
        o.group(8);
        o.w(c.throttle); o.w(c.steer); o.w(c.pitch); o.w(c.yaw); o.w(c.roll);
        o.u8(c.boost); o.u8(c.jump); o.u8(c.handbrake);
        o.group(9);
        o.w(cc.dodge_deadzone); o.vec(cc.hitbox_pos_offset); o.vec(cc.hitbox_size);
        o.vec(cc.front_wheels.connection_point_offset); o.w(cc.front_wheels.suspension_rest_length);
        o.w(cc.front_wheels.wheel_radius);
        o.vec(cc.back_wheels.connection_point_offset); o.w(cc.back_wheels.suspension_rest_length);
        o.w(cc.back_wheels.wheel_radius);
        const rsg_ball_hit_info& h = st.ball_hit_info;  // CarState::Serialize (Car.cpp:308-314)
        o.u8(h.is_valid);
        if (h.is_valid) {
            o.group(5);
            o.vec(h.relative_pos_on_ball); o.vec(h.ball_pos); o.vec(h.extra_hit_vel);
            o.w(h.tick_count_when_hit); o.w(h.tick_count_when_extra_impulse_applied);
        }
        o.group(30);
        o.vec(st.pos); o.rot(st.rot_mat); o.vec(st.vel); o.vec(st.ang_vel);
        o.u8(st.is_on_ground); o.u8(st.has_jumped); o.u8(st.has_double_jumped); o.u8(st.has_flipped);
        o.vec(st.flip_rel_torque); o.w(st.jump_time); o.u8(st.is_flipping); o.w(st.flip_time); o.u8(st.is_jumping);
        o.w(st.air_time_since_jump); o.w(st.boost); o.u8(st.is_boosting); o.w(st.boosting_time);
        o.w(st.time_since_boosted); o.w(st.supersonic_time); o.w(st.handbrake_val); o.u8(st.is_auto_flipping);
        o.w(st.auto_flip_timer); o.w(st.auto_flip_torque_scale); o.u8(st.is_demoed); o.w(st.demo_respawn_timer);
        put_controls_raw(o, st.last_controls);
        o.u8(st.world_contact_has_contact); o.vec(st.world_contact_normal);
        o.w(st.car_contact_other_car_id); o.w(st.car_contact_cooldown_timer);
    }
    if (b->buf.has_arena && b->buf.npads > 0) {
        o.w<uint32_t>((uint32_t)b->buf.npads);
        for (int i = 0; i < b->buf.npads; i++) {  // BoostPadState::Serialize
            rsg_pad_state ps;
            if ((rc = rsg_get_pad_state(b, arena, (uint32_t)i, &ps))) return rc;
            o.group(3);
            o.u8(ps.is_active); o.w(ps.cooldown); o.w(ps.prev_locked_car_id);
        }
    }
    rsg_ball_state bs;
    if ((rc = rsg_get_ball_state(b, arena, &bs))) return rc;
    rsg_heatseeker_info hs;
    if ((rc = rsg_get_ball_heatseeker(b, arena, &hs))) return rc;
    o.group(12);  // BallState::Serialize (Ball.cpp:19-21); no dropshot state here
    o.vec(bs.pos); o.rot(bs.rot_mat); o.vec(bs.vel); o.vec(bs.ang_vel);
    o.w(hs.y_target_dir); o.w(hs.cur_target_speed); o.w(hs.time_since_hit);  // hsInfo
    o.w<int32_t>(1); o.w(0.f); o.w(0.f);    // dsInfo: chargeLevel, accumulatedHitForce, yTargetDir
    o.u8(0); o.w<uint64_t>(0);              // dsInfo: hasDamaged, lastDamageTick
    put_mutators(o, b->mutators);
    *len = o.d.size();
    if (!out) return RSG_OK;
    if (cap < o.d.size()) return fail(RSG_ERR_ARG, "output buffer smaller than the serialized arena");
    std::memcpy(out, o.d.data(), o.d.size());
    return RSG_OK;
}

// Arena::DeserializeNew (Arena.cpp:576-643) into arena `arena` of the batch: its cars are replaced by
// the serialized ones (ids, teams, configurations, controls and states), then the pads, the ball, the
// tick count and the last car id.  The game mode, tick time, arena config and pad count must be the
// batch's; different mutators are applied when the batch holds this one arena only.
// `spawn_boost`: DeserializeNewCar (Arena.cpp:676-687) runs Car::_BulletSetup after reading the state,
// which sets the boost to the spawn amount of the new arena's mutators (Car.cpp:291); those are still
// the game mode's defaults then, the serialized mutators being read after the cars.
static int deserialize_impl(rsg_batch* b, uint32_t arena, const uint8_t* data, uint64_t len, bool spawn_boost) {
    int rc = check_arena(b, arena);
    if (rc) return rc;
    if (!data) return fail(RSG_ERR_ARG, "null data");
    StreamIn in{data, (size_t)len};
    if (!in.group(4)) return fail(RSG_ERR_ARG, "not a serialized arena (header)");
    const int mode = in.u8();
    const float tick_time = in.r<float>();
    const uint64_t tick = in.r<uint64_t>();
    const uint32_t last_id = in.r<uint32_t>();
    if (mode != b->game_mode || tick_time != b->buf.dt)
        return fail(RSG_ERR_ARG, "serialized arena has another game mode or tick rate than the batch");
    if (!in.group(5)) return fail(RSG_ERR_ARG, "not a serialized arena (arena config)");
    rsg_arena_config ac{};
    ac.min_pos = in.vec(); ac.max_pos = in.vec(); ac.max_aabb_len = in.r<float>();
    ac.no_ball_rot = in.u8(); ac.use_custom_broadphase = in.u8(); ac.use_custom_boost_pads = in.u8();
    std::vector<rsg_boost_pad_config> pads;
    if (ac.use_custom_boost_pads) {
        const uint32_t np = in.r<uint32_t>();
        for (uint32_t i = 0; i < np && in.ok; i++) {
            rsg_boost_pad_config pc{};
            if (!in.group(2)) break;
            pc.pos = in.vec();
            pc.is_big = in.u8();
            pads.push_back(pc);
        }
    }
    const rsg_arena_config& mine = b->arena_cfg;
    bool same = in.ok && (ac.no_ball_rot != 0) == (mine.no_ball_rot != 0) &&
                (ac.use_custom_boost_pads != 0) == (mine.use_custom_boost_pads != 0) &&
                pads.size() == b->custom_pads.size();
    for (size_t i = 0; same && i < pads.size(); i++)
        same = std::memcmp(&pads[i].pos, &b->custom_pads[i].pos, sizeof(rsg_vec3)) == 0 &&
               (pads[i].is_big != 0) == (b->custom_pads[i].is_big != 0);
    if (!same) return fail(RSG_ERR_ARG, "serialized arena config differs from the batch's");
    struct CarRec {
        uint8_t team;
        uint32_t id;
        rsg_car_controls ctl;
        rsg_car_config cfg;
        rsg_car_state st;
    };
    std::vector<CarRec> cars;
    const float spawn_boost_amount = default_mutators(mode).car_spawn_boost_amount;
    const uint32_t ncars = in.r<uint32_t>();
    if (!in.ok || ncars > (uint32_t)b->buf.MC) return fail(RSG_ERR_ARG, "serialized arena has more cars than the batch holds");
    for (uint32_t k = 0; k < ncars && in.ok; k++) {
        CarRec c{};
        c.team = in.u8();
        c.id = in.r<uint32_t>();
        if (!in.group(8)) break;
        c.ctl.throttle = in.r<float>(); c.ctl.steer = in.r<float>(); c.ctl.pitch = in.r<float>();
        c.ctl.yaw = in.r<float>(); c.ctl.roll = in.r<float>();
        c.ctl.boost = in.u8(); c.ctl.jump = in.u8(); c.ctl.handbrake = in.u8();
        if (!in.group(9)) break;
        rsg_get_car_config_preset(RSG_CAR_OCTANE, &c.cfg);  // three_wheels is not serialized
        c.cfg.dodge_deadzone = in.r<float>(); c.cfg.hitbox_pos_offset = in.vec(); c.cfg.hitbox_size = in.vec();
        c.cfg.front_wheels.connection_point_offset = in.vec(); c.cfg.front_wheels.suspension_rest_length = in.r<float>();
        c.cfg.front_wheels.wheel_radius = in.r<float>();
        c.cfg.back_wheels.connection_point_offset = in.vec(); c.cfg.back_wheels.suspension_rest_length = in.r<float>();
        c.cfg.back_wheels.wheel_radius = in.r<float>();
        c.cfg.three_wheels = 0;
        rsg_car_state& st = c.st;
        std::memset(&st, 0, sizeof(st));
        st.ball_hit_info.is_valid = in.u8();
        st.ball_hit_info.tick_count_when_hit = ~0ull;
        st.ball_hit_info.tick_count_when_extra_impulse_applied = ~0ull;
        if (st.ball_hit_info.is_valid) {
            if (!in.group(5)) break;
            st.ball_hit_info.relative_pos_on_ball = in.vec(); st.ball_hit_info.ball_pos = in.vec();
            st.ball_hit_info.extra_hit_vel = in.vec();
            st.ball_hit_info.tick_count_when_hit = in.r<uint64_t>();
            st.ball_hit_info.tick_count_when_extra_impulse_applied = in.r<uint64_t>();
        }
        if (!in.group(30)) break;
        st.pos = in.vec(); st.rot_mat = in.rot(); st.vel = in.vec(); st.ang_vel = in.vec();
        st.is_on_ground = in.u8(); st.has_jumped = in.u8(); st.has_double_jumped = in.u8(); st.has_flipped = in.u8();
        st.flip_rel_torque = in.vec(); st.jump_time = in.r<float>(); st.is_flipping = in.u8(); st.flip_time = in.r<float>();
        st.is_jumping = in.u8(); st.air_time_since_jump = in.r<float>(); st.boost = in.r<float>();
        st.is_boosting = in.u8(); st.boosting_time = in.r<float>(); st.time_since_boosted = in.r<float>();
        st.supersonic_time = in.r<float>(); st.handbrake_val = in.r<float>(); st.is_auto_flipping = in.u8();
        st.auto_flip_timer = in.r<float>(); st.auto_flip_torque_scale = in.r<float>(); st.is_demoed = in.u8();
        st.demo_respawn_timer = in.r<float>();
        st.last_controls = get_controls_raw(in);
        st.world_contact_has_contact = in.u8(); st.world_contact_normal = in.vec();
        st.car_contact_other_car_id = in.r<uint32_t>(); st.car_contact_cooldown_timer = in.r<float>();
        if (spawn_boost) st.boost = spawn_boost_amount;
        cars.push_back(c);
    }
    if (!in.ok) return fail(RSG_ERR_ARG, "serialized arena is truncated or malformed (cars)");
    std::vector<rsg_pad_state> pad_states;
    if (b->buf.has_arena && b->buf.npads > 0) {
        const uint32_t np = in.r<uint32_t>();
        if (np != (uint32_t)b->buf.npads) return fail(RSG_ERR_ARG, "serialized arena has another boost pad count");
        for (uint32_t i = 0; i < np && in.ok; i++) {
            rsg_pad_state ps{};
            if (!in.group(3)) break;
            ps.is_active = in.u8(); ps.cooldown = in.r<float>(); ps.prev_locked_car_id = in.r<uint32_t>();
            pad_states.push_back(ps);
        }
    }
    rsg_ball_state bs{};
    rsg_heatseeker_info hs{0.f, RL::HS::INITIAL_TARGET_SPEED, 0.f};
    if (in.group(12)) {
        bs.pos = in.vec(); bs.rot_mat = in.rot(); bs.vel = in.vec(); bs.ang_vel = in.vec();
        hs.y_target_dir = in.r<float>(); hs.cur_target_speed = in.r<float>(); hs.time_since_hit = in.r<float>();
        in.r<int32_t>(); in.r<float>(); in.r<float>(); in.u8();
        in.r<uint64_t>();
    }
    rsg_mutator_config mut;
    if (!in.ok || !get_mutators(in, mut)) return fail(RSG_ERR_ARG, "serialized arena is truncated or malformed");
    if (std::memcmp(&mut, &b->mutators, sizeof(mut)) != 0) {
        if (b->buf.A != 1) return fail(RSG_ERR_ARG, "serialized mutators differ from the batch's (a batch shares them)");
    }
    // replace the cars
    while (b->ncars[arena] > 0) {
        if ((rc = rsg_remove_car(b, arena, b->ids[arena * b->buf.MC]))) return rc;
    }
    if (std::memcmp(&mut, &b->mutators, sizeof(mut)) != 0)
        if ((rc = rsg_set_mutator_config(b, &mut))) return rc;
    for (const CarRec& c : cars) {
        uint32_t id;
        if ((rc = add_car_impl(b, arena, c.team, &c.cfg, 0, c.id, &id))) return rc;
        if ((rc = rsg_set_car_state(b, arena, id, &c.st))) return rc;
        if ((rc = rsg_set_car_controls(b, arena, id, &c.ctl))) return rc;
    }
    b->last_id[arena] = last_id;
    for (size_t i = 0; i < pad_states.size(); i++)
        if ((rc = rsg_set_pad_state(b, arena, (uint32_t)i, &pad_states[i]))) return rc;
    if ((rc = rsg_set_ball_state(b, arena, &bs))) return rc;
    if ((rc = rsg_set_ball_heatseeker(b, arena, &hs))) return rc;
    return rsg_set_tick_count(b, arena, tick);
}

int rsg_deserialize_arena(rsg_batch* b, uint32_t arena, const uint8_t* data, uint64_t len) {
    return deserialize_impl(b, arena, data, len, true);
}

// Arena::Clone (Arena.cpp:646-674) from one batch arena into another: the cars, pads, tick count and
// last car id through the serialized form, then every car state and the ball state whole, as Clone
// copies them with Car::SetState / Ball::SetState (the fields the byte format leaves out, such as
// the air time, included).
int rsg_clone_arena(rsg_batch* dst, uint32_t dst_arena, rsg_batch* src, uint32_t src_arena) {
    uint64_t n = 0;
    int rc = rsg_serialize_arena(src, src_arena, nullptr, 0, &n);
    if (rc) return rc;
    std::vector<uint8_t> buf(n);
    if ((rc = rsg_serialize_arena(src, src_arena, buf.data(), n, &n))) return rc;
    const std::vector<uint32_t> ids(src->ids.begin() + (size_t)src_arena * src->buf.MC,
                                    src->ids.begin() + (size_t)src_arena * src->buf.MC + src->ncars[src_arena]);
    std::vector<rsg_car_state> states(ids.size());
    for (size_t k = 0; k < ids.size(); k++)
        if ((rc = rsg_get_car_state(src, src_arena, ids[k], &states[k]))) return rc;
    rsg_ball_state bs;
    rsg_heatseeker_info hs;
    if ((rc = rsg_get_ball_state(src, src_arena, &bs))) return rc;
    if ((rc = rsg_get_ball_heatseeker(src, src_arena, &hs))) return rc;
    if ((rc = deserialize_impl(dst, dst_arena, buf.data(), n, false))) return rc;
    for (size_t k = 0; k < ids.size(); k++)
        if ((rc = rsg_set_car_state(dst, dst_arena, ids[k], &states[k]))) return rc;
    if ((rc = rsg_set_ball_state(dst, dst_arena, &bs))) return rc;
    return rsg_set_ball_heatseeker(dst, dst_arena, &hs);
}

}  // extern "C"

// ---------------------------------------------------------------- kickoff
namespace {

// std::default_random_engine of libstdc++ (minstd_rand0: x <- 16807 x mod 2^31 - 1, seed 0 -> 1)
struct MinStd0 {  // the engine's word is 64 bits wide on LP64 (uint_fast32_t): a negative seed wraps there
    uint32_t x;
    explicit MinStd0(int64_t seed) { x = (uint32_t)((uint64_t)seed % 2147483647u); if (x == 0) x = 1; }
    uint32_t operator()() { x = (uint32_t)(((uint64_t)x * 16807u) % 2147483647u); return x; }
};

// std::uniform_int_distribution<size_t>{0, hi} over it (libstdc++'s down-scaling with rejection: the
// engine's range [1, 2^31 - 2] is cut into hi + 1 equal buckets, draws past the last one are redrawn)
uint32_t uniform_upto(MinStd0& g, uint32_t hi) {
    const uint32_t range = 2147483646u - 1u, buckets = hi + 1;
    const uint32_t scaling = range / buckets, past = buckets * scaling;
    uint32_t r;
    do r = g() - 1u; while (r >= past);
    return r / scaling;
}

// std::shuffle of libstdc++ for an engine whose range exceeds n^2: after an up-front swap when n is
// even, positions are drawn two at a time, (i, i + 1) from one uniform draw over (i + 1)(i + 2).
void shuffle5(int* v, int n, MinStd0& g) {
    if (n < 2) return;
    int i = 1;
    if (n % 2 == 0) std::swap(v[i++], v[uniform_upto(g, 1)]);
    while (i != n) {
        const uint32_t r0 = (uint32_t)i + 1, r1 = r0 + 1;
        const uint32_t x = uniform_upto(g, r0 * r1 - 1);
        std::swap(v[i++], v[x / r1]);
        std::swap(v[i++], v[x % r1]);
    }
}

MinStd0& process_engine() {  // Math::GetRandEngine: one engine for the process, seeded from the clock
    static MinStd0 g((int64_t)(std::chrono::steady_clock::now().time_since_epoch().count() & 0x7fffffff));
    return g;
}

}  // namespace

extern "C" {

// Arena::ResetToRandomKickoff (src/Sim/Arena/Arena.cpp:113-222) for arenas[k] with seeds[k] (-1:
// the process-wide engine): the five soccar kickoff spots shuffled, blue cars placed in update
// order on them (then on the respawn spots, 250 uu further back for each car already there),
// orange cars mirrored; the ball at rest at the centre and every pad reset.
int rsg_reset_to_random_kickoff_many(rsg_batch* b, const uint32_t* arenas, const int32_t* seeds, uint32_t n) {
    if (!b || (n && !arenas)) return fail(RSG_ERR_ARG, "null batch or arena list");
    const bool hs = b->game_mode == RSG_GAMEMODE_HEATSEEKER;
    if (b->game_mode != RSG_GAMEMODE_SOCCAR && !hs) return fail(RSG_ERR_STATE, "kickoffs need the soccar arena");
    static const float SPAWN[5][3] = {{-2048, -2560, (float)(M_PI_4 * 1)}, {2048, -2560, (float)(M_PI_4 * 3)},
                                      {-256, -3840, (float)(M_PI_4 * 2)}, {256, -3840, (float)(M_PI_4 * 2)},
                                      {0, -4608, (float)(M_PI_4 * 2)}};
    static const float RESPAWN[4][3] = {{-2304, -4608, (float)(M_PI / 2)}, {-2688, -4608, (float)(M_PI / 2)},
                                        {2304, -4608, (float)(M_PI / 2)}, {2688, -4608, (float)(M_PI / 2)}};
    // CAR_SPAWN_LOCATIONS_HEATSEEKER (src/RLConst.h:364-370): four spots, the soccar respawn spots past them
    static const float SPAWN_HS[4][3] = {{-1000, -4620, (float)(M_PI / 2)}, {1000, -4620, (float)(M_PI / 2)},
                                         {-2000, -4620, (float)(M_PI / 2)}, {2000, -4620, (float)(M_PI / 2)}};
    const int nloc = hs ? 4 : 5;
    std::vector<float> ball_side(n, 1.f);
    const int MC = b->buf.MC;
    std::vector<uint32_t> idx;
    std::vector<rsg_car_state> cars;
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t ar = arenas[k];
        int rc = check_arena(b, ar);
        if (rc) return rc;
        int order[5] = {0, 1, 2, 3, 4};
        const int32_t seed = seeds ? seeds[k] : -1;
        MinStd0 local((int64_t)(seed == -1 ? 1 : seed));
        MinStd0& g = seed == -1 ? process_engine() : local;
        shuffle5(order, nloc, g);
        // heatseeker's ball starts on the side of the next draw of the same engine (Arena.cpp:200-204)
        if (hs) ball_side[k] = ((int)g() % 2) ? 1.f : -1.f;
        std::vector<int> team_slots[2];
        for (uint32_t p = 0; p < b->ncars[ar]; p++) {
            const int slot = b->order[(size_t)ar * MC + p];
            team_slots[b->car_team[(size_t)ar * MC + slot] == RSG_TEAM_BLUE ? 0 : 1].push_back(slot);
        }
        int at_respawn[4] = {};
        const int npos = (int)std::max(team_slots[0].size(), team_slots[1].size());
        for (int i = 0; i < npos; i++) {
            float x, y, yaw;
            if (i < nloc) {
                const float* sp = hs ? SPAWN_HS[std::min(order[i], nloc - 1)] : SPAWN[std::min(order[i], nloc - 1)];
                x = sp[0]; y = sp[1]; yaw = sp[2];
            } else {
                const int r = (i - nloc) % nloc;
                const float* sp = RESPAWN[r < 4 ? r : 3];
                x = sp[0]; y = sp[1]; yaw = sp[2];
                if (r < 4) y += 250.f * at_respawn[r]++;
            }
            for (int t = 0; t < 2; t++) {
                if (i >= (int)team_slots[t].size()) continue;
                rsg_car_state st = respawn_state(RSG_TEAM_BLUE, 0, b->mutators.car_spawn_boost_amount);
                float yy = yaw;
                st.pos = rsg_vec3{x, y, RL::CAR_SPAWN_REST_Z};
                if (t == 1) {
                    st.pos.x *= -1; st.pos.y *= -1;
                    yy = (float)((double)yaw + M_PI);
                }
                const M3 m = m_euler_ypr(yy, -0.f, -0.f);
                const V3 f = m.col(0), r = m.col(1), u = m.col(2);
                st.rot_mat.forward = {f.x, f.y, f.z};
                st.rot_mat.right = {r.x, r.y, r.z};
                st.rot_mat.up = {u.x, u.y, u.z};
                idx.push_back(ar);
                idx.push_back((uint32_t)team_slots[t][i]);
                cars.push_back(st);
            }
        }
    }
    if (!n) return RSG_OK;
    int rc;
    if ((rc = set_device(b))) return rc;
    std::vector<rsg_ball_state> balls(n);
    for (uint32_t k = 0; k < n; k++) {
        rsg_ball_state& bs = balls[k];
        std::memset(&bs, 0, sizeof(bs));
        bs.pos.z = RL::BALL_REST_Z;
        bs.rot_mat.forward.x = bs.rot_mat.right.y = bs.rot_mat.up.z = 1;
        if (hs) {  // Heatseeker::BALL_START_POS / BALL_START_VEL (RLConst.h:186-188), y flipped by the side
            const float* p = RL::HS::BALL_START_POS;
            const float* v = RL::HS::BALL_START_VEL;
            bs.pos = rsg_vec3{p[0] * 1, p[1] * ball_side[k], p[2] * 1};
            bs.vel = rsg_vec3{v[0] * 1, v[1] * ball_side[k], v[2] * 1};
        }
    }
    std::vector<rsg_pad_state> pads((size_t)n * b->buf.npads);
    for (auto& ps : pads) {
        std::memset(&ps, 0, sizeof(ps));
        ps.is_active = 1;
    }
    const size_t ib = idx.size() * 4, cb = cars.size() * sizeof(rsg_car_state), ab = (size_t)n * 4;
    const size_t bb = balls.size() * sizeof(rsg_ball_state), pb = pads.size() * sizeof(rsg_pad_state);
    auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
    if ((rc = ensure_stage(b, al(ib) + al(cb) + al(ab) + al(bb) + al(pb) + 16))) return rc;
    char* st = (char*)b->d_stage;
    char *d_idx = st, *d_cars = d_idx + al(ib), *d_ar = d_cars + al(cb), *d_balls = d_ar + al(ab), *d_pads = d_balls + al(bb);
    if (!cars.empty()) {
        RSG_CUDA(cudaMemcpyAsync(d_idx, idx.data(), ib, cudaMemcpyHostToDevice, b->stream));
        RSG_CUDA(cudaMemcpyAsync(d_cars, cars.data(), cb, cudaMemcpyHostToDevice, b->stream));
        RSG_CUDA(launch_set_cars(b->buf, (const uint32_t*)d_idx, (int)cars.size(), (const rsg_car_state*)d_cars, b->stream));
    }
    RSG_CUDA(cudaMemcpyAsync(d_ar, arenas, ab, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(cudaMemcpyAsync(d_balls, balls.data(), bb, cudaMemcpyHostToDevice, b->stream));
    RSG_CUDA(launch_set_balls(b->buf, (const uint32_t*)d_ar, (int)n, (const rsg_ball_state*)d_balls, b->stream));
    if (pb) {
        RSG_CUDA(cudaMemcpyAsync(d_pads, pads.data(), pb, cudaMemcpyHostToDevice, b->stream));
        RSG_CUDA(launch_set_pads(b->buf, (const uint32_t*)d_ar, (int)n, (const rsg_pad_state*)d_pads, b->stream));
    }
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

int rsg_reset_to_random_kickoff(rsg_batch* b, uint32_t arena, int32_t seed) {
    return rsg_reset_to_random_kickoff_many(b, &arena, &seed, 1);
}

}  // extern "C"

// ---------------------------------------------------------------- game events
struct rsg_game_event_tracker {
    int A = 0, device = 0;
    GameEventCfgDev cfg{};
    GameEventDev d{};
    rsg_game_event* d_ev = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t src_done = nullptr;
};

namespace {
void event_tracker_free(rsg_game_event_tracker* t) {
    if (!t) return;
    cudaFree(t->d.shot_cooldown); cudaFree(t->d.ball_shot); cudaFree(t->d.shot_goal_team); cudaFree(t->d.scored_last);
    cudaFree(t->d.last_update); cudaFree(t->d_ev);
    if (t->src_done) cudaEventDestroy(t->src_done);
    if (t->stream) cudaStreamDestroy(t->stream);
    delete t;
}
}  // namespace

extern "C" {

// GameEventTrackerConfig's defaults (GameEventTracker.h:10-40), autoStateSetDetection on
int rsg_get_default_game_event_tracker_config(rsg_game_event_tracker_config* out) {
    if (!out) return fail(RSG_ERR_ARG, "null output");
    std::memset(out, 0, sizeof(*out));
    out->shot_min_speed = 1750;
    out->shot_touch_min_delay = 0.3f;
    out->pred_score_extra_margin = 0;
    out->shot_event_cooldown = 1.0f;
    out->shot_min_score_time = 2.0f;
    out->goal_max_touch_time = 4.0f;
    out->pass_max_touch_time = 2.0f;
    out->auto_state_set_detection = 1;
    return RSG_OK;
}

rsg_game_event_tracker* rsg_game_event_tracker_create(rsg_batch* b, const rsg_game_event_tracker_config* config) {
    if (!b) { fail(RSG_ERR_ARG, "null batch"); return nullptr; }
    if (b->game_mode != RSG_GAMEMODE_SOCCAR) { fail(RSG_ERR_STATE, "game events need the soccar arena"); return nullptr; }
    if (set_device(b)) return nullptr;
    rsg_game_event_tracker_config c;
    if (config) c = *config; else rsg_get_default_game_event_tracker_config(&c);
    rsg_game_event_tracker* t = new rsg_game_event_tracker();
    t->A = b->buf.A;
    t->device = b->device;
    t->cfg = GameEventCfgDev{c.shot_min_speed, c.shot_touch_min_delay, c.pred_score_extra_margin, c.shot_event_cooldown,
                             c.shot_min_score_time, c.goal_max_touch_time, c.pass_max_touch_time,
                             c.auto_state_set_detection ? 1 : 0};
    const size_t A = (size_t)t->A;
    bool ok = true;
    auto alloc = [&](void** q, size_t bytes) {
        if (!ok) return;
        cudaError_t e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) e = cudaMemset(*q, 0, bytes);
        if (e != cudaSuccess) { cuda_fail(e, "cudaMalloc(game events)"); ok = false; }
    };
    alloc((void**)&t->d.shot_cooldown, 4 * A);
    alloc((void**)&t->d.ball_shot, 4 * A);
    alloc((void**)&t->d.shot_goal_team, 4 * A);
    alloc((void**)&t->d.scored_last, 4 * A);
    alloc((void**)&t->d.last_update, 8 * A);
    alloc((void**)&t->d_ev, sizeof(rsg_game_event) * A);
    if (ok && cudaDeviceSynchronize() != cudaSuccess) ok = false;  // the zeroing done before any stream uses them
    if (ok && cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) ok = false;
    if (ok && cudaEventCreateWithFlags(&t->src_done, cudaEventDisableTiming) != cudaSuccess) ok = false;
    if (!ok) {
        fail(RSG_ERR_CUDA, "game event tracker allocation");
        event_tracker_free(t);
        return nullptr;
    }
    return t;
}

void rsg_game_event_tracker_destroy(rsg_game_event_tracker* t) {
    if (t) cudaSetDevice(t->device);
    event_tracker_free(t);
}

int rsg_game_event_tracker_update(rsg_game_event_tracker* t, rsg_batch* b, rsg_game_event* events) {
    if (!t || !b || !events) return fail(RSG_ERR_ARG, "null tracker, batch or output");
    if (b->buf.A != t->A || b->device != t->device) return fail(RSG_ERR_ARG, "the batch is not the tracker's shape or device");
    int rc;
    if ((rc = set_device(b))) return rc;
    RSG_CUDA(cudaEventRecord(t->src_done, b->stream));
    RSG_CUDA(cudaStreamWaitEvent(t->stream, t->src_done, 0));
    RSG_CUDA(launch_game_events(b->buf, t->d, t->cfg, b->mutators.gravity.x, b->mutators.gravity.z, t->d_ev, t->stream));
    RSG_CUDA(cudaMemcpyAsync(events, t->d_ev, sizeof(rsg_game_event) * (size_t)t->A, cudaMemcpyDeviceToHost, t->stream));
    RSG_CUDA(cudaStreamSynchronize(t->stream));
    return RSG_OK;
}

int rsg_game_event_tracker_reset_persistent_info(rsg_game_event_tracker* t, int32_t arena) {
    if (!t) return fail(RSG_ERR_ARG, "null tracker");
    if (arena < -1 || arena >= t->A) return fail(RSG_ERR_ARG, "arena index out of range");
    RSG_CUDA(cudaSetDevice(t->device));
    const size_t off = arena < 0 ? 0 : (size_t)arena, n = arena < 0 ? (size_t)t->A : 1;
    RSG_CUDA(cudaMemsetAsync(t->d.scored_last + off, 0, 4 * n, t->stream));
    RSG_CUDA(cudaMemsetAsync(t->d.ball_shot + off, 0, 4 * n, t->stream));
    RSG_CUDA(cudaMemsetAsync(t->d.shot_cooldown + off, 0, 4 * n, t->stream));
    RSG_CUDA(cudaStreamSynchronize(t->stream));
    return RSG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- ball prediction
// BallPredTracker (src/Sim/BallPredTracker/BallPredTracker.cpp) for every arena of a batch: the
// tracker batch holds one ball-only arena per source arena (Arena::Create with the source's game
// mode, arena config and tick rate, BallPredTracker.cpp:5-12: default mutators, no cars) and the
// device side (BallPredDev) the predictions and the run list of an update.
struct rsg_ball_pred {
    rsg_batch* arena = nullptr;
    int A = 0, T = 0;
    float tick_time = 0;
    BallPredDev d{};
    void* d_in = nullptr;  // staging: cur [A] states, ticks [A], mask [A]
    cudaEvent_t src_done = nullptr;
};

namespace {

void ball_pred_free(rsg_ball_pred* p) {
    if (!p) return;
    cudaFree(p->d.pred); cudaFree(p->d.head); cudaFree(p->d.last_update); cudaFree(p->d.valid);
    cudaFree(p->d.list); cudaFree(p->d.count); cudaFree(p->d.steps); cudaFree(p->d.base); cudaFree(p->d_in);
    if (p->src_done) cudaEventDestroy(p->src_done);
    if (p->arena) rsg_batch_destroy(p->arena);
    delete p;
}

size_t in_bytes(int A) { return (size_t)A * (sizeof(rsg_ball_state) + sizeof(int32_t) + 1); }

// Stages the host inputs of an update (any may be null) and runs it on the tracker's stream.
int ball_pred_update(rsg_ball_pred* p, rsg_batch* src, int mode, const rsg_ball_state* cur, const int32_t* ticks,
                     const uint8_t* mask) {
    if (!p) return fail(RSG_ERR_ARG, "null tracker");
    rsg_batch* b = p->arena;
    int rc = set_device(b);
    if (rc) return rc;
    const size_t A = (size_t)p->A;
    char* in = (char*)p->d_in;
    rsg_ball_state* d_cur = (rsg_ball_state*)in;
    int32_t* d_ticks = (int32_t*)(in + A * sizeof(rsg_ball_state));
    uint8_t* d_mask = (uint8_t*)(in + A * (sizeof(rsg_ball_state) + sizeof(int32_t)));
    if (cur) RSG_CUDA(cudaMemcpyAsync(d_cur, cur, A * sizeof(rsg_ball_state), cudaMemcpyHostToDevice, b->stream));
    if (ticks) RSG_CUDA(cudaMemcpyAsync(d_ticks, ticks, A * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    if (mask) RSG_CUDA(cudaMemcpyAsync(d_mask, mask, A, cudaMemcpyHostToDevice, b->stream));
    if (src) {  // the source batch's queued ticks come first
        RSG_CUDA(cudaEventRecord(p->src_done, src->stream));
        RSG_CUDA(cudaStreamWaitEvent(b->stream, p->src_done, 0));
    }
    RSG_CUDA(launch_ball_pred(b->buf, p->d, src ? &src->buf : nullptr, mode, d_cur, d_ticks, mask ? d_mask : nullptr,
                              b->stream));
    RSG_CUDA(cudaStreamSynchronize(b->stream));
    return RSG_OK;
}

}  // namespace

extern "C" {

rsg_ball_pred* rsg_ball_pred_create(rsg_batch* src, uint32_t num_pred_ticks) {
    if (!src) { fail(RSG_ERR_ARG, "null batch"); return nullptr; }
    if (src->game_mode == RSG_GAMEMODE_HEATSEEKER) {  // the prediction inputs carry no heatseeker state
        fail(RSG_ERR_STATE, "ball prediction supports soccar and the void");
        return nullptr;
    }
    if (num_pred_ticks == 0 || num_pred_ticks > (1u << 20)) {
        fail(RSG_ERR_ARG, "num_pred_ticks must be 1..1048576");
        return nullptr;
    }
    if (set_device(src)) return nullptr;
    const size_t A = (size_t)src->buf.A, T = num_pred_ticks;
    rsg_ball_pred* p = new rsg_ball_pred();
    p->A = (int)A;
    p->T = (int)T;
    // Arena::Create(arena->gameMode, arena->GetArenaConfig(), arena->GetTickRate())
    p->arena = rsg_batch_create_ex(src->game_mode, (uint32_t)A, 1, 1.f / src->buf.dt, &src->arena_cfg);
    if (!p->arena) { ball_pred_free(p); return nullptr; }
    p->tick_time = p->arena->buf.dt;
    p->d.T = (int)T;
    bool ok = true;
    auto alloc = [&](void** q, size_t bytes) {
        if (!ok) return;
        cudaError_t e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) e = cudaMemset(*q, 0, bytes);
        if (e != cudaSuccess) { cuda_fail(e, "cudaMalloc(ball prediction)"); ok = false; }
    };
    alloc((void**)&p->d.pred, sizeof(rsg_ball_state) * A * T);
    alloc((void**)&p->d.head, sizeof(uint32_t) * A);
    alloc((void**)&p->d.last_update, sizeof(int32_t) * A);
    alloc((void**)&p->d.valid, A);
    alloc((void**)&p->d.list, sizeof(int) * A);
    alloc((void**)&p->d.count, sizeof(int));
    alloc((void**)&p->d.steps, sizeof(int) * A);
    alloc((void**)&p->d.base, sizeof(uint32_t) * A);
    alloc(&p->d_in, in_bytes((int)A));
    if (ok && cudaDeviceSynchronize() != cudaSuccess) ok = false;  // the zeroing done before any stream uses them
    if (ok && cudaEventCreateWithFlags(&p->src_done, cudaEventDisableTiming) != cudaSuccess) {
        fail(RSG_ERR_CUDA, "cudaEventCreate");
        ok = false;
    }
    // the constructor's UpdatePredFromArena (BallPredTracker.cpp:11)
    if (!ok || ball_pred_update(p, src, 0, nullptr, nullptr, nullptr) != RSG_OK) {
        ball_pred_free(p);
        return nullptr;
    }
    return p;
}

void rsg_ball_pred_destroy(rsg_ball_pred* p) {
    if (p && p->arena) set_device(p->arena);
    ball_pred_free(p);
}

int rsg_ball_pred_update_from_batch(rsg_ball_pred* p, rsg_batch* src, const uint8_t* mask) {
    if (!p || !src) return fail(RSG_ERR_ARG, "null tracker or batch");
    if (src->buf.A != p->A) return fail(RSG_ERR_ARG, "the batch has another arena count than the tracker");
    if (src->device != p->arena->device) return fail(RSG_ERR_ARG, "the batch is on another device");
    return ball_pred_update(p, src, 0, nullptr, nullptr, mask);
}

int rsg_ball_pred_update_manual(rsg_ball_pred* p, const rsg_ball_state* cur, const int32_t* ticks_since_last_update,
                                const uint8_t* mask) {
    if (!p || !cur || !ticks_since_last_update) return fail(RSG_ERR_ARG, "null tracker or input");
    return ball_pred_update(p, nullptr, 1, cur, ticks_since_last_update, mask);
}

int rsg_ball_pred_force_update_all(rsg_ball_pred* p, const rsg_ball_state* initial, const uint8_t* mask) {
    if (!p || !initial) return fail(RSG_ERR_ARG, "null tracker or input");
    return ball_pred_update(p, nullptr, 2, initial, nullptr, mask);
}

uint32_t rsg_ball_pred_num_pred_ticks(const rsg_ball_pred* p) { return p ? (uint32_t)p->T : 0; }

int rsg_ball_pred_get_pred(rsg_ball_pred* p, uint32_t arena, rsg_ball_state* out) {
    if (!p || !out) return fail(RSG_ERR_ARG, "null tracker or output");
    if (arena >= (uint32_t)p->A) return fail(RSG_ERR_ARG, "arena index out of range");
    int rc = set_device(p->arena);
    if (rc) return rc;
    uint32_t head = 0;
    cudaStream_t st = p->arena->stream;
    RSG_CUDA(cudaMemcpyAsync(&head, p->d.head + arena, sizeof(head), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    const size_t T = (size_t)p->T;
    const rsg_ball_state* ring = p->d.pred + (size_t)arena * T;
    RSG_CUDA(cudaMemcpyAsync(out, ring + head, (T - head) * sizeof(rsg_ball_state), cudaMemcpyDeviceToHost, st));
    if (head) RSG_CUDA(cudaMemcpyAsync(out + (T - head), ring, head * sizeof(rsg_ball_state), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    return RSG_OK;
}

int rsg_ball_pred_get_all(rsg_ball_pred* p, rsg_ball_state* out) {
    if (!p || !out) return fail(RSG_ERR_ARG, "null tracker or output");
    int rc = set_device(p->arena);
    if (rc) return rc;
    const size_t A = (size_t)p->A, T = (size_t)p->T;
    std::vector<uint32_t> head(A);
    std::vector<rsg_ball_state> ring(A * T);
    cudaStream_t st = p->arena->stream;
    RSG_CUDA(cudaMemcpyAsync(head.data(), p->d.head, A * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaMemcpyAsync(ring.data(), p->d.pred, A * T * sizeof(rsg_ball_state), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    for (size_t a = 0; a < A; a++) {
        const rsg_ball_state* r = ring.data() + a * T;
        rsg_ball_state* o = out + a * T;
        std::memcpy(o, r + head[a], (T - head[a]) * sizeof(rsg_ball_state));
        std::memcpy(o + (T - head[a]), r, head[a] * sizeof(rsg_ball_state));
    }
    return RSG_OK;
}

// GetBallStateForTime (BallPredTracker.cpp:74-79): predData[(int)RS_CLAMP(predTime / tickTime, 0, size - 1)],
// the clamp in float as the macro's conditional expressions give it.
int rsg_ball_pred_get_state_for_time(rsg_ball_pred* p, uint32_t arena, float pred_time, rsg_ball_state* out) {
    if (!p || !out) return fail(RSG_ERR_ARG, "null tracker or output");
    if (arena >= (uint32_t)p->A) return fail(RSG_ERR_ARG, "arena index out of range");
    int rc = set_device(p->arena);
    if (rc) return rc;
    float x = pred_time / p->tick_time;
    x = x > 0 ? x : 0.f;
    const float hi = (float)(p->T - 1);
    x = x < hi ? x : hi;
    const uint32_t idx = (uint32_t)(int)x;
    uint32_t head = 0;
    cudaStream_t st = p->arena->stream;
    RSG_CUDA(cudaMemcpyAsync(&head, p->d.head + arena, sizeof(head), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    const size_t slot = (size_t)arena * p->T + (head + idx) % (uint32_t)p->T;
    RSG_CUDA(cudaMemcpyAsync(out, p->d.pred + slot, sizeof(rsg_ball_state), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    return RSG_OK;
}

int rsg_ball_pred_get_last_update_tick(rsg_ball_pred* p, uint32_t arena, int32_t* out) {
    if (!p || !out) return fail(RSG_ERR_ARG, "null tracker or output");
    if (arena >= (uint32_t)p->A) return fail(RSG_ERR_ARG, "arena index out of range");
    int rc = set_device(p->arena);
    if (rc) return rc;
    RSG_CUDA(cudaMemcpyAsync(out, p->d.last_update + arena, sizeof(int32_t), cudaMemcpyDeviceToHost, p->arena->stream));
    RSG_CUDA(cudaStreamSynchronize(p->arena->stream));
    return RSG_OK;
}

int rsg_ball_pred_device_buffers(rsg_ball_pred* p, const rsg_ball_state** d_pred, const uint32_t** d_head) {
    if (!p || !d_pred || !d_head) return fail(RSG_ERR_ARG, "null tracker or output");
    *d_pred = p->d.pred;
    *d_head = p->d.head;
    return RSG_OK;
}

int rsg_ball_pred_device_flags(rsg_ball_pred* p, uint32_t* out) {
    if (!p) return fail(RSG_ERR_ARG, "null tracker");
    return rsg_get_device_flags(p->arena, out);
}

}  // extern "C"
